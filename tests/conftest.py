import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

SEED0 = 0x70E0F0F7
GOLDEN = ROOT / "tests" / "golden" / "reference_golden.npz"


def pytest_addoption(parser):
    parser.addoption("--emu-sanitize", action="store_true", default=False,
                     help="build the host emulation of the library with AddressSanitizer and "
                          "UBSan (the interpreter must preload their runtimes)")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle.Oracle()


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def T():
    """The library's Python mirror (loads libtopefft.so; builds it if absent)."""
    import __graft_entry__ as g
    lib = ROOT / "tope-fft_gb300" / "libtopefft.so"
    if not lib.exists():
        g._load_build_module().build_library()
    return g.load_package()


@pytest.fixture(params=["fp64", "df64"])
def fw(T, request):
    """A fresh framework on cuda:0 (GPU tests only), once per butterfly
    arithmetic: native FP64 and double-float (FP32 pairs)."""
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.check(f)
    T.topeSetArith(f, T.TOPE_ARITH_DF64 if request.param == "df64" else T.TOPE_ARITH_FP64)
    T.check(f)
    yield f
    T.topeFFTDestroy(f)


def tol_fp64(n_points: int) -> float:
    """The plain FP64 gate: rel-L2 <= 1e-13 * log2(N)."""
    return 1e-13 * max(1.0, float(np.log2(max(n_points, 2))))
