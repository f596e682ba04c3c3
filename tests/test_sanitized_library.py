"""The host build of the whole library (tests/emu/emu_build.py) under
AddressSanitizer, LeakSanitizer and UBSan, driven by two C callers:

- tests/drivers/tope_driver.c: the reference drivers' sequence (test/1d.c,
  test/2d.c, test/3d.c): PlanInit, Exec forward and inverse, Destroy;
- tests/drivers/ext_driver.c: the whole public surface in one process.
  That covers batched, real-data, FP32 split-precision, device-resident and
  uneven-batch plans, the pass timing and geometry queries, the bit-reversal
  permutation and the refused requests, with several plans alive at once.

In the host build every device allocation is a host heap block and every
kernel runs on the CPU.  So a kernel's global access outside its buffer, a
host-code overrun or undefined operation, and a buffer that a Destroy (or a
refused PlanInit) leaves allocated each end the run with a sanitizer report.

The emulated-library tests can also run against this build:
    LD_PRELOAD=$(gcc -print-file-name=libasan.so):$(gcc -print-file-name=libubsan.so) \\
    ASAN_OPTIONS=detect_leaks=0 python -m pytest tests/test_emulated_library.py --emu-sanitize
(leak checks are off there because the Python interpreter itself keeps
allocations until exit)."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

from conftest import ROOT

sys.path.insert(0, str(Path(__file__).resolve().parent / "emu"))
import emu_build  # noqa: E402

INCLUDE = ROOT / "include"
DRIVERS = ROOT / "tests" / "drivers"


@pytest.fixture(scope="module")
def san_lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("sanlib")
    if not emu_build.host_cxx_ok(d):
        pytest.skip("no C++20 host compiler (std::barrier)")
    if not emu_build.sanitizer_ok(d):
        pytest.skip("no sanitizer runtime for the host compiler")
    return emu_build.build_library(d, sanitize=True)


def build_driver(lib: Path, name: str) -> Path:
    exe = lib.parent / name
    subprocess.run(["gcc", "-std=gnu11", "-O1", *emu_build.SANITIZE, "-Wall", "-Werror",
                    f"-I{INCLUDE}", str(DRIVERS / f"{name}.c"), "-o", str(exe),
                    f"-L{lib.parent}", "-ltopefft_emu", f"-Wl,-rpath,{lib.parent}", "-lm"],
                   check=True)
    return exe


def run_sanitized(cmd, timeout=900):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1")
    env.pop("LD_PRELOAD", None)
    return subprocess.run([str(c) for c in cmd], capture_output=True, text=True, timeout=timeout,
                          env=env)


def test_whole_surface_under_sanitizers(san_lib):
    exe = build_driver(san_lib, "ext_driver")
    r = run_sanitized([exe])
    assert r.returncode == 0, (r.stdout + r.stderr)[-4000:]
    assert "Sanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-4000:]
    assert r.stdout.startswith("ok "), r.stdout


@pytest.mark.parametrize("shape", [["1000"], ["60", "40"]], ids=lambda s: "x".join(s))
def test_reference_driver_under_sanitizers(san_lib, shape):
    exe = san_lib.parent / "tope_driver"
    if not exe.exists():
        build_driver(san_lib, "tope_driver")
    r = run_sanitized([exe, *shape], timeout=300)
    assert r.returncode == 0, (r.stdout + r.stderr)[-4000:]
    assert "Sanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-4000:]
