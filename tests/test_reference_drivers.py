"""The reference's own benchmark drivers, unchanged, against this library.

test/1d.c, test/2d.c and test/3d.c of the reference include
"../src/topefft.h" (test/1d.c:14-17), call topeFFTInit and
tope{1,2,3}D{PlanInit,Exec,Destroy} with C2C/FORWARD/INVERSE, and read
plan.totalKernel and plan.totalPreKernel (test/1d.c:74-90, 140-143).  This
test copies the three files, byte for byte, from the reference checkout into
a scratch tree whose src/topefft.h is one line including this repository's
include/topefft.h, compiles them with the CUDA toolkit's own headers for
their cuFFT column and a test-only FFTW stand-in (tests/drivers/stubs) for
their FFTW column, and links them against libtopefft.so (and cuFFT).  That
is the drop-in claim: a caller of the reference builds against this library
without editing its source.

The reference checkout is read where it lies (TOPEFFT_REFERENCE, else a
directory named "reference" beside this repository); the test skips where it
is absent.  No GPU is needed (nothing is run).
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def reference_dir():
    p = Path(os.environ.get("TOPEFFT_REFERENCE", ROOT.parent / "reference"))
    return p if (p / "test" / "1d.c").exists() else None


@pytest.fixture(scope="module")
def tree(tmp_path_factory):
    ref = reference_dir()
    if ref is None:
        pytest.skip("reference checkout not present")
    if shutil.which("gcc") is None or not (CUDA / "include" / "cufft.h").exists():
        pytest.skip("gcc or the CUDA toolkit's cuFFT header missing")
    t = tmp_path_factory.mktemp("refdrivers")
    (t / "src").mkdir()
    (t / "test").mkdir()
    (t / "src" / "topefft.h").write_text(f'#include "{ROOT / "include" / "topefft.h"}"\n')
    for name in ("1d.c", "2d.c", "3d.c"):
        data = (ref / "test" / name).read_bytes()
        (t / "test" / name).write_bytes(data)
        assert (t / "test" / name).read_bytes() == data
    return t


def compile_args(tree, name):
    stubs = ROOT / "tests" / "drivers" / "stubs"
    return ["gcc", "-std=gnu11", "-Wall", "-Werror=implicit-function-declaration",
            "-Werror=incompatible-pointer-types", "-Wno-unused-variable",
            "-Wno-unused-but-set-variable", "-Wno-unused-function",
            "-I", str(stubs), "-I", str(CUDA / "include"), str(tree / "test" / name)]


@pytest.mark.parametrize("name", ["1d.c", "2d.c", "3d.c"])
def test_reference_driver_compiles_unchanged(tree, name):
    r = subprocess.run(compile_args(tree, name) + ["-c", "-o", str(tree / (name + ".o"))],
                       capture_output=True, text=True, cwd=tree / "test")
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("name", ["1d.c", "2d.c", "3d.c"])
def test_reference_driver_links_against_library(T, tree, name):
    lib = ROOT / "tope-fft_gb300" / "libtopefft.so"
    cufft = CUDA / "lib64" / "libcufft.so"
    if not lib.exists() or not cufft.exists():
        pytest.skip("libtopefft.so or libcufft.so not built/installed")
    stubs = ROOT / "tests" / "drivers" / "stubs"
    exe = tree / name.replace(".c", "")
    r = subprocess.run(compile_args(tree, name) + [
        str(stubs / "fftw_stub.c"), "-o", str(exe),
        "-L", str(lib.parent), "-ltopefft", f"-Wl,-rpath,{lib.parent}",
        "-L", str(CUDA / "lib64"), "-lcufft", "-lcudart", f"-Wl,-rpath,{CUDA / 'lib64'}", "-lm"],
        capture_output=True, text=True, cwd=tree / "test")
    assert r.returncode == 0, r.stderr
    assert exe.exists()
