"""The tensor form's stage arithmetic on the CPU (no GPU needed).

tests/emu/tc_split_driver.cpp compiles the same split and matrix functions
the tcgen05 kernel uses (tope-fft_gb300/csrc/fft_tc_split.cuh) with the host
compiler and forms the tensor cores' products itself: FP16 operands
(_Float16), the leading-piece accumulator summed exactly, the cross-product
accumulator summed in FP32.  It checks the properties the kernel relies on:
  - the B matrices B0..B4 are exact FP16 values with no subnormals, and the
    three pieces of F represent the DFT-16 within 2^-33;
  - x0 and x1 are FP16 integers, |x0| <= 513, |x1| <= 2048;
  - the leading accumulator is an integer sum below 2^24 (exact in FP32 in
    any summation order);
  - one stage's error per 16-point row, plain and twiddled, over 20,000 rows
    (uniform, 60-octave dynamic range, a 1e6 spike, 1e-30 values, zeros),
    below 2e-9 rel-L2 against a long-double DFT-16;
  - whole lines of 2^8 .. 2^12 points through the kernel's Stockham stages
    (its first stage of radix 2/4/8 through the pass code's double-float
    butterflies, then the renormalising read), uniform, with a 1e6 pulse,
    and a pure tone whose first-stage sums cancel exactly, below 1e-8 rel-L2
    before the FP32 store.
The GPU tests (test_gpu_f32.py) check the compiled kernel end to end.
"""
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

CSRC = ROOT / "tope-fft_gb300" / "csrc"
HEADERS = ["fft_pass.cuh", "fft_arith.cuh", "fft_tc_split.cuh", "tfft_abi.h"]


def host_headers(d):
    """The kernel headers as the host compiler takes them (as the kernel
    emulation does): extern __shared__ arrays become plain externs and
    kernel launches are dropped."""
    for h in HEADERS:
        src = (CSRC / h).read_text()
        src = src.replace("extern __shared__", "extern")
        src = re.sub(r"^\s*\w+(<A>)?<<<.*>>>\(p\);\s*$", "    (void)0;", src, flags=re.M)
        (d / h).write_text(src)
    return d


def test_tensor_stage_arithmetic(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "tc_split"
    inc = host_headers(tmp_path)
    r = subprocess.run([cxx, "-std=c++20", "-pthread", "-O2", "-ffp-contract=off",
                        "-I", str(ROOT / "tests" / "emu"), "-I", str(inc),
                        str(ROOT / "tests" / "emu" / "tc_split_driver.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0 and ("_Float16" in r.stderr or "barrier" in r.stderr):
        pytest.skip("host compiler lacks _Float16 or C++20 barriers")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0, out.stdout
    assert "FAIL" not in out.stdout
