"""The double-float FP64 path's conversions on the CPU (no GPU needed).

tests/emu/split_join_driver.cpp compiles split_double and join_double from
tope-fft_gb300/csrc/fft_arith.cuh with the host compiler and checks them
against exact references: the split bit for bit against hi/lo built from
the FP64 value's bits, the join against the binary128 sum rounded once to
the nearest double, over 4 million pairs (normalised and unnormalised,
cancellation, powers of two with a remainder of the other sign, ties,
FP32-subnormal parts, zeros, FP64-subnormal and overflowing results), on
its fast path and its general one.
"""
import shutil
import subprocess

import pytest

from conftest import ROOT
from test_tc_split import host_headers


def test_split_and_join_exact(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "split_join"
    inc = host_headers(tmp_path)
    r = subprocess.run([cxx, "-std=c++20", "-pthread", "-O2", "-ffp-contract=off",
                        "-I", str(ROOT / "tests" / "emu"), "-I", str(inc),
                        str(ROOT / "tests" / "emu" / "split_join_driver.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0 and ("__float128" in r.stderr or "barrier" in r.stderr):
        pytest.skip("host compiler lacks __float128 or C++20 barriers")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0, out.stdout
    assert "FAIL" not in out.stdout
