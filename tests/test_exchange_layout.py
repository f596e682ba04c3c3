"""The pass kernel's shared-memory exchange layout against a bank model (no
GPU needed).

tests/emu/exchange_banks_driver.cpp compiles the kernel's own index function
(sidx in tope-fft_gb300/csrc/fft_pass.cuh) with the host compiler, replays
every Stockham stage's shared-memory reads and writes for each warp of every
tile shape the kernels use (8- and 16-byte elements, lines of 2^5 .. 2^13
points, tiles of 1 .. 32 lines), and requires each request to take the
minimum number of wavefronts (no bank conflicts), and the layout to be a
one-to-one map into the exchange buffer.
"""
import shutil
import subprocess

import pytest

from conftest import ROOT
from test_tc_split import host_headers


def test_exchange_layout_conflict_free(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "exchange_banks"
    inc = host_headers(tmp_path)
    r = subprocess.run([cxx, "-std=c++20", "-pthread", "-O2",
                        "-I", str(ROOT / "tests" / "emu"), "-I", str(inc),
                        str(ROOT / "tests" / "emu" / "exchange_banks_driver.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0 and "barrier" in r.stderr:
        pytest.skip("host compiler lacks C++20 barriers")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0, out.stdout
    assert "FAIL" not in out.stdout
