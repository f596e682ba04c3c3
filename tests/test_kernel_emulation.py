"""The pass kernels' own source, run on the CPU.  fft_pass.cuh and
fft_mixed.cuh are compiled with the host C++ compiler against a stand-in for
the CUDA names they use (tests/emu/cuda_runtime.h): each CTA runs as one
std::thread per CUDA thread, __syncthreads as a barrier, warp reductions as
barrier-based reductions, __shared__ arrays shared by the CTA's threads.  The
driver (tests/emu/emu_driver.cpp) transforms a few lines per case, in the
power-of-two kernel (16 and 4 points per thread) and the mixed-radix kernel,
for every arithmetic, with row and strided layouts, two-level and whole
four-step tables, inverse conjugation and scale, and double-float tiles that
take the 2^600 lift, and compares with a long-double DFT of the same lines.
This checks the kernels' index arithmetic and butterflies without a GPU; the
GPU tests check the compiled device code."""
import re
import subprocess

import pytest

from conftest import ROOT

CSRC = ROOT / "tope-fft_gb300" / "csrc"
EMU = ROOT / "tests" / "emu"
HEADERS = ["fft_pass.cuh", "fft_mixed.cuh", "fft_arith.cuh", "tfft_abi.h", "fft_mixed_consts.inc"]
NCASES = 12


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    d = tmp_path_factory.mktemp("emu")
    for h in HEADERS:
        src = (CSRC / h).read_text()
        # dynamic shared memory is the stand-in's static buffer; the launch
        # statements have no host meaning
        src = src.replace("extern __shared__", "extern")
        src = re.sub(r"^\s*\w+(<A>)?<<<.*>>>\(p\);\s*$", "    (void)0;", src, flags=re.M)
        (d / h).write_text(src)
    exe = d / "emu"
    subprocess.run(["g++", "-std=c++20", "-O1", "-pthread", f"-I{d}", f"-I{EMU}",
                    str(EMU / "emu_driver.cpp"), "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("case", range(NCASES))
def test_kernel_on_cpu(emu, case):
    r = subprocess.run([str(emu), str(case)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    m = re.search(r"rel=(\S+) tol=(\S+)", r.stdout)
    assert m, r.stdout
    rel, tol = float(m.group(1)), float(m.group(2))
    assert rel <= tol, r.stdout
