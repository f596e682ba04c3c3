"""The pass kernels' own source, run on the CPU.  fft_pass.cuh and
fft_mixed.cuh are compiled with the host C++ compiler against a stand-in for
the CUDA names they use (tests/emu/cuda_runtime.h): each CTA runs as one
std::thread per CUDA thread, __syncthreads as a barrier, warp reductions as
barrier-based reductions, __shared__ arrays shared by the CTA's threads.  The
driver (tests/emu/emu_driver.cpp) transforms a few lines per case, in the
power-of-two kernel (16 and 4 points per thread) and the mixed-radix kernel,
for every arithmetic, with row and strided layouts, two-level and whole
four-step tables indexed by the line or (the middle pass of a three-pass
line) by the group along the grid's second dimension, inverse conjugation
and scale, and double-float tiles that
take the 2^600 lift, and compares with a long-double DFT of the same lines.
This checks the kernels' index arithmetic and butterflies without a GPU; the
GPU tests check the compiled device code.

The auxiliary kernels' file (fft_aux.cu: twiddle and four-step tables,
real-data steps, Bluestein pieces, the exact-index DFT) runs the same way,
its launches rewritten as a loop over the grid's threads (those kernels use
neither shared memory nor barriers) and its runtime calls on host memory,
through the library's own tfft_* entry points (tests/emu/aux_driver.cpp);
sincospi is a long-double stand-in, so these cases check the angle
reductions and indexing, not the device's sincospi."""
import re
import subprocess

import pytest

from conftest import ROOT

CSRC = ROOT / "tope-fft_gb300" / "csrc"
EMU = ROOT / "tests" / "emu"
HEADERS = ["fft_pass.cuh", "fft_mixed.cuh", "fft_arith.cuh", "tfft_abi.h", "fft_mixed_consts.inc"]
NCASES = 17
NAUX = 7


def split_top(s):
    """Split a launch configuration at its top-level commas."""
    parts, depth, cur = [], 0, ""
    for ch in s:
        depth += ch in "(["
        depth -= ch in ")]"
        if ch == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
    parts.append(cur.strip())
    return parts


def host_launches(src):
    """name<<<grid, block, ...>>>(args) -> emu_launch(dim3(grid), dim3(block), ...)"""
    out, i = [], 0
    while True:
        j = src.find("<<<", i)
        if j < 0:
            out.append(src[i:])
            return "".join(out)
        k = j
        while k > 0 and (src[k - 1].isalnum() or src[k - 1] == "_"):
            k -= 1
        e = src.find(">>>", j)
        cfg = split_top(src[j + 3:e])
        a0 = e + 3
        while src[a0].isspace():
            a0 += 1
        depth, a = 0, a0
        while True:
            depth += src[a] == "("
            depth -= src[a] == ")"
            if depth == 0:
                break
            a += 1
        out.append(src[i:k])
        out.append(f"emu_launch(dim3({cfg[0]}), dim3({cfg[1]}), [&] {{ {src[k:j]}({src[a0 + 1:a]}); }})")
        i = a + 1


def cxx20_ok(d):
    src = d / "probe.cpp"
    src.write_text("#include <barrier>\nint main() { std::barrier<> b(1); b.arrive_and_wait(); }\n")
    return subprocess.run(["g++", "-std=c++20", "-pthread", str(src), "-o", str(d / "probe")],
                          capture_output=True).returncode == 0


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    d = tmp_path_factory.mktemp("emu")
    if not cxx20_ok(d):
        pytest.skip("no C++20 host compiler (std::barrier)")
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


@pytest.fixture(scope="module")
def emu_san(tmp_path_factory, emu):
    """The same driver under AddressSanitizer and UndefinedBehaviorSanitizer:
    the part of the shared-memory buffer beyond each launch's dynamic size is
    poisoned, so an access outside the launch's allocation is an error."""
    d = emu.parent
    exe = d / "emu_san"
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-g", "-pthread",
                        "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                        f"-I{d}", f"-I{EMU}", str(EMU / "emu_driver.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode:
        pytest.skip("no sanitizer runtime for the host compiler")
    return exe


@pytest.mark.parametrize("case", [0, 2, 3, 4, 5, 6, 7, 9, 10, 12, 14])
def test_kernel_under_sanitizers(emu_san, case):
    r = subprocess.run([str(emu_san), str(case)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "runtime error" not in r.stderr, r.stderr[-2000:]
    m = re.search(r"rel=(\S+) tol=(\S+)", r.stdout)
    assert m and float(m.group(1)) <= float(m.group(2)), r.stdout


@pytest.mark.parametrize("case", range(NCASES))
def test_kernel_on_cpu(emu, case):
    r = subprocess.run([str(emu), str(case)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    m = re.search(r"rel=(\S+) tol=(\S+)", r.stdout)
    assert m, r.stdout
    rel, tol = float(m.group(1)), float(m.group(2))
    assert rel <= tol, r.stdout


@pytest.fixture(scope="module")
def aux(tmp_path_factory):
    d = tmp_path_factory.mktemp("aux")
    if not cxx20_ok(d):
        pytest.skip("no C++20 host compiler (std::barrier)")
    for h in ("fft_arith.cuh", "tfft_abi.h"):
        (d / h).write_text((CSRC / h).read_text())
    (d / "fft_aux.cpp").write_text(host_launches((CSRC / "fft_aux.cu").read_text()))
    exe = d / "aux"
    subprocess.run(["g++", "-std=c++20", "-O1", "-pthread", f"-I{EMU}", f"-I{d}",
                    str(d / "fft_aux.cpp"), str(EMU / "aux_driver.cpp"), "-o", str(exe)],
                   check=True)
    return exe


@pytest.mark.parametrize("case", range(NAUX))
def test_aux_kernel_on_cpu(aux, case):
    r = subprocess.run([str(aux), str(case)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    m = re.search(r"err=(\S+) tol=(\S+)", r.stdout)
    assert m, r.stdout
    assert float(m.group(1)) <= float(m.group(2)), r.stdout
