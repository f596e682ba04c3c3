"""Builds host versions of the library's CUDA sources for the CPU tests: the
kernel launches are rewritten as calls of the host stand-ins in
tests/emu/cuda_runtime.h (emu_cta_launch for kernels that synchronise their
CTA, emu_launch for grid-stride kernels), and dynamic shared memory becomes a
static buffer."""
from __future__ import annotations

import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
CSRC = ROOT / "tope-fft_gb300" / "csrc"
INCLUDE = ROOT / "include"
EMU = Path(__file__).resolve().parent


def host_cxx_ok(tmp: Path) -> bool:
    """Can the host C++ compiler build the stand-in (C++20 <barrier>)?"""
    src = tmp / "probe.cpp"
    src.write_text("#include <barrier>\nint main() { std::barrier<> b(1); b.arrive_and_wait(); }\n")
    r = subprocess.run(["g++", "-std=c++20", "-pthread", str(src), "-o", str(tmp / "probe")],
                       capture_output=True, text=True)
    return r.returncode == 0


def split_top(s: str) -> list[str]:
    """Split a launch configuration at its top-level commas (brackets and
    template angle brackets nest; << and >> are shifts)."""
    parts, depth, cur, i = [], 0, "", 0
    while i < len(s):
        ch = s[i]
        if s.startswith("<<", i) or s.startswith(">>", i):
            cur += s[i:i + 2]
            i += 2
            continue
        depth += ch in "([<"
        depth -= ch in ")]>"
        if ch == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
        i += 1
    parts.append(cur.strip())
    return parts


def host_launches(src: str, fn: str) -> str:
    """name<<<grid, block, ...>>>(args) -> fn(dim3(grid), dim3(block), [=] { name(args); });
    the arguments are copied, so a launch recorded in a graph can run later"""
    out, i = [], 0
    while True:
        j = src.find("<<<", i)
        if j < 0:
            out.append(src[i:])
            return "".join(out)
        k = j
        while k > 0 and (src[k - 1].isalnum() or src[k - 1] in "_<>"):
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
        out.append(f"{fn}(dim3({cfg[0]}), dim3({cfg[1]}), [=] {{ {src[k:j]}({src[a0 + 1:a]}); }})")
        i = a + 1


ACQUIRE_ASM = 'asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");'


def host_source(name: str) -> str:
    src = (CSRC / name).read_text().replace("extern __shared__", "extern")
    # the batch kernel's acquire load, as a host atomic load
    src = src.replace(ACQUIRE_ASM, "v = __atomic_load_n(p, __ATOMIC_ACQUIRE);")
    fn = "emu_launch" if name == "fft_aux.cu" else "emu_cta_launch"
    return host_launches(src, fn)


def prepare(dst: Path, names: list[str]) -> None:
    """Copy the sources into dst as host C++ (kernel files) or unchanged."""
    dst.mkdir(parents=True, exist_ok=True)
    for name in names:
        text = host_source(name) if name.endswith((".cu", ".cuh")) else (CSRC / name).read_text()
        out = dst / (name[:-3] + ".cpp" if name.endswith(".cu") else name)
        out.write_text(text)


SANITIZE = ["-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
            "-fno-sanitize-recover=undefined"]


def sanitizer_ok(tmp: Path) -> bool:
    """Does the host compiler have the AddressSanitizer and UBSan runtimes?"""
    src = tmp / "probe_san.c"
    src.write_text("int main(void) { return 0; }\n")
    r = subprocess.run(["gcc", *SANITIZE, str(src), "-o", str(tmp / "probe_san")],
                       capture_output=True, text=True)
    return r.returncode == 0


def build_library(dst: Path, sanitize: bool = False) -> Path:
    """The library with every kernel on the host (tests/test_emulated_library.py):
    host code (topefft.c, batch.c), the auxiliary kernels, the pass dispatch,
    the mixed-radix and 4-points-per-thread kernels, and the power-of-two pass
    kernel for log2 L <= 8 in all four arithmetics (tests/emu/emu_launchers.cpp),
    and the persistent batch kernel with its graphs (one CTA, recorded launches).
    The tensor form and the allocation-free entry point are left out
    (tests/emu/emu_rest.cpp).  With sanitize, every object is built with
    AddressSanitizer and UBSan: device allocations are host heap blocks, so a
    kernel's global access outside its buffer, a host-code overrun and a
    buffer that Destroy does not free are all reported."""
    batch = ["fft_batch_host", "fft_batch_f64", "fft_batch_df64", "fft_batch_f32", "fft_batch_df32"]
    prepare(dst, ["fft_arith.cuh", "fft_pass.cuh", "fft_mixed.cuh", "fft_batch.cuh", "tfft_abi.h",
                  "fft_mixed_consts.inc", "topefft_internal.h", "fft_aux.cu", "fft_dispatch.cu",
                  "fft_inst_mixed.cu", "fft_inst_small.cu"] + [b + ".cu" for b in batch])
    san = SANITIZE if sanitize else []
    cxx = ["g++", "-std=c++20", "-O1", "-fPIC", "-pthread", *san, f"-I{EMU}", f"-I{dst}", f"-I{INCLUDE}"]
    cc = ["gcc", "-std=gnu11", "-O1", "-fPIC", *san, f"-I{dst}", f"-I{INCLUDE}"]
    jobs = [cc + ["-c", str(CSRC / "topefft.c"), "-o", str(dst / "topefft.o")],
            cc + ["-c", str(CSRC / "batch.c"), "-o", str(dst / "batch.o")]]
    for name in ["fft_aux", "fft_dispatch", "fft_inst_mixed", "fft_inst_small"] + batch:
        jobs.append(cxx + ["-c", str(dst / f"{name}.cpp"), "-o", str(dst / f"{name}.o")])
    for arith in range(4):
        jobs.append(cxx + [f"-DEMU_ARITH={arith}", "-c", str(EMU / "emu_launchers.cpp"),
                           "-o", str(dst / f"emu_launchers_{arith}.o")])
    jobs.append(cxx + ["-c", str(EMU / "emu_rest.cpp"), "-o", str(dst / "emu_rest.o")])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(run, jobs))
    lib = dst / "libtopefft_emu.so"
    objs = [str(p) for p in sorted(dst.glob("*.o"))]
    run(["g++", "-shared", "-pthread", *san, "-o", str(lib), *objs])
    return lib
