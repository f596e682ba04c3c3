"""Build the library (libtopefft.so) in-tree.

libtopefft.so: the C host library (csrc/*.c, gcc) plus the CUDA kernels
(csrc/*.cu, nvcc for sm_103a only), linked with the static CUDA runtime.
Translation units compile in parallel; outputs go to _build/ and the
package directory.  Nothing here needs torch.  (The CPU oracle, test
infrastructure, is built by oracle.build(), not here.)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libtopefft.so"
INCLUDE = ROOT / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    steps = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            steps.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                          f"-I{CSRC}", f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.c")):
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            steps.append(["gcc", "-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wno-unused-function",
                          f"-I{CSRC}", f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)])
    jobs = jobs or max(2, os.cpu_count() or 2)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in steps]:
            if verbose:
                print(" ".join(cmd[:1] + cmd[-3:]), file=sys.stderr)
            fut.result()
    if steps or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
