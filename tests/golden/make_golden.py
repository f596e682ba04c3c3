"""Generate tests/golden/reference_golden.npz from the reference's own kernels.

The reference (matze/tope-fft) ships no golden vectors or known-answer
tests: its test drivers only print timings (test/1d.c:140-143).  These
fixtures are outputs of the reference's OpenCL kernel source
(src/kernels{1,2,3}D.cl) compiled as C++ and run in the reference's host
order by oracle/_ref/librefemu.so (built by oracle/ref_build.sh from the
reference tree).  Inputs are regenerated from their seeds by the SplitMix64
generator (oracle_fill_uniform), whose first values are stored too so the
generator itself is pinned.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle  # noqa: E402

SEED0 = 0x70E0F0F7
OUT = Path(__file__).resolve().parent / "reference_golden.npz"


def main() -> None:
    oracle.build()
    if not oracle.build_ref():
        raise SystemExit("reference tree unavailable: cannot generate golden vectors")
    orc, ref = oracle.Oracle(), oracle.RefEmu()
    ref.set_threads(1)
    g: dict[str, np.ndarray] = {}
    # generator pin: first 64 uniform and normal values for seed SEED0
    g["gen_uniform"] = orc.uniform(32, SEED0)
    g["gen_normal"] = orc.normal(32, SEED0)
    cases = []
    # 1D powers of two (radix 4, 8, 2 plans) and the two-point host path
    for n in (2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 4096):
        cases.append((n, 1, 1))
    for shape in ((4, 4, 1), (8, 4, 1), (4, 8, 1), (16, 32, 1), (64, 16, 1), (32, 32, 1),
                  (4, 4, 4), (8, 16, 32), (16, 4, 64), (4, 8, 16)):
        cases.append(shape)
    for idx, (nx, ny, nz) in enumerate(cases):
        n = nx * ny * nz
        seed = SEED0 + 1000 + idx
        x = orc.uniform(n, seed)
        key = f"{nx}x{ny}x{nz}"
        g[f"seed_{key}"] = np.array([seed], dtype=np.uint64)
        g[f"fwd_{key}"] = ref.exec(x, nx, ny, nz, 1)
        g[f"inv_{key}"] = ref.exec(x, nx, ny, nz, 0)
    # the reference drivers' own inputs: ramp i+1 (test/1d.c:69-71) and
    # sin(2 pi count / N) on the real part (test/2d.c:75-80, test/3d.c:76-83)
    for n in (8, 64, 1024):
        x = np.zeros(2 * n)
        x[0::2] = np.arange(1, n + 1)
        g[f"ramp_fwd_{n}"] = ref.exec(x, n, 1, 1, 1)
    for (nx, ny, nz) in ((16, 8, 1), (8, 8, 4)):
        n = nx * ny * nz
        x = np.zeros(2 * n)
        x[0::2] = np.sin(2 * np.pi * np.arange(n) / n)
        g[f"sin_fwd_{nx}x{ny}x{nz}"] = ref.exec(x, nx, ny, nz, 1)
    # non-power-of-two lengths: the reference's DFT kernel (forward only)
    for n in (3, 5, 6, 7, 11, 12, 13, 27, 100, 1000, 1001):
        seed = SEED0 + 2000 + n
        x = orc.uniform(n, seed)
        g[f"dftseed_{n}"] = np.array([seed], dtype=np.uint64)
        g[f"dft_{n}"] = ref.dft(x, n)
    # plan tables: quarter-wave twiddles and bit-reversal indices
    for n in (8, 16, 64, 256, 4096):
        g[f"twiddle_{n}"] = ref.twiddles(n)
    for lg in range(1, 15):
        g[f"bitrev_{lg}"] = ref.bitrev(lg)
    # the swap (bit-reversal permutation) pass on a 3D array, each axis
    x = orc.uniform(8 * 16 * 4, SEED0 + 3000)
    for ax in (1, 2, 3):
        g[f"swap3d_8x16x4_type{ax}"] = ref.swap_3d(x, 8, 16, 4, ax)
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(g)} arrays)")


if __name__ == "__main__":
    main()
