"""CPU oracle for the topeFFT C2C path - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
this package, and only as the checker (or, for the baseline, as the timed
CPU implementation of the reference's algorithm).  The library never does.

Two shared objects:
  liboracle.so          oracle/topefft_oracle.c: restatement of the
                        reference's algorithm + long-double FFT/DFT + the
                        SplitMix64 generator (built from committed sources).
  _ref/librefemu.so     the reference's own kernels (src/kernels{1,2,3}D.cl)
                        compiled as C++ and driven in its host order
                        (oracle/ref_build.sh); only present where the
                        reference tree was available at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_SO = HERE / "_ref" / "librefemu.so"

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


def build(force: bool = False) -> None:
    src = HERE / "topefft_oracle.c"
    if force or not ORACLE_SO.exists() or ORACLE_SO.stat().st_mtime < src.stat().st_mtime:
        tmp = ORACLE_SO.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                        str(src), "-o", str(tmp), "-lm"], check=True)
        os.replace(tmp, ORACLE_SO)


def build_ref() -> bool:
    """Build the reference-kernel emulator; False if the reference is unavailable."""
    r = subprocess.run(["sh", str(HERE / "ref_build.sh")], capture_output=True, text=True)
    if r.returncode == 3:
        return False
    if r.returncode != 0:
        raise RuntimeError("reference emulator build failed:\n" + r.stdout + r.stderr)
    return True


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    if a.dtype == np.float64:
        return a.ctypes.data_as(_D)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_I)
    raise TypeError(a.dtype)


class Oracle:
    """ctypes view of liboracle.so."""

    def __init__(self, path: Path = ORACLE_SO):
        if not path.exists():
            build()
        L = C.CDLL(str(path))
        L.oracle_splitmix64.restype = C.c_uint64
        L.oracle_splitmix64.argtypes = [C.c_uint64, C.c_uint64]
        for n in ("oracle_fill_uniform", "oracle_fill_normal"):
            getattr(L, n).argtypes = [_D, C.c_int64, C.c_uint64]
        L.oracle_radix.argtypes = [C.c_int]
        L.oracle_ilog2.argtypes = [C.c_int64]
        L.oracle_twiddle_table.argtypes = [C.c_int, _D]
        L.oracle_bitrev_table.argtypes = [C.c_int, _I]
        L.oracle_axis.argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.oracle_exec.argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_int]
        L.oracle_exec_n2.argtypes = [_D, C.c_int]
        L.oracle_dft_ref.argtypes = [_D, _D, C.c_int]
        L.oracle_fft_ld.argtypes = [_D, C.c_int64, C.c_int]
        L.oracle_fftnd_ld.argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_int]
        L.oracle_dft_ld.argtypes = [_D, _D, C.c_int, C.c_int]
        L.oracle_bluestein_ld.argtypes = [_D, _D, C.c_int64, C.c_int]
        for n in ("oracle_rel_l2", "oracle_max_abs"):
            getattr(L, n).restype = C.c_double
            getattr(L, n).argtypes = [_D, _D, C.c_int64]
        L.oracle_set_threads.argtypes = [C.c_int]
        self.lib = L

    # generators -----------------------------------------------------------
    def uniform(self, n_complex: int, seed: int) -> np.ndarray:
        a = np.empty(2 * n_complex)
        self.lib.oracle_fill_uniform(_ptr(a), n_complex, seed)
        return a

    def normal(self, n_complex: int, seed: int) -> np.ndarray:
        a = np.empty(2 * n_complex)
        self.lib.oracle_fill_normal(_ptr(a), n_complex, seed)
        return a

    # restatement of the reference ---------------------------------------
    def radix(self, log2n: int) -> int:
        return self.lib.oracle_radix(log2n)

    def twiddle_table(self, n: int) -> np.ndarray:
        a = np.empty(2 * max(n // 4, 1))
        self.lib.oracle_twiddle_table(n, _ptr(a))
        return a[: 2 * (n // 4)]

    def bitrev_table(self, log2n: int) -> np.ndarray:
        a = np.empty(1 << log2n, dtype=np.int32)
        self.lib.oracle_bitrev_table(log2n, _ptr(a))
        return a

    def exec(self, d: np.ndarray, nx: int, ny: int = 1, nz: int = 1, dir_: int = 1,
             batch: int = 1) -> np.ndarray:
        """Transform a copy of d in the reference's order; batch repeats 1D rows."""
        out = np.ascontiguousarray(d, dtype=np.float64).copy()
        if nx == 2 and ny == 1 and nz == 1:
            for b in range(batch):
                row = out[4 * b: 4 * b + 4].copy()
                self.lib.oracle_exec_n2(_ptr(row), dir_)
                out[4 * b: 4 * b + 4] = row
            return out
        if batch == 1:
            rc = self.lib.oracle_exec(_ptr(out), nx, ny, nz, dir_)
        else:  # a batch of 1D rows is a 2D array transformed along x only
            assert ny == 1 and nz == 1
            rc = 0
            self.lib.oracle_axis(_ptr(out), nx, batch, 1, 0, dir_)
            if dir_ == 0:
                out /= nx
        if rc:
            raise ValueError("size not supported by the reference algorithm")
        return out

    def dft_ref(self, d: np.ndarray, n: int) -> np.ndarray:
        out = np.empty(2 * n)
        self.lib.oracle_dft_ref(_ptr(np.ascontiguousarray(d)), _ptr(out), n)
        return out

    # long-double oracles ----------------------------------------------------
    def fft_ld(self, d: np.ndarray, nx: int, ny: int = 1, nz: int = 1, dir_: int = 1) -> np.ndarray:
        out = np.ascontiguousarray(d, dtype=np.float64).copy()
        if ny == 1 and nz == 1 and nx & (nx - 1):
            return self.dft_ld(out, nx, dir_)
        if ny == 1 and nz == 1:
            self.lib.oracle_fft_ld(_ptr(out), nx, dir_)
        else:
            self.lib.oracle_fftnd_ld(_ptr(out), nx, ny, nz, dir_)
        return out

    def dft_ld(self, d: np.ndarray, n: int, dir_: int = 1) -> np.ndarray:
        out = np.empty(2 * n)
        self.lib.oracle_dft_ld(_ptr(np.ascontiguousarray(d)), _ptr(out), n, dir_)
        return out

    def bluestein_ld(self, d: np.ndarray, n: int, dir_: int = 1) -> np.ndarray:
        out = np.empty(2 * n)
        self.lib.oracle_bluestein_ld(_ptr(np.ascontiguousarray(d)), _ptr(out), n, dir_)
        return out

    # metrics ------------------------------------------------------------------
    def rel_l2(self, a: np.ndarray, ref: np.ndarray) -> float:
        return self.lib.oracle_rel_l2(_ptr(np.ascontiguousarray(a)), _ptr(np.ascontiguousarray(ref)), a.size)

    def max_abs(self, a: np.ndarray, ref: np.ndarray) -> float:
        return self.lib.oracle_max_abs(_ptr(np.ascontiguousarray(a)), _ptr(np.ascontiguousarray(ref)), a.size)

    def set_threads(self, n: int) -> None:
        self.lib.oracle_set_threads(n)


class RefEmu:
    """ctypes view of _ref/librefemu.so (the reference's own kernels)."""

    def __init__(self, path: Path = REF_SO):
        if not path.exists():
            raise FileNotFoundError(path)
        L = C.CDLL(str(path))
        L.refemu_twiddles.argtypes = [C.c_int, _D]
        L.refemu_bitrev.argtypes = [C.c_int, _I]
        L.refemu_dft.argtypes = [_D, _D, C.c_int, C.c_int]
        L.refemu_exec_1d.argtypes = [_D, C.c_int, C.c_int]
        L.refemu_exec_2d.argtypes = [_D, C.c_int, C.c_int, C.c_int]
        L.refemu_exec_3d.argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_int]
        L.refemu_swap_3d.argtypes = [_D, C.c_int, C.c_int, C.c_int, C.c_int]
        L.refemu_set_threads.argtypes = [C.c_int]
        self.lib = L

    def exec(self, d: np.ndarray, nx: int, ny: int = 1, nz: int = 1, dir_: int = 1) -> np.ndarray:
        out = np.ascontiguousarray(d, dtype=np.float64).copy()
        if ny == 1 and nz == 1:
            rc = self.lib.refemu_exec_1d(_ptr(out), nx, dir_)
        elif nz == 1:
            rc = self.lib.refemu_exec_2d(_ptr(out), nx, ny, dir_)
        else:
            rc = self.lib.refemu_exec_3d(_ptr(out), nx, ny, nz, dir_)
        if rc:
            raise ValueError("size not supported by the reference kernels")
        return out

    def twiddles(self, n: int) -> np.ndarray:
        a = np.empty(2 * (n // 4))
        self.lib.refemu_twiddles(n, _ptr(a))
        return a

    def bitrev(self, log2n: int) -> np.ndarray:
        a = np.empty(1 << log2n, dtype=np.int32)
        self.lib.refemu_bitrev(log2n, _ptr(a))
        return a

    def dft(self, d: np.ndarray, n: int) -> np.ndarray:
        src = np.ascontiguousarray(d, dtype=np.float64).copy()
        out = np.empty(2 * n)
        self.lib.refemu_dft(_ptr(src), _ptr(out), n, 1)
        return out

    def swap_3d(self, d: np.ndarray, x: int, y: int, z: int, type_: int) -> np.ndarray:
        out = np.ascontiguousarray(d, dtype=np.float64).copy()
        if self.lib.refemu_swap_3d(_ptr(out), x, y, z, type_):
            raise ValueError("bad size")
        return out

    def set_threads(self, n: int) -> None:
        self.lib.refemu_set_threads(n)


def rel_l2(a: np.ndarray, ref: np.ndarray) -> float:
    """rel-L2 in extended precision via numpy (no library needed)."""
    a = np.asarray(a, dtype=np.longdouble)
    r = np.asarray(ref, dtype=np.longdouble)
    den = np.sqrt(np.sum(r * r))
    num = np.sqrt(np.sum((a - r) ** 2))
    return float(num / den) if den > 0 else float(num)
