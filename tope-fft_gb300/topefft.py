"""Python mirror of the topeFFT C interface, over libtopefft.so (ctypes).

The functions keep the reference's names and argument meaning
(src/topefft.h, src/util.c:21, src/fft1d.c:12/303/372, src/fft2d.c:136/319/442,
src/fft3d.c:216/474/628) so tests read like the reference's own drivers
(test/1d.c:74-90):

    f = TopeFFT(); topeFFTInit(f)
    t = TopePlan1D(); tope1DPlanInit(f, t, n, C2C, data)
    tope1DExec(f, t, data, FORWARD)
    tope1DDestroy(f, t)

`data` is a C-contiguous float64 numpy array of 2*points values (re, im
interleaved, x fastest).  There is no fallback: if libtopefft.so is missing
the import fails.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

C2C, R2C = 1, 0
FORWARD, INVERSE = 1, 0

TOPE_SUCCESS = 0
TOPE_ERR_INVALID_SIZE = 1
TOPE_ERR_INVALID_ARG = 2
TOPE_ERR_ALLOC = 3
TOPE_ERR_CUDA = 4
TOPE_ERR_NOT_INITIALIZED = 5
TOPE_ERR_DESTROYED = 6
TOPE_ERR_UNSUPPORTED = 7
TOPE_ERR_TIMEOUT = 8
TOPE_ARITH_FP64, TOPE_ARITH_DF64 = 0, 1
TOPE_SPLIT_ACCURATE, TOPE_SPLIT_FAST, TOPE_SPLIT_TENSOR = 0, 1, 2

LIB_PATH = Path(__file__).resolve().parent / "libtopefft.so"

_vp = C.c_void_p
_u64 = C.c_uint64


class TopeFFT(C.Structure):
    _fields_ = [("error", C.c_int), ("event", _vp), ("platform_id", _vp), ("device", _vp),
                ("program1D", _vp), ("program2D", _vp), ("program3D", _vp), ("context", _vp),
                ("command_queue", _vp), ("ret_num_platforms", C.c_uint),
                ("ret_num_devices", C.c_uint), ("device_ordinal", C.c_int), ("arith", C.c_int),
                ("live_plans", C.c_int), ("pass_timing", C.c_int), ("split_mode", C.c_int)]


class TopePlan1D(C.Structure):
    _fields_ = [("x", C.c_int), ("log", C.c_int), ("type", C.c_int), ("radix", C.c_int),
                ("kernel", _vp), ("kernel_bit", _vp), ("kernel_swap", _vp),
                ("kernel_twid", _vp), ("kernel_div", _vp), ("data", _vp), ("bitrev", _vp),
                ("twiddle", _vp), ("scratch", _vp), ("dataSize", C.c_size_t),
                ("totalMemory", _u64), ("totalPreKernel", _u64), ("totalKernel", _u64),
                ("dim", C.c_uint), ("globalSize", _vp), ("localSize", _vp), ("impl", _vp)]


class TopePlan2D(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("logX", C.c_int), ("logY", C.c_int),
                ("type", C.c_int), ("radX", C.c_int), ("radY", C.c_int), ("kernelX", _vp),
                ("kernelY", _vp), ("kernel_bit", _vp), ("kernel_swap", _vp),
                ("kernel_twid", _vp), ("kernel_div", _vp), ("data", _vp), ("bitX", _vp),
                ("bitY", _vp), ("twdX", _vp), ("twdY", _vp), ("dataSize", C.c_size_t),
                ("totalMemory", _u64), ("totalPreKernel", _u64), ("totalKernel", _u64),
                ("dim", C.c_uint), ("globalSize", _vp), ("localSize", _vp), ("impl", _vp)]


class TopePlan3D(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int), ("logX", C.c_int),
                ("logY", C.c_int), ("logZ", C.c_int), ("type", C.c_int), ("radX", C.c_int),
                ("radY", C.c_int), ("radZ", C.c_int), ("kernelX", _vp), ("kernelY", _vp),
                ("kernelZ", _vp), ("kernel_bit", _vp), ("kernel_swap", _vp),
                ("kernel_twid", _vp), ("kernel_div", _vp), ("data", _vp), ("bitX", _vp),
                ("bitY", _vp), ("bitZ", _vp), ("twdX", _vp), ("twdY", _vp), ("twdZ", _vp),
                ("dataSize", C.c_size_t), ("totalMemory", _u64), ("totalPreKernel", _u64),
                ("totalKernel", _u64), ("dim", C.c_uint), ("globalSize", _vp),
                ("localSize", _vp), ("impl", _vp)]


class TopeBatch(C.Structure):
    _fields_ = [("count", C.c_int), ("type", C.c_int), ("dataSize", C.c_size_t),
                ("totalMemory", _u64), ("totalPreKernel", _u64), ("totalKernel", _u64),
                ("data", _vp), ("mode", C.c_int), ("elem_bytes", C.c_int), ("classes", C.c_int),
                ("ctas", C.c_int), ("work_items", C.c_int64), ("impl", _vp)]


TOPE_BATCH_PERSISTENT, TOPE_BATCH_LAUNCHES, TOPE_BATCH_LOOP = 0, 1, 2

_F = C.POINTER(TopeFFT)
_PB = C.POINTER(TopeBatch)
_IP = C.POINTER(C.c_int)
_P1, _P2, _P3 = C.POINTER(TopePlan1D), C.POINTER(TopePlan2D), C.POINTER(TopePlan3D)
_D = C.POINTER(C.c_double)
_FL = C.POINTER(C.c_float)

# (name, restype, argtypes) of every exported entry point of include/topefft.h
# and include/topefft_ext.h
SIGNATURES = [
    ("profileThis", _u64, [_vp]),
    ("topeFFTInit", None, [_F]),
    ("tope1DPlanInit", None, [_F, _P1, C.c_int, C.c_int, _D]),
    ("tope1DExec", None, [_F, _P1, _D, C.c_int]),
    ("tope1DDestroy", None, [_F, _P1]),
    ("tope2DPlanInit", None, [_F, _P2, C.c_int, C.c_int, C.c_int, _D]),
    ("tope2DExec", None, [_F, _P2, _D, C.c_int]),
    ("tope2DExecX", None, [_F, _P2]),
    ("tope2DExecY", None, [_F, _P2]),
    ("tope2DDestroy", None, [_F, _P2]),
    ("tope3DPlanInit", None, [_F, _P3, C.c_int, C.c_int, C.c_int, C.c_int, _D]),
    ("tope3DExec", None, [_F, _P3, _D, C.c_int]),
    ("tope3DExecX", None, [_F, _P3]),
    ("tope3DExecY", None, [_F, _P3]),
    ("tope3DExecZ", None, [_F, _P3]),
    ("tope3DDestroy", None, [_F, _P3]),
    ("topeGetLastError", C.c_int, []),
    ("topePeekLastError", C.c_int, []),
    ("topeErrorString", C.c_char_p, [C.c_int]),
    ("topeLastCudaError", C.c_int, []),
    ("topeSetArith", None, [_F, C.c_int]),
    ("topeFFTDestroy", None, [_F]),
    ("tope1DExecDevice", None, [_F, _P1, C.c_int]),
    ("tope2DExecDevice", None, [_F, _P2, C.c_int]),
    ("tope3DExecDevice", None, [_F, _P3, C.c_int]),
    ("tope1DUpload", None, [_F, _P1, _D]),
    ("tope1DDownload", None, [_F, _P1, _D]),
    ("tope1DUploadSpectrum", None, [_F, _P1, _D]),
    ("tope2DUploadSpectrum", None, [_F, _P2, _D]),
    ("tope3DUploadSpectrum", None, [_F, _P3, _D]),
    ("tope2DUpload", None, [_F, _P2, _D]),
    ("tope2DDownload", None, [_F, _P2, _D]),
    ("tope3DUpload", None, [_F, _P3, _D]),
    ("tope3DDownload", None, [_F, _P3, _D]),
    ("topeSync", None, [_F]),
    ("tope1DBatchPlanInit", None, [_F, _P1, C.c_int, C.c_int, C.c_int, _D]),
    ("topeCopyToHost", None, [_F, _vp, _vp, C.c_size_t]),
    ("tope3DBitrevPermute", None, [_F, _P3, C.c_int]),
    ("topeHostAlloc", _vp, [C.c_size_t]),
    ("topeHostFree", None, [_vp]),
    ("topeSetPassTiming", None, [_F, C.c_int]),
    ("topePassTimes", C.c_int, [_F, _vp, C.POINTER(_u64), C.POINTER(_u64), C.c_int]),
    ("topeResetPassTimes", None, [_F, _vp]),
    ("topePassInfo", C.c_int, [_F, _vp, C.c_int, C.POINTER(C.c_int64)]),
    ("topeExec1DNoAlloc", C.c_int, [_vp, _vp, C.c_int, C.c_int, _vp]),
    ("tope1DBatchPlanInitF32", None, [_F, _P1, C.c_int, C.c_int, C.c_int, _FL]),
    ("tope2DPlanInitF32", None, [_F, _P2, C.c_int, C.c_int, C.c_int, _FL]),
    ("tope3DPlanInitF32", None, [_F, _P3, C.c_int, C.c_int, C.c_int, C.c_int, _FL]),
    ("tope1DExecF32", None, [_F, _P1, _FL, C.c_int]),
    ("tope2DExecF32", None, [_F, _P2, _FL, C.c_int]),
    ("tope3DExecF32", None, [_F, _P3, _FL, C.c_int]),
    ("topeUploadF32", None, [_F, _vp, _FL]),
    ("topeDownloadF32", None, [_F, _vp, _FL]),
    ("topeUploadSpectrumF32", None, [_F, _vp, _FL]),
    ("topeSetSplitMode", None, [_F, C.c_int]),
    ("topeBatchPlanInit", None, [_F, _PB, C.c_int, _IP, _IP, C.c_int, _D]),
    ("topeBatchPlanInitF32", None, [_F, _PB, C.c_int, _IP, _IP, C.c_int, _FL]),
    ("topeBatchExec", None, [_F, _PB, _D, C.c_int]),
    ("topeBatchExecF32", None, [_F, _PB, _FL, C.c_int]),
    ("topeBatchExecDevice", None, [_F, _PB, C.c_int]),
    ("topeBatchUpload", None, [_F, _PB, _vp]),
    ("topeBatchDownload", None, [_F, _PB, _vp]),
    ("topeBatchSetMode", None, [_F, _PB, C.c_int]),
    ("topeBatchDestroy", None, [_F, _PB]),
]


def load_library(path: Path | str = LIB_PATH) -> C.CDLL:
    path = Path(path)
    if not path.exists():
        raise ImportError(f"{path} is missing: build it first (__graft_entry__.build())")
    lib = C.CDLL(str(path))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = load_library()


def _ptr(d):
    if d is None:
        return None
    if isinstance(d, np.ndarray):
        if d.dtype != np.float64 or not d.flags.c_contiguous:
            raise TypeError("data must be a C-contiguous float64 array")
        return d.ctypes.data_as(_D)
    if isinstance(d, int):  # raw host address (pinned buffers)
        return C.cast(d, _D)
    raise TypeError("unsupported data argument")


def _need(d, x, rows, type_) -> None:
    """A host array handed to a PlanInit must hold the data the library
    uploads: 2 x doubles per row for C2C, x reals per row for R2C."""
    if isinstance(d, np.ndarray):
        want = (x if type_ == R2C else 2 * x) * rows
        if d.size < want:
            raise ValueError(f"data holds {d.size} values, the plan reads {want}")


def _need_out(d, t, dir_) -> None:
    """A host array handed to an Exec receives what the transform writes:
    the plan's dataSize bytes, or for a real-data plan's forward transform
    its spectrum, (x + 2)/x times the reals.  Checked only for numpy arrays
    and live plans (the library reports the rest with a status)."""
    if not isinstance(d, np.ndarray) or not t.impl or not t.dataSize:
        return
    want = t.dataSize
    if t.type == R2C and dir_ == FORWARD and t.x > 0:
        want = t.dataSize // t.x * (t.x + 2)
    if d.nbytes < want:
        raise ValueError(f"data holds {d.nbytes} bytes, the transform writes {want}")


def topeFFTInit(f: TopeFFT) -> None:
    lib.topeFFTInit(C.byref(f))


def topeFFTDestroy(f: TopeFFT) -> None:
    lib.topeFFTDestroy(C.byref(f))


def topeSetArith(f: TopeFFT, arith: int) -> None:
    lib.topeSetArith(C.byref(f), arith)


def topeSetSplitMode(f: TopeFFT, mode: int) -> None:
    lib.topeSetSplitMode(C.byref(f), mode)


def topeSetPassTiming(f: TopeFFT, enable: int) -> None:
    lib.topeSetPassTiming(C.byref(f), int(enable))


def topeResetPassTimes(f: TopeFFT, t) -> None:
    lib.topeResetPassTimes(C.byref(f), t.impl)


def tope1DPlanInit(f, t, x, type_, d) -> None:
    _need(d, x, 1, type_)
    lib.tope1DPlanInit(C.byref(f), C.byref(t), x, type_, _ptr(d))


def tope1DBatchPlanInit(f, t, x, batch, type_, d) -> None:
    _need(d, x, batch, type_)
    lib.tope1DBatchPlanInit(C.byref(f), C.byref(t), x, batch, type_, _ptr(d))


def tope1DExec(f, t, d, dir_) -> None:
    _need_out(d, t, dir_)
    lib.tope1DExec(C.byref(f), C.byref(t), _ptr(d), dir_)


def tope1DDestroy(f, t) -> None:
    lib.tope1DDestroy(C.byref(f), C.byref(t))


def tope2DPlanInit(f, t, x, y, type_, d) -> None:
    _need(d, x, y, type_)
    lib.tope2DPlanInit(C.byref(f), C.byref(t), x, y, type_, _ptr(d))


def tope2DExec(f, t, d, dir_) -> None:
    _need_out(d, t, dir_)
    lib.tope2DExec(C.byref(f), C.byref(t), _ptr(d), dir_)


def tope2DExecX(f, t) -> None:
    lib.tope2DExecX(C.byref(f), C.byref(t))


def tope2DExecY(f, t) -> None:
    lib.tope2DExecY(C.byref(f), C.byref(t))


def tope2DDestroy(f, t) -> None:
    lib.tope2DDestroy(C.byref(f), C.byref(t))


def tope3DPlanInit(f, t, x, y, z, type_, d) -> None:
    _need(d, x, y * z, type_)
    lib.tope3DPlanInit(C.byref(f), C.byref(t), x, y, z, type_, _ptr(d))


def tope3DExec(f, t, d, dir_) -> None:
    _need_out(d, t, dir_)
    lib.tope3DExec(C.byref(f), C.byref(t), _ptr(d), dir_)


def tope3DExecX(f, t) -> None:
    lib.tope3DExecX(C.byref(f), C.byref(t))


def tope3DExecY(f, t) -> None:
    lib.tope3DExecY(C.byref(f), C.byref(t))


def tope3DExecZ(f, t) -> None:
    lib.tope3DExecZ(C.byref(f), C.byref(t))


def tope3DDestroy(f, t) -> None:
    lib.tope3DDestroy(C.byref(f), C.byref(t))


def tope3DBitrevPermute(f, t, axis) -> None:
    lib.tope3DBitrevPermute(C.byref(f), C.byref(t), axis)


def execDevice(f, t, dir_) -> None:
    fn = {TopePlan1D: lib.tope1DExecDevice, TopePlan2D: lib.tope2DExecDevice,
          TopePlan3D: lib.tope3DExecDevice}[type(t)]
    fn(C.byref(f), C.byref(t), dir_)


def upload(f, t, d) -> None:
    fn = {TopePlan1D: lib.tope1DUpload, TopePlan2D: lib.tope2DUpload,
          TopePlan3D: lib.tope3DUpload}[type(t)]
    fn(C.byref(f), C.byref(t), _ptr(d))


def download(f, t, d) -> None:
    fn = {TopePlan1D: lib.tope1DDownload, TopePlan2D: lib.tope2DDownload,
          TopePlan3D: lib.tope3DDownload}[type(t)]
    fn(C.byref(f), C.byref(t), _ptr(d))


def upload_spectrum(f, t, spec) -> None:
    """R2C plans: the x/2 + 1 complex outputs per row, for an inverse
    (a float32 array for the split-precision plans)."""
    if isinstance(spec, np.ndarray) and spec.dtype == np.float32:
        lib.topeUploadSpectrumF32(C.byref(f), t.impl, _fptr(spec))
        return
    fn = {TopePlan1D: lib.tope1DUploadSpectrum, TopePlan2D: lib.tope2DUploadSpectrum,
          TopePlan3D: lib.tope3DUploadSpectrum}[type(t)]
    fn(C.byref(f), C.byref(t), _ptr(spec))


def topeSync(f) -> None:
    lib.topeSync(C.byref(f))


def topeGetLastError() -> int:
    return lib.topeGetLastError()


def topeErrorString(st: int) -> str:
    return lib.topeErrorString(st).decode()


def _fptr(d):
    if d is None:
        return None
    if isinstance(d, np.ndarray):
        if d.dtype != np.float32 or not d.flags.c_contiguous:
            raise TypeError("data must be a C-contiguous float32 array")
        return d.ctypes.data_as(_FL)
    if isinstance(d, int):
        return C.cast(d, _FL)
    raise TypeError("unsupported data argument")


def tope1DBatchPlanInitF32(f, t, x, batch, type_, d) -> None:
    _need(d, x, batch, type_)
    lib.tope1DBatchPlanInitF32(C.byref(f), C.byref(t), x, batch, type_, _fptr(d))


def tope2DPlanInitF32(f, t, x, y, type_, d) -> None:
    _need(d, x, y, type_)
    lib.tope2DPlanInitF32(C.byref(f), C.byref(t), x, y, type_, _fptr(d))


def tope3DPlanInitF32(f, t, x, y, z, type_, d) -> None:
    _need(d, x, y * z, type_)
    lib.tope3DPlanInitF32(C.byref(f), C.byref(t), x, y, z, type_, _fptr(d))


def execF32(f, t, d, dir_) -> None:
    fn = {TopePlan1D: lib.tope1DExecF32, TopePlan2D: lib.tope2DExecF32,
          TopePlan3D: lib.tope3DExecF32}[type(t)]
    _need_out(d, t, dir_)
    fn(C.byref(f), C.byref(t), _fptr(d), dir_)


def uploadF32(f, t, d) -> None:
    lib.topeUploadF32(C.byref(f), t.impl, _fptr(d))


def downloadF32(f, t, d) -> None:
    lib.topeDownloadF32(C.byref(f), t.impl, _fptr(d))


def _iarr(v):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.int32))
    return a, a.ctypes.data_as(_IP)


def topeBatchPlanInit(f, b, nx, ny, type_, d) -> None:
    """nx, ny: sequences of per-transform sizes (ny[i] == 1 for 1D)."""
    ax, px = _iarr(nx)
    ay, py = _iarr(ny)
    if np.asarray(d).dtype == np.float32:
        lib.topeBatchPlanInitF32(C.byref(f), C.byref(b), len(ax), px, py, type_, _fptr(d))
    else:
        lib.topeBatchPlanInit(C.byref(f), C.byref(b), len(ax), px, py, type_, _ptr(d))


def topeBatchExec(f, b, d, dir_) -> None:
    if isinstance(d, np.ndarray) and b.impl and d.nbytes < b.dataSize:
        raise ValueError(f"data holds {d.nbytes} bytes, the batch writes {b.dataSize}")
    if d is not None and np.asarray(d).dtype == np.float32:
        lib.topeBatchExecF32(C.byref(f), C.byref(b), _fptr(d), dir_)
    else:
        lib.topeBatchExec(C.byref(f), C.byref(b), _ptr(d), dir_)


def topeBatchExecDevice(f, b, dir_) -> None:
    lib.topeBatchExecDevice(C.byref(f), C.byref(b), dir_)


def topeBatchUpload(f, b, d) -> None:
    lib.topeBatchUpload(C.byref(f), C.byref(b), d if isinstance(d, int) else d.ctypes.data)


def topeBatchDownload(f, b, d) -> None:
    lib.topeBatchDownload(C.byref(f), C.byref(b), d if isinstance(d, int) else d.ctypes.data)


def topeBatchSetMode(f, b, mode) -> None:
    lib.topeBatchSetMode(C.byref(f), C.byref(b), mode)


def topeBatchDestroy(f, b) -> None:
    lib.topeBatchDestroy(C.byref(f), C.byref(b))


def pass_times(f, t):
    """Per-pass (total ns, launches) since the last reset, and pass geometry."""
    ns = (_u64 * 16)()
    cnt = (_u64 * 16)()
    n = lib.topePassTimes(C.byref(f), t.impl, ns, cnt, 16)
    out = []
    for i in range(max(n, 0)):
        info = (C.c_int64 * 6)()
        lib.topePassInfo(C.byref(f), t.impl, i, info)
        out.append({"ns": int(ns[i]), "launches": int(cnt[i]), "log_l": int(info[0]),
                    "len": (1 << int(info[0])) if info[0] >= 0 else -int(info[0]),
                    "b_tile": int(info[1]), "ctas": int(info[2]), "threads": int(info[3]),
                    "out_of_place": int(info[4]), "four_step_twiddle": int(info[5])})
    return out


def copy_to_host(f, dst: np.ndarray, device_ptr: int) -> None:
    lib.topeCopyToHost(C.byref(f), dst.ctypes.data_as(_vp), device_ptr, dst.nbytes)


def check(f: TopeFFT) -> None:
    """Raise if the last call on f failed."""
    if f.error != TOPE_SUCCESS:
        st = f.error
        raise RuntimeError(f"topeFFT error {st}: {topeErrorString(st)}"
                           + (f" (CUDA {lib.topeLastCudaError()})" if st == TOPE_ERR_CUDA else ""))
