"""The whole library on the CPU: its C host code, the auxiliary kernels, the
pass dispatch, and the power-of-two (log2 L <= 8, and the 4-points-per-thread
shape), mixed-radix and real-data kernels, all built from the repository's
own sources for the host (tests/emu/emu_build.py), each kernel launch run as
one CTA after another with one std::thread per CUDA thread; the persistent
batch kernel runs as a single CTA and a captured graph as its recorded
launches.  The tensor form and the allocation-free entry point are not built
for the host.

The tests call the public C entry points through the same ctypes mirror as
the GPU tests and compare with the oracle: one- and multi-pass power-of-two
lines, mixed radix, Bluestein and the exact DFT, 2D/3D, real data, both
FP64-storage arithmetics and the split-precision modes.  Gates as on the GPU."""
import numpy as np
import pytest

from conftest import SEED0, tol_fp64

import sys
from pathlib import Path
sys.path.insert(0, str(Path(__file__).resolve().parent / "emu"))
import emu_build  # noqa: E402


@pytest.fixture(scope="module")
def E(T, tmp_path_factory, pytestconfig):
    """The package's ctypes mirror, bound to the host build of the library
    (with sanitizers under --emu-sanitize, see tests/test_sanitized_library.py)."""
    d = tmp_path_factory.mktemp("emulib")
    if not emu_build.host_cxx_ok(d):
        pytest.skip("no C++20 host compiler (std::barrier)")
    sanitize = pytestconfig.getoption("--emu-sanitize")
    lib = T.load_library(emu_build.build_library(d, sanitize=sanitize))
    saved = T.topefft.lib
    T.topefft.lib = lib
    yield T
    T.topefft.lib = saved


@pytest.fixture(params=["fp64", "df64"])
def fw(E, request):
    f = E.TopeFFT()
    E.topeFFTInit(f)
    E.check(f)
    E.topeSetArith(f, E.TOPE_ARITH_DF64 if request.param == "df64" else E.TOPE_ARITH_FP64)
    yield f
    E.topeFFTDestroy(f)


def oracle_1d(orc, x, n, dir_, batch=1):
    rows = []
    for i in range(batch):
        xi = x[2 * n * i: 2 * n * (i + 1)]
        rows.append(orc.fft_ld(xi, n, dir_=dir_) if n & (n - 1) == 0 or n < 5000 else
                    orc.bluestein_ld(xi, n, dir_))
    return np.concatenate(rows)


@pytest.mark.parametrize("n,batch", [(2, 1), (8, 1), (64, 1), (256, 4), (4096, 1), (1 << 14, 1),
                                     (1000, 1), (60, 8), (1001, 1), (131, 1), (127, 2)])
def test_1d(E, fw, orc, n, batch):
    x = orc.uniform(n * batch, SEED0 + n)
    for dir_ in (1, 0):
        d = x.copy()
        t = E.TopePlan1D()
        E.tope1DBatchPlanInit(fw, t, n, batch, E.C2C, d)
        E.check(fw)
        E.tope1DExec(fw, t, d, dir_)
        E.check(fw)
        assert orc.rel_l2(d, oracle_1d(orc, x, n, dir_, batch)) <= tol_fp64(n)
        E.tope1DDestroy(fw, t)


@pytest.mark.parametrize("shape", [(32, 16, 1), (12, 10, 1), (8, 16, 4), (6, 10, 14)])
def test_nd(E, fw, orc, shape):
    nx, ny, nz = shape
    x = orc.uniform(nx * ny * nz, SEED0 + nx + ny)
    for dir_ in (1, 0):
        d = x.copy()
        if nz == 1:
            t = E.TopePlan2D()
            E.tope2DPlanInit(fw, t, nx, ny, E.C2C, d)
            E.check(fw)
            E.tope2DExec(fw, t, d, dir_)
            E.tope2DDestroy(fw, t)
        else:
            t = E.TopePlan3D()
            E.tope3DPlanInit(fw, t, nx, ny, nz, E.C2C, d)
            E.check(fw)
            E.tope3DExec(fw, t, d, dir_)
            E.tope3DDestroy(fw, t)
        E.check(fw)
        assert orc.rel_l2(d, orc.fft_ld(x, nx, ny, nz, dir_=dir_)) <= tol_fp64(nx * ny * nz)


def test_single_axes_compose(E, fw, orc):
    """ExecX then ExecY on device data equals Exec (fft2d.c:12-133)."""
    nx, ny = 16, 8
    x = orc.uniform(nx * ny, SEED0 + 9)
    t = E.TopePlan2D()
    E.tope2DPlanInit(fw, t, nx, ny, E.C2C, x.copy())
    E.tope2DExecX(fw, t)
    E.tope2DExecY(fw, t)
    got = np.empty_like(x)
    E.download(fw, t, got)
    E.check(fw)
    assert orc.rel_l2(got, orc.fft_ld(x, nx, ny, 1, dir_=1)) <= tol_fp64(nx * ny)
    E.tope2DDestroy(fw, t)


@pytest.mark.parametrize("dims", [(64, 1, 1), (2000, 1, 1), (16, 8, 1), (20, 12, 1)])
def test_real_data(E, fw, orc, dims):
    nx, ny, nz = dims
    n = nx * ny * nz
    xr = orc.uniform(n // 2, SEED0 + nx)
    d = np.zeros((nx + 2) * ny * nz)
    d[:n] = xr
    if ny == 1:
        t = E.TopePlan1D()
        E.tope1DPlanInit(fw, t, nx, E.R2C, d)
        ex, ds = E.tope1DExec, E.tope1DDestroy
    else:
        t = E.TopePlan2D()
        E.tope2DPlanInit(fw, t, nx, ny, E.R2C, d)
        ex, ds = E.tope2DExec, E.tope2DDestroy
    E.check(fw)
    ex(fw, t, d, E.FORWARD)
    E.check(fw)
    z = np.zeros(2 * n)
    z[0::2] = xr
    full = orc.fft_ld(z, nx, ny, nz, dir_=1).reshape(nz, ny, nx, 2)
    want = np.ascontiguousarray(full[:, :, : nx // 2 + 1, :]).ravel()
    assert orc.rel_l2(d, want) <= tol_fp64(n)
    ex(fw, t, d, E.INVERSE)
    E.check(fw)
    assert orc.rel_l2(d[:n], xr) <= tol_fp64(n)
    ds(fw, t)


@pytest.mark.parametrize("mode,gate", [(0, 1e-7), (1, 2.5e-7)])
@pytest.mark.parametrize("dims,batch,real", [((256, 1, 1), 4, False), ((32, 16, 1), 1, False),
                                             ((1000, 1, 1), 2, False), ((64, 1, 1), 3, True)])
def test_split_precision(E, orc, mode, gate, dims, batch, real):
    f = E.TopeFFT()
    E.topeFFTInit(f)
    E.topeSetSplitMode(f, mode)
    nx, ny, nz = dims
    n = nx * ny * nz
    if real:
        xr = orc.uniform(n * batch // 2, SEED0 + 3)
        d = np.zeros((nx + 2) * batch, dtype=np.float32)
        d[:n * batch] = xr
    else:
        x = orc.uniform(n * batch, SEED0 + 3)
        d = x.astype(np.float32)
    if ny == 1:
        t = E.TopePlan1D()
        E.tope1DBatchPlanInitF32(f, t, nx, batch, E.R2C if real else E.C2C, d)
    else:
        t = E.TopePlan2D()
        E.tope2DPlanInitF32(f, t, nx, ny, E.C2C, d)
    E.check(f)
    E.execF32(f, t, d, E.FORWARD)
    E.check(f)
    if real:
        want = []
        for b in range(batch):
            z = np.zeros(2 * nx)
            z[0::2] = xr[b * nx:(b + 1) * nx]
            want.append(orc.fft_ld(z, nx, dir_=1)[: nx + 2])
        want = np.concatenate(want)
    elif ny == 1:
        want = oracle_1d(orc, x, nx, 1, batch)
    else:
        want = orc.fft_ld(x, nx, ny, nz, dir_=1)
    assert orc.rel_l2(d.astype(np.float64), want) <= gate
    {E.TopePlan1D: E.tope1DDestroy, E.TopePlan2D: E.tope2DDestroy}[type(t)](f, t)
    E.topeFFTDestroy(f)


@pytest.mark.parametrize("shape", [(2, 2, 1), (2, 4, 8), (1, 16, 2), (4, 1, 2)])
def test_short_axes(E, fw, orc, shape):
    """Axes of length 1 and 2 (the reference divides by n/4 == 0 there,
    src/kernels2D.cl:51)."""
    nx, ny, nz = shape
    x = orc.uniform(nx * ny * nz, SEED0 + 17)
    d = x.copy()
    t = E.TopePlan3D()
    E.tope3DPlanInit(fw, t, nx, ny, nz, E.C2C, d)
    E.check(fw)
    E.tope3DExec(fw, t, d, E.FORWARD)
    E.check(fw)
    assert orc.rel_l2(d, orc.fft_ld(x, nx, ny, nz, dir_=1)) <= tol_fp64(nx * ny * nz)
    E.tope3DDestroy(fw, t)


@pytest.mark.parametrize("scale", [1e300, 1e-300, 2.0 ** -1060])
def test_extreme_magnitudes(E, fw, orc, scale):
    """Inputs near the top and bottom of the FP64 range, subnormals included.
    The double-float arithmetic's tile scaling keeps its (hi, lo) pairs in
    FP32 range; at 2^-1060 the inputs and outputs are FP64 subnormals with
    about 14 significant bits, which bounds either path's accuracy (native
    FP64 rounds every intermediate to that spacing)."""
    n = 256
    x = orc.uniform(n, SEED0 + 5) * scale
    d = x.copy()
    t = E.TopePlan1D()
    E.tope1DPlanInit(fw, t, n, E.C2C, d)
    E.tope1DExec(fw, t, d, E.FORWARD)
    E.check(fw)
    want = orc.fft_ld(x, n, dir_=1)
    tol = tol_fp64(n) if scale >= 1e-300 else (1e-6 if fw.arith else 1e-4)
    assert orc.rel_l2(d, want) <= tol
    E.tope1DDestroy(fw, t)


@pytest.mark.parametrize("n", [3, 5, 6, 7, 11, 12, 13, 27, 100, 1000, 1001])
def test_reference_dft_outputs(E, fw, orc, golden, n):
    """The reference's own DFT kernel outputs (tests/golden), reproduced by
    the mixed-radix passes to the FP64 gate."""
    x = orc.uniform(n, int(golden[f"dftseed_{n}"][0]))
    d = x.copy()
    t = E.TopePlan1D()
    E.tope1DPlanInit(fw, t, n, E.C2C, d)
    E.tope1DExec(fw, t, d, E.FORWARD)
    E.check(fw)
    assert orc.rel_l2(d, golden[f"dft_{n}"]) <= tol_fp64(n)
    E.tope1DDestroy(fw, t)


# ---------------------------------------------------------------- uneven batches
# lines of at most 2^8 points per pass: the host build's launch tables stop
# there (2^14 is two passes of 2^7)
BATCH_SHAPES = [(64, 1), (256, 1), (16, 1), (1 << 14, 1), (64, 1), (32, 16), (8, 64), (128, 1),
                (8, 1), (2, 1)]


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["persistent", "launch_graph", "loop"])
@pytest.mark.parametrize("arith", ["fp64", "df64", "split"])
def test_uneven_batch(E, orc, mode, arith, tmp_path, monkeypatch):
    """A batch of mixed 1D/2D power-of-two transforms packed in one buffer, in
    each execution structure: the persistent kernel (a single CTA on the host,
    taking the work items in their topological order), the captured per-class
    launch graph, and the per-transform loop."""
    monkeypatch.setenv("TOPEFFT_TUNE_CACHE", str(tmp_path / "tune.txt"))
    f = E.TopeFFT()
    E.topeFFTInit(f)
    if arith == "df64":
        E.topeSetArith(f, E.TOPE_ARITH_DF64)
    nx = [s[0] for s in BATCH_SHAPES]
    ny = [s[1] for s in BATCH_SHAPES]
    total = sum(a * b for a, b in BATCH_SHAPES)
    x = orc.uniform(total, SEED0 + 77)
    b = E.TopeBatch()
    d = x.astype(np.float32) if arith == "split" else x.copy()
    E.topeBatchPlanInit(f, b, nx, ny, E.C2C, d)  # FP32 data: the split-precision form
    E.check(f)
    assert b.classes == 9
    E.topeBatchSetMode(f, b, mode)
    E.check(f)
    E.topeBatchExec(f, b, d, E.FORWARD)
    E.check(f)
    off = 0
    for (a, c) in BATCH_SHAPES:
        n = a * c
        want = orc.fft_ld(x[2 * off: 2 * (off + n)], a, c, 1, dir_=1)
        got = d[2 * off: 2 * (off + n)].astype(np.float64)
        assert orc.rel_l2(got, want) <= (1e-7 if arith == "split" else tol_fp64(n)), (a, c)
        off += n
    E.topeBatchDestroy(f, b)
    E.topeFFTDestroy(f)


def test_sliced_readback_rows(E, orc):
    """Exec into a host buffer of 32 MB (256-point rows x 8192): the last pass
    runs in slices, each copied back while the next computes; the result is
    bit for bit that of ExecDevice + Download, and the oracle's."""
    f = E.TopeFFT()
    E.topeFFTInit(f)
    nx, batch = 256, 8192
    x = orc.uniform(nx * batch, SEED0 + 81)
    t = E.TopePlan1D()
    E.tope1DBatchPlanInit(f, t, nx, batch, E.C2C, x.copy())
    E.check(f)
    got = np.full_like(x, np.nan)
    E.tope1DExec(f, t, got, E.FORWARD)
    E.check(f)
    E.upload(f, t, x)
    E.execDevice(f, t, E.FORWARD)
    want = np.empty_like(x)
    E.download(f, t, want)
    E.check(f)
    assert np.array_equal(got, want)
    rows = np.arange(0, batch, 911)
    ref = np.concatenate([orc.fft_ld(x[2 * nx * r: 2 * nx * (r + 1)], nx, dir_=1) for r in rows])
    sub = np.concatenate([got[2 * nx * r: 2 * nx * (r + 1)] for r in rows])
    assert orc.rel_l2(sub, ref) <= tol_fp64(nx)
    E.tope1DDestroy(f, t)
    E.topeFFTDestroy(f)


def test_sliced_readback_3d(E, orc):
    """128^3 (32 MB): the z pass is sliced along its (x, y) lines and each
    slice goes back as a 2D copy of 128 rows."""
    f = E.TopeFFT()
    E.topeFFTInit(f)
    n = 128
    x = orc.uniform(n ** 3, SEED0 + 82)
    t = E.TopePlan3D()
    E.tope3DPlanInit(f, t, n, n, n, E.C2C, x.copy())
    E.check(f)
    got = np.full_like(x, np.nan)
    E.tope3DExec(f, t, got, E.FORWARD)
    E.check(f)
    assert orc.rel_l2(got, orc.fft_ld(x, n, n, n, dir_=1)) <= tol_fp64(n ** 3)
    E.tope3DDestroy(f, t)
    E.topeFFTDestroy(f)


def test_inverse_from_uploaded_spectrum(E, orc):
    """2D R2C (FP64) and 1D R2C (FP32): a spectrum uploaded from the host goes
    back to the reals through the inverse."""
    f = E.TopeFFT()
    E.topeFFTInit(f)
    nx, ny = 32, 8
    xr = orc.uniform(nx * ny // 2, SEED0 + 91)
    z = np.zeros(2 * nx * ny)
    z[0::2] = xr
    spec = np.ascontiguousarray(orc.fft_ld(z, nx, ny, 1, dir_=1).reshape(ny, nx, 2)[:, : nx // 2 + 1])
    t = E.TopePlan2D()
    E.tope2DPlanInit(f, t, nx, ny, E.R2C, np.zeros(nx * ny))
    E.check(f)
    E.upload_spectrum(f, t, spec.ravel())
    E.check(f)
    out = np.zeros((nx + 2) * ny)
    E.tope2DExec(f, t, out, E.INVERSE)
    E.check(f)
    assert orc.rel_l2(out[: nx * ny], xr) <= tol_fp64(nx * ny)
    E.tope2DDestroy(f, t)
    E.topeSetSplitMode(f, 0)
    n = 128
    zr = np.zeros(2 * n)
    zr[0::2] = xr[:n]
    spec1 = orc.fft_ld(zr, n, dir_=1)[: n + 2].astype(np.float32)
    t1 = E.TopePlan1D()
    E.tope1DBatchPlanInitF32(f, t1, n, 1, E.R2C, np.zeros(n, dtype=np.float32))
    E.check(f)
    E.upload_spectrum(f, t1, spec1)
    E.check(f)
    back = np.zeros(n + 2, dtype=np.float32)
    E.execF32(f, t1, back, E.INVERSE)
    E.check(f)
    assert orc.rel_l2(back[:n].astype(np.float64), xr[:n]) <= 1e-7
    E.tope1DDestroy(f, t1)
    E.topeFFTDestroy(f)


def test_status_paths(E, orc):
    """Errors come back as statuses: a bad direction, a destroyed plan, the
    tensor form where this build has no kernel for it, an FP64 call on an FP32
    plan."""
    f = E.TopeFFT()
    E.topeFFTInit(f)
    t = E.TopePlan1D()
    x = orc.uniform(64, 1)
    E.tope1DPlanInit(f, t, 64, E.C2C, x.copy())
    E.check(f)
    E.tope1DExec(f, t, x.copy(), 7)
    assert f.error == E.TOPE_ERR_INVALID_ARG
    E.tope1DDestroy(f, t)
    E.tope1DDestroy(f, t)
    assert f.error == E.TOPE_ERR_DESTROYED
    E.topeSetSplitMode(f, 2)
    t2 = E.TopePlan1D()
    E.tope1DBatchPlanInitF32(f, t2, 256, 4, E.C2C, np.zeros(2048, dtype=np.float32))
    assert f.error == E.TOPE_ERR_UNSUPPORTED and not t2.impl
    E.topeSetSplitMode(f, 0)
    E.tope1DBatchPlanInitF32(f, t2, 256, 4, E.C2C, np.zeros(2048, dtype=np.float32))
    E.check(f)
    E.tope1DExec(f, t2, np.zeros(2048), E.FORWARD)
    assert f.error == E.TOPE_ERR_INVALID_ARG
    E.tope1DDestroy(f, t2)
    E.topeFFTDestroy(f)


def _smooth(rng, maxn):
    while True:
        n = 1
        for p in (2, 3, 5, 7, 11, 13):
            n *= p ** int(rng.integers(0, 4 if p < 7 else 2))
        if 2 <= n <= maxn:
            return n


@pytest.mark.parametrize("seed", range(4))
def test_random_plans(E, orc, seed):
    """Seeded random plans: 1D/2D/3D, C2C and R2C, FP64, double-float and
    split precision, products of 2..13 and powers of two, batched rows, both
    directions, each against the oracle.  Plans whose pass lengths the host
    build has no kernel for (power-of-two passes above 2^8) are skipped."""
    rng = np.random.default_rng(seed)
    checked = 0
    for it in range(12):
        mode = ["fp64", "df64", "f32acc", "f32fast"][int(rng.integers(0, 4))]
        real = bool(rng.integers(0, 3) == 0)
        nd = int(rng.choice([1, 1, 2, 3]))
        dir_ = int(rng.integers(0, 2))
        nx = 2 * _smooth(rng, 150) if real else _smooth(rng, 300)
        ny = _smooth(rng, 20) if nd >= 2 else 1
        nz = _smooth(rng, 10) if nd == 3 else 1
        batch = int(rng.integers(1, 4)) if nd == 1 else 1
        if real:
            dir_ = 1
        f32 = mode.startswith("f32")
        f = E.TopeFFT()
        E.topeFFTInit(f)
        E.topeSetArith(f, E.TOPE_ARITH_DF64 if mode == "df64" else E.TOPE_ARITH_FP64)
        E.topeSetSplitMode(f, 1 if mode == "f32fast" else 0)
        n = nx * ny * nz
        if real:
            xr = orc.uniform(n * batch // 2, seed * 100 + it)
            d = np.zeros((nx + 2) * ny * nz * batch, dtype=np.float32 if f32 else np.float64)
            d[: n * batch] = xr
        else:
            x = orc.uniform(n * batch, seed * 100 + it)
            d = x.astype(np.float32) if f32 else x.copy()
        kind = E.R2C if real else E.C2C
        if nd == 1:
            t = E.TopePlan1D()
            (E.tope1DBatchPlanInitF32 if f32 else E.tope1DBatchPlanInit)(f, t, nx, batch, kind, d)
        elif nd == 2:
            t = E.TopePlan2D()
            (E.tope2DPlanInitF32 if f32 else E.tope2DPlanInit)(f, t, nx, ny, kind, d)
        else:
            t = E.TopePlan3D()
            (E.tope3DPlanInitF32 if f32 else E.tope3DPlanInit)(f, t, nx, ny, nz, kind, d)
        if f.error == E.TOPE_ERR_UNSUPPORTED:
            E.topeFFTDestroy(f)
            continue
        E.check(f)
        if f32:
            E.execF32(f, t, d, dir_)
        else:
            {E.TopePlan1D: E.tope1DExec, E.TopePlan2D: E.tope2DExec,
             E.TopePlan3D: E.tope3DExec}[type(t)](f, t, d, dir_)
        E.check(f)
        if real:
            want = []
            for b in range(batch):
                z = np.zeros(2 * n)
                z[0::2] = xr[b * n:(b + 1) * n]
                full = orc.fft_ld(z, nx, ny, nz, dir_=1).reshape(nz, ny, nx, 2)
                want.append(np.ascontiguousarray(full[:, :, : nx // 2 + 1, :]).ravel())
            want = np.concatenate(want)
        else:
            want = np.concatenate([orc.fft_ld(x[2 * n * b: 2 * n * (b + 1)], nx, ny, nz, dir_=dir_)
                                   for b in range(batch)])
        gate = {"f32acc": 1e-7, "f32fast": 2.5e-7}.get(mode, tol_fp64(n))
        assert orc.rel_l2(d.astype(np.float64), want) <= gate, (mode, real, nx, ny, nz, batch)
        {E.TopePlan1D: E.tope1DDestroy, E.TopePlan2D: E.tope2DDestroy,
         E.TopePlan3D: E.tope3DDestroy}[type(t)](f, t)
        E.topeFFTDestroy(f)
        checked += 1
    assert checked >= 6


def test_binding_refuses_short_output_arrays(E, orc):
    """The Python binding checks a numpy array against what an Exec writes
    before the C code runs: the plan's data, or for a real-data plan's
    forward transform its x/2 + 1 complex outputs per row."""
    f = E.TopeFFT()
    E.topeFFTInit(f)
    n, rows = 64, 3
    x = orc.uniform(n * rows // 2, SEED0 + 91)
    t = E.TopePlan1D()
    E.tope1DBatchPlanInit(f, t, n, rows, E.R2C, x)
    E.check(f)
    with pytest.raises(ValueError):
        E.tope1DExec(f, t, np.zeros(n * rows), E.FORWARD)  # reals-sized: too short
    spec = np.zeros((n + 2) * rows)
    E.tope1DExec(f, t, spec, E.FORWARD)
    E.check(f)
    E.tope1DExec(f, t, np.zeros(n * rows), E.INVERSE)  # the inverse writes the reals
    E.check(f)
    E.tope1DDestroy(f, t)
    c = E.TopePlan2D()
    E.tope2DPlanInit(f, c, 8, 4, E.C2C, np.zeros(64))
    with pytest.raises(ValueError):
        E.tope2DExec(f, c, np.zeros(63), E.FORWARD)
    E.tope2DDestroy(f, c)
    E.topeFFTDestroy(f)
