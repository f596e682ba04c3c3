"""GPU parity of the split-precision form (FP32 data, FP64-accurate hi/lo
twiddles), through the C interface, in its three modes: accurate
(double-float butterflies on chip), fast (FP32 butterflies) and tensor (the
radix-16 stages as tcgen05 GEMMs on three-piece FP16 splits with an exact
leading accumulator, double-float around them).

Inputs follow the benchmark configuration of this form: the uniform[-1,1)
field plus a Gaussian pulse of amplitude 1e6 (sigma = 4 samples per axis)
added to the real part at the grid centre (per row for batched 1D), which
stresses dynamic range.  The FP64 oracle runs on the FP64 values before
they are rounded to FP32.  Gate: rel-L2 <= 1e-7 (accurate and tensor modes,
the benchmark's gate); max-abs is reported.
"""
import numpy as np
import pytest

from conftest import SEED0

pytestmark = pytest.mark.gpu

# the accurate and tensor modes (about 32 bits on chip, FP32 only in memory)
# meet the benchmark gate; the fast mode (FP32 butterflies) carries an FP32
# FFT's own rounding error, measured 1.0e-7..1.6e-7 on these inputs
GATES = {"accurate": 1e-7, "fast": 2.5e-7, "tensor": 1e-7}
MODES = {"accurate": 0, "fast": 1, "tensor": 2}


@pytest.fixture(params=["accurate", "fast", "tensor"])
def fw(T, request):
    """One framework per split mode (FP32 plans ignore the FP64-storage
    arithmetic setting)."""
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.check(f)
    T.topeSetSplitMode(f, MODES[request.param])
    T.check(f)
    f.gate = GATES[request.param]
    yield f
    T.topeFFTDestroy(f)


def pulse_field(orc, dims, batch=1, seed=SEED0 + 4, amp=1e6, sigma=4.0):
    nx, ny, nz = dims
    x = orc.uniform(nx * ny * nz * batch, seed)
    grids = np.meshgrid(*[np.arange(n) - n // 2 for n in (nz, ny, nx)], indexing="ij")
    r2 = sum(g.astype(np.float64) ** 2 for g, n in zip(grids, (nz, ny, nx)) if n > 1)
    p = amp * np.exp(-r2 / (2 * sigma * sigma)).ravel()
    x[0::2] += np.tile(p, batch)
    return x


def run_f32(T, fw, x32, dims, dir_, batch=1):
    nx, ny, nz = dims
    d = x32.copy()
    if ny == 1 and nz == 1:
        t = T.TopePlan1D()
        T.tope1DBatchPlanInitF32(fw, t, nx, batch, T.C2C, d)
    elif nz == 1:
        t = T.TopePlan2D()
        T.tope2DPlanInitF32(fw, t, nx, ny, T.C2C, d)
    else:
        t = T.TopePlan3D()
        T.tope3DPlanInitF32(fw, t, nx, ny, nz, T.C2C, d)
    T.check(fw)
    T.execF32(fw, t, d, dir_)
    T.check(fw)
    {T.TopePlan1D: T.tope1DDestroy, T.TopePlan2D: T.tope2DDestroy,
     T.TopePlan3D: T.tope3DDestroy}[type(t)](fw, t)
    return d


def oracle_fp64(orc, x, dims, dir_, batch=1):
    nx, ny, nz = dims
    return orc.exec(x, nx, ny, nz, dir_, batch=batch)


CASES = [((1 << 14, 1, 1), 64), ((1 << 16, 1, 1), 16), ((1 << 20, 1, 1), 1), ((4096, 1, 1), 256),
         ((512, 512, 1), 1), ((64, 64, 64), 1), ((128, 128, 128), 1), ((32, 64, 128), 1),
         ((16384, 8, 1), 1), ((8, 8, 16384), 1)]


@pytest.mark.parametrize("dims,batch", CASES, ids=lambda c: "x".join(map(str, c)) if isinstance(c, tuple) else str(c))
def test_f32_error_vs_fp64_oracle(T, fw, orc, dims, batch):
    x = pulse_field(orc, dims, batch)
    x32 = x.astype(np.float32)
    for dir_ in (1, 0):
        got = run_f32(T, fw, x32, dims, dir_, batch).astype(np.float64)
        ref = oracle_fp64(orc, x, dims, dir_, batch)
        err = orc.rel_l2(got, ref)
        # the algorithm's own error: oracle on the FP32-rounded input
        ref_r = oracle_fp64(orc, x32.astype(np.float64), dims, dir_, batch)
        err_alg = orc.rel_l2(got, ref_r)
        print(f"{dims} x{batch} dir={dir_}: rel-L2 {err:.2e} (vs rounded input {err_alg:.2e}), "
              f"max-abs {orc.max_abs(got, ref):.3e}")
        assert err <= fw.gate and err_alg <= fw.gate


@pytest.mark.parametrize("dims,batch", [((512, 512, 512), 1), ((1 << 14, 1, 1), 4096), ((1 << 24, 1, 1), 1)],
                         ids=["512^3", "4096x2^14", "2^24"])
def test_f32_full_size(T, fw, orc, dims, batch):
    """The split-precision benchmark configurations themselves, and the 2^24
    line of the default benchmark's split-precision companion."""
    x = pulse_field(orc, dims, batch)
    x32 = x.astype(np.float32)
    got = run_f32(T, fw, x32, dims, 1, batch).astype(np.float64)
    ref = oracle_fp64(orc, x, dims, 1, batch)
    err = orc.rel_l2(got, ref)
    print(f"{dims} x{batch}: rel-L2 {err:.2e}, max-abs {orc.max_abs(got, ref):.3e}")
    assert err <= fw.gate


@pytest.mark.parametrize("dims,batch", [((128, 128, 128), 1), ((512, 256, 1), 1),
                                        ((1 << 14, 1, 1), 64), ((64, 32, 256), 1)],
                         ids=["128^3", "512x256", "64x2^14", "64x32x256"])
def test_load_paths_agree(T, fw, orc, monkeypatch, dims, batch):
    """Tiles loaded directly (TOPEFFT_BULK=0), contiguous tiles by bulk
    copies (1, the default) and strided tiles by TMA boxes from tensor maps
    as well (2): the same transform bit for bit, and within the gate."""
    x = pulse_field(orc, dims, batch)
    x32 = x.astype(np.float32)
    outs = []
    for level in ("0", "1", "2"):
        monkeypatch.setenv("TOPEFFT_BULK", level)
        outs.append(run_f32(T, fw, x32, dims, 1, batch))
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    err = orc.rel_l2(outs[2].astype(np.float64), oracle_fp64(orc, x, dims, 1, batch))
    assert err <= fw.gate


def test_f32_round_trip_and_type_checks(T, fw, orc):
    n, b = 1 << 15, 8
    x32 = orc.uniform(n * b, 3).astype(np.float32)
    d = x32.copy()
    t = T.TopePlan1D()
    T.tope1DBatchPlanInitF32(fw, t, n, b, T.C2C, d)
    T.check(fw)
    T.execF32(fw, t, d, T.FORWARD)
    T.execF32(fw, t, d, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(d.astype(np.float64), x32.astype(np.float64)) <= 1e-6
    T.tope1DExec(fw, t, np.zeros(2 * n * b), T.FORWARD)  # FP64 entry point on an FP32 plan
    assert fw.error == T.TOPE_ERR_INVALID_ARG
    T.tope1DDestroy(fw, t)
    T.check(fw)


@pytest.mark.parametrize("lg,batch", [(4, 256), (4, 3), (5, 100), (8, 16), (9, 5), (10, 4),
                                      (11, 2), (12, 1), (12, 3), (13, 2), (14, 2), (2, 8)])
def test_tensor_mode_shapes(T, orc, lg, batch):
    """Every line length of the tensor form (one row group per 128 16-point
    sub-transforms, ragged last tiles, the four-step split above 2^13, the
    accurate form's kernel below 16 points) against the FP64 oracle, at the
    benchmark's gate."""
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.topeSetSplitMode(f, T.TOPE_SPLIT_TENSOR)
    T.check(f)
    n = 1 << lg
    x32 = orc.uniform(n * batch, SEED0 + lg).astype(np.float32)
    for dir_ in (1, 0):
        got = run_f32(T, f, x32, (n, 1, 1), dir_, batch).astype(np.float64)
        ref = orc.exec(x32.astype(np.float64), n, 1, 1, dir_, batch=batch)
        err = orc.rel_l2(got, ref)
        print(f"tensor L=2^{lg} x{batch} dir={dir_}: rel-L2 {err:.2e}")
        assert err <= 1e-7
    T.topeFFTDestroy(f)


@pytest.mark.parametrize("lg", [5, 6, 7, 9, 10, 11, 12, 13])
def test_tensor_mode_pure_tones(T, orc, lg):
    """Lines holding one tone each: the first stage's double-float sums
    cancel exactly in many rows, leaving values whose low part is the whole
    value; the tensor stages must renormalise them before splitting.  Every
    line length with a first stage of radix 2, 4 or 8 on the CUDA cores,
    against the FP64 oracle."""
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.topeSetSplitMode(f, T.TOPE_SPLIT_TENSOR)
    T.check(f)
    n, batch = 1 << lg, 4
    j = np.arange(n)
    x = np.concatenate([np.exp(2j * np.pi * ((j * (3 + 7 * b)) % n) / n) for b in range(batch)])
    x32 = x.astype(np.complex64).view(np.float32)
    for dir_ in (1, 0):
        got = run_f32(T, f, x32, (n, 1, 1), dir_, batch).astype(np.float64)
        assert np.all(np.isfinite(got))
        ref = orc.exec(x32.astype(np.float64), n, 1, 1, dir_, batch=batch)
        err = orc.rel_l2(got, ref)
        print(f"tensor tones L=2^{lg} dir={dir_}: rel-L2 {err:.2e}")
        assert err <= 1e-7
    T.topeFFTDestroy(f)


def test_tensor_mode_rejected_by_batches(T):
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.topeSetSplitMode(f, T.TOPE_SPLIT_TENSOR)
    b = T.TopeBatch()
    d = np.zeros(2 * 64, dtype=np.float32)
    T.topeBatchPlanInit(f, b, [64], [1], T.C2C, d)
    assert f.error == T.TOPE_ERR_UNSUPPORTED and not b.impl
    T.topeFFTDestroy(f)
