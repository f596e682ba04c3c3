"""GPU parity of the FP64 C2C path, through the C interface (libtopefft.so).

Every case compares the GPU result with the CPU oracle on the same seeded
input: the restatement of the reference's algorithm (oracle.exec) and, where
it finishes quickly, the long-double FFT.  Gate (BASELINE): rel-L2 <=
1e-13 * log2(N).  Integer work (bit-reversal tables, the swap permutation)
is compared bit for bit with fixtures from the reference's own kernels.
Full-size cases use size-independent properties as well (round trip,
Parseval, linearity).
"""
import numpy as np
import pytest

from conftest import SEED0, tol_fp64

pytestmark = pytest.mark.gpu


# ---------------------------------------------------------------- helpers
def run1d(T, f, x, n, dir_=1, batch=1):
    d = x.copy()
    t = T.TopePlan1D()
    if batch == 1:
        T.tope1DPlanInit(f, t, n, T.C2C, d)
    else:
        T.tope1DBatchPlanInit(f, t, n, batch, T.C2C, d)
    T.check(f)
    T.tope1DExec(f, t, d, dir_)
    T.check(f)
    T.tope1DDestroy(f, t)
    T.check(f)
    return d


def run_nd(T, f, x, shape, dir_=1):
    nx, ny, nz = shape
    d = x.copy()
    if nz == 1:
        t = T.TopePlan2D()
        T.tope2DPlanInit(f, t, nx, ny, T.C2C, d)
        T.check(f)
        T.tope2DExec(f, t, d, dir_)
        T.check(f)
        T.tope2DDestroy(f, t)
    else:
        t = T.TopePlan3D()
        T.tope3DPlanInit(f, t, nx, ny, nz, T.C2C, d)
        T.check(f)
        T.tope3DExec(f, t, d, dir_)
        T.check(f)
        T.tope3DDestroy(f, t)
    T.check(f)
    return d


# ---------------------------------------------------------------- 1D
POW2_1D = [1, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 1 << 14, 1 << 15,
           1 << 16, 1 << 17, 1 << 18, 1 << 20]


@pytest.mark.parametrize("n", POW2_1D)
@pytest.mark.parametrize("dir_", [1, 0], ids=["fwd", "inv"])
def test_1d_matches_oracle(T, fw, orc, n, dir_):
    x = orc.uniform(n, SEED0 + n)
    got = run1d(T, fw, x, n, dir_)
    tol = tol_fp64(n)
    assert orc.rel_l2(got, orc.exec(x, n, dir_=dir_)) <= tol
    if n <= 1 << 14:
        assert orc.rel_l2(got, orc.fft_ld(x, n, dir_=dir_)) <= tol


@pytest.mark.parametrize("n", [4096, 1 << 16, 1 << 20])
def test_1d_round_trip_on_device_data(T, fw, orc, n):
    """Exec reuses the device-resident array: forward then inverse is a round
    trip even though d is overwritten in between (test/1d.c:79-82)."""
    x = orc.uniform(n, SEED0 + 1)
    d = x.copy()
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, n, T.C2C, d)
    T.tope1DExec(fw, t, d, T.FORWARD)
    d[:] = 12345.0  # ignored by the next Exec
    T.tope1DExec(fw, t, d, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(d, x) <= tol_fp64(n)
    assert t.totalKernel > 0 and t.totalMemory > 0 and t.totalPreKernel > 0
    T.tope1DDestroy(fw, t)


def test_1d_2pow24_full_size(T, fw, orc):
    """Config 2, single N = 2^24: forward vs oracle, round trip, Parseval."""
    n = 1 << 24
    x = orc.uniform(n, SEED0 + 2)
    d = x.copy()
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, n, T.C2C, d)
    T.tope1DExec(fw, t, d, T.FORWARD)
    T.check(fw)
    tol = tol_fp64(n)
    assert orc.rel_l2(d, orc.exec(x, n)) <= tol
    assert abs(np.dot(d, d) / n / np.dot(x, x) - 1) < 1e-12
    T.tope1DExec(fw, t, d, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(d, x) <= tol
    T.tope1DDestroy(fw, t)


def test_1d_batched_256x65536(T, fw, orc):
    """Config 2, batched 256 x 2^16 contiguous rows."""
    n, b = 1 << 16, 256
    x = orc.uniform(n * b, SEED0 + 3)
    got = run1d(T, fw, x, n, 1, batch=b)
    assert orc.rel_l2(got, orc.exec(x, n, batch=b)) <= tol_fp64(n)
    inv = run1d(T, fw, x, n, 0, batch=b)
    assert orc.rel_l2(inv, orc.exec(x, n, dir_=0, batch=b)) <= tol_fp64(n)


@pytest.mark.parametrize("n,b", [(16, 3), (256, 7), (4096, 5), (1 << 15, 3), (2, 6)])
def test_1d_batched_ragged(T, fw, orc, n, b):
    x = orc.uniform(n * b, SEED0 + 4)
    for dir_ in (1, 0):
        got = run1d(T, fw, x, n, dir_, batch=b)
        want = np.concatenate([orc.fft_ld(x[2 * n * i: 2 * n * (i + 1)], n, dir_=dir_)
                               for i in range(b)])
        assert orc.rel_l2(got, want) <= tol_fp64(n)


def test_1d_two_point(T, fw, orc, golden):
    x = orc.uniform(2, int(golden["seed_2x1x1"][0]))
    assert np.array_equal(run1d(T, fw, x, 2, 1), golden["fwd_2x1x1"])
    # true inverse (the reference halves only the real parts, fft1d.c:23-26)
    assert orc.rel_l2(run1d(T, fw, x, 2, 0), orc.fft_ld(x, 2, dir_=0)) <= 1e-16


@pytest.mark.parametrize("n", [3, 5, 6, 7, 11, 12, 13, 27, 100, 1000, 1001])
def test_1d_non_power_of_two(T, fw, orc, golden, n):
    key = f"dftseed_{n}"
    x = orc.uniform(n, int(golden[key][0]) if key in golden else SEED0 + n)
    fwd = run1d(T, fw, x, n, 1)
    tol = 1e-13 * np.log2(n)
    if f"dft_{n}" in golden:
        assert orc.rel_l2(fwd, golden[f"dft_{n}"]) <= tol
    assert orc.rel_l2(fwd, orc.dft_ld(x, n, 1)) <= tol
    assert orc.rel_l2(run1d(T, fw, x, n, 0), orc.dft_ld(x, n, 0)) <= tol


@pytest.mark.parametrize("n", [127, 128, 129, 4095, 10007, 100000, 999983, 3 << 16])
def test_1d_non_power_of_two_long(T, fw, orc, n):
    """Lengths from 128 on that are not powers of two: mixed-radix passes
    when every prime factor is at most 13 (4095, 10^5, 3 * 2^16), else
    chirp-z convolutions; compared with
    the long-double chirp-z oracle (itself pinned to the O(n^2) sum) and,
    where that is quick, with the O(n^2) long-double sum."""
    x = orc.uniform(n, SEED0 + 7 * n)
    tol = 1e-13 * np.log2(n)
    for dir_ in (1, 0):
        got = run1d(T, fw, x, n, dir_)
        assert orc.rel_l2(got, orc.bluestein_ld(x, n, dir_)) <= tol
        if n <= 4095:
            assert orc.rel_l2(got, orc.dft_ld(x, n, dir_)) <= tol


@pytest.mark.parametrize("n,b", [(3, 5), (100, 3), (127, 2), (1000, 4), (4095, 3), (10007, 2)])
def test_1d_non_power_of_two_batched(T, fw, orc, n, b):
    """Batched rows of a non-power-of-two length (mixed-radix passes for 3,
    100, 1000, 4095; the DFT for 127; Bluestein for 10007), each row against
    the long-double oracle."""
    x = orc.uniform(n * b, SEED0 + 11 * n)
    tol = 1e-13 * np.log2(n)
    for dir_ in (1, 0):
        got = run1d(T, fw, x, n, dir_, batch=b)
        want = np.concatenate([orc.bluestein_ld(x[2 * n * i: 2 * n * (i + 1)], n, dir_)
                               for i in range(b)])
        assert orc.rel_l2(got, want) <= tol


def test_1d_non_power_of_two_round_trip(T, fw, orc):
    n = 1000003
    x = orc.uniform(n, SEED0 + 8)
    d = x.copy()
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, n, T.C2C, d)
    T.tope1DExec(fw, t, d, T.FORWARD)
    assert abs(np.dot(d, d) / n / np.dot(x, x) - 1) < 1e-12
    T.tope1DExec(fw, t, d, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(d, x) <= 1e-13 * np.log2(n)
    T.tope1DDestroy(fw, t)


@pytest.mark.parametrize("n", [16, 4096, 1 << 16])
def test_known_answers(T, fw, n):
    delta = np.zeros(2 * n)
    delta[0] = 1.0
    ones = np.zeros(2 * n)
    ones[0::2] = 1.0
    assert np.allclose(run1d(T, fw, delta, n), ones, atol=1e-14, rtol=0)
    want = np.zeros(2 * n)
    want[0] = n
    assert np.allclose(run1d(T, fw, ones, n), want, atol=1e-12 * n, rtol=0)
    k0 = 7
    j = np.arange(n)
    tone = np.empty(2 * n)
    tone[0::2], tone[1::2] = np.cos(2 * np.pi * k0 * j / n), np.sin(2 * np.pi * k0 * j / n)
    want = np.zeros(2 * n)
    want[2 * k0] = n
    assert np.allclose(run1d(T, fw, tone, n), want, atol=1e-11 * n, rtol=0)


@pytest.mark.parametrize("scale_exp", [-1016, -1000, -300, -60, 0, 60, 300, 1000])
def test_scaled_inputs(T, fw, orc, scale_exp):
    """Inputs far outside FP32's range: the double-float path scales each
    tile by a power of two, so results track FP64 at any magnitude."""
    n = 1 << 14
    x = orc.uniform(n, 21) * 2.0 ** scale_exp
    for dir_ in (1, 0):
        assert orc.rel_l2(run1d(T, fw, x, n, dir_), orc.exec(x, n, dir_=dir_)) <= tol_fp64(n)


def test_wide_dynamic_range(T, fw, orc):
    """A tile mixing magnitudes 2^600 apart: the small values are below the
    large ones' rounding level, and the result still meets the gate."""
    n = 4096
    x = orc.uniform(n, 22)
    x[::7] *= 2.0 ** 300
    x[1::7] *= 2.0 ** -300
    for dir_ in (1, 0):
        assert orc.rel_l2(run1d(T, fw, x, n, dir_), orc.fft_ld(x, n, dir_=dir_)) <= tol_fp64(n)


def test_linearity(T, fw, orc):
    n = 1 << 18
    x, y = orc.uniform(n, 11), orc.uniform(n, 12)
    X, Y = run1d(T, fw, x, n), run1d(T, fw, y, n)
    Z = run1d(T, fw, 3.0 * x - 0.5 * y, n)
    assert orc.rel_l2(Z, 3.0 * X - 0.5 * Y) <= tol_fp64(n)


# ---------------------------------------------------------------- 2D / 3D
ND_SHAPES = [(4, 4, 1), (8, 4, 1), (4, 8, 1), (16, 32, 1), (64, 16, 1), (2, 8, 1), (8, 2, 1),
             (1, 16, 1), (512, 4, 1), (4, 512, 1), (4, 65536, 1), (65536, 4, 1), (256, 256, 1),
             (1024, 1024, 1), (4096, 4, 1), (4, 4096, 1), (32, 16384, 1), (16384, 32, 1),
             (4, 4, 4), (8, 16, 32), (16, 4, 64), (4, 8, 16), (2, 4, 8), (64, 64, 64),
             (4, 4096, 4), (4096, 4, 4), (4, 4, 4096), (4, 4, 32768), (128, 32, 256)]


@pytest.mark.parametrize("shape", ND_SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_nd_matches_oracle(T, fw, orc, shape):
    nx, ny, nz = shape
    n = nx * ny * nz
    x = orc.normal(n, SEED0 + n + nx)
    tol = tol_fp64(n)
    for dir_ in (1, 0):
        got = run_nd(T, fw, x, shape, dir_)
        assert orc.rel_l2(got, orc.exec(x, nx, ny, nz, dir_)) <= tol
        if n <= 1 << 14:
            assert orc.rel_l2(got, orc.fft_ld(x, nx, ny, nz, dir_)) <= tol


@pytest.mark.parametrize("shape", [(4096, 4096, 1), (256, 256, 256)], ids=["4096^2", "256^3"])
def test_nd_full_size(T, fw, orc, shape):
    """Config 3: forward vs oracle, then inverse with 1/N back to the input."""
    nx, ny, nz = shape
    n = nx * ny * nz
    x = orc.normal(n, SEED0 + 3)
    d = x.copy()
    if nz == 1:
        t = T.TopePlan2D()
        T.tope2DPlanInit(fw, t, nx, ny, T.C2C, d)
        T.tope2DExec(fw, t, d, T.FORWARD)
        fwd = d.copy()
        T.tope2DExec(fw, t, d, T.INVERSE)
        T.tope2DDestroy(fw, t)
    else:
        t = T.TopePlan3D()
        T.tope3DPlanInit(fw, t, nx, ny, nz, T.C2C, d)
        T.tope3DExec(fw, t, d, T.FORWARD)
        fwd = d.copy()
        T.tope3DExec(fw, t, d, T.INVERSE)
        T.tope3DDestroy(fw, t)
    T.check(fw)
    tol = tol_fp64(n)
    assert orc.rel_l2(fwd, orc.exec(x, nx, ny, nz, 1)) <= tol
    assert orc.rel_l2(d, x) <= tol


@pytest.mark.parametrize("shape", [(64, 64, 64), (256, 128, 1), (32, 16, 512)],
                         ids=["64^3", "256x128", "32x16x512"])
def test_load_paths_agree(T, fw, orc, monkeypatch, shape):
    """Direct tile loads (TOPEFFT_BULK=0), bulk copies of contiguous tiles
    (1, the default) and TMA boxes for strided tiles as well (2) give the
    same transform bit for bit, at the oracle's gate."""
    nx, ny, nz = shape
    x = orc.uniform(nx * ny * nz, SEED0 + 21)
    outs = []
    for level in ("0", "1", "2"):
        monkeypatch.setenv("TOPEFFT_BULK", level)
        outs.append(run_nd(T, fw, x, shape))
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    ref = orc.exec(x, nx, ny, nz, 1)
    assert orc.rel_l2(outs[2], ref) <= tol_fp64(nx * ny * nz)


def test_per_axis_exec(T, fw, orc):
    """tope2DExecX then tope2DExecY == the X and Y passes of a forward Exec."""
    nx, ny = 64, 32
    x = orc.normal(nx * ny, 5)
    d = x.copy()
    t = T.TopePlan2D()
    T.tope2DPlanInit(fw, t, nx, ny, T.C2C, d)
    T.tope2DExecX(fw, t)
    T.check(fw)
    got = np.empty_like(x)
    T.download(fw, t, got)
    want = x.copy()
    orc.lib.oracle_axis(want.ctypes.data_as(orc.lib.oracle_exec.argtypes[0]), nx, ny, 1, 0, 1)
    assert orc.rel_l2(got, want) <= tol_fp64(nx)
    T.tope2DExecY(fw, t)
    T.download(fw, t, got)
    assert orc.rel_l2(got, orc.exec(x, nx, ny, 1, 1)) <= tol_fp64(nx * ny)
    T.tope2DDestroy(fw, t)


# ---------------------------------------------------------------- tables
@pytest.mark.parametrize("lg", [1, 2, 3, 5, 8, 12, 14])
def test_plan_bitrev_table_bit_exact(T, fw, golden, lg):
    n = 1 << lg
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, n, T.C2C, np.zeros(2 * n))
    T.check(fw)
    got = np.empty(n, dtype=np.int32)
    T.copy_to_host(fw, got, t.bitrev)
    assert np.array_equal(got, golden[f"bitrev_{lg}"])
    T.tope1DDestroy(fw, t)


@pytest.mark.parametrize("n", [8, 16, 64, 256, 4096])
def test_plan_twiddle_table(T, fw, golden, n):
    """The plan's quarter-wave table comes from CUDA's sincospi of the exact
    argument 2k/n.  sincospi is not correctly rounded: measured on GB300 its
    worst entry up to n = 8192 is 1.30 ulp from the exact value, so the
    bound is 1.5 ulp.  The reference's cos/sin(2pi*k/n) rounds the angle
    first, so its near-zero components are hundreds of ulps off; both tables
    agree within 4e-16 in absolute terms."""
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, n, T.C2C, np.zeros(2 * n))
    got = np.empty(2 * (n // 4))
    T.copy_to_host(fw, got, t.twiddle)
    T.tope1DDestroy(fw, t)
    k = np.arange(n // 4, dtype=np.longdouble)
    ang = 2 * np.arccos(np.longdouble(-1)) * k / np.longdouble(n)
    exact = np.empty(2 * (n // 4), dtype=np.longdouble)
    exact[0::2], exact[1::2] = np.cos(ang), -np.sin(ang)
    err_ulp = np.abs(got.astype(np.longdouble) - exact) / np.spacing(
        np.maximum(np.abs(got), np.finfo(np.float64).tiny)).astype(np.longdouble)
    assert np.all(err_ulp <= 1.5)
    assert np.max(np.abs(got - golden[f"twiddle_{n}"])) <= 4e-16


def test_swap_permutation_bit_exact(T, fw, orc, golden):
    x = orc.uniform(8 * 16 * 4, SEED0 + 3000)
    for axis in range(3):
        d = x.copy()
        t = T.TopePlan3D()
        T.tope3DPlanInit(fw, t, 8, 16, 4, T.C2C, d)
        T.tope3DBitrevPermute(fw, t, axis)
        T.check(fw)
        T.download(fw, t, d)
        assert np.array_equal(d, golden[f"swap3d_8x16x4_type{axis + 1}"])
        T.tope3DDestroy(fw, t)


# ---------------------------------------------------------------- API edges
def test_exec_device_then_download(T, fw, orc):
    n = 1 << 16
    x = orc.uniform(n, 9)
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, n, T.C2C, x.copy())
    T.execDevice(fw, t, T.FORWARD)
    T.check(fw)
    got = np.empty_like(x)
    T.download(fw, t, got)
    assert orc.rel_l2(got, orc.exec(x, n)) <= tol_fp64(n)
    T.upload(fw, t, x)
    T.execDevice(fw, t, T.INVERSE)
    T.download(fw, t, got)
    assert orc.rel_l2(got, orc.exec(x, n, dir_=0)) <= tol_fp64(n)
    T.tope1DDestroy(fw, t)


def test_errors_do_not_crash(T, fw):
    d = np.zeros(2 * 17 * 8)
    t2 = T.TopePlan2D()
    T.tope2DPlanInit(fw, t2, 17, 8, T.C2C, d)  # the reference exit()s here
    assert fw.error == T.TOPE_ERR_INVALID_SIZE and t2.impl is None
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, 64, T.C2C, np.zeros(128))
    T.check(fw)
    T.tope1DExec(fw, t, np.zeros(128), 5)  # bad direction
    assert fw.error == T.TOPE_ERR_INVALID_ARG
    T.tope1DDestroy(fw, t)
    T.check(fw)
    T.tope1DDestroy(fw, t)  # double destroy
    assert fw.error == T.TOPE_ERR_DESTROYED
    T.tope1DExec(fw, t, np.zeros(128), T.FORWARD)  # use after destroy
    assert fw.error == T.TOPE_ERR_DESTROYED


def test_many_plans_one_framework(T, fw, orc):
    plans = []
    xs = []
    for k, n in enumerate((64, 4096, 1 << 15)):
        x = orc.uniform(n, 100 + k)
        t = T.TopePlan1D()
        T.tope1DPlanInit(fw, t, n, T.C2C, x.copy())
        T.check(fw)
        plans.append((t, n))
        xs.append(x)
    T.tope1DDestroy(fw, plans[0][0])  # the others must survive
    for (t, n), x in list(zip(plans, xs))[1:]:
        d = np.empty_like(x)
        T.tope1DExec(fw, t, d, T.FORWARD)
        T.check(fw)
        assert orc.rel_l2(d, orc.exec(x, n)) <= tol_fp64(n)
        T.tope1DDestroy(fw, t)


@pytest.mark.parametrize("args", [["4096"], ["1048576"], ["64", "64"], ["4", "4096"],
                                  ["32", "32", "32"], ["4", "8", "2048"],
                                  ["1000"], ["100", "60"], ["30", "20", "50"]])
def test_reference_style_c_driver(T, tmp_path, args):
    import subprocess
    from conftest import ROOT
    exe = tmp_path / "tope_driver"
    subprocess.run(["gcc", "-O2", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "drivers" / "tope_driver.c"), "-o", str(exe),
                    f"-L{T.LIB_PATH.parent}", "-ltopefft", f"-Wl,-rpath,{T.LIB_PATH.parent}",
                    "-lm"], check=True)
    r = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


# plans whose Exec reads back 32 MB or more run their last pass in slices and
# copy each slice to the host while the next one computes: contiguous slices
# (batched rows), 2D slices along the sliced line dimension (four-step 1D,
# the y pass of 2D, the z pass of 3D, three-pass 1D lines)
READBACK = [((1 << 24, 1, 1), 1), ((1 << 16, 1, 1), 256), ((1 << 12, 1, 1), 2048),
            ((4096, 4096, 1), 1), ((256, 256, 256), 1), ((64, 128, 512), 1),
            ((1 << 21, 1, 1), 3)]


@pytest.mark.parametrize("shape,batch", READBACK)
def test_overlapped_readback_matches_download(T, fw, orc, shape, batch):
    """Exec into a host buffer (sliced last pass, overlapped copies) returns
    bit for bit what ExecDevice + Download returns, and matches the oracle."""
    nx, ny, nz = shape
    x = orc.uniform(nx * ny * nz * batch, SEED0 + 41)
    if ny == 1 and nz == 1:
        t = T.TopePlan1D()
        T.tope1DBatchPlanInit(fw, t, nx, batch, T.C2C, x.copy())
        ex, ds = T.tope1DExec, T.tope1DDestroy
    elif nz == 1:
        t = T.TopePlan2D()
        T.tope2DPlanInit(fw, t, nx, ny, T.C2C, x.copy())
        ex, ds = T.tope2DExec, T.tope2DDestroy
    else:
        t = T.TopePlan3D()
        T.tope3DPlanInit(fw, t, nx, ny, nz, T.C2C, x.copy())
        ex, ds = T.tope3DExec, T.tope3DDestroy
    T.check(fw)
    for dir_ in (T.FORWARD, T.INVERSE):
        T.upload(fw, t, x)
        got = np.full_like(x, np.nan)
        ex(fw, t, got, dir_)
        T.check(fw)
        T.upload(fw, t, x)
        T.execDevice(fw, t, dir_)
        want = np.full_like(x, np.nan)
        T.download(fw, t, want)
        T.check(fw)
        assert np.array_equal(got, want)
    if batch == 1:
        assert orc.rel_l2(want, orc.exec(x, nx, ny, nz, dir_=0)) <= tol_fp64(nx * ny * nz)
    ds(fw, t)
