"""GPU parity of lines whose length is not a power of two but a product of
2, 3, 5, 7, 11 and 13: they run as mixed-radix Stockham passes (one pass up
to 4096 points, four-step splits beyond), not through the reference's O(N^2)
DFT kernel (src/kernels1D.cl:549-573), which also ignores the direction.

Checked against the long-double O(N^2) sum (dft_ld) where it is quick, else
the long-double chirp-z oracle (bluestein_ld, itself pinned to the sum); 2D
and 3D shapes against the long-double sum applied along each axis.  Gate:
rel-L2 <= 1e-13 * log2 N (FP64 storage); the split-precision forms use
their own gates.
"""
import numpy as np
import pytest

from conftest import SEED0

pytestmark = pytest.mark.gpu


def tol(n):
    return 1e-13 * max(1.0, float(np.log2(n)))


def oracle_1d(orc, x, n, dir_):
    return orc.dft_ld(x, n, dir_) if n <= 5000 else orc.bluestein_ld(x, n, dir_)


def run1d(T, f, x, n, dir_, batch=1):
    d = x.copy()
    t = T.TopePlan1D()
    T.tope1DBatchPlanInit(f, t, n, batch, T.C2C, d)
    T.check(f)
    info = T.pass_times(f, t)
    T.tope1DExec(f, t, d, dir_)
    T.check(f)
    T.tope1DDestroy(f, t)
    return d, info


SIZES = [9, 11, 13, 25, 49, 121, 143, 169, 360, 1001, 1331, 2187, 2197, 2310, 2401, 3125,
         4095, 6000, 12288, 5 ** 7, 100000, 3 ** 11]


@pytest.mark.parametrize("n", SIZES)
def test_1d_mixed(T, fw, orc, n):
    x = orc.uniform(n, SEED0 + 13 * n)
    for dir_ in (1, 0):
        got, info = run1d(T, fw, x, n, dir_)
        assert orc.rel_l2(got, oracle_1d(orc, x, n, dir_)) <= tol(n)
    assert any(p["log_l"] < 0 for p in info)  # at least one mixed-radix pass
    assert int(np.prod([p["len"] for p in info])) == n


_CACHE = {}


def test_1d_mixed_pass_shapes(T, fw, orc):
    """10^6 = 1000 x 1000: two passes of 1000-point lines (8 5 5 5)."""
    n = 10 ** 6
    x = orc.uniform(n, SEED0 + 5)
    got, info = run1d(T, fw, x, n, 1)
    if n not in _CACHE:
        _CACHE[n] = orc.bluestein_ld(x, n, 1)
    assert orc.rel_l2(got, _CACHE[n]) <= tol(n)
    assert [p["len"] for p in info] == [1000, 1000]
    assert [p["four_step_twiddle"] for p in info] == [1, 0]
    _, info = run1d(T, fw, orc.uniform(1000 * 64, 3), 1000, 1, batch=64)
    assert [p["len"] for p in info] == [1000]


@pytest.mark.parametrize("n,b", [(3, 7), (60, 100), (1000, 33), (6000, 3), (4095, 2),
                                 (100000, 2), (400, 250), (250, 400)])
def test_1d_mixed_batched(T, fw, orc, n, b):
    x = orc.uniform(n * b, SEED0 + 17 * n)
    for dir_ in (1, 0):
        got, _ = run1d(T, fw, x, n, dir_, batch=b)
        want = np.concatenate([oracle_1d(orc, x[2 * n * i: 2 * n * (i + 1)], n, dir_)
                               for i in range(b)])
        assert orc.rel_l2(got, want) <= tol(n)


def dft_nd_ld(orc, x, shape, dir_):
    """The long-double O(N^2) sum along each axis in turn (x fastest)."""
    nx, ny, nz = shape
    a = x.reshape(nz, ny, nx, 2)
    for axis, n in ((2, nx), (1, ny), (0, nz)):
        if n == 1:
            continue
        a = np.moveaxis(a, axis, 2).copy()
        flat = a.reshape(-1, n * 2)
        for r in range(flat.shape[0]):
            flat[r] = orc.dft_ld(flat[r].copy(), n, dir_)
        a = np.moveaxis(flat.reshape(a.shape), 2, axis)
    return np.ascontiguousarray(a).reshape(-1)


@pytest.mark.parametrize("shape", [(100, 60, 1), (48, 36, 1), (7, 256, 1), (1024, 10, 1),
                                   (30, 20, 50), (12, 18, 10), (64, 45, 16), (6, 6, 6)])
def test_nd_mixed(T, fw, orc, shape):
    """2D and 3D arrays whose sides are not all powers of two (the reference
    exits on them, src/fft2d.c:355-362)."""
    nx, ny, nz = shape
    x = orc.uniform(nx * ny * nz, SEED0 + nx * ny + nz)
    for dir_ in (1, 0):
        d = x.copy()
        if nz == 1:
            t = T.TopePlan2D()
            T.tope2DPlanInit(fw, t, nx, ny, T.C2C, d)
            T.check(fw)
            T.tope2DExec(fw, t, d, dir_)
            T.tope2DDestroy(fw, t)
        else:
            t = T.TopePlan3D()
            T.tope3DPlanInit(fw, t, nx, ny, nz, T.C2C, d)
            T.check(fw)
            T.tope3DExec(fw, t, d, dir_)
            T.tope3DDestroy(fw, t)
        T.check(fw)
        assert orc.rel_l2(d, dft_nd_ld(orc, x, shape, dir_)) <= tol(nx * ny * nz)


@pytest.mark.parametrize("n", [2000, 2 * 3 ** 7, 2 * 10 ** 6])
def test_r2c_mixed(T, fw, orc, n):
    """Real data of even length n whose half n/2 is a mixed-radix length:
    x/2 + 1 outputs against the complex oracle of the complexified input."""
    rng = np.random.default_rng(n)
    xr = rng.uniform(-1, 1, n)
    d = np.zeros(n + 2)
    d[:n] = xr
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, n, T.R2C, d)
    T.check(fw)
    T.tope1DExec(fw, t, d, T.FORWARD)
    T.check(fw)
    xc = np.zeros(2 * n)
    xc[0::2] = xr
    want = oracle_1d(orc, xc, n, 1)[: n + 2]
    assert orc.rel_l2(d, want) <= tol(n)
    T.tope1DExec(fw, t, d, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(d[:n], xr) <= tol(n)
    T.tope1DDestroy(fw, t)


def smallest_smooth(m, primes=(2, 3, 5, 7)):
    while True:
        r = m
        for p in primes:
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


def bluestein_size(n):
    """The convolution length of a chirp-z plan: the next power of two
    M >= 2N - 1, or the smallest 2^a 3^b 5^c 7^d >= 2N - 1 when that is at
    most 0.6 of it."""
    mp = 1
    while mp < 2 * n - 1:
        mp *= 2
    ms = smallest_smooth(2 * n - 1)
    return ms if 10 * ms <= 6 * mp else mp


@pytest.mark.parametrize("n,m", [(131, 270), (10007, 32768), (17 * 1031, 35280),
                                 (999983, 1 << 21)])
def test_bluestein_size(T, fw, orc, n, m):
    """A length with a prime factor above 13 runs as a chirp-z convolution;
    its sub-transform length follows bluestein_size."""
    assert bluestein_size(n) == m
    x = orc.uniform(n, SEED0 + 3)
    got, info = run1d(T, fw, x, n, 1)
    assert orc.rel_l2(got, orc.bluestein_ld(x, n, 1)) <= tol(n)
    assert int(np.prod([p["len"] for p in info])) == m


@pytest.mark.parametrize("mode", ["accurate", "fast"])
@pytest.mark.parametrize("shape,batch", [((1000, 1, 1), 16), ((60, 60, 60), 1),
                                         ((100000, 1, 1), 1)])
def test_split_precision_mixed(T, orc, mode, shape, batch):
    """The FP32-storage forms on mixed-radix lengths, against the FP64
    oracle of the unrounded input (gates as for powers of two)."""
    gate = {"accurate": 1e-7, "fast": 2.5e-7}[mode]
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.topeSetSplitMode(f, {"accurate": 0, "fast": 1}[mode])
    nx, ny, nz = shape
    x = orc.uniform(nx * ny * nz * batch, SEED0 + 23)
    d = x.astype(np.float32)
    if ny == 1:
        t = T.TopePlan1D()
        T.tope1DBatchPlanInitF32(f, t, nx, batch, T.C2C, d)
        want = np.concatenate([oracle_1d(orc, x[2 * nx * i: 2 * nx * (i + 1)], nx, 1)
                               for i in range(batch)])
    else:
        t = T.TopePlan3D()
        T.tope3DPlanInitF32(f, t, nx, ny, nz, T.C2C, d)
        want = dft_nd_ld(orc, x, shape, 1)
    T.check(f)
    T.execF32(f, t, d, T.FORWARD)
    T.check(f)
    assert orc.rel_l2(d.astype(np.float64), want) <= gate
    T.execF32(f, t, d, T.INVERSE)
    T.check(f)
    assert orc.rel_l2(d.astype(np.float64), x) <= gate
    {T.TopePlan1D: T.tope1DDestroy, T.TopePlan3D: T.tope3DDestroy}[type(t)](f, t)
    T.topeFFTDestroy(f)
