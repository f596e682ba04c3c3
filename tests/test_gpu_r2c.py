"""GPU parity of the real-data (R2C) plans, through the C interface.

topefft.h defines R2C (src/topefft.h:9) but the reference never implements
it; these plans follow the usual convention: x real points per row in, the
x/2 + 1 non-redundant outputs X[0..x/2] out (unnormalised forward), and an
inverse that returns the reals scaled by 1/x.  The oracle is the long-double
transform of the same reals taken as complex values with zero imaginary
parts.  Gate: rel-L2 <= 1e-13 * log2(x).
"""
import numpy as np
import pytest

from conftest import SEED0

pytestmark = pytest.mark.gpu


def oracle_spectrum(orc, xr, n, batch):
    """X[0..n/2] of each row, long double, from the complexified reals."""
    out = []
    for b in range(batch):
        z = np.zeros(2 * n)
        z[0::2] = xr[b * n:(b + 1) * n]
        if n & (n - 1) == 0:
            zz = orc.fft_ld(z, n, dir_=1)
        elif n <= 4096:
            zz = orc.dft_ld(z, n, 1)
        else:
            zz = orc.bluestein_ld(z, n, 1)
        out.append(zz[:2 * (n // 2 + 1)])
    return np.concatenate(out)


def make_plan(T, f, n, batch, d):
    t = T.TopePlan1D()
    if batch == 1:
        T.tope1DPlanInit(f, t, n, T.R2C, d)
    else:
        T.tope1DBatchPlanInit(f, t, n, batch, T.R2C, d)
    T.check(f)
    return t


SIZES = [(2, 1), (4, 1), (8, 3), (16, 1), (64, 5), (4096, 1), (4096, 7), (1 << 16, 2), (1 << 20, 1),
         (6, 1), (100, 2), (1000, 1), (514, 3), (100000, 1)]


@pytest.mark.parametrize("n,batch", SIZES, ids=lambda v: str(v))
def test_r2c_forward_and_round_trip(T, fw, orc, n, batch):
    xr = orc.uniform(n * batch // 2, SEED0 + n)
    d = np.zeros((n + 2) * batch)
    d[:n * batch] = xr
    t = make_plan(T, fw, n, batch, d)
    T.tope1DExec(fw, t, d, T.FORWARD)
    T.check(fw)
    tol = 1e-13 * max(1.0, np.log2(n))
    want = oracle_spectrum(orc, xr, n, batch)
    assert orc.rel_l2(d, want) <= tol
    # the device now holds the spectrum: the inverse brings the reals back
    back = np.zeros((n + 2) * batch)
    T.tope1DExec(fw, t, back, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(back[:n * batch], xr) <= tol
    T.tope1DDestroy(fw, t)
    T.check(fw)


@pytest.mark.parametrize("n", [16, 4096, 1 << 18, 1000])
def test_c2r_from_uploaded_spectrum(T, fw, orc, n):
    """An inverse from a spectrum given by the caller: the reals whose forward
    transform it is (a Hermitian-consistent spectrum from the oracle)."""
    xr = orc.uniform(n // 2, SEED0 + 3 * n)
    spec = oracle_spectrum(orc, xr, n, 1)
    t = make_plan(T, fw, n, 1, np.zeros(n + 2))
    T.upload_spectrum(fw, t, spec)
    T.check(fw)
    out = np.zeros(n + 2)
    T.tope1DExec(fw, t, out, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(out[:n], xr) <= 1e-13 * np.log2(n)
    # Download after an inverse returns the real rows
    got = np.zeros(n)
    T.download(fw, t, got)
    assert np.array_equal(got, out[:n])
    T.tope1DDestroy(fw, t)


def test_r2c_device_resident_chain(T, fw, orc):
    """Upload / ExecDevice / Download on a real-data plan."""
    n, batch = 1 << 14, 4
    xr = orc.uniform(n * batch // 2, SEED0 + 9)
    t = make_plan(T, fw, n, batch, np.zeros((n + 2) * batch))
    T.upload(fw, t, xr)
    T.execDevice(fw, t, T.FORWARD)
    spec = np.zeros((n + 2) * batch)
    T.download(fw, t, spec)
    T.check(fw)
    assert orc.rel_l2(spec, oracle_spectrum(orc, xr, n, batch)) <= 1e-13 * 14
    T.execDevice(fw, t, T.INVERSE)
    back = np.zeros(n * batch)
    T.download(fw, t, back)
    T.check(fw)
    assert orc.rel_l2(back, xr) <= 1e-13 * 14
    T.tope1DDestroy(fw, t)


def test_r2c_rejects_bad_shapes(T, fw):
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, 7, T.R2C, np.zeros(16))
    assert fw.error == T.TOPE_ERR_INVALID_SIZE and not t.impl
    t2 = T.TopePlan2D()
    T.tope2DPlanInit(fw, t2, 7, 8, T.R2C, np.zeros(128))  # odd x
    assert fw.error == T.TOPE_ERR_INVALID_SIZE and not t2.impl
    T.tope2DPlanInit(fw, t2, 8, 17, T.R2C, np.zeros(8 * 17))  # y with a prime factor > 13
    assert fw.error == T.TOPE_ERR_INVALID_SIZE and not t2.impl


# ---------------------------------------------------------------- 2D / 3D
def oracle_spectrum_nd(orc, xr, dims):
    """X[kz][ky][kx], kx <= nx/2, kx fastest, long double, from the
    complexified reals."""
    nx, ny, nz = dims
    z = np.zeros(2 * nx * ny * nz)
    z[0::2] = xr
    zz = orc.fft_ld(z, nx, ny, nz, dir_=1).reshape(nz, ny, nx, 2)
    return np.ascontiguousarray(zz[:, :, : nx // 2 + 1, :]).ravel()


def make_plan_nd(T, f, dims, d):
    nx, ny, nz = dims
    if nz == 1:
        t = T.TopePlan2D()
        T.tope2DPlanInit(f, t, nx, ny, T.R2C, d)
    else:
        t = T.TopePlan3D()
        T.tope3DPlanInit(f, t, nx, ny, nz, T.R2C, d)
    T.check(f)
    return t


def destroy_nd(T, f, t):
    (T.tope2DDestroy if isinstance(t, T.TopePlan2D) else T.tope3DDestroy)(f, t)
    T.check(f)


ND = [(8, 4, 1), (64, 32, 1), (512, 256, 1), (4096, 4096, 1), (2, 2, 1), (16, 8, 4),
      (64, 32, 16), (256, 256, 256), (32, 1 << 14, 1),
      # sides with factors 3, 5, 7 (x/2 = 50, 45, 21): mixed-radix passes
      (100, 60, 1), (90, 12, 14), (42, 25, 1)]


@pytest.mark.parametrize("dims", ND, ids=lambda d: "x".join(map(str, d)))
def test_r2c_nd_forward_and_round_trip(T, fw, orc, dims):
    nx, ny, nz = dims
    n = nx * ny * nz
    xr = orc.uniform(n // 2, SEED0 + 5 * nx + ny)
    d = np.zeros((nx + 2) * ny * nz)
    d[:n] = xr
    t = make_plan_nd(T, fw, dims, d)
    exec_fn = T.tope2DExec if nz == 1 else T.tope3DExec
    exec_fn(fw, t, d, T.FORWARD)
    T.check(fw)
    tol = 1e-13 * max(1.0, np.log2(n))
    if n <= 1 << 20:
        assert orc.rel_l2(d, oracle_spectrum_nd(orc, xr, dims)) <= tol
    back = np.zeros((nx + 2) * ny * nz)
    exec_fn(fw, t, back, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(back[:n], xr) <= tol
    destroy_nd(T, fw, t)


@pytest.mark.parametrize("dims", [(64, 32, 1), (16, 8, 4)], ids=lambda d: "x".join(map(str, d)))
def test_c2r_nd_from_uploaded_spectrum(T, fw, orc, dims):
    nx, ny, nz = dims
    n = nx * ny * nz
    xr = orc.uniform(n // 2, SEED0 + 13)
    t = make_plan_nd(T, fw, dims, np.zeros(n))
    T.upload_spectrum(fw, t, oracle_spectrum_nd(orc, xr, dims))
    T.check(fw)
    out = np.zeros((nx + 2) * ny * nz)
    (T.tope2DExec if nz == 1 else T.tope3DExec)(fw, t, out, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(out[:n], xr) <= 1e-13 * np.log2(n)
    # single-axis execution is for complex plans only
    if nz == 1:
        T.tope2DExecX(fw, t)
        assert fw.error == T.TOPE_ERR_UNSUPPORTED
    destroy_nd(T, fw, t)


# ---------------------------------------------------------------- FP32 storage
SPLIT_GATES = {"accurate": 1e-7, "fast": 2.5e-7, "tensor": 1e-7}
SPLIT_CASES = [((4096, 1, 1), 1), ((1 << 20, 1, 1), 1), ((64, 1, 1), 33), ((1 << 14, 1, 1), 64),
               ((1000, 1, 1), 8), ((256, 128, 1), 1), ((64, 32, 16), 1), ((100, 60, 1), 1)]


@pytest.mark.parametrize("mode", ["accurate", "fast", "tensor"])
@pytest.mark.parametrize("dims,batch", SPLIT_CASES, ids=lambda v: str(v))
def test_r2c_split_precision(T, orc, mode, dims, batch):
    """R2C/C2R with FP32 storage in each split mode, against the FP64 oracle
    of the unrounded reals; the spectrum uploaded back gives the reals."""
    nx, ny, nz = dims
    if mode == "tensor" and any(v & (v - 1) for v in (nx // 2, ny, nz)):
        pytest.skip("the tensor form runs power-of-two lines only")
    gate = SPLIT_GATES[mode]
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.topeSetSplitMode(f, {"accurate": 0, "fast": 1, "tensor": 2}[mode])
    n = nx * ny * nz
    xr = orc.uniform(n * batch // 2, SEED0 + 31 + nx)
    d = np.zeros((nx + 2) * ny * nz * batch, dtype=np.float32)
    d[:n * batch] = xr
    if ny == 1 and nz == 1:
        t = T.TopePlan1D()
        T.tope1DBatchPlanInitF32(f, t, nx, batch, T.R2C, d)
        want = oracle_spectrum(orc, xr, nx, batch)
    elif nz == 1:
        t = T.TopePlan2D()
        T.tope2DPlanInitF32(f, t, nx, ny, T.R2C, d)
        want = oracle_spectrum_nd(orc, xr, dims)
    else:
        t = T.TopePlan3D()
        T.tope3DPlanInitF32(f, t, nx, ny, nz, T.R2C, d)
        want = oracle_spectrum_nd(orc, xr, dims)
    T.check(f)
    T.execF32(f, t, d, T.FORWARD)
    T.check(f)
    assert orc.rel_l2(d.astype(np.float64), want) <= gate
    # a round trip carries the error of two transforms: 1.5x the gate
    T.execF32(f, t, d, T.INVERSE)
    T.check(f)
    assert orc.rel_l2(d[:n * batch].astype(np.float64), xr) <= 1.5 * gate
    T.upload_spectrum(f, t, want.astype(np.float32))
    T.check(f)
    back = np.zeros_like(d)
    T.execF32(f, t, back, T.INVERSE)
    T.check(f)
    assert orc.rel_l2(back[:n * batch].astype(np.float64), xr) <= gate
    {T.TopePlan1D: T.tope1DDestroy, T.TopePlan2D: T.tope2DDestroy,
     T.TopePlan3D: T.tope3DDestroy}[type(t)](f, t)
    T.topeFFTDestroy(f)
