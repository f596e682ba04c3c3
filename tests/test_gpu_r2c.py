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


def test_r2c_rejects_odd_and_split_precision(T, fw):
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, 7, T.R2C, np.zeros(16))
    assert fw.error == T.TOPE_ERR_INVALID_SIZE and not t.impl
    T.tope1DBatchPlanInitF32(fw, t, 64, 1, T.R2C, np.zeros(130, dtype=np.float32))
    assert fw.error == T.TOPE_ERR_UNSUPPORTED and not t.impl
    t2 = T.TopePlan2D()
    T.tope2DPlanInit(fw, t2, 8, 8, T.R2C, np.zeros(128))
    assert fw.error == T.TOPE_ERR_UNSUPPORTED and not t2.impl
