"""Pin the CPU oracle (CPU only).

The reference ships no golden vectors (its test drivers only print
timings), so the oracle is pinned against fixtures produced by the
reference's own kernel source run on host cores (tests/golden/make_golden.py)
and against independent long-double transforms.
"""
import numpy as np
import pytest

from conftest import SEED0

SHAPES = [(2, 1, 1), (4, 1, 1), (8, 1, 1), (16, 1, 1), (32, 1, 1), (64, 1, 1), (128, 1, 1),
          (256, 1, 1), (512, 1, 1), (1024, 1, 1), (4096, 1, 1), (4, 4, 1), (8, 4, 1), (4, 8, 1),
          (16, 32, 1), (64, 16, 1), (32, 32, 1), (4, 4, 4), (8, 16, 32), (16, 4, 64), (4, 8, 16)]

# Rounding-level agreement with the reference's kernels: the oracle evaluates
# the radix-8 butterfly as three radix-2 layers, the reference in its own
# order, so results differ by a few ulps, not bit for bit.
PIN_TOL = 2e-15


def splitmix64_np(seed: int, idx: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (idx.astype(np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def test_generator_pinned(orc, golden):
    assert np.array_equal(orc.uniform(32, SEED0), golden["gen_uniform"])
    assert np.array_equal(orc.normal(32, SEED0), golden["gen_normal"])
    # the same stream restated in numpy (element 2e -> re, 2e+1 -> im)
    z = splitmix64_np(SEED0, np.arange(64))
    u = (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    assert np.array_equal(2 * u - 1, golden["gen_uniform"])
    x = orc.uniform(1 << 12, 7)
    assert x.min() >= -1 and x.max() < 1 and abs(x.mean()) < 0.05


def test_radix_rule(orc):
    # fft1d.c:317-329: 8 if log2n % 3 == 0, else 4 if even, else 2
    expect = {12: 8, 16: 4, 24: 8, 8: 4, 9: 8, 14: 4, 13: 2, 1: 2, 2: 4, 3: 8}
    for lg, r in expect.items():
        assert orc.radix(lg) == r


@pytest.mark.parametrize("lg", range(1, 15))
def test_bitrev_table_bit_exact(orc, golden, lg):
    assert np.array_equal(orc.bitrev_table(lg), golden[f"bitrev_{lg}"])


@pytest.mark.parametrize("n", [8, 16, 64, 256, 4096])
def test_twiddle_table(orc, golden, n):
    a, b = orc.twiddle_table(n), golden[f"twiddle_{n}"]
    ulp = np.abs(a - b) / np.spacing(np.maximum(np.abs(b), 1e-300))
    assert np.all((a == b) | (ulp <= 1.0))


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("dir_", [1, 0], ids=["fwd", "inv"])
def test_oracle_matches_reference_kernels(orc, golden, shape, dir_):
    nx, ny, nz = shape
    key = f"{nx}x{ny}x{nz}"
    x = orc.uniform(nx * ny * nz, int(golden[f"seed_{key}"][0]))
    ref = golden[("fwd_" if dir_ else "inv_") + key]
    got = orc.exec(x, nx, ny, nz, dir_)
    assert orc.rel_l2(got, ref) <= PIN_TOL
    if nx * ny * nz <= 4:
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_oracle_matches_long_double(orc, golden, shape):
    nx, ny, nz = shape
    n = nx * ny * nz
    x = orc.uniform(n, SEED0 + 17)
    # the reference's two-point inverse is not an inverse (see below)
    dirs = (1,) if n == 2 else (1, 0)
    for dir_ in dirs:
        assert orc.rel_l2(orc.exec(x, nx, ny, nz, dir_), orc.fft_ld(x, nx, ny, nz, dir_)) <= 1e-15


def test_reference_two_point_inverse_quirk(orc, golden):
    """fft1d.c:23-26 divides only d[0] and d[2] (the real parts) by 2 on the
    inverse, so the imaginary parts come back twice too large.  The oracle
    restates that; the library returns the true inverse by default."""
    x = orc.uniform(2, int(golden["seed_2x1x1"][0]))
    quirk = golden["inv_2x1x1"]
    assert np.array_equal(orc.exec(x, 2, dir_=0), quirk)
    true_inv = orc.fft_ld(x, 2, dir_=0)
    assert np.allclose(quirk[0::2], true_inv[0::2], rtol=0, atol=1e-16)
    assert np.allclose(quirk[1::2], 2 * true_inv[1::2], rtol=0, atol=1e-16)


def test_reference_driver_inputs(orc, golden):
    for n in (8, 64, 1024):
        x = np.zeros(2 * n)
        x[0::2] = np.arange(1, n + 1)
        assert orc.rel_l2(orc.exec(x, n), golden[f"ramp_fwd_{n}"]) <= PIN_TOL
    for (nx, ny, nz) in ((16, 8, 1), (8, 8, 4)):
        n = nx * ny * nz
        x = np.zeros(2 * n)
        x[0::2] = np.sin(2 * np.pi * np.arange(n) / n)
        assert orc.rel_l2(orc.exec(x, nx, ny, nz), golden[f"sin_fwd_{nx}x{ny}x{nz}"]) <= PIN_TOL


@pytest.mark.parametrize("n", [3, 5, 6, 7, 11, 12, 13, 27, 100, 1000, 1001])
def test_dft_path(orc, golden, n):
    x = orc.uniform(n, int(golden[f"dftseed_{n}"][0]))
    ref = golden[f"dft_{n}"]
    # same expression order as kernels1D.cl:561-564, so bit for bit
    assert np.array_equal(orc.dft_ref(x, n), ref)
    # the reference's DFT is a correct forward transform, to the FP64 gate
    # (its unreduced angle 2 pi j k / n loses accuracy as j k grows: 1.8e-13
    # at n = 1000 against 2e-16 for an exact-index sum)
    assert orc.rel_l2(ref, orc.dft_ld(x, n, 1)) <= 1e-13 * max(1.0, np.log2(n))


def test_swap_pass_is_bit_reversal(orc, golden):
    x = orc.uniform(8 * 16 * 4, SEED0 + 3000).reshape(4, 16, 8, 2)
    for ax, (axis, lg) in zip((1, 2, 3), ((2, 3), (1, 4), (0, 2))):
        rev = orc.bitrev_table(lg)
        want = np.take(x, rev, axis=axis).ravel()
        assert np.array_equal(want, golden[f"swap3d_8x16x4_type{ax}"])


@pytest.mark.parametrize("n", [16, 1024, 1 << 14])
def test_known_answers(orc, n):
    delta = np.zeros(2 * n)
    delta[0] = 1.0
    ones = np.zeros(2 * n)
    ones[0::2] = 1.0
    assert np.allclose(orc.exec(delta, n), ones, atol=1e-15, rtol=0)
    const = ones.copy()
    want = np.zeros(2 * n)
    want[0] = n
    assert np.allclose(orc.exec(const, n), want, atol=1e-12 * n, rtol=0)
    k0 = 5
    j = np.arange(n)
    tone = np.empty(2 * n)
    tone[0::2], tone[1::2] = np.cos(2 * np.pi * k0 * j / n), np.sin(2 * np.pi * k0 * j / n)
    want = np.zeros(2 * n)
    want[2 * k0] = n
    assert np.allclose(orc.exec(tone, n), want, atol=1e-11 * n, rtol=0)


def test_parseval_linearity_roundtrip(orc):
    n = 1 << 12
    x, y = orc.uniform(n, 1), orc.uniform(n, 2)
    X = orc.exec(x, n)
    assert abs(np.sum(X * X) / n / np.sum(x * x) - 1) < 1e-13
    Z = orc.exec(2.5 * x - y, n)
    assert orc.rel_l2(Z, 2.5 * X - orc.exec(y, n)) < 1e-15
    assert orc.rel_l2(orc.exec(X, n, dir_=0), x) < 1e-15


@pytest.mark.parametrize("n", [3, 7, 100, 129, 1000, 4095])
@pytest.mark.parametrize("dir_", [1, 0], ids=["fwd", "inv"])
def test_bluestein_ld_matches_direct_sum(orc, n, dir_):
    """The long-double chirp-z oracle (used for long non-power-of-two lines)
    agrees with the O(n^2) long-double sum and, for powers of two, with the
    long-double FFT."""
    x = orc.uniform(n, 300 + n)
    assert orc.rel_l2(orc.bluestein_ld(x, n, dir_), orc.dft_ld(x, n, dir_)) <= 5e-17
    p = 1 << 11
    y = orc.uniform(p, 301)
    assert orc.rel_l2(orc.bluestein_ld(y, p, dir_), orc.fft_ld(y, p, dir_=dir_)) <= 5e-17


@pytest.mark.parametrize("shape", [(6, 10, 1), (12, 8, 5), (7, 3, 9), (16, 15, 1)])
@pytest.mark.parametrize("dir_", [1, 0], ids=["fwd", "inv"])
def test_nd_long_double_any_sides(orc, shape, dir_):
    """The long-double ND oracle on sides that are not powers of two (the
    O(n^2) sum along such axes) agrees with numpy's FFT, and its 1D form
    with the direct sum."""
    nx, ny, nz = shape
    x = orc.uniform(nx * ny * nz, 400 + nx)
    got = orc.fft_ld(x, nx, ny, nz, dir_=dir_)
    c = (x[0::2] + 1j * x[1::2]).reshape(nz, ny, nx)
    want = np.fft.fftn(c) if dir_ == 1 else np.fft.ifftn(c)
    w = np.empty(2 * c.size)
    w[0::2], w[1::2] = want.real.ravel(), want.imag.ravel()
    assert orc.rel_l2(got, w) <= 1e-15
    assert orc.rel_l2(orc.fft_ld(x[: 2 * nx], nx, dir_=dir_), orc.dft_ld(x[: 2 * nx], nx, dir_)) <= 1e-17
