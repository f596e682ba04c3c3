"""GPU parity of 1D lines longer than two on-chip passes cover: more than 2^26
points with FP64 storage (2^13 per pass), more than 2^28 with FP32 storage
(2^14 per pass).  Such a line runs as three four-step passes; the
reference's own 1D path takes any power of two its int32 indices allow
(fft1d.c:303-370).

FP64 storage: 2^27 points against the oracle's restatement of the reference
(gate rel-L2 <= 1e-13 * log2 N), single and batched, plus the round trip.
FP32 storage: 2^29 points (4 GB), a sum of three tones whose exact spectrum
is known, and the round trip, gated per split mode as in test_gpu_f32.
"""
import numpy as np
import pytest

from conftest import SEED0, tol_fp64

pytestmark = pytest.mark.gpu

_ORACLE = {}


def oracle_fwd(orc, x, n, batch, key):
    """The oracle's forward transform, computed once per input for both
    butterfly arithmetics."""
    if key not in _ORACLE:
        _ORACLE[key] = orc.exec(x, n, batch=batch)
    return _ORACLE[key]


@pytest.mark.parametrize("batch", [1, 2])
def test_1d_three_passes(T, fw, orc, batch):
    lg = 27
    n = 1 << lg
    x = orc.uniform(n * batch, SEED0 + 27 + batch)
    d = x.copy()
    t = T.TopePlan1D()
    if batch == 1:
        T.tope1DPlanInit(fw, t, n, T.C2C, d)
    else:
        T.tope1DBatchPlanInit(fw, t, n, batch, T.C2C, d)
    T.check(fw)
    passes = T.pass_times(fw, t)
    assert [p["log_l"] for p in passes] == [9, 9, 9]
    assert [p["four_step_twiddle"] for p in passes] == [1, 1, 0]
    assert [p["out_of_place"] for p in passes] == [0, 0, 1]
    T.tope1DExec(fw, t, d, T.FORWARD)
    T.check(fw)
    tol = tol_fp64(n)
    assert orc.rel_l2(d, oracle_fwd(orc, x, n, batch, (n, batch))) <= tol
    T.tope1DExec(fw, t, d, T.INVERSE)
    T.check(fw)
    assert orc.rel_l2(d, x) <= tol
    T.tope1DDestroy(fw, t)


GATES = {"accurate": 1e-7, "fast": 2.5e-7, "tensor": 1e-7}
MODES = {"accurate": 0, "fast": 1, "tensor": 2}
TONES = ((1, 1.0), (12345677, 0.5), (-3, 0.25j))


def three_tones(n):
    """x_j = sum_t a_t exp(2 pi i k_t j / n) in FP64, and its FP32 rounding
    interleaved as (re, im)."""
    j = np.arange(n, dtype=np.int64)
    x = np.zeros(n, dtype=np.complex128)
    for k, a in TONES:
        m = (j * (k % n)) & (n - 1)
        x += a * np.exp(2j * np.pi * (m.astype(np.float64) / n))
    return x.astype(np.complex64).view(np.float32)


@pytest.mark.parametrize("mode", ["accurate", "fast", "tensor"])
def test_1d_three_passes_f32(T, mode):
    lg = 29
    n = 1 << lg
    if "x29" not in _ORACLE:
        _ORACLE.clear()
        _ORACLE["x29"] = three_tones(n)
    x32 = _ORACLE["x29"]
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.check(f)
    T.topeSetSplitMode(f, MODES[mode])
    d = x32.copy()
    t = T.TopePlan1D()
    T.tope1DBatchPlanInitF32(f, t, n, 1, T.C2C, d)
    T.check(f)
    assert len(T.pass_times(f, t)) == 3
    T.execF32(f, t, d, T.FORWARD)
    T.check(f)
    y = d.view(np.complex64).astype(np.complex128)
    ref2 = 0.0
    for k, a in TONES:
        y[k % n] -= n * a
        ref2 += abs(n * a) ** 2
    assert np.sqrt(float(np.vdot(y, y).real) / ref2) <= GATES[mode]
    del y
    T.execF32(f, t, d, T.INVERSE)
    T.check(f)
    a = d.astype(np.float64)
    b = x32.astype(np.float64)
    assert np.sqrt(np.sum((a - b) ** 2) / np.sum(b * b)) <= GATES[mode]
    T.tope1DDestroy(f, t)
    T.topeFFTDestroy(f)


LINE_TONES = (((7, 1.0), ((1 << 29) + 12345, 0.5), (-3, 0.25j)),
              ((1, 0.75j), (99999989, -0.5), ((1 << 30) - 7, 0.125)))


def tones_on_device(n, tones, chunk=1 << 26):
    """sum_t a_t exp(2 pi i k_t j / n), j < n, computed on the GPU in FP64
    (exact integer phases j k mod n) in chunks and rounded to complex64 on
    the host."""
    import torch
    dev = torch.device("cuda", 0)
    out = np.empty(n, dtype=np.complex64)
    for s in range(0, n, chunk):
        j = torch.arange(s, min(s + chunk, n), dtype=torch.int64, device=dev)
        re = torch.zeros(j.numel(), dtype=torch.float64, device=dev)
        im = torch.zeros_like(re)
        for k, a in tones:
            ph = (j * (k % n)) % n
            ang = ph.to(torch.float64) * (2 * np.pi / n)
            c, sn = torch.cos(ang), torch.sin(ang)
            re += a.real * c - a.imag * sn
            im += a.real * sn + a.imag * c
        out[s:s + j.numel()] = (re.cpu().numpy() + 1j * im.cpu().numpy()).astype(np.complex64)
        del j, re, im
    torch.cuda.synchronize(dev)
    return out


@pytest.mark.parametrize("mode", ["accurate", "tensor"])
def test_1d_offsets_beyond_2p31_f32(T, mode):
    """Two lines of 2^30 FP32 points (16 GB per buffer): the second line's
    elements sit at offsets 2^30 .. 2^31 - 1 of the array (2^31 .. 2^32 - 1
    floats), past any int32 index (the reference's are int32,
    src/kernels3D.cl:71-78).  Three four-step passes of 2^10 each; every
    line's spectrum is three known tones (different per line, so a mix-up
    of lines shows), then the round trip."""
    lg = 30
    n = 1 << lg
    if "x30" not in _ORACLE:
        _ORACLE.clear()
        _ORACLE["x30"] = np.concatenate([tones_on_device(n, t) for t in LINE_TONES])
    x32 = _ORACLE["x30"].view(np.float32)
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.check(f)
    T.topeSetSplitMode(f, MODES[mode])
    d = x32.copy()
    t = T.TopePlan1D()
    T.tope1DBatchPlanInitF32(f, t, n, 2, T.C2C, d)
    T.check(f)
    assert [p["log_l"] for p in T.pass_times(f, t)] == [10, 10, 10]
    T.execF32(f, t, d, T.FORWARD)
    T.check(f)
    y = d.view(np.complex64)
    err2, ref2 = 0.0, 0.0
    chunk = 1 << 26
    for line, tones in enumerate(LINE_TONES):
        spikes = {(k % n): n * a for k, a in tones}
        ref2 += sum(abs(v) ** 2 for v in spikes.values())
        for s in range(0, n, chunk):
            seg = y[line * n + s: line * n + s + chunk].astype(np.complex128)
            for k, v in spikes.items():
                if s <= k < s + chunk:
                    seg[k - s] -= v
            err2 += float(np.vdot(seg, seg).real)
    assert np.sqrt(err2 / ref2) <= GATES[mode]
    T.execF32(f, t, d, T.INVERSE)
    T.check(f)
    num, den = 0.0, 0.0
    for s in range(0, 4 * n, chunk):
        a = d[s:s + chunk].astype(np.float64)
        b = x32[s:s + chunk].astype(np.float64)
        num += float(np.sum((a - b) ** 2))
        den += float(np.sum(b * b))
    assert np.sqrt(num / den) <= GATES[mode]
    T.tope1DDestroy(f, t)
    T.topeFFTDestroy(f)


def test_1d_three_passes_mixed_radix(T, fw):
    """3^16 = 43,046,721 points: more than two 4096-point passes can hold, so
    three mixed-radix passes (243 x 243 x 729), with
    four-step factors of a length that is not a power of two at two levels.
    Input: two tones, whose spectrum is known exactly; then the round trip."""
    n = 3 ** 16
    tones = ((1234567, 1.0), (n - 5, 0.5j))
    j = np.arange(n, dtype=np.int64)
    z = np.zeros(n, dtype=np.complex128)
    for k, a in tones:
        z += a * np.exp(2j * np.pi * (((j * k) % n).astype(np.float64) / n))
    x = z.view(np.float64).copy()
    del z, j
    d = x.copy()
    t = T.TopePlan1D()
    T.tope1DPlanInit(fw, t, n, T.C2C, d)
    T.check(fw)
    passes = T.pass_times(fw, t)
    assert len(passes) == 3 and int(np.prod([p["len"] for p in passes])) == n
    T.tope1DExec(fw, t, d, T.FORWARD)
    T.check(fw)
    y = d.view(np.complex128).copy()
    ref2 = 0.0
    for k, a in tones:
        y[k] -= n * a
        ref2 += abs(n * a) ** 2
    assert np.sqrt(float(np.vdot(y, y).real) / ref2) <= 1e-13 * np.log2(n)
    del y
    T.tope1DExec(fw, t, d, T.INVERSE)
    T.check(fw)
    assert np.sqrt(np.sum((d - x) ** 2) / np.sum(x * x)) <= 1e-13 * np.log2(n)
    T.tope1DDestroy(fw, t)
