"""GPU parity of batches of uneven transforms (topeBatch*), through the C
interface: every transform of the batch against the CPU oracle, in the three
execution modes (one persistent launch from a CUDA graph, a graph of one
launch per class pass, a loop of per-transform launches)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, SEED0, tol_fp64

pytestmark = pytest.mark.gpu

MODES = {"persistent": 0, "launches": 1, "loop": 2}


def uneven_batch(seed, n1d=120, n2d=8, kmax=18):
    """1D lengths 2^1..2^kmax (direct and four-step classes) and 2D shapes
    with sides 2..512, shuffled, packed back to back."""
    rng = np.random.default_rng(seed)
    nx = list(2 ** rng.integers(1, kmax + 1, n1d))
    ny = [1] * n1d
    sides = [2, 4, 8, 16, 64, 128, 256, 512]
    for _ in range(n2d):
        nx.append(int(rng.choice(sides)))
        ny.append(int(rng.choice(sides)))
    order = rng.permutation(len(nx))
    return [int(nx[i]) for i in order], [int(ny[i]) for i in order]


def oracle_batch(orc, x, nx, ny, dir_):
    out = np.empty_like(x)
    off = 0
    for a, b in zip(nx, ny):
        n = 2 * a * b
        if a * b == 2:
            # the reference's two-point inverse halves only the real parts;
            # the library returns the true inverse
            out[off:off + n] = orc.fft_ld(x[off:off + n], a, b, 1, dir_)
        else:
            out[off:off + n] = orc.exec(x[off:off + n], a, b, 1, dir_)
        off += n
    return out


def per_transform_rel(orc, got, ref, nx, ny):
    errs, off = [], 0
    for a, b in zip(nx, ny):
        n = 2 * a * b
        errs.append(orc.rel_l2(got[off:off + n], ref[off:off + n]))
        off += n
    return np.array(errs)


@pytest.fixture
def tune_cache(tmp_path, monkeypatch):
    path = tmp_path / "tune.txt"
    monkeypatch.setenv("TOPEFFT_TUNE_CACHE", str(path))
    return path


@pytest.mark.parametrize("mode", list(MODES))
def test_batch_matches_oracle(T, fw, orc, tune_cache, mode):
    nx, ny = uneven_batch(7)
    total = sum(a * b for a, b in zip(nx, ny))
    x = orc.uniform(total, SEED0 + 50)
    b = T.TopeBatch()
    T.topeBatchPlanInit(fw, b, nx, ny, T.C2C, x.copy())
    T.check(fw)
    assert b.classes >= 10 and b.work_items > 0 and b.ctas > 0
    T.topeBatchSetMode(fw, b, MODES[mode])
    T.check(fw)
    for dir_ in (T.FORWARD, T.INVERSE):
        T.topeBatchUpload(fw, b, x)
        got = np.empty_like(x)
        T.topeBatchExec(fw, b, got, dir_)
        T.check(fw)
        ref = oracle_batch(orc, x, nx, ny, dir_)
        errs = per_transform_rel(orc, got, ref, nx, ny)
        tols = np.array([tol_fp64(a * bb) for a, bb in zip(nx, ny)])
        bad = np.nonzero(errs > tols)[0]
        assert bad.size == 0, [(nx[i], ny[i], errs[i]) for i in bad[:5]]
    T.topeBatchDestroy(fw, b)
    T.check(fw)


def test_batch_round_trip_device_resident(T, fw, orc, tune_cache):
    nx, ny = uneven_batch(11, n1d=60, n2d=4)
    total = sum(a * b for a, b in zip(nx, ny))
    x = orc.uniform(total, SEED0 + 51)
    b = T.TopeBatch()
    T.topeBatchPlanInit(fw, b, nx, ny, T.C2C, x.copy())
    T.topeBatchExecDevice(fw, b, T.FORWARD)
    T.topeBatchExecDevice(fw, b, T.INVERSE)
    back = np.empty_like(x)
    T.topeBatchDownload(fw, b, back)
    T.check(fw)
    assert orc.rel_l2(back, x) <= tol_fp64(1 << 18)
    assert b.totalKernel > 0
    T.topeBatchDestroy(fw, b)


def test_batch_split_precision(T, orc, tune_cache):
    f = T.TopeFFT()
    T.topeFFTInit(f)
    nx, ny = uneven_batch(13, n1d=80, n2d=6)
    total = sum(a * b for a, b in zip(nx, ny))
    x = orc.uniform(total, SEED0 + 52)
    x32 = x.astype(np.float32)
    b = T.TopeBatch()
    T.topeBatchPlanInit(f, b, nx, ny, T.C2C, x32.copy())
    T.check(f)
    assert b.elem_bytes == 8
    got = np.empty_like(x32)
    T.topeBatchExec(f, b, got, T.FORWARD)
    T.check(f)
    ref = oracle_batch(orc, x, nx, ny, 1)
    errs = per_transform_rel(orc, got.astype(np.float64), ref, nx, ny)
    assert errs.max() <= 1e-7, errs.max()
    T.topeBatchDestroy(f, b)
    T.topeFFTDestroy(f)


def test_batch_autotune_cache_written_and_reused(T, fw, orc, tune_cache):
    nx, ny = [1 << 14] * 8 + [1 << 16] * 4, [1] * 12
    total = sum(nx)
    x = orc.uniform(total, 3)
    b = T.TopeBatch()
    T.topeBatchPlanInit(fw, b, nx, ny, T.C2C, x.copy())
    T.check(fw)
    text = tune_cache.read_text()
    assert "log2n=14" in text and "log2n=16" in text
    T.topeBatchDestroy(fw, b)
    b2 = T.TopeBatch()
    T.topeBatchPlanInit(fw, b2, nx, ny, T.C2C, x.copy())  # served from the cache
    T.check(fw)
    assert tune_cache.read_text() == text
    got = np.empty_like(x)
    T.topeBatchExec(fw, b2, got, T.FORWARD)
    assert orc.rel_l2(got, oracle_batch(orc, x, nx, ny, 1)) <= tol_fp64(1 << 16)
    T.topeBatchDestroy(fw, b2)


def config5_shapes():
    """The uneven-batch benchmark configuration, drawn as bench.py draws it:
    20,000 1D transforms of 2^k points, k uniform on 6..16, then 500 2D
    transforms with sides drawn independently from {64, ..., 1024}."""
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    import bench
    return bench.uneven_shapes()


def config5_sample(nx, ny, count=500, seed=SEED0 + 55):
    """At least `count` transform indices: the first transform of every
    shape class (all eleven 1D lengths and every 2D class, those with a 1024
    side among them), then a seeded draw of the rest."""
    first = {}
    for i, shape in enumerate(zip(nx, ny)):
        first.setdefault(shape, i)
    idx = set(first.values())
    for i in np.random.default_rng(seed).permutation(len(nx)):
        if len(idx) >= count:
            break
        idx.add(int(i))
    return sorted(idx)


@pytest.mark.parametrize("arith", ["fp64", "split_accurate"])
def test_batch_full_size_configuration(T, orc, tune_cache, arith):
    """The whole benchmark batch (20,500 transforms, 322 M points) in one plan,
    in the persistent structure and in the per-class launch graph; a seeded
    sample of at least 500 transforms, one of every shape class among them,
    against the oracle (FP64 gate, or 1e-7 for FP32 data against the oracle
    of the unrounded input)."""
    nx, ny = config5_shapes()
    assert len(nx) == 20500 and max(nx) == 1 << 16
    assert {(a, b) for a, b in zip(nx, ny) if b > 1 and 1024 in (a, b)}
    offs = np.concatenate([[0], np.cumsum([2 * a * b for a, b in zip(nx, ny)])]).astype(np.int64)
    x = orc.uniform(int(offs[-1]) // 2, SEED0 + 6)
    sample = config5_sample(nx, ny)
    assert len(sample) >= 500
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.check(f)
    if arith == "fp64":
        T.topeSetArith(f, T.TOPE_ARITH_FP64)
        data = x
    else:
        T.topeSetSplitMode(f, 0)
        data = x.astype(np.float32)
    b = T.TopeBatch()
    T.topeBatchPlanInit(f, b, nx, ny, T.C2C, data)
    T.check(f)
    refs = {i: orc.exec(x[offs[i]:offs[i + 1]], nx[i], ny[i], 1, 1) for i in sample}
    got = np.empty_like(data)
    for mode in ("persistent", "launches"):
        T.topeBatchSetMode(f, b, MODES[mode])
        T.check(f)
        got[:] = np.nan
        T.topeBatchUpload(f, b, data)
        T.topeBatchExec(f, b, got, T.FORWARD)
        T.check(f)
        bad = []
        for i in sample:
            n = nx[i] * ny[i]
            err = orc.rel_l2(got[offs[i]:offs[i + 1]].astype(np.float64), refs[i])
            gate = tol_fp64(n) if arith == "fp64" else 1e-7
            if not err <= gate:
                bad.append((mode, nx[i], ny[i], err))
        assert not bad, bad[:5]
    T.topeBatchDestroy(f, b)
    T.topeFFTDestroy(f)


def test_batch_rejects_bad_sizes(T, fw):
    b = T.TopeBatch()
    T.topeBatchPlanInit(fw, b, [64, 48], [1, 1], T.C2C, np.zeros(2 * 112))
    assert fw.error == T.TOPE_ERR_INVALID_SIZE and b.impl is None
    T.topeBatchPlanInit(fw, b, [64, 8192], [64, 2], T.C2C, np.zeros(2 * (4096 + 16384)))
    assert fw.error == T.TOPE_ERR_INVALID_SIZE
    T.topeBatchExec(fw, b, None, T.FORWARD)
    assert fw.error == T.TOPE_ERR_DESTROYED


STALL_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import __graft_entry__ as g
T = g.load_package()
f = T.TopeFFT(); T.topeFFTInit(f); T.check(f)
nx, ny = [64, 128, 256], [64, 32, 16]
x = np.ones(2 * sum(a * b for a, b in zip(nx, ny)))
b = T.TopeBatch(); T.topeBatchPlanInit(f, b, nx, ny, T.C2C, x.copy()); T.check(f)
T.topeBatchExec(f, b, x, T.FORWARD)
print("status", f.error)
T.topeBatchDestroy(f, b)
# the context is still usable: a normal transform after the timeout
d = np.zeros(2 * 1024); d[0] = 1.0
t = T.TopePlan1D(); T.tope1DPlanInit(f, t, 1024, T.C2C, d); T.tope1DExec(f, t, d, T.FORWARD)
T.check(f)
print("after", float(d[0::2].min()), float(d[0::2].max()))
T.tope1DDestroy(f, t)
"""


def test_batch_bounded_wait_reports_timeout(tmp_path):
    """A dependency that can never be met (test hook) makes the persistent
    kernel's bounded wait run out: the kernel raises its error flag and
    returns, the host reports TOPE_ERR_TIMEOUT, and the GPU stays usable."""
    env = dict(os.environ, TOPEFFT_BATCH_TEST_STALL="1", TOPEFFT_AUTOTUNE="0",
               TOPEFFT_TUNE_CACHE=str(tmp_path / "t.txt"))
    r = subprocess.run([sys.executable, "-c", STALL_SCRIPT.format(root=str(ROOT))],
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    assert int(lines["status"]) == 8  # TOPE_ERR_TIMEOUT
    lo, hi = map(float, lines["after"].split())
    assert lo == pytest.approx(1.0) and hi == pytest.approx(1.0)
