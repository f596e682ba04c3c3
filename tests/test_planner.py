"""The host planner on the CPU.  topefft.c and batch.c are linked with a
host-only stand-in for the CUDA side (tests/drivers/abi_stub.c): plans are
built through the public entry points and their pass structure is read back
with topePassInfo, with no GPU.  Covers the decisions the GPU tests rely on:
one pass or a four-step split, three-pass lines, the small-transform shape,
mixed-radix splits, the Bluestein sub-transform size, real-data row plans and
the tensor form's tiles, plans of up to 2^33 points in every form, staged
tiles and tensor maps, and (with hypothesis) random power-of-two and smooth
plans whose passes must cover every axis.

The host code is built with UndefinedBehaviorSanitizer where the compiler has
its runtime: a signed overflow, an out-of-range shift or a misaligned access in
the planner is reported on stderr, and every test here fails on such a report."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from conftest import ROOT

UBSAN = ["-fsanitize=undefined"]


def ubsan_ok(tmp):
    src = tmp / "probe_ub.c"
    src.write_text("int main(void) { return 0; }\n")
    return subprocess.run(["gcc", *UBSAN, str(src), "-o", str(tmp / "probe_ub")],
                          capture_output=True).returncode == 0


@pytest.fixture(scope="module")
def S(T, tmp_path_factory):
    d = tmp_path_factory.mktemp("stub")
    out = d / "libtopefft_stub.so"
    csrc = ROOT / "tope-fft_gb300" / "csrc"
    san = UBSAN if ubsan_ok(d) else []
    subprocess.run(["gcc", "-O1", "-g", "-fPIC", "-shared", "-std=gnu11", *san, f"-I{csrc}",
                    f"-I{ROOT / 'include'}", str(csrc / "topefft.c"), str(csrc / "batch.c"),
                    str(ROOT / "tests" / "drivers" / "abi_stub.c"), "-o", str(out)], check=True)
    return T.load_library(out)


@pytest.fixture(autouse=True)
def no_ubsan_report(capfd):
    yield
    err = capfd.readouterr().err
    assert "runtime error" not in err, err[-2000:]


@pytest.fixture
def fw(T, S):
    f = T.TopeFFT()
    S.topeFFTInit(C.byref(f))
    assert f.error == T.TOPE_SUCCESS
    yield f
    S.topeFFTDestroy(C.byref(f))


def passes(S, f, t):
    n = S.topePassTimes(C.byref(f), t.impl, None, None, 0)
    info = (C.c_int64 * 6)()
    out = []
    for i in range(n):
        assert S.topePassInfo(C.byref(f), t.impl, i, info) == 0
        out.append({"len": (1 << info[0]) if info[0] >= 0 else -info[0], "b": info[1],
                    "ctas": info[2], "threads": info[3], "oop": info[4], "tw": info[5]})
    return out


def plan1d(T, S, f, n, batch=1, real=False, f32=False):
    t = T.TopePlan1D()
    fn = S.tope1DBatchPlanInitF32 if f32 else S.tope1DBatchPlanInit
    fn(C.byref(f), C.byref(t), n, batch, T.R2C if real else T.C2C, None)
    return t


@pytest.mark.parametrize("n,lens,tw,oop", [
    (1 << 20, [1024, 1024], [1, 0], [0, 1]),
    (1 << 27, [512, 512, 512], [1, 1, 0], [0, 0, 1]),
    (10 ** 6, [1000, 1000], [1, 0], [0, 1]),
    (4096, [64, 64], [1, 0], [0, 1]),
    (1001, [1001], [0], [0]),
    (6000, [80, 75], [1, 0], [0, 1]),
    (2048 * 3, [64, 96], [1, 0], [0, 1]),
])
def test_1d_pass_structure(T, S, fw, n, lens, tw, oop):
    t = plan1d(T, S, fw, n)
    assert fw.error == T.TOPE_SUCCESS
    p = passes(S, fw, t)
    assert [q["len"] for q in p] == lens
    assert [q["tw"] for q in p] == tw
    assert [q["oop"] for q in p] == oop
    S.tope1DDestroy(C.byref(fw), C.byref(t))


def test_small_transform_runs_4_points_per_thread(T, S, fw):
    """A lone 4096-point line: two passes of 64-point lines, 32 CTAs of 32
    threads (4 points per thread); batched, one 4096-point pass."""
    p = passes(S, fw, plan1d(T, S, fw, 4096))
    assert [(q["b"], q["ctas"], q["threads"]) for q in p] == [(2, 32, 32), (2, 32, 32)]
    p = passes(S, fw, plan1d(T, S, fw, 4096, batch=64))
    assert [q["len"] for q in p] == [4096] and p[0]["threads"] == 256


@pytest.mark.parametrize("n", [12288, 3 ** 16, 5 ** 9, 2 * 3 * 5 * 7 * 11 * 13 * 16])
def test_mixed_splits(T, S, fw, n):
    """Every pass fits one CTA (<= 4096 points, or a power of two <= 2^13) and
    the pass lengths multiply to n."""
    p = passes(S, fw, plan1d(T, S, fw, n))
    assert fw.error == T.TOPE_SUCCESS
    assert int(np.prod([q["len"] for q in p])) == n
    for q in p:
        L = q["len"]
        assert (L & (L - 1) == 0 and L <= 8192) or L <= 4096
    assert len(p) == (3 if n > 4096 * 4096 else 2)


@pytest.mark.parametrize("n,m", [(131, 270), (10007, 32768), (17 * 1031, 35280),
                                 (999983, 1 << 21)])
def test_bluestein_sub_transform_size(T, S, fw, n, m):
    p = passes(S, fw, plan1d(T, S, fw, n))
    assert int(np.prod([q["len"] for q in p])) == m


def test_small_primes_use_the_dft(T, S, fw):
    t = plan1d(T, S, fw, 127)
    assert fw.error == T.TOPE_SUCCESS and passes(S, fw, t) == []


@pytest.mark.parametrize("dims,lens", [((100, 60, 1), [100, 60]), ((30, 20, 50), [30, 20, 50]),
                                       ((1 << 14, 4, 1), [128, 128, 4])])
def test_nd_pass_structure(T, S, fw, dims, lens):
    nx, ny, nz = dims
    if nz == 1:
        t = T.TopePlan2D()
        S.tope2DPlanInit(C.byref(fw), C.byref(t), nx, ny, T.C2C, None)
    else:
        t = T.TopePlan3D()
        S.tope3DPlanInit(C.byref(fw), C.byref(t), nx, ny, nz, T.C2C, None)
    assert fw.error == T.TOPE_SUCCESS
    assert [q["len"] for q in passes(S, fw, t)] == lens


def test_nd_rejects_large_prime_sides(T, S, fw):
    t = T.TopePlan2D()
    S.tope2DPlanInit(C.byref(fw), C.byref(t), 17, 8, T.C2C, None)
    assert fw.error == T.TOPE_ERR_INVALID_SIZE and not t.impl


def test_real_plans_transform_half_length_rows(T, S, fw):
    p = passes(S, fw, plan1d(T, S, fw, 2000, real=True))
    assert [q["len"] for q in p] == [1000]
    # 2D: the rows (50 complex points each), then the y pass over the
    # 51-column spectrum, 51 lines of 60 points
    t = T.TopePlan2D()
    S.tope2DPlanInit(C.byref(fw), C.byref(t), 100, 60, T.R2C, None)
    assert fw.error == T.TOPE_SUCCESS
    p = passes(S, fw, t)
    assert [q["len"] for q in p] == [50, 60]
    assert p[1]["ctas"] * p[1]["b"] >= 51
    assert S.topePassInfo(C.byref(fw), t.impl, 2, (C.c_int64 * 6)()) == -1
    fw.error = 0
    t3 = T.TopePlan3D()
    S.tope3DPlanInit(C.byref(fw), C.byref(t3), 16, 12, 10, T.R2C, None)
    assert fw.error == T.TOPE_SUCCESS
    assert [q["len"] for q in passes(S, fw, t3)] == [8, 12, 10]


def test_split_precision_shapes(T, S, fw):
    """FP32 storage takes 2^14-point lines in one pass, so 2^29 points are three
    passes; 2^24..2^26 points take three short passes too (2^23, as a real
    plan's line, keeps two); the tensor form uses its fixed tiles and rejects
    mixed radix."""
    p = passes(S, fw, plan1d(T, S, fw, 1 << 29, f32=True))
    assert [q["len"] for q in p] == [1024, 1024, 512]
    p = passes(S, fw, plan1d(T, S, fw, 1 << 24, f32=True))
    assert [q["len"] for q in p] == [256, 256, 256]
    p = passes(S, fw, plan1d(T, S, fw, 1 << 23, f32=True))
    assert [q["len"] for q in p] == [4096, 2048]
    p = passes(S, fw, plan1d(T, S, fw, 1 << 24))
    assert [q["len"] for q in p] == [4096, 4096]
    S.topeSetSplitMode(C.byref(fw), 2)
    p = passes(S, fw, plan1d(T, S, fw, 1 << 20, f32=True))
    assert [(q["len"], q["b"]) for q in p] == [(1024, 4), (1024, 4)]
    t = plan1d(T, S, fw, 1000, f32=True)
    assert fw.error == T.TOPE_ERR_INVALID_SIZE and not t.impl


# ---------------------------------------------------------------- read-back slicing
def call_log(S):
    S.stub_log_count.restype = C.c_int
    S.stub_log_get.argtypes = [C.c_int, C.POINTER(C.c_int64)]
    rec = (C.c_int64 * 8)()
    out = []
    for i in range(S.stub_log_count()):
        S.stub_log_get(i, rec)
        out.append(list(rec))
    return out


def exec_log(T, S, f, t, exec_fn, host):
    S.stub_log_clear()
    exec_fn(C.byref(f), C.byref(t), host.ctypes.data_as(C.POINTER(C.c_double)), T.FORWARD)
    assert f.error == T.TOPE_SUCCESS
    return call_log(S), host.ctypes.data


def test_readback_slices_1d_four_step(T, S, fw):
    """2^24 points = 4096 x 4096: pass B runs as 8 launches of 512 lines, each
    followed by a 2D copy of 4096 rows of 512 elements (8 KB), 64 KB apart."""
    n = 1 << 24
    t = plan1d(T, S, fw, n)
    log, base = exec_log(T, S, fw, t, S.tope1DExec, np.zeros(2))
    launches = [r for r in log if r[0] == 1]
    copies = [r for r in log if r[0] == 3]
    assert len(launches) == 1 + 8 and not [r for r in log if r[0] == 2]
    assert [r[1] for r in launches[1:]] == [512] * 8
    out = launches[1][5]
    for k, r in enumerate(copies):
        assert r[1] - base == 16 * 512 * k and r[2] - out == 16 * 512 * k
        assert r[3:7] == [16 * 512, 4096, 16 * 4096, 16 * 4096]
    assert [r[5] - launches[1][5] for r in launches[1:]] == [16 * 512 * k for k in range(8)]


def test_readback_slices_batched_rows(T, S, fw):
    """256 rows of 2^16: the last pass is cut along the rows, 32 rows (32 MB)
    per contiguous copy."""
    t = plan1d(T, S, fw, 1 << 16, batch=256)
    log, base = exec_log(T, S, fw, t, S.tope1DExec, np.zeros(2))
    copies = [r for r in log if r[0] == 2]
    assert len(copies) == 8
    assert [r[1] - base for r in copies] == [k * 32 * 16 * 65536 for k in range(8)]
    assert all(r[3] == 32 * 16 * 65536 for r in copies)


def test_readback_slices_3d_z_pass(T, S, fw):
    """256^3: the z pass is cut along its 65536 (x, y) lines, 8192 per slice;
    each slice is 256 rows of 8192 elements, one per z, 1 MB apart."""
    t = T.TopePlan3D()
    S.tope3DPlanInit(C.byref(fw), C.byref(t), 256, 256, 256, T.C2C, None)
    log, base = exec_log(T, S, fw, t, S.tope3DExec, np.zeros(2))
    copies = [r for r in log if r[0] == 3]
    assert len(copies) == 8
    for k, r in enumerate(copies):
        assert r[1] - base == 16 * 8192 * k
        assert r[3:7] == [16 * 8192, 256, 16 * 65536, 16 * 65536]


def test_readback_not_sliced_when_small_or_real(T, S, fw):
    for t in (plan1d(T, S, fw, 1 << 20), plan1d(T, S, fw, 1 << 22, real=True)):
        log, _ = exec_log(T, S, fw, t, S.tope1DExec, np.zeros(2))
        assert len([r for r in log if r[0] == 2]) == 1 and not [r for r in log if r[0] == 3]


@pytest.mark.parametrize("n,batch", [(1 << 24, 1), (1 << 16, 256), (1 << 27, 1), (10 ** 6, 1)])
def test_inverse_flags_on_first_and_last_pass(T, S, fw, n, batch):
    """An inverse runs as conj(F(conj x)) / N: the first launch conjugates on
    load, every launch of the last pass (each read-back slice) conjugates and
    scales on store, and nothing in between does."""
    t = plan1d(T, S, fw, n, batch=batch)
    S.stub_log_clear()
    S.tope1DExec(C.byref(fw), C.byref(t), np.zeros(2).ctypes.data_as(C.POINTER(C.c_double)),
                 T.INVERSE)
    assert fw.error == T.TOPE_SUCCESS
    launches = [r for r in call_log(S) if r[0] == 1]
    npass = len(passes(S, fw, t))
    flags = [r[7] for r in launches]
    assert flags[0] & 1 and not any(f & 1 for f in flags[1:])
    last = len(launches) - (npass - 1)  # launches of the last pass
    assert all(f & 6 == 6 for f in flags[-last:])
    assert not any(f & 6 for f in flags[:-last])


@pytest.mark.parametrize("dir_,flags", [(1, [0, 0, 1, 6]), (0, [0, 0, 1, 6])])
def test_bluestein_runs_the_convolution_both_ways(T, S, fw, dir_, flags):
    """N = 10007: each Exec runs the 32768-point sub-plan forward (plain) and
    inverse (conjugated in and out, scaled by 1/M), whatever the direction;
    the direction only conjugates the chirp steps around it."""
    t = plan1d(T, S, fw, 10007)
    S.stub_log_clear()
    S.tope1DExec(C.byref(fw), C.byref(t), np.zeros(2).ctypes.data_as(C.POINTER(C.c_double)),
                 dir_)
    assert fw.error == T.TOPE_SUCCESS
    launches = [r for r in call_log(S) if r[0] == 1]
    assert [r[7] for r in launches] == flags


# ---------------------------------------------------------------- the largest plans
BIG = 1 << 31


def smooth(n):
    for p in (2, 3, 5, 7, 11, 13):
        while n % p == 0:
            n //= p
    return n == 1


@pytest.mark.parametrize("f32,real,dims,batch,status", [
    (0, 0, (1 << 30, 1, 1), 1, 0),            # three power-of-two passes
    (0, 0, (BIG - 1, 1, 1), 1, 0),            # prime: Bluestein over 2^32 points
    (0, 0, (3 ** 19, 1, 1), 1, 0),            # three mixed-radix passes
    (0, 0, (1000, 1, 1), 1 << 21, 0),         # 2^31 points in short rows
    (0, 0, (2, 1, 1), 1 << 30, 0),
    (0, 0, (65536, 32768, 1), 1, 0),
    (0, 0, (46656, 46656, 1), 1, 0),          # 6^6 sides
    (0, 0, (2048, 2048, 1024), 1, 0),         # 2^32 points
    (0, 0, (1, 2, 1 << 30), 1, 0),            # length-1 and length-2 axes
    (0, 0, (1536, 1536, 1536), 1, 0),         # 3.6e9 points, mixed radix
    (1, 0, (1 << 30, 1, 1), 1, 0),
    (1, 0, (3 ** 19, 1, 1), 1, 0),
    (1, 0, (BIG - 1, 1, 1), 1, 1),            # FP32 storage: no Bluestein
    (1, 0, (2048, 2048, 2048), 1, 0),         # 2^33 points (64 GB of FP32)
    (0, 1, (BIG - 2, 1, 1), 1, 0),            # real rows of 2^30 - 1 complex points
    (0, 1, (2, 1, 1), 1 << 30, 0),            # one complex point per row: no pass
    (0, 1, (65536, 32768, 1), 1, 0),
    (0, 1, (1536, 1536, 1536), 1, 0),
    (1, 1, (BIG - 2, 1, 1), 1, 1),
    (1, 1, (2048, 2048, 2048), 1, 0),
], ids=lambda v: str(v))
def test_largest_plans(T, S, fw, f32, real, dims, batch, status):
    """Plans of 2^31 to 2^33 points (int-sized sides, 64-bit totals): the
    status, and for every pass a grid that fits a launch (at most 2^31 - 1
    CTAs) and tiles that cover the pass's points.  Each plan also runs both
    directions through the stand-in's launches and is destroyed."""
    nx, ny, nz = dims
    ndim = 1 if batch > 1 or (ny == 1 and nz == 1) else (2 if nz == 1 else 3)
    kind = T.R2C if real else T.C2C
    if ndim == 1:
        t = T.TopePlan1D()
        init = S.tope1DBatchPlanInitF32 if f32 else S.tope1DBatchPlanInit
        init(C.byref(fw), C.byref(t), nx, batch, kind, None)
        run, destroy = S.tope1DExecDevice, S.tope1DDestroy
    elif ndim == 2:
        t = T.TopePlan2D()
        init = S.tope2DPlanInitF32 if f32 else S.tope2DPlanInit
        init(C.byref(fw), C.byref(t), nx, ny, kind, None)
        run, destroy = S.tope2DExecDevice, S.tope2DDestroy
    else:
        t = T.TopePlan3D()
        init = S.tope3DPlanInitF32 if f32 else S.tope3DPlanInit
        init(C.byref(fw), C.byref(t), nx, ny, nz, kind, None)
        run, destroy = S.tope3DExecDevice, S.tope3DDestroy
    assert fw.error == status
    if status:
        assert not t.impl
        fw.error = 0
        return
    points = nx * ny * nz * batch
    # the complex points each pass covers: all of them, half of them for real
    # rows (at least that for the y/z passes over the x/2 + 1 spectrum
    # columns), or the Bluestein sub-transform's M >= 2N - 1
    covered = points // 2 if real else points
    line = nx // 2 if real else nx
    bluestein = ndim == 1 and not smooth(line)
    for q in passes(S, fw, t):
        assert 1 <= q["ctas"] <= BIG - 1, q
        tile = q["ctas"] * q["b"] * q["len"]
        if bluestein:
            assert tile >= 2 * covered - 1, q
        else:
            assert covered <= tile < 2 * covered, q
    for dir_ in (T.FORWARD, T.INVERSE):
        run(C.byref(fw), C.byref(t), dir_)
        assert fw.error == T.TOPE_SUCCESS
    destroy(C.byref(fw), C.byref(t))
    assert fw.error == T.TOPE_SUCCESS and not t.impl


# ---------------------------------------------------------------- staged tiles
def staging_log(T, S, fw, monkeypatch, arith, level):
    """Plan 256^3 in `arith` with TOPEFFT_BULK=`level` (None: unset) and the
    stub answering as the real library, run it on the device (no read-back
    slicing) and return (tensor maps as (rank, dims, strides, box), launch
    flags per pass)."""
    if level is None:
        monkeypatch.delenv("TOPEFFT_BULK", raising=False)
    else:
        monkeypatch.setenv("TOPEFFT_BULK", level)
    S.topeSetArith(C.byref(fw), arith)
    S.stub_set_staging(1)
    try:
        S.stub_log_clear()
        t = T.TopePlan3D()
        S.tope3DPlanInit(C.byref(fw), C.byref(t), 256, 256, 256, T.C2C, None)
        assert fw.error == T.TOPE_SUCCESS
        recs = call_log(S)
        maps = []
        for a, b in zip(recs, recs[1:]):
            if a[0] == 4:
                rank = a[1]
                maps.append((rank, a[2:2 + rank], b[1:rank], [a[6], a[7], b[4], b[5]][:rank]))
        S.stub_log_clear()
        S.tope3DExecDevice(C.byref(fw), C.byref(t), T.FORWARD)
        assert fw.error == T.TOPE_SUCCESS
        flags = [r[7] & 24 for r in call_log(S) if r[0] == 1]
        S.tope3DDestroy(C.byref(fw), C.byref(t))
        return maps, flags
    finally:
        S.stub_set_staging(0)


def test_staged_tiles_and_tensor_maps(T, S, fw, monkeypatch):
    """256^3: the x pass (contiguous lines, 16 per CTA) stages its tiles by
    bulk copies; the y and z passes (adjacent strided lines) by TMA boxes
    from tensor maps in 8-byte units, dimension 0 the adjacent lines, then the
    line and the other line dimensions by stride, box 16 lines x 256 points.
    By default only the double-float FP64 arithmetic takes the maps;
    TOPEFFT_BULK=2 gives them to native FP64 too, 1 keeps the bulk copies
    only, 0 loads every tile directly."""
    y_map = (3, [512, 256, 256], [16 * 256, 16 * 65536], [32, 256, 1])
    z_map = (2, [2 * 65536, 256], [16 * 65536], [32, 256])
    maps, flags = staging_log(T, S, fw, monkeypatch, T.TOPE_ARITH_DF64, None)
    assert maps == [y_map, z_map] and flags == [16, 8, 8]
    maps, flags = staging_log(T, S, fw, monkeypatch, T.TOPE_ARITH_FP64, None)
    assert maps == [] and flags == [16, 0, 0]
    maps, flags = staging_log(T, S, fw, monkeypatch, T.TOPE_ARITH_FP64, "2")
    assert maps == [y_map, z_map] and flags == [16, 8, 8]
    maps, flags = staging_log(T, S, fw, monkeypatch, T.TOPE_ARITH_DF64, "1")
    assert maps == [] and flags == [16, 0, 0]
    maps, flags = staging_log(T, S, fw, monkeypatch, T.TOPE_ARITH_DF64, "0")
    assert maps == [] and flags == [0, 0, 0]


def test_readback_slices_drop_the_tensor_map(T, S, fw, monkeypatch):
    """A read-back slice of the last pass covers part of the array, which the
    pass's tensor map does not describe: its launches load directly."""
    monkeypatch.delenv("TOPEFFT_BULK", raising=False)
    S.topeSetArith(C.byref(fw), T.TOPE_ARITH_DF64)
    S.stub_set_staging(1)
    try:
        t = T.TopePlan3D()
        S.tope3DPlanInit(C.byref(fw), C.byref(t), 256, 256, 256, T.C2C, None)
        log, _ = exec_log(T, S, fw, t, S.tope3DExec, np.zeros(2))
        launches = [r for r in log if r[0] == 1]
        assert len(launches) == 2 + 8
        assert launches[1][7] & 8 and not any(r[7] & 8 for r in launches[2:])
        S.tope3DDestroy(C.byref(fw), C.byref(t))
    finally:
        S.stub_set_staging(0)


# ---------------------------------------------------------------- properties
hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")


@hyp.settings(max_examples=200, deadline=None,
              suppress_health_check=[hyp.HealthCheck.function_scoped_fixture])
@hyp.given(dims=st.lists(st.integers(0, 13), min_size=1, max_size=3),
           lg1d=st.integers(1, 30), batch_lg=st.integers(0, 6),
           form=st.sampled_from(["fp64", "df64", "accurate", "fast", "tensor"]))
def test_power_of_two_plans_cover_every_axis(T, S, fw, dims, lg1d, batch_lg, form):
    """Any power-of-two plan within the limits: every pass is a shape the
    kernels have, runs at most 1024 threads per CTA, and the pass lengths
    multiply to the transform's size (each axis split into passes whose
    lengths multiply to its own length); FP32-storage lines of 2^24..2^26
    points take three passes, FP64-storage ones two."""
    f32 = form in ("accurate", "fast", "tensor")
    S.topeSetArith(C.byref(fw), T.TOPE_ARITH_DF64 if form == "df64" else T.TOPE_ARITH_FP64)
    S.topeSetSplitMode(C.byref(fw), {"accurate": 0, "fast": 1, "tensor": 2}.get(form, 0))
    if len(dims) == 1:
        n, batch = 1 << lg1d, 1 << batch_lg
        if n * batch > 1 << 30:
            return
        t = plan1d(T, S, fw, n, batch=batch, f32=f32)
        total = n
        destroy = S.tope1DDestroy
    else:
        sides = [1 << (d + 1) for d in dims] + [1] * (3 - len(dims))
        total = sides[0] * sides[1] * sides[2]
        if total > 1 << 30:
            return
        if len(dims) == 2:
            t = T.TopePlan2D()
            (S.tope2DPlanInitF32 if f32 else S.tope2DPlanInit)(
                C.byref(fw), C.byref(t), sides[0], sides[1], T.C2C, None)
            destroy = S.tope2DDestroy
        else:
            t = T.TopePlan3D()
            (S.tope3DPlanInitF32 if f32 else S.tope3DPlanInit)(
                C.byref(fw), C.byref(t), sides[0], sides[1], sides[2], T.C2C, None)
            destroy = S.tope3DDestroy
    assert fw.error == T.TOPE_SUCCESS, (dims, lg1d, batch_lg, form)
    p = passes(S, fw, t)
    if len(dims) == 1 and lg1d == 1 and batch_lg == 0 and not f32:
        # a lone 2-point line is the reference's own N == 2 kernel (fft1d.c:16-28)
        assert p == []
        destroy(C.byref(fw), C.byref(t))
        return
    prod = 1
    for q in p:
        assert q["threads"] <= 1024 and q["ctas"] >= 1
        prod *= q["len"]
    assert prod == total
    if len(dims) == 1 and 24 <= lg1d <= 26:
        assert len(p) == (3 if f32 else 2)
    destroy(C.byref(fw), C.byref(t))
    assert fw.error == T.TOPE_SUCCESS


@hyp.settings(max_examples=200, deadline=None,
              suppress_health_check=[hyp.HealthCheck.function_scoped_fixture])
@hyp.given(a=st.integers(0, 12), b=st.integers(0, 8), c=st.integers(0, 6), d=st.integers(0, 4),
           e=st.integers(0, 2), g=st.integers(0, 2),
           form=st.sampled_from(["fp64", "df64", "accurate", "fast"]))
def test_smooth_lengths_split_into_their_factors(T, S, fw, a, b, c, d, e, g, form):
    """1D lengths 2^a 3^b 5^c 7^d 11^e 13^f up to 2^30 points: the plan
    succeeds and its passes' lengths multiply to n (mixed-radix passes for the
    odd factors, power-of-two passes otherwise)."""
    n = 2 ** a * 3 ** b * 5 ** c * 7 ** d * 11 ** e * 13 ** g
    if n < 3 or n > 1 << 30:
        return
    f32 = form in ("accurate", "fast")
    S.topeSetArith(C.byref(fw), T.TOPE_ARITH_DF64 if form == "df64" else T.TOPE_ARITH_FP64)
    S.topeSetSplitMode(C.byref(fw), {"accurate": 0, "fast": 1}.get(form, 0))
    t = plan1d(T, S, fw, n, f32=f32)
    assert fw.error == T.TOPE_SUCCESS, (n, form)
    p = passes(S, fw, t)
    prod = 1
    for q in p:
        assert q["threads"] <= 1024 and q["ctas"] >= 1
        prod *= q["len"]
    assert prod == n, (n, form, [q["len"] for q in p])
    S.tope1DDestroy(C.byref(fw), C.byref(t))
