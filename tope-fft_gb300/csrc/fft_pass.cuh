/*
 * The pass kernel: batched power-of-two FFTs of length L = 2^LOG_L <= 8192,
 * one tile of B lines per CTA, entirely on chip.
 *
 * Algorithm (replaces the reference's swap pass plus one global-memory pass
 * per radix stage, src/fft1d.c:41-114, src/kernels1D.cl:15-547):
 *   - each thread owns E = min(16, L) points of one line, loaded with a
 *     coalesced pattern: thread j holds elements j + q*L/E (q < E);
 *   - Stockham autosort stages: an optional first stage of radix
 *     2^(LOG_L mod 4) and then radix-16 stages, each a register butterfly
 *     preceded by W_{Ns*R}^{r*k} twiddles from a per-L table (one rounding
 *     per factor, sincospi in FP64); stages exchange through shared memory
 *     laid out as (q + q/16) * B + b, q = p with low bits flipped per shape
 *     (sidx), which keeps every stage's reads and writes free of bank
 *     conflicts;
 *   - the result comes out in natural order in the same registers, so no
 *     bit-reversal permutation pass is needed;
 *   - fused on the way out: optional four-step twiddle, conjugation and the
 *     exact 1/N scaling of the inverse (src/kernels1D.cl:499-503).
 * Thread (j, b) maps to threadIdx.x = j*B + b, so the B lines of a tile are
 * the fastest-varying thread index: when lines are adjacent in memory
 * (strided axes of 2D/3D arrays and the four-step passes) each group of B
 * threads reads or writes B*16 contiguous bytes.
 */
#pragma once
#include <type_traits>
#include <utility>

#include "fft_arith.cuh"
#include "tfft_abi.h"

namespace tfft {

template <class A>
__host__ __device__ __forceinline__ void dft2(typename A::C &a0, typename A::C &a1)
{
    typename A::C t = A::sub(a0, a1);
    a0 = A::add(a0, a1);
    a1 = t;
}

template <class A>
__host__ __device__ __forceinline__ void dft4(typename A::C &a0, typename A::C &a1,
                                     typename A::C &a2, typename A::C &a3)
{
    using C = typename A::C;
    C t0 = A::add(a0, a2), t1 = A::sub(a0, a2);
    C t2 = A::add(a1, a3), t3 = A::mul_mi(A::sub(a1, a3));
    a0 = A::add(t0, t2);
    a2 = A::sub(t0, t2);
    a1 = A::add(t1, t3);
    a3 = A::sub(t1, t3);
}

/* 8 = 4 (inner, stride-2 inputs) x 2 (outer) */
template <class A>
__host__ __device__ __forceinline__ void dft8(typename A::C *c)
{
    using C = typename A::C;
    dft4<A>(c[0], c[2], c[4], c[6]);
    dft4<A>(c[1], c[3], c[5], c[7]);
    c[3] = A::mul_w8(c[3]);
    c[5] = A::mul_mi(c[5]);
    c[7] = A::mul_w8_3(c[7]);
    C y[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        y[k] = A::add(c[2 * k], c[2 * k + 1]);
        y[k + 4] = A::sub(c[2 * k], c[2 * k + 1]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) c[k] = y[k];
}

/* 16 = 4 (inner, stride-4 inputs) x 4 (outer), internal twiddles W16^{n2 k1} */
template <class A>
__host__ __device__ __forceinline__ void dft16(typename A::C *c)
{
    using C = typename A::C;
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) dft4<A>(c[n2], c[n2 + 4], c[n2 + 8], c[n2 + 12]);
    /* Y[n2][k1] lives in c[n2 + 4*k1] */
    c[5] = A::template mul_w16<1>(c[5]);
    c[9] = A::mul_w8(c[9]);
    c[13] = A::template mul_w16<3>(c[13]);
    c[6] = A::mul_w8(c[6]);
    c[10] = A::mul_mi(c[10]);
    c[14] = A::mul_w8_3(c[14]);
    c[7] = A::template mul_w16<3>(c[7]);
    c[11] = A::mul_w8_3(c[11]);
    c[15] = A::neg(A::template mul_w16<1>(c[15]));
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) dft4<A>(c[4 * k1], c[4 * k1 + 1], c[4 * k1 + 2], c[4 * k1 + 3]);
    /* X[k1 + 4*k2] is in c[4*k1 + k2]: transpose the 4x4 register block */
    C y[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
        for (int k2 = 0; k2 < 4; k2++) y[k1 + 4 * k2] = c[4 * k1 + k2];
#pragma unroll
    for (int k = 0; k < 16; k++) c[k] = y[k];
}

template <class A, int R>
__host__ __device__ __forceinline__ void dft(typename A::C *c)
{
    if constexpr (R == 2) dft2<A>(c[0], c[1]);
    else if constexpr (R == 4) dft4<A>(c[0], c[1], c[2], c[3]);
    else if constexpr (R == 8) dft8<A>(c);
    else if constexpr (R == 16) dft16<A>(c);
}

/* largest biased FP64 exponent over the CTA's tile (NT threads) */
template <int NT, int E>
__device__ __forceinline__ unsigned tile_max_exp(const double2 (&raw)[E])
{
    unsigned m = 0;
#pragma unroll
    for (int q = 0; q < E; q++) m = max(m, max(dexp(raw[q].x), dexp(raw[q].y)));
    constexpr unsigned mask = NT >= 32 ? 0xffffffffu : ((1u << NT) - 1u);
    m = __reduce_max_sync(mask, m);
    if constexpr (NT <= 32) {
        return m;
    } else {
        __shared__ unsigned s_m[NT / 32];
        if ((threadIdx.x & 31) == 0) s_m[threadIdx.x >> 5] = m;
        __syncthreads();
        unsigned r = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; w++) r = max(r, s_m[w]);
        return r;
    }
}

/*
 * Bit flips of the exchange layout, as source bits for target bits 0, 1, 2
 * (a | b << 4 | c << 8, 0 = no flip), for a first stage of radix 2^lr0 and
 * rows of w 8-byte words.  A warp's shared-memory request is served in
 * 128-byte phases covering 16 / w rows; those rows must land in distinct
 * groups of w words.  Reads (p = j + q * TPL) step rows by one; the
 * first stage's writes (p = 2^lr0 * jj + r) step them by 2^lr0, which puts
 * all rows of a phase in one group.  Flipping low bits by the bits those
 * writes step through separates both patterns.  The table is the minimum
 * found by a bank model of every stage's reads and writes for each L and
 * row width the kernels use; rows of 1 word and of 16 or more need none.
 */
__host__ __device__ constexpr int exch_flip(int lr0, int w)
{
    return lr0 == 0 ? 0
         : w == 8   ? lr0
         : w == 4   ? (lr0 == 1 ? 0x002 : lr0 == 2 ? 0x032 : 0x030)
         : w == 2   ? (lr0 == 1 ? 0x003 : lr0 == 2 ? 0x030 : 0x300)
                    : 0;
}

/* shared-memory index of element p of tile line b (elements of ES bytes,
 * EPT points per thread): row q + q/16 with q = p after the bit flips of
 * exch_flip, column b.  The pad row every 16 keeps the radix-16 stages'
 * accesses, which step by 16 rows, in distinct bank groups. */
template <int LOG_L, int B, int ES, int EPT = 16>
__host__ __device__ __forceinline__ int sidx(int p, int b)
{
    constexpr int LR0 = (EPT == 16 && LOG_L > 4) ? LOG_L % 4 : 0;
    constexpr int F = exch_flip(LR0, B * ES / 8);
    constexpr int FA = F & 15, FB = (F >> 4) & 15, FC = F >> 8;
    int q = p;
    if constexpr (FA != 0) q ^= (p >> FA) & 1;
    if constexpr (FB != 0) q ^= ((p >> FB) & 1) << 1;
    if constexpr (FC != 0) q ^= ((p >> FC) & 1) << 2;
    return (q + (q >> 4)) * B + b;
}

/* Stage structure of a line of 2^LOG_L points, EPT (16 or 4) points per
 * thread: an optional first stage of radix 2^(LOG_L mod log2 EPT), then
 * stages of radix EPT.  EPT = 4 serves small single transforms, where more
 * threads per point shorten each thread's chain of dependent instructions. */
template <int LOG_L, int EPT = 16>
struct Shape {
    static constexpr int LE = EPT == 16 ? 4 : 2;   /* log2 of the main radix */
    static constexpr int L = 1 << LOG_L;
    static constexpr int E = L < EPT ? L : EPT;    /* points per thread */
    static constexpr int TPL = L / E;              /* threads per line */
    static constexpr int LR0 = LOG_L <= LE ? LOG_L : (LOG_L % LE);
    static constexpr int R0 = 1 << LR0;            /* first-stage radix */
    static constexpr int NSTAGE = LOG_L <= LE ? 1 : (LR0 ? 1 : 0) + LOG_L / LE;
    static_assert(EPT == 16 || EPT == 4, "16 or 4 points per thread");
};

template <class A, int LOG_L, int B, int EPT = 16>
__host__ __device__ constexpr size_t pass_smem_bytes()
{
    return Shape<LOG_L, EPT>::TPL > 1
               ? (size_t)((1 << LOG_L) + ((1 << LOG_L) >> 4)) * B * sizeof(typename A::S)
               : 0;
}

/*
 * One Stockham stage of radix R after Ns points have been combined.
 * Reads its inputs from shared memory unless it is the first stage (the
 * registers then already hold the loaded points); writes to shared memory
 * unless it is the last stage (the registers then hold natural-order output).
 */
template <class A, int LOG_L, int B, int R, int NS, bool FROM_SMEM, bool TO_SMEM, int EPT = 16>
__device__ __forceinline__ void stage(typename A::C *a, typename A::S *sm, int j, int b,
                                      const void *tw)
{
    using C = typename A::C;
    using SH = Shape<LOG_L, EPT>;
    constexpr int L = SH::L, E = SH::E, TPL = SH::TPL;
    if constexpr (FROM_SMEM) {
#pragma unroll
        for (int q = 0; q < E; q++) a[q] = A::from_smem(sm[sidx<LOG_L, B, sizeof(typename A::S), EPT>(j + q * TPL, b)]);
    }
#pragma unroll
    for (int u = 0; u < E / R; u++) {
        C c[R];
#pragma unroll
        for (int r = 0; r < R; r++) c[r] = a[u + r * (E / R)];
        if constexpr (NS > 1) {
            const int k = (j + u * TPL) & (NS - 1);
#pragma unroll
            for (int r = 1; r < R; r++)
                c[r] = A::mul_tw(c[r], A::load_tw(tw, (int64_t)(r * k) * (L / (NS * R))));
        }
        dft<A, R>(c);
#pragma unroll
        for (int r = 0; r < R; r++) a[u + r * (E / R)] = c[r];
    }
    if constexpr (TO_SMEM) {
        if constexpr (FROM_SMEM) __syncthreads();
#pragma unroll
        for (int u = 0; u < E / R; u++) {
            const int jj = j + u * TPL;
            const int k = jj & (NS - 1);
            const int o = (jj / NS) * NS * R + k;
#pragma unroll
            for (int r = 0; r < R; r++)
                sm[sidx<LOG_L, B, sizeof(typename A::S), EPT>(o + r * NS, b)] = A::to_smem(a[u + r * (E / R)]);
        }
        __syncthreads();
    }
}

/* stages after the first: radix EPT, Ns = R0 * EPT^(s-1) */
template <class A, int LOG_L, int B, int S, int EPT = 16>
__device__ __forceinline__ void stages16(typename A::C *a, typename A::S *sm, int j, int b,
                                         const void *tw)
{
    using SH = Shape<LOG_L, EPT>;
    if constexpr (S < SH::NSTAGE) {
        constexpr int first_log = SH::LR0 ? SH::LR0 : SH::LE;
        constexpr int NS = 1 << (first_log + SH::LE * (S - 1));
        constexpr bool last = (S == SH::NSTAGE - 1);
        stage<A, LOG_L, B, EPT, NS, true, !last, EPT>(a, sm, j, b, tw);
        stages16<A, LOG_L, B, S + 1, EPT>(a, sm, j, b, tw);
    }
}

/*
 * A radix-EPT stage after 2^lns points have been combined, with lns and
 * whether it is the last stage known at run time: the same reads, twiddles,
 * butterfly and writes as stage<A, LOG_L, B, EPT, 2^lns, true, !last>.
 */
template <class A, int LOG_L, int B, int EPT>
__device__ __forceinline__ void stage_rt(typename A::C *a, typename A::S *sm, int j, int b,
                                         const void *tw, int lns, bool last)
{
    using C = typename A::C;
    using SH = Shape<LOG_L, EPT>;
    constexpr int E = SH::E, TPL = SH::TPL, R = EPT, LR = SH::LE;
    constexpr int ES = (int)sizeof(typename A::S);
#pragma unroll
    for (int q = 0; q < E; q++) a[q] = A::from_smem(sm[sidx<LOG_L, B, ES, EPT>(j + q * TPL, b)]);
    const int ns = 1 << lns;
#pragma unroll
    for (int u = 0; u < E / R; u++) {
        C c[R];
#pragma unroll
        for (int r = 0; r < R; r++) c[r] = a[u + r * (E / R)];
        const int k = (j + u * TPL) & (ns - 1);
        const int sh = LOG_L - lns - LR; /* W_{ns R}^{r k} = W_L^{r k L / (ns R)} */
#pragma unroll
        for (int r = 1; r < R; r++) c[r] = A::mul_tw(c[r], A::load_tw(tw, (int64_t)(r * k) << sh));
        dft<A, R>(c);
#pragma unroll
        for (int r = 0; r < R; r++) a[u + r * (E / R)] = c[r];
    }
    if (!last) { /* CTA-uniform */
        __syncthreads();
#pragma unroll
        for (int u = 0; u < E / R; u++) {
            const int jj = j + u * TPL;
            const int k = jj & (ns - 1);
            const int o = ((jj >> lns) << (lns + LR)) + k;
#pragma unroll
            for (int r = 0; r < R; r++)
                sm[sidx<LOG_L, B, ES, EPT>(o + r * ns, b)] = A::to_smem(a[u + r * (E / R)]);
        }
        __syncthreads();
    }
}

/* Double-float butterflies are long (a radix-16 stage is over a thousand
 * instructions per thread).  The FP64-storage kernel's lines of three or
 * more stages run the stages after the first as one loop with the stage
 * index at run time: one copy of the butterfly instead of one per stage,
 * which keeps the kernel's code within the instruction cache (measured 5.6%
 * faster at 2^24; the FP32-storage double-float kernel measured 0.9% slower
 * rolled at 512^3 and keeps its stages unrolled). */
template <class A, int LOG_L, int EPT>
__host__ __device__ constexpr bool roll_stages()
{
    return A::kId == 1 && Shape<LOG_L, EPT>::NSTAGE >= 3;
}

template <class A, int LOG_L, int B, int EPT = 16>
__device__ __forceinline__ void fft_line_regs(typename A::C *a, typename A::S *sm, int j, int b,
                                              const void *tw)
{
    using SH = Shape<LOG_L, EPT>;
    if constexpr (LOG_L == 0) {
        return;
    } else if constexpr (SH::NSTAGE == 1) {
        stage<A, LOG_L, B, SH::R0, 1, false, false, EPT>(a, sm, j, b, tw);
    } else {
        constexpr int R_first = SH::LR0 ? SH::R0 : EPT;
        stage<A, LOG_L, B, R_first, 1, false, true, EPT>(a, sm, j, b, tw);
        if constexpr (roll_stages<A, LOG_L, EPT>()) {
            constexpr int first_log = SH::LR0 ? SH::LR0 : SH::LE;
#pragma unroll 1
            for (int s = 1; s < SH::NSTAGE; s++)
                stage_rt<A, LOG_L, B, EPT>(a, sm, j, b, tw, first_log + SH::LE * (s - 1), s == SH::NSTAGE - 1);
        } else {
            stages16<A, LOG_L, B, 1, EPT>(a, sm, j, b, tw);
        }
    }
}

/* the in-register line transform of run_tile: all stages on the CUDA cores */
struct CoreLine {
    template <class A, int LOG_L, int B, int EPT = 16>
    __device__ __forceinline__ void run(typename A::C *a, typename A::S *sm, int j, int b,
                                        const tfft_pass &p)
    {
        fft_line_regs<A, LOG_L, B, EPT>(a, sm, j, b, p.tw);
    }
};

/* where one thread's line of a tile lives */
struct TileGeom {
    int64_t g0, g1;       /* line coordinates (g0 may lie past n[0]) */
    int64_t ibase, obase; /* first element of the input and output line */
    bool live;            /* g0 < n[0]: the line exists and is stored */
};

/*
 * Lines tile*B .. tile*B+B-1 of the pass's g0 dimension (the last tile may be
 * ragged: its missing lines compute on a copy of the last line and store
 * nothing), for the g1/g2 coordinates encoded in tile; b is this thread's
 * line within the tile.
 */
template <int B>
__device__ __forceinline__ TileGeom tile_geom(const tfft_pass &p, int64_t tile, int b)
{
    TileGeom g;
    const int64_t tiles0 = (p.n[0] + B - 1) / B;
    g.g0 = (tile % tiles0) * B + b;
    const int64_t rest = tile / tiles0;
    g.g1 = rest % p.n[1];
    const int64_t g2 = rest / p.n[1];
    g.live = g.g0 < p.n[0];
    /* a line past the end of a ragged tile reads the last line again (no
     * predicated loads: they cost 16 registers) and stores nothing */
    const int64_t g0c = g.live ? g.g0 : p.n[0] - 1;
    /* line bases from the strides or the per-line tables */
    const int64_t t0 = p.tab0 ? __ldg(p.tab0 + g0c) : -1;
    const int64_t t1 = p.tab1 ? __ldg(p.tab1 + g.g1) : -1;
    g.ibase = (t0 >= 0 ? t0 : g0c * p.is[0]) + (t1 >= 0 ? t1 : g.g1 * p.is[1]) + g2 * p.is[2];
    g.obase = (t0 >= 0 ? t0 : g0c * p.os[0]) + (t1 >= 0 ? t1 : g.g1 * p.os[1]) + g2 * p.os[2];
    return g;
}

/* Everything after the loads: the tile scaling of the double-float FP64
 * arithmetic, conjugation, the line transform, the four-step twiddle, and
 * the store (conjugation and scale fused) */
template <class A, int LOG_L, int B, class LINE, int EPT = 16>
__device__ __forceinline__ void finish_tile(const tfft_pass &p, const TileGeom &g,
                                            typename A::Store (&raw)[Shape<LOG_L, EPT>::E],
                                            typename A::S *sm, int j, int b, LINE &line)
{
    using C = typename A::C;
    using SH = Shape<LOG_L, EPT>;
    using Store = typename A::Store;
    constexpr int E = SH::E, TPL = SH::TPL;
    /* arithmetics with a narrower exponent range than their storage work on
     * the tile scaled by 2^-delta, delta = the tile's largest FP64 exponent */
    int delta = 0, delta_out = 0;
    if constexpr (A::kScaled) {
        delta = delta_out = (int)tile_max_exp<TPL * B>(raw) - 1023;
        /* the split takes normal FP64 values only: a tile whose largest
         * magnitude is below 2^-900 may hold subnormals that matter, so the
         * whole tile (a CTA-uniform branch) is lifted by 2^600, exactly, and
         * the store puts the factor back */
        if (delta < -900) {
#pragma unroll
            for (int q = 0; q < E; q++) {
                raw[q].x *= 0x1p600;
                raw[q].y *= 0x1p600;
            }
            delta += 600;
        }
    }
    C a[E];
#pragma unroll
    for (int q = 0; q < E; q++) {
        C v = A::load_s(raw[q], delta);
        a[q] = p.conj_in ? A::conj(v) : v;
    }

    line.template run<A, LOG_L, B, EPT>(a, sm, j, b, p);

    if (p.post_tw) {
        const int64_t t = p.tw_level == 0 ? g.g0 : g.g1;
        const int64_t mask = (int64_t(1) << p.tw_shift) - 1;
#pragma unroll
        for (int q = 0; q < E; q++) {
            /* t < N / L and k < L, so m = t k < N needs no reduction (N
             * need not be a power of two) */
            const int64_t m = t * (int64_t)(j + q * TPL);
            /* tw_lo NULL: tw_hi is the whole table W_N^m, m < N */
            typename A::TW w = p.tw_lo ? A::tw_mul(A::load_tw(p.tw_hi, m >> p.tw_shift),
                                                   A::load_tw(p.tw_lo, m & mask))
                                       : A::load_tw(p.tw_hi, m);
            a[q] = A::mul_tw(a[q], w);
        }
    }

    Store *out = reinterpret_cast<Store *>(p.out) + g.obase;
    if (g.live) {
        /* scale 1 (every pass but an inverse's last) in a loop of its own,
         * so the per-element test of the double-precision scale folds away
         * (it would take an FP64 instruction per point) */
        if (p.scale == 1.0) {
#pragma unroll
            for (int q = 0; q < E; q++) {
                C v = p.conj_out ? A::conj(a[q]) : a[q];
                __stcs(out + (int64_t)(j + q * TPL) * p.oes, A::store_s(v, delta_out, 1.0));
            }
        } else {
            const double scale = p.scale;
#pragma unroll
            for (int q = 0; q < E; q++) {
                C v = p.conj_out ? A::conj(a[q]) : a[q];
                __stcs(out + (int64_t)(j + q * TPL) * p.oes, A::store_s(v, delta_out, scale));
            }
        }
    }
}

/* kernel shapes that may stage a full tile of contiguous lines with bulk
 * copies: 16 points per thread, at least 8 lines per tile (a tile of one or
 * two long lines loads as well directly: measured up to 6% slower staged),
 * lines of at least 512 bytes (the staging slots then fit the exchange
 * buffer), the ordinary pass kernel only */
template <class A, int LOG_L, int B, bool L2ONLY, class LINE, int EPT>
__host__ __device__ constexpr bool bulk_capable()
{
    return !L2ONLY && std::is_same<LINE, CoreLine>::value && EPT == 16 && B >= 8 &&
           LOG_L >= 5 && ((size_t)1 << LOG_L) * sizeof(typename A::Store) >= 512;
}

/* bytes of shared memory a launch needs: the exchange buffer, plus the
 * bulk copies' mbarrier where the shape stages tiles */
template <class A, int LOG_L, int B, int EPT = 16>
__host__ __device__ constexpr size_t pass_launch_smem_bytes()
{
    return pass_smem_bytes<A, LOG_L, B, EPT>() +
           (bulk_capable<A, LOG_L, B, false, CoreLine, EPT>() ? 16 : 0);
}

#ifdef __CUDA_ARCH__
__device__ __forceinline__ uint32_t smem_addr32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

/* poll an mbarrier for the phase of parity 0; false if it did not complete
 * within 2^22 polls */
__device__ __forceinline__ bool mbar_wait0(uint32_t mbar)
{
    for (int it = 0; it < (1 << 22); it++) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred P1;\nmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], 0;\n"
            "selp.b32 %0, 1, 0, P1;\n}\n"
            : "=r"(ok)
            : "r"(mbar)
            : "memory");
        if (ok) return true;
    }
    return false;
}
#endif

/*
 * A full tile of B contiguous lines (ies == 1, is[0] == L) staged through
 * shared memory: an mbarrier after the exchange buffer, one bulk
 * asynchronous copy per line (issued by threads 0..B-1, evict-first in L2)
 * into a slot of L elements plus 16 bytes, then each thread reads its E
 * points from its line's slot.  The 16-byte pad (the least a bulk copy's
 * destination alignment allows) makes the slot stride an odd number of
 * 16-byte units: the B lines' elements of one phase of a warp's read (8
 * lines of 16-byte or 2 x 8 lines of 8-byte elements) then fall in distinct
 * banks; a 32-byte pad put lines b and b + 4 on the same banks.
 * Ends with a barrier: the stages reuse the buffer.  A wait that gives up
 * sets *p.err and waits once more (bounded) for the copies in flight.
 */
/* bytes per line slot of bulk_load_tile: the line plus a 16-byte pad */
__host__ __device__ constexpr size_t bulk_slot_bytes(int log_l, int store_bytes)
{
    return ((size_t)1 << log_l) * (size_t)store_bytes + 16;
}

template <class A, int LOG_L, int B, int E, int TPL>
__device__ __forceinline__ void bulk_load_tile(const tfft_pass &p, const TileGeom &g,
                                               typename A::Store (&raw)[E], unsigned char *smem_raw,
                                               int j, int b)
{
#ifdef __CUDA_ARCH__
    using Store = typename A::Store;
    constexpr int L = 1 << LOG_L;
    constexpr uint32_t LINE_BYTES = (uint32_t)(L * sizeof(Store));
    constexpr size_t SLOT = bulk_slot_bytes(LOG_L, (int)sizeof(Store));
    static_assert(B * SLOT <= pass_smem_bytes<A, LOG_L, B>(), "staging slots inside the exchange buffer");
    const uint32_t mbar = smem_addr32(smem_raw + pass_smem_bytes<A, LOG_L, B>());
    const int t = threadIdx.x;
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar),
                     "r"(B * LINE_BYTES)
                     : "memory");
    }
    __syncthreads();
    if (t < B) { /* thread t's tile line is line t (b = t % B, t < B) */
        const Store *src = reinterpret_cast<const Store *>(p.in) + g.ibase;
        /* evict-first in L2, as the direct path's streaming loads: a pass's
         * input must not push out the output the next pass reads */
        asm volatile(
            "{\n.reg .b64 pol;\n"
            "createpolicy.fractional.L2::evict_first.b64 pol, 1.0;\n"
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint "
            "[%0], [%1], %2, [%3], pol;\n}\n" ::"r"(smem_addr32(smem_raw + t * SLOT)),
            "l"(src), "r"(LINE_BYTES), "r"(mbar)
            : "memory");
    }
    if (!mbar_wait0(mbar)) {
        if (p.err) atomicExch(p.err, 1);
        mbar_wait0(mbar);
    }
    const Store *ln = reinterpret_cast<const Store *>(smem_raw + b * SLOT);
#pragma unroll
    for (int q = 0; q < E; q++) raw[q] = ln[j + q * TPL];
    __syncthreads();
#else
    (void)p; (void)g; (void)raw; (void)smem_raw; (void)j; (void)b;
#endif
}

/*
 * A full tile of B adjacent strided lines (is[0] == 1) staged by TMA: the
 * pass's tensor map (p.tmap, dimension 0 the lines) gives one box per 256
 * elements of the line, issued by threads 0..NCH-1 with an evict-first L2
 * policy; the boxes land as rows of B elements, row i of the tile at
 * i * B elements, so thread (j, b) reads element (j + q * TPL) * B + b and a
 * warp reads consecutive words.  Bounded wait and error word as
 * bulk_load_tile; ends with a barrier.
 */
template <class A, int LOG_L, int B, int E, int TPL>
__device__ __forceinline__ void tma_load_tile(const tfft_pass &p, int64_t tile, int64_t first,
                                              typename A::Store (&raw)[E], unsigned char *smem_raw,
                                              int j, int b)
{
#ifdef __CUDA_ARCH__
    using Store = typename A::Store;
    constexpr int L = 1 << LOG_L;
    constexpr int ROWS = L < 256 ? L : 256, NCH = L / ROWS;
    constexpr uint32_t CH_BYTES = (uint32_t)(ROWS * B * sizeof(Store));
    static_assert((size_t)L * B * sizeof(Store) <= pass_smem_bytes<A, LOG_L, B>(),
                  "tile inside the exchange buffer");
    static_assert(CH_BYTES % 128 == 0, "boxes on 128-byte boundaries");
    const uint32_t mbar = smem_addr32(smem_raw + pass_smem_bytes<A, LOG_L, B>());
    const int t = threadIdx.x;
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar),
                     "r"((uint32_t)NCH * CH_BYTES)
                     : "memory");
    }
    __syncthreads();
    if (t < NCH) {
        const int64_t tiles0 = (p.n[0] + B - 1) / B;
        const int64_t rest = tile / tiles0;
        const int64_t src[3] = {(int64_t)t * ROWS, rest % p.n[1], rest / p.n[1]};
        int c[4] = {(int)(first * (int64_t)(sizeof(Store) / 8)), 0, 0, 0};
#pragma unroll
        for (int k = 1; k < 4; k++)
            if (k < p.tmap_rank) c[k] = (int)src[p.tmap_src[k - 1]];
        const uint32_t dst = smem_addr32(smem_raw + t * CH_BYTES);
        const unsigned long long map = (unsigned long long)p.tmap;
        if (p.tmap_rank == 2) {
            asm volatile(
                "{\n.reg .b64 pol;\ncreatepolicy.fractional.L2::evict_first.b64 pol, 1.0;\n"
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
                " [%0], [%1, {%2, %3}], [%4], pol;\n}\n" ::"r"(dst),
                "l"(map), "r"(c[0]), "r"(c[1]), "r"(mbar)
                : "memory");
        } else if (p.tmap_rank == 3) {
            asm volatile(
                "{\n.reg .b64 pol;\ncreatepolicy.fractional.L2::evict_first.b64 pol, 1.0;\n"
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
                " [%0], [%1, {%2, %3, %4}], [%5], pol;\n}\n" ::"r"(dst),
                "l"(map), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(mbar)
                : "memory");
        } else {
            asm volatile(
                "{\n.reg .b64 pol;\ncreatepolicy.fractional.L2::evict_first.b64 pol, 1.0;\n"
                "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
                " [%0], [%1, {%2, %3, %4, %5}], [%6], pol;\n}\n" ::"r"(dst),
                "l"(map), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(mbar)
                : "memory");
        }
    }
    if (!mbar_wait0(mbar)) {
        if (p.err) atomicExch(p.err, 1);
        mbar_wait0(mbar);
    }
    const Store *rows = reinterpret_cast<const Store *>(smem_raw);
#pragma unroll
    for (int q = 0; q < E; q++) raw[q] = rows[(j + q * TPL) * B + b];
    __syncthreads();
#else
    (void)p; (void)tile; (void)first; (void)raw; (void)smem_raw; (void)j; (void)b;
#endif
}

/*
 * One tile.  L2ONLY selects loads that bypass L1 (ld.global.cg): needed when
 * another CTA of the same launch wrote the data (the persistent batch
 * kernel); a plain pass launch reads with the streaming hint, or, for a full
 * tile of contiguous lines in a shape that takes it (bulk_capable, p.bulk
 * set), through shared memory by bulk asynchronous copies.  LINE transforms
 * the loaded points (CoreLine, or the tensor-core stages of fft_tc.cuh).
 */
template <class A, int LOG_L, int B, bool L2ONLY, class LINE = CoreLine, int EPT = 16>
__device__ __forceinline__ void run_tile(const tfft_pass &p, int64_t tile, unsigned char *smem_raw,
                                         LINE line = LINE{})
{
    using SH = Shape<LOG_L, EPT>;
    using Store = typename A::Store;
    constexpr int E = SH::E, TPL = SH::TPL;
    typename A::S *sm = reinterpret_cast<typename A::S *>(smem_raw);
    const int b = threadIdx.x % B, j = threadIdx.x / B;
    const TileGeom g = tile_geom<B>(p, tile, b);
    const Store *in = reinterpret_cast<const Store *>(p.in) + g.ibase;
    Store raw[E];
#if defined(__CUDA_ARCH__)
    if constexpr (bulk_capable<A, LOG_L, B, L2ONLY, LINE, EPT>()) {
        /* CTA-uniform: the pass qualifies, the tile is full (and for the
         * contiguous path, its base is 16-byte aligned) */
        const int64_t tiles0 = (p.n[0] + B - 1) / B;
        const int64_t first = (tile % tiles0) * B;
        const Store *base = reinterpret_cast<const Store *>(p.in) + (g.ibase - (int64_t)b * p.is[0]);
        if (p.tmap && first + B <= p.n[0]) {
            tma_load_tile<A, LOG_L, B, E, TPL>(p, tile, first, raw, smem_raw, j, b);
            finish_tile<A, LOG_L, B, LINE, EPT>(p, g, raw, sm, j, b, line);
            return;
        }
        if (p.bulk && first + B <= p.n[0] && ((uintptr_t)base & 15) == 0) {
            bulk_load_tile<A, LOG_L, B, E, TPL>(p, g, raw, smem_raw, j, b);
            finish_tile<A, LOG_L, B, LINE, EPT>(p, g, raw, sm, j, b, line);
            return;
        }
    }
#endif
#pragma unroll
    for (int q = 0; q < E; q++) {
        if constexpr (L2ONLY) {
            raw[q] = __ldcg(in + (int64_t)(j + q * TPL) * p.ies);
        } else {
            raw[q] = __ldcs(in + (int64_t)(j + q * TPL) * p.ies);
        }
    }
    finish_tile<A, LOG_L, B, LINE, EPT>(p, g, raw, sm, j, b, line);
}

/* Minimum CTAs per SM in the launch bounds.  0 leaves the register count to
 * ptxas's default heuristic (128 for the double-float FP32 kernel); an
 * explicit 1 lets it take up to 255 (225 and 161 registers: one CTA per SM,
 * measured 20-35% slower).  The double-float FP64-storage kernel asks for
 * 16 resident warps (16/W CTAs of W warps, at most 128 registers).  The FP32
 * kernel's 256-thread CTAs ask for three per SM (at most 85 registers):
 * left alone, the staged-tile path took it to 92 registers and two CTAs,
 * 7.5% slower on 512^3 despite the few spills the cap costs. */
template <class A, int T>
constexpr int pass_min_blocks()
{
    constexpr int W = (T + 31) / 32;
    return A::kScaled && W < 16 ? 16 / W : (A::kId == 2 && W == 8) ? 3 : 0;
}

template <class A, int LOG_L, int B, int EPT = 16>
__global__ void
__launch_bounds__(Shape<LOG_L, EPT>::TPL * B, pass_min_blocks<A, Shape<LOG_L, EPT>::TPL * B>())
    pass_kernel(const tfft_pass p)
{
    extern __shared__ __align__(128) unsigned char smem_raw[]; /* TMA boxes: 128-byte aligned */
    run_tile<A, LOG_L, B, false, CoreLine, EPT>(p, blockIdx.x, smem_raw);
}

template <class A, int LOG_L, int LOG_B, int EPT = 16>
int launch_pass(const tfft_pass &p, cudaStream_t s)
{
    constexpr int B = 1 << LOG_B;
    constexpr size_t smem = pass_launch_smem_bytes<A, LOG_L, B, EPT>();
    static unsigned attr_done = 0; /* one bit per device ordinal */
    auto kern = pass_kernel<A, LOG_L, B, EPT>;
    if constexpr (smem > 48 * 1024) {
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned bit = 1u << (dev & 31);
        if (!(attr_done & bit)) {
            cudaError_t e = cudaFuncSetAttribute(
                kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return (int)e;
            attr_done |= bit;
        }
    }
    const int64_t blocks = ((p.n[0] + B - 1) / B) * p.n[1] * p.n[2];
    if (blocks <= 0) return 0;
    kern<<<(unsigned)blocks, Shape<LOG_L, EPT>::TPL * B, smem, s>>>(p);
    return (int)cudaGetLastError();
}

/* lines whose length is not a power of two (fft_mixed.cuh) */
int launch_mixed(const tfft_pass &p, cudaStream_t s);
bool mixed_supported(int len, int b_tile, int arith);

/* launch table over (log2 L, log2 B): at most 512 threads per CTA for
 * 16-byte elements (L*B <= 8192, 136 KB of shared memory) and 1024 for FP32
 * complex (L*B <= 16384, 139 KB) */
using LaunchFn = int (*)(const tfft_pass &, cudaStream_t);
constexpr int kMaxLogB = 5;

template <class A>
constexpr int max_log_points()
{
    return sizeof(typename A::S) == 8 ? 14 : 13;
}

template <class A, int LOG_L, int LOG_B>
constexpr LaunchFn pick()
{
    if constexpr (LOG_L + LOG_B <= max_log_points<A>()) return &launch_pass<A, LOG_L, LOG_B>;
    else return nullptr;
}

template <class A, int LOG_L, int... LB>
constexpr void fill_row(LaunchFn *row, std::integer_sequence<int, LB...>)
{
    ((row[LB] = pick<A, LOG_L, LB>()), ...);
}

template <class A, int... LL>
struct Table {
    LaunchFn fn[TFFT_MAX_LOG_L + 1][kMaxLogB + 1];
    constexpr Table() : fn{}
    {
        (fill_row<A, LL>(fn[LL], std::make_integer_sequence<int, kMaxLogB + 1>{}), ...);
    }
};

template <class A, int... LL>
constexpr Table<A, LL...> make_table(std::integer_sequence<int, LL...>)
{
    return Table<A, LL...>();
}

/* the rows LO..LO+sizeof(I)-1 only: one translation unit per range of L
 * keeps each compile short and lets them run in parallel */
template <class A, int LO, int... I>
struct RangeTable {
    LaunchFn fn[TFFT_MAX_LOG_L + 1][kMaxLogB + 1];
    constexpr RangeTable() : fn{}
    {
        (fill_row<A, LO + I>(fn[LO + I], std::make_integer_sequence<int, kMaxLogB + 1>{}), ...);
    }
};

template <class A, int LO, int HI, int... I>
constexpr RangeTable<A, LO, I...> range_table(std::integer_sequence<int, I...>)
{
    return RangeTable<A, LO, I...>();
}

/* defined by the instantiation units fft_inst_*.cu: launcher for
 * (arith, log2 L, log2 B) or nullptr */
LaunchFn launcher_f64_lo(int log_l, int log_b);
LaunchFn launcher_f64_hi(int log_l, int log_b);
LaunchFn launcher_df64_0(int log_l, int log_b);
LaunchFn launcher_df64_1(int log_l, int log_b);
LaunchFn launcher_df64_2(int log_l, int log_b);
LaunchFn launcher_df64_3(int log_l, int log_b);
LaunchFn launcher_df64_4(int log_l, int log_b);
LaunchFn launcher_df64_5(int log_l, int log_b);
LaunchFn launcher_f32_lo(int log_l, int log_b);
LaunchFn launcher_f32_hi(int log_l, int log_b);
LaunchFn launcher_df32_0(int log_l, int log_b);
LaunchFn launcher_df32_1(int log_l, int log_b);
LaunchFn launcher_df32_2(int log_l, int log_b);
LaunchFn launcher_df32_3(int log_l, int log_b);
LaunchFn launcher_df32_4(int log_l, int log_b);
LaunchFn launcher_df32_5(int log_l, int log_b);
/* tensor form (fft_inst_tc.cu): one lines-per-CTA value per log2 L */
LaunchFn launcher_tc(int log_l);
/* 4 points per thread (fft_inst_small.cu): FP64-storage arithmetics,
 * log2 L = 2..7, log2 L + log2 B <= 12 */
LaunchFn launcher_small(int arith, int log_l, int log_b);

} // namespace tfft

/* one instantiation unit: arith A, rows LO..HI, function NAME */
#define TFFT_INSTANTIATE(A, LO, HI, NAME)                                                     \
    namespace tfft {                                                                          \
    static const auto g_tab_##NAME =                                                          \
        range_table<A, LO, HI>(std::make_integer_sequence<int, (HI) - (LO) + 1>{});           \
    LaunchFn NAME(int log_l, int log_b)                                                       \
    {                                                                                         \
        return (log_l >= (LO) && log_l <= (HI)) ? g_tab_##NAME.fn[log_l][log_b] : nullptr;    \
    }                                                                                         \
    }
