/*
 * Split precision, tensor form: FP32 complex lines whose radix-16 Stockham
 * stages run on the fifth-generation tensor cores (tcgen05) of sm_103a.
 *
 * A radix-16 stage computes, for every 16-point sub-transform (a "row"), the
 * real product y = F x, where x holds the 32 reals of the twiddled inputs
 * (re0, im0, re1, im1, ...) and F is the real 32x32 form of the DFT-16 (row
 * 2k gives re X_k, row 2k+1 gives im X_k).  A CTA's rows go 128 at a time,
 * one row per thread, into GEMMs D[128x32] = X[128x32] * B^T
 * (tcgen05.mma kind::f16, M = 128, N = 32, K = 16, FP16 in, FP32 out):
 *   - each row is put on a fixed-point grid of its own (a power-of-two
 *     scale from its largest value) and split into three FP16 pieces, F into
 *     three as well (fft_tc_split.cuh); the integer leading pieces give an
 *     exact accumulator D_hi, the five cross products a second one, D_lo:
 *     12 MMAs per 128 rows;
 *   - the pieces of x go from registers to tensor memory (tcgen05.st, the A
 *     operand in TMEM with lane = row); the six B matrices sit in shared
 *     memory in the canonical K-major layout without swizzle (one descriptor
 *     per 16-element K half);
 *   - one thread issues the MMAs of every row group and commits them to an
 *     mbarrier; every thread waits for it (bounded) and reads its row of
 *     D_hi and D_lo back with tcgen05.ld, and renormalises their sum into
 *     the double-float result.
 * Everything around the GEMMs is the accurate split form's (ArithDF32):
 * exact FP32 loads, double-float twiddles from FP64-accurate (hi, lo) tables
 * (fused into the split), the first stage of radix 2^(log2 L mod 4) and the
 * exchange between stages in double-float, and one rounding at the FP32
 * store.  So the data carries about 32 bits through a pass.
 *
 * A CTA holds 2^12 points (two row groups, 256 threads, 224 of 256 TMEM
 * columns) or, for L = 2^13, 2^13 points (four groups, 512 threads, 448 of
 * 512 columns).  Its dynamic shared memory is at least 80 KB (116 KB) so that
 * no more CTAs share an SM than its 512 TMEM columns serve.
 *
 * A wait for the tensor cores that runs out sets the device error word; the
 * CTA then agrees on it at the next barrier, issues no further MMAs, waits
 * (bounded) for every group's MMAs in flight and frees its tensor memory.
 */
#pragma once
#include <stdint.h>

#include "fft_pass.cuh"
#include "fft_tc_split.cuh"

namespace tfft {
namespace tc {

using tcs::kNB;
constexpr int kRows = 128;                            /* rows per MMA (M)             */
constexpr int kDCols = 32;                            /* FP32 columns of D (N)        */
constexpr int kAPieceCols = 16;                       /* 32 FP16 K values, packed     */
constexpr int kDHi = 0, kDLo = kDCols, kAOff = 2 * kDCols;
constexpr int kGroupCols = 2 * kDCols + 3 * kAPieceCols; /* TMEM columns per group    */
constexpr int kBPieceBytes = 2048;                    /* 32 x 32 FP16                 */
constexpr int kBBytes = kNB * kBPieceBytes;
constexpr int kWaitLimit = 1 << 22; /* mbarrier polls before a wait gives up */

static_assert(kBBytes == TFFT_TC_MATRIX_BYTES, "matrix table size");

/* shape of a CTA for log2 L: 2^12 points (2^13 for L = 2^13), one 16-point
 * row per thread, TMEM columns for all row groups, and dynamic shared
 * memory (data tile, the B matrices, mbarrier, TMEM address slot) padded so
 * that at most 512 / TCOLS CTAs fit an SM */
template <int LOG_L>
struct Cfg {
    static constexpr int TILE_LOG = LOG_L > 12 ? LOG_L : 12;
    static constexpr int B = 1 << (TILE_LOG - LOG_L);
    static constexpr int NT = (1 << TILE_LOG) / 16;
    static constexpr int NG = NT / kRows;
    static constexpr int TCOLS = NG * kGroupCols <= 256 ? 256 : 512;
    static constexpr size_t TILE_BYTES =
        (pass_smem_bytes<ArithDF32, LOG_L, B>() + 1023) & ~(size_t)1023;
    static constexpr size_t NEED = TILE_BYTES + kBBytes + 8 * NG + 8;
    static constexpr size_t FLOOR = TCOLS == 256 ? 80 * 1024 : 116 * 1024;
    static constexpr size_t SMEM = NEED > FLOOR ? NEED : FLOOR;
    static_assert(NG * kGroupCols <= TCOLS, "tensor memory");
};

/* byte offset of B[n][k] inside one matrix: 8x8 core matrices of 16-bit
 * values, each 8 rows (n) of 16 contiguous bytes (k); the next 8 rows lie
 * 128 B further on (SBO), the next 8 k 512 B further on (LBO) */
__host__ __device__ constexpr int b_offset(int n, int k)
{
    return (k >> 3) * 512 + (n >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2;
}

/* instruction descriptor of kind::f16: D FP32, A and B FP16, both K-major,
 * dense, N = 32, M = 128 */
constexpr uint32_t kIdesc = (1u << 4) | ((uint32_t)(kDCols >> 3) << 17) |
                            ((uint32_t)(kRows >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

/* shared-memory descriptor of one K half of a piece: start address, LBO =
 * 512 B, SBO = 128 B, descriptor version 1, no swizzle */
__device__ __forceinline__ uint64_t b_desc(uint32_t addr)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(512 >> 4) << 16) |
           ((uint64_t)(128 >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ void fence_before()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

/* two FP32 values as one FP16 pair: the low half is the even K element */
__device__ __forceinline__ uint32_t pack_h2(float lo, float hi)
{
    const __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&h);
}

/* the three A pieces of this thread's row into its lane, columns
 * col .. col + 47, then wait until they are written */
__device__ __forceinline__ void store_pieces(uint32_t taddr, const uint32_t (&a)[16],
                                             const uint32_t (&b)[16], const uint32_t (&c)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
        "%13, %14, %15, %16, %17, %18};\n"
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%1], {%19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31, %32, %33, %34};\n"
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%2], {%35, %36, %37, %38, %39, %40, %41, %42, %43, "
        "%44, %45, %46, %47, %48, %49, %50};\n"
        "tcgen05.wait::st.sync.aligned;\n" ::"r"(taddr),
        "r"(taddr + kAPieceCols), "r"(taddr + 2 * kAPieceCols), "r"(a[0]), "r"(a[1]), "r"(a[2]),
        "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]),
        "r"(a[11]), "r"(a[12]), "r"(a[13]), "r"(a[14]), "r"(a[15]), "r"(b[0]), "r"(b[1]), "r"(b[2]),
        "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]),
        "r"(b[11]), "r"(b[12]), "r"(b[13]), "r"(b[14]), "r"(b[15]), "r"(c[0]), "r"(c[1]), "r"(c[2]),
        "r"(c[3]), "r"(c[4]), "r"(c[5]), "r"(c[6]), "r"(c[7]), "r"(c[8]), "r"(c[9]), "r"(c[10]),
        "r"(c[11]), "r"(c[12]), "r"(c[13]), "r"(c[14]), "r"(c[15])
        : "memory");
}

/* 32 FP32 columns of this thread's lane, complete on return */
__device__ __forceinline__ void load_row(uint32_t taddr, uint32_t (&d)[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
        "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
        "%30, %31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]),
          "=r"(d[7]), "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]), "=r"(d[12]), "=r"(d[13]),
          "=r"(d[14]), "=r"(d[15]), "=r"(d[16]), "=r"(d[17]), "=r"(d[18]), "=r"(d[19]),
          "=r"(d[20]), "=r"(d[21]), "=r"(d[22]), "=r"(d[23]), "=r"(d[24]), "=r"(d[25]),
          "=r"(d[26]), "=r"(d[27]), "=r"(d[28]), "=r"(d[29]), "=r"(d[30]), "=r"(d[31])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void mma(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
        "r"(a), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void commit(uint32_t mbar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
        : "memory");
}

/* poll the mbarrier for the phase of the given parity; false if it did not
 * complete within kWaitLimit polls */
__device__ __forceinline__ bool wait_phase(uint32_t mbar, uint32_t parity)
{
    for (int it = 0; it < kWaitLimit; it++) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred P1;\nmbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
            "selp.b32 %0, 1, 0, P1;\n}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

/* the per-CTA state of the tensor stages */
struct Ctx {
    uint32_t tm;   /* TMEM base address (lane 0, first allocated column) */
    uint32_t mbar; /* shared address of row group 0's MMA-completion
                      mbarrier; group g's lies 8 g bytes further on */
    uint32_t bsm;  /* shared address of the six B matrices */
    int *err;      /* set to 1 when a wait gives up */
    uint32_t phase;
    uint32_t fail_phase; /* parity of the wait that gave up */
    int dead;            /* CTA-uniform: a wait gave up, issue no more MMAs */
};

/*
 * One radix-16 Stockham stage after NS points have been combined (the index
 * arithmetic of tfft::stage with R = 16), the DFT-16 on the tensor cores.
 * a[] holds the thread's row in double-float on entry (FROM_SMEM false) or
 * is read from the exchange buffer, and holds the stage's output on return.
 * RENORM: the row was written by a first stage on the CUDA cores, whose
 * double-float sums are unnormalised (where high parts cancel exactly, a
 * low part is the whole value); each part is renormalised with a two-sum,
 * since the split needs low parts below an ulp of the high parts.
 */
template <int LOG_L, int B, int NS, bool FROM_SMEM, bool TO_SMEM, bool RENORM = false>
__device__ __forceinline__ void stage16(ArithDF32::C *a, float4 *sm, int j, int b, const void *tw,
                                        Ctx &cx)
{
    using A = ArithDF32;
    constexpr int L = 1 << LOG_L, TPL = L / 16, NT = TPL * B;
    static_assert(NT % kRows == 0, "whole row groups");
    if (cx.dead) return; /* CTA-uniform */
    if constexpr (FROM_SMEM) {
#pragma unroll
        for (int q = 0; q < 16; q++) a[q] = A::from_smem(sm[sidx<LOG_L, B, sizeof(float4)>(j + q * TPL, b)]);
    }
    if constexpr (FROM_SMEM && TO_SMEM) {
        /* every thread's reads of the exchange buffer before any thread's
         * writes at the end of this stage: a line spans both row groups,
         * which otherwise meet only at their own named barriers until the
         * stage's closing barrier */
        __syncthreads();
    }
    if constexpr (RENORM) {
#pragma unroll
        for (int q = 0; q < 16; q++) {
            two_sum(a[q].r.h, a[q].r.l, a[q].r.h, a[q].r.l);
            two_sum(a[q].i.h, a[q].i.l, a[q].i.h, a[q].i.l);
        }
    }
    /* the row's bound before the twiddle; the twiddled parts stay below
     * sqrt2 times it (1.4375 > sqrt2 with room for rounding) */
    float m = 0.f;
#pragma unroll
    for (int q = 0; q < 16; q++)
        m = fmaxf(m, fmaxf(fabsf(a[q].r.h) + fabsf(a[q].r.l), fabsf(a[q].i.h) + fabsf(a[q].i.l)));
    if constexpr (NS > 1) m *= 1.4375f;
    const int sexp = tcs::scale_exp(m);
    const float sc = tcs::pow2f(sexp);
    const int t = threadIdx.x;
    const uint32_t grp = cx.tm + (uint32_t)((t / kRows) * kGroupCols);
    const uint32_t lane = (uint32_t)(t & 96) << 16; /* this warp's 32 TMEM lanes */
    {
        uint32_t x0[16], x1[16], x2[16];
        const int k = j & (NS - 1);
#pragma unroll
        for (int r = 0; r < 16; r++) {
            float pr[3], pi[3];
            if (NS > 1 && r > 0) {
                tcs::split_tw(a[r].r, a[r].i,
                              A::load_tw(tw, (int64_t)(r * k) * (L / (NS * 16))), sc, pr, pi);
            } else {
                tcs::split_plain(a[r].r, a[r].i, sc, pr, pi);
            }
            x0[r] = pack_h2(pr[0], pi[0]);
            x1[r] = pack_h2(pr[1], pi[1]);
            x2[r] = pack_h2(pr[2], pi[2]);
        }
        store_pieces(grp + lane + kAOff, x0, x1, x2);
    }
    fence_before();
    /* each row group (4 warps, 128 threads) on its own: a named barrier,
     * then one thread issues the group's MMAs and commits them to the
     * group's mbarrier, so one group's MMAs overlap the other's split */
    const int g = t / kRows;
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kRows) : "memory");
    const uint32_t gmbar = cx.mbar + 8u * (uint32_t)g;
    if ((t & (kRows - 1)) == 0) {
        fence_after();
        const uint32_t base = cx.tm + (uint32_t)(g * kGroupCols);
#pragma unroll
        for (int q = 0; q < kNB; q++)
#pragma unroll
            for (int h = 0; h < 2; h++)
                mma(base + (q == 0 ? kDHi : kDLo), base + kAOff + tcs::prod_a(q) * kAPieceCols + 8 * h,
                    b_desc(cx.bsm + tcs::prod_b(q) * kBPieceBytes + h * 1024),
                    (q >= 2 || h) ? 1u : 0u);
        commit(gmbar);
    }
    const uint32_t this_phase = cx.phase;
    const bool ok = wait_phase(gmbar, this_phase);
    cx.phase ^= 1;
    fence_after();
    {
        uint32_t dh[32], dl[32];
        load_row(grp + lane + kDHi, dh);
        load_row(grp + lane + kDLo, dl);
        const float sh = tcs::pow2f(-sexp - tcs::kFB);
        const float sl = tcs::pow2f(-sexp - tcs::kFB - tcs::kLoShift);
#pragma unroll
        for (int r = 0; r < 16; r++) {
            a[r].r = tcs::join_d(__uint_as_float(dh[2 * r]), __uint_as_float(dl[2 * r]), sh, sl);
            a[r].i = tcs::join_d(__uint_as_float(dh[2 * r + 1]), __uint_as_float(dl[2 * r + 1]), sh, sl);
        }
    }
    if constexpr (TO_SMEM) {
        const int k = j & (NS - 1);
        const int o = (j / NS) * NS * 16 + k;
#pragma unroll
        for (int r = 0; r < 16; r++) sm[sidx<LOG_L, B, sizeof(float4)>(o + r * NS, b)] = A::to_smem(a[r]);
    }
    /* the exchange barrier, which also makes a give-up CTA-uniform */
    if (__syncthreads_or(!ok)) {
        cx.dead = 1;
        cx.fail_phase = this_phase;
        if (t == 0) atomicExch(cx.err, 1);
    }
}

/* radix-16 stages S .. NSTAGE-1 */
template <int LOG_L, int B, int S>
__device__ __forceinline__ void stages(ArithDF32::C *a, float4 *sm, int j, int b, const void *tw,
                                       Ctx &cx)
{
    using SH = Shape<LOG_L>;
    if constexpr (S < SH::NSTAGE) {
        constexpr int first_log = SH::LR0 ? SH::LR0 : 4;
        constexpr int NS = 1 << (first_log + 4 * (S - 1));
        constexpr bool last = (S == SH::NSTAGE - 1);
        /* the first tensor stage after a first stage on the CUDA cores
         * renormalises its row */
        stage16<LOG_L, B, NS, true, !last, (S == 1 && SH::LR0 != 0)>(a, sm, j, b, tw, cx);
        stages<LOG_L, B, S + 1>(a, sm, j, b, tw, cx);
    }
}

/* run_tile's line transform for the tensor form (one tile per CTA) */
struct Line {
    Ctx cx;
    template <class A, int LOG_L, int B, int EPT = 16>
    __device__ __forceinline__ void run(typename A::C *a, typename A::S *sm, int j, int b,
                                        const tfft_pass &p)
    {
        static_assert(EPT == 16, "the tensor stages hold 16 points per thread");
        static_assert(LOG_L >= 4, "a radix-16 stage needs 16 points");
        static_assert(sizeof(typename A::S) == sizeof(float4), "double-float exchange");
        using SH = Shape<LOG_L>;
        if constexpr (SH::LR0) {
            /* first stage of radix 2, 4 or 8 on the CUDA cores, double-float */
            stage<ArithDF32, LOG_L, B, SH::R0, 1, false, true>(a, sm, j, b, p.tw);
        } else {
            stage16<LOG_L, B, 1, false, (SH::NSTAGE > 1)>(a, sm, j, b, p.tw, cx);
        }
        stages<LOG_L, B, 1>(a, sm, j, b, p.tw, cx);
    }
};

}  // namespace tc
}  // namespace tfft
