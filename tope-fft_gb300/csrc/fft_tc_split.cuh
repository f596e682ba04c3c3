/*
 * Arithmetic of the tensor form's radix-16 stages (fft_tc.cuh), kept apart
 * so that the host can run it too (tests/emu: the same functions against
 * exact sums).
 *
 * A stage computes y = F x for every 16-point row, F the real 32x32 form of
 * the DFT-16 and x the row's 32 reals (re0, im0, re1, im1, ...).  The tensor
 * cores multiply FP16 operands into FP32 accumulators; a value of about 32
 * significant bits is carried as three FP16 pieces on a per-row fixed-point
 * grid:
 *   x s = x0 + 2^-11 x1 + 2^-22 x2     s = 2^(9 - e), the row's values < 2^e
 *   F 2^10 = F0 + 2^-11 F1 + 2^-22 F2
 * x0, x1, F0, F1 are integers (|x0| <= 513, |x1| <= 2048, |F0|, |F1| <=
 * 1024), so every x0 F0 product is an integer and their sum over a row is
 * at most 513 * 20592 < 2^24 (20592: the largest row sum of |F0|): the FP32
 * accumulator D_hi = sum x0 F0 is EXACT whatever order the tensor core adds
 * in.  The cross products of the next
 * two levels,
 *   2^-11 (x1 F0 + x0 F1) + 2^-22 (x1 F1 + x2 F0 + x0 F2),
 * are 2^-11 below D_hi, so one FP32 accumulator D_lo holds them with an
 * error near 2^-35 of the result.  They enter it through matrices scaled by
 * 2^8 (B1..B5 below) so that no FP16 operand is subnormal.  The products
 * left out (level 3 and beyond) are below 2^-32.  The stage's output is
 * D_hi + 2^-8 D_lo rescaled by powers of two and renormalised with an
 * error-free two-sum (join_d): for an output small against its row the two
 * accumulators are of like size, and the next split needs a low part below
 * half an ulp of the high part.  The next stage's twiddle product is formed
 * as three FP32 terms whose integer parts are taken separately, so the data
 * keeps about 32 bits between stages and only the FP32 stores round (rel-L2
 * of a 512^3 transform is then the FP32 storage rounding, about 5e-8).
 *
 * This replaces, for the split-precision form, the reference's radix-8/4/2
 * DIT stage loop (src/kernels3D.cl:15-298, src/fft3d.c:55-77).
 */
#pragma once
#include <stdint.h>

#include "fft_arith.cuh"

#ifdef __CUDACC__
#include <cuda_fp16.h>
#endif

namespace tfft {
namespace tcs {

constexpr int kSB = 9;       /* row scale: |x0| stays below 2^kSB + 1      */
constexpr int kFB = 10;      /* F0 = rint(F 2^kFB)                          */
constexpr int kPB = 11;      /* bits between pieces                         */
constexpr int kLoShift = 8;  /* D_lo holds the cross products times 2^8     */
constexpr int kNB = 6;       /* B matrices: F0 and the five cross products  */

/* product q of a stage: x piece prod_a(q) times B matrix prod_b(q); q = 0
 * into D_hi, then into D_lo smallest first (x2 F0, x1 F1, x0 F2, x1 F0,
 * x0 F1); B_m = an F piece times 2^(kLoShift - level * kPB) */
__host__ __device__ constexpr int prod_a(int q)
{
    return q == 0 ? 0 : q == 1 ? 2 : q == 2 ? 1 : q == 3 ? 0 : q == 4 ? 1 : 0;
}
__host__ __device__ constexpr int prod_b(int q)
{
    return q == 0 ? 0 : q == 1 ? 4 : q == 2 ? 3 : q == 3 ? 5 : q == 4 ? 1 : 2;
}

/* v rounded to the nearest integer (ties to even) for |v| < 2^22, with two
 * FP32 additions: v + 1.5 * 2^23 lies in (2^23, 2^24), where the ulp is 1,
 * and the subtraction is exact (the FMA pipe, not the conversion unit) */
__host__ __device__ __forceinline__ float rint_(float v)
{
    return sub_rn(add_rn(v, 12582912.f), 12582912.f);
}

__host__ __device__ __forceinline__ double rint_d(double v)
{
#ifdef __CUDA_ARCH__
    return rint(v);
#else
    return __builtin_rint(v);
#endif
}

/* 2^k as a float for -149 <= k <= 127 (0 below) */
__host__ __device__ __forceinline__ float pow2f(int k)
{
    return k >= -126 ? u2f((unsigned)(k + 127) << 23) : (k >= -149 ? u2f(1u << (k + 149)) : 0.f);
}

/* the row's scale exponent: s = 2^sexp with (row bound m) * s < 2^kSB,
 * clamped so that s stays a normal FP32 power of two */
__host__ __device__ __forceinline__ int scale_exp(float m)
{
    const int eb = (int)((f2u(m) >> 23) & 0xffu); /* m < 2^(eb - 126) */
    int sexp = kSB - (eb - 126);
    return sexp < -126 ? -126 : (sexp > 126 ? 126 : sexp);
}

/* pieces of t0 + t1 + t2 (already on the row's grid, |t0| + |t1| <= 2^9,
 * |t2| below 2^-13: the row's values are normalised double-floats):
 * x0 + 2^-11 x1 + 2^-22 x2, with x0, x1 integers and x2 the rest (rounded
 * to FP16 when packed).  t0 - rint(t0) and t1 - rint(t1) are exact, the
 * remainder r lies in [-1, 1] up to t2, so x1 = rint(2^11 r) <= 2048 is an
 * FP16 integer. */
__host__ __device__ __forceinline__ void split_terms(float t0, float t1, float t2, float &x0,
                                                     float &x1, float &x2)
{
    const float r0 = rint_(t0), r1 = rint_(t1);
    x0 = add_rn(r0, r1);
    const float r = add_rn(add_rn(sub_rn(t0, r0), sub_rn(t1, r1)), t2);
    const float u = mul_rn(r, 2048.f);
    x1 = rint_(u);
    x2 = mul_rn(sub_rn(u, x1), 2048.f);
}

/* (re, im) of a double-float complex value times s, no twiddle */
__host__ __device__ __forceinline__ void split_plain(df2 re, df2 im, float s, float (&pr)[3],
                                                     float (&pi)[3])
{
    split_terms(mul_rn(re.h, s), 0.f, mul_rn(re.l, s), pr[0], pr[1], pr[2]);
    split_terms(mul_rn(im.h, s), 0.f, mul_rn(im.l, s), pi[0], pi[1], pi[2]);
}

/* (re + i im) * (wr + i wi) * s, the twiddle a (hi, lo) pair per part:
 * each output part is three FP32 terms (two exact-hi products and their
 * error and cross terms), split without forming their sum */
__host__ __device__ __forceinline__ void split_tw(df2 re, df2 im, float4 w, float s,
                                                  float (&pr)[3], float (&pi)[3])
{
    const float wrh = mul_rn(w.x, s), wrl = mul_rn(w.y, s);
    const float wih = mul_rn(w.z, s), wil = mul_rn(w.w, s);
    /* re = xr wr - xi wi */
    const float a0 = mul_rn(re.h, wrh), a1 = mul_rn(im.h, wih);
    float e = sub_rn(fmaf_(re.h, wrh, -a0), fmaf_(im.h, wih, -a1));
    e = fmaf_(re.l, wrh, e);
    e = fmaf_(re.h, wrl, e);
    e = fmaf_(-im.l, wih, e);
    e = fmaf_(-im.h, wil, e);
    /* im = xr wi + xi wr */
    const float b0 = mul_rn(re.h, wih), b1 = mul_rn(im.h, wrh);
    float f = add_rn(fmaf_(re.h, wih, -b0), fmaf_(im.h, wrh, -b1));
    f = fmaf_(re.l, wih, f);
    f = fmaf_(re.h, wil, f);
    f = fmaf_(im.l, wrh, f);
    f = fmaf_(im.h, wrl, f);
    split_terms(a0, -a1, e, pr[0], pr[1], pr[2]);
    split_terms(b0, b1, f, pi[0], pi[1], pi[2]);
}

/* a stage's output from its accumulators, renormalised: hi + lo ==
 * dhi * sh + dlo * sl exactly (sh = 2^(-sexp - kFB), sl = sh 2^-kLoShift,
 * both products exact), |lo| <= ulp(hi) / 2 */
__host__ __device__ __forceinline__ df2 join_d(float dhi, float dlo, float sh, float sl)
{
    df2 r;
    two_sum(mul_rn(dhi, sh), mul_rn(dlo, sl), r.h, r.l);
    return r;
}

/* entry (n, k) of the real 32x32 DFT-16: row 2k' = re X_k', row 2k'+1 =
 * im X_k'; column 2p = re x_p, column 2p+1 = im x_p; c, s = cos, sin of
 * 2 pi k'p/16 */
__host__ __device__ __forceinline__ double dft16_entry(int n, int k, double c, double s)
{
    if ((n & 1) == 0) return (k & 1) ? s : c; /* re X: xr cos + xi sin */
    return (k & 1) ? c : -s;                  /* im X: xi cos - xr sin */
}

/* the six B matrices' entries (as exact doubles; FP16 rounding only for
 * B5) from one entry v of F */
__host__ __device__ __forceinline__ void b_values(double v, double (&b)[kNB])
{
    const double F0 = rint_d(v * 1024.0);
    const double r1 = (v * 1024.0 - F0) * 2048.0;
    const double F1 = rint_d(r1);
    const double F2 = (r1 - F1) * 2048.0;
    b[0] = F0;
    b[1] = F0 * 0x1p-3;  /* x1 F0 2^-11, times 2^8 */
    b[2] = F1 * 0x1p-3;  /* x0 F1 2^-11 */
    b[3] = F1 * 0x1p-14; /* x1 F1 2^-22 */
    b[4] = F0 * 0x1p-14; /* x2 F0 2^-22 */
    b[5] = F2 * 0x1p-14; /* x0 F2 2^-22 */
}

}  // namespace tcs
}  // namespace tfft
