/*
 * Arithmetic policies for the butterfly kernels.
 *
 * A policy provides the in-register complex type C, the twiddle-table
 * element TW, the shared-memory element S, conversions from/to the FP64
 * storage element (double2) and the few complex operations a radix-2/4/8/16
 * butterfly needs.  The FFT code in fft_pass.cuh is written once against
 * this interface.
 *
 *   ArithF64   native double-precision instructions (DADD/DMUL/DFMA).
 *
 * Forward transforms only: an inverse is run as conj(F(conj(x))) with the
 * conjugations fused into the first load and the last store.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

/* a function kept out of line (a rare path called from many unrolled sites) */
#if defined(__CUDACC__)
#define TFFT_NOINLINE __noinline__
#else
#define TFFT_NOINLINE __attribute__((noinline))
#endif

namespace tfft {

/* cos(pi/8), sin(pi/8), sqrt(1/2): nearest doubles */
#define TFFT_C8 0.92387953251128675613
#define TFFT_S8 0.38268343236508977173
#define TFFT_R2 0.70710678118654752440

struct ArithF64 {
    using C = double2;
    using TW = double2;
    using S = double2;
    using Store = double2;
    static constexpr int kId = 0;

    static __device__ __forceinline__ C load(double2 v) { return v; }
    static __device__ __forceinline__ double2 store(C v) { return v; }
    static __device__ __forceinline__ S to_smem(C v) { return v; }
    static __device__ __forceinline__ C from_smem(S v) { return v; }

    static __device__ __forceinline__ C add(C a, C b) { return make_double2(a.x + b.x, a.y + b.y); }
    static __device__ __forceinline__ C sub(C a, C b) { return make_double2(a.x - b.x, a.y - b.y); }
    static __device__ __forceinline__ C conj(C a) { return make_double2(a.x, -a.y); }
    static __device__ __forceinline__ C neg(C a) { return make_double2(-a.x, -a.y); }
    /* a * (-i) */
    static __device__ __forceinline__ C mul_mi(C a) { return make_double2(a.y, -a.x); }
    /* a * (1 - i)/sqrt2 */
    static __device__ __forceinline__ C mul_w8(C a)
    {
        return make_double2((a.x + a.y) * TFFT_R2, (a.y - a.x) * TFFT_R2);
    }
    /* a * (-1 - i)/sqrt2 */
    static __device__ __forceinline__ C mul_w8_3(C a)
    {
        return make_double2((a.y - a.x) * TFFT_R2, -(a.x + a.y) * TFFT_R2);
    }
    /* a * (c - i s) for the constants of W16^1 (c=cos pi/8, s=sin pi/8) and
     * W16^3 (c=sin pi/8, s=cos pi/8) */
    template <int K>
    static __device__ __forceinline__ C mul_w16(C a)
    {
        constexpr double c = K == 1 ? TFFT_C8 : TFFT_S8;
        constexpr double s = K == 1 ? TFFT_S8 : TFFT_C8;
        return make_double2(fma(a.x, c, a.y * s), fma(a.y, c, -(a.x * s)));
    }
    static __device__ __forceinline__ C mul_tw(C a, TW w)
    {
        return make_double2(fma(a.x, w.x, -(a.y * w.y)), fma(a.x, w.y, a.y * w.x));
    }
    static __device__ __forceinline__ TW load_tw(const void *tab, int64_t m)
    {
        return __ldg(reinterpret_cast<const double2 *>(tab) + m);
    }
    static __device__ __forceinline__ TW tw_mul(TW a, TW b) { return mul_tw(a, b); }

    /* real constants (odd-radix butterflies): a * c and acc + a * c */
    using R = double;
    static __host__ __device__ constexpr R rc(double d, float, float) { return d; }
    static __device__ __forceinline__ C mulr(C a, R c) { return make_double2(a.x * c, a.y * c); }
    static __device__ __forceinline__ C fmar(C acc, C a, R c)
    {
        return make_double2(fma(a.x, c, acc.x), fma(a.y, c, acc.y));
    }

    /* storage conversion; FP64 needs no tile scaling */
    static constexpr bool kScaled = false;
    static __device__ __forceinline__ C load_s(double2 v, int) { return v; }
    static __device__ __forceinline__ double2 store_s(C v, int, double scale)
    {
        return scale != 1.0 ? make_double2(v.x * scale, v.y * scale) : v;
    }
};

/* ------------------------------------------------------------------------ */
/* double-float: a value is an unevaluated sum hi + lo of two FP32 numbers.   */
/* ------------------------------------------------------------------------ */

/* bit casts usable on host (for CPU checks of the arithmetic) and device */
__host__ __device__ __forceinline__ unsigned f2u(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    unsigned u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}
__host__ __device__ __forceinline__ float u2f(unsigned u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}
__host__ __device__ __forceinline__ unsigned long long d2ull(double d)
{
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(d);
#else
    unsigned long long u;
    __builtin_memcpy(&u, &d, 8);
    return u;
#endif
}
__host__ __device__ __forceinline__ double ull2d(unsigned long long u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    __builtin_memcpy(&d, &u, 8);
    return d;
#endif
}
__host__ __device__ __forceinline__ int clz64(unsigned long long v)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}
__host__ __device__ __forceinline__ float fmaf_(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}
/* a + b, never contracted into an FMA (error-free transforms rely on it) */
__host__ __device__ __forceinline__ float add_rn(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float s = a + b;
    return s;
#endif
}
__host__ __device__ __forceinline__ float sub_rn(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    volatile float s = a - b;
    return s;
#endif
}
__host__ __device__ __forceinline__ float mul_rn(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float s = a * b;
    return s;
#endif
}

/* biased FP64 exponent field of v */
__host__ __device__ __forceinline__ unsigned dexp(double v)
{
    return (unsigned)(d2ull(v) >> 52) & 0x7ffu;
}

/* nearest integer (ties to even) of x, |x| < 2^31 */
__host__ __device__ __forceinline__ int f2i_rn(float x)
{
#ifdef __CUDA_ARCH__
    return __float2int_rn(x);
#else
    return (int)__builtin_nearbyint((double)x);
#endif
}

/*
 * v * 2^-delta as a (hi, lo) FP32 pair, with integer operations only (no
 * FP64 instruction).  hi keeps the top 24 significant bits (truncated), lo
 * the next 23; the 6 lowest mantissa bits are dropped (relative error below
 * 2^-46).  Values more than 2^100 below 2^delta become 0: delta is the
 * tile's largest exponent, so they are far below the tile's rounding level.
 * hi comes from the high word shifted left by 3 (the exponent's low 9 bits
 * over FP32's exponent field, the top 23 mantissa bits below it): adding the
 * bias change 127 - 1023 - delta to that field and keeping its low 8 bits
 * gives E + 127, which lies in 27..127.
 */
__host__ __device__ __forceinline__ void split_double(double v, int delta, float &hi, float &lo)
{
    const unsigned long long b = d2ull(v);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const int e = (int)((hw >> 20) & 0x7ffu);
    /* zeros and FP64 subnormals: a tile that can hold a subnormal within
     * 2^100 of its largest value is lifted by 2^600 before the split (see
     * run_tile), so here they are always far below the tile's rounding level */
    if (e == 0 || e - 1023 - delta < -100) {
        hi = 0.f;
        lo = 0.f;
        return;
    }
    const unsigned top = (hw << 3) | (lw >> 29);
    const unsigned hb = ((top + ((unsigned)(127 - 1023 - delta) << 23)) & 0x7fffffffu) | (hw & 0x80000000u);
    const unsigned base = (hb & 0xff800000u) - (23u << 23); /* sign, 2^(E - 23) */
    hi = u2f(hb);
    lo = sub_rn(u2f(base | ((lw >> 6) & 0x7fffffu)), u2f(base));
}

/*
 * (s + e) * 2^delta for a renormalised pair (|e| <= ulp(s)/2) in every case
 * the fast join leaves out: FP32-subnormal parts, FP64-subnormal and
 * overflowing results (infinities and NaNs give infinity).  The sum is formed
 * in a 64-bit integer S in units of 2^(es - 182) (s's 24 bits shifted up by
 * 32; e's bits below the unit folded into a sticky bit), then rounded once,
 * to nearest even, to the 53 bits of a normal result or the fewer bits of a
 * subnormal one.
 */
static __host__ __device__ TFFT_NOINLINE double join_double_any(float s, float e, int delta)
{
    const unsigned sb = f2u(s), eb = f2u(e);
    if ((sb & 0x7fffffffu) == 0) return 0.0;
    const unsigned long long sgn = (unsigned long long)(sb & 0x80000000u) << 32;
    const int es = (int)((sb >> 23) & 0xffu);
    if (es == 255) return ull2d(sgn | 0x7ff0000000000000ull);
    const int esn = es ? es : 1;
    long long S = (long long)((sb & 0x7fffffu) | (es ? 0x800000u : 0u)) << 32;
    if (eb & 0x7fffffffu) {
        const int ee = (int)((eb >> 23) & 0xffu);
        const unsigned long long Me = (eb & 0x7fffffu) | (ee ? 0x800000u : 0u);
        const int d = esn - (ee ? ee : 1); /* at least 24 */
        unsigned long long term;
        if (d <= 32) term = Me << (32 - d);
        else if (d - 32 < 64) term = (Me >> (d - 32)) | ((Me & ((1ull << (d - 32)) - 1)) ? 1ull : 0ull);
        else term = 1; /* a sticky bit only */
        S += ((sb ^ eb) & 0x80000000u) ? -(long long)term : (long long)term;
    }
    const int top = 63 - clz64((unsigned long long)S);
    long long be = (long long)esn - 182 + top + delta + 1023; /* biased exponent at 53 bits */
    int sh = top - 52;
    if (be <= 0) sh += (int)(1 - be); /* a subnormal result keeps fewer bits */
    unsigned long long m;
    if (sh <= 0) {
        m = (unsigned long long)S << (-sh);
    } else if (sh >= 64) {
        m = 0;
    } else {
        const unsigned long long u = (unsigned long long)S;
        const unsigned long long half = 1ull << (sh - 1), rem = u & ((half << 1) - 1);
        m = u >> sh;
        if (rem > half || (rem == half && (m & 1))) m++;
    }
    /* a subnormal (or, after a carry, the smallest normal) encodes as m */
    if (be <= 0) return ull2d(sgn | m);
    if (m >> 53) { /* the rounding carried into a new binade */
        m >>= 1;
        be++;
    }
    if (be >= 2047) return ull2d(sgn | 0x7ff0000000000000ull);
    return ull2d(sgn | ((unsigned long long)be << 52) | (m & 0xfffffffffffffull));
}

/*
 * (hi + lo) * 2^delta rounded to the nearest double (ties to even), on the
 * FP32 pipe and integer units only.  After a two-sum, s + e == hi + lo with
 * |e| <= ulp(s)/2.  s's bits, shifted into FP64 position with the exponent
 * rebiased, are the result's top 24 bits; e rounded to the result's unit
 * (one scale by a power of two in its exponent field and one
 * float-to-integer conversion, at most 2^28 in magnitude) is added to that
 * bit pattern as an integer.  When s is a power of two and e points the
 * other way, the result lies in the binade below, whose unit is half as
 * large: e is rounded to that unit and the subtraction borrows from the
 * exponent field, which is exactly that binade's encoding.  s below 2^-71
 * (where e could be an FP32 subnormal that matters), zeros, infinities and
 * results near the ends of FP64's exponent range take join_double_any.
 */
__host__ __device__ __forceinline__ double join_double(float hi, float lo, int delta)
{
    float s, e;
    {
        s = add_rn(hi, lo);
        const float bb = sub_rn(s, hi);
        e = add_rn(sub_rn(hi, sub_rn(s, bb)), sub_rn(lo, bb));
    }
    const unsigned sb = f2u(s), eb = f2u(e);
    const int es = (int)((sb >> 23) & 0xffu);
    const int bexp = es + 896 + delta; /* the result's biased FP64 exponent */
    if (es < 56 || es == 255 || bexp < 2 || bexp > 2045) return join_double_any(s, e, delta);
    const int ee = (int)((eb >> 23) & 0xffu);
    const bool below = ((sb & 0x7fffffu) == 0) && ((sb ^ eb) & 0x80000000u) && ee != 0;
    const int ek = ee + 179 - es + (below ? 1 : 0); /* e's exponent field in result units */
    const int t = (ee != 0 && ek > 0) ? f2i_rn(u2f((eb & 0x807fffffu) | ((unsigned)ek << 23))) : 0;
    const unsigned long long mag = ((unsigned long long)(sb & 0x7fffffffu) << 29) +
                                   ((unsigned long long)(896 + delta) << 52);
    const long long ts = (sb & 0x80000000u) ? -(long long)t : (long long)t;
    return ull2d((mag + (unsigned long long)ts) | ((unsigned long long)(sb & 0x80000000u) << 32));
}

struct df2 {
    float h, l;
};

/* error-free sum: s + e == a + b exactly */
__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = add_rn(a, b);
    const float bb = sub_rn(s, a);
    e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
}

/* sum of two pairs, left unnormalised (hi exact sum, lo collects the rest) */
__host__ __device__ __forceinline__ df2 dadd(df2 x, df2 y)
{
    df2 r;
    float e;
    two_sum(x.h, y.h, r.h, e);
    r.l = add_rn(e, add_rn(x.l, y.l));
    return r;
}
__host__ __device__ __forceinline__ df2 dsub(df2 x, df2 y)
{
    df2 r;
    float e;
    two_sum(x.h, -y.h, r.h, e);
    r.l = add_rn(e, sub_rn(x.l, y.l));
    return r;
}
/* x * c for a constant pair c */
__host__ __device__ __forceinline__ df2 dmul(df2 x, df2 c)
{
    df2 r;
    r.h = mul_rn(x.h, c.h);
    float e = fmaf_(x.h, c.h, -r.h);
    e = fmaf_(x.h, c.l, e);
    r.l = fmaf_(x.l, c.h, e);
    return r;
}
/* a*b - c*d of pairs, the result's hi from one exact two-sum */
__host__ __device__ __forceinline__ df2 ddiffprod(df2 a, df2 b, df2 c, df2 d)
{
    const float p1 = mul_rn(a.h, b.h), p2 = mul_rn(c.h, d.h);
    float t = fmaf_(a.h, b.h, -p1);
    t = sub_rn(t, fmaf_(c.h, d.h, -p2));
    df2 r;
    float e;
    two_sum(p1, -p2, r.h, e);
    t = fmaf_(a.h, b.l, t);
    t = fmaf_(a.l, b.h, t);
    t = fmaf_(-c.h, d.l, t);
    t = fmaf_(-c.l, d.h, t);
    r.l = add_rn(e, t);
    return r;
}

/* double-float constants of cos(pi/8), sin(pi/8), sqrt(1/2): hi is the
 * nearest FP32, lo the nearest FP32 to the remainder (|error| < 7e-16) */
#define TFFT_DF_C8 {0x1.d906bcp-1f, 0x1.e651a8p-26f}
#define TFFT_DF_S8 {0x1.87de2ap-2f, 0x1.abaa58p-28f}
#define TFFT_DF_R2 {0x1.6a09e6p-1f, 0x1.9fcef4p-27f}

/* a scale factor as a (hi, lo) float pair */
__host__ __device__ __forceinline__ df2 scale_pair(double s)
{
    const float h = (float)s;
    return df2{h, (float)(s - (double)h)};
}
/* is s a power of two (the 1/N of a power-of-two transform)? */
__host__ __device__ __forceinline__ bool pow2_scale(double s)
{
    return (d2ull(s) & 0xfffffffffffffull) == 0;
}

struct ArithDF64 {
    struct C {
        df2 r, i;
    };
    using TW = float4; /* re_hi, re_lo, im_hi, im_lo */
    using S = float4;
    using Store = double2;
    static constexpr int kId = 1;
    static constexpr bool kScaled = true;

    static __host__ __device__ __forceinline__ C load_s(double2 v, int delta)
    {
        C c;
        split_double(v.x, delta, c.r.h, c.r.l);
        split_double(v.y, delta, c.i.h, c.i.l);
        return c;
    }
    static __host__ __device__ __forceinline__ double2 store_s(C v, int delta, double scale)
    {
        int ds = 0;
        if (scale != 1.0) {
            unsigned long long sb = d2ull(scale);
            if (sb & 0xfffffffffffffull) {
                /* 1/N for N not a power of two: a pair product */
                v.r = dmul(v.r, scale_pair(scale));
                v.i = dmul(v.i, scale_pair(scale));
            } else { /* 2^-k: fold it into the exponent */
                ds = (int)((sb >> 52) & 0x7ff) - 1023;
            }
        }
        return make_double2(join_double(v.r.h, v.r.l, delta + ds),
                            join_double(v.i.h, v.i.l, delta + ds));
    }
    static __host__ __device__ __forceinline__ S to_smem(C v) { return make_float4(v.r.h, v.r.l, v.i.h, v.i.l); }
    static __host__ __device__ __forceinline__ C from_smem(S v)
    {
        C c;
        c.r.h = v.x; c.r.l = v.y; c.i.h = v.z; c.i.l = v.w;
        return c;
    }
    static __host__ __device__ __forceinline__ C add(C a, C b)
    {
        C c;
        c.r = dadd(a.r, b.r);
        c.i = dadd(a.i, b.i);
        return c;
    }
    static __host__ __device__ __forceinline__ C sub(C a, C b)
    {
        C c;
        c.r = dsub(a.r, b.r);
        c.i = dsub(a.i, b.i);
        return c;
    }
    static __host__ __device__ __forceinline__ df2 dneg(df2 x) { return df2{-x.h, -x.l}; }
    static __host__ __device__ __forceinline__ C conj(C a)
    {
        a.i = dneg(a.i);
        return a;
    }
    static __host__ __device__ __forceinline__ C neg(C a)
    {
        a.r = dneg(a.r);
        a.i = dneg(a.i);
        return a;
    }
    static __host__ __device__ __forceinline__ C mul_mi(C a)
    {
        C c;
        c.r = a.i;
        c.i = dneg(a.r);
        return c;
    }
    static __host__ __device__ __forceinline__ C mul_w8(C a)
    {
        const df2 r2 = TFFT_DF_R2;
        C c;
        c.r = dmul(dadd(a.r, a.i), r2);
        c.i = dmul(dsub(a.i, a.r), r2);
        return c;
    }
    static __host__ __device__ __forceinline__ C mul_w8_3(C a)
    {
        const df2 r2 = TFFT_DF_R2;
        C c;
        c.r = dmul(dsub(a.i, a.r), r2);
        c.i = dneg(dmul(dadd(a.r, a.i), r2));
        return c;
    }
    /* a * (c - i s): re = a.r c + a.i s, im = a.i c - a.r s */
    template <int K>
    static __host__ __device__ __forceinline__ C mul_w16(C a)
    {
        const df2 c8 = TFFT_DF_C8, s8 = TFFT_DF_S8;
        const df2 c = K == 1 ? c8 : s8, s = K == 1 ? s8 : c8;
        C o;
        o.r = ddiffprod(a.r, c, dneg(a.i), s);
        o.i = ddiffprod(a.i, c, a.r, s);
        return o;
    }
    static __host__ __device__ __forceinline__ C mul_tw(C a, TW w)
    {
        const df2 wr = {w.x, w.y}, wi = {w.z, w.w};
        C o;
        o.r = ddiffprod(a.r, wr, a.i, wi);
        o.i = ddiffprod(a.r, wi, dneg(a.i), wr);
        return o;
    }
    static __device__ __forceinline__ TW load_tw(const void *tab, int64_t m)
    {
        return __ldg(reinterpret_cast<const float4 *>(tab) + m);
    }
    /* real constants as (hi, lo) pairs: a * c and acc + a * c */
    using R = df2;
    static __host__ __device__ constexpr R rc(double, float h, float l) { return df2{h, l}; }
    static __host__ __device__ __forceinline__ C mulr(C a, R c)
    {
        C o;
        o.r = dmul(a.r, c);
        o.i = dmul(a.i, c);
        return o;
    }
    static __host__ __device__ __forceinline__ C fmar(C acc, C a, R c) { return add(acc, mulr(a, c)); }
    static __host__ __device__ __forceinline__ TW tw_mul(TW a, TW b)
    {
        C x;
        x.r = df2{a.x, a.y};
        x.i = df2{a.z, a.w};
        C y = mul_tw(x, b);
        /* renormalise table products so later products see |lo| << |hi| */
        float rh, rl, ih, il;
        two_sum(y.r.h, y.r.l, rh, rl);
        two_sum(y.i.h, y.i.l, ih, il);
        return make_float4(rh, rl, ih, il);
    }
};

/* ------------------------------------------------------------------------ */
/* split precision, accurate: FP32 in memory, double-float on chip.  A load  */
/* is exact (hi = x, lo = 0); a store rounds hi + lo once.  FP32 storage has */
/* FP32's exponent range, so no tile scaling is needed.                      */
/* ------------------------------------------------------------------------ */
struct ArithDF32 : ArithDF64 {
    using Store = float2;
    static constexpr int kId = 3;
    static constexpr bool kScaled = false;
    static __host__ __device__ __forceinline__ C load_s(float2 v, int)
    {
        C c;
        c.r = df2{v.x, 0.f};
        c.i = df2{v.y, 0.f};
        return c;
    }
    static __host__ __device__ __forceinline__ float2 store_s(C v, int, double scale)
    {
        if (scale != 1.0 && !pow2_scale(scale)) {
            v.r = dmul(v.r, scale_pair(scale));
            v.i = dmul(v.i, scale_pair(scale));
            return make_float2(add_rn(v.r.h, v.r.l), add_rn(v.i.h, v.i.l));
        }
        float2 o = make_float2(add_rn(v.r.h, v.r.l), add_rn(v.i.h, v.i.l));
        if (scale != 1.0) {
            const float s = (float)scale; /* a power of two: exact */
            o.x *= s;
            o.y *= s;
        }
        return o;
    }
};

/* ------------------------------------------------------------------------ */
/* split precision: FP32 data, FP32 arithmetic, twiddles and the DFT-16      */
/* constants carried as FP64-accurate (hi, lo) FP32 pairs, so every product */
/* with an irrational factor has one rounding instead of two.               */
/* ------------------------------------------------------------------------ */
struct ArithF32 {
    using C = float2;
    using TW = float4; /* re_hi, re_lo, im_hi, im_lo */
    using S = float2;
    using Store = float2;
    static constexpr int kId = 2;
    static constexpr bool kScaled = false;

    static __host__ __device__ __forceinline__ C load_s(float2 v, int) { return v; }
    static __host__ __device__ __forceinline__ float2 store_s(C v, int, double scale)
    {
        if (scale != 1.0) {
            if (!pow2_scale(scale)) return make_float2(mulc(v.x, scale_pair(scale)),
                                                       mulc(v.y, scale_pair(scale)));
            const float s = (float)scale; /* a power of two: exact */
            v.x *= s;
            v.y *= s;
        }
        return v;
    }
    static __host__ __device__ __forceinline__ S to_smem(C v) { return v; }
    static __host__ __device__ __forceinline__ C from_smem(S v) { return v; }
    static __host__ __device__ __forceinline__ C add(C a, C b) { return make_float2(add_rn(a.x, b.x), add_rn(a.y, b.y)); }
    static __host__ __device__ __forceinline__ C sub(C a, C b) { return make_float2(sub_rn(a.x, b.x), sub_rn(a.y, b.y)); }
    static __host__ __device__ __forceinline__ C conj(C a) { return make_float2(a.x, -a.y); }
    static __host__ __device__ __forceinline__ C neg(C a) { return make_float2(-a.x, -a.y); }
    static __host__ __device__ __forceinline__ C mul_mi(C a) { return make_float2(a.y, -a.x); }
    /* x * (ch + cl) with one rounding of the sum of both products */
    static __host__ __device__ __forceinline__ float mulc(float x, df2 c)
    {
        return fmaf_(x, c.h, mul_rn(x, c.l));
    }
    static __host__ __device__ __forceinline__ C mul_w8(C a)
    {
        const df2 r2 = TFFT_DF_R2;
        return make_float2(mulc(add_rn(a.x, a.y), r2), mulc(sub_rn(a.y, a.x), r2));
    }
    static __host__ __device__ __forceinline__ C mul_w8_3(C a)
    {
        const df2 r2 = TFFT_DF_R2;
        return make_float2(mulc(sub_rn(a.y, a.x), r2), -mulc(add_rn(a.x, a.y), r2));
    }
    /* x*c + y*s with c, s as pairs: lo products first, hi products last */
    static __host__ __device__ __forceinline__ float dot2(float x, df2 c, float y, df2 s)
    {
        float t = fmaf_(x, c.l, mul_rn(y, s.l));
        t = fmaf_(y, s.h, t);
        return fmaf_(x, c.h, t);
    }
    template <int K>
    static __host__ __device__ __forceinline__ C mul_w16(C a)
    {
        const df2 c8 = TFFT_DF_C8, s8 = TFFT_DF_S8;
        const df2 c = K == 1 ? c8 : s8, s = K == 1 ? s8 : c8;
        const df2 ns = {-s.h, -s.l};
        /* re = a.x c + a.y s, im = a.y c - a.x s */
        return make_float2(dot2(a.x, c, a.y, s), dot2(a.y, c, a.x, ns));
    }
    static __host__ __device__ __forceinline__ C mul_tw(C a, TW w)
    {
        const df2 wr = {w.x, w.y}, wi = {w.z, w.w};
        const df2 nwi = {-w.z, -w.w};
        /* re = a.x wr - a.y wi, im = a.x wi + a.y wr */
        return make_float2(dot2(a.x, wr, a.y, nwi), dot2(a.x, wi, a.y, wr));
    }
    static __device__ __forceinline__ TW load_tw(const void *tab, int64_t m)
    {
        return __ldg(reinterpret_cast<const float4 *>(tab) + m);
    }
    /* product of two table pairs, kept as a pair */
    static __host__ __device__ __forceinline__ TW tw_mul(TW a, TW b)
    {
        return ArithDF64::tw_mul(a, b);
    }
    /* real constants as (hi, lo) pairs: a * c and acc + a * c */
    using R = df2;
    static __host__ __device__ constexpr R rc(double, float h, float l) { return df2{h, l}; }
    static __host__ __device__ __forceinline__ C mulr(C a, R c)
    {
        return make_float2(mulc(a.x, c), mulc(a.y, c));
    }
    static __host__ __device__ __forceinline__ C fmar(C acc, C a, R c)
    {
        return make_float2(fmaf_(a.x, c.h, fmaf_(a.x, c.l, acc.x)),
                           fmaf_(a.y, c.h, fmaf_(a.y, c.l, acc.y)));
    }
};

} // namespace tfft
