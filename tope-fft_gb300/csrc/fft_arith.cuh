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

namespace tfft {

/* cos(pi/8), sin(pi/8), sqrt(1/2): nearest doubles */
#define TFFT_C8 0.92387953251128675613
#define TFFT_S8 0.38268343236508977173
#define TFFT_R2 0.70710678118654752440

struct ArithF64 {
    using C = double2;
    using TW = double2;
    using S = double2;
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
    static __device__ __forceinline__ C scale(C a, double s) { return make_double2(a.x * s, a.y * s); }
};

} // namespace tfft
