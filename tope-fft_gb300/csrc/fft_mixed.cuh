/*
 * Lines whose length L is not a power of two: L = 2^a 3^b 5^c 7^d 11^e 13^f
 * (the reference's 1D path runs such lengths through its O(N^2) DFT
 * kernel, src/kernels1D.cl:549-573).
 *
 * One CTA of 256 threads transforms b_tile lines (L * b_tile <= 4096 points)
 * in shared memory, in Stockham autosort stages of the radices the host put
 * in tfft_pass::radix (natural order out, no permutation pass).  Stage s of
 * radix R with span Ns (the product of the earlier radices) takes, for each
 * j < L/R with k = j mod Ns, the R points j + q L/R, multiplies point q by
 * W_{Ns R}^{q k} (a per-L table of W_L^m), runs an R-point DFT and writes
 * output q to (j - k) R + k + q Ns.  Radix 2, 4, 8 use the power-of-two
 * butterflies of fft_pass.cuh; odd radices use the symmetric form
 *   y_0 = x_0 + sum_q a_q,  y_k, y_{R-k} = A_k -/+ i B_k,
 *   A_k = x_0 + sum_q cos(2 pi q k/R) a_q,  B_k = sum_q sin(2 pi q k/R) b_q,
 * with a_q = x_q + x_{R-q}, b_q = x_q - x_{R-q}, q = 1..(R-1)/2.
 * Shared memory holds two buffers (ping-pong) at index e + e/8 for
 * e = point * b_tile + line, so that 16-byte accesses of consecutive
 * threads along either index spread over the banks.
 *
 * Loads and stores are coalesced along whichever of the element stride and
 * the line stride is 1; the four-step twiddle W_N^{t k}, conjugation and
 * the inverse scale are fused into the store as in the power-of-two pass.
 */
#pragma once
#include <type_traits>
#include "fft_pass.cuh"

namespace tfft {

constexpr int kMixedThreads = 256;

__host__ __device__ constexpr int mixed_pad(int e) { return e + (e >> 3); }

/* bytes of shared memory for a tile of pts points (two buffers plus the
 * tile-exponent word) */
constexpr size_t mixed_smem_bytes(int pts, int sbytes)
{
    return 2 * (size_t)mixed_pad(pts) * (size_t)sbytes + 16;
}

/* cos(2 pi m / r), sin(2 pi m / r) for r = 3, 5, 7, 11, 13, m < r: nearest
 * doubles, and as (hi, lo) float pairs (hi the nearest float, lo the nearest
 * float to the remainder) */
#include "fft_mixed_consts.inc"

template <class A>
__device__ __forceinline__ typename A::R odd_c(int r, int m)
{
    return A::rc(odd_cos(r, m), odd_cos_hi(r, m), odd_cos_lo(r, m));
}
template <class A>
__device__ __forceinline__ typename A::R odd_s(int r, int m)
{
    return A::rc(odd_sin(r, m), odd_sin_hi(r, m), odd_sin_lo(r, m));
}

/* forward R-point DFT (R odd) in place */
template <class A, int R>
__device__ __forceinline__ void dft_odd(typename A::C *x)
{
    using C = typename A::C;
    constexpr int H = (R - 1) / 2;
    C a[H], b[H];
#pragma unroll
    for (int q = 1; q <= H; q++) {
        a[q - 1] = A::add(x[q], x[R - q]);
        b[q - 1] = A::sub(x[q], x[R - q]);
    }
    C y0 = x[0];
#pragma unroll
    for (int q = 0; q < H; q++) y0 = A::add(y0, a[q]);
#pragma unroll
    for (int k = 1; k <= H; k++) {
        C ak = x[0];
        C bk = A::mulr(b[0], odd_s<A>(R, k % R));
#pragma unroll
        for (int q = 1; q <= H; q++) {
            ak = A::fmar(ak, a[q - 1], odd_c<A>(R, (q * k) % R));
            if (q > 1) bk = A::fmar(bk, b[q - 1], odd_s<A>(R, (q * k) % R));
        }
        const C t = A::mul_mi(bk); /* -i B_k */
        x[k] = A::add(ak, t);
        x[R - k] = A::sub(ak, t);
    }
    x[0] = y0;
}

template <class A, int R>
__device__ __forceinline__ void mixed_dft(typename A::C *x)
{
    if constexpr (R == 2 || R == 4 || R == 8) dft<A, R>(x);
    else dft_odd<A, R>(x);
}

/* One stage.  FIRST: the source holds the tile as loaded (storage elements),
 * converted here with the tile exponent delta (and lifted by 2^600 when
 * lift), conjugated for an inverse. */
template <class A, int R, bool FIRST>
__device__ __forceinline__ void mixed_stage(const tfft_pass &p, const void *src,
                                            typename A::S *dst, int L, int B, int Ns, int delta,
                                            bool lift)
{
    using C = typename A::C;
    const int LR = L / R, nb = LR * B, tw_step = L / (Ns * R);
    for (int u = threadIdx.x; u < nb; u += kMixedThreads) {
        const int b = u & (B - 1), j = u / B;
        const int k = j % Ns;
        C x[R];
#pragma unroll
        for (int q = 0; q < R; q++) {
            const int e = mixed_pad((j + q * LR) * B + b);
            if constexpr (FIRST) {
                typename A::Store v = reinterpret_cast<const typename A::Store *>(src)[e];
                if constexpr (A::kScaled) {
                    if (lift) {
                        v.x *= 0x1p600;
                        v.y *= 0x1p600;
                    }
                }
                const C c = A::load_s(v, delta);
                x[q] = p.conj_in ? A::conj(c) : c;
            } else {
                x[q] = A::from_smem(reinterpret_cast<const typename A::S *>(src)[e]);
            }
            if (!FIRST && q > 0) x[q] = A::mul_tw(x[q], A::load_tw(p.tw, (int64_t)(q * k * tw_step)));
        }
        mixed_dft<A, R>(x);
        const int o = (j - k) * R + k;
#pragma unroll
        for (int q = 0; q < R; q++) dst[mixed_pad((o + q * Ns) * B + b)] = A::to_smem(x[q]);
    }
}

template <class A, bool FIRST>
__device__ __forceinline__ void mixed_stage_r(int r, const tfft_pass &p, const void *src,
                                              typename A::S *dst, int L, int B, int Ns, int delta,
                                              bool lift)
{
    switch (r) {
    case 2: mixed_stage<A, 2, FIRST>(p, src, dst, L, B, Ns, delta, lift); break;
    case 3: mixed_stage<A, 3, FIRST>(p, src, dst, L, B, Ns, delta, lift); break;
    case 4: mixed_stage<A, 4, FIRST>(p, src, dst, L, B, Ns, delta, lift); break;
    case 5: mixed_stage<A, 5, FIRST>(p, src, dst, L, B, Ns, delta, lift); break;
    case 7: mixed_stage<A, 7, FIRST>(p, src, dst, L, B, Ns, delta, lift); break;
    case 8: mixed_stage<A, 8, FIRST>(p, src, dst, L, B, Ns, delta, lift); break;
    case 11: mixed_stage<A, 11, FIRST>(p, src, dst, L, B, Ns, delta, lift); break;
    case 13: mixed_stage<A, 13, FIRST>(p, src, dst, L, B, Ns, delta, lift); break;
    default: break;
    }
}

template <class A>
__global__ void __launch_bounds__(kMixedThreads, pass_min_blocks<A, kMixedThreads>())
    mixed_kernel(const tfft_pass p)
{
    using S = typename A::S;
    using Store = typename A::Store;
    using C = typename A::C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = p.len, B = p.b_tile, pts = L * B, padded = mixed_pad(pts);
    S *buf0 = reinterpret_cast<S *>(smem_raw);
    S *buf1 = buf0 + padded;
    unsigned *sh_exp = reinterpret_cast<unsigned *>(buf1 + padded);

    /* tile: lines g0first .. g0first + B - 1 of dimension 0 (a ragged last
     * tile reads its missing lines from the last line and stores nothing) */
    const int64_t tiles0 = (p.n[0] + B - 1) / B;
    const int64_t g0first = ((int64_t)blockIdx.x % tiles0) * B;
    const int64_t rest = (int64_t)blockIdx.x / tiles0;
    const int64_t g1 = rest % p.n[1], g2 = rest / p.n[1];
    const int64_t ibase = g1 * p.is[1] + g2 * p.is[2];
    const int64_t obase = g1 * p.os[1] + g2 * p.os[2];
    if (A::kScaled && threadIdx.x == 0) *sh_exp = 0;

    /* load: along the elements when they are contiguous, else along lines */
    const Store *in = reinterpret_cast<const Store *>(p.in);
    Store *raw = reinterpret_cast<Store *>(buf0);
    const bool rows_in = p.ies == 1;
    unsigned mexp = 0;
    for (int idx = threadIdx.x; idx < pts; idx += kMixedThreads) {
        const int b = rows_in ? idx / L : idx & (B - 1);
        const int i = rows_in ? idx - b * L : idx / B;
        const int64_t g0 = min(g0first + b, p.n[0] - 1);
        const Store v = __ldcs(in + ibase + g0 * p.is[0] + (int64_t)i * p.ies);
        if constexpr (A::kScaled) mexp = max(mexp, max(dexp(v.x), dexp(v.y)));
        raw[mixed_pad(i * B + b)] = v;
    }
    int delta = 0, delta_out = 0;
    bool lift = false;
    if constexpr (A::kScaled) {
        /* the tile's largest FP64 exponent (see finish_tile in fft_pass.cuh) */
        __syncthreads();
        mexp = __reduce_max_sync(0xffffffffu, mexp);
        if ((threadIdx.x & 31) == 0) atomicMax(sh_exp, mexp);
        __syncthreads();
        delta = delta_out = (int)*sh_exp - 1023;
        if (delta < -900) {
            lift = true;
            delta += 600;
        }
    }

    /* stages, ping-pong between the two buffers */
    const void *src = buf0;
    S *dst = buf1;
    int Ns = 1;
    for (int s = 0; s < p.nrad; s++) {
        __syncthreads();
        const int r = p.radix[s];
        if (s == 0) mixed_stage_r<A, true>(r, p, src, dst, L, B, Ns, delta, lift);
        else mixed_stage_r<A, false>(r, p, src, dst, L, B, Ns, delta, lift);
        S *t = const_cast<S *>(reinterpret_cast<const S *>(src));
        src = dst;
        dst = t;
        Ns *= r;
    }
    __syncthreads();

    /* store, with the four-step twiddle, conjugation and scale */
    const S *res = reinterpret_cast<const S *>(src);
    Store *out = reinterpret_cast<Store *>(p.out);
    const bool rows_out = p.oes == 1;
    const int64_t mask = (int64_t(1) << p.tw_shift) - 1;
    /* scale 1 (every pass but an inverse's last) in a loop of its own, so
     * the per-element test of the double-precision scale folds away */
    auto store_all = [&](auto unit_scale) {
        const double scale = decltype(unit_scale)::value ? 1.0 : p.scale;
        for (int idx = threadIdx.x; idx < pts; idx += kMixedThreads) {
            const int b = rows_out ? idx / L : idx & (B - 1);
            const int i = rows_out ? idx - b * L : idx / B;
            const int64_t g0 = g0first + b;
            if (g0 >= p.n[0]) continue;
            C v = A::from_smem(res[mixed_pad(i * B + b)]);
            if (p.post_tw) {
                const int64_t t = p.tw_level == 0 ? g0 : g1;
                const int64_t m = t * (int64_t)i; /* < N: no reduction needed */
                v = A::mul_tw(v, p.tw_lo ? A::tw_mul(A::load_tw(p.tw_hi, m >> p.tw_shift),
                                                     A::load_tw(p.tw_lo, m & mask))
                                         : A::load_tw(p.tw_hi, m));
            }
            if (p.conj_out) v = A::conj(v);
            __stcs(out + obase + g0 * p.os[0] + (int64_t)i * p.oes, A::store_s(v, delta_out, scale));
        }
    };
    if (p.scale == 1.0) store_all(std::true_type{});
    else store_all(std::false_type{});
}

template <class A>
int launch_mixed_t(const tfft_pass &p, cudaStream_t s)
{
    constexpr size_t smem_max =
        mixed_smem_bytes(TFFT_MIXED_MAX_POINTS, (int)sizeof(typename A::S));
    static unsigned attr_done = 0; /* one bit per device ordinal */
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned bit = 1u << (dev & 31);
    if (!(attr_done & bit)) {
        cudaError_t e = cudaFuncSetAttribute(
            mixed_kernel<A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
        if (e != cudaSuccess) return (int)e;
        attr_done |= bit;
    }
    const size_t smem = mixed_smem_bytes(p.len * p.b_tile, (int)sizeof(typename A::S));
    const int64_t blocks = ((p.n[0] + p.b_tile - 1) / p.b_tile) * p.n[1] * p.n[2];
    if (blocks <= 0) return 0;
    mixed_kernel<A><<<(unsigned)blocks, kMixedThreads, smem, s>>>(p);
    return (int)cudaGetLastError();
}

} // namespace tfft
