/*
 * Runtime wrappers, plan-time table kernels and the small auxiliary kernels
 * of the C2C path.  Every entry point is extern "C" with plain types; the C
 * host library (topefft.c) is the only caller.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_arith.cuh"
#include "tfft_abi.h"

/* ------------------------------------------------------------------------ */
/* runtime                                                                  */
/* ------------------------------------------------------------------------ */
extern "C" {

int tfft_set_device(int dev) { return (int)cudaSetDevice(dev); }
int tfft_get_device(int *dev) { return (int)cudaGetDevice(dev); }
int tfft_device_count(int *n) { return (int)cudaGetDeviceCount(n); }
int tfft_malloc(void **p, size_t bytes) { return (int)cudaMalloc(p, bytes ? bytes : 16); }
int tfft_free(void *p) { return p ? (int)cudaFree(p) : 0; }
int tfft_host_alloc(void **p, size_t bytes) { return (int)cudaMallocHost(p, bytes ? bytes : 16); }
int tfft_host_free(void *p) { return p ? (int)cudaFreeHost(p) : 0; }
int tfft_memset_async(void *p, int v, size_t bytes, void *s)
{
    return (int)cudaMemsetAsync(p, v, bytes, (cudaStream_t)s);
}
int tfft_h2d(void *dst, const void *src, size_t bytes, void *s)
{
    return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)s);
}
int tfft_d2h(void *dst, const void *src, size_t bytes, void *s)
{
    return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)s);
}
int tfft_d2h_2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                size_t height, void *s)
{
    return (int)cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, cudaMemcpyDeviceToHost,
                                  (cudaStream_t)s);
}
int tfft_d2d(void *dst, const void *src, size_t bytes, void *s)
{
    return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)s);
}
int tfft_stream_create(void **s)
{
    cudaStream_t st;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    *s = (void *)st;
    return (int)e;
}
int tfft_stream_destroy(void *s) { return s ? (int)cudaStreamDestroy((cudaStream_t)s) : 0; }
int tfft_stream_sync(void *s) { return (int)cudaStreamSynchronize((cudaStream_t)s); }
int tfft_stream_wait(void *s, void *e)
{
    return (int)cudaStreamWaitEvent((cudaStream_t)s, (cudaEvent_t)e, 0);
}
int tfft_event_create(void **e)
{
    cudaEvent_t ev;
    cudaError_t r = cudaEventCreate(&ev);
    *e = (void *)ev;
    return (int)r;
}
int tfft_event_destroy(void *e) { return e ? (int)cudaEventDestroy((cudaEvent_t)e) : 0; }
int tfft_event_record(void *e, void *s) { return (int)cudaEventRecord((cudaEvent_t)e, (cudaStream_t)s); }
int tfft_event_elapsed_ns(void *a, void *b, uint64_t *ns)
{
    float ms = 0.f;
    cudaError_t r = cudaEventElapsedTime(&ms, (cudaEvent_t)a, (cudaEvent_t)b);
    *ns = r == cudaSuccess ? (uint64_t)((double)ms * 1.0e6 + 0.5) : 0;
    return (int)r;
}
int tfft_last_launch_error(void) { return (int)cudaGetLastError(); }
const char *tfft_error_string(int code) { return cudaGetErrorString((cudaError_t)code); }

} /* extern "C" */

/* ------------------------------------------------------------------------ */
/* tables                                                                   */
/* ------------------------------------------------------------------------ */
namespace {

/* exp(-2 pi i m / n) for n = 2^log_n: the argument 2m/n is exact, so the
 * only rounding is sincospi's own. */
__device__ __forceinline__ double2 w_pow2(int64_t m, int log_n)
{
    double s, c;
    sincospi(ldexp((double)m, 1 - log_n), &s, &c);
    return make_double2(c, -s);
}

/* exp(-2 pi i m / n) for any n, m < n: the angle pi*2m/n is first brought
 * to pi*x with |x| <= 1/2 by exact integer steps (W^m = conj(W^(n-m)) and a
 * half turn), so the one rounding of the quotient x stays below 2^-54. */
__device__ __forceinline__ double2 w_any(int64_t m, int64_t n)
{
    int64_t num = 2 * m; /* angle pi * num / n, num in [0, 2n) */
    if (num > n) num -= 2 * n; /* (-n, n] */
    bool flip = false;
    if (2 * num > n) {
        num -= n;
        flip = true;
    } else if (2 * num < -n) {
        num += n;
        flip = true;
    }
    double s, c;
    sincospi((double)num / (double)n, &s, &c);
    return flip ? make_double2(-c, s) : make_double2(c, -s);
}

__device__ __forceinline__ void put_tw(void *tab, int64_t i, double2 w, int arith)
{
    if (arith == TFFT_ARITH_F64) {
        reinterpret_cast<double2 *>(tab)[i] = w;
    } else {
        float rh = __double2float_rn(w.x), ih = __double2float_rn(w.y);
        float rl = __double2float_rn(w.x - (double)rh), il = __double2float_rn(w.y - (double)ih);
        reinterpret_cast<float4 *>(tab)[i] = make_float4(rh, rl, ih, il);
    }
}

__global__ void k_twiddle(void *tw, int log_l, int arith)
{
    const int64_t L = int64_t(1) << log_l;
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < L;
         m += (int64_t)gridDim.x * blockDim.x)
        put_tw(tw, m, w_pow2(m, log_l), arith);
}

/* log_n < 0: n is not a power of two */
__global__ void k_fourstep(void *hi, void *lo, int64_t n, int log_n, int shift, int arith)
{
    const int64_t nlo = int64_t(1) << shift, nhi = (n + nlo - 1) >> shift;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nlo + nhi;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = i < nlo ? i : (i - nlo) << shift;
        const double2 w = log_n >= 0 ? w_pow2(m, log_n) : w_any(m % n, n);
        put_tw(i < nlo ? lo : hi, i < nlo ? i : i - nlo, w, arith);
    }
}

__global__ void k_table_any(void *tw, int len, int arith)
{
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < len; m += gridDim.x * blockDim.x)
        put_tw(tw, m, w_any(m, len), arith);
}

__global__ void k_bitrev(int *rev, int log2n)
{
    const int64_t n = int64_t(1) << log2n;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n;
         g += (int64_t)gridDim.x * blockDim.x)
        rev[g] = log2n ? (int)(__brev((unsigned)g) >> (32 - log2n)) : 0;
}

/* The reference's plan table, src/kernels1D.cl:7-13: entries k < n/4. */
__global__ void k_quarter(double2 *tw, int n)
{
    int log_n = 0;
    while ((1 << log_n) < n) log_n++;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n / 4; k += gridDim.x * blockDim.x)
        tw[k] = w_pow2(k, log_n);
}

/* W_n^m for any n (DFT path): sincospi(2m/n) with the quotient rounded once */
__global__ void k_dft_table(double2 *tw, int n)
{
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(2.0 * (double)m / (double)n, &s, &c);
        tw[m] = make_double2(c, -s);
    }
}

/* out[k] = sum_j in[j] W_n^{jk}; twiddle index advanced modulo n exactly */
__global__ void k_dft(const double2 *__restrict__ in, double2 *__restrict__ out,
                      const double2 *__restrict__ tw, int n, int dir, int64_t rows)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
        const double2 *x_row = in + r * n;
        double sr = 0.0, si = 0.0;
        int m = 0;
        for (int j = 0; j < n; j++) {
            const double2 x = x_row[j];
            double2 w = __ldg(tw + m);
            if (!dir) w.y = -w.y;
            sr = fma(x.x, w.x, fma(-x.y, w.y, sr));
            si = fma(x.x, w.y, fma(x.y, w.x, si));
            m += k;
            if (m >= n) m -= n;
        }
        const double s = dir ? 1.0 : 1.0 / (double)n;
        out[r * n + k] = make_double2(sr * s, si * s);
    }
}

/* In-place bit-reversal permutation along an axis, the reference's swap
 * (src/kernels3D.cl:574-637): element i of a line trades places with
 * rev[i] when i < rev[i].  One thread per (line, i). */
__global__ void k_bitrev_permute(double2 *d, const int *__restrict__ rev, int log2n, int64_t es,
                                 int64_t n0, int64_t s0, int64_t n1, int64_t s1)
{
    const int64_t n = int64_t(1) << log2n;
    const int64_t total = n * n0 * n1;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g0 = t % n0, rest = t / n0;
        const int64_t i = rest % n, g1 = rest / n;
        const int64_t r = rev[i];
        if (i < r) {
            double2 *line = d + g0 * s0 + g1 * s1;
            const double2 a = line[i * es], b = line[r * es];
            line[i * es] = b;
            line[r * es] = a;
        }
    }
}

/* ---- Bluestein (chirp-z) for lengths that are not powers of two --------- */
__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(fma(a.x, b.x, -(a.y * b.y)), fma(a.x, b.y, a.y * b.x));
}

/* c[k] = exp(-pi i k^2 / n): k^2 reduced mod 2n exactly, one rounding */
__global__ void k_chirp(double2 *c, int64_t n)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        /* k < 2^31, so k*k fits in 64 bits */
        const int64_t m = (int64_t)(((uint64_t)k * (uint64_t)k) % (uint64_t)(2 * n));
        double s, co;
        sincospi((double)m / (double)n, &s, &co);
        c[k] = make_double2(co, -s);
    }
}

/* b[k] = conj(c[|k|]) on the cyclic index range of length m (zero between) */
__global__ void k_bluestein_b(double2 *b, const double2 *__restrict__ c, int64_t n, int64_t m)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m;
         k += (int64_t)gridDim.x * blockDim.x) {
        double2 v = make_double2(0.0, 0.0);
        if (k < n) v = c[k];
        else if (k > m - n) v = c[m - k];
        b[k] = make_double2(v.x, -v.y);
    }
}

/* per row: w[k] = x[k] c[k] (x conjugated first for an inverse), zero-padded to m */
__global__ void k_bluestein_pre(const double2 *__restrict__ x, const double2 *__restrict__ c,
                                double2 *__restrict__ w, int64_t n, int64_t m, int conj_in,
                                int64_t rows)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m * rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / m, k = i - r * m;
        double2 v = make_double2(0.0, 0.0);
        if (k < n) {
            double2 a = x[r * n + k];
            if (conj_in) a.y = -a.y;
            v = cmul(a, c[k]);
        }
        w[i] = v;
    }
}

/* w *= h, h of length m shared by every row */
__global__ void k_pointwise(double2 *__restrict__ w, const double2 *__restrict__ h, int64_t m,
                            int64_t rows)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m * rows;
         i += (int64_t)gridDim.x * blockDim.x)
        w[i] = cmul(w[i], h[i % m]);
}

/* per row: x[k] = w[k] c[k], conjugated and scaled for an inverse */
__global__ void k_bluestein_post(const double2 *__restrict__ w, const double2 *__restrict__ c,
                                 double2 *__restrict__ x, int64_t n, int64_t m, int conj_out,
                                 double scale, int64_t rows)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / n, k = i - r * n;
        double2 v = cmul(w[r * m + k], c[k]);
        if (conj_out) v.y = -v.y;
        x[i] = make_double2(v.x * scale, v.y * scale);
    }
}

/* real-data transforms of length n = 2m through a complex transform of
 * length m: lo[i] = W_n^i (i < 2^shift), hi[h] = W_n^(h << shift) (h <= m >> shift),
 * angles from the exact ratio (i mod n)/n, one rounding each */
__global__ void k_real_tables(void *hi, void *lo, int64_t n, int shift, int64_t nhi, int arith)
{
    const int64_t nlo = int64_t(1) << shift;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nlo + nhi;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i < nlo ? i : (i - nlo) << shift;
        double s, c;
        sincospi(2.0 * (double)(e % n) / (double)n, &s, &c);
        put_tw(i < nlo ? lo : hi, i < nlo ? i : i - nlo, make_double2(c, -s),
               arith == TFFT_ARITH_F64 || arith == TFFT_ARITH_DF64 ? TFFT_ARITH_F64 : arith);
    }
}

__device__ __forceinline__ double2 w_real(const double2 *hi, const double2 *lo, int shift, int64_t k)
{
    return cmul(hi[k >> shift], lo[k & ((int64_t(1) << shift) - 1)]);
}

/* forward: Z = FFT_m(x[2j] + i x[2j+1]) per row -> X[k], k = 0..m, with
 * E = (Z[k] + conj Z[m-k])/2, O = (Z[k] - conj Z[m-k])/(2i), X = E + W_n^k O */
__global__ void k_r2c_post(const double2 *__restrict__ z, double2 *__restrict__ x,
                           const double2 *__restrict__ hi, const double2 *__restrict__ lo, int shift,
                           int64_t m, int64_t rows)
{
    const int64_t per = m + 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < per * rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / per, k = i - r * per;
        const double2 a = z[r * m + (k == m ? 0 : k)];
        double2 b = z[r * m + (k == 0 ? 0 : m - k)];
        b.y = -b.y;
        const double2 e = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
        const double2 o = make_double2(0.5 * (a.y - b.y), -0.5 * (a.x - b.x));
        const double2 wo = cmul(w_real(hi, lo, shift, k), o);
        x[i] = make_double2(e.x + wo.x, e.y + wo.y);
    }
}

/* inverse: X[0..m] per row -> Z[k] = E + i O, k < m, with E = (X[k] + conj X[m-k])/2,
 * O = (X[k] - conj X[m-k]) conj(W_n^k) / 2; FFT_m^-1(Z) then holds x[2j] + i x[2j+1] */
__global__ void k_c2r_pre(const double2 *__restrict__ x, double2 *__restrict__ z,
                          const double2 *__restrict__ hi, const double2 *__restrict__ lo, int shift,
                          int64_t m, int64_t rows)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m * rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / m, k = i - r * m;
        const double2 a = x[r * (m + 1) + k];
        double2 b = x[r * (m + 1) + m - k];
        b.y = -b.y;
        const double2 e = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
        double2 w = w_real(hi, lo, shift, k);
        w.y = -w.y;
        const double2 o = cmul(make_double2(0.5 * (a.x - b.x), 0.5 * (a.y - b.y)), w);
        z[i] = make_double2(e.x - o.y, e.y + o.x);
    }
}

/* The same two steps for FP32 storage (the split-precision forms): the
 * loads are exact in double-float, E, O and W_n^k O are formed in
 * double-float with W_n^k from (hi, lo) float pair tables, and each output
 * rounds once to FP32.  A = ArithDF32. */
using DF = tfft::ArithDF32;

__device__ __forceinline__ DF::C df_half(DF::C v)
{
    v.r.h *= 0.5f;
    v.r.l *= 0.5f;
    v.i.h *= 0.5f;
    v.i.l *= 0.5f;
    return v;
}

__device__ __forceinline__ DF::TW w_real32(const float4 *hi, const float4 *lo, int shift, int64_t k)
{
    return DF::tw_mul(__ldg(hi + (k >> shift)), __ldg(lo + (k & ((int64_t(1) << shift) - 1))));
}

__global__ void k_r2c_post32(const float2 *__restrict__ z, float2 *__restrict__ x,
                             const float4 *__restrict__ hi, const float4 *__restrict__ lo, int shift,
                             int64_t m, int64_t rows)
{
    const int64_t per = m + 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < per * rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / per, k = i - r * per;
        const DF::C a = DF::load_s(z[r * m + (k == m ? 0 : k)], 0);
        const DF::C b = DF::conj(DF::load_s(z[r * m + (k == 0 ? 0 : m - k)], 0));
        const DF::C e = df_half(DF::add(a, b));
        const DF::C o = df_half(DF::mul_mi(DF::sub(a, b))); /* (a - b) / (2i) */
        x[i] = DF::store_s(DF::add(e, DF::mul_tw(o, w_real32(hi, lo, shift, k))), 0, 1.0);
    }
}

__global__ void k_c2r_pre32(const float2 *__restrict__ x, float2 *__restrict__ z,
                            const float4 *__restrict__ hi, const float4 *__restrict__ lo, int shift,
                            int64_t m, int64_t rows)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m * rows;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / m, k = i - r * m;
        const DF::C a = DF::load_s(x[r * (m + 1) + k], 0);
        const DF::C b = DF::conj(DF::load_s(x[r * (m + 1) + m - k], 0));
        const DF::C e = df_half(DF::add(a, b));
        float4 w = w_real32(hi, lo, shift, k);
        w.z = -w.z;
        w.w = -w.w;
        const DF::C o = df_half(DF::mul_tw(DF::sub(a, b), w));
        /* z = e + i o */
        z[i] = DF::store_s(DF::sub(e, DF::mul_mi(o)), 0, 1.0);
    }
}

__global__ void k_n2(double2 *d, int dir)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double2 a = d[0], b = d[1];
        double2 x = make_double2(a.x + b.x, a.y + b.y), y = make_double2(a.x - b.x, a.y - b.y);
        if (!dir) {
            x.x *= 0.5; x.y *= 0.5;
            y.x *= 0.5; y.y *= 0.5;
        }
        d[0] = x;
        d[1] = y;
    }
}

inline unsigned grid_for(int64_t n, int threads)
{
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > 152 * 32) g = 152 * 32;
    return (unsigned)g;
}

} // namespace

extern "C" {

int tfft_twiddle_table(void *tw, int log_l, int arith, void *s)
{
    k_twiddle<<<grid_for(int64_t(1) << log_l, 256), 256, 0, (cudaStream_t)s>>>(tw, log_l, arith);
    return (int)cudaGetLastError();
}

int tfft_fourstep_tables(void *hi, void *lo, int64_t n, int shift, int arith, void *s)
{
    int log_n = 0;
    while ((int64_t(1) << log_n) < n) log_n++;
    if ((int64_t(1) << log_n) != n) log_n = -1;
    const int64_t nlo = int64_t(1) << shift, cnt = nlo + ((n + nlo - 1) >> shift);
    k_fourstep<<<grid_for(cnt, 256), 256, 0, (cudaStream_t)s>>>(hi, lo, n, log_n, shift, arith);
    return (int)cudaGetLastError();
}

int tfft_table_any(void *tw, int len, int arith, void *s)
{
    k_table_any<<<grid_for(len, 256), 256, 0, (cudaStream_t)s>>>(tw, len, arith);
    return (int)cudaGetLastError();
}

int tfft_bitrev_table(int *rev, int log2n, void *s)
{
    k_bitrev<<<grid_for(int64_t(1) << log2n, 256), 256, 0, (cudaStream_t)s>>>(rev, log2n);
    return (int)cudaGetLastError();
}

int tfft_quarter_table(void *tw, int n, void *s)
{
    if (n < 4) return 0;
    k_quarter<<<grid_for(n / 4, 256), 256, 0, (cudaStream_t)s>>>((double2 *)tw, n);
    return (int)cudaGetLastError();
}

int tfft_dft_table(void *tw, int n, void *s)
{
    k_dft_table<<<grid_for(n, 256), 256, 0, (cudaStream_t)s>>>((double2 *)tw, n);
    return (int)cudaGetLastError();
}

int tfft_launch_dft(const void *in, void *out, const void *tw, int n, int dir, int64_t rows,
                    void *s)
{
    const dim3 grid((unsigned)((n + 127) / 128), (unsigned)(rows < 65535 ? rows : 65535));
    k_dft<<<grid, 128, 0, (cudaStream_t)s>>>((const double2 *)in, (double2 *)out,
                                             (const double2 *)tw, n, dir, rows);
    return (int)cudaGetLastError();
}

int tfft_launch_bitrev_permute(void *d, const int *rev, int log2n, int64_t es, int64_t n0,
                               int64_t s0, int64_t n1, int64_t s1, void *s)
{
    const int64_t total = (int64_t(1) << log2n) * n0 * n1;
    k_bitrev_permute<<<grid_for(total, 256), 256, 0, (cudaStream_t)s>>>((double2 *)d, rev, log2n,
                                                                       es, n0, s0, n1, s1);
    return (int)cudaGetLastError();
}

int tfft_bluestein_tables(void *chirp, void *b, int64_t n, int64_t m, void *s)
{
    cudaStream_t st = (cudaStream_t)s;
    k_chirp<<<grid_for(n, 256), 256, 0, st>>>((double2 *)chirp, n);
    k_bluestein_b<<<grid_for(m, 256), 256, 0, st>>>((double2 *)b, (const double2 *)chirp, n, m);
    return (int)cudaGetLastError();
}

int tfft_bluestein_pre(const void *x, const void *chirp, void *w, int64_t n, int64_t m,
                       int conj_in, int64_t rows, void *s)
{
    k_bluestein_pre<<<grid_for(m * rows, 256), 256, 0, (cudaStream_t)s>>>(
        (const double2 *)x, (const double2 *)chirp, (double2 *)w, n, m, conj_in, rows);
    return (int)cudaGetLastError();
}

int tfft_pointwise(void *w, const void *h, int64_t m, int64_t rows, void *s)
{
    k_pointwise<<<grid_for(m * rows, 256), 256, 0, (cudaStream_t)s>>>((double2 *)w,
                                                                     (const double2 *)h, m, rows);
    return (int)cudaGetLastError();
}

int tfft_bluestein_post(const void *w, const void *chirp, void *x, int64_t n, int64_t m,
                        int conj_out, double scale, int64_t rows, void *s)
{
    k_bluestein_post<<<grid_for(n * rows, 256), 256, 0, (cudaStream_t)s>>>(
        (const double2 *)w, (const double2 *)chirp, (double2 *)x, n, m, conj_out, scale, rows);
    return (int)cudaGetLastError();
}

int tfft_real_tables(void *hi, void *lo, int64_t n, int shift, int arith, void *s)
{
    const int64_t nhi = ((n / 2) >> shift) + 1;
    k_real_tables<<<grid_for((int64_t(1) << shift) + nhi, 256), 256, 0, (cudaStream_t)s>>>(
        hi, lo, n, shift, nhi, arith);
    return (int)cudaGetLastError();
}

int tfft_r2c_post(const void *z, void *x, const void *hi, const void *lo, int shift, int64_t m,
                  int64_t rows, int arith, void *s)
{
    if (TFFT_ELEM_BYTES(arith) == 8)
        k_r2c_post32<<<grid_for((m + 1) * rows, 256), 256, 0, (cudaStream_t)s>>>(
            (const float2 *)z, (float2 *)x, (const float4 *)hi, (const float4 *)lo, shift, m, rows);
    else
        k_r2c_post<<<grid_for((m + 1) * rows, 256), 256, 0, (cudaStream_t)s>>>(
            (const double2 *)z, (double2 *)x, (const double2 *)hi, (const double2 *)lo, shift, m,
            rows);
    return (int)cudaGetLastError();
}

int tfft_c2r_pre(const void *x, void *z, const void *hi, const void *lo, int shift, int64_t m,
                 int64_t rows, int arith, void *s)
{
    if (TFFT_ELEM_BYTES(arith) == 8)
        k_c2r_pre32<<<grid_for(m * rows, 256), 256, 0, (cudaStream_t)s>>>(
            (const float2 *)x, (float2 *)z, (const float4 *)hi, (const float4 *)lo, shift, m, rows);
    else
        k_c2r_pre<<<grid_for(m * rows, 256), 256, 0, (cudaStream_t)s>>>(
            (const double2 *)x, (double2 *)z, (const double2 *)hi, (const double2 *)lo, shift, m,
            rows);
    return (int)cudaGetLastError();
}

int tfft_launch_n2(void *d, int dir, void *s)
{
    k_n2<<<1, 32, 0, (cudaStream_t)s>>>((double2 *)d, dir);
    return (int)cudaGetLastError();
}

} /* extern "C" */
