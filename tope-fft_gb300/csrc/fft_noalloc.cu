/*
 * topeExec1DNoAlloc: the 1D FP64 transform without any allocation.
 *
 * Some callers cannot allocate device memory while they run.  Typical cases:
 * a host framework that owns the GPU's memory pool and forbids cudaMalloc
 * behind its back, a pipeline with a memory budget fixed at start-up, and code
 * on a latency-critical path where cudaMalloc/cudaFree would synchronise the
 * device.  This entry point serves them: the caller passes device input and
 * output buffers, and everything else the transform needs lives in
 * file-scope device arrays that exist on every GPU that loads the library,
 * until the process exits:
 *   g_na_scratch   the four-step intermediate, 2^20 complex doubles (16 MiB)
 *   g_na_wl        the W_L twiddle tables for L = 2^1 .. 2^13
 *   g_na_fs        the four-step factor tables for n = 2^10 .. 2^20
 * Lengths are powers of two from 1 to 2^20 (TOPE_NOALLOC_MAX_N); anything
 * else is rejected with TOPE_ERR_INVALID_SIZE before any work is queued.
 * Up to 2^9 points the transform is one pass; from 2^10 on it is two
 * four-step passes (short passes with 4 points per thread), the split the
 * allocating path makes for a single line of that length.
 *
 * Set-up: the first call on each device computes the tables with that
 * device current, queued on the caller's stream, and waits for that stream
 * to finish, so make the first call before any stream capture.  Later calls
 * only queue kernels.  The set-up is published with a release store and read
 * with an acquire load, so a thread that sees it finished also sees the
 * device addresses it resolved.  Those addresses and tables belong to the
 * device's context as it was at set-up: after cudaDeviceReset (or any other
 * teardown of the primary context) the entry point must not be called again
 * in that process.  Nothing in the scratch has to start at zero: the first
 * pass writes every element the second pass reads.  All calls share the one
 * scratch array, so calls whose kernels overlap on the GPU (two streams, or
 * two host threads) race on it; serialise them.
 */
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdint.h>

#include "../../include/topefft_ext.h"
#include "tfft_abi.h"

#define NA_MAX_LOG 20
#define NA_MAX_LOG_L 13
#define NA_FS_MIN_LOG 10
#define NA_FS_ENTRIES 2048 /* 2^shift + 2^(log n - shift) <= 2 * 2^10 */

static __device__ __align__(256) double2 g_na_scratch[1 << NA_MAX_LOG];
static __device__ __align__(256) double2 g_na_wl[1 << (NA_MAX_LOG_L + 1)];
static __device__ __align__(256) double2 g_na_fs[NA_MAX_LOG - NA_FS_MIN_LOG + 1][NA_FS_ENTRIES];

#define NA_MAX_DEVICES 64

typedef struct na_dev {
    int ready; /* 1 once set-up finished: release store, acquire load */
    double2 *scratch, *wl, *fs;
} na_dev;

static na_dev g_na[NA_MAX_DEVICES];
static pthread_mutex_t g_na_lock = PTHREAD_MUTEX_INITIALIZER;

/* Resolve the arrays' device addresses on the current device and fill the
 * tables; returns a topeStatus. */
static int na_setup(int dev, cudaStream_t s)
{
    na_dev *d = &g_na[dev];
    void *p = NULL;
    if (cudaGetSymbolAddress(&p, g_na_scratch) != cudaSuccess || !p) return TOPE_ERR_CUDA;
    d->scratch = (double2 *)p;
    if (cudaGetSymbolAddress(&p, g_na_wl) != cudaSuccess || !p) return TOPE_ERR_CUDA;
    d->wl = (double2 *)p;
    if (cudaGetSymbolAddress(&p, g_na_fs) != cudaSuccess || !p) return TOPE_ERR_CUDA;
    d->fs = (double2 *)p;
    for (int lg = 1; lg <= NA_MAX_LOG_L; lg++)
        if (tfft_twiddle_table(d->wl + ((size_t)1 << lg), lg, TFFT_ARITH_F64, s)) return TOPE_ERR_CUDA;
    for (int lg = NA_FS_MIN_LOG; lg <= NA_MAX_LOG; lg++) {
        const int shift = (lg + 1) / 2;
        double2 *row = d->fs + (size_t)(lg - NA_FS_MIN_LOG) * NA_FS_ENTRIES;
        if (tfft_fourstep_tables(row + ((size_t)1 << shift), row, (int64_t)1 << lg, shift,
                                 TFFT_ARITH_F64, s))
            return TOPE_ERR_CUDA;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return TOPE_ERR_CUDA;
    __atomic_store_n(&d->ready, 1, __ATOMIC_RELEASE);
    return TOPE_SUCCESS;
}

/* lines per CTA for a pass of `lines` strided lines of 2^log_l points and
 * ept points per thread: the allocating planner's rule (about 256 threads,
 * at least 8 adjacent lines, at most 8192 points per CTA, 4096 with 4
 * points per thread), narrowed until the pass has at least 32 CTAs */
static int na_lines_per_cta(int log_l, int64_t lines, int ept)
{
    const int64_t L = (int64_t)1 << log_l;
    const int64_t e = L < ept ? L : ept;
    int64_t want = 256 * e / L;
    if (want < 8) want = 8;
    int64_t maxb = (ept == 4 ? 4096 : 8192) / L;
    if (maxb > 32) maxb = 32;
    if (want > maxb) want = maxb;
    if (want > lines) want = lines;
    if (want < 1) want = 1;
    while (want > 1 && lines / want < 32) want >>= 1;
    return (int)want;
}

/* 4 points per thread for short passes of at most 2^16 points */
static int na_ept(int log_l, int64_t points)
{
    return log_l >= 2 && log_l <= 7 && points <= 65536 ? 4 : 0;
}

static void na_pass_init(tfft_pass *p, int log_l, const double2 *tw)
{
    p->log_l = log_l;
    p->arith = TFFT_ARITH_F64;
    p->scale = 1.0;
    p->n[0] = p->n[1] = p->n[2] = 1;
    p->tw = tw;
}

extern "C" int topeExec1DNoAlloc(const double *d_in, double *d_out, int n, int dir,
                                 void *stream)
{
    if (!d_in || !d_out || (dir != FORWARD && dir != INVERSE)) return TOPE_ERR_INVALID_ARG;
    int lg = 0;
    while (lg <= NA_MAX_LOG && (1 << lg) < n) lg++;
    if (n < 1 || lg > NA_MAX_LOG || (1 << lg) != n) return TOPE_ERR_INVALID_SIZE;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return TOPE_ERR_CUDA;
    if (!__atomic_load_n(&g_na[dev].ready, __ATOMIC_ACQUIRE)) {
        pthread_mutex_lock(&g_na_lock);
        int st = __atomic_load_n(&g_na[dev].ready, __ATOMIC_ACQUIRE) ? TOPE_SUCCESS
                                                                     : na_setup(dev, s);
        pthread_mutex_unlock(&g_na_lock);
        if (st) return st;
    }
    const na_dev *d = &g_na[dev];
    const int inv = dir == INVERSE;
    const double scale = inv ? 1.0 / (double)n : 1.0;
    tfft_pass p = {0};
    if (lg < NA_FS_MIN_LOG) {
        /* one pass, input to output */
        na_pass_init(&p, lg, d->wl + ((size_t)1 << lg));
        p.in = d_in;
        p.out = d_out;
        p.ies = p.oes = 1;
        p.b_tile = 1;
        p.ept = na_ept(lg, n);
        p.conj_in = p.conj_out = inv;
        p.scale = scale;
        return tfft_launch_pass(&p, stream) ? TOPE_ERR_CUDA : TOPE_SUCCESS;
    }
    /* four-step, n = n1 * n2: pass A input -> scratch along i2 with the
     * W_n^{i1 k2} factors, pass B scratch -> output along i1, transposed */
    const int l1 = lg / 2, l2 = lg - l1;
    const int64_t n1 = (int64_t)1 << l1, n2 = (int64_t)1 << l2;
    const int shift = (lg + 1) / 2;
    const double2 *fs = d->fs + (size_t)(lg - NA_FS_MIN_LOG) * NA_FS_ENTRIES;
    na_pass_init(&p, l2, d->wl + ((size_t)1 << l2));
    p.in = d_in;
    p.out = d->scratch;
    p.ies = p.oes = n1;
    p.n[0] = n1;
    p.is[0] = p.os[0] = 1;
    p.ept = na_ept(l2, n);
    p.b_tile = na_lines_per_cta(l2, n1, p.ept ? 4 : 16);
    p.conj_in = inv;
    p.post_tw = 1;
    p.tw_level = 0;
    p.tw_shift = shift;
    p.tw_n = n;
    p.tw_lo = fs;
    p.tw_hi = fs + ((size_t)1 << shift);
    if (tfft_launch_pass(&p, stream)) return TOPE_ERR_CUDA;
    tfft_pass q = {0};
    na_pass_init(&q, l1, d->wl + ((size_t)1 << l1));
    q.in = d->scratch;
    q.out = d_out;
    q.ies = 1;
    q.oes = n2;
    q.n[0] = n2;
    q.is[0] = n1;
    q.os[0] = 1;
    q.ept = na_ept(l1, n);
    q.b_tile = na_lines_per_cta(l1, n2, q.ept ? 4 : 16);
    q.conj_out = inv;
    q.scale = scale;
    return tfft_launch_pass(&q, stream) ? TOPE_ERR_CUDA : TOPE_SUCCESS;
}
