/*
 * Host side of the GB300 FFT library: the reference's plan / execute /
 * destroy surface (include/topefft.h) and its extensions (topefft_ext.h),
 * in C.  Device work goes through the plain-C ABI of tfft_abi.h.
 *
 * A plan, whatever its dimensionality, is an array of up to three axes
 * (x fastest) plus a batch count, resident in device memory, and a list of
 * passes.  Each axis of length n = 2^lg becomes
 *   - one pass when lg <= 13 (one CTA transforms a whole line on chip), or
 *   - two passes (four-step, n = n1*n2) when lg > 13: pass A transforms
 *     along i2 in place and multiplies by W_n^{i1 k2}; pass B transforms
 *     along i1 and writes the transposed, natural-order result into the
 *     plan's second buffer, which then holds the data.
 * This replaces the reference's swap pass plus one global-memory pass per
 * radix stage (fft1d.c:41-114, fft2d.c:12-133, fft3d.c:12-213).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/topefft.h"
#include "../../include/topefft_ext.h"
#include "tfft_abi.h"
#include "topefft_internal.h"

#define TOPE_MAGIC 0x70EFF7u
#define MAX_PASSES 12
#define MAX_TABS 16

/* ------------------------------------------------------------------------ */
/* errors                                                                   */
/* ------------------------------------------------------------------------ */
static __thread int g_last_error = TOPE_SUCCESS;
static __thread int g_last_cuda = 0;

static int set_status(struct topeFFT *f, int st)
{
    if (f) f->error = st;
    if (st != TOPE_SUCCESS) g_last_error = st;
    return st;
}

static int cuda_status(struct topeFFT *f, int cuda_rc)
{
    if (cuda_rc == 0) return TOPE_SUCCESS;
    g_last_cuda = cuda_rc;
    return set_status(f, TOPE_ERR_CUDA);
}

int topeGetLastError(void)
{
    int e = g_last_error;
    g_last_error = TOPE_SUCCESS;
    return e;
}

int topePeekLastError(void) { return g_last_error; }
int topeLastCudaError(void) { return g_last_cuda; }

const char *topeErrorString(int st)
{
    switch (st) {
    case TOPE_SUCCESS: return "success";
    case TOPE_ERR_INVALID_SIZE: return "unsupported transform size";
    case TOPE_ERR_INVALID_ARG: return "invalid argument";
    case TOPE_ERR_ALLOC: return "allocation failed";
    case TOPE_ERR_CUDA: return "CUDA call failed";
    case TOPE_ERR_NOT_INITIALIZED: return "framework not initialised";
    case TOPE_ERR_DESTROYED: return "plan already destroyed";
    case TOPE_ERR_UNSUPPORTED: return "operation not supported";
    case TOPE_ERR_TIMEOUT: return "device-side wait timed out";
    default: return "unknown status";
    }
}

/* ------------------------------------------------------------------------ */
/* framework                                                                */
/* ------------------------------------------------------------------------ */
typedef struct tope_evpair {
    void *a, *b;
} tope_evpair;

/* slices of the last pass whose read-back overlaps the next slice */
#define RB_SLICES 8

typedef struct tope_fw {
    unsigned magic;
    void *stream;
    tope_evpair pair;
    /* overlapped read-back: a copy stream and one event per slice, made on
     * first use */
    void *copy;
    void *slice_ev[RB_SLICES];
} tope_fw;

uint64_t profileThis(void *event)
{
    tope_evpair *p = (tope_evpair *)event;
    uint64_t ns = 0;
    if (p && p->a && p->b) tfft_event_elapsed_ns(p->a, p->b, &ns);
    return ns;
}

static tope_fw *fw_of(struct topeFFT *f)
{
    tope_fw *w = f ? (tope_fw *)f->context : NULL;
    return (w && w->magic == TOPE_MAGIC) ? w : NULL;
}

static int fw_open(struct topeFFT *f)
{
    int dev = 0, n = 0, rc;
    const char *ed = getenv("TOPEFFT_DEVICE");
    rc = tfft_device_count(&n);
    if (rc || n < 1) return cuda_status(f, rc ? rc : 100 /* cudaErrorNoDevice */);
    if (ed) dev = atoi(ed);
    else tfft_get_device(&dev);
    if (dev < 0 || dev >= n) return set_status(f, TOPE_ERR_INVALID_ARG);
    if ((rc = tfft_set_device(dev))) return cuda_status(f, rc);
    tope_fw *w = (tope_fw *)calloc(1, sizeof(tope_fw));
    if (!w) return set_status(f, TOPE_ERR_ALLOC);
    if ((rc = tfft_stream_create(&w->stream)) || (rc = tfft_event_create(&w->pair.a)) ||
        (rc = tfft_event_create(&w->pair.b))) {
        tfft_event_destroy(w->pair.a);
        tfft_stream_destroy(w->stream);
        free(w);
        return cuda_status(f, rc);
    }
    w->magic = TOPE_MAGIC;
    f->context = w;
    f->command_queue = w->stream;
    f->event = &w->pair;
    f->device_ordinal = dev;
    f->ret_num_platforms = 1;
    f->ret_num_devices = (unsigned)n;
    return TOPE_SUCCESS;
}

static void fw_close(struct topeFFT *f)
{
    tope_fw *w = fw_of(f);
    if (!w) return;
    tfft_stream_sync(w->stream);
    if (w->copy) tfft_stream_sync(w->copy);
    tfft_event_destroy(w->pair.a);
    tfft_event_destroy(w->pair.b);
    for (int i = 0; i < RB_SLICES; i++) tfft_event_destroy(w->slice_ev[i]);
    tfft_stream_destroy(w->copy);
    tfft_stream_destroy(w->stream);
    w->magic = 0;
    free(w);
    f->context = NULL;
    f->command_queue = NULL;
    f->event = NULL;
}

void topeFFTInit(struct topeFFT *f)
{
    if (!f) {
        set_status(NULL, TOPE_ERR_INVALID_ARG);
        return;
    }
    memset(f, 0, sizeof(*f));
    const char *ea = getenv("TOPEFFT_ARITH");
    f->arith = (ea && (!strcmp(ea, "df64") || !strcmp(ea, "DF64"))) ? TOPE_ARITH_DF64
                                                                     : TOPE_ARITH_FP64;
    set_status(f, fw_open(f));
}

void topeFFTDestroy(struct topeFFT *f)
{
    if (!f) return;
    fw_close(f);
    f->live_plans = 0;
    set_status(f, TOPE_SUCCESS);
}

void topeSetArith(struct topeFFT *f, int arith)
{
    if (!f || (arith != TOPE_ARITH_FP64 && arith != TOPE_ARITH_DF64)) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    f->arith = arith;
    set_status(f, TOPE_SUCCESS);
}

void topeSetSplitMode(struct topeFFT *f, int mode)
{
    if (!f || (mode != TOPE_SPLIT_ACCURATE && mode != TOPE_SPLIT_FAST &&
               mode != TOPE_SPLIT_TENSOR)) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    f->split_mode = mode;
    set_status(f, TOPE_SUCCESS);
}

/* arithmetic of FP32 plans: double-float on chip unless the fast or the
 * tensor-core mode */
static int split_arith(const struct topeFFT *f)
{
    if (f && f->split_mode == TOPE_SPLIT_FAST) return TFFT_ARITH_F32;
    if (f && f->split_mode == TOPE_SPLIT_TENSOR) return TFFT_ARITH_TC;
    return TFFT_ARITH_DF32;
}

/* ------------------------------------------------------------------------ */
/* plan                                                                     */
/* ------------------------------------------------------------------------ */
enum { MODE_FFT = 0, MODE_N2 = 1, MODE_DFT = 2, MODE_BLUESTEIN = 3 };

/* lengths that are not powers of two: the O(N^2) DFT below this, Bluestein
 * (three power-of-two FFTs of length >= 2N-1) from it on */
#define BLUESTEIN_MIN_N 128

typedef struct tope_impl {
    unsigned magic;
    int ndim;            /* 1, 2, 3 */
    int64_t c[4];        /* x, y, z, batch */
    int64_t st[4];       /* strides in complex elements */
    int64_t volume;      /* x*y*z: points of one transform */
    int64_t total;       /* volume * batch */
    int arith;
    int es;              /* bytes per complex element in memory */
    int mode;
    void *buf[2];
    int cur;
    int npass;
    tfft_pass pass[MAX_PASSES];
    int oop[MAX_PASSES];
    int axis_first[3], axis_count[3];
    void *tabs[MAX_TABS];
    int tab_key[MAX_TABS]; /* log_l * 8 + arith for W_L tables, -1 otherwise */
    int ntabs;
    int *bitrev[3];
    void *quarter[3];
    void *dft_tab;
    /* Bluestein: power-of-two sub-plan of length m, chirp and transformed kernel */
    struct tope_impl *sub;
    void *chirp, *bhat;
    int64_t bl_m;
    void *tc_matrix; /* tensor form: the DFT-16 matrix pieces */
    int *err_word;   /* device word set when a wait for bulk or TMA tile copies
                        gives up (allocated with the first pass that stages tiles) */
    /* strided passes of adjacent lines that may stage tiles by TMA, and their
     * tensor maps over buf[0] and buf[1] (NULL where none was built) */
    int tma_cand[MAX_PASSES];
    void *tmap_dev[MAX_PASSES][2];
    /* real-data plan (R2C): the complex transform of length m = n/2 runs on
     * the packed reals; spec holds the m + 1 outputs per row */
    int real;
    void *spec;
    void *rtw_hi, *rtw_lo;
    int rtw_shift;
    int spec_cur; /* the spectrum, not the real array, is the current data */
    /* 2D/3D real-data plan: the C2C plan over the spectrum's y (and z) axes,
     * whose buffer holds the spectrum (x/2 + 1 points per row) */
    struct tope_impl *specp;
    tope_evpair kev, mev;
    int pending;         /* kev recorded by an async exec, not yet accounted */
    int last_dir;
    /* per-launch timing: a pool of event pairs, one per recorded launch */
    void **pev;
    int *pev_pass;
    int pev_cap, pev_used;
    uint64_t pass_ns[MAX_PASSES], pass_launches[MAX_PASSES];
} tope_impl;

static int ilog2_exact64(int64_t n)
{
    if (n < 1) return -1;
    int l = 0;
    while (((int64_t)1 << l) < n) l++;
    return (((int64_t)1 << l) == n) ? l : -1;
}

/* reference radix rule (fft1d.c:317-329) and its stage count (:366-369) */
static int ref_radix(int lg) { return lg % 3 == 0 ? 8 : lg % 2 == 0 ? 4 : 2; }
static int ref_stages(int lg)
{
    int r = ref_radix(lg);
    return r == 8 ? lg / 3 : r == 4 ? lg / 2 : lg;
}

static int impl_alloc_tab(tope_impl *P, size_t bytes, int key, void **out)
{
    if (P->ntabs >= MAX_TABS) return TOPE_ERR_UNSUPPORTED;
    int rc = tfft_malloc(out, bytes);
    if (rc) return TOPE_ERR_ALLOC;
    P->tabs[P->ntabs] = *out;
    P->tab_key[P->ntabs] = key;
    P->ntabs++;
    return TOPE_SUCCESS;
}

static size_t tw_elem_bytes(int arith) { (void)arith; return 16; }

/* W_L table shared by every pass of length L */
static int impl_wl_table(struct topeFFT *f, tope_impl *P, int log_l, const void **out)
{
    int key = log_l * 8 + P->arith;
    for (int i = 0; i < P->ntabs; i++)
        if (P->tab_key[i] == key) {
            *out = P->tabs[i];
            return TOPE_SUCCESS;
        }
    void *t;
    int st = impl_alloc_tab(P, tw_elem_bytes(P->arith) << log_l, key, &t);
    if (st) return set_status(f, st);
    int rc = tfft_twiddle_table(t, log_l, P->arith, f->command_queue);
    if (rc) return cuda_status(f, rc);
    *out = t;
    return TOPE_SUCCESS;
}

/* largest power of two dividing v, capped */
static int pow2_divisor(int64_t v, int cap)
{
    int b = 1;
    while (b < cap && v % (2 * b) == 0) b *= 2;
    return b;
}

/* lines per CTA: about 256 threads, at least 8 adjacent lines when the
 * line itself is strided (128-byte segments), at most 8192 points per CTA.
 * Strided native-FP64 lines of 4096 points are the exception (f64): their
 * pass is bound by the FP64 pipe, and one line per CTA (256-thread CTAs, two
 * per SM) measured 4.8% faster at 2^24 than two lines per 512-thread CTA;
 * the double-float and FP32-storage passes measured up to 12% slower so. */
static int choose_b(int log_l, int64_t n0, int strided, int ept, int f64)
{
    int64_t L = (int64_t)1 << log_l;
    int64_t e = L < ept ? L : ept;
    int64_t want = 256 * e / L;
    if (want < 1) want = 1;
    if (strided && want < 8 && !(f64 && L >= 4096)) want = 8;
    int64_t maxb = (ept == 4 ? 4096 : 8192) / L;
    if (maxb > 32) maxb = 32;
    if (want > maxb) want = maxb;
    if (want < 1) want = 1;
    /* a line count with no large power-of-two divisor (a real plan's
     * spectrum width x/2 + 1, odd batch counts) takes full tiles and one
     * ragged last tile rather than narrow tiles */
    int b = pow2_divisor(n0, (int)want);
    if (b < want && n0 > want) b = (int)want;
    return b;
}

/* radices a line length is built from: the mixed-radix kernel's set */
static const int k_smooth_primes[] = {2, 3, 5, 7, 11, 13};

/* n = 2^a 3^b 5^c 7^d 11^e 13^f? */
static int is_smooth(int64_t n)
{
    if (n < 1) return 0;
    for (int i = 0; i < 6; i++)
        while (n % k_smooth_primes[i] == 0) n /= k_smooth_primes[i];
    return n == 1;
}

/* Stockham radices of a mixed-radix line: 8s, then a 4 or a 2, then the
 * odd primes; returns the count */
static int mixed_radices(int64_t len, unsigned char *radix)
{
    int n = 0;
    while (len % 8 == 0 && n < TFFT_MAX_RADICES) {
        radix[n++] = 8;
        len /= 8;
    }
    if (len % 4 == 0) {
        radix[n++] = 4;
        len /= 4;
    }
    if (len % 2 == 0) {
        radix[n++] = 2;
        len /= 2;
    }
    for (int i = 1; i < 6; i++)
        while (len % k_smooth_primes[i] == 0 && n < TFFT_MAX_RADICES) {
            radix[n++] = (unsigned char)k_smooth_primes[i];
            len /= k_smooth_primes[i];
        }
    return len == 1 ? n : -1;
}

/* four-step factors of at most this many points come from one whole table
 * of W_N (16 N bytes, at most 64 MB, which stays in the 129 MB L2) in FP64
 * plans; at 2^24 points a 256 MB table read at scattered indices gained
 * under 1% for 50% more memory */
#define FULL_TW_MAX ((int64_t)1 << 22)

/* lines per CTA of a mixed-radix pass: a power of two (at most 256) with
 * about 2048 points per CTA (4096 for lines longer than 2048) */
static int choose_b_mixed(int64_t len, int64_t n0)
{
    const int64_t pts = len <= 2048 ? 2048 : TFFT_MIXED_MAX_POINTS;
    int64_t want = 1;
    while (want * 2 <= 256 && len * want * 2 <= pts) want *= 2;
    while (want > 1 && want / 2 >= n0) want /= 2;
    return (int)want;
}

/* W_L table of a mixed-radix pass of length L */
static int impl_mixed_table(struct topeFFT *f, tope_impl *P, int64_t len, const void **out)
{
    int key = -2 - (int)(len * 8 + P->arith); /* below the four-step tables' -1 */
    for (int i = 0; i < P->ntabs; i++)
        if (P->tab_key[i] == key) {
            *out = P->tabs[i];
            return TOPE_SUCCESS;
        }
    void *t;
    int st = impl_alloc_tab(P, tw_elem_bytes(P->arith) * (size_t)len, key, &t);
    if (st) return set_status(f, st);
    int rc = tfft_table_any(t, (int)len, P->arith, f->command_queue);
    if (rc) return cuda_status(f, rc);
    *out = t;
    return TOPE_SUCCESS;
}

typedef struct dimref {
    int64_t count, in_stride, out_stride;
    int is_twiddle; /* the four-step index i1 */
} dimref;

static void sort_dims(dimref *d, int n)
{
    for (int i = 1; i < n; i++)
        for (int j = i; j > 0 && d[j].out_stride < d[j - 1].out_stride; j--) {
            dimref t = d[j];
            d[j] = d[j - 1];
            d[j - 1] = t;
        }
}

/* merge neighbours that are contiguous in both input and output */
static int merge_dims(dimref *d, int n)
{
    int m = 0;
    for (int i = 0; i < n; i++) {
        if (d[i].count == 1) continue;
        if (m > 0 && !d[m - 1].is_twiddle && !d[i].is_twiddle &&
            d[i].in_stride == d[m - 1].in_stride * d[m - 1].count &&
            d[i].out_stride == d[m - 1].out_stride * d[m - 1].count) {
            d[m - 1].count *= d[i].count;
            continue;
        }
        d[m++] = d[i];
    }
    return m;
}

/* How plans load full tiles (the same transform, other load paths: for
 * comparing them).  TOPEFFT_BULK=0: every tile directly; 1: tiles of
 * contiguous lines by bulk copies, strided ones directly; 2: strided tiles by
 * TMA boxes from tensor maps as well.  Unset (-1): contiguous tiles by bulk
 * copies, and strided tiles by TMA boxes in the double-float FP64-storage
 * arithmetic only, the one where they measured faster (256^3: 1.3%; FP32
 * storage and native FP64 were 0-4% slower so). */
static int bulk_level(void)
{
    const char *e = getenv("TOPEFFT_BULK");
    return !e || !e[0] ? -1 : e[0] == '0' ? 0 : e[0] == '2' ? 2 : 1;
}

/* stage full tiles of adjacent strided lines by TMA in this arithmetic? */
static int tma_enabled(int arith)
{
    const int lv = bulk_level();
    return lv == 2 || (lv < 0 && arith == TFFT_ARITH_DF64);
}

/* one pass over lines of len points (a power of two, or a smooth length for
 * the mixed-radix kernel) */
static int add_pass(struct topeFFT *f, tope_impl *P, int64_t len, int64_t ies, int64_t oes,
                    dimref *lines, int nl, int oop, int post_tw, int64_t tw_n)
{
    if (P->npass >= MAX_PASSES || nl > 3) return set_status(f, TOPE_ERR_UNSUPPORTED);
    tfft_pass *p = &P->pass[P->npass];
    memset(p, 0, sizeof(*p));
    const int log_l = ilog2_exact64(len);
    const int mixed = log_l < 0;
    if (mixed) {
        if (P->arith == TFFT_ARITH_TC) return set_status(f, TOPE_ERR_UNSUPPORTED);
        p->len = (int)len;
        p->nrad = mixed_radices(len, p->radix);
        if (p->nrad < 1) return set_status(f, TOPE_ERR_INVALID_SIZE);
    }
    p->log_l = mixed ? 0 : log_l;
    p->arith = P->arith;
    p->scale = 1.0;
    p->ies = ies;
    p->oes = oes;
    int lvl_tw = 0;
    for (int i = 0; i < 3; i++) {
        if (i < nl) {
            p->n[i] = lines[i].count;
            p->is[i] = lines[i].in_stride;
            p->os[i] = lines[i].out_stride;
            if (lines[i].is_twiddle) lvl_tw = i;
        } else {
            p->n[i] = 1;
        }
    }
    int strided = (ies != 1) || (oes != 1);
    /* small transforms in FP64 storage (at most 2^16 points in the pass) run
     * 4 points per thread: more threads, shorter dependent chains each */
    const int64_t lines_total = p->n[0] * p->n[1] * p->n[2];
    p->ept = (!mixed && (P->arith == TFFT_ARITH_F64 || P->arith == TFFT_ARITH_DF64) &&
              log_l >= 2 && log_l <= 7 && (lines_total << log_l) <= 65536)
                 ? 4
                 : 0;
    int b = (nl == 0) ? 1
            : mixed   ? choose_b_mixed(len, p->n[0])
                      : choose_b(log_l, p->n[0], strided, p->ept ? 4 : 16,
                                 P->arith == TFFT_ARITH_F64);
    /* few lines (small single transforms): spread them over at least 32 CTAs
     * rather than keep wide tiles */
    while (b > 1 && p->n[0] * p->n[1] * p->n[2] / b < 32) b >>= 1;
    if (P->arith == TFFT_ARITH_TC && log_l >= 4 && !mixed) {
        /* the tensor form's CTA shape is fixed per length (ragged last tile) */
        b = tfft_tc_b_tile(log_l);
        p->mma_b = P->tc_matrix;
    }
    p->b_tile = b;
    /* whole contiguous lines in a kernel shape that stages full tiles with
     * bulk asynchronous copies; a wait for them that gives up sets the plan's
     * device word, which the synchronous Exec reports */
    if (!mixed && nl > 0 && ies == 1 && p->is[0] == ((int64_t)1 << log_l) && !p->tab0 &&
        bulk_level() != 0 && tfft_pass_bulk_capable(log_l, b, P->arith, p->ept)) {
        if (!P->err_word) {
            void *w;
            int st = impl_alloc_tab(P, 16, -1, &w);
            if (st) return set_status(f, st);
            int rc = tfft_memset_async(w, 0, 16, f->command_queue);
            if (rc) return cuda_status(f, rc);
            P->err_word = (int *)w;
        }
        p->bulk = 1;
        p->err = P->err_word;
    } else if (!mixed && nl > 0 && ies != 1 && p->is[0] == 1 && !p->tab0 && tma_enabled(P->arith) &&
               tfft_pass_bulk_capable(log_l, b, P->arith, p->ept)) {
        /* adjacent strided lines: TMA boxes from a tensor map, built once
         * the plan's buffers exist (plan_tensor_maps) */
        P->tma_cand[P->npass] = 1;
    }
    if (post_tw && P->arith == TFFT_ARITH_F64 && tw_n <= FULL_TW_MAX) {
        /* FP64 butterflies: one load from the whole table W_N^m instead of
         * the product of two table entries saves 4 of the pass's ~45 FP64
         * instructions per point (the FP64 pipe bounds this path) */
        const void *full;
        const int lgn = ilog2_exact64(tw_n);
        int st = lgn >= 0 ? impl_wl_table(f, P, lgn, &full) : impl_mixed_table(f, P, tw_n, &full);
        if (st) return st;
        p->post_tw = 1;
        p->tw_level = lvl_tw;
        p->tw_shift = 0;
        p->tw_n = tw_n;
        p->tw_hi = full;
        p->tw_lo = NULL;
    } else if (post_tw) {
        /* two-level table of W_N^m: 2^shift low entries, ceil(N / 2^shift)
         * high ones */
        int lgn = 0;
        while (((int64_t)1 << lgn) < tw_n) lgn++;
        int shift = (lgn + 1) / 2;
        const int64_t nhi = (tw_n + ((int64_t)1 << shift) - 1) >> shift;
        void *hi, *lo;
        int st = impl_alloc_tab(P, tw_elem_bytes(P->arith) * (size_t)nhi, -1, &hi);
        if (!st) st = impl_alloc_tab(P, tw_elem_bytes(P->arith) << shift, -1, &lo);
        if (st) return set_status(f, st);
        int rc = tfft_fourstep_tables(hi, lo, tw_n, shift, P->arith, f->command_queue);
        if (rc) return cuda_status(f, rc);
        p->post_tw = 1;
        p->tw_level = lvl_tw;
        p->tw_shift = shift;
        p->tw_n = tw_n;
        p->tw_hi = hi;
        p->tw_lo = lo;
    }
    if (mixed ? !tfft_mixed_supported((int)len, b, P->arith)
              : !tfft_pass_supported(log_l, b, P->arith, p->ept))
        return set_status(f, TOPE_ERR_UNSUPPORTED);
    int st = mixed ? impl_mixed_table(f, P, len, &p->tw) : impl_wl_table(f, P, log_l, &p->tw);
    if (st) return st;
    P->oop[P->npass] = oop;
    P->npass++;
    return TOPE_SUCCESS;
}

/* can one pass take lines of len points? */
static int fits_one(const tope_impl *P, int64_t len)
{
    const int lg = ilog2_exact64(len);
    if (lg >= 0) return lg <= TFFT_MAX_LOG_L_ARITH(P->arith);
    return P->arith != TFFT_ARITH_TC && len <= TFFT_MIXED_MAX_POINTS && is_smooth(len);
}

/* the divisors of a smooth n (at most cap of them); returns the count */
static int smooth_divisors(int64_t n, int64_t *out, int cap)
{
    int cnt = 1;
    out[0] = 1;
    for (int i = 0; i < 6; i++) {
        const int pr = k_smooth_primes[i];
        const int base = cnt;
        int64_t pk = 1, m = n;
        while (m % pr == 0) {
            m /= pr;
            pk *= pr;
            for (int j = 0; j < base && cnt < cap; j++) out[cnt++] = out[j] * pk;
        }
    }
    return cnt;
}

static int64_t split_first(const tope_impl *P, int64_t n, int parts);

/* can lines of n points be transformed in `parts` passes? */
static int fits_parts(const tope_impl *P, int64_t n, int parts)
{
    if (parts == 1) return fits_one(P, n);
    return split_first(P, n, parts) > 1;
}

/*
 * Length of the first pass of a `parts`-pass split of n, or 0.  Powers of
 * two take 2^ceil(log2(n)/parts).  Other smooth lengths take the divisor d
 * that fits one pass, leaves n/d for the other parts - 1 passes, and has d^parts
 * closest to n.
 */
static int64_t split_first(const tope_impl *P, int64_t n, int parts)
{
    const int lg = ilog2_exact64(n);
    if (lg >= 0) {
        const int l2 = (lg + parts - 1) / parts;
        return l2 >= 1 && lg - l2 >= 1 && fits_one(P, (int64_t)1 << l2) &&
                       fits_parts(P, n >> l2, parts - 1)
                   ? (int64_t)1 << l2
                   : 0;
    }
    if (!is_smooth(n)) return 0;
    enum { CAP = 4096 };
    int64_t *dv = (int64_t *)malloc(sizeof(int64_t) * CAP);
    if (!dv) return 0;
    const int nd = smooth_divisors(n, dv, CAP);
    int64_t best = 0;
    double best_score = 0;
    for (int i = 0; i < nd; i++) {
        const int64_t d = dv[i];
        if (d < 2 || d >= n || !fits_one(P, d)) continue;
        double pw = 1.0;
        for (int k = 0; k < parts; k++) pw *= (double)d;
        const double score = pw > (double)n ? pw / (double)n : (double)n / pw;
        if (best && score >= best_score) continue;
        if (!fits_parts(P, n / d, parts - 1)) continue;
        best = d;
        best_score = score;
    }
    free(dv);
    return best;
}

/*
 * Out-of-place transform of length n in `parts` passes: element strides
 * ies (input) and oes (output), over the lines lines[0..nl) with their own
 * input and output strides.  With n = n1*n2 (n2 = split_first):
 *   pass A transforms along i2 (stride ies*n1) in place, lines i1 (stride ies)
 *          x lines, and multiplies element k2 by W_n^{i1 k2};
 *   then, for each k2 (input stride ies*n1, output stride oes), the length-n1
 *          transform along i1 (stride ies) whose element k1 goes to
 *          oes*(k1*n2 + k2): one pass into the other buffer, or again this
 *          split when n1 needs more than one pass.
 */
static int plan_split(struct topeFFT *f, tope_impl *P, int64_t n, int parts, int64_t ies,
                      int64_t oes, const dimref *lines, int nl)
{
    dimref d[5];
    int st, m;
    if (nl > 3) return set_status(f, TOPE_ERR_UNSUPPORTED);
    if (parts == 1) {
        memcpy(d, lines, sizeof(dimref) * nl);
        sort_dims(d, nl);
        m = merge_dims(d, nl);
        return add_pass(f, P, n, ies, oes, d, m, 1, 0, 0);
    }
    const int64_t n2 = split_first(P, n, parts), n1 = n2 ? n / n2 : 0;
    if (!n2) return set_status(f, TOPE_ERR_INVALID_SIZE);
    /* pass A, in place: every line keeps its input strides */
    for (int i = 0; i < nl; i++) {
        d[i] = lines[i];
        d[i].out_stride = d[i].in_stride;
    }
    d[nl].count = n1;
    d[nl].in_stride = d[nl].out_stride = ies;
    d[nl].is_twiddle = 1;
    sort_dims(d, nl + 1);
    m = merge_dims(d, nl + 1);
    st = add_pass(f, P, n2, ies * n1, ies * n1, d, m, 0, 1, n);
    if (st) return st;
    /* the length-n1 transforms of the columns k2 */
    memcpy(d, lines, sizeof(dimref) * nl);
    d[nl].count = n2;
    d[nl].in_stride = ies * n1;
    d[nl].out_stride = oes;
    d[nl].is_twiddle = 0;
    return plan_split(f, P, n1, parts - 1, ies, oes * n2, d, nl + 1);
}

/*
 * Tensor maps for the passes marked in tma_cand, one per allocated buffer
 * (a pass reads buf[cur], which alternates where the plan has out-of-place
 * passes).  The map is the pass's input array in 8-byte units: dimension 0
 * the adjacent lines (n[0] * S / 8 units), then the line's elements (L,
 * stride ies) and the other line dimensions (n[1], n[2]) in stride order;
 * the strides must nest and be multiples of 16 bytes.  A pass whose layout
 * does not fit, or a driver without the call, keeps direct loads; only an
 * allocation failure is an error.
 */
static int plan_tensor_maps(struct topeFFT *f, tope_impl *P)
{
    const int64_t u = P->es / 8; /* 8-byte units per element */
    for (int i = 0; i < P->npass; i++) {
        tfft_pass *p = &P->pass[i];
        if (!P->tma_cand[i] || p->tab1) continue;
        int64_t cnt[3] = {(int64_t)1 << p->log_l, p->n[1], p->n[2]};
        int64_t str[3] = {p->ies * P->es, p->is[1] * P->es, p->is[2] * P->es};
        int ord[3], no = 0;
        for (int k = 0; k < 3; k++)
            if (k == 0 || cnt[k] > 1) ord[no++] = k;
        for (int a = 1; a < no; a++) /* by stride */
            for (int c = a; c > 0 && str[ord[c]] < str[ord[c - 1]]; c--) {
                int tmp = ord[c];
                ord[c] = ord[c - 1];
                ord[c - 1] = tmp;
            }
        int64_t dims[4], strides[3];
        int box[4];
        dims[0] = p->n[0] * u;
        box[0] = p->b_tile * (int)u;
        int ok = 1;
        int64_t extent = dims[0] * 8;
        for (int k = 0; k < no; k++) {
            dims[k + 1] = cnt[ord[k]];
            strides[k] = str[ord[k]];
            box[k + 1] = ord[k] == 0 ? (cnt[0] < 256 ? (int)cnt[0] : 256) : 1;
            if (strides[k] < extent || strides[k] % 16) ok = 0;
            extent = strides[k] * dims[k + 1];
            p->tmap_src[k] = (signed char)ord[k];
        }
        if (!ok) continue;
        p->tmap_rank = no + 1;
        for (int k = 0; k < 2; k++) {
            if (!P->buf[k]) continue;
            void *map;
            int st = impl_alloc_tab(P, TFFT_TENSOR_MAP_BYTES, -1, &map);
            if (st) return set_status(f, st);
            if (tfft_tensor_map(map, P->buf[k], p->tmap_rank, dims, strides, box)) continue;
            P->tmap_dev[i][k] = map;
        }
        if ((P->tmap_dev[i][0] || P->tmap_dev[i][1]) && !P->err_word) {
            void *w;
            int st = impl_alloc_tab(P, 16, -1, &w);
            if (st) return set_status(f, st);
            int rc = tfft_memset_async(w, 0, 16, f->command_queue);
            if (rc) return cuda_status(f, rc);
            P->err_word = (int *)w;
        }
        p->err = P->err_word;
    }
    return TOPE_SUCCESS;
}

/* passes for one axis (0 = x, 1 = y, 2 = z) */
static int plan_axis(struct topeFFT *f, tope_impl *P, int axis)
{
    int64_t n = P->c[axis], s = P->st[axis];
    P->axis_first[axis] = P->npass;
    P->axis_count[axis] = 0;
    if (n <= 1) return TOPE_SUCCESS; /* length 1: identity */
    dimref others[4];
    int no = 0;
    for (int k = 0; k < 4; k++)
        if (k != axis && P->c[k] > 1) {
            others[no].count = P->c[k];
            others[no].in_stride = others[no].out_stride = P->st[k];
            others[no].is_twiddle = 0;
            no++;
        }
    int st;
    const int max_lg = TFFT_MAX_LOG_L_ARITH(P->arith);
    /* a lone line of 2^10..2^13 points would be one CTA on one SM (about 70
     * microseconds for 2^12 in FP64); two four-step passes spread it over
     * tens of CTAs */
    const int lone = no == 0 && n >= 1024 && P->arith != TFFT_ARITH_TC;
    int parts = 1;
    if (!fits_one(P, n) || lone) {
        const int lg = ilog2_exact64(n);
        if (lg >= 0) {
            /* four-step: two passes up to 2^(2*max_lg) points, one more per
             * further factor of 2^max_lg */
            parts = lg <= 2 * max_lg ? 2 : (lg + max_lg - 1) / max_lg;
            /* FP32 storage moves half the bytes per pass, and its 2^12-point
             * passes cost more per bit than short ones (three radix-16 stages
             * in one CTA of two strided lines): 2^24..2^26-point lines take
             * three passes of 2^8..2^9 points.  Measured at 2^24: accurate
             * 1.24 -> 1.12 ms per step, fast 0.82 -> 0.62, tensor 1.62 ->
             * 1.26; a real plan's 2^23-point line was 7% slower so, and keeps
             * two passes. */
            if (parts == 2 && lg >= 24 &&
                (P->arith == TFFT_ARITH_DF32 || P->arith == TFFT_ARITH_F32 || P->arith == TFFT_ARITH_TC))
                parts = 3;
        } else {
            parts = 2;
            while (parts <= 6 && !fits_parts(P, n, parts)) parts++;
            if (parts > 6) parts = fits_one(P, n) ? 1 : 0;
        }
    }
    if (parts == 0) return set_status(f, TOPE_ERR_INVALID_SIZE);
    if (parts == 1) {
        dimref d[4];
        memcpy(d, others, sizeof(dimref) * no);
        sort_dims(d, no);
        int m = merge_dims(d, no);
        st = add_pass(f, P, n, s, s, d, m, 0, 0, 0);
    } else {
        st = plan_split(f, P, n, parts, s, s, others, no);
    }
    if (st) return st;
    P->axis_count[axis] = P->npass - P->axis_first[axis];
    return TOPE_SUCCESS;
}

static void impl_free(tope_impl *P)
{
    if (!P) return;
    for (int i = 0; i < P->ntabs; i++) tfft_free(P->tabs[i]);
    for (int a = 0; a < 3; a++) {
        tfft_free(P->bitrev[a]);
        tfft_free(P->quarter[a]);
    }
    tfft_free(P->dft_tab);
    tfft_free(P->chirp);
    tfft_free(P->bhat);
    tfft_free(P->tc_matrix);
    tfft_free(P->spec);
    tfft_free(P->rtw_hi);
    tfft_free(P->rtw_lo);
    impl_free(P->specp);
    impl_free(P->sub);
    tfft_free(P->buf[0]);
    tfft_free(P->buf[1]);
    tfft_event_destroy(P->kev.a);
    tfft_event_destroy(P->kev.b);
    tfft_event_destroy(P->mev.a);
    tfft_event_destroy(P->mev.b);
    for (int i = 0; i < 2 * P->pev_cap; i++) tfft_event_destroy(P->pev[i]);
    free(P->pev);
    free(P->pev_pass);
    P->magic = 0;
    free(P);
}

/* next event pair of the per-launch pool (grown in chunks); NULL on failure */
static void **pev_take(tope_impl *P, int pass)
{
    if (P->pev_used == P->pev_cap) {
        int cap = P->pev_cap ? 2 * P->pev_cap : 64;
        void **ev = (void **)realloc(P->pev, sizeof(void *) * 2 * (size_t)cap);
        if (!ev) return NULL;
        P->pev = ev;
        int *pp = (int *)realloc(P->pev_pass, sizeof(int) * (size_t)cap);
        if (!pp) return NULL;
        P->pev_pass = pp;
        for (int i = 2 * P->pev_cap; i < 2 * cap; i++) {
            if (tfft_event_create(&P->pev[i])) {
                for (int j = 2 * P->pev_cap; j < i; j++) tfft_event_destroy(P->pev[j]);
                return NULL;
            }
        }
        P->pev_cap = cap;
    }
    P->pev_pass[P->pev_used] = pass;
    return &P->pev[2 * P->pev_used++];
}

/* fold recorded per-launch durations (the stream has been synchronised) */
static void pev_settle(tope_impl *P)
{
    for (int k = 0; k < P->pev_used; k++) {
        uint64_t ns = 0;
        tfft_event_elapsed_ns(P->pev[2 * k], P->pev[2 * k + 1], &ns);
        P->pass_ns[P->pev_pass[k]] += ns;
        P->pass_launches[P->pev_pass[k]]++;
    }
    P->pev_used = 0;
}

static int run_passes(struct topeFFT *f, tope_impl *P, int first, int count, int dir,
                      double scale);

/* kinds of impl_create's `real` argument */
#define IMPL_REAL 1 /* rows of a real-data plan: x complex points carry 2x reals */
#define IMPL_SPEC 2 /* the spectrum of a 2D/3D real-data plan: only y and z are
                       transformed, x (= half length + 1) is a line count */

/* Build the device state of a plan and upload d (complex elements of the
 * arithmetic's storage type; arith < 0 takes the framework's setting).
 * real: 0, IMPL_REAL or IMPL_SPEC (FP64 storage only).  Returns a status. */
static int impl_create(struct topeFFT *f, tope_impl **out, int ndim, int64_t x, int64_t y,
                       int64_t z, int64_t batch, const void *d, int arith, int real,
                       uint64_t *t_pre, uint64_t *t_mem)
{
    *out = NULL;
    if (!f) return set_status(NULL, TOPE_ERR_INVALID_ARG);
    if (!fw_of(f)) {
        int st = fw_open(f);
        if (st) return st;
    }
    if (x < 1 || y < 1 || z < 1 || batch < 1) return set_status(f, TOPE_ERR_INVALID_SIZE);
    tope_impl *P = (tope_impl *)calloc(1, sizeof(tope_impl));
    if (!P) return set_status(f, TOPE_ERR_ALLOC);
    P->magic = TOPE_MAGIC;
    P->ndim = ndim;
    P->c[0] = x;
    P->c[1] = y;
    P->c[2] = z;
    P->c[3] = batch;
    P->st[0] = 1;
    P->st[1] = x;
    P->st[2] = x * y;
    P->st[3] = x * y * z;
    P->volume = x * y * z;
    P->total = P->volume * batch;
    P->arith = arith >= 0 ? arith : f->arith;
    P->es = TFFT_ELEM_BYTES(P->arith);
    P->last_dir = FORWARD;
    int st = TOPE_SUCCESS, rc;
    void *stream = f->command_queue;
    tope_fw *w = fw_of(f);

    if ((rc = tfft_event_create(&P->kev.a)) || (rc = tfft_event_create(&P->kev.b)) ||
        (rc = tfft_event_create(&P->mev.a)) || (rc = tfft_event_create(&P->mev.b))) {
        impl_free(P);
        return cuda_status(f, rc);
    }

    int lgx = ilog2_exact64(x), lgy = ilog2_exact64(y), lgz = ilog2_exact64(z);
    const int fp64_io = P->es == 16;
    P->real = real == IMPL_REAL;
    const int spec = real == IMPL_SPEC;
    if (P->real && ndim != 1) {
        impl_free(P);
        return set_status(f, TOPE_ERR_UNSUPPORTED);
    }
    /* axes of 2^a 3^b 5^c 7^d 11^e 13^f points run as passes (the mixed-radix
     * kernel for lines that are not powers of two; not in the tensor form) */
    const int okx = lgx >= 0 || (P->arith != TFFT_ARITH_TC && is_smooth(x));
    const int oky = lgy >= 0 || (P->arith != TFFT_ARITH_TC && is_smooth(y));
    const int okz = lgz >= 0 || (P->arith != TFFT_ARITH_TC && is_smooth(z));
    if (spec) P->mode = (oky && okz) ? MODE_FFT : -1;
    else if (ndim == 1 && x == 2 && batch == 1 && fp64_io && !real) P->mode = MODE_N2;
    else if (ndim == 1 && !okx)
        P->mode = !fp64_io ? -1 : x < BLUESTEIN_MIN_N ? MODE_DFT : MODE_BLUESTEIN;
    else if (!okx || !oky || !okz) P->mode = -1;
    else P->mode = MODE_FFT;
    if (P->mode < 0) {
        impl_free(P);
        return set_status(f, TOPE_ERR_INVALID_SIZE);
    }
    if (P->mode == MODE_DFT && x > 46340 * 2) {
        impl_free(P);
        return set_status(f, TOPE_ERR_INVALID_SIZE);
    }

    size_t bytes = (size_t)P->total * P->es;
    if (tfft_malloc(&P->buf[0], bytes)) {
        impl_free(P);
        return set_status(f, TOPE_ERR_ALLOC);
    }
    tfft_event_record(w->pair.a, stream);
    tfft_event_record(P->kev.a, stream);
    if (P->mode == MODE_FFT) {
        if (P->arith == TFFT_ARITH_TC) {
            if (tfft_malloc(&P->tc_matrix, TFFT_TC_MATRIX_BYTES)) st = set_status(f, TOPE_ERR_ALLOC);
            else if ((rc = tfft_tc_matrix(P->tc_matrix, stream))) st = cuda_status(f, rc);
        }
        for (int a = spec ? 1 : 0; a < 3 && !st; a++) st = plan_axis(f, P, a);
        int need2 = 0;
        for (int i = 0; i < P->npass; i++) need2 |= P->oop[i];
        if (!st && need2 && tfft_malloc(&P->buf[1], bytes)) st = set_status(f, TOPE_ERR_ALLOC);
        if (!st) st = plan_tensor_maps(f, P);
        /* per-axis bit-reversal and quarter-wave tables of the reference's plan */
        for (int a = spec ? 1 : 0; a < ndim && !st; a++) {
            int lg = ilog2_exact64(P->c[a]);
            if (lg < 0) continue; /* the reference's tables exist for 2^k only */
            if (tfft_malloc((void **)&P->bitrev[a], sizeof(int) * (size_t)P->c[a])) {
                st = set_status(f, TOPE_ERR_ALLOC);
                break;
            }
            if ((rc = tfft_bitrev_table(P->bitrev[a], lg, stream))) st = cuda_status(f, rc);
            if (!st && P->c[a] >= 4) {
                if (tfft_malloc(&P->quarter[a], 16 * (size_t)(P->c[a] / 4)))
                    st = set_status(f, TOPE_ERR_ALLOC);
                else if ((rc = tfft_quarter_table(P->quarter[a], (int)P->c[a], stream)))
                    st = cuda_status(f, rc);
            }
        }
    } else if (P->mode == MODE_DFT) {
        if (tfft_malloc(&P->buf[1], bytes) || tfft_malloc(&P->dft_tab, 16 * (size_t)x))
            st = set_status(f, TOPE_ERR_ALLOC);
        else if ((rc = tfft_dft_table(P->dft_tab, (int)x, stream)))
            st = cuda_status(f, rc);
    } else if (P->mode == MODE_BLUESTEIN) {
        /* X[k] = c[k] sum_j (x[j] c[j]) conj(c[k-j]), c[k] = exp(-pi i k^2/N):
         * a cyclic convolution of length M >= 2N-1 through a sub-plan; the
         * kernel conj(c) is transformed once here.  M is the next power of
         * two, or the smallest 2^a 3^b 5^c 7^d when that is at most 0.6 of it
         * (mixed-radix passes run at about 0.6 of the power-of-two pass's
         * rate on GB300: 391 against about 650 GFLOP/s in FP64) */
        int64_t m = 2 * x - 1, mp = 1;
        while (mp < m) mp <<= 1;
        for (;;) {
            int64_t r = m;
            for (int i = 0; i < 4; i++)
                while (r % k_smooth_primes[i] == 0) r /= k_smooth_primes[i];
            if (r == 1) break;
            m++;
        }
        if (P->arith == TFFT_ARITH_TC || 10 * m > 6 * mp) m = mp;
        P->bl_m = m;
        uint64_t t0 = 0, t1 = 0;
        st = impl_create(f, &P->sub, 1, m, 1, 1, batch, NULL, P->arith, 0, &t0, &t1);
        if (!st) {
            f->live_plans--; /* the sub-plan lives and dies with this plan */
            if (tfft_malloc(&P->chirp, 16 * (size_t)x) || tfft_malloc(&P->bhat, 16 * (size_t)m))
                st = set_status(f, TOPE_ERR_ALLOC);
        }
        tope_impl *S = P->sub;
        if (!st && (rc = tfft_bluestein_tables(P->chirp, S->buf[S->cur], x, m, stream)))
            st = cuda_status(f, rc);
        if (!st) st = run_passes(f, S, 0, S->npass, FORWARD, 1.0);
        if (!st && (rc = tfft_d2d(P->bhat, S->buf[S->cur], 16 * (size_t)m, stream)))
            st = cuda_status(f, rc);
    } else if (P->mode == MODE_N2) {
        /* the two-point plan keeps the reference's one-bit reversal table */
        if (tfft_malloc((void **)&P->bitrev[0], 2 * sizeof(int)))
            st = set_status(f, TOPE_ERR_ALLOC);
        else if ((rc = tfft_bitrev_table(P->bitrev[0], 1, stream)))
            st = cuda_status(f, rc);
    }
    if (!st && P->real) {
        /* spectrum rows of x + 1 points; W_{2x}^k from two tables of about
         * sqrt(2x) entries each */
        int shift = 0;
        while (((int64_t)1 << (2 * shift)) < 2 * x) shift++;
        P->rtw_shift = shift;
        const size_t nhi = (size_t)(x >> shift) + 1;
        if (tfft_malloc(&P->spec, (size_t)P->es * (size_t)(x + 1) * (size_t)batch) ||
            tfft_malloc(&P->rtw_hi, 16 * nhi) || tfft_malloc(&P->rtw_lo, (size_t)16 << shift))
            st = set_status(f, TOPE_ERR_ALLOC);
        else if ((rc = tfft_real_tables(P->rtw_hi, P->rtw_lo, 2 * x, shift, P->arith, stream)))
            st = cuda_status(f, rc);
    }
    tfft_event_record(P->kev.b, stream);
    if (!st) {
        if (d) rc = tfft_h2d(P->buf[0], d, bytes, stream);
        else rc = tfft_memset_async(P->buf[0], 0, bytes, stream);
        tfft_event_record(w->pair.b, stream);
        tfft_event_record(P->mev.b, stream);
        if (!rc) rc = tfft_stream_sync(stream);
        if (rc) st = cuda_status(f, rc);
    }
    if (st) {
        tfft_stream_sync(stream);
        impl_free(P);
        return st;
    }
    uint64_t ns = 0;
    tfft_event_elapsed_ns(P->kev.a, P->kev.b, &ns);
    *t_pre += ns;
    tfft_event_elapsed_ns(P->kev.b, P->mev.b, &ns);
    *t_mem += ns;
    f->live_plans++;
    *out = P;
    return set_status(f, TOPE_SUCCESS);
}

static tope_impl *impl_of(struct topeFFT *f, void *impl)
{
    tope_impl *P = (tope_impl *)impl;
    if (!f) {
        set_status(NULL, TOPE_ERR_INVALID_ARG);
        return NULL;
    }
    if (!P || P->magic != TOPE_MAGIC) {
        set_status(f, TOPE_ERR_DESTROYED);
        return NULL;
    }
    if (!fw_of(f)) {
        set_status(f, TOPE_ERR_NOT_INITIALIZED);
        return NULL;
    }
    return P;
}

/* fold pending async kernel time into *t_kernel (caller has synchronised) */
static void settle(tope_impl *P, uint64_t *t_kernel)
{
    pev_settle(P);
    if (P->sub) pev_settle(P->sub);
    if (P->pending) {
        uint64_t ns = 0;
        tfft_event_elapsed_ns(P->kev.a, P->kev.b, &ns);
        *t_kernel += ns;
        P->pending = 0;
    }
}

/* launch arguments of pass i inside the sequence [first, last] on the
 * current buffer: conj/scale make the sequence an inverse when dir == INVERSE */
static tfft_pass pass_args(const tope_impl *P, int i, int first, int last, int dir, double scale)
{
    tfft_pass p = P->pass[i];
    p.in = P->buf[P->cur];
    p.tmap = P->tmap_dev[i][P->cur];
    p.out = P->oop[i] ? P->buf[1 - P->cur] : P->buf[P->cur];
    p.conj_in = (dir == INVERSE) && (i == first);
    p.conj_out = (dir == INVERSE) && (i == last);
    p.scale = i == last ? scale : 1.0;
    return p;
}

/* Queue passes [first, first+count) on the current buffer, but the last
 * `hold` of them, which the caller launches itself. */
static int run_passes_hold(struct topeFFT *f, tope_impl *P, int first, int count, int dir,
                           double scale, int hold)
{
    void *stream = f->command_queue;
    for (int i = first; i < first + count - hold; i++) {
        tfft_pass p = pass_args(P, i, first, first + count - 1, dir, scale);
        void **ev = f->pass_timing ? pev_take(P, i) : NULL;
        if (ev) tfft_event_record(ev[0], stream);
        int rc = tfft_launch_pass(&p, stream);
        if (ev) tfft_event_record(ev[1], stream);
        if (rc) return cuda_status(f, rc);
        if (P->oop[i]) P->cur = 1 - P->cur;
    }
    return TOPE_SUCCESS;
}

static int run_passes(struct topeFFT *f, tope_impl *P, int first, int count, int dir,
                      double scale)
{
    return run_passes_hold(f, P, first, count, dir, scale, 0);
}

/* where a real-data plan's spectrum lives: its own buffer (1D) or the
 * current buffer of its spectrum plan (2D/3D) */
static void *spec_buf(const tope_impl *P)
{
    return P->specp ? P->specp->buf[P->specp->cur] : P->spec;
}

/* queue the whole transform; events bracket the kernels.  hold = 1 (FFT
 * plans only) leaves the last pass and the closing events to the caller. */
static int impl_exec_async(struct topeFFT *f, tope_impl *P, int dir, int hold)
{
    void *stream = f->command_queue;
    int rc, st = TOPE_SUCCESS;
    if (dir != FORWARD && dir != INVERSE) return set_status(f, TOPE_ERR_INVALID_ARG);
    P->last_dir = dir;
    tope_fw *w = fw_of(f);
    tfft_event_record(P->kev.a, stream);
    tfft_event_record(w->pair.a, stream);
    const int64_t rows = P->c[3], m = P->c[0];
    if (P->real && dir == INVERSE) {
        /* 2D/3D: the inverse along y (and z) on the spectrum first */
        if (P->specp) {
            tope_impl *Q = P->specp;
            st = run_passes(f, Q, 0, Q->npass, INVERSE, 1.0 / (double)(Q->c[1] * Q->c[2]));
        }
        /* spectrum -> packed spectrum of the half-length transform */
        if (!st && (rc = tfft_c2r_pre(spec_buf(P), P->buf[P->cur], P->rtw_hi, P->rtw_lo,
                                      P->rtw_shift, m, rows, P->arith, stream)))
            st = cuda_status(f, rc);
        P->spec_cur = 0;
    }
    if (st) {
        /* nothing more to queue */
    } else if (P->mode == MODE_FFT) {
        double scale = dir == INVERSE ? 1.0 / (double)P->volume : 1.0;
        if (P->npass == 0) {
            /* all axes of length 1: identity (inverse divides by 1) */
        } else {
            st = run_passes_hold(f, P, 0, P->npass, dir, scale, hold);
        }
    } else if (P->mode == MODE_N2) {
        if ((rc = tfft_launch_n2(P->buf[P->cur], dir, stream))) st = cuda_status(f, rc);
    } else if (P->mode == MODE_DFT) {
        rc = tfft_launch_dft(P->buf[P->cur], P->buf[1 - P->cur], P->dft_tab, (int)P->c[0], dir,
                             P->c[3], stream);
        if (rc) st = cuda_status(f, rc);
        else P->cur = 1 - P->cur;
    } else if (P->mode == MODE_BLUESTEIN) {
        /* an inverse runs as conj(F(conj x))/N around the same convolution */
        tope_impl *S = P->sub;
        const int inv = dir == INVERSE;
        const int64_t n = P->c[0], m = P->bl_m, nr = P->c[3];
        if ((rc = tfft_bluestein_pre(P->buf[P->cur], P->chirp, S->buf[S->cur], n, m, inv, nr,
                                     stream)))
            st = cuda_status(f, rc);
        if (!st) st = run_passes(f, S, 0, S->npass, FORWARD, 1.0);
        if (!st && (rc = tfft_pointwise(S->buf[S->cur], P->bhat, m, nr, stream)))
            st = cuda_status(f, rc);
        if (!st) st = run_passes(f, S, 0, S->npass, INVERSE, 1.0 / (double)m);
        if (!st && (rc = tfft_bluestein_post(S->buf[S->cur], P->chirp, P->buf[P->cur], n, m, inv,
                                             inv ? 1.0 / (double)n : 1.0, nr, stream)))
            st = cuda_status(f, rc);
    }
    if (!st && P->real && dir == FORWARD) {
        if ((rc = tfft_r2c_post(P->buf[P->cur], spec_buf(P), P->rtw_hi, P->rtw_lo, P->rtw_shift,
                                m, rows, P->arith, stream)))
            st = cuda_status(f, rc);
        /* 2D/3D: then the forward along y (and z) on the spectrum */
        if (!st && P->specp) st = run_passes(f, P->specp, 0, P->specp->npass, FORWARD, 1.0);
        P->spec_cur = 1;
    }
    if (!hold) {
        tfft_event_record(P->kev.b, stream);
        tfft_event_record(w->pair.b, stream);
    }
    P->pending = 1;
    return st;
}

/* the plan's current data: its device buffer and size in bytes */
static void *cur_data(const tope_impl *P, size_t *bytes)
{
    if (P->real && P->spec_cur) {
        *bytes = (size_t)P->es * (size_t)(P->c[0] + 1) * (size_t)P->c[3];
        return spec_buf(P);
    }
    *bytes = (size_t)P->total * P->es;
    return P->buf[P->cur];
}

/* the status of a finished exec: a wait for the tensor cores that gave up
 * leaves a flag on the device */
static int tc_status(struct topeFFT *f, const tope_impl *P, void *stream)
{
    if (P->arith == TFFT_ARITH_TC) {
        int flag = 0, rc;
        if ((rc = tfft_tc_error(&flag, stream))) return cuda_status(f, rc);
        if (flag) return set_status(f, TOPE_ERR_TIMEOUT);
    }
    if (P->err_word) { /* a wait for bulk tile copies that gave up */
        int flag = 0, rc;
        if ((rc = tfft_d2h(&flag, P->err_word, sizeof(int), stream)) || (rc = tfft_stream_sync(stream)))
            return cuda_status(f, rc);
        if (flag) {
            tfft_memset_async(P->err_word, 0, sizeof(int), stream);
            tfft_stream_sync(stream);
            return set_status(f, TOPE_ERR_TIMEOUT);
        }
    }
    return set_status(f, TOPE_SUCCESS);
}

/*
 * Read-back overlapped with the last pass.  That pass runs as up to RB_SLICES
 * launches, each over a slice of its outermost line dimension, and each
 * slice's output goes to the host on the framework's copy stream while the
 * next slice computes.  A slice's output must be a dense rectangle: a
 * contiguous range when the element axis lies inside the sliced dimension,
 * else `rows` rows (one per element of the line) of `width` elements, `pitch`
 * apart.  Returns 0 when the plan does not qualify (the read-back then
 * follows the transform).
 */
#define RB_MIN_BYTES ((size_t)32 << 20) /* below this a single copy is as fast */
#define RB_MIN_ROW 2048                 /* bytes per row of a 2D slice copy */

typedef struct rb_geom {
    int dim;       /* sliced line dimension of the last pass */
    int64_t step;  /* lines of that dimension per slice */
    int64_t rows;  /* 0: contiguous slices; else rows per slice */
    int64_t pitch; /* elements between rows */
} rb_geom;

static int rb_plan(const struct topeFFT *f, const tope_impl *P, rb_geom *g)
{
    if (P->mode != MODE_FFT || P->real || P->npass < 1 || f->pass_timing) return 0;
    if ((size_t)P->total * (size_t)P->es < RB_MIN_BYTES) return 0;
    const tfft_pass *p = &P->pass[P->npass - 1];
    /* a slice must not shift a line index the pass itself uses */
    if (p->post_tw || p->tab0 || p->tab1) return 0;
    int64_t cnt[4], str[4];
    int nd = 0, dim = -1;
    for (int i = 0; i < 3; i++) {
        if (p->n[i] <= 1) continue;
        if (dim < 0 || p->os[i] > p->os[dim]) dim = i;
        cnt[nd] = p->n[i];
        str[nd++] = p->os[i];
    }
    if (dim < 0) return 0;
    cnt[nd] = (int64_t)1 << p->log_l;
    str[nd++] = p->oes;
    /* dense output: by increasing stride, each stride is the product of the
     * counts below it */
    for (int i = 1; i < nd; i++)
        for (int j = i; j > 0 && str[j] < str[j - 1]; j--) {
            int64_t t = str[j];
            str[j] = str[j - 1];
            str[j - 1] = t;
            t = cnt[j];
            cnt[j] = cnt[j - 1];
            cnt[j - 1] = t;
        }
    int64_t expect = 1;
    for (int i = 0; i < nd; i++) {
        if (str[i] != expect) return 0;
        expect *= cnt[i];
    }
    if (expect != P->total) return 0;
    const int64_t n = p->n[dim];
    int64_t step = (n + RB_SLICES - 1) / RB_SLICES;
    if (dim == 0) step = (step + p->b_tile - 1) / p->b_tile * p->b_tile;
    if (step >= n) return 0;
    g->dim = dim;
    g->step = step;
    g->rows = 0;
    g->pitch = 0;
    if (p->oes > p->os[dim]) {
        g->rows = (int64_t)1 << p->log_l;
        g->pitch = p->oes;
        if ((size_t)step * (size_t)p->os[dim] * (size_t)P->es < RB_MIN_ROW) return 0;
        if ((size_t)p->oes * (size_t)P->es >= ((size_t)1 << 31)) return 0;
    }
    return 1;
}

/* the framework's copy stream and slice events (made once) */
static int rb_open(tope_fw *w)
{
    if (w->copy) return 0;
    for (int i = 0; i < RB_SLICES; i++)
        if (!w->slice_ev[i] && tfft_event_create(&w->slice_ev[i])) return 1;
    return tfft_stream_create(&w->copy) ? 1 : 0;
}

/* launch the last pass slice by slice and copy each slice's output to d on
 * the copy stream; the caller synchronises both streams */
static int rb_run(struct topeFFT *f, tope_impl *P, const rb_geom *g, int dir, double scale,
                  char *d)
{
    tope_fw *w = fw_of(f);
    void *stream = f->command_queue;
    const int last = P->npass - 1;
    tfft_pass p = pass_args(P, last, 0, last, dir, scale);
    const int64_t n = p.n[g->dim];
    const size_t es = (size_t)P->es;
    char *src = (char *)p.out;
    int ns = 0, rc;
    for (int64_t a = 0; a < n; a += g->step, ns++) {
        tfft_pass q = p;
        q.tmap = NULL; /* the map covers the whole array, not the slice */
        q.n[g->dim] = (a + g->step <= n) ? g->step : n - a;
        q.in = (const char *)p.in + (size_t)(a * p.is[g->dim]) * es;
        q.out = (char *)p.out + (size_t)(a * p.os[g->dim]) * es;
        if ((rc = tfft_launch_pass(&q, stream))) return cuda_status(f, rc);
        if ((rc = tfft_event_record(w->slice_ev[ns], stream))) return cuda_status(f, rc);
    }
    if (P->oop[last]) P->cur = 1 - P->cur;
    tfft_event_record(P->kev.b, stream);
    tfft_event_record(w->pair.b, stream);
    ns = 0;
    for (int64_t a = 0; a < n; a += g->step, ns++) {
        const int64_t lines = (a + g->step <= n) ? g->step : n - a;
        const size_t off = (size_t)(a * p.os[g->dim]) * es;
        const size_t width = (size_t)(lines * p.os[g->dim]) * es;
        if ((rc = tfft_stream_wait(w->copy, w->slice_ev[ns]))) return cuda_status(f, rc);
        if (ns == 0) tfft_event_record(P->mev.a, w->copy);
        if (g->rows)
            rc = tfft_d2h_2d(d + off, (size_t)g->pitch * es, src + off, (size_t)g->pitch * es,
                             width, (size_t)g->rows, w->copy);
        else
            rc = tfft_d2h(d + off, src + off, width, w->copy);
        if (rc) return cuda_status(f, rc);
    }
    tfft_event_record(P->mev.b, w->copy);
    return TOPE_SUCCESS;
}

/* synchronous: exec, then read back into d (if non-NULL).  es_caller is the
 * element size the calling entry point deals in (16 FP64, 8 FP32). */
static int impl_exec(struct topeFFT *f, tope_impl *P, void *d, int es_caller, int dir,
                     uint64_t *t_kernel, uint64_t *t_mem)
{
    void *stream = f->command_queue;
    int st, rc;
    if (P->es != es_caller) return set_status(f, TOPE_ERR_INVALID_ARG);
    if (P->mode == MODE_N2) {
        /* fft1d.c:16-28 transforms the caller's buffer itself */
        if (!d) return set_status(f, TOPE_ERR_INVALID_ARG);
        if ((rc = tfft_h2d(P->buf[P->cur], d, 32, stream))) return cuda_status(f, rc);
    }
    rb_geom g;
    if (d && rb_plan(f, P, &g) && !rb_open(fw_of(f))) {
        /* the last pass in slices, each read back while the next computes */
        tope_fw *w = fw_of(f);
        st = impl_exec_async(f, P, dir, 1);
        if (!st) st = rb_run(f, P, &g, dir, dir == INVERSE ? 1.0 / (double)P->volume : 1.0,
                             (char *)d);
        rc = tfft_stream_sync(stream);
        int rc2 = tfft_stream_sync(w->copy);
        if (st) {
            P->pending = 0;
            return st;
        }
        if (rc || rc2) return cuda_status(f, rc ? rc : rc2);
        settle(P, t_kernel);
        uint64_t ns = 0;
        tfft_event_elapsed_ns(P->mev.a, P->mev.b, &ns);
        *t_mem += ns;
        return tc_status(f, P, stream);
    }
    st = impl_exec_async(f, P, dir, 0);
    if (st) {
        tfft_stream_sync(stream);
        return st;
    }
    if (d) {
        size_t nb;
        void *src = cur_data(P, &nb);
        tfft_event_record(P->mev.a, stream);
        rc = tfft_d2h(d, src, nb, stream);
        tfft_event_record(P->mev.b, stream);
        if (rc) {
            tfft_stream_sync(stream);
            return cuda_status(f, rc);
        }
    }
    if ((rc = tfft_stream_sync(stream))) return cuda_status(f, rc);
    settle(P, t_kernel);
    if (d) {
        uint64_t ns = 0;
        tfft_event_elapsed_ns(P->mev.a, P->mev.b, &ns);
        *t_mem += ns;
    }
    return tc_status(f, P, stream);
}

static int impl_axis(struct topeFFT *f, tope_impl *P, int axis, uint64_t *t_kernel)
{
    if (P->real) return set_status(f, TOPE_ERR_UNSUPPORTED); /* whole transforms only */
    if (axis >= P->ndim || P->mode != MODE_FFT) return set_status(f, TOPE_ERR_INVALID_ARG);
    void *stream = f->command_queue;
    tfft_event_record(P->kev.a, stream);
    int st = run_passes(f, P, P->axis_first[axis], P->axis_count[axis], P->last_dir, 1.0);
    tfft_event_record(P->kev.b, stream);
    int rc = tfft_stream_sync(stream);
    if (st) return st;
    if (rc) return cuda_status(f, rc);
    P->pending = 1;
    settle(P, t_kernel);
    return set_status(f, TOPE_SUCCESS);
}

static int impl_destroy(struct topeFFT *f, tope_impl *P)
{
    if (f && f->command_queue) tfft_stream_sync(f->command_queue);
    impl_free(P);
    if (f) {
        if (f->live_plans > 0) f->live_plans--;
        if (f->live_plans == 0) fw_close(f);
    }
    return set_status(f, TOPE_SUCCESS);
}

static int impl_upload(struct topeFFT *f, tope_impl *P, const void *d, int es_caller,
                       uint64_t *t_mem)
{
    if (!d || P->es != es_caller) return set_status(f, TOPE_ERR_INVALID_ARG);
    void *stream = f->command_queue;
    P->spec_cur = 0; /* a real-data plan takes its real array here */
    tfft_event_record(P->mev.a, stream);
    int rc = tfft_h2d(P->buf[P->cur], d, (size_t)P->total * P->es, stream);
    tfft_event_record(P->mev.b, stream);
    if (!rc) rc = tfft_stream_sync(stream);
    if (rc) return cuda_status(f, rc);
    uint64_t ns = 0;
    tfft_event_elapsed_ns(P->mev.a, P->mev.b, &ns);
    *t_mem += ns;
    return set_status(f, TOPE_SUCCESS);
}

static int impl_download(struct topeFFT *f, tope_impl *P, void *d, int es_caller,
                         uint64_t *t_kernel, uint64_t *t_mem)
{
    if (!d || P->es != es_caller) return set_status(f, TOPE_ERR_INVALID_ARG);
    void *stream = f->command_queue;
    size_t nb;
    void *src = cur_data(P, &nb);
    tfft_event_record(P->mev.a, stream);
    int rc = tfft_d2h(d, src, nb, stream);
    tfft_event_record(P->mev.b, stream);
    if (!rc) rc = tfft_stream_sync(stream);
    if (rc) return cuda_status(f, rc);
    settle(P, t_kernel);
    uint64_t ns = 0;
    tfft_event_elapsed_ns(P->mev.a, P->mev.b, &ns);
    *t_mem += ns;
    return set_status(f, TOPE_SUCCESS);
}

/* ------------------------------------------------------------------------ */
/* public: 1D                                                               */
/* ------------------------------------------------------------------------ */
static void sync_fields_1d(struct topePlan1D *t, tope_impl *P)
{
    t->data = P->buf[P->cur];
    t->scratch = P->buf[1 - P->cur];
}

static void plan1d(struct topeFFT *f, struct topePlan1D *t, int x, int batch, int type,
                   const void *d, int arith)
{
    if (!t) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    memset(t, 0, sizeof(*t));
    t->x = x;
    t->type = type;
    t->dim = 1;
    /* R2C (topefft.h defines it; the reference implements only C2C): x real
     * points per row in, x/2 + 1 complex points per row out */
    const int real = type == R2C;
    if (type != C2C && !real) {
        set_status(f, TOPE_ERR_UNSUPPORTED);
        return;
    }
    if (real && (x < 2 || x % 2)) {
        set_status(f, TOPE_ERR_INVALID_SIZE);
        return;
    }
    int lg = ilog2_exact64(x);
    t->radix = lg >= 0 ? ref_radix(lg) : -1;
    t->log = lg >= 0 ? ref_stages(lg) : 0;
    tope_impl *P;
    if (impl_create(f, &P, 1, real ? x / 2 : x, 1, 1, batch, d, arith, real, &t->totalPreKernel,
                    &t->totalMemory))
        return;
    t->impl = P;
    t->dataSize = (size_t)P->total * P->es;
    t->bitrev = P->bitrev[0];
    t->twiddle = P->mode == MODE_DFT         ? P->dft_tab
                 : P->mode == MODE_BLUESTEIN ? P->chirp
                                             : P->quarter[0];
    sync_fields_1d(t, P);
}

void tope1DPlanInit(struct topeFFT *f, struct topePlan1D *t, int x, int type, double *d)
{
    plan1d(f, t, x, 1, type, d, -1);
}

void tope1DBatchPlanInit(struct topeFFT *f, struct topePlan1D *t, int x, int batch, int type,
                         double *d)
{
    plan1d(f, t, x, batch, type, d, -1);
}

void tope1DBatchPlanInitF32(struct topeFFT *f, struct topePlan1D *t, int x, int batch, int type,
                            float *d)
{
    plan1d(f, t, x, batch, type, d, split_arith(f));
}

void tope1DExecF32(struct topeFFT *f, struct topePlan1D *t, float *d, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_exec(f, P, d, 8, dir, &t->totalKernel, &t->totalMemory);
    sync_fields_1d(t, P);
}

void tope1DExec(struct topeFFT *f, struct topePlan1D *t, double *d, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_exec(f, P, d, 16, dir, &t->totalKernel, &t->totalMemory);
    sync_fields_1d(t, P);
}

void tope1DExecDevice(struct topeFFT *f, struct topePlan1D *t, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    if (impl_exec_async(f, P, dir, 0) == TOPE_SUCCESS) set_status(f, TOPE_SUCCESS);
    sync_fields_1d(t, P);
}

void tope1DUpload(struct topeFFT *f, struct topePlan1D *t, const double *d)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_upload(f, P, d, 16, &t->totalMemory);
}

void tope1DDownload(struct topeFFT *f, struct topePlan1D *t, double *d)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_download(f, P, d, 16, &t->totalKernel, &t->totalMemory);
}

/* es_caller: the element size of the calling entry point (16 FP64, 8 FP32) */
static void impl_upload_spectrum(struct topeFFT *f, tope_impl *P, const void *spec, int es_caller,
                                 uint64_t *t_mem)
{
    if (!P->real || !spec || P->es != es_caller) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    void *stream = f->command_queue;
    tfft_event_record(P->mev.a, stream);
    int rc = tfft_h2d(spec_buf(P), spec,
                      (size_t)P->es * (size_t)(P->c[0] + 1) * (size_t)P->c[3], stream);
    tfft_event_record(P->mev.b, stream);
    if (!rc) rc = tfft_stream_sync(stream);
    if (rc) {
        cuda_status(f, rc);
        return;
    }
    P->spec_cur = 1;
    uint64_t ns = 0;
    tfft_event_elapsed_ns(P->mev.a, P->mev.b, &ns);
    *t_mem += ns;
    set_status(f, TOPE_SUCCESS);
}

void tope1DUploadSpectrum(struct topeFFT *f, struct topePlan1D *t, const double *spec)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_upload_spectrum(f, P, spec, 16, &t->totalMemory);
}

void tope2DUploadSpectrum(struct topeFFT *f, struct topePlan2D *t, const double *spec)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_upload_spectrum(f, P, spec, 16, &t->totalMemory);
}

void tope3DUploadSpectrum(struct topeFFT *f, struct topePlan3D *t, const double *spec)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_upload_spectrum(f, P, spec, 16, &t->totalMemory);
}

void tope1DDestroy(struct topeFFT *f, struct topePlan1D *t)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_destroy(f, P);
    t->impl = NULL;
    t->data = t->scratch = t->bitrev = t->twiddle = NULL;
}

/* ------------------------------------------------------------------------ */
/* public: 2D                                                               */
/* ------------------------------------------------------------------------ */
/* A 2D/3D real-data plan of x * y * z reals (x even; x/2, y and z products
 * of 2, 3, 5, 7, 11, 13):
 * the rows along x as a batched 1D real-data plan of y*z rows, whose
 * spectrum (x/2 + 1 points per row) is the buffer of a second plan that
 * transforms along y and z only. */
static int real_nd_create(struct topeFFT *f, tope_impl **out, int ndim, int64_t x, int64_t y,
                          int64_t z, const void *d, int arith, uint64_t *t_pre, uint64_t *t_mem)
{
    *out = NULL;
    if (x < 2 || x % 2 || !is_smooth(x / 2) || !is_smooth(y) || !is_smooth(z))
        return set_status(f, TOPE_ERR_INVALID_SIZE);
    tope_impl *P, *Q;
    int st = impl_create(f, &P, 1, x / 2, 1, 1, y * z, d, arith, IMPL_REAL, t_pre, t_mem);
    if (st) return st;
    st = impl_create(f, &Q, ndim, x / 2 + 1, y, z, 1, NULL, P->arith, IMPL_SPEC, t_pre, t_mem);
    if (st) {
        impl_destroy(f, P);
        return set_status(f, st);
    }
    f->live_plans--; /* the spectrum plan lives and dies with P */
    P->specp = Q;
    tfft_free(P->spec); /* the spectrum lives in Q's buffer */
    P->spec = NULL;
    *out = P;
    return set_status(f, TOPE_SUCCESS);
}

static void plan2d(struct topeFFT *f, struct topePlan2D *t, int x, int y, int type,
                   const void *d, int arith)
{
    if (!t) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    memset(t, 0, sizeof(*t));
    t->x = x;
    t->y = y;
    t->type = type;
    t->dim = 2;
    if (type == R2C) {
        tope_impl *P;
        if (real_nd_create(f, &P, 2, x, y, 1, d, arith, &t->totalPreKernel, &t->totalMemory))
            return;
        t->impl = P;
        t->dataSize = (size_t)(P->es / 2) * (size_t)x * (size_t)y;
        t->data = P->buf[P->cur];
        return;
    }
    if (type != C2C) {
        set_status(f, TOPE_ERR_UNSUPPORTED);
        return;
    }
    /* sides of 2^a 3^b 5^c 7^d 11^e 13^f points (the reference exits on any
     * side that is not a power of two, fft2d.c:355-362) */
    if (!is_smooth(x) || !is_smooth(y)) {
        set_status(f, TOPE_ERR_INVALID_SIZE);
        return;
    }
    int lx = ilog2_exact64(x), ly = ilog2_exact64(y);
    t->radX = lx >= 0 ? ref_radix(lx) : -1;
    t->radY = ly >= 0 ? ref_radix(ly) : -1;
    t->logX = lx >= 0 ? ref_stages(lx) : 0;
    t->logY = ly >= 0 ? ref_stages(ly) : 0;
    tope_impl *P;
    if (impl_create(f, &P, 2, x, y, 1, 1, d, arith, 0, &t->totalPreKernel, &t->totalMemory))
        return;
    t->impl = P;
    t->dataSize = (size_t)P->total * P->es;
    t->bitX = P->bitrev[0];
    t->bitY = P->bitrev[1];
    t->twdX = P->quarter[0];
    t->twdY = P->quarter[1];
    t->data = P->buf[P->cur];
}

void tope2DPlanInit(struct topeFFT *f, struct topePlan2D *t, int x, int y, int type, double *d)
{
    plan2d(f, t, x, y, type, d, -1);
}

void tope2DPlanInitF32(struct topeFFT *f, struct topePlan2D *t, int x, int y, int type, float *d)
{
    plan2d(f, t, x, y, type, d, split_arith(f));
}

void tope2DExecF32(struct topeFFT *f, struct topePlan2D *t, float *d, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_exec(f, P, d, 8, dir, &t->totalKernel, &t->totalMemory);
    t->data = P->buf[P->cur];
}

void tope2DExec(struct topeFFT *f, struct topePlan2D *t, double *d, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_exec(f, P, d, 16, dir, &t->totalKernel, &t->totalMemory);
    t->data = P->buf[P->cur];
}

void tope2DExecDevice(struct topeFFT *f, struct topePlan2D *t, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    if (impl_exec_async(f, P, dir, 0) == TOPE_SUCCESS) set_status(f, TOPE_SUCCESS);
    t->data = P->buf[P->cur];
}

void tope2DExecX(struct topeFFT *f, struct topePlan2D *t)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_axis(f, P, 0, &t->totalKernel);
    t->data = P->buf[P->cur];
}

void tope2DExecY(struct topeFFT *f, struct topePlan2D *t)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_axis(f, P, 1, &t->totalKernel);
    t->data = P->buf[P->cur];
}

void tope2DUpload(struct topeFFT *f, struct topePlan2D *t, const double *d)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_upload(f, P, d, 16, &t->totalMemory);
}

void tope2DDownload(struct topeFFT *f, struct topePlan2D *t, double *d)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_download(f, P, d, 16, &t->totalKernel, &t->totalMemory);
}

void tope2DDestroy(struct topeFFT *f, struct topePlan2D *t)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_destroy(f, P);
    t->impl = NULL;
    t->data = t->bitX = t->bitY = t->twdX = t->twdY = NULL;
}

/* ------------------------------------------------------------------------ */
/* public: 3D                                                               */
/* ------------------------------------------------------------------------ */
static void plan3d(struct topeFFT *f, struct topePlan3D *t, int x, int y, int z, int type,
                   const void *d, int arith)
{
    if (!t) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    memset(t, 0, sizeof(*t));
    t->x = x;
    t->y = y;
    t->z = z;
    t->type = type;
    t->dim = 3;
    if (type == R2C) {
        tope_impl *P;
        if (real_nd_create(f, &P, 3, x, y, z, d, arith, &t->totalPreKernel, &t->totalMemory))
            return;
        t->impl = P;
        t->dataSize = (size_t)(P->es / 2) * (size_t)x * (size_t)y * (size_t)z;
        t->data = P->buf[P->cur];
        return;
    }
    if (type != C2C) {
        set_status(f, TOPE_ERR_UNSUPPORTED);
        return;
    }
    /* smooth sides as in 2D (fft3d.c:522-533 exits on other than 2^k) */
    if (!is_smooth(x) || !is_smooth(y) || !is_smooth(z)) {
        set_status(f, TOPE_ERR_INVALID_SIZE);
        return;
    }
    int lx = ilog2_exact64(x), ly = ilog2_exact64(y), lz = ilog2_exact64(z);
    t->radX = lx >= 0 ? ref_radix(lx) : -1;
    t->radY = ly >= 0 ? ref_radix(ly) : -1;
    t->radZ = lz >= 0 ? ref_radix(lz) : -1;
    t->logX = lx >= 0 ? ref_stages(lx) : 0;
    t->logY = ly >= 0 ? ref_stages(ly) : 0;
    t->logZ = lz >= 0 ? ref_stages(lz) : 0;
    tope_impl *P;
    if (impl_create(f, &P, 3, x, y, z, 1, d, arith, 0, &t->totalPreKernel, &t->totalMemory))
        return;
    t->impl = P;
    t->dataSize = (size_t)P->total * P->es;
    t->bitX = P->bitrev[0];
    t->bitY = P->bitrev[1];
    t->bitZ = P->bitrev[2];
    t->twdX = P->quarter[0];
    t->twdY = P->quarter[1];
    t->twdZ = P->quarter[2];
    t->data = P->buf[P->cur];
}

void tope3DPlanInit(struct topeFFT *f, struct topePlan3D *t, int x, int y, int z, int type,
                    double *d)
{
    plan3d(f, t, x, y, z, type, d, -1);
}

void tope3DPlanInitF32(struct topeFFT *f, struct topePlan3D *t, int x, int y, int z, int type,
                       float *d)
{
    plan3d(f, t, x, y, z, type, d, split_arith(f));
}

void tope3DExecF32(struct topeFFT *f, struct topePlan3D *t, float *d, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_exec(f, P, d, 8, dir, &t->totalKernel, &t->totalMemory);
    t->data = P->buf[P->cur];
}

void topeUploadF32(struct topeFFT *f, void *impl, const float *d)
{
    tope_impl *P = impl_of(f, impl);
    uint64_t ns = 0;
    if (P) impl_upload(f, P, d, 8, &ns);
}

void topeUploadSpectrumF32(struct topeFFT *f, void *impl, const float *spec)
{
    tope_impl *P = impl_of(f, impl);
    uint64_t ns = 0;
    if (P) impl_upload_spectrum(f, P, spec, 8, &ns);
}

void topeDownloadF32(struct topeFFT *f, void *impl, float *d)
{
    tope_impl *P = impl_of(f, impl);
    uint64_t k = 0, m = 0;
    if (P) impl_download(f, P, d, 8, &k, &m);
}

void tope3DExec(struct topeFFT *f, struct topePlan3D *t, double *d, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_exec(f, P, d, 16, dir, &t->totalKernel, &t->totalMemory);
    t->data = P->buf[P->cur];
}

void tope3DExecDevice(struct topeFFT *f, struct topePlan3D *t, int dir)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    if (impl_exec_async(f, P, dir, 0) == TOPE_SUCCESS) set_status(f, TOPE_SUCCESS);
    t->data = P->buf[P->cur];
}

void tope3DExecX(struct topeFFT *f, struct topePlan3D *t)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_axis(f, P, 0, &t->totalKernel);
    t->data = P->buf[P->cur];
}

void tope3DExecY(struct topeFFT *f, struct topePlan3D *t)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_axis(f, P, 1, &t->totalKernel);
    t->data = P->buf[P->cur];
}

void tope3DExecZ(struct topeFFT *f, struct topePlan3D *t)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_axis(f, P, 2, &t->totalKernel);
    t->data = P->buf[P->cur];
}

void tope3DUpload(struct topeFFT *f, struct topePlan3D *t, const double *d)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_upload(f, P, d, 16, &t->totalMemory);
}

void tope3DDownload(struct topeFFT *f, struct topePlan3D *t, double *d)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (P) impl_download(f, P, d, 16, &t->totalKernel, &t->totalMemory);
}

void tope3DBitrevPermute(struct topeFFT *f, struct topePlan3D *t, int axis)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    if (axis < 0 || axis > 2 || P->mode != MODE_FFT || P->c[axis] < 2) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    if (!P->bitrev[axis]) { /* a bit reversal needs a power-of-two axis */
        set_status(f, TOPE_ERR_INVALID_SIZE);
        return;
    }
    /* lines: the two other axes; g0 the one with the smaller stride */
    int o[2], k = 0;
    for (int a = 0; a < 3; a++)
        if (a != axis) o[k++] = a;
    int rc = tfft_launch_bitrev_permute(P->buf[P->cur], P->bitrev[axis],
                                        ilog2_exact64(P->c[axis]), P->st[axis], P->c[o[0]],
                                        P->st[o[0]], P->c[o[1]], P->st[o[1]], f->command_queue);
    if (!rc) rc = tfft_stream_sync(f->command_queue);
    if (rc) cuda_status(f, rc);
    else set_status(f, TOPE_SUCCESS);
}

void tope3DDestroy(struct topeFFT *f, struct topePlan3D *t)
{
    tope_impl *P = t ? impl_of(f, t->impl) : NULL;
    if (!P) return;
    impl_destroy(f, P);
    t->impl = NULL;
    t->data = t->bitX = t->bitY = t->bitZ = t->twdX = t->twdY = t->twdZ = NULL;
}

/* ------------------------------------------------------------------------ */
/* misc                                                                     */
/* ------------------------------------------------------------------------ */
void topeSync(struct topeFFT *f)
{
    if (!fw_of(f)) {
        set_status(f, TOPE_ERR_NOT_INITIALIZED);
        return;
    }
    int rc = tfft_stream_sync(f->command_queue);
    if (rc) cuda_status(f, rc);
    else set_status(f, TOPE_SUCCESS);
}

void topeCopyToHost(struct topeFFT *f, void *dst, const void *src, size_t bytes)
{
    if (!fw_of(f) || !dst || !src) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    int rc = tfft_d2h(dst, src, bytes, f->command_queue);
    if (!rc) rc = tfft_stream_sync(f->command_queue);
    if (rc) cuda_status(f, rc);
    else set_status(f, TOPE_SUCCESS);
}

void topeSetPassTiming(struct topeFFT *f, int enable)
{
    if (!f) {
        set_status(NULL, TOPE_ERR_INVALID_ARG);
        return;
    }
    f->pass_timing = enable ? 1 : 0;
    set_status(f, TOPE_SUCCESS);
}

/* the plan whose passes carry the work: a Bluestein plan's power-of-two
 * sub-plan, otherwise the plan itself */
static tope_impl *passes_of(tope_impl *P)
{
    return (P && P->mode == MODE_BLUESTEIN && P->sub) ? P->sub : P;
}

/* The plans whose passes a plan's pass list shows, in execution order: the
 * plan (or its Bluestein sub-plan), then, for a 2D/3D real-data plan, the
 * spectrum plan's y/z passes.  Returns how many (0 for no plan). */
static int pass_plans(tope_impl *P, tope_impl *out[2])
{
    if (!P) return 0;
    out[0] = passes_of(P);
    out[1] = P->specp;
    return out[1] ? 2 : 1;
}

int topePassTimes(struct topeFFT *f, void *impl, uint64_t *ns, uint64_t *launches, int max)
{
    tope_impl *Q[2];
    const int nq = pass_plans(impl_of(f, impl), Q);
    if (!nq) return -1;
    int rc = tfft_stream_sync(f->command_queue);
    if (rc) {
        cuda_status(f, rc);
        return -1;
    }
    int k = 0;
    for (int q = 0; q < nq; q++) {
        pev_settle(Q[q]);
        for (int i = 0; i < Q[q]->npass; i++, k++)
            if (k < max) {
                if (ns) ns[k] = Q[q]->pass_ns[i];
                if (launches) launches[k] = Q[q]->pass_launches[i];
            }
    }
    set_status(f, TOPE_SUCCESS);
    return k;
}

void topeResetPassTimes(struct topeFFT *f, void *impl)
{
    tope_impl *Q[2];
    const int nq = pass_plans(impl_of(f, impl), Q);
    if (!nq) return;
    tfft_stream_sync(f->command_queue);
    for (int q = 0; q < nq; q++) {
        Q[q]->pev_used = 0;
        memset(Q[q]->pass_ns, 0, sizeof(Q[q]->pass_ns));
        memset(Q[q]->pass_launches, 0, sizeof(Q[q]->pass_launches));
    }
    set_status(f, TOPE_SUCCESS);
}

int topePassInfo(struct topeFFT *f, void *impl, int i, int64_t info[6])
{
    tope_impl *Q[2];
    const int nq = pass_plans(impl_of(f, impl), Q);
    if (!nq || !info) return -1;
    tope_impl *P = Q[0];
    if (nq == 2 && i >= Q[0]->npass) {
        i -= Q[0]->npass;
        P = Q[1];
    }
    if (i < 0 || i >= P->npass) {
        set_status(f, TOPE_ERR_INVALID_ARG);
        return -1;
    }
    const tfft_pass *p = &P->pass[i];
    int64_t L = (int64_t)1 << p->log_l;
    int64_t e = L < (p->ept ? p->ept : 16) ? L : (p->ept ? p->ept : 16);
    info[0] = p->len ? -(int64_t)p->len : p->log_l;
    info[1] = p->b_tile;
    info[2] = ((p->n[0] + p->b_tile - 1) / p->b_tile) * p->n[1] * p->n[2];
    info[3] = p->len ? 256 : (L / e) * p->b_tile;
    info[4] = P->oop[i];
    info[5] = p->post_tw;
    set_status(f, TOPE_SUCCESS);
    return 0;
}

void *topeHostAlloc(size_t bytes)
{
    void *p = NULL;
    if (tfft_host_alloc(&p, bytes)) {
        set_status(NULL, TOPE_ERR_ALLOC);
        return NULL;
    }
    return p;
}

void topeHostFree(void *p) { tfft_host_free(p); }

/* ------------------------------------------------------------------------ */
/* helpers shared with batch.c (hidden: not part of the ABI)                */
/* ------------------------------------------------------------------------ */
TOPE_INTERNAL int tope_status(struct topeFFT *f, int st) { return set_status(f, st); }
TOPE_INTERNAL int tope_cuda_status(struct topeFFT *f, int rc) { return cuda_status(f, rc); }
TOPE_INTERNAL int tope_framework_ready(struct topeFFT *f)
{
    if (!f) return set_status(NULL, TOPE_ERR_INVALID_ARG);
    return fw_of(f) ? TOPE_SUCCESS : fw_open(f);
}
TOPE_INTERNAL void tope_framework_plan_added(struct topeFFT *f) { f->live_plans++; }
TOPE_INTERNAL void tope_framework_plan_removed(struct topeFFT *f)
{
    if (f->live_plans > 0) f->live_plans--;
    if (f->live_plans == 0) fw_close(f);
}
