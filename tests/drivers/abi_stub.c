/*
 * Host-only stand-in for the CUDA side of the library's internal ABI
 * (tope-fft_gb300/csrc/tfft_abi.h), for CPU tests of the host planner:
 * linked with topefft.c and batch.c it lets plans be built and their pass
 * structure read back (topePassInfo) without a GPU.  Device pointers are
 * opaque tokens that are never dereferenced, every copy and launch is a
 * no-op that succeeds, and the shape checks mirror the kernels' launch
 * tables (fft_dispatch.cu, fft_inst_mixed.cu, fft_inst_tc.cu).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../../tope-fft_gb300/csrc/tfft_abi.h"
#include "../../include/topefft_ext.h"

static uintptr_t g_next = 0x100000;

/* call log for the tests: kind 1 = pass launch {n0, n1, n2, in, out, len or
 * -log2 L, flags: 1 conj_in, 2 conj_out, 4 scaled, 8 tensor map, 16 bulk
 * copies}, kind 2 = device-to-host copy {dst, src, bytes}, kind 3 = 2D
 * device-to-host copy {dst, src, width, height, pitch}, kind 4 = tensor map
 * {rank, dims[0..3], box[0], box[1]} followed by kind 5 {strides[0..2],
 * box[2], box[3], base} */
#define LOG_MAX 4096
static int64_t g_log[LOG_MAX][8];
static int g_nlog = 0;

static void log_rec(int64_t kind, int64_t a, int64_t b, int64_t c, int64_t d, int64_t e,
                    int64_t f, int64_t g)
{
    if (g_nlog >= LOG_MAX) return;
    int64_t *r = g_log[g_nlog++];
    r[0] = kind;
    r[1] = a;
    r[2] = b;
    r[3] = c;
    r[4] = d;
    r[5] = e;
    r[6] = f;
    r[7] = g;
}

void stub_log_clear(void) { g_nlog = 0; }
int stub_log_count(void) { return g_nlog; }
void stub_log_get(int i, int64_t *rec)
{
    for (int k = 0; k < 8; k++) rec[k] = (i >= 0 && i < g_nlog) ? g_log[i][k] : 0;
}

static void *token(void)
{
    g_next += 0x1000;
    return (void *)g_next;
}

int tfft_set_device(int dev) { return dev == 0 ? 0 : 101; }
int tfft_get_device(int *dev) { *dev = 0; return 0; }
int tfft_device_count(int *n) { *n = 1; return 0; }
int tfft_malloc(void **p, size_t bytes) { (void)bytes; *p = token(); return 0; }
int tfft_free(void *p) { (void)p; return 0; }
int tfft_host_alloc(void **p, size_t bytes) { *p = malloc(bytes ? bytes : 16); return *p ? 0 : 2; }
int tfft_host_free(void *p) { free(p); return 0; }
int tfft_memset_async(void *p, int v, size_t b, void *s) { (void)p; (void)v; (void)b; (void)s; return 0; }
int tfft_h2d(void *d, const void *s, size_t b, void *st) { (void)d; (void)s; (void)b; (void)st; return 0; }
int tfft_d2h(void *d, const void *s, size_t b, void *st)
{
    (void)st;
    /* small reads are status words (the batch kernel's flags): zeros */
    if (b <= 64) memset(d, 0, b);
    log_rec(2, (int64_t)(uintptr_t)d, (int64_t)(uintptr_t)s, (int64_t)b, 0, 0, 0, 0);
    return 0;
}
int tfft_d2h_2d(void *d, size_t dp, const void *s, size_t sp, size_t w, size_t h, void *st)
{
    (void)st;
    log_rec(3, (int64_t)(uintptr_t)d, (int64_t)(uintptr_t)s, (int64_t)w, (int64_t)h,
            (int64_t)dp, (int64_t)sp, 0);
    return 0;
}
int tfft_d2d(void *d, const void *s, size_t b, void *st) { (void)d; (void)s; (void)b; (void)st; return 0; }
int tfft_stream_create(void **s) { *s = token(); return 0; }
int tfft_stream_destroy(void *s) { (void)s; return 0; }
int tfft_stream_sync(void *s) { (void)s; return 0; }
int tfft_stream_wait(void *s, void *e) { (void)s; (void)e; return 0; }
int tfft_event_create(void **e) { *e = token(); return 0; }
int tfft_event_destroy(void *e) { (void)e; return 0; }
int tfft_event_record(void *e, void *s) { (void)e; (void)s; return 0; }
int tfft_event_elapsed_ns(void *a, void *b, uint64_t *ns) { (void)a; (void)b; *ns = 0; return 0; }
int tfft_last_launch_error(void) { return 0; }
const char *tfft_error_string(int code) { (void)code; return "host stub"; }

int tfft_twiddle_table(void *t, int l, int a, void *s) { (void)t; (void)l; (void)a; (void)s; return 0; }
int tfft_fourstep_tables(void *h, void *l, int64_t n, int sh, int a, void *s)
{
    (void)h; (void)l; (void)n; (void)sh; (void)a; (void)s;
    return 0;
}
int tfft_bitrev_table(int *r, int l, void *s) { (void)r; (void)l; (void)s; return 0; }
int tfft_quarter_table(void *t, int n, void *s) { (void)t; (void)n; (void)s; return 0; }
int tfft_dft_table(void *t, int n, void *s) { (void)t; (void)n; (void)s; return 0; }
int tfft_table_any(void *t, int n, int a, void *s) { (void)t; (void)n; (void)a; (void)s; return 0; }

int tfft_tc_matrix(void *d, void *s) { (void)d; (void)s; return 0; }
int tfft_tc_b_tile(int log_l)
{
    if (log_l < 4 || log_l > 13) return 0;
    return log_l > 12 ? 1 : 1 << (12 - log_l);
}
int tfft_tc_error(int *flag, void *s) { (void)s; *flag = 0; return 0; }

int tfft_launch_pass(const tfft_pass *p, void *s)
{
    (void)s;
    log_rec(1, p->n[0], p->n[1], p->n[2], (int64_t)(uintptr_t)p->in, (int64_t)(uintptr_t)p->out,
            p->len ? p->len : -(int64_t)p->log_l,
            (p->conj_in ? 1 : 0) | (p->conj_out ? 2 : 0) | (p->scale != 1.0 ? 4 : 0) |
                (p->tmap ? 8 : 0) | (p->bulk ? 16 : 0));
    return 0;
}

static int log2_exact(int v)
{
    int l = 0;
    while ((1 << l) < v) l++;
    return (1 << l) == v ? l : -1;
}

int tfft_pass_supported(int log_l, int b_tile, int arith, int ept)
{
    const int lb = log2_exact(b_tile);
    if (lb < 0 || log_l < 0) return 0;
    if (ept == 4)
        return (arith == TFFT_ARITH_F64 || arith == TFFT_ARITH_DF64) && log_l >= 2 &&
               log_l <= 7 && log_l + lb <= 12;
    if (ept != 0 && ept != 16) return 0;
    if (arith == TFFT_ARITH_TC && log_l >= 4) return log_l <= 13 && b_tile == tfft_tc_b_tile(log_l);
    if (log_l > TFFT_MAX_LOG_L_ARITH(arith) || lb > 5) return 0;
    return (log_l + lb) <= (arith == TFFT_ARITH_F32 ? 14 : 13);
}

/* Staged tiles: off by default (no stand-in kernel stages tiles, and every
 * tensor map fails, so the plans load directly); stub_set_staging(1) answers
 * as the real library does (fft_dispatch.cu, fft_tma.cu), logging each map */
static int g_staging = 0;
void stub_set_staging(int on) { g_staging = on; }

int tfft_pass_bulk_capable(int log_l, int b_tile, int arith, int ept)
{
    if (!g_staging) return 0;
    if (arith == TFFT_ARITH_TC || (ept != 0 && ept != 16)) return 0;
    if (b_tile < 8 || log_l < 5 || ((int64_t)TFFT_ELEM_BYTES(arith) << log_l) < 512) return 0;
    return tfft_pass_supported(log_l, b_tile, arith, ept);
}

int tfft_tensor_map(void *dev_map, const void *base, int rank, const int64_t *dims,
                    const int64_t *strides, const int *box)
{
    (void)dev_map;
    if (!g_staging) return 1;
    if (rank < 2 || rank > 4) return 1;
    int64_t d[4] = {0, 0, 0, 0}, st[3] = {0, 0, 0}, bx[4] = {0, 0, 0, 0};
    for (int k = 0; k < rank; k++) {
        d[k] = dims[k];
        bx[k] = box[k];
        if (k > 0) st[k - 1] = strides[k - 1];
    }
    log_rec(4, rank, d[0], d[1], d[2], d[3], bx[0], bx[1]);
    log_rec(5, st[0], st[1], st[2], bx[2], bx[3], (int64_t)(uintptr_t)base, 0);
    return 0;
}

int tfft_mixed_supported(int len, int b_tile, int arith)
{
    int m = len;
    static const int pr[] = {2, 3, 5, 7, 11, 13};
    for (int i = 0; i < 6; i++)
        while (m > 1 && m % pr[i] == 0) m /= pr[i];
    if (len < 2 || m != 1 || log2_exact(b_tile) < 0 || b_tile > 256) return 0;
    if ((int64_t)len * b_tile > TFFT_MIXED_MAX_POINTS) return 0;
    return arith != TFFT_ARITH_TC;
}

int tfft_launch_dft(const void *i, void *o, const void *t, int n, int d, int64_t r, void *s)
{
    (void)i; (void)o; (void)t; (void)n; (void)d; (void)r; (void)s;
    return 0;
}
int tfft_launch_bitrev_permute(void *d, const int *r, int l, int64_t es, int64_t n0, int64_t s0,
                               int64_t n1, int64_t s1, void *s)
{
    (void)d; (void)r; (void)l; (void)es; (void)n0; (void)s0; (void)n1; (void)s1; (void)s;
    return 0;
}
int tfft_launch_n2(void *d, int dir, void *s) { (void)d; (void)dir; (void)s; return 0; }
int tfft_bluestein_tables(void *c, void *b, int64_t n, int64_t m, void *s)
{
    (void)c; (void)b; (void)n; (void)m; (void)s;
    return 0;
}
int tfft_bluestein_pre(const void *x, const void *c, void *w, int64_t n, int64_t m, int ci,
                       int64_t r, void *s)
{
    (void)x; (void)c; (void)w; (void)n; (void)m; (void)ci; (void)r; (void)s;
    return 0;
}
int tfft_pointwise(void *w, const void *h, int64_t m, int64_t r, void *s)
{
    (void)w; (void)h; (void)m; (void)r; (void)s;
    return 0;
}
int tfft_bluestein_post(const void *w, const void *c, void *x, int64_t n, int64_t m, int co,
                        double sc, int64_t r, void *s)
{
    (void)w; (void)c; (void)x; (void)n; (void)m; (void)co; (void)sc; (void)r; (void)s;
    return 0;
}
int tfft_real_tables(void *h, void *l, int64_t n, int sh, int a, void *s)
{
    (void)h; (void)l; (void)n; (void)sh; (void)a; (void)s;
    return 0;
}
int tfft_r2c_post(const void *z, void *x, const void *h, const void *l, int sh, int64_t m,
                  int64_t r, int a, void *s)
{
    (void)z; (void)x; (void)h; (void)l; (void)sh; (void)m; (void)r; (void)a; (void)s;
    return 0;
}
int tfft_c2r_pre(const void *x, void *z, const void *h, const void *l, int sh, int64_t m,
                 int64_t r, int a, void *s)
{
    (void)x; (void)z; (void)h; (void)l; (void)sh; (void)m; (void)r; (void)a; (void)s;
    return 0;
}

int tfft_batch_lines_per_tile(int log_l)
{
    if (log_l < 1 || log_l > TFFT_BATCH_MAX_LOG_L) return 0;
    return log_l <= 4 ? TFFT_BATCH_THREADS : (TFFT_BATCH_THREADS * 16) >> log_l;
}
int tfft_batch_max_ctas(int arith, int *ctas) { (void)arith; *ctas = 152; return 0; }
int tfft_launch_batch(const tfft_bpass *p, const tfft_bitem *i, int64_t n, int *st, int np,
                      int a, int c, long long sl, void *s)
{
    (void)p; (void)i; (void)n; (void)st; (void)np; (void)a; (void)c; (void)sl; (void)s;
    return 0;
}
int tfft_batch_graph(void **g, const tfft_bpass *p, const tfft_bitem *i, int64_t n, int *st,
                     int np, int a, int c, long long sl, void *s)
{
    (void)p; (void)i; (void)n; (void)st; (void)np; (void)a; (void)c; (void)sl; (void)s;
    *g = token();
    return 0;
}
int tfft_graph_launch(void *g, void *s) { (void)g; (void)s; return 0; }
int tfft_graph_destroy(void *g) { (void)g; return 0; }
int tfft_capture_begin(void *s) { (void)s; return 0; }
int tfft_capture_end(void **g, void *s) { (void)s; *g = token(); return 0; }

/* the allocation-free entry point lives in CUDA code */
int topeExec1DNoAlloc(const double *i, double *o, int n, int dir, void *s)
{
    (void)i; (void)o; (void)n; (void)dir; (void)s;
    return TOPE_ERR_UNSUPPORTED;
}
