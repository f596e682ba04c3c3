/*
 * Batches of independent transforms of uneven power-of-two sizes
 * (include/topefft_ext.h, topeBatch*).
 *
 * Planning: transforms of the same shape form a class.  Every class becomes
 * one or two passes of the pass kernel, addressing its transforms through a
 * per-class table of offsets into the caller's packed buffer (no data
 * movement), exactly as a batched plan of that shape would:
 *   1D, 2^k <= 2^12        one pass, B transforms per tile;
 *   1D, 2^13 .. 2^24       four-step: pass A into the second buffer with the
 *                          W_n^{i1 k2} factors, pass B back, transposed;
 *   2D                     an x pass then a y pass, in place.
 * Execution: every tile of every pass is a work item of one queue, first
 * passes before second passes; the persistent kernel (fft_batch.cuh) drains
 * it in one launch, replayed from a captured CUDA graph.  Alternatives for
 * comparison: a graph of one launch per class pass, and a loop of one
 * launch sequence per transform.
 *
 * Autotuning: the two-pass split of long 1D classes is chosen by timing
 * each candidate on the class itself; the persistent grid size by timing
 * the whole queue; split results are cached per (arithmetic, length, count)
 * in a text file.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include "../../include/topefft.h"
#include "../../include/topefft_ext.h"
#include "tfft_abi.h"
#include "topefft_internal.h"

#define BATCH_MAGIC 0xBA7C4u
#define MAX_BTABS 96

typedef struct bclass {
    int64_t nx, ny; /* ny == 1: 1D */
    int count;
    int64_t *h_off; /* caller offsets (complex elements) of its transforms */
    int64_t *d_off;
    int lx, ly;
    int l1, l2; /* four-step split of a long 1D class (0 if one pass) */
    int first_cp, ncp;
} bclass;

typedef struct bimpl {
    unsigned magic;
    int arith, es;
    int count;
    int64_t total;
    int64_t *h_toff;
    int *h_class;
    void *buf[2];
    int nclass;
    bclass *cls;
    int npass;
    tfft_bpass *hp[2]; /* forward, inverse */
    void *dp[2];
    tfft_bitem *hitems;
    void *ditems;
    int64_t nitems;
    int *dstate;
    void *graph[2];
    void *lgraph[2];
    int ctas;
    void *tabs[MAX_BTABS];
    int tab_key[MAX_BTABS];
    int ntabs;
    void *ev[4];
    int pending;
    int mode;
    long long spin_limit; /* bound of each device-side dependency wait */
    int test_stall;       /* test hook: one dependency can never be met */
} bimpl;

static int ilog2_exact(int64_t n)
{
    if (n < 1) return -1;
    int l = 0;
    while (((int64_t)1 << l) < n) l++;
    return (((int64_t)1 << l) == n) ? l : -1;
}

static int cuda_st(struct topeFFT *f, int rc) { return tope_cuda_status(f, rc); }

/* ------------------------------------------------------------------------ */
/* tables                                                                   */
/* ------------------------------------------------------------------------ */
static int tab_alloc(bimpl *P, size_t bytes, int key, void **out)
{
    if (P->ntabs >= MAX_BTABS) return TOPE_ERR_UNSUPPORTED;
    if (tfft_malloc(out, bytes)) return TOPE_ERR_ALLOC;
    P->tabs[P->ntabs] = *out;
    P->tab_key[P->ntabs++] = key;
    return TOPE_SUCCESS;
}

static int wl_table(struct topeFFT *f, bimpl *P, int log_l, const void **out)
{
    for (int i = 0; i < P->ntabs; i++)
        if (P->tab_key[i] == log_l) {
            *out = P->tabs[i];
            return TOPE_SUCCESS;
        }
    void *t;
    int st = tab_alloc(P, (size_t)16 << log_l, log_l, &t);
    if (st) return tope_status(f, st);
    int rc = tfft_twiddle_table(t, log_l, P->arith, f->command_queue);
    if (rc) return cuda_st(f, rc);
    *out = t;
    return TOPE_SUCCESS;
}

/* ------------------------------------------------------------------------ */
/* passes of a class                                                        */
/* ------------------------------------------------------------------------ */
static void pass_init(tfft_pass *p, int log_l, int arith)
{
    memset(p, 0, sizeof(*p));
    p->log_l = log_l;
    p->arith = arith;
    p->scale = 1.0;
    p->n[0] = p->n[1] = p->n[2] = 1;
    p->b_tile = tfft_batch_lines_per_tile(log_l);
}

static int64_t pass_tiles(const tfft_pass *p)
{
    return ((p->n[0] + p->b_tile - 1) / p->b_tile) * p->n[1] * p->n[2];
}

/* Fill out[0..1] with the forward passes of class c; returns their count
 * or a negative status. */
static int class_passes(struct topeFFT *f, bimpl *P, bclass *c, tfft_pass out[2])
{
    const void *tw;
    int st;
    if (c->ny == 1 && c->lx <= TFFT_BATCH_MAX_LOG_L) {
        if ((st = wl_table(f, P, c->lx, &tw))) return -st;
        pass_init(&out[0], c->lx, P->arith);
        out[0].tw = tw;
        out[0].ies = out[0].oes = 1;
        out[0].n[0] = c->count;
        out[0].tab0 = c->d_off;
        out[0].in = out[0].out = P->buf[0];
        return 1;
    }
    if (c->ny == 1) {
        const int lg = c->lx, l1 = c->l1, l2 = c->l2;
        const int64_t n1 = (int64_t)1 << l1, n2 = (int64_t)1 << l2;
        const int shift = (lg + 1) / 2;
        void *hi, *lo;
        if ((st = tab_alloc(P, (size_t)16 << (lg - shift), -1, &hi)) ||
            (st = tab_alloc(P, (size_t)16 << shift, -1, &lo)))
            return -tope_status(f, st);
        int rc = tfft_fourstep_tables(hi, lo, (int64_t)1 << lg, shift, P->arith, f->command_queue);
        if (rc) return -cuda_st(f, rc);
        if ((st = wl_table(f, P, l2, &tw))) return -st;
        pass_init(&out[0], l2, P->arith);
        out[0].tw = tw;
        out[0].ies = out[0].oes = n1;
        out[0].n[0] = n1;
        out[0].is[0] = out[0].os[0] = 1;
        out[0].n[1] = c->count;
        out[0].tab1 = c->d_off;
        out[0].post_tw = 1;
        out[0].tw_level = 0;
        out[0].tw_shift = shift;
        out[0].tw_n = (int64_t)1 << lg;
        out[0].tw_hi = hi;
        out[0].tw_lo = lo;
        out[0].in = P->buf[0];
        out[0].out = P->buf[1];
        if ((st = wl_table(f, P, l1, &tw))) return -st;
        pass_init(&out[1], l1, P->arith);
        out[1].tw = tw;
        out[1].ies = 1;
        out[1].oes = n2;
        out[1].n[0] = n2;
        out[1].is[0] = n1;
        out[1].os[0] = 1;
        out[1].n[1] = c->count;
        out[1].tab1 = c->d_off;
        out[1].in = P->buf[1];
        out[1].out = P->buf[0];
        return 2;
    }
    /* 2D: x then y, in place */
    if ((st = wl_table(f, P, c->lx, &tw))) return -st;
    pass_init(&out[0], c->lx, P->arith);
    out[0].tw = tw;
    out[0].ies = out[0].oes = 1;
    out[0].n[0] = c->ny;
    out[0].is[0] = out[0].os[0] = c->nx;
    out[0].n[1] = c->count;
    out[0].tab1 = c->d_off;
    out[0].in = out[0].out = P->buf[0];
    if ((st = wl_table(f, P, c->ly, &tw))) return -st;
    pass_init(&out[1], c->ly, P->arith);
    out[1].tw = tw;
    out[1].ies = out[1].oes = c->nx;
    out[1].n[0] = c->nx;
    out[1].is[0] = out[1].os[0] = 1;
    out[1].n[1] = c->count;
    out[1].tab1 = c->d_off;
    out[1].in = out[1].out = P->buf[0];
    return 2;
}

/* inverse variant of pass i of class c: conjugate on entry and exit, 1/N */
static void make_inverse(tfft_pass *p, const bclass *c, int i)
{
    p->conj_in = i == 0;
    p->conj_out = i == c->ncp - 1;
    p->scale = (i == c->ncp - 1) ? 1.0 / (double)(c->nx * c->ny) : 1.0;
}

/* the per-class standalone launch of a class pass: lines per CTA within the
 * standalone kernel's limits (<= 32, L*B <= 8192) */
static tfft_pass standalone(const tfft_pass *p)
{
    tfft_pass q = *p;
    int b = q.b_tile;
    int cap = 8192 >> q.log_l;
    if (cap > 32) cap = 32;
    if (cap < 1) cap = 1;
    while (b > cap) b >>= 1;
    q.b_tile = b;
    return q;
}

/* ------------------------------------------------------------------------ */
/* tuning cache                                                             */
/* ------------------------------------------------------------------------ */
static const char *tune_path(char *buf, size_t n)
{
    const char *e = getenv("TOPEFFT_TUNE_CACHE");
    if (e && *e) return e;
    const char *h = getenv("HOME");
    snprintf(buf, n, "%s/.cache/topefft_tune.txt", h && *h ? h : "/tmp");
    return buf;
}

static int tune_lookup(int arith, int lg, int count_log, int *l2)
{
    char pb[512];
    FILE *fp = fopen(tune_path(pb, sizeof pb), "r");
    if (!fp) return 0;
    char line[256];
    int found = 0;
    while (fgets(line, sizeof line, fp)) {
        int a, n, c, v;
        if (sscanf(line, "split arith=%d log2n=%d log2count=%d l2=%d", &a, &n, &c, &v) == 4 &&
            a == arith && n == lg && c == count_log) {
            *l2 = v;
            found = 1;
        }
    }
    fclose(fp);
    return found;
}

static void tune_store(int arith, int lg, int count_log, int l2, unsigned long long ns)
{
    char pb[512];
    const char *path = tune_path(pb, sizeof pb);
    FILE *fp = fopen(path, "a");
    if (!fp) {
        /* create the file's directory (last component only) and retry */
        char dir[512];
        snprintf(dir, sizeof dir, "%s", path);
        char *slash = strrchr(dir, '/');
        if (slash) {
            *slash = 0;
            mkdir(dir, 0755);
        }
        fp = fopen(path, "a");
        if (!fp) return;
    }
    fprintf(fp, "split arith=%d log2n=%d log2count=%d l2=%d ns=%llu\n", arith, lg, count_log, l2, ns);
    fclose(fp);
}

static int autotune_enabled(void)
{
    const char *e = getenv("TOPEFFT_AUTOTUNE");
    return !(e && !strcmp(e, "0"));
}

/* time `reps` runs of a class's passes launched standalone; ns per run */
static unsigned long long time_class(struct topeFFT *f, bimpl *P, tfft_pass *ps, int n, int reps)
{
    void *stream = f->command_queue;
    for (int r = -1; r < reps; r++) {
        if (r == 0) tfft_event_record(P->ev[0], stream);
        for (int i = 0; i < n; i++) {
            tfft_pass q = standalone(&ps[i]);
            if (tfft_launch_pass(&q, stream)) return ~0ull;
        }
    }
    tfft_event_record(P->ev[1], stream);
    if (tfft_stream_sync(stream)) return ~0ull;
    uint64_t ns = 0;
    tfft_event_elapsed_ns(P->ev[0], P->ev[1], &ns);
    return reps > 0 ? ns / (unsigned long long)reps : ns;
}

/* choose the split (l1 = lg - l2) of a long 1D class */
static int tune_split(struct topeFFT *f, bimpl *P, bclass *c)
{
    const int lg = c->lx;
    int clog = 0;
    while ((1 << clog) < c->count) clog++;
    int best = (lg + 1) / 2, cached;
    if (best > TFFT_BATCH_MAX_LOG_L) best = TFFT_BATCH_MAX_LOG_L;
    if (lg - best > TFFT_BATCH_MAX_LOG_L) best = lg - TFFT_BATCH_MAX_LOG_L;
    if (tune_lookup(P->arith, lg, clog, &cached) && cached >= lg - TFFT_BATCH_MAX_LOG_L &&
        cached <= TFFT_BATCH_MAX_LOG_L && cached >= 1 && cached < lg) {
        c->l2 = cached;
        c->l1 = lg - cached;
        return TOPE_SUCCESS;
    }
    if (!autotune_enabled()) {
        c->l2 = best;
        c->l1 = lg - best;
        return TOPE_SUCCESS;
    }
    unsigned long long best_ns = ~0ull;
    int chosen = best;
    for (int l2 = best - 2; l2 <= best + 2; l2++) {
        if (l2 < 1 || l2 >= lg || l2 > TFFT_BATCH_MAX_LOG_L || lg - l2 > TFFT_BATCH_MAX_LOG_L) continue;
        c->l2 = l2;
        c->l1 = lg - l2;
        tfft_pass ps[2];
        int n = class_passes(f, P, c, ps);
        if (n < 0) return -n;
        unsigned long long ns = time_class(f, P, ps, n, 3);
        if (ns < best_ns) {
            best_ns = ns;
            chosen = l2;
        }
    }
    c->l2 = chosen;
    c->l1 = lg - chosen;
    tune_store(P->arith, lg, clog, chosen, best_ns);
    return TOPE_SUCCESS;
}

/* ------------------------------------------------------------------------ */
/* plan                                                                     */
/* ------------------------------------------------------------------------ */
static void bimpl_free(bimpl *P)
{
    if (!P) return;
    for (int i = 0; i < 2; i++) {
        tfft_graph_destroy(P->graph[i]);
        tfft_graph_destroy(P->lgraph[i]);
        tfft_free(P->dp[i]);
        free(P->hp[i]);
        tfft_free(P->buf[i]);
    }
    for (int i = 0; i < P->ntabs; i++) tfft_free(P->tabs[i]);
    for (int i = 0; i < P->nclass; i++) {
        free(P->cls[i].h_off);
        tfft_free(P->cls[i].d_off);
    }
    free(P->cls);
    tfft_free(P->ditems);
    free(P->hitems);
    tfft_free(P->dstate);
    free(P->h_toff);
    free(P->h_class);
    for (int i = 0; i < 4; i++) tfft_event_destroy(P->ev[i]);
    P->magic = 0;
    free(P);
}

static int cmp_items_desc(const void *a, const void *b)
{
    /* sort key packed by the caller: higher log_l first, then class pass, tile */
    const int64_t *x = (const int64_t *)a, *y = (const int64_t *)b;
    return x[0] < y[0] ? 1 : x[0] > y[0] ? -1 : 0;
}

/* Build queue, device descriptors and graphs for the current class splits. */
static int build_queue(struct topeFFT *f, bimpl *P)
{
    tfft_bpass *fw = (tfft_bpass *)calloc((size_t)2 * P->nclass, sizeof(tfft_bpass));
    if (!fw) return tope_status(f, TOPE_ERR_ALLOC);
    int np = 0;
    for (int ci = 0; ci < P->nclass; ci++) {
        bclass *c = &P->cls[ci];
        tfft_pass ps[2];
        int n = class_passes(f, P, c, ps);
        if (n < 0) {
            free(fw);
            return -n;
        }
        c->first_cp = np;
        c->ncp = n;
        for (int i = 0; i < n; i++) {
            fw[np].p = ps[i];
            fw[np].tiles = pass_tiles(&ps[i]);
            fw[np].dep = i ? np - 1 : -1;
            fw[np].extra = 0;
            np++;
        }
    }
    if (P->test_stall) {
        /* failure-detection test: the first dependent pass waits for one
         * tile more than its dependency has, so its bounded wait runs out */
        for (int i = 0; i < np; i++)
            if (fw[i].dep >= 0) {
                fw[i].extra = 1;
                break;
            }
    }
    P->npass = np;
    for (int d = 0; d < 2; d++) {
        free(P->hp[d]);
        P->hp[d] = (tfft_bpass *)calloc((size_t)np, sizeof(tfft_bpass));
        if (!P->hp[d]) {
            free(fw);
            return tope_status(f, TOPE_ERR_ALLOC);
        }
        memcpy(P->hp[d], fw, sizeof(tfft_bpass) * (size_t)np);
    }
    free(fw);
    for (int ci = 0; ci < P->nclass; ci++) {
        bclass *c = &P->cls[ci];
        for (int i = 0; i < c->ncp; i++) make_inverse(&P->hp[0][c->first_cp + i].p, c, i);
    }
    /* hp[0] = inverse (dir 0), hp[1] = forward (dir 1) */
    /* work items: phase 0 (first passes) then phase 1; inside a phase the
     * longer lines first (more work per tile) */
    int64_t n_items = 0;
    for (int i = 0; i < np; i++) n_items += P->hp[1][i].tiles;
    int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)n_items);
    free(P->hitems);
    P->hitems = (tfft_bitem *)malloc(sizeof(tfft_bitem) * (size_t)n_items);
    if (!keys || !P->hitems) {
        free(keys);
        return tope_status(f, TOPE_ERR_ALLOC);
    }
    int64_t k = 0;
    for (int phase = 0; phase < 2; phase++) {
        int64_t start = k;
        for (int ci = 0; ci < P->nclass; ci++) {
            bclass *c = &P->cls[ci];
            if (phase >= c->ncp) continue;
            int cp = c->first_cp + phase;
            for (int64_t t = 0; t < P->hp[1][cp].tiles; t++) {
                keys[2 * k] = ((int64_t)P->hp[1][cp].p.log_l << 40) | ((int64_t)(np - cp) << 20);
                keys[2 * k + 1] = ((int64_t)cp << 32) | t;
                k++;
            }
        }
        qsort(keys + 2 * start, (size_t)(k - start), 2 * sizeof(int64_t), cmp_items_desc);
    }
    for (int64_t i = 0; i < n_items; i++) {
        P->hitems[i].cp = (int)(keys[2 * i + 1] >> 32);
        P->hitems[i].pad = 0;
        P->hitems[i].tile = keys[2 * i + 1] & 0xffffffffll;
    }
    free(keys);
    P->nitems = n_items;
    void *stream = f->command_queue;
    int rc;
    tfft_free(P->ditems);
    P->ditems = NULL;
    for (int d = 0; d < 2; d++) {
        tfft_free(P->dp[d]);
        P->dp[d] = NULL;
    }
    tfft_free(P->dstate);
    P->dstate = NULL;
    if (tfft_malloc(&P->ditems, sizeof(tfft_bitem) * (size_t)n_items) ||
        tfft_malloc(&P->dp[0], sizeof(tfft_bpass) * (size_t)np) ||
        tfft_malloc(&P->dp[1], sizeof(tfft_bpass) * (size_t)np) ||
        tfft_malloc((void **)&P->dstate, sizeof(int) * (size_t)(2 + np)))
        return tope_status(f, TOPE_ERR_ALLOC);
    if ((rc = tfft_h2d(P->ditems, P->hitems, sizeof(tfft_bitem) * (size_t)n_items, stream)) ||
        (rc = tfft_h2d(P->dp[0], P->hp[0], sizeof(tfft_bpass) * (size_t)np, stream)) ||
        (rc = tfft_h2d(P->dp[1], P->hp[1], sizeof(tfft_bpass) * (size_t)np, stream)) ||
        (rc = tfft_stream_sync(stream)))
        return cuda_st(f, rc);
    return TOPE_SUCCESS;
}

static int build_graphs(struct topeFFT *f, bimpl *P)
{
    void *stream = f->command_queue;
    int rc;
    for (int d = 0; d < 2; d++) {
        tfft_graph_destroy(P->graph[d]);
        tfft_graph_destroy(P->lgraph[d]);
        P->graph[d] = P->lgraph[d] = NULL;
        rc = tfft_batch_graph(&P->graph[d], (const tfft_bpass *)P->dp[d],
                              (const tfft_bitem *)P->ditems, P->nitems, P->dstate, P->npass,
                              P->arith, P->ctas, P->spin_limit, stream);
        if (rc) return cuda_st(f, rc);
        /* one launch per class pass, in class order */
        if ((rc = tfft_capture_begin(stream))) return cuda_st(f, rc);
        int lrc = 0;
        for (int i = 0; i < P->npass && !lrc; i++) {
            tfft_pass q = standalone(&P->hp[d][i].p);
            lrc = tfft_launch_pass(&q, stream);
        }
        rc = tfft_capture_end(&P->lgraph[d], stream);
        if (lrc) return cuda_st(f, lrc);
        if (rc) return cuda_st(f, rc);
    }
    return TOPE_SUCCESS;
}

/* time the persistent queue (forward) with ctas CTAs */
static unsigned long long time_queue(struct topeFFT *f, bimpl *P, int ctas, int reps)
{
    void *stream = f->command_queue;
    for (int r = -1; r < reps; r++) {
        if (r == 0) tfft_event_record(P->ev[0], stream);
        if (tfft_launch_batch((const tfft_bpass *)P->dp[1], (const tfft_bitem *)P->ditems,
                              P->nitems, P->dstate, P->npass, P->arith, ctas, P->spin_limit,
                              stream))
            return ~0ull;
    }
    tfft_event_record(P->ev[1], stream);
    if (tfft_stream_sync(stream)) return ~0ull;
    uint64_t ns = 0;
    tfft_event_elapsed_ns(P->ev[0], P->ev[1], &ns);
    return ns / (unsigned long long)reps;
}

static void batch_init(struct topeFFT *f, struct topeBatch *b, int count, const int *nx,
                       const int *ny, int type, const void *d, int arith)
{
    if (!b) {
        tope_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    memset(b, 0, sizeof(*b));
    b->count = count;
    b->type = type;
    if (type != C2C) {
        tope_status(f, TOPE_ERR_UNSUPPORTED);
        return;
    }
    if (count < 1 || !nx || !ny) {
        tope_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    int st = tope_framework_ready(f);
    if (st) return;
    bimpl *P = (bimpl *)calloc(1, sizeof(bimpl));
    if (!P) {
        tope_status(f, TOPE_ERR_ALLOC);
        return;
    }
    P->magic = BATCH_MAGIC;
    P->arith = arith;
    P->spin_limit = 1ll << 24; /* ~2 s: far beyond any legitimate wait */
    {
        const char *ts = getenv("TOPEFFT_BATCH_TEST_STALL");
        if (ts && *ts && strcmp(ts, "0")) {
            P->test_stall = 1;
            P->spin_limit = 1ll << 12; /* ~1 ms */
        }
    }
    P->es = TFFT_ELEM_BYTES(arith);
    P->count = count;
    P->h_toff = (int64_t *)malloc(sizeof(int64_t) * (size_t)count);
    P->h_class = (int *)malloc(sizeof(int) * (size_t)count);
    P->cls = (bclass *)calloc((size_t)count < 64 ? (size_t)count : 64, sizeof(bclass));
    int cap = count < 64 ? count : 64;
    int rc = 0;
    void *stream = f->command_queue;
    if (!P->h_toff || !P->h_class || !P->cls) {
        st = TOPE_ERR_ALLOC;
        goto fail;
    }
    for (int i = 0; i < 4; i++)
        if ((rc = tfft_event_create(&P->ev[i]))) goto fail_cuda;
    /* validate, offsets, classes */
    int64_t off = 0;
    for (int i = 0; i < count; i++) {
        int lx = ilog2_exact(nx[i]), ly = ilog2_exact(ny[i]);
        if (lx < 1 || ly < 0 || (ny[i] == 1 && lx > 2 * TFFT_BATCH_MAX_LOG_L) ||
            (ny[i] > 1 && (ly < 1 || lx > TFFT_BATCH_MAX_LOG_L || ly > TFFT_BATCH_MAX_LOG_L))) {
            st = TOPE_ERR_INVALID_SIZE;
            goto fail;
        }
        P->h_toff[i] = off;
        off += (int64_t)nx[i] * ny[i];
        int ci;
        for (ci = 0; ci < P->nclass; ci++)
            if (P->cls[ci].nx == nx[i] && P->cls[ci].ny == ny[i]) break;
        if (ci == P->nclass) {
            if (P->nclass == cap) {
                cap *= 2;
                bclass *nc = (bclass *)realloc(P->cls, sizeof(bclass) * (size_t)cap);
                if (!nc) {
                    st = TOPE_ERR_ALLOC;
                    goto fail;
                }
                P->cls = nc;
            }
            memset(&P->cls[ci], 0, sizeof(bclass));
            P->cls[ci].nx = nx[i];
            P->cls[ci].ny = ny[i];
            P->cls[ci].lx = lx;
            P->cls[ci].ly = ly;
            P->nclass++;
        }
        P->cls[ci].count++;
        P->h_class[i] = ci;
    }
    P->total = off;
    for (int ci = 0; ci < P->nclass; ci++) {
        P->cls[ci].h_off = (int64_t *)malloc(sizeof(int64_t) * (size_t)P->cls[ci].count);
        if (!P->cls[ci].h_off) {
            st = TOPE_ERR_ALLOC;
            goto fail;
        }
        P->cls[ci].count = 0;
    }
    for (int i = 0; i < count; i++) {
        bclass *c = &P->cls[P->h_class[i]];
        c->h_off[c->count++] = P->h_toff[i];
    }
    int need2 = 0;
    for (int ci = 0; ci < P->nclass; ci++) {
        bclass *c = &P->cls[ci];
        if (tfft_malloc((void **)&c->d_off, sizeof(int64_t) * (size_t)c->count)) {
            st = TOPE_ERR_ALLOC;
            goto fail;
        }
        if ((rc = tfft_h2d(c->d_off, c->h_off, sizeof(int64_t) * (size_t)c->count, stream)))
            goto fail_cuda;
        if (c->ny == 1 && c->lx > TFFT_BATCH_MAX_LOG_L) need2 = 1;
    }
    size_t bytes = (size_t)P->total * (size_t)P->es;
    if (tfft_malloc(&P->buf[0], bytes) || (need2 && tfft_malloc(&P->buf[1], bytes))) {
        st = TOPE_ERR_ALLOC;
        goto fail;
    }
    if ((rc = tfft_memset_async(P->buf[0], 0, bytes, stream)) ||
        (need2 && (rc = tfft_memset_async(P->buf[1], 0, bytes, stream))))
        goto fail_cuda;
    tfft_event_record(P->ev[2], stream);
    /* long 1D classes: autotuned split */
    for (int ci = 0; ci < P->nclass; ci++) {
        bclass *c = &P->cls[ci];
        if (c->ny == 1 && c->lx > TFFT_BATCH_MAX_LOG_L && (st = tune_split(f, P, c))) goto fail;
    }
    if ((st = build_queue(f, P))) goto fail;
    /* persistent grid: all co-resident CTAs, or half of them if faster */
    int maxc = 0;
    if ((rc = tfft_batch_max_ctas(P->arith, &maxc))) goto fail_cuda;
    if (maxc < 1) {
        st = TOPE_ERR_UNSUPPORTED;
        goto fail;
    }
    P->ctas = maxc;
    if (autotune_enabled() && maxc > 1) {
        unsigned long long a = time_queue(f, P, maxc, 2), h = time_queue(f, P, maxc / 2, 2);
        if (h < a) P->ctas = maxc / 2;
    }
    if ((st = build_graphs(f, P))) goto fail;
    /* execution structure: the persistent launch unless the per-class
     * launch graph measures at least 5% faster */
    P->mode = TOPE_BATCH_PERSISTENT;
    if (autotune_enabled() && !P->test_stall) {
        unsigned long long tp = ~0ull, tl = ~0ull;
        for (int m = 0; m < 2; m++) {
            void *g = m == 0 ? P->graph[1] : P->lgraph[1];
            if (tfft_graph_launch(g, stream)) continue;
            tfft_event_record(P->ev[0], stream);
            for (int r = 0; r < 2; r++) tfft_graph_launch(g, stream);
            tfft_event_record(P->ev[1], stream);
            if (tfft_stream_sync(stream)) continue;
            uint64_t ns = 0;
            tfft_event_elapsed_ns(P->ev[0], P->ev[1], &ns);
            if (m == 0) tp = ns;
            else tl = ns;
        }
        if (tl < tp && (double)tl < 0.95 * (double)tp) P->mode = TOPE_BATCH_LAUNCHES;
    }
    tfft_event_record(P->ev[3], stream);
    /* upload the caller's data */
    if (d) rc = tfft_h2d(P->buf[0], d, bytes, stream);
    tfft_event_record(P->ev[1], stream);
    if (!rc) rc = tfft_stream_sync(stream);
    if (rc) goto fail_cuda;
    uint64_t ns = 0;
    tfft_event_elapsed_ns(P->ev[2], P->ev[3], &ns);
    b->totalPreKernel += ns;
    tfft_event_elapsed_ns(P->ev[3], P->ev[1], &ns);
    b->totalMemory += ns;
    b->dataSize = bytes;
    b->data = P->buf[0];
    b->elem_bytes = P->es;
    b->classes = P->nclass;
    b->ctas = P->ctas;
    b->work_items = P->nitems;
    b->mode = P->mode;
    b->impl = P;
    tope_framework_plan_added(f);
    tope_status(f, TOPE_SUCCESS);
    return;
fail_cuda:
    tfft_stream_sync(stream);
    bimpl_free(P);
    cuda_st(f, rc);
    return;
fail:
    tfft_stream_sync(stream);
    bimpl_free(P);
    tope_status(f, st);
}

void topeBatchPlanInit(struct topeFFT *f, struct topeBatch *b, int count, const int *nx,
                       const int *ny, int type, double *d)
{
    batch_init(f, b, count, nx, ny, type, d, f ? f->arith : 0);
}

void topeBatchPlanInitF32(struct topeFFT *f, struct topeBatch *b, int count, const int *nx,
                          const int *ny, int type, float *d)
{
    if (f && f->split_mode == TOPE_SPLIT_TENSOR) {
        /* the persistent kernel has no tensor-core stages */
        if (b) b->impl = NULL;
        tope_status(f, TOPE_ERR_UNSUPPORTED);
        return;
    }
    int arith = (f && f->split_mode == TOPE_SPLIT_FAST) ? TFFT_ARITH_F32 : TFFT_ARITH_DF32;
    batch_init(f, b, count, nx, ny, type, d, arith);
}

static bimpl *bimpl_of(struct topeFFT *f, struct topeBatch *b)
{
    if (!f || !b) {
        tope_status(f, TOPE_ERR_INVALID_ARG);
        return NULL;
    }
    bimpl *P = (bimpl *)b->impl;
    if (!P || P->magic != BATCH_MAGIC) {
        tope_status(f, TOPE_ERR_DESTROYED);
        return NULL;
    }
    if (!f->command_queue) {
        tope_status(f, TOPE_ERR_NOT_INITIALIZED);
        return NULL;
    }
    return P;
}

/* read the persistent kernel's error flag after a synchronisation */
static int check_flag(struct topeFFT *f, bimpl *P)
{
    if (P->mode != TOPE_BATCH_PERSISTENT) return TOPE_SUCCESS;
    int flags[2] = {0, 0};
    int rc = tfft_d2h(flags, P->dstate, sizeof flags, f->command_queue);
    if (!rc) rc = tfft_stream_sync(f->command_queue);
    if (rc) return cuda_st(f, rc);
    return flags[1] ? tope_status(f, TOPE_ERR_TIMEOUT) : TOPE_SUCCESS;
}

static void settle(struct topeBatch *b, bimpl *P)
{
    if (P->pending) {
        uint64_t ns = 0;
        tfft_event_elapsed_ns(P->ev[0], P->ev[1], &ns);
        b->totalKernel += ns;
        P->pending = 0;
    }
}

/* queue one transform of the batch in the current mode */
static int exec_async(struct topeFFT *f, struct topeBatch *b, bimpl *P, int dir)
{
    if (dir != FORWARD && dir != INVERSE) return tope_status(f, TOPE_ERR_INVALID_ARG);
    void *stream = f->command_queue;
    const int di = dir == FORWARD ? 1 : 0;
    int rc = 0;
    tfft_event_record(P->ev[0], stream);
    if (P->mode == TOPE_BATCH_PERSISTENT) {
        rc = tfft_graph_launch(P->graph[di], stream);
    } else if (P->mode == TOPE_BATCH_LAUNCHES) {
        rc = tfft_graph_launch(P->lgraph[di], stream);
    } else {
        /* one launch sequence per transform, in the caller's order */
        for (int t = 0; t < P->count && !rc; t++) {
            const bclass *c = &P->cls[P->h_class[t]];
            for (int i = 0; i < c->ncp && !rc; i++) {
                tfft_pass q = P->hp[di][c->first_cp + i].p;
                q.n[1] = 1;
                q.tab1 = NULL;
                if (q.tab0) { /* 1D single pass: one line */
                    q.n[0] = 1;
                    q.tab0 = NULL;
                }
                q.in = (const char *)q.in + P->h_toff[t] * P->es;
                q.out = (char *)q.out + P->h_toff[t] * P->es;
                q = standalone(&q);
                while (q.b_tile > 1 && q.n[0] % q.b_tile) q.b_tile >>= 1;
                rc = tfft_launch_pass(&q, stream);
            }
        }
    }
    tfft_event_record(P->ev[1], stream);
    P->pending = 1;
    (void)b;
    return rc ? cuda_st(f, rc) : TOPE_SUCCESS;
}

void topeBatchExecDevice(struct topeFFT *f, struct topeBatch *b, int dir)
{
    bimpl *P = bimpl_of(f, b);
    if (!P) return;
    if (exec_async(f, b, P, dir) == TOPE_SUCCESS) tope_status(f, TOPE_SUCCESS);
}

static void batch_exec(struct topeFFT *f, struct topeBatch *b, void *d, int es, int dir)
{
    bimpl *P = bimpl_of(f, b);
    if (!P) return;
    if (P->es != es) {
        tope_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    void *stream = f->command_queue;
    int st = exec_async(f, b, P, dir), rc = 0;
    if (!st && d) {
        tfft_event_record(P->ev[2], stream);
        rc = tfft_d2h(d, P->buf[0], (size_t)P->total * P->es, stream);
        tfft_event_record(P->ev[3], stream);
    }
    int rc2 = tfft_stream_sync(stream);
    if (st) return;
    if (rc || rc2) {
        cuda_st(f, rc ? rc : rc2);
        return;
    }
    settle(b, P);
    if (d) {
        uint64_t ns = 0;
        tfft_event_elapsed_ns(P->ev[2], P->ev[3], &ns);
        b->totalMemory += ns;
    }
    if (check_flag(f, P)) return;
    tope_status(f, TOPE_SUCCESS);
}

void topeBatchExec(struct topeFFT *f, struct topeBatch *b, double *d, int dir)
{
    batch_exec(f, b, d, 16, dir);
}

void topeBatchExecF32(struct topeFFT *f, struct topeBatch *b, float *d, int dir)
{
    batch_exec(f, b, d, 8, dir);
}

void topeBatchUpload(struct topeFFT *f, struct topeBatch *b, const void *d)
{
    bimpl *P = bimpl_of(f, b);
    if (!P) return;
    if (!d) {
        tope_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    void *stream = f->command_queue;
    tfft_event_record(P->ev[2], stream);
    int rc = tfft_h2d(P->buf[0], d, (size_t)P->total * P->es, stream);
    tfft_event_record(P->ev[3], stream);
    if (!rc) rc = tfft_stream_sync(stream);
    if (rc) {
        cuda_st(f, rc);
        return;
    }
    uint64_t ns = 0;
    tfft_event_elapsed_ns(P->ev[2], P->ev[3], &ns);
    b->totalMemory += ns;
    tope_status(f, TOPE_SUCCESS);
}

void topeBatchDownload(struct topeFFT *f, struct topeBatch *b, void *d)
{
    bimpl *P = bimpl_of(f, b);
    if (!P) return;
    if (!d) {
        tope_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    void *stream = f->command_queue;
    int rc = tfft_d2h(d, P->buf[0], (size_t)P->total * P->es, stream);
    if (!rc) rc = tfft_stream_sync(stream);
    if (rc) {
        cuda_st(f, rc);
        return;
    }
    settle(b, P);
    if (check_flag(f, P)) return;
    tope_status(f, TOPE_SUCCESS);
}

void topeBatchSetMode(struct topeFFT *f, struct topeBatch *b, int mode)
{
    bimpl *P = bimpl_of(f, b);
    if (!P) return;
    if (mode != TOPE_BATCH_PERSISTENT && mode != TOPE_BATCH_LAUNCHES && mode != TOPE_BATCH_LOOP) {
        tope_status(f, TOPE_ERR_INVALID_ARG);
        return;
    }
    tfft_stream_sync(f->command_queue);
    P->mode = mode;
    b->mode = mode;
    tope_status(f, TOPE_SUCCESS);
}

void topeBatchDestroy(struct topeFFT *f, struct topeBatch *b)
{
    bimpl *P = bimpl_of(f, b);
    if (!P) return;
    tfft_stream_sync(f->command_queue);
    bimpl_free(P);
    b->impl = NULL;
    b->data = NULL;
    tope_framework_plan_removed(f);
    tope_status(f, TOPE_SUCCESS);
}
