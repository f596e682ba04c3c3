/*
 * Internal C ABI between the C host library (topefft.c, planner.c) and the
 * CUDA translation units.  Plain C types only: no CUDA or torch types cross
 * this boundary, so the host side compiles with a plain C compiler.
 */
#ifndef TFFT_ABI_H
#define TFFT_ABI_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic used inside the butterflies.  Storage is FP64 for both. */
enum tfft_arith {
    TFFT_ARITH_F64 = 0,  /* native double-precision instructions          */
    TFFT_ARITH_DF64 = 1, /* double-float: FP32 (hi, lo) pairs on the FP32
                            pipe; FP64 loads/stores and FP64-accurate tables */
    TFFT_ARITH_F32 = 2,  /* split precision, fast: FP32 storage and FP32
                            butterflies, twiddles as FP64-accurate (hi, lo)
                            FP32 pairs                                        */
    TFFT_ARITH_DF32 = 3, /* split precision, accurate: FP32 storage, double-
                            float butterflies on chip, so only the FP32 loads
                            and stores round                                  */
    TFFT_ARITH_TC = 4,   /* split precision, tensor: FP32 storage, radix-16
                            stages as tcgen05 GEMMs on 3-piece FP16 splits
                            (an exact and a cross-product FP32 accumulator);
                            everything else as TFFT_ARITH_DF32              */
};

/* bytes of one complex element in memory for an arithmetic */
#define TFFT_ELEM_BYTES(arith) ((arith) >= TFFT_ARITH_F32 ? 8 : 16)

/* Largest line length one CTA transforms: 2^13 complex points for 16-byte
 * on-chip elements and for the tensor form, 2^14 for FP32 complex. */
#define TFFT_MAX_LOG_L 14
#define TFFT_MAX_LOG_L_ARITH(arith) ((arith) == TFFT_ARITH_F32 ? 14 : 13)

/*
 * One pass = batched FFTs of length L = 2^log_l over "lines".  Line
 * (g0, g1, g2) starts at in + g0*is[0] + g1*is[1] + g2*is[2] and its element
 * i sits at + i*ies (all in complex elements).  The output line is laid out
 * the same way with os[]/oes, so a pass may transpose on its way out.
 * A CTA takes b_tile consecutive g0 values (n[0] % b_tile == 0).
 *
 * Optional fused extras, applied in this order:
 *   conj_in   conjugate on load (inverse transforms run as conj(F(conj x)))
 *   post_tw   multiply output element k of a line by W_N^{t*k}, where t is
 *             g0 (tw_level 0) or g1 (tw_level 1) and N = tw_n; the factor is
 *             tw_hi[m >> tw_shift] * tw_lo[m & (2^tw_shift - 1)], m = t*k < N,
 *             or tw_hi[m] when tw_lo is NULL (a whole table of N entries)
 *   conj_out  conjugate on store
 *   scale     multiply on store (1.0 = none; 1/N is exact for N = 2^k)
 */
#define TFFT_MAX_RADICES 24

typedef struct tfft_pass {
    int log_l;
    int b_tile;
    int arith;
    int conj_in, conj_out;
    double scale;
    const void *in;
    void *out;
    int64_t n[3];
    int64_t is[3], os[3];
    int64_t ies, oes;
    const void *tw;      /* W_L^m, m < L, layout per arith */
    int post_tw;
    int tw_level;
    int tw_shift;
    int64_t tw_n;
    const void *tw_hi, *tw_lo;
    /* optional per-line base tables (device int64, in complex elements):
     * when set, tab0[g0] replaces g0*is[0] (and g0*os[0]) and tab1[g1]
     * replaces g1*is[1] (and g1*os[1]); used by batches of transforms that
     * sit at arbitrary offsets of the caller's packed buffer */
    const int64_t *tab0, *tab1;
    /* TFFT_ARITH_TC: the six FP16 B matrices (pieces of the real 32x32
     * DFT-16) in the tensor cores' shared-memory layout (tfft_tc_matrix) */
    const void *mma_b;
    /* points per thread: 0 or 16 (radix-16 stages), or 4 (radix-4 stages,
     * FP64 storage, log2 L = 2..7: small transforms) */
    int ept;
    /* lines whose length is not a power of two: len = L (log_l unused),
     * transformed in nrad Stockham stages of the radices radix[] (2, 3, 4,
     * 5, 7, 8, 11, 13; product L) by the mixed-radix kernel; 0 otherwise */
    int len;
    int nrad;
    unsigned char radix[TFFT_MAX_RADICES];
    /* tiles of whole contiguous lines (ies == 1, is[0] == L): a full tile may
     * arrive by bulk asynchronous copies (cp.async.bulk, one per line) into
     * shared memory instead of direct loads, in the kernel shapes that take
     * it (tfft_pass_bulk_capable); err, a device word, is set to 1 when a
     * wait for those copies gives up (NULL: not reported) */
    int bulk;
    int *err;
    /* strided passes of adjacent lines (is[0] == 1): a tensor map of the
     * pass's input array (device memory, TFFT_TENSOR_MAP_BYTES) in 8-byte
     * units, dimension 0 the lines, dimension k + 1 the source tmap_src[k]
     * (0: the line's elements, 1: g1, 2: g2) in stride order; full tiles
     * then arrive by TMA, boxes of the tile's lines by up to 256 elements
     * (NULL: not used) */
    const void *tmap;
    int tmap_rank;
    signed char tmap_src[4];
} tfft_pass;

/* mixed-radix lines: at most TFFT_MIXED_MAX_POINTS points per CTA (L * b_tile) */
#define TFFT_MIXED_MAX_POINTS 4096

/* ---- batches of independent transforms (persistent kernel) --------------- */
/* one pass over one class of same-shaped transforms */
typedef struct tfft_bpass {
    tfft_pass p;
    int64_t tiles; /* work items of this pass */
    int dep;       /* class-pass whose completion this one waits for, or -1 */
    int extra;     /* tiles required of dep beyond its count (0; a test hook
                      sets 1 to make the wait run out) */
} tfft_bpass;

/* one work item: tile `tile` of class-pass `cp` */
typedef struct tfft_bitem {
    int cp;
    int pad;
    int64_t tile;
} tfft_bitem;

/* lines per tile of the batch kernel for log2 L (256 threads per CTA) */
#define TFFT_BATCH_THREADS 256
#define TFFT_BATCH_MAX_LOG_L 12
int tfft_batch_lines_per_tile(int log_l);
/* CTAs of the persistent kernel that fit on the device at once */
int tfft_batch_max_ctas(int arith, int *ctas);
/* state: int32 [0] queue head, [1] error flag, [2 + i] tiles done of pass i;
 * spin_limit bounds each dependency wait (iterations of ~100 ns) */
int tfft_launch_batch(const tfft_bpass *d_passes, const tfft_bitem *d_items, int64_t n_items,
                      int *d_state, int n_passes, int arith, int ctas, long long spin_limit,
                      void *stream);
/* capture "clear state + batch launch" on stream into an executable graph */
int tfft_batch_graph(void **graph_exec, const tfft_bpass *d_passes, const tfft_bitem *d_items,
                     int64_t n_items, int *d_state, int n_passes, int arith, int ctas,
                     long long spin_limit, void *stream);
int tfft_graph_launch(void *graph_exec, void *stream);
int tfft_graph_destroy(void *graph_exec);
/* capture a sequence of pass launches into an executable graph */
int tfft_capture_begin(void *stream);
int tfft_capture_end(void **graph_exec, void *stream);

/* ---- device memory / streams / events (thin wrappers, return 0 or a
 *      CUDA error code) --------------------------------------------------- */
int tfft_set_device(int dev);
int tfft_get_device(int *dev);
int tfft_device_count(int *n);
int tfft_malloc(void **p, size_t bytes);
int tfft_free(void *p);
int tfft_host_alloc(void **p, size_t bytes);
int tfft_host_free(void *p);
int tfft_memset_async(void *p, int v, size_t bytes, void *stream);
int tfft_h2d(void *dst, const void *src, size_t bytes, void *stream);
int tfft_d2h(void *dst, const void *src, size_t bytes, void *stream);
/* height rows of width bytes, rows pitch bytes apart on each side */
int tfft_d2h_2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                size_t height, void *stream);
int tfft_d2d(void *dst, const void *src, size_t bytes, void *stream);
int tfft_stream_create(void **s);
int tfft_stream_destroy(void *s);
int tfft_stream_sync(void *s);
/* later work on stream s waits for event e */
int tfft_stream_wait(void *s, void *e);
int tfft_event_create(void **e);
int tfft_event_destroy(void *e);
int tfft_event_record(void *e, void *stream);
int tfft_event_elapsed_ns(void *start, void *stop, uint64_t *ns);
int tfft_last_launch_error(void);
const char *tfft_error_string(int code);

/* ---- tables --------------------------------------------------------------- */
/* W_L^m = (cospi(2m/L), -sinpi(2m/L)) for m < L; arith selects double2 or
 * the double-float layout (float4: re_hi, re_lo, im_hi, im_lo). */
int tfft_twiddle_table(void *tw, int log_l, int arith, void *stream);
/* four-step factors: lo[m] = W_N^m (m < 2^shift), hi[h] = W_N^(h<<shift) for
 * h < ceil(N / 2^shift); any N */
int tfft_fourstep_tables(void *hi, void *lo, int64_t n, int shift, int arith, void *stream);
/* rev[g] = bit reversal of g over log2n bits, g < 2^log2n */
int tfft_bitrev_table(int *rev, int log2n, void *stream);
/* quarter-wave table of the reference's plan: (cos(2pi k/n), -sin(2pi k/n)),
 * k < n/4, via sincospi */
int tfft_quarter_table(void *tw, int n, void *stream);
/* W_n^m for m < n, any n (DFT path) */
int tfft_dft_table(void *tw, int n, void *stream);
/* W_L^m for m < L, any L, in the layout of arith (mixed-radix passes) */
int tfft_table_any(void *tw, int len, int arith, void *stream);

/* ---- tensor-core form ------------------------------------------------------ */
/* bytes of the table of the six B matrices */
#define TFFT_TC_MATRIX_BYTES 12288
int tfft_tc_matrix(void *dst, void *stream);
/* lines per CTA the tensor form needs for log2 L (its CTAs hold 2^12 points,
 * 2^13 for L = 2^13) */
int tfft_tc_b_tile(int log_l);
/* read (and clear) the device's tensor-form error word: nonzero when a wait
 * for the tensor cores gave up (synchronous on stream) */
int tfft_tc_error(int *flag, void *stream);

/* ---- kernels -------------------------------------------------------------- */
int tfft_launch_pass(const tfft_pass *p, void *stream);
/* can this (log_l, b_tile, arith, points per thread) be launched? */
int tfft_pass_supported(int log_l, int b_tile, int arith, int ept);
/* does that kernel shape stage full contiguous tiles with bulk copies? */
int tfft_pass_bulk_capable(int log_l, int b_tile, int arith, int ept);
/* encode a tiled tensor map of 8-byte elements (rank 2..5, dims and box per
 * dimension, strides in bytes of dimensions 1..rank-1) over base and copy it
 * to dev_map (TFFT_TENSOR_MAP_BYTES of device memory); nonzero when the
 * driver lacks the call or the layout does not fit its rules */
#define TFFT_TENSOR_MAP_BYTES 128
int tfft_tensor_map(void *dev_map, const void *base, int rank, const int64_t *dims,
                    const int64_t *strides, const int *box);
/* can the mixed-radix kernel run lines of len points, b_tile per CTA? */
int tfft_mixed_supported(int len, int b_tile, int arith);
/* out[k] = sum_j in[j] W_n^{jk} (dir 1) or conjugate kernel scaled by 1/n,
 * for `rows` contiguous rows of n points */
int tfft_launch_dft(const void *in, void *out, const void *tw, int n, int dir, int64_t rows,
                    void *stream);
/* in-place bit-reversal permutation of each line of an axis: lines are
 * (g0, g1) with strides s0, s1; element stride es; uses rev[] */
int tfft_launch_bitrev_permute(void *data, const int *rev, int log2n, int64_t es,
                               int64_t n0, int64_t s0, int64_t n1, int64_t s1,
                               void *stream);
/* two-point transform in place (the reference's N == 2 case) */
int tfft_launch_n2(void *data, int dir, void *stream);

/* Bluestein (chirp-z) pieces for a length n that is not a power of two,
 * computed through cyclic convolutions of length m >= 2n-1 (FP64), for
 * `rows` rows (x rows of n points, w rows of m points, back to back):
 *   tables: chirp[k] = exp(-pi i k^2/n), k < n; b = conj(chirp) laid out
 *           cyclically over m points (to be transformed by the caller);
 *   pre:    w = x * chirp zero-padded to m (x conjugated when conj_in);
 *   pointwise: w *= h (h: m points shared by every row);
 *   post:   x = w * chirp, conjugated when conj_out, times scale. */
int tfft_bluestein_tables(void *chirp, void *b, int64_t n, int64_t m, void *stream);
int tfft_bluestein_pre(const void *x, const void *chirp, void *w, int64_t n, int64_t m,
                       int conj_in, int64_t rows, void *stream);
int tfft_pointwise(void *w, const void *h, int64_t m, int64_t rows, void *stream);
int tfft_bluestein_post(const void *w, const void *chirp, void *x, int64_t n, int64_t m,
                        int conj_out, double scale, int64_t rows, void *stream);

/* Real-data transforms of even length n = 2m through a complex transform of
 * length m over the same bytes, in the storage of arith (FP64 for
 * TFFT_ARITH_F64/DF64, FP32 for the split-precision forms, whose tables are
 * (hi, lo) float pairs and whose steps run in double-float):
 *   tables:   lo[i] = W_n^i (i < 2^shift), hi[h] = W_n^(h << shift), h <= m >> shift;
 *   r2c_post: z = FFT_m of the packed reals, row by row (m complex) -> the
 *             m + 1 non-redundant outputs x[0..m] of each row;
 *   c2r_pre:  x[0..m] per row -> z, whose inverse FFT_m is the packed reals. */
int tfft_real_tables(void *hi, void *lo, int64_t n, int shift, int arith, void *stream);
int tfft_r2c_post(const void *z, void *x, const void *hi, const void *lo, int shift, int64_t m,
                  int64_t rows, int arith, void *stream);
int tfft_c2r_pre(const void *x, void *z, const void *hi, const void *lo, int shift, int64_t m,
                 int64_t rows, int arith, void *stream);

#ifdef __cplusplus
}
#endif
#endif
