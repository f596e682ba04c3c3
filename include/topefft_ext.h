/*
 * topefft_ext.h - extensions of the GB300 FFT library beyond the reference's
 * surface.  None of these has a counterpart in the reference's topefft.h;
 * each is named for what it adds.  Include after topefft.h.
 */
#ifndef TOPEFFT_EXT_H
#define TOPEFFT_EXT_H

#include "topefft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference asserts instead, topefft.h:6) ---------- */
enum topeStatus {
    TOPE_SUCCESS = 0,
    TOPE_ERR_INVALID_SIZE = 1,   /* length not supported (e.g. a 2D/3D side with a
                                    prime factor above 13) */
    TOPE_ERR_INVALID_ARG = 2,    /* NULL pointer, bad direction or type */
    TOPE_ERR_ALLOC = 3,          /* device or host allocation failed */
    TOPE_ERR_CUDA = 4,           /* a CUDA call failed; see topeLastCudaError() */
    TOPE_ERR_NOT_INITIALIZED = 5,/* framework not initialised */
    TOPE_ERR_DESTROYED = 6,      /* plan already destroyed (double destroy, use after destroy) */
    TOPE_ERR_UNSUPPORTED = 7,    /* valid request this build cannot run (e.g. the tensor
                                    form for an uneven batch) */
    TOPE_ERR_TIMEOUT = 8         /* a bounded device-side wait expired */
};

/* Status of the most recent failing call on this thread; reading it resets
 * it to TOPE_SUCCESS (the same contract as cudaGetLastError). */
int topeGetLastError(void);
/* Same, without resetting. */
int topePeekLastError(void);
const char *topeErrorString(int status);
/* CUDA error code behind the last TOPE_ERR_CUDA on this thread. */
int topeLastCudaError(void);

/* ---- arithmetic option --------------------------------------------------- */
/* Storage and I/O are FP64 for both.  TOPE_ARITH_FP64 computes butterflies
 * with double-precision instructions.  TOPE_ARITH_DF64 computes them as
 * FP32 (hi, lo) pairs with error-free transformations on the FP32 pipe
 * (about 2^-44 relative per operation), which on GB300 runs much faster
 * than its FP64 pipe; accuracy is gated by the same rel-L2 <= 1e-13*log2(N)
 * bound.  Applies to plans created after the call. */
enum topeArith { TOPE_ARITH_FP64 = 0, TOPE_ARITH_DF64 = 1 };
void topeSetArith(struct topeFFT *f, int arith);

/* ---- framework lifetime -------------------------------------------------- */
/* Releases the framework's stream.  The reference releases its queue and
 * context inside every Destroy (fft1d.c:385-392); here plans are counted
 * and the stream is released when the last plan goes, or by this call. */
void topeFFTDestroy(struct topeFFT *f);

/* ---- device-resident execution (no host copies) ------------------------- */
/* Transform the plan's device array in place without the read-back of
 * tope*Exec.  Asynchronous on f->command_queue; kernel time is added to
 * totalKernel at the next synchronising call. */
void tope1DExecDevice(struct topeFFT *f, struct topePlan1D *t, int dir);
void tope2DExecDevice(struct topeFFT *f, struct topePlan2D *t, int dir);
void tope3DExecDevice(struct topeFFT *f, struct topePlan3D *t, int dir);
/* Copy host data into / out of the plan's device array (synchronous). */
void tope1DUpload(struct topeFFT *f, struct topePlan1D *t, const double *d);
void tope1DDownload(struct topeFFT *f, struct topePlan1D *t, double *d);
void tope2DUpload(struct topeFFT *f, struct topePlan2D *t, const double *d);
void tope2DDownload(struct topeFFT *f, struct topePlan2D *t, double *d);
void tope3DUpload(struct topeFFT *f, struct topePlan3D *t, const double *d);
void tope3DDownload(struct topeFFT *f, struct topePlan3D *t, double *d);
/* Wait for all work queued on the framework's stream. */
void topeSync(struct topeFFT *f);

/* ---- batched 1D ----------------------------------------------------------- */
/* batch contiguous transforms of length x (row b at d + 2*b*x), any x >= 1
 * (lengths whose prime factors are all at most 13 run as mixed-radix
 * passes; others as an O(x^2) DFT below 128 points and as Bluestein
 * convolutions above).  The plan is a topePlan1D;
 * tope1DExec / tope1DExecDevice / Upload / Download / Destroy apply to all
 * rows.  dataSize = 16*x*batch. */
void tope1DBatchPlanInit(struct topeFFT *f, struct topePlan1D *t, int x, int batch, int type,
                         double *d);

/* ---- real data: type R2C ------------------------------------------------- */
/* topefft.h defines R2C (src/topefft.h:9) but the reference implements only
 * C2C; here tope1DPlanInit / tope1DBatchPlanInit with type R2C and an even
 * length x make a real-data plan (FP64 storage, either arithmetic):
 *   - PlanInit and tope1DUpload take x real doubles per row (row b at d + b*x);
 *   - Exec(FORWARD) transforms the rows and writes the x/2 + 1 non-redundant
 *     outputs X[0..x/2] of each row (e^{-2 pi i jk/x}, unnormalised) as
 *     interleaved complex, row b at d + b*(x + 2): d must hold (x + 2)*batch
 *     doubles;
 *   - Exec(INVERSE) takes that spectrum (the device-resident one, or one
 *     given to tope1DUploadSpectrum) and writes the x real values per row,
 *     scaled by 1/x, so forward then inverse is a round trip;
 *   - tope1DDownload returns the current data: the spectrum after a forward
 *     transform, the real rows otherwise.
 * The complex work is a transform of length x/2 on the packed reals
 * (x[2j] + i x[2j+1]) plus one pre/post pass with W_x^k twiddles. */
void tope1DUploadSpectrum(struct topeFFT *f, struct topePlan1D *t, const double *spec);
/* tope2DPlanInit / tope3DPlanInit with type R2C (x even; x/2, y and z
 * products of 2, 3, 5, 7, 11, 13): x*y(*z) reals in, x fastest;
 * Exec(FORWARD) writes the (x/2 + 1)*y(*z)
 * complex outputs X[kx][ky][kz], kx <= x/2, kx fastest, so d must hold
 * (x + 2)*y(*z) doubles; Exec(INVERSE) returns the reals scaled by
 * 1/(x*y*z).  The rows along x are a batched 1D real-data transform, then
 * y (and z) are complex passes over the spectrum.  tope2DExecX/Y and
 * tope3DExecX/Y/Z reject these plans (TOPE_ERR_UNSUPPORTED). */
void tope2DUploadSpectrum(struct topeFFT *f, struct topePlan2D *t, const double *spec);
void tope3DUploadSpectrum(struct topeFFT *f, struct topePlan3D *t, const double *spec);

/* ---- split-precision form: FP32 complex data ----------------------------- */
/* Same plans and semantics as the FP64 entry points, with interleaved FP32
 * complex data (half the memory traffic), for lengths whose prime factors are
 * all at most 13 (others, the DFT and Bluestein paths, are FP64 only:
 * TOPE_ERR_INVALID_SIZE).  Twiddle factors and the radix-16
 * constants are FP64-accurate (hi, lo) FP32 pairs from FP64 sincospi.
 * Two arithmetics, chosen by topeSetSplitMode before the plan is made:
 *   TOPE_SPLIT_ACCURATE (default): double-float butterflies on chip, so only
 *     the FP32 loads and stores round; rel-L2 <= 1e-7 against an FP64
 *     transform of the unrounded input at 512^3;
 *   TOPE_SPLIT_FAST: FP32 butterflies; about 1e-7 to 1.6e-7 rel-L2 at the
 *     same sizes (an FP32 FFT's own rounding error, ~u*sqrt(log2 N));
 *   TOPE_SPLIT_TENSOR: the radix-16 stages as tensor-core GEMMs on 3-way
 *     BF16 splits with FP32 accumulation (lines up to 2^13 per pass, longer
 *     ones in two or more passes); FP32-level error like TOPE_SPLIT_FAST.  Single
 *     plans only: topeBatchPlanInitF32 rejects it with TOPE_ERR_UNSUPPORTED.
 *     A wait for the tensor cores that gives up is reported by the
 *     synchronous Exec as TOPE_ERR_TIMEOUT.
 * The FP64 Exec/Upload/Download entry points reject these plans (and the
 * F32 ones reject FP64 plans) with TOPE_ERR_INVALID_ARG.  Device-resident
 * execution uses tope*DExecDevice.
 * type = R2C works as for FP64 (x + 2 floats per row of output); the
 * real-data steps around the half-length complex transform run in
 * double-float and round once, in every split mode. */
enum topeSplitMode { TOPE_SPLIT_ACCURATE = 0, TOPE_SPLIT_FAST = 1, TOPE_SPLIT_TENSOR = 2 };
void topeSetSplitMode(struct topeFFT *f, int mode);
void tope1DBatchPlanInitF32(struct topeFFT *f, struct topePlan1D *t, int x, int batch, int type,
                            float *d);
void tope2DPlanInitF32(struct topeFFT *f, struct topePlan2D *t, int x, int y, int type, float *d);
void tope3DPlanInitF32(struct topeFFT *f, struct topePlan3D *t, int x, int y, int z, int type,
                       float *d);
void tope1DExecF32(struct topeFFT *f, struct topePlan1D *t, float *d, int dir);
void tope2DExecF32(struct topeFFT *f, struct topePlan2D *t, float *d, int dir);
void tope3DExecF32(struct topeFFT *f, struct topePlan3D *t, float *d, int dir);
/* impl is the plan's t->impl */
void topeUploadF32(struct topeFFT *f, void *impl, const float *d);
void topeDownloadF32(struct topeFFT *f, void *impl, float *d);
/* the spectrum of an FP32 R2C plan (x/2 + 1 complex floats per row), for an
 * inverse, as tope{1,2,3}DUploadSpectrum */
void topeUploadSpectrumF32(struct topeFFT *f, void *impl, const float *spec);

/* ---- batches of independent transforms of uneven sizes ------------------ */
/* count transforms packed back to back in one buffer, transform i of
 * nx[i] x ny[i] complex points (ny[i] == 1: a 1D transform of length
 * nx[i]; else 2D, x fastest), all powers of two; 1D lengths up to 2^24,
 * 2D sides up to 2^12.  The data stay in the caller's order; transforms of
 * the same shape form a class, and every pass of every class becomes tiles
 * of one work queue.  Execution modes (topeBatchSetMode):
 *   TOPE_BATCH_PERSISTENT: one persistent launch over the whole queue,
 *     replayed from a captured CUDA graph;
 *   TOPE_BATCH_LAUNCHES: one launch per class and pass, captured in a graph;
 *   TOPE_BATCH_LOOP: one launch sequence per transform, as a loop over
 *     single-transform plans would do (the comparison baseline).
 * Autotuning at plan time times candidates on the plan's own buffers: the
 * split of long 1D transforms into two passes (cached per size in the file
 * named by TOPEFFT_TUNE_CACHE, default $HOME/.cache/topefft_tune.txt), the
 * persistent grid size, and the mode (persistent unless the per-class
 * launch graph is at least 5% faster; b->mode reports the choice).
 * TOPEFFT_AUTOTUNE=0 disables tuning (persistent mode, balanced splits). */
enum topeBatchMode { TOPE_BATCH_PERSISTENT = 0, TOPE_BATCH_LAUNCHES = 1, TOPE_BATCH_LOOP = 2 };

struct topeBatch {
    int count;              /* transforms */
    int type;               /* C2C */
    size_t dataSize;        /* bytes of the packed data */
    uint64_t totalMemory;   /* ns: host<->device copies */
    uint64_t totalPreKernel;/* ns: plan-time kernels (tables, tuning) */
    uint64_t totalKernel;   /* ns: execute kernels */
    void *data;             /* device copy of the packed data */
    int mode;               /* TOPE_BATCH_* */
    int elem_bytes;         /* 16 (FP64) or 8 (FP32) */
    int classes;            /* distinct shapes */
    int ctas;               /* persistent grid size chosen */
    int64_t work_items;     /* tiles in the persistent queue */
    void *impl;
};

void topeBatchPlanInit(struct topeFFT *f, struct topeBatch *b, int count, const int *nx,
                       const int *ny, int type, double *d);
void topeBatchPlanInitF32(struct topeFFT *f, struct topeBatch *b, int count, const int *nx,
                          const int *ny, int type, float *d);
/* transform the device copy and read it back into d (d may be NULL) */
void topeBatchExec(struct topeFFT *f, struct topeBatch *b, double *d, int dir);
void topeBatchExecF32(struct topeFFT *f, struct topeBatch *b, float *d, int dir);
/* asynchronous, no read-back */
void topeBatchExecDevice(struct topeFFT *f, struct topeBatch *b, int dir);
/* synchronous copies of the packed data (elem_bytes per complex value) */
void topeBatchUpload(struct topeFFT *f, struct topeBatch *b, const void *d);
void topeBatchDownload(struct topeFFT *f, struct topeBatch *b, void *d);
void topeBatchSetMode(struct topeFFT *f, struct topeBatch *b, int mode);
void topeBatchDestroy(struct topeFFT *f, struct topeBatch *b);

/* ---- tables and permutation (plan internals, exposed for inspection) ---- */
/* Copy a device buffer to host memory (synchronous). */
void topeCopyToHost(struct topeFFT *f, void *dst, const void *device_src, size_t bytes);
/* Apply the bit-reversal permutation of length 2^log2n in place along axis
 * (0 = x, 1 = y, 2 = z) of the plan's device array: the reference's swap
 * pass (kernels3D.cl:574-637), bit for bit. */
void tope3DBitrevPermute(struct topeFFT *f, struct topePlan3D *t, int axis);
/* Pinned host memory, for callers that want fast copies. */
void *topeHostAlloc(size_t bytes);
void topeHostFree(void *p);

/* ---- per-launch kernel timing ------------------------------------------- */
/* When enabled, every pass launch of plans of this framework is bracketed
 * by a CUDA event pair on f->command_queue; durations are folded in at the
 * next synchronising call.  impl is a plan's t->impl. */
void topeSetPassTiming(struct topeFFT *f, int enable);
/* Writes up to max per-pass totals (ns) and launch counts; returns the
 * plan's number of passes.  For a Bluestein plan (a length of 128 points or
 * more with a prime factor above 13) these are the passes of its
 * sub-transforms (run twice per transform), as for topePassInfo; for a 2D or
 * 3D real-data plan, the passes of its rows along x, then its y (and z)
 * passes over the spectrum. */
int topePassTimes(struct topeFFT *f, void *impl, uint64_t *ns, uint64_t *launches, int max);
void topeResetPassTimes(struct topeFFT *f, void *impl);
/* Geometry of pass i of a plan: {log2 L (or -L for a line length L that is
 * not a power of two), lines per CTA, CTAs, threads per CTA, out-of-place,
 * four-step twiddle}; returns 0, or -1 if i is out of range. */
int topePassInfo(struct topeFFT *f, void *impl, int i, int64_t info[6]);

/* ---- allocation-free 1D transform ---------------------------------------- */
/* No counterpart in the reference.  For callers that must not allocate
 * device memory while they run (a host framework that owns the memory pool,
 * a budget fixed at start-up, a path where cudaMalloc's device-wide
 * synchronisation is not acceptable): transforms n complex FP64 values from
 * device buffer d_in to device buffer d_out (they may be the same) on
 * stream, FP64 arithmetic, same direction and scaling rules as tope1DExec.
 * Its scratch (16 MiB) and tables are static device arrays that every GPU
 * loading the library holds until exit; nothing is allocated.  n must be a
 * power of two from 1 to TOPE_NOALLOC_MAX_N, else TOPE_ERR_INVALID_SIZE.
 * The first call on a device builds the tables and waits for the stream:
 * make it before any stream capture.  The tables belong to the device's
 * context as it was at that first call: after cudaDeviceReset the entry
 * point must not be called again in the same process.  All calls share one
 * scratch array, so calls whose kernels may overlap on the GPU race:
 * serialise them.  Returns a topeStatus. */
#define TOPE_NOALLOC_MAX_N (1 << 20)
int topeExec1DNoAlloc(const double *d_in, double *d_out, int n, int dir, void *stream);

#ifdef __cplusplus
}
#endif
#endif
