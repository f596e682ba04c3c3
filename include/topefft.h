/*
 * topefft.h - drop-in C interface of the GB300 FFT library.
 *
 * Replaces the reference header src/topefft.h (matze/tope-fft) for C callers:
 * the same macros (topefft.h:8-11), the same struct names and caller-visible
 * fields (topefft.h:13-95) and the same void plan/execute/destroy functions
 * (util.c:21, fft1d.c:12/303/372, fft2d.c:136/319/442, fft3d.c:216/474/628),
 * with no OpenCL types: every cl_* member becomes an opaque pointer or a
 * plain integer, and the header now carries prototypes (the reference's did
 * not).  Extensions (status codes, device-resident execution, batched 1D,
 * the double-float arithmetic option) live in topefft_ext.h so this header
 * stays a drop-in.
 *
 * Semantics kept from the reference:
 *   - data is interleaved complex FP64 (re, im), x fastest: element (i,j,k)
 *     is d[2*(k*x*y + j*x + i)];
 *   - PlanInit uploads d to a device-resident array (fft1d.c:358);
 *   - Exec transforms that device array in place and copies the result back
 *     into d (fft2d.c:193); the contents of d at Exec time are not read, so
 *     a forward Exec followed by an inverse Exec is a round trip on the
 *     device copy (test/1d.c:79-82);
 *   - FORWARD is e^{-2 pi i jk/n}, unnormalised; INVERSE uses the conjugate
 *     kernel and divides by the number of points (kernels1D.cl:499-503);
 *   - the 1D two-point case transforms the caller's d directly, as
 *     fft1d.c:16-28 does;
 *   - totalMemory / totalPreKernel / totalKernel accumulate nanoseconds of
 *     copies / plan-time kernels / execute kernels (topefft.h:28-30).
 * Differences, all in the caller's favour: no assert or exit() on errors
 * (the status goes to f->error and topeGetLastError()); non-power-of-two 1D
 * lengths honour the direction (the reference's DFT kernel ignores it); 2D
 * and 3D sides may be products of 2, 3, 5, 7, 11 and 13 (the reference
 * exits on anything but powers of two); axes of length 1 and 2 work;
 * indexing is 64-bit.
 */
/* The guard is not TOPEFFT_H: the reference's own drivers define TOPEFFT_H
 * themselves before they include the header (test/1d.c:14-17), and the
 * reference header has no guard of its own. */
#ifndef TOPEFFT_GB300_DROPIN_H
#define TOPEFFT_GB300_DROPIN_H

#include <assert.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MAX_BINARY_SIZE (0x100000)
#define MAX_SOURCE_SIZE (0x100000)
#define $CHECKERROR assert(f->error == 0);

#define C2C 1
#define R2C 0
#define FORWARD 1
#define INVERSE 0

struct topePlan1D {
    int x;                  /* length */
    int log;                /* butterfly stage count of the reference's radix plan */
    int type;               /* C2C */
    int radix;              /* reference radix rule: 8, 4, 2, or -1 (DFT path) */
    void *kernel;           /* unused (OpenCL kernel handles in the reference) */
    void *kernel_bit;
    void *kernel_swap;
    void *kernel_twid;
    void *kernel_div;
    void *data;             /* device array holding the transform's current data */
    void *bitrev;           /* device int32[x]: bit-reversal table */
    void *twiddle;          /* device double2[x/4]: quarter-wave table */
    void *scratch;          /* device ping-pong buffer (multi-pass plans) */
    size_t dataSize;        /* bytes of data */
    uint64_t totalMemory;   /* ns: host<->device copies */
    uint64_t totalPreKernel;/* ns: plan-time kernels */
    uint64_t totalKernel;   /* ns: execute kernels */
    unsigned int dim;
    size_t *globalSize;     /* unused */
    size_t *localSize;      /* unused */
    void *impl;             /* library-internal plan; NULL once destroyed */
};

struct topePlan2D {
    int x, y;
    int logX, logY;
    int type;
    int radX, radY;
    void *kernelX;
    void *kernelY;
    void *kernel_bit;
    void *kernel_swap;
    void *kernel_twid;
    void *kernel_div;
    void *data;
    void *bitX, *bitY;
    void *twdX, *twdY;
    size_t dataSize;
    uint64_t totalMemory;
    uint64_t totalPreKernel;
    uint64_t totalKernel;
    unsigned int dim;
    size_t *globalSize;
    size_t *localSize;
    void *impl;
};

struct topePlan3D {
    int x, y, z;
    int logX, logY, logZ;
    int type;
    int radX, radY, radZ;
    void *kernelX;
    void *kernelY;
    void *kernelZ;
    void *kernel_bit;
    void *kernel_swap;
    void *kernel_twid;
    void *kernel_div;
    void *data;
    void *bitX, *bitY, *bitZ;
    void *twdX, *twdY, *twdZ;
    size_t dataSize;
    uint64_t totalMemory;
    uint64_t totalPreKernel;
    uint64_t totalKernel;
    unsigned int dim;
    size_t *globalSize;
    size_t *localSize;
    void *impl;
};

struct topeFFT {
    int error;                   /* status of the last call (0 = success) */
    void *event;                 /* last timing event pair */
    void *platform_id;           /* unused */
    void *device;                /* unused */
    void *program1D;             /* unused */
    void *program2D;
    void *program3D;
    void *context;               /* unused */
    void *command_queue;         /* the cudaStream_t every call runs on */
    unsigned int ret_num_platforms;
    unsigned int ret_num_devices;
    int device_ordinal;          /* CUDA device used by this framework */
    int arith;                   /* TOPE_ARITH_* for plans made afterwards */
    int live_plans;
    int pass_timing;             /* per-launch timing on (topeSetPassTiming) */
    int split_mode;              /* TOPE_SPLIT_* for FP32 plans made afterwards */
};

/* util.c:12 - elapsed nanoseconds of an event pair (f->event) */
uint64_t profileThis(void *event);

/* util.c:21 */
void topeFFTInit(struct topeFFT *f);

/* fft1d.c:303, :12, :372 */
void tope1DPlanInit(struct topeFFT *f, struct topePlan1D *t, int x, int type, double *d);
void tope1DExec(struct topeFFT *f, struct topePlan1D *t, double *d, int dir);
void tope1DDestroy(struct topeFFT *f, struct topePlan1D *t);

/* fft2d.c:319, :136, :442; per-axis passes :12 and :74 */
void tope2DPlanInit(struct topeFFT *f, struct topePlan2D *t, int x, int y, int type, double *d);
void tope2DExec(struct topeFFT *f, struct topePlan2D *t, double *d, int dir);
void tope2DExecX(struct topeFFT *f, struct topePlan2D *t);
void tope2DExecY(struct topeFFT *f, struct topePlan2D *t);
void tope2DDestroy(struct topeFFT *f, struct topePlan2D *t);

/* fft3d.c:474, :216, :628; per-axis passes :12, :80, :148 */
void tope3DPlanInit(struct topeFFT *f, struct topePlan3D *t, int x, int y, int z, int type,
                    double *d);
void tope3DExec(struct topeFFT *f, struct topePlan3D *t, double *d, int dir);
void tope3DExecX(struct topeFFT *f, struct topePlan3D *t);
void tope3DExecY(struct topeFFT *f, struct topePlan3D *t);
void tope3DExecZ(struct topeFFT *f, struct topePlan3D *t);
void tope3DDestroy(struct topeFFT *f, struct topePlan3D *t);

#ifdef __cplusplus
}
#endif
#endif
