/*
 * A C caller of the whole public surface (topefft.h and topefft_ext.h) in
 * one process: plans of every kind made, run and destroyed on one
 * framework, several alive at once, with the status paths in between.  Built
 * against the host build of the library under AddressSanitizer, LeakSanitizer
 * and UBSan (tests/test_sanitized_library.py), where every device allocation
 * is a host heap block: a kernel access outside its buffer, a host-code
 * overrun, or an allocation that Destroy leaves behind makes the run fail.
 *
 * Each case checks its numbers too: forward outputs of short 1D lines against
 * a direct DFT, and forward-then-inverse round trips everywhere.
 * Prints one line per failed check and "ok <checks>" at the end; exit
 * status 1 on any failure.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "topefft.h"
#include "topefft_ext.h"

static int checks, fails;

#define CHECK(cond, ...)                                                                           \
    do {                                                                                           \
        checks++;                                                                                  \
        if (!(cond)) {                                                                             \
            fails++;                                                                               \
            fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__);                                   \
            fprintf(stderr, __VA_ARGS__);                                                          \
            fputc('\n', stderr);                                                                   \
        }                                                                                          \
    } while (0)

/* uniform [-1, 1) from a 64-bit LCG (Knuth's MMIX constants) */
static void fill(double *d, long n, unsigned long long seed)
{
    for (long i = 0; i < n; i++) {
        seed = seed * 6364136223846793005ull + 1442695040888963407ull;
        d[i] = (double)(seed >> 11) * 0x1p-52 - 1.0;
    }
}

static double max_diff(const double *a, const double *b, long n)
{
    double m = 0;
    for (long i = 0; i < n; i++) {
        double e = fabs(a[i] - b[i]);
        if (e > m || e != e) m = e;
    }
    return m;
}

static double max_diff_f(const float *a, const double *b, long n)
{
    double m = 0;
    for (long i = 0; i < n; i++) {
        double e = fabs((double)a[i] - b[i]);
        if (e > m || e != e) m = e;
    }
    return m;
}

/* forward rows of length n against a direct long-double DFT, max-abs error
 * relative to the largest output */
static double dft_error(const double *in, const double *out, int n, int batch)
{
    const long double tau = 6.283185307179586476925286766559005768L;
    double err = 0, big = 0;
    for (int b = 0; b < batch; b++) {
        const double *x = in + 2L * n * b, *y = out + 2L * n * b;
        for (int k = 0; k < n; k++) {
            long double re = 0, im = 0;
            for (int j = 0; j < n; j++) {
                long double a = -tau * (long double)((long)j * k % n) / n;
                long double c = cosl(a), s = sinl(a);
                re += x[2 * j] * c - x[2 * j + 1] * s;
                im += x[2 * j] * s + x[2 * j + 1] * c;
            }
            double e = fmax(fabs(y[2 * k] - (double)re), fabs(y[2 * k + 1] - (double)im));
            if (e > err || e != e) err = e;
            big = fmax(big, fmax(fabs((double)re), fabs((double)im)));
        }
    }
    return big > 0 ? err / big : err;
}

static void c2c_1d(struct topeFFT *f, int n, int batch)
{
    long m = 2L * n * batch;
    double *x = malloc(m * sizeof *x), *d = malloc(m * sizeof *d);
    fill(x, m, 1000u + n);
    memcpy(d, x, m * sizeof *d);
    struct topePlan1D t;
    if (batch == 1) tope1DPlanInit(f, &t, n, C2C, d);
    else tope1DBatchPlanInit(f, &t, n, batch, C2C, d);
    CHECK(f->error == 0, "1D plan n=%d batch=%d: status %d", n, batch, f->error);
    tope1DExec(f, &t, d, FORWARD);
    CHECK(f->error == 0, "1D forward n=%d: status %d", n, f->error);
    if (n <= 1024) {
        double e = dft_error(x, d, n, batch);
        CHECK(e <= 1e-13, "1D forward n=%d batch=%d: DFT error %.3e", n, batch, e);
    }
    tope1DExec(f, &t, d, INVERSE);
    double e = max_diff(d, x, m);
    CHECK(e <= 1e-12, "1D round trip n=%d batch=%d: %.3e", n, batch, e);
    tope1DDestroy(f, &t);
    CHECK(f->error == 0 && t.impl == NULL, "1D destroy n=%d", n);
    free(x);
    free(d);
}

static void c2c_nd(struct topeFFT *f, int nx, int ny, int nz)
{
    long m = 2L * nx * ny * nz;
    double *x = malloc(m * sizeof *x), *d = malloc(m * sizeof *d);
    fill(x, m, 2000u + nx * 7 + ny * 13 + nz);
    memcpy(d, x, m * sizeof *d);
    if (nz == 1) {
        struct topePlan2D t;
        tope2DPlanInit(f, &t, nx, ny, C2C, d);
        CHECK(f->error == 0, "2D plan %dx%d: status %d", nx, ny, f->error);
        tope2DExec(f, &t, d, FORWARD);
        tope2DExec(f, &t, d, INVERSE);
        tope2DDestroy(f, &t);
    } else {
        struct topePlan3D t;
        tope3DPlanInit(f, &t, nx, ny, nz, C2C, d);
        CHECK(f->error == 0, "3D plan %dx%dx%d: status %d", nx, ny, nz, f->error);
        tope3DExec(f, &t, d, FORWARD);
        tope3DExec(f, &t, d, INVERSE);
        tope3DDestroy(f, &t);
    }
    double e = max_diff(d, x, m);
    CHECK(f->error == 0 && e <= 1e-12, "%dx%dx%d round trip: status %d, %.3e", nx, ny, nz,
          f->error, e);
    free(x);
    free(d);
}

/* real data: rows of x reals in, x/2 + 1 complex per row out, and back */
static void r2c(struct topeFFT *f, int ndim, int nx, int ny, int nz)
{
    long rows = (long)ny * nz, nreal = (long)nx * rows;
    double *x = malloc(nreal * sizeof *x), *d = calloc((nx + 2) * rows, sizeof *d);
    fill(x, nreal, 3000u + nx + ny + nz);
    memcpy(d, x, nreal * sizeof *d);
    if (ndim == 1) {
        struct topePlan1D t;
        tope1DBatchPlanInit(f, &t, nx, (int)rows, R2C, d);
        CHECK(f->error == 0, "1D R2C plan %d x %ld: status %d", nx, rows, f->error);
        tope1DExec(f, &t, d, FORWARD);
        /* X[0] of row 0 is the sum of its reals, imaginary part zero */
        double s = 0;
        for (int i = 0; i < nx; i++) s += x[i];
        CHECK(fabs(d[0] - s) <= 1e-12 * nx && fabs(d[1]) <= 1e-12 * nx,
              "1D R2C DC term %.17g vs %.17g", d[0], s);
        /* the inverse from an uploaded copy of the spectrum */
        double *spec = malloc((nx + 2) * rows * sizeof *spec);
        memcpy(spec, d, (nx + 2) * rows * sizeof *spec);
        tope1DUploadSpectrum(f, &t, spec);
        tope1DExec(f, &t, d, INVERSE);
        free(spec);
        tope1DDestroy(f, &t);
    } else if (ndim == 2) {
        struct topePlan2D t;
        tope2DPlanInit(f, &t, nx, ny, R2C, d);
        CHECK(f->error == 0, "2D R2C plan %dx%d: status %d", nx, ny, f->error);
        /* the pass list: the rows along x, then the y pass over the spectrum,
         * each launched once per direction */
        topeSetPassTiming(f, 1);
        tope2DExec(f, &t, d, FORWARD);
        uint64_t ns[8], launches[8];
        int np = topePassTimes(f, t.impl, ns, launches, 8);
        int64_t info[6] = {0};
        long long last = 0; /* the last pass's line length */
        if (np >= 2 && np <= 8 && topePassInfo(f, t.impl, np - 1, info) == 0)
            last = info[0] < 0 ? -info[0] : (info[0] < 62 ? 1LL << info[0] : 0);
        CHECK(last == ny, "2D R2C pass list: %d passes, last of length %lld", np, last);
        for (int i = 0; i < np && i < 8; i++)
            CHECK(launches[i] == 1, "2D R2C pass %d: %llu launches", i,
                  (unsigned long long)launches[i]);
        topeResetPassTimes(f, t.impl);
        topeSetPassTiming(f, 0);
        tope2DExec(f, &t, d, INVERSE);
        tope2DDestroy(f, &t);
    } else {
        struct topePlan3D t;
        tope3DPlanInit(f, &t, nx, ny, nz, R2C, d);
        CHECK(f->error == 0, "3D R2C plan %dx%dx%d: status %d", nx, ny, nz, f->error);
        tope3DExec(f, &t, d, FORWARD);
        tope3DExec(f, &t, d, INVERSE);
        tope3DDestroy(f, &t);
    }
    double e = max_diff(d, x, nreal);
    CHECK(f->error == 0 && e <= 1e-12, "R2C %dD %dx%dx%d round trip: status %d, %.3e", ndim, nx,
          ny, nz, f->error, e);
    free(x);
    free(d);
}

/* FP32 storage in the split-precision modes, C2C or R2C */
static void split(struct topeFFT *f, int mode, int ndim, int nx, int ny, int nz, int type)
{
    long rows = (long)ny * nz;
    long nin = type == C2C ? 2L * nx * rows : (long)nx * rows;
    long nbuf = type == C2C ? nin : (long)(nx + 2) * rows;
    double *x = malloc(nin * sizeof *x);
    float *d = calloc(nbuf, sizeof *d);
    fill(x, nin, 4000u + mode * 31 + nx + ny);
    for (long i = 0; i < nin; i++) {
        d[i] = (float)x[i];
        x[i] = d[i];
    }
    topeSetSplitMode(f, mode);
    struct topePlan1D t1;
    struct topePlan2D t2;
    struct topePlan3D t3;
    if (ndim == 1) {
        tope1DBatchPlanInitF32(f, &t1, nx, (int)rows, type, d);
        CHECK(f->error == 0, "F32 1D plan: status %d", f->error);
        tope1DExecF32(f, &t1, d, FORWARD);
        tope1DExecF32(f, &t1, d, INVERSE);
        /* the FP64 entry points reject an FP32 plan */
        double *wrong = calloc(2 * nbuf, sizeof *wrong);
        tope1DExec(f, &t1, wrong, FORWARD);
        free(wrong);
        CHECK(f->error == TOPE_ERR_INVALID_ARG, "FP64 exec of an FP32 plan: status %d", f->error);
        f->error = 0;
        tope1DDestroy(f, &t1);
    } else if (ndim == 2) {
        tope2DPlanInitF32(f, &t2, nx, ny, type, d);
        CHECK(f->error == 0, "F32 2D plan: status %d", f->error);
        tope2DExecF32(f, &t2, d, FORWARD);
        tope2DExecF32(f, &t2, d, INVERSE);
        tope2DDestroy(f, &t2);
    } else {
        tope3DPlanInitF32(f, &t3, nx, ny, nz, type, d);
        CHECK(f->error == 0, "F32 3D plan: status %d", f->error);
        tope3DExecF32(f, &t3, d, FORWARD);
        tope3DExecF32(f, &t3, d, INVERSE);
        tope3DDestroy(f, &t3);
    }
    double e = max_diff_f(d, x, nin);
    CHECK(f->error == 0 && e <= 2e-6, "F32 mode %d %dD %dx%dx%d type %d round trip: status %d, %.3e",
          mode, ndim, nx, ny, nz, type, f->error, e);
    topeSetSplitMode(f, TOPE_SPLIT_ACCURATE);
    free(x);
    free(d);
}

/* device-resident execution, explicit copies, pinned host memory, pass
 * timing and geometry */
static void device_resident(struct topeFFT *f)
{
    const int n = 4096;
    double *x = malloc(2 * n * sizeof *x);
    double *h = topeHostAlloc(2 * n * sizeof *h);
    CHECK(h != NULL, "topeHostAlloc");
    fill(x, 2 * n, 5000);
    memcpy(h, x, 2 * n * sizeof *h);
    topeSetPassTiming(f, 1);
    struct topePlan1D t;
    tope1DPlanInit(f, &t, n, C2C, h);
    tope1DUpload(f, &t, h);
    tope1DExecDevice(f, &t, FORWARD);
    tope1DExecDevice(f, &t, INVERSE);
    topeSync(f);
    memset(h, 0, 2 * n * sizeof *h);
    tope1DDownload(f, &t, h);
    double e = max_diff(h, x, 2 * n);
    CHECK(f->error == 0 && e <= 1e-12, "device-resident round trip: status %d, %.3e", f->error, e);
    uint64_t ns[8], launches[8];
    int passes = topePassTimes(f, t.impl, ns, launches, 8);
    CHECK(passes >= 1 && passes <= 8, "pass timing: %d passes", passes);
    for (int i = 0; i < passes && i < 8; i++)
        CHECK(launches[i] == 2, "pass %d: %llu launches for two transforms", i,
              (unsigned long long)launches[i]);
    int64_t info[6];
    CHECK(topePassInfo(f, t.impl, 0, info) == 0 && topePassInfo(f, t.impl, passes, info) == -1,
          "pass info range");
    topeResetPassTimes(f, t.impl);
    topeSetPassTiming(f, 0);
    /* the device copy through topeCopyToHost */
    topeCopyToHost(f, h, t.data, 2 * n * sizeof *h);
    CHECK(f->error == 0 && max_diff(h, x, 2 * n) <= 1e-12, "topeCopyToHost");
    tope1DDestroy(f, &t);
    topeHostFree(h);
    free(x);
}

/* the bit-reversal permutation twice is the identity */
static void bitrev(struct topeFFT *f)
{
    const int nx = 8, ny = 16, nz = 4;
    long m = 2L * nx * ny * nz;
    double *x = malloc(m * sizeof *x), *d = malloc(m * sizeof *d);
    fill(x, m, 6000);
    memcpy(d, x, m * sizeof *d);
    struct topePlan3D t;
    tope3DPlanInit(f, &t, nx, ny, nz, C2C, d);
    for (int axis = 0; axis < 3; axis++) {
        tope3DBitrevPermute(f, &t, axis);
        tope3DBitrevPermute(f, &t, axis);
    }
    tope3DDownload(f, &t, d);
    CHECK(f->error == 0 && max_diff(d, x, m) == 0, "bit reversal twice: status %d", f->error);
    tope3DDestroy(f, &t);
    free(x);
    free(d);
}

/* uneven batches in each execution structure, FP64 and FP32 data (the
 * 2^14-point lines take two passes; a batch class of up to 2^13 points is a
 * single pass, which the host build has only up to 2^8) */
static void uneven(struct topeFFT *f, int fp32)
{
    static const int nx[] = {64, 256, 16, 1 << 14, 64, 32, 8, 128, 2};
    static const int ny[] = {1, 1, 1, 1, 1, 16, 64, 1, 1};
    const int count = 9;
    long pts = 0;
    for (int i = 0; i < count; i++) pts += (long)nx[i] * ny[i];
    double *x = malloc(2 * pts * sizeof *x);
    fill(x, 2 * pts, 7000u + fp32);
    for (int mode = 0; mode < 3; mode++) {
        struct topeBatch b;
        double *d = NULL;
        float *s = NULL;
        if (fp32) {
            s = malloc(2 * pts * sizeof *s);
            for (long i = 0; i < 2 * pts; i++) s[i] = (float)x[i];
            topeBatchPlanInitF32(f, &b, count, nx, ny, C2C, s);
        } else {
            d = malloc(2 * pts * sizeof *d);
            memcpy(d, x, 2 * pts * sizeof *d);
            topeBatchPlanInit(f, &b, count, nx, ny, C2C, d);
        }
        CHECK(f->error == 0 && b.classes == 8, "batch plan: status %d, %d classes", f->error,
              b.classes);
        topeBatchSetMode(f, &b, mode);
        if (fp32) {
            topeBatchExecF32(f, &b, s, FORWARD);
            topeBatchExecF32(f, &b, s, INVERSE);
        } else {
            topeBatchExec(f, &b, d, FORWARD);
            topeBatchExecDevice(f, &b, INVERSE);
            topeBatchDownload(f, &b, d);
        }
        double e = fp32 ? max_diff_f(s, x, 2 * pts) : max_diff(d, x, 2 * pts);
        CHECK(f->error == 0 && e <= (fp32 ? 2e-6 : 1e-12),
              "batch mode %d fp32 %d round trip: status %d, %.3e", mode, fp32, f->error, e);
        topeBatchDestroy(f, &b);
        free(d);
        free(s);
    }
    free(x);
}

/* requests the library refuses leave nothing behind */
static void refusals(struct topeFFT *f)
{
    double d[2 * 64] = {0};
    struct topePlan2D t2;
    tope2DPlanInit(f, &t2, 17, 4, C2C, d);
    CHECK(f->error == TOPE_ERR_INVALID_SIZE, "2D side 17: status %d", f->error);
    f->error = 0;
    struct topePlan1D t1;
    tope1DBatchPlanInit(f, &t1, 7, 2, R2C, d);
    CHECK(f->error == TOPE_ERR_INVALID_SIZE, "odd R2C length: status %d", f->error);
    f->error = 0;
    tope1DPlanInit(f, &t1, 16, C2C, d);
    tope1DExec(f, &t1, d, 5);
    CHECK(f->error == TOPE_ERR_INVALID_ARG, "bad direction: status %d", f->error);
    f->error = 0;
    tope1DDestroy(f, &t1);
    tope1DDestroy(f, &t1);
    CHECK(f->error == TOPE_ERR_DESTROYED, "double destroy: status %d", f->error);
    f->error = 0;
    struct topeBatch b;
    static const int nx[] = {64, 48}, ny[] = {1, 1};
    topeBatchPlanInit(f, &b, 2, nx, ny, C2C, d);
    CHECK(f->error != 0, "uneven batch of a non-power-of-two length accepted");
    f->error = 0;
    topeGetLastError();
}

int main(void)
{
    /* no tuning runs and no tuning cache file */
    setenv("TOPEFFT_AUTOTUNE", "0", 1);
    struct topeFFT f;
    topeFFTInit(&f);
    if (f.error) {
        fprintf(stderr, "topeFFTInit failed: %d\n", f.error);
        return 1;
    }
    for (int arith = 0; arith < 2; arith++) {
        topeSetArith(&f, arith);
        c2c_1d(&f, 2, 1);       /* the two-point host path */
        c2c_1d(&f, 64, 3);      /* one pass */
        c2c_1d(&f, 4096, 1);    /* two power-of-two passes */
        c2c_1d(&f, 1000, 1);    /* mixed radix */
        c2c_1d(&f, 13, 2);      /* exact DFT */
        c2c_1d(&f, 131, 1);     /* Bluestein */
        c2c_nd(&f, 60, 8, 1);
        r2c(&f, 1, 64, 3, 1);
        r2c(&f, 2, 16, 12, 1);
        if (arith == TOPE_ARITH_DF64) continue;
        /* 3D in the native arithmetic only: the host build runs each CTA's
         * 256 threads as threads of its own, so small strided tiles are slow */
        c2c_nd(&f, 6, 4, 5);
        c2c_nd(&f, 2, 1, 4);
        r2c(&f, 3, 8, 4, 3);
    }
    topeSetArith(&f, TOPE_ARITH_FP64);
    /* several plans alive at once, destroyed out of order */
    {
        double a[2 * 256], b[2 * 100], c[2 * 8 * 8];
        fill(a, 2 * 256, 1);
        fill(b, 2 * 100, 2);
        fill(c, 2 * 64, 3);
        struct topePlan1D pa, pb;
        struct topePlan2D pc;
        tope1DPlanInit(&f, &pa, 256, C2C, a);
        tope1DPlanInit(&f, &pb, 100, C2C, b);
        tope2DPlanInit(&f, &pc, 8, 8, C2C, c);
        tope1DDestroy(&f, &pb);
        tope1DExec(&f, &pa, a, FORWARD);
        tope2DExec(&f, &pc, c, FORWARD);
        tope1DDestroy(&f, &pa);
        tope2DDestroy(&f, &pc);
        CHECK(f.error == 0, "plans out of order: status %d", f.error);
    }
    split(&f, TOPE_SPLIT_ACCURATE, 1, 256, 4, 1, C2C);
    split(&f, TOPE_SPLIT_FAST, 1, 4096, 1, 1, C2C);
    split(&f, TOPE_SPLIT_ACCURATE, 2, 32, 16, 1, C2C);
    split(&f, TOPE_SPLIT_FAST, 3, 4, 2, 6, C2C);
    split(&f, TOPE_SPLIT_ACCURATE, 1, 64, 2, 1, R2C);
    split(&f, TOPE_SPLIT_ACCURATE, 3, 8, 4, 4, R2C);
    device_resident(&f);
    bitrev(&f);
    uneven(&f, 0);
    uneven(&f, 1);
    refusals(&f);
    topeFFTDestroy(&f);
    printf("ok %d\n", checks);
    if (fails) fprintf(stderr, "%d of %d checks failed\n", fails, checks);
    return fails ? 1 : 0;
}
