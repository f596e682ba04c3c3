/*
 * CPU oracle for the topeFFT complex-to-complex execute path.
 *
 * TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the benchmark's
 * CPU-baseline leg load this file's shared object as the checker.  The
 * library itself never links it.
 *
 * Citations are to the reference project (matze/tope-fft) by path:line.
 * The restatement follows the reference's algorithm, not its code: the
 * radix-8 butterfly is evaluated as three radix-2 layers, so results agree
 * with the reference's kernels to rounding (about 1e-16 relative), not bit
 * for bit.  Integer work (radix rule, bit reversal, swap) is bit-exact.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (no FMA
 * contraction, so x86 and aarch64 hosts produce identical results).
 */
#include "topefft_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Same literals as the reference kernels (src/kernels1D.cl:3-5). */
#define ORACLE_2PI 6.283185307179586476925286766559
#define ORACLE_R2 0.707106781186547524400844362104

/* ------------------------------------------------------------------------ */
/* SplitMix64 generator, element-addressable                                */
/* ------------------------------------------------------------------------ */
uint64_t oracle_splitmix64(uint64_t seed, uint64_t index)
{
    uint64_t z = seed + (index + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double unit53(uint64_t z) { return (double)(z >> 11) * 0x1.0p-53; }

void oracle_fill_uniform(double *d, int64_t n, uint64_t seed)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < 2 * n; e++)
        d[e] = 2.0 * unit53(oracle_splitmix64(seed, (uint64_t)e)) - 1.0;
}

void oracle_fill_normal(double *d, int64_t n, uint64_t seed)
{
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n; e++) {
        double u1 = unit53(oracle_splitmix64(seed, (uint64_t)(2 * e)));
        double u2 = unit53(oracle_splitmix64(seed, (uint64_t)(2 * e + 1)));
        double r = sqrt(-2.0 * log(1.0 - u1));
        d[2 * e] = r * cos(ORACLE_2PI * u2);
        d[2 * e + 1] = r * sin(ORACLE_2PI * u2);
    }
}

/* ------------------------------------------------------------------------ */
/* Restatement of the reference algorithm                                   */
/* ------------------------------------------------------------------------ */
int oracle_ilog2(int64_t n)
{
    if (n < 1) return -1;
    int l = 0;
    while (((int64_t)1 << l) < n) l++;
    return (((int64_t)1 << l) == n) ? l : -1;
}

/* Radix rule, src/fft1d.c:317-329 (same in src/fft2d.c:335-354 and
 * src/fft3d.c:491-520): 8 if log2n % 3 == 0, else 4 if even, else 2. */
int oracle_radix(int log2n)
{
    if (log2n < 0) return 0;
    if (log2n % 3 == 0) return 8;
    if (log2n % 2 == 0) return 4;
    return 2;
}

/* Quarter-wave table, src/kernels1D.cl:7-13: tw[k] = (cos(2 pi k/n),
 * -sin(2 pi k/n)) for k < n/4, angle formed as (2pi*k)/n in double. */
void oracle_twiddle_table(int n, double *tw)
{
    for (int k = 0; k < n / 4; k++) {
        double a = ORACLE_2PI * (double)k / (double)n;
        tw[2 * k] = cos(a);
        tw[2 * k + 1] = -sin(a);
    }
}

/* Bit reversal of log2n bits, src/kernels1D.cl:526-547 (launched with n/2
 * items at src/fft1d.c:286-300; the upper half is rev(g)+1). */
void oracle_bitrev_table(int log2n, int *rev)
{
    int n = 1 << log2n;
    for (int g = 0; g < n; g++) {
        int r = 0;
        for (int b = 0; b < log2n; b++)
            if (g & (1 << b)) r |= 1 << (log2n - 1 - b);
        rev[g] = r;
    }
}

/* W_n^m (forward) from the quarter table with the quadrant switch of
 * src/kernels1D.cl:62-70; dir == 0 conjugates. */
static inline void quad_twiddle(const double *tw, int n, int m, int dir,
                                double *wr, double *wi)
{
    int red = n / 4;
    int quad = m / red, b = m % red;
    double x = tw[2 * b], y = tw[2 * b + 1];
    switch (quad) {
    case 0: *wr = x; *wi = y; break;
    case 1: *wr = y; *wi = -x; break;
    case 2: *wr = -x; *wi = -y; break;
    default: *wr = -y; *wi = x; break;
    }
    if (dir == 0) *wi = -*wi;
}

static inline int brev_bits(int v, int bits)
{
    int r = 0;
    for (int b = 0; b < bits; b++)
        if (v & (1 << b)) r |= 1 << (bits - 1 - b);
    return r;
}

/* Axis addressing, src/kernels3D.cl:47-68: axis 0 -> BASE row, STRIDE 1;
 * axis 1 -> STRIDE x; axis 2 -> STRIDE x*y. */
static void axis_geometry(int nx, int ny, int nz, int axis, int *n,
                          int64_t *stride, int64_t *lines)
{
    int64_t total = (int64_t)nx * ny * nz;
    if (axis == 0) { *n = nx; *stride = 1; }
    else if (axis == 1) { *n = ny; *stride = nx; }
    else { *n = nz; *stride = (int64_t)nx * ny; }
    *lines = total / *n;
}

static inline int64_t line_base(int nx, int ny, int axis, int64_t line)
{
    if (axis == 0) return line * nx;
    if (axis == 1) {
        int64_t ix = line % nx, iz = line / nx;
        return iz * (int64_t)nx * ny + ix;
    }
    return line;
}

/* One radix-r DIT stage on bit-reversed data (src/kernels1D.cl:15-164 for
 * r=4, :166-420 for r=8, :422-497 for r=2).  Butterfly id -> (y = id/sub,
 * k = id%sub), inputs at k + y*span + i*sub, coefficient c = k*(n/span);
 * input i is twiddled by W_n^{brev_r(i)*c} (skipped when k == 0), then an
 * r-point DFT of bit-reversed inputs gives natural-order outputs. */
static void dit_stage(double *d, int nx, int ny, int nz, int axis, int r,
                      int stage, int dir, const double *tw)
{
    int n;
    int64_t stride, lines;
    axis_geometry(nx, ny, nz, axis, &n, &stride, &lines);
    int lr = (r == 8) ? 3 : (r == 4) ? 2 : 1;
    int64_t span = (int64_t)1 << (lr * stage);
    int64_t sub = span / r;
    int64_t nb = n / r;
    double sgn = dir ? -1.0 : 1.0; /* sign of the exponent's imaginary unit */

#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < lines * nb; t++) {
        int64_t line = t / nb, id = t % nb;
        int64_t base = line_base(nx, ny, axis, line);
        int64_t y = id / sub, k = id % sub;
        int64_t c = k * (n / span);
        double ar[8], ai[8];
        int64_t pos[8];
        for (int i = 0; i < r; i++) {
            pos[i] = base + stride * (k + y * span + i * sub);
            ar[i] = d[2 * pos[i]];
            ai[i] = d[2 * pos[i] + 1];
        }
        if (k != 0) {
            for (int i = 1; i < r; i++) {
                double wr, wi;
                quad_twiddle(tw, n, (int)(brev_bits(i, lr) * c), dir, &wr, &wi);
                double xr = ar[i] * wr - ai[i] * wi;
                double xi = ai[i] * wr + ar[i] * wi;
                ar[i] = xr;
                ai[i] = xi;
            }
        }
        /* r-point DFT on bit-reversed storage: radix-2 DIT layers.  Layer
         * with half-width h multiplies the odd partner at offset j by
         * W_{2h}^j, evaluated exactly for j/2h in {0, 1/4} and through the
         * sqrt(1/2) constant for the eighth-turns. */
        for (int h = 1; h < r; h <<= 1) {
            for (int g = 0; g < r; g += 2 * h) {
                for (int j = 0; j < h; j++) {
                    int p = g + j, q = g + j + h;
                    double br = ar[q], bi = ai[q], tr, ti;
                    int e8 = j * (8 / (2 * h)); /* twiddle in eighths of a turn */
                    switch (e8) {
                    case 0: tr = br; ti = bi; break;
                    case 2: /* multiply by -i (forward) / +i (inverse) */
                        tr = -sgn * bi; ti = sgn * br; break;
                    case 1: /* (1 -+ i)/sqrt2 */
                        if (dir) { tr = (br + bi) * ORACLE_R2; ti = (bi - br) * ORACLE_R2; }
                        else { tr = (br - bi) * ORACLE_R2; ti = (bi + br) * ORACLE_R2; }
                        break;
                    default: /* e8 == 3: (-1 -+ i)/sqrt2 */
                        if (dir) { tr = (bi - br) * ORACLE_R2; ti = -(br + bi) * ORACLE_R2; }
                        else { tr = -(br + bi) * ORACLE_R2; ti = (br - bi) * ORACLE_R2; }
                        break;
                    }
                    ar[q] = ar[p] - tr; ai[q] = ai[p] - ti;
                    ar[p] = ar[p] + tr; ai[p] = ai[p] + ti;
                }
            }
        }
        for (int i = 0; i < r; i++) {
            d[2 * pos[i]] = ar[i];
            d[2 * pos[i] + 1] = ai[i];
        }
    }
}

/* Bit-reversal permutation along one axis, src/kernels3D.cl:574-637:
 * element i swaps with rev[i] when i < rev[i]. */
static void swap_axis(double *d, int nx, int ny, int nz, int axis, const int *rev)
{
    int n;
    int64_t stride, lines;
    axis_geometry(nx, ny, nz, axis, &n, &stride, &lines);
#pragma omp parallel for schedule(static)
    for (int64_t line = 0; line < lines; line++) {
        int64_t base = line_base(nx, ny, axis, line);
        for (int i = 0; i < n; i++) {
            if (i < rev[i]) {
                int64_t a = base + stride * i, b = base + stride * rev[i];
                double tr = d[2 * b], ti = d[2 * b + 1];
                d[2 * b] = d[2 * a];
                d[2 * b + 1] = d[2 * a + 1];
                d[2 * a] = tr;
                d[2 * a + 1] = ti;
            }
        }
    }
}

/* One axis in the reference's order (src/fft3d.c:12-78): swap, then
 * log2n/log2r stages of the planned radix.  Length 1 is the identity; for
 * length 2 (where the reference divides by n/4 == 0) a radix-2 stage. */
void oracle_axis(double *d, int nx, int ny, int nz, int axis, int dir)
{
    int n = axis == 0 ? nx : axis == 1 ? ny : nz;
    int lg = oracle_ilog2(n);
    if (lg <= 0) return;
    int *rev = (int *)malloc(sizeof(int) * n);
    double *tw = (double *)malloc(sizeof(double) * 2 * (n / 4 + 1));
    oracle_bitrev_table(lg, rev);
    oracle_twiddle_table(n, tw);
    swap_axis(d, nx, ny, nz, axis, rev);
    int r = oracle_radix(lg);
    if (n == 2) r = 2;
    int lr = r == 8 ? 3 : r == 4 ? 2 : 1;
    for (int s = 1; s <= lg / lr; s++) dit_stage(d, nx, ny, nz, axis, r, s, dir, tw);
    free(rev);
    free(tw);
}

/* Host order of src/fft3d.c:216-285 (2D: src/fft2d.c:136-199, 1D:
 * src/fft1d.c:12-146): axes X, Y, Z, then divide by the volume for the
 * inverse (src/kernels3D.cl:566-572). */
int oracle_exec(double *d, int nx, int ny, int nz, int dir)
{
    if (oracle_ilog2(nx) < 0 || oracle_ilog2(ny) < 0 || oracle_ilog2(nz) < 0) return -1;
    oracle_axis(d, nx, ny, nz, 0, dir);
    if (ny > 1) oracle_axis(d, nx, ny, nz, 1, dir);
    if (nz > 1) oracle_axis(d, nx, ny, nz, 2, dir);
    if (dir == 0) {
        int64_t total = (int64_t)nx * ny * nz;
        double vol = (double)total;
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < 2 * total; e++) d[e] /= vol;
    }
    return 0;
}

/* src/fft1d.c:16-28 */
void oracle_exec_n2(double *d, int dir)
{
    double hr = d[0], hi = d[1];
    d[0] += d[2];
    d[1] += d[3];
    d[2] = hr - d[2];
    d[3] = hi - d[3];
    if (dir == 0) {
        d[0] /= 2;
        d[2] /= 2;
    }
}

/* src/kernels1D.cl:549-573: out[k] = sum_i d[i] * (cos(2pi k i/n),
 * -sin(2pi k i/n)) with the angle formed left to right as ((2pi*k)*i)/n in
 * double, unreduced.  Forward only. */
void oracle_dft_ref(const double *d, double *out, int n)
{
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; k++) {
        double sr = 0, si = 0;
        for (int i = 0; i < n; i++) {
            double a = ORACLE_2PI * (double)k * (double)i / (double)n;
            double wr = cos(a), wi = -sin(a);
            sr += d[2 * i] * wr - d[2 * i + 1] * wi;
            si += d[2 * i] * wi + d[2 * i + 1] * wr;
        }
        out[2 * k] = sr;
        out[2 * k + 1] = si;
    }
}

/* ------------------------------------------------------------------------ */
/* Long-double oracles (from the DFT definition)                            */
/* ------------------------------------------------------------------------ */
typedef long double ld;

static ld ld_2pi(void) { return 2.0L * acosl(-1.0L); }

/* table[m] = exp(-2 pi i m / n), m < n, angle from the exact ratio m/n */
static void ld_table(int64_t n, ld *tr, ld *ti)
{
    ld tp = ld_2pi();
#pragma omp parallel for schedule(static)
    for (int64_t m = 0; m < n; m++) {
        ld a = tp * ((ld)m / (ld)n);
        tr[m] = cosl(a);
        ti[m] = -sinl(a);
    }
}

static void fft_ld_line(ld *xr, ld *xi, int64_t n, const ld *tr, const ld *ti, int dir)
{
    int lg = oracle_ilog2(n);
    for (int64_t i = 0; i < n; i++) {
        int64_t r = 0;
        for (int b = 0; b < lg; b++)
            if (i & ((int64_t)1 << b)) r |= (int64_t)1 << (lg - 1 - b);
        if (i < r) {
            ld t = xr[i]; xr[i] = xr[r]; xr[r] = t;
            t = xi[i]; xi[i] = xi[r]; xi[r] = t;
        }
    }
    for (int64_t len = 2; len <= n; len <<= 1) {
        int64_t h = len / 2, step = n / len;
        for (int64_t g = 0; g < n; g += len) {
            for (int64_t j = 0; j < h; j++) {
                ld wr = tr[j * step], wi = dir ? ti[j * step] : -ti[j * step];
                ld br = xr[g + j + h] * wr - xi[g + j + h] * wi;
                ld bi = xr[g + j + h] * wi + xi[g + j + h] * wr;
                xr[g + j + h] = xr[g + j] - br;
                xi[g + j + h] = xi[g + j] - bi;
                xr[g + j] += br;
                xi[g + j] += bi;
            }
        }
    }
}

/* unscaled O(n^2) sum for an axis whose length is not a power of two (the
 * same sum as oracle_dft_ld below, on one line; y is scratch) */
static void dft_ld_line(ld *xr, ld *xi, int n, const ld *tr, const ld *ti, int dir, ld *yr,
                        ld *yi)
{
    for (int k = 0; k < n; k++) {
        ld sr = 0, si = 0;
        for (int j = 0; j < n; j++) {
            int64_t m = ((int64_t)j * k) % n;
            ld wr = tr[m], wi = dir ? ti[m] : -ti[m];
            sr += xr[j] * wr - xi[j] * wi;
            si += xr[j] * wi + xi[j] * wr;
        }
        yr[k] = sr;
        yi[k] = si;
    }
    for (int k = 0; k < n; k++) {
        xr[k] = yr[k];
        xi[k] = yi[k];
    }
}

/* every line of one axis: the radix-2 long-double FFT for 2^k points, the
 * O(n^2) sum for other lengths */
static void fft_ld_axis(double *d, int nx, int ny, int nz, int axis, int dir)
{
    int n;
    int64_t stride, lines;
    axis_geometry(nx, ny, nz, axis, &n, &stride, &lines);
    if (n <= 1) return;
    ld *tr = (ld *)malloc(sizeof(ld) * n), *ti = (ld *)malloc(sizeof(ld) * n);
    ld_table(n, tr, ti);
#pragma omp parallel
    {
        ld *xr = (ld *)malloc(sizeof(ld) * n), *xi = (ld *)malloc(sizeof(ld) * n);
        ld *yr = (ld *)malloc(sizeof(ld) * n), *yi = (ld *)malloc(sizeof(ld) * n);
#pragma omp for schedule(static)
        for (int64_t line = 0; line < lines; line++) {
            int64_t base = line_base(nx, ny, axis, line);
            for (int i = 0; i < n; i++) {
                xr[i] = d[2 * (base + stride * i)];
                xi[i] = d[2 * (base + stride * i) + 1];
            }
            if (n & (n - 1)) dft_ld_line(xr, xi, n, tr, ti, dir, yr, yi);
            else fft_ld_line(xr, xi, n, tr, ti, dir);
            ld s = dir ? 1.0L : 1.0L / (ld)n;
            for (int i = 0; i < n; i++) {
                d[2 * (base + stride * i)] = (double)(xr[i] * s);
                d[2 * (base + stride * i) + 1] = (double)(xi[i] * s);
            }
        }
        free(xr);
        free(xi);
        free(yr);
        free(yi);
    }
    free(tr);
    free(ti);
}

/* Note: the per-axis rounding back to double costs one double rounding per
 * axis; for 1D it is a single rounding of the long-double result. */
void oracle_fftnd_ld(double *d, int nx, int ny, int nz, int dir)
{
    fft_ld_axis(d, nx, ny, nz, 0, dir);
    if (ny > 1) fft_ld_axis(d, nx, ny, nz, 1, dir);
    if (nz > 1) fft_ld_axis(d, nx, ny, nz, 2, dir);
}

void oracle_fft_ld(double *d, int64_t n, int dir)
{
    ld *tr = (ld *)malloc(sizeof(ld) * n), *ti = (ld *)malloc(sizeof(ld) * n);
    ld *xr = (ld *)malloc(sizeof(ld) * n), *xi = (ld *)malloc(sizeof(ld) * n);
    ld_table(n, tr, ti);
    for (int64_t i = 0; i < n; i++) { xr[i] = d[2 * i]; xi[i] = d[2 * i + 1]; }
    fft_ld_line(xr, xi, n, tr, ti, dir);
    ld s = dir ? 1.0L : 1.0L / (ld)n;
    for (int64_t i = 0; i < n; i++) {
        d[2 * i] = (double)(xr[i] * s);
        d[2 * i + 1] = (double)(xi[i] * s);
    }
    free(tr); free(ti); free(xr); free(xi);
}

void oracle_dft_ld(const double *d, double *out, int n, int dir)
{
    ld *tr = (ld *)malloc(sizeof(ld) * n), *ti = (ld *)malloc(sizeof(ld) * n);
    ld_table(n, tr, ti);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; k++) {
        ld sr = 0, si = 0;
        for (int j = 0; j < n; j++) {
            int64_t m = ((int64_t)j * k) % n;
            ld wr = tr[m], wi = dir ? ti[m] : -ti[m];
            sr += (ld)d[2 * j] * wr - (ld)d[2 * j + 1] * wi;
            si += (ld)d[2 * j] * wi + (ld)d[2 * j + 1] * wr;
        }
        ld s = dir ? 1.0L : 1.0L / (ld)n;
        out[2 * k] = (double)(sr * s);
        out[2 * k + 1] = (double)(si * s);
    }
    free(tr);
    free(ti);
}

/* Long-double transform of any length n through Bluestein's identity
 * jk = (j^2 + k^2 - (k-j)^2)/2: X[k] = c[k] sum_j (x[j] c[j]) conj(c[k-j]),
 * c[k] = exp(-pi i k^2/n), evaluated as a cyclic convolution of power-of-two
 * length m >= 2n-1 with the long-double FFT above.  Fast enough for lengths
 * where the O(n^2) sum is not; checked against oracle_dft_ld in the tests. */
void oracle_bluestein_ld(const double *d, double *out, int64_t n, int dir)
{
    int64_t m = 1;
    while (m < 2 * n - 1) m <<= 1;
    ld *tr = (ld *)malloc(sizeof(ld) * m), *ti = (ld *)malloc(sizeof(ld) * m);
    ld *cr = (ld *)malloc(sizeof(ld) * n), *ci = (ld *)malloc(sizeof(ld) * n);
    ld *ar = (ld *)calloc(m, sizeof(ld)), *ai = (ld *)calloc(m, sizeof(ld));
    ld *br = (ld *)calloc(m, sizeof(ld)), *bi = (ld *)calloc(m, sizeof(ld));
    ld pi = acosl(-1.0L);
    ld_table(m, tr, ti);
    for (int64_t k = 0; k < n; k++) {
        /* k^2 mod 2n exactly: k < 2^31 */
        uint64_t q = ((uint64_t)k * (uint64_t)k) % (uint64_t)(2 * n);
        ld a = pi * ((ld)q / (ld)n);
        cr[k] = cosl(a);
        ci[k] = dir ? -sinl(a) : sinl(a); /* the inverse uses conj(c) */
    }
    for (int64_t k = 0; k < n; k++) {
        ar[k] = (ld)d[2 * k] * cr[k] - (ld)d[2 * k + 1] * ci[k];
        ai[k] = (ld)d[2 * k] * ci[k] + (ld)d[2 * k + 1] * cr[k];
        br[k] = cr[k];
        bi[k] = -ci[k];
        if (k) {
            br[m - k] = cr[k];
            bi[m - k] = -ci[k];
        }
    }
    fft_ld_line(ar, ai, m, tr, ti, 1);
    fft_ld_line(br, bi, m, tr, ti, 1);
    for (int64_t k = 0; k < m; k++) {
        ld r = ar[k] * br[k] - ai[k] * bi[k];
        ai[k] = ar[k] * bi[k] + ai[k] * br[k];
        ar[k] = r;
    }
    fft_ld_line(ar, ai, m, tr, ti, 0);
    ld s = (dir ? 1.0L : 1.0L / (ld)n) / (ld)m;
    for (int64_t k = 0; k < n; k++) {
        ld r = ar[k] * cr[k] - ai[k] * ci[k];
        ld i = ar[k] * ci[k] + ai[k] * cr[k];
        out[2 * k] = (double)(r * s);
        out[2 * k + 1] = (double)(i * s);
    }
    free(tr); free(ti); free(cr); free(ci);
    free(ar); free(ai); free(br); free(bi);
}

/* ------------------------------------------------------------------------ */
double oracle_rel_l2(const double *a, const double *ref, int64_t nd)
{
    ld num = 0, den = 0;
    for (int64_t i = 0; i < nd; i++) {
        ld e = (ld)a[i] - (ld)ref[i];
        num += e * e;
        den += (ld)ref[i] * (ld)ref[i];
    }
    if (den == 0) return num == 0 ? 0.0 : INFINITY;
    return (double)sqrtl(num / den);
}

double oracle_max_abs(const double *a, const double *ref, int64_t nd)
{
    double m = 0;
    for (int64_t i = 0; i < nd; i++) {
        double e = fabs(a[i] - ref[i]);
        if (e > m || e != e) m = e;
    }
    return m;
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
