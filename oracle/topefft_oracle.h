/*
 * CPU oracle for the topeFFT complex-to-complex execute path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the library links or calls this code;
 * only the tests, the smoke check and the CPU-baseline leg of the benchmark
 * load it, and only as the checker.
 *
 * Three independent oracles live here:
 *   1. a restatement of the reference's own algorithm (FP64, the same radix
 *      rule, quarter-wave twiddle table, bit-reversal table, swap pass, DIT
 *      stages and 1/N divide, in the reference's host order);
 *   2. a long-double iterative radix-2 FFT written from the definition;
 *   3. a long-double O(N^2) DFT.
 * plus the SplitMix64 input generator shared by C, CUDA and Python.
 *
 * Data layout everywhere: interleaved complex double (re, im), x fastest.
 */
#ifndef TOPEFFT_ORACLE_H
#define TOPEFFT_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- generator ---------------------------------------------------------- */
uint64_t oracle_splitmix64(uint64_t seed, uint64_t index);
/* uniform[-1,1): complex element e uses stream indices 2e (re) and 2e+1 (im) */
void oracle_fill_uniform(double *d, int64_t n_complex, uint64_t seed);
/* N(0,1) via Box-Muller over the same two stream indices */
void oracle_fill_normal(double *d, int64_t n_complex, uint64_t seed);

/* ---- restatement of the reference algorithm ----------------------------- */
int  oracle_radix(int log2n);                     /* 8, 4 or 2; 0 if log2n<0 */
int  oracle_ilog2(int64_t n);                     /* -1 if n is not 2^k       */
void oracle_twiddle_table(int n, double *tw);     /* n/4 complex entries      */
void oracle_bitrev_table(int log2n, int *rev);    /* 2^log2n int32 entries    */
/* one axis: swap + all DIT stages (no divide) */
void oracle_axis(double *d, int nx, int ny, int nz, int axis, int dir);
/* whole transform in the reference's order: axes X, Y, Z then divide if
 * dir == 0 (INVERSE).  ny = nz = 1 for 1D, nz = 1 for 2D.  Returns 0, or -1
 * for a size the reference cannot plan (non power of two). */
int  oracle_exec(double *d, int nx, int ny, int nz, int dir);
/* the reference's 1D N==2 path: butterfly in place, /2 on inverse */
void oracle_exec_n2(double *d, int dir);
/* the reference's O(N^2) DFT used for non power-of-two 1D lengths; it is
 * always a forward transform, whatever the direction, and writes out[] */
void oracle_dft_ref(const double *d, double *out, int n);

/* ---- independent long-double oracles ------------------------------------ */
/* in place, forward (dir=1) is e^{-2 pi i jk/n}; inverse (dir=0) conjugate
 * kernel scaled by 1/n.  n must be a power of two. */
void oracle_fft_ld(double *d, int64_t n, int dir);
void oracle_fftnd_ld(double *d, int nx, int ny, int nz, int dir);
/* O(n^2), any n; out-of-place */
void oracle_dft_ld(const double *d, double *out, int n, int dir);
/* any n in O(n log n): Bluestein's chirp-z identity over long-double FFTs */
void oracle_bluestein_ld(const double *d, double *out, int64_t n, int dir);

/* ---- metrics ------------------------------------------------------------- */
double oracle_rel_l2(const double *a, const double *ref, int64_t n_doubles);
double oracle_max_abs(const double *a, const double *ref, int64_t n_doubles);

int oracle_num_threads(void);
void oracle_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
