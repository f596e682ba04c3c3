/* Test-only stand-in for FFTW 3's public header (FFTW is not installed
 * here).  It declares the part of FFTW 3's published interface that the
 * reference's benchmark drivers (test/1d.c, 2d.c, 3d.c) call for their
 * comparison column, so that those drivers compile unchanged against the
 * library's topefft.h.  fftw_stub.c gives bodies that do nothing; the FFTW
 * column is out of scope. */
#ifndef TOPE_TEST_FFTW3_STUB_H
#define TOPE_TEST_FFTW3_STUB_H
#include <stddef.h>

typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign,
                           unsigned flags);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign,
                           unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#endif
