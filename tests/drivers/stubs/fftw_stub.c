/* Bodies for the test-only FFTW stand-in (stubs/fftw3.h): no transform is
 * computed; a plan is NULL. */
#include <stdlib.h>

#include "fftw3.h"

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }
fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{
    (void)n; (void)in; (void)out; (void)sign; (void)flags;
    return NULL;
}
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign,
                           unsigned flags)
{
    (void)n0; (void)n1; (void)in; (void)out; (void)sign; (void)flags;
    return NULL;
}
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign,
                           unsigned flags)
{
    (void)n0; (void)n1; (void)n2; (void)in; (void)out; (void)sign; (void)flags;
    return NULL;
}
void fftw_execute(const fftw_plan p) { (void)p; }
void fftw_destroy_plan(fftw_plan p) { (void)p; }
