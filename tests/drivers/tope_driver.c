/*
 * A C caller in the style of the reference's drivers (test/1d.c:61-158,
 * test/2d.c:62-210, test/3d.c:62-220): one input, topeFFTInit, PlanInit,
 * Exec FORWARD, then (unlike the reference, whose inverse is #if 0) Exec
 * INVERSE as a round trip, Destroy, and one result line
 *     log2N  tope_seconds  roundtrip_max_abs_error  checksum
 * Inputs are the reference drivers' own: the ramp i+1 in 1D (test/1d.c:69-71)
 * and sin(2 pi count/N) on the real part in 2D/3D (test/2d.c:75-80).
 * Usage: tope_driver NX [NY [NZ]]   (exit status 1 if the round trip fails)
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "topefft.h"

int main(int argc, char *argv[])
{
    if (argc < 2 || argc > 4) {
        printf("<exec> NX [NY [NZ]]\n");
        return 2;
    }
    int NX = atoi(argv[1]), NY = argc > 2 ? atoi(argv[2]) : 1, NZ = argc > 3 ? atoi(argv[3]) : 1;
    long N = (long)NX * NY * NZ;
    double *data = calloc(2 * N, sizeof(double));
    double *orig = calloc(2 * N, sizeof(double));
    double PI = acos(-1);
    for (long i = 0; i < N; i++)
        data[2 * i] = (argc == 2) ? (double)(i + 1) : sin(2 * PI * i / N);
    for (long i = 0; i < 2 * N; i++) orig[i] = data[i];

    struct topeFFT framework;
    topeFFTInit(&framework);
    if (framework.error) {
        fprintf(stderr, "topeFFTInit failed: %d\n", framework.error);
        return 1;
    }
    double checksum = 0, secs = 0;
    if (argc == 2) {
        struct topePlan1D plan;
        tope1DPlanInit(&framework, &plan, NX, C2C, data);
        tope1DExec(&framework, &plan, data, FORWARD);
        for (long i = 0; i < 2 * N; i++) checksum += fabs(data[i]);
        tope1DExec(&framework, &plan, data, INVERSE);
        secs = 1.0e-9 * (plan.totalKernel + plan.totalPreKernel);
        tope1DDestroy(&framework, &plan);
    } else if (argc == 3) {
        struct topePlan2D plan;
        tope2DPlanInit(&framework, &plan, NX, NY, C2C, data);
        tope2DExec(&framework, &plan, data, FORWARD);
        for (long i = 0; i < 2 * N; i++) checksum += fabs(data[i]);
        tope2DExec(&framework, &plan, data, INVERSE);
        secs = 1.0e-9 * (plan.totalKernel + plan.totalPreKernel);
        tope2DDestroy(&framework, &plan);
    } else {
        struct topePlan3D plan;
        tope3DPlanInit(&framework, &plan, NX, NY, NZ, C2C, data);
        tope3DExec(&framework, &plan, data, FORWARD);
        for (long i = 0; i < 2 * N; i++) checksum += fabs(data[i]);
        tope3DExec(&framework, &plan, data, INVERSE);
        secs = 1.0e-9 * (plan.totalKernel + plan.totalPreKernel);
        tope3DDestroy(&framework, &plan);
    }
    if (framework.error) {
        fprintf(stderr, "topeFFT error %d\n", framework.error);
        return 1;
    }
    double maxerr = 0, maxval = 0;
    for (long i = 0; i < 2 * N; i++) {
        double e = fabs(data[i] - orig[i]);
        if (e > maxerr || e != e) maxerr = e;
        if (fabs(orig[i]) > maxval) maxval = fabs(orig[i]);
    }
    printf("%d\t%f\t%.3e\t%.17g\n", (int)log2((double)N), secs, maxerr, checksum);
    free(data);
    free(orig);
    return maxerr <= 1e-11 * (maxval > 1 ? maxval : 1) ? 0 : 1;
}
