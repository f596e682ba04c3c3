/*
 * Helpers shared between the C translation units of the library (hidden
 * visibility: not exported from libtopefft.so).
 */
#ifndef TOPEFFT_INTERNAL_H
#define TOPEFFT_INTERNAL_H
#include "../../include/topefft.h"

#define TOPE_INTERNAL __attribute__((visibility("hidden")))

/* record st in f->error and the thread's last error; returns st */
TOPE_INTERNAL int tope_status(struct topeFFT *f, int st);
/* map a CUDA return code (0 = success) to a status */
TOPE_INTERNAL int tope_cuda_status(struct topeFFT *f, int rc);
/* make sure f has its stream (re-opening it after the last plan went) */
TOPE_INTERNAL int tope_framework_ready(struct topeFFT *f);
TOPE_INTERNAL void tope_framework_plan_added(struct topeFFT *f);
TOPE_INTERNAL void tope_framework_plan_removed(struct topeFFT *f);

#endif
