/* Persistent batch kernel instantiation: ArithF64. */
#include "fft_batch.cuh"

TFFT_BATCH_INSTANTIATE(ArithF64, batch_f64)
