/* Persistent batch kernel instantiation: ArithF32. */
#include "fft_batch.cuh"

TFFT_BATCH_INSTANTIATE(ArithF32, batch_f32)
