/* Persistent batch kernel instantiation: ArithDF64. */
#include "fft_batch.cuh"

TFFT_BATCH_INSTANTIATE(ArithDF64, batch_df64)
