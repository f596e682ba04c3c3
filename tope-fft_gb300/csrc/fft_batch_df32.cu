/* Persistent batch kernel instantiation: ArithDF32. */
#include "fft_batch.cuh"

TFFT_BATCH_INSTANTIATE(ArithDF32, batch_df32)
