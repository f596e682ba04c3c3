/* Pass-kernel instantiations: ArithDF32, log2 L = 5..6. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF32, 5, 6, launcher_df32_1)
