/* Pass-kernel instantiations: ArithDF32, log2 L = 12..13. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF32, 12, 13, launcher_df32_5)
