/* Pass-kernel instantiations: ArithDF32, log2 L = 7..8. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF32, 7, 8, launcher_df32_2)
