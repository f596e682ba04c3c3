/* Pass-kernel instantiations: ArithDF32, log2 L = 10..11. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF32, 10, 11, launcher_df32_4)
