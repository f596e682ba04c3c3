/* Pass-kernel instantiations: ArithDF32, log2 L = 9..9. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF32, 9, 9, launcher_df32_3)
