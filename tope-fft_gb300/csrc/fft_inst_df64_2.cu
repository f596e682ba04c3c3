/* Pass-kernel instantiations: ArithDF64, log2 L = 7..8. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF64, 7, 8, launcher_df64_2)
