/* Pass-kernel instantiations: ArithDF64, log2 L = 12..13. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF64, 12, 13, launcher_df64_5)
