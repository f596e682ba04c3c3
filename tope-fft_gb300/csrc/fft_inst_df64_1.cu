/* Pass-kernel instantiations: ArithDF64, log2 L = 5..6. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF64, 5, 6, launcher_df64_1)
