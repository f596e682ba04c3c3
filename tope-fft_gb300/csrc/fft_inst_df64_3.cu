/* Pass-kernel instantiations: ArithDF64, log2 L = 9..9. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF64, 9, 9, launcher_df64_3)
