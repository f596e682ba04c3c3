/* Pass-kernel instantiations: ArithDF64, log2 L = 10..11. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF64, 10, 11, launcher_df64_4)
