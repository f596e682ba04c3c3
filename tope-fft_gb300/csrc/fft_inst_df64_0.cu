/* Pass-kernel instantiations: ArithDF64, log2 L = 0..4. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF64, 0, 4, launcher_df64_0)
