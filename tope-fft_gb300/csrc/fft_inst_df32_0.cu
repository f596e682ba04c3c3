/* Pass-kernel instantiations: ArithDF32, log2 L = 0..4. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithDF32, 0, 4, launcher_df32_0)
