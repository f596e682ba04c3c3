/* Pass-kernel instantiations: ArithF32, log2 L = 0..9. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithF32, 0, 9, launcher_f32_lo)
