/* Pass-kernel instantiations: ArithF32, log2 L = 10..14. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithF32, 10, 14, launcher_f32_hi)
