/* Pass-kernel instantiations: ArithF64, log2 L = 10..13. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithF64, 10, 13, launcher_f64_hi)
