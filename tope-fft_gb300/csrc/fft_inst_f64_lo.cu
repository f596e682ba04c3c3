/* Pass-kernel instantiations: ArithF64, log2 L = 0..9. */
#include "fft_pass.cuh"

TFFT_INSTANTIATE(tfft::ArithF64, 0, 9, launcher_f64_lo)
