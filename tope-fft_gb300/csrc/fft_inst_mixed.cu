/* Instantiations of the mixed-radix kernel (fft_mixed.cuh) per arithmetic. */
#include "fft_mixed.cuh"

namespace tfft {

static bool smooth_radices(int len)
{
    for (int r : {2, 3, 5, 7, 11, 13})
        while (len % r == 0) len /= r;
    return len == 1;
}

bool mixed_supported(int len, int b_tile, int arith)
{
    if (len < 2 || b_tile < 1 || (b_tile & (b_tile - 1)) || b_tile > 256) return false;
    if ((int64_t)len * b_tile > TFFT_MIXED_MAX_POINTS || !smooth_radices(len)) return false;
    return arith == TFFT_ARITH_F64 || arith == TFFT_ARITH_DF64 || arith == TFFT_ARITH_F32 ||
           arith == TFFT_ARITH_DF32;
}

int launch_mixed(const tfft_pass &p, cudaStream_t s)
{
    if (!mixed_supported(p.len, p.b_tile, p.arith) || p.nrad < 1 || p.nrad > TFFT_MAX_RADICES)
        return (int)cudaErrorInvalidValue;
    int prod = 1;
    for (int i = 0; i < p.nrad; i++) prod *= p.radix[i];
    if (prod != p.len) return (int)cudaErrorInvalidValue;
    switch (p.arith) {
    case TFFT_ARITH_F64: return launch_mixed_t<ArithF64>(p, s);
    case TFFT_ARITH_DF64: return launch_mixed_t<ArithDF64>(p, s);
    case TFFT_ARITH_F32: return launch_mixed_t<ArithF32>(p, s);
    case TFFT_ARITH_DF32: return launch_mixed_t<ArithDF32>(p, s);
    default: return (int)cudaErrorInvalidValue;
    }
}

} // namespace tfft

extern "C" int tfft_mixed_supported(int len, int b_tile, int arith)
{
    return tfft::mixed_supported(len, b_tile, arith) ? 1 : 0;
}
