// The rest of the host build of the library: the stand-in's globals, the
// dynamic shared-memory buffer, and the parts that are not run on the host.
// The tensor form is tcgen05 code and the allocation-free entry point is
// device-symbol code; both report failure, so the plans that need them fail
// with a status.
#include "fft_pass.cuh"
#include "../../include/topefft_ext.h"

thread_local uint3v threadIdx;
uint3v blockIdx;
dim3 blockDim, gridDim;
std::barrier<> *g_cta_bar;
std::barrier<> *g_warp_bar[32];
unsigned g_warp_val[32][32];
emu_graph *g_capture;

namespace tfft {
alignas(128) unsigned char smem_raw[1 << 18];
LaunchFn launcher_tc(int) { return nullptr; }
} // namespace tfft

extern "C" {
int tfft_tc_matrix(void *, void *) { return 0; }
int tfft_tc_b_tile(int log_l)
{
    if (log_l < 4 || log_l > 13) return 0;
    return log_l > 12 ? 1 : 1 << (12 - log_l);
}
int tfft_tc_error(int *flag, void *)
{
    *flag = 0;
    return 0;
}
int topeExec1DNoAlloc(const double *, double *, int, int, void *) { return TOPE_ERR_UNSUPPORTED; }
/* no tensor maps on the host: strided passes load directly */
int tfft_tensor_map(void *, const void *, int, const int64_t *, const int64_t *, const int *)
{
    return 1;
}
}
