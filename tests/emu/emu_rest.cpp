// The rest of the host build of the library: the stand-in's globals, the
// dynamic shared-memory buffer, and the parts that are not run on the host.
// The tensor form is tcgen05 code; the persistent batch kernel's CTAs wait on
// one another, which a one-CTA-at-a-time host run cannot do; CUDA graphs have
// no host form; the allocation-free entry point is device-symbol code.  Each
// reports failure, so the plans that need them fail with a status.
#include "fft_pass.cuh"
#include "../../include/topefft_ext.h"

thread_local uint3v threadIdx;
uint3v blockIdx;
dim3 blockDim, gridDim;
std::barrier<> *g_cta_bar;
std::barrier<> *g_warp_bar[32];
unsigned g_warp_val[32][32];

namespace tfft {
alignas(16) unsigned char smem_raw[1 << 18];
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
int tfft_batch_lines_per_tile(int log_l)
{
    if (log_l < 1 || log_l > TFFT_BATCH_MAX_LOG_L) return 0;
    return log_l <= 4 ? TFFT_BATCH_THREADS : (TFFT_BATCH_THREADS * 16) >> log_l;
}
int tfft_batch_max_ctas(int, int *ctas)
{
    *ctas = 152;
    return 0;
}
int tfft_launch_batch(const tfft_bpass *, const tfft_bitem *, int64_t, int *, int, int, int,
                      long long, void *)
{
    return 1;
}
int tfft_batch_graph(void **g, const tfft_bpass *, const tfft_bitem *, int64_t, int *, int, int,
                     int, long long, void *)
{
    *g = nullptr;
    return 1;
}
int tfft_graph_launch(void *, void *) { return 1; }
int tfft_graph_destroy(void *) { return 0; }
int tfft_capture_begin(void *) { return 1; }
int tfft_capture_end(void **g, void *)
{
    *g = nullptr;
    return 1;
}
int topeExec1DNoAlloc(const double *, double *, int, int, void *) { return TOPE_ERR_UNSUPPORTED; }
}
