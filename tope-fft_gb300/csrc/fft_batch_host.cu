/*
 * Host side of the persistent batch kernel and of CUDA-graph capture:
 * launch, occupancy query, and the executable graphs that replay a batch
 * (or a sequence of pass launches) with one call.
 */
#include <cuda_runtime.h>

#include "fft_batch.cuh"

namespace tfft {
using BatchFn = int (*)(const tfft_bpass *, const tfft_bitem *, int64_t, int *, int, long long,
                        cudaStream_t, int, int *);
int batch_f64(const tfft_bpass *, const tfft_bitem *, int64_t, int *, int, long long, cudaStream_t,
              int, int *);
int batch_df64(const tfft_bpass *, const tfft_bitem *, int64_t, int *, int, long long, cudaStream_t,
               int, int *);
int batch_df32(const tfft_bpass *, const tfft_bitem *, int64_t, int *, int, long long, cudaStream_t,
               int, int *);
int batch_f32(const tfft_bpass *, const tfft_bitem *, int64_t, int *, int, long long, cudaStream_t,
              int, int *);

static BatchFn batch_fn(int arith)
{
    switch (arith) {
    case TFFT_ARITH_F64: return batch_f64;
    case TFFT_ARITH_DF64: return batch_df64;
    case TFFT_ARITH_DF32: return batch_df32;
    case TFFT_ARITH_F32: return batch_f32;
    default: return nullptr;
    }
}
} // namespace tfft

extern "C" {

int tfft_batch_lines_per_tile(int log_l)
{
    if (log_l < 1 || log_l > TFFT_BATCH_MAX_LOG_L) return 0;
    return log_l <= 4 ? TFFT_BATCH_THREADS : (TFFT_BATCH_THREADS * 16) >> log_l;
}

int tfft_batch_max_ctas(int arith, int *ctas)
{
    tfft::BatchFn fn = tfft::batch_fn(arith);
    if (!fn) return (int)cudaErrorInvalidValue;
    return fn(nullptr, nullptr, 0, nullptr, 0, 0, 0, 1, ctas);
}

int tfft_launch_batch(const tfft_bpass *d_passes, const tfft_bitem *d_items, int64_t n_items,
                      int *d_state, int n_passes, int arith, int ctas, long long spin_limit,
                      void *stream)
{
    tfft::BatchFn fn = tfft::batch_fn(arith);
    if (!fn || ctas < 1) return (int)cudaErrorInvalidValue;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(d_state, 0, sizeof(int) * (size_t)(2 + n_passes), s);
    if (e != cudaSuccess) return (int)e;
    return fn(d_passes, d_items, n_items, d_state, ctas, spin_limit, s, 0, nullptr);
}

int tfft_capture_begin(void *stream)
{
    return (int)cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal);
}

int tfft_capture_end(void **graph_exec, void *stream)
{
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture((cudaStream_t)stream, &g);
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return (int)e;
    }
    cudaGraphExec_t x = nullptr;
    e = cudaGraphInstantiate(&x, g, 0);
    cudaGraphDestroy(g);
    *graph_exec = (void *)x;
    return (int)e;
}

int tfft_batch_graph(void **graph_exec, const tfft_bpass *d_passes, const tfft_bitem *d_items,
                     int64_t n_items, int *d_state, int n_passes, int arith, int ctas,
                     long long spin_limit, void *stream)
{
    *graph_exec = nullptr;
    int rc = tfft_capture_begin(stream);
    if (rc) return rc;
    int launch_rc = tfft_launch_batch(d_passes, d_items, n_items, d_state, n_passes, arith, ctas,
                                      spin_limit, stream);
    void *x = nullptr;
    rc = tfft_capture_end(&x, stream);
    if (launch_rc) {
        if (x) cudaGraphExecDestroy((cudaGraphExec_t)x);
        return launch_rc;
    }
    *graph_exec = x;
    return rc;
}

int tfft_graph_launch(void *graph_exec, void *stream)
{
    return (int)cudaGraphLaunch((cudaGraphExec_t)graph_exec, (cudaStream_t)stream);
}

int tfft_graph_destroy(void *graph_exec)
{
    return graph_exec ? (int)cudaGraphExecDestroy((cudaGraphExec_t)graph_exec) : 0;
}

} /* extern "C" */
