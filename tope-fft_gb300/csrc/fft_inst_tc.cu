/*
 * The tensor form of the split-precision pass (fft_tc.cuh): kernel,
 * launchers for log2 L = 4..13, the table of the six B matrices and the
 * error word.
 */
#include <cuda_runtime.h>

#include "fft_tc.cuh"

namespace tfft {
namespace tc {

/* set by a CTA whose wait for the tensor cores gave up */
__device__ int g_tc_err;

template <int LOG_L>
__global__ void __launch_bounds__(Cfg<LOG_L>::NT, 512 / Cfg<LOG_L>::TCOLS) tc_pass_kernel(const tfft_pass p)
{
    constexpr int B = Cfg<LOG_L>::B;
    constexpr int NT = Cfg<LOG_L>::NT;
    constexpr int NCOL = Cfg<LOG_L>::TCOLS;
    static_assert(Shape<LOG_L>::TPL * B == NT, "one row per thread");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *bsm = smem_raw + Cfg<LOG_L>::TILE_BYTES;
    constexpr int NG = Cfg<LOG_L>::NG;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(bsm + kBBytes); /* one per row group */
    uint32_t *slot = reinterpret_cast<uint32_t *>(bsm + kBBytes + 8 * NG);
    const int t = threadIdx.x;

    /* the six B matrices (12 KB, L2-resident) into shared memory */
    const uint4 *src = reinterpret_cast<const uint4 *>(p.mma_b);
    for (int i = t; i < kBBytes / 16; i += NT) reinterpret_cast<uint4 *>(bsm)[i] = __ldg(src + i);
    if (t < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(slot)),
                     "r"(NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        for (int g = 0; g < NG; g++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar + g)), "r"(1)
                         : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    /* F as written by these threads becomes visible to the tensor cores */
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before();
    __syncthreads();
    fence_after();

    Line line;
    line.cx.tm = *slot;
    line.cx.mbar = smem_u32(mbar);
    line.cx.bsm = smem_u32(bsm);
    line.cx.err = &g_tc_err;
    line.cx.phase = 0;
    line.cx.fail_phase = 0;
    line.cx.dead = 0;
    run_tile<ArithDF32, LOG_L, B, false, Line>(p, blockIdx.x, smem_raw, line);

    /* after a wait that gave up: the MMAs it waited for may still be in
     * flight in any group; give each group's one more bounded wait before
     * the columns are freed */
    if (line.cx.dead)
        for (int g = 0; g < NG; g++) wait_phase(line.cx.mbar + 8u * (uint32_t)g, line.cx.fail_phase);
    fence_before();
    __syncthreads();
    if (t < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(line.cx.tm),
                     "r"(NCOL)
                     : "memory");
}

template <int LOG_L>
int launch(const tfft_pass &p, cudaStream_t s)
{
    constexpr int B = Cfg<LOG_L>::B;
    constexpr size_t smem = Cfg<LOG_L>::SMEM;
    static_assert(smem <= 227 * 1024, "shared memory");
    if (p.b_tile != B || !p.mma_b) return (int)cudaErrorInvalidValue;
    static unsigned attr_done = 0; /* one bit per device ordinal */
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned bit = 1u << (dev & 31);
    if (!(attr_done & bit)) {
        cudaError_t e = cudaFuncSetAttribute(tc_pass_kernel<LOG_L>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
        attr_done |= bit;
    }
    const int64_t blocks = ((p.n[0] + B - 1) / B) * p.n[1] * p.n[2];
    if (blocks <= 0) return 0;
    tc_pass_kernel<LOG_L><<<(unsigned)blocks, Cfg<LOG_L>::NT, smem, s>>>(p);
    return (int)cudaGetLastError();
}

using TcFn = int (*)(const tfft_pass &, cudaStream_t);
static const TcFn g_launch[14] = {nullptr,     nullptr,     nullptr,     nullptr,     &launch<4>,
                                  &launch<5>,  &launch<6>,  &launch<7>,  &launch<8>,  &launch<9>,
                                  &launch<10>, &launch<11>, &launch<12>, &launch<13>};

/* the six B matrices of the tensor stages (fft_tc_split.cuh b_values):
 * F = the real 32x32 DFT-16 (row 2k: re X_k, row 2k+1: im X_k; column 2p:
 * re x_p, column 2p+1: im x_p) from FP64 sincospi, split into integer FP16
 * pieces and scaled; matrix m at m * 2048 bytes in b_offset layout */
__global__ void k_tc_matrix(unsigned short *out)
{
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int n = i >> 5, k = i & 31;
        double s, c;
        sincospi((double)(((n >> 1) * (k >> 1)) & 15) / 8.0, &s, &c);
        double b[kNB];
        tcs::b_values(tcs::dft16_entry(n, k, c, s), b);
#pragma unroll
        for (int m = 0; m < kNB; m++)
            out[m * (kBPieceBytes / 2) + b_offset(n, k) / 2] = __half_as_ushort(__double2half(b[m]));
    }
}

}  // namespace tc

LaunchFn launcher_tc(int log_l)
{
    return (log_l >= 4 && log_l <= 13) ? tc::g_launch[log_l] : nullptr;
}

}  // namespace tfft

extern "C" int tfft_tc_matrix(void *dst, void *stream)
{
    tfft::tc::k_tc_matrix<<<1, 256, 0, (cudaStream_t)stream>>>((unsigned short *)dst);
    return (int)cudaGetLastError();
}

extern "C" int tfft_tc_b_tile(int log_l)
{
    if (log_l < 4 || log_l > 13) return 0;
    return log_l > 12 ? 1 : 1 << (12 - log_l);
}

extern "C" int tfft_tc_error(int *flag, void *stream)
{
    static const int zero = 0;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyFromSymbolAsync(flag, tfft::tc::g_tc_err, sizeof(int), 0,
                                              cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && *flag)
        e = cudaMemcpyToSymbolAsync(tfft::tc::g_tc_err, &zero, sizeof(int), 0,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && *flag) e = cudaStreamSynchronize(s);
    return (int)e;
}
