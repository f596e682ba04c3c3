/*
 * Persistent kernel for batches of independent transforms of uneven sizes.
 *
 * The host lists every tile of every pass of every class of same-shaped
 * transforms as a work item, in topological order (all first passes, then
 * all second passes).  A grid of co-resident CTAs of 256 threads takes work
 * items from one atomic counter; a tile whose pass depends on another pass
 * of its class waits until that pass's "tiles done" counter is complete.
 * The wait is bounded: past its spin limit the CTA raises the error flag
 * and every CTA leaves, so the host sees TOPE_ERR_TIMEOUT instead of a hang.
 *
 * Ordering: a finishing tile fences its stores (every thread), meets the
 * others at a barrier, and thread 0 increments the counter; a dependent
 * tile's thread 0 acquires the counter and the tile's loads bypass L1
 * (ld.global.cg), so they see the producer's data at L2.
 */
#pragma once
#include "fft_pass.cuh"

namespace tfft {

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <class A, int LOG_L>
__device__ __forceinline__ void batch_tile(const tfft_pass &p, int64_t tile, unsigned char *sm)
{
    constexpr int B = LOG_L <= 4 ? TFFT_BATCH_THREADS : (TFFT_BATCH_THREADS * 16) >> LOG_L;
    static_assert(Shape<LOG_L>::TPL * B == TFFT_BATCH_THREADS, "256 threads per tile");
    run_tile<A, LOG_L, B, true>(p, tile, sm);
}

template <class A>
__global__ void __launch_bounds__(TFFT_BATCH_THREADS, 2)
    batch_kernel(const tfft_bpass *__restrict__ passes, const tfft_bitem *__restrict__ items,
                 int64_t n_items, int *state, long long spin_limit)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_item;
    __shared__ int s_stop;
    int *head = state, *err = state + 1, *done = state + 2;
    for (;;) {
        if (threadIdx.x == 0) {
            long long it = atomicAdd(head, 1);
            int stop = it >= n_items;
            if (!stop) {
                const int cp = items[it].cp;
                const int dep = passes[cp].dep;
                if (dep >= 0) {
                    const int need = (int)passes[dep].tiles + passes[cp].extra;
                    long long spins = 0;
                    while (ld_acquire(done + dep) < need) {
                        if (++spins > spin_limit || *(volatile int *)err) {
                            atomicExch(err, 1);
                            stop = 1;
                            break;
                        }
                        __nanosleep(100);
                    }
                }
            }
            s_item = it;
            s_stop = stop;
        }
        __syncthreads();
        if (s_stop) break;
        const tfft_bitem w = items[s_item];
        const tfft_pass &p = passes[w.cp].p;
        switch (p.log_l) {
        case 1: batch_tile<A, 1>(p, w.tile, smem_raw); break;
        case 2: batch_tile<A, 2>(p, w.tile, smem_raw); break;
        case 3: batch_tile<A, 3>(p, w.tile, smem_raw); break;
        case 4: batch_tile<A, 4>(p, w.tile, smem_raw); break;
        case 5: batch_tile<A, 5>(p, w.tile, smem_raw); break;
        case 6: batch_tile<A, 6>(p, w.tile, smem_raw); break;
        case 7: batch_tile<A, 7>(p, w.tile, smem_raw); break;
        case 8: batch_tile<A, 8>(p, w.tile, smem_raw); break;
        case 9: batch_tile<A, 9>(p, w.tile, smem_raw); break;
        case 10: batch_tile<A, 10>(p, w.tile, smem_raw); break;
        case 11: batch_tile<A, 11>(p, w.tile, smem_raw); break;
        case 12: batch_tile<A, 12>(p, w.tile, smem_raw); break;
        default: break;
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) atomicAdd(done + w.cp, 1);
    }
}

/* dynamic shared memory of the batch kernel: the largest tile exchange */
template <class A>
constexpr size_t batch_smem_bytes()
{
    return pass_smem_bytes<A, 12, 1>();
}

} // namespace tfft

#define TFFT_BATCH_INSTANTIATE(A, NAME)                                                      \
    namespace tfft {                                                                         \
    int NAME(const tfft_bpass *ps, const tfft_bitem *its, int64_t n, int *st, int ctas,      \
             long long spin_limit, cudaStream_t s, int query_only, int *max_ctas)             \
    {                                                                                        \
        constexpr size_t smem = batch_smem_bytes<A>();                                        \
        auto k = batch_kernel<A>;                                                            \
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                             (int)smem);                                     \
        if (e != cudaSuccess) return (int)e;                                                 \
        if (query_only) {                                                                    \
            int per_sm = 0, dev = 0, sms = 0;                                                \
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, TFFT_BATCH_THREADS, \
                                                              smem);                         \
            if (e != cudaSuccess) return (int)e;                                             \
            cudaGetDevice(&dev);                                                             \
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);               \
            *max_ctas = per_sm * sms;                                                        \
            return 0;                                                                        \
        }                                                                                    \
        k<<<ctas, TFFT_BATCH_THREADS, smem, s>>>(ps, its, n, st, spin_limit);                 \
        return (int)cudaGetLastError();                                                      \
    }                                                                                        \
    }
