// Host stand-in for the CUDA names the library's kernel headers use, so that
// the kernel source can be compiled with a host C++ compiler and one CTA run
// as one std::thread per CUDA thread (tests/test_kernel_emulation.py).
// __syncthreads is a barrier over the CTA's threads; __reduce_max_sync a
// barrier-based reduction over a warp's threads; __shared__ arrays are static,
// so every thread of the CTA sees the same array.
#pragma once
#include <algorithm>
#include <atomic>
#include <barrier>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>
#define __device__
#define __host__
#define __global__
#define __shared__ static
#define __forceinline__ inline
#define __align__(x) __attribute__((aligned(x)))
#define __launch_bounds__(...)
struct double2 { double x, y; };
struct float2 { float x, y; };
struct float4 { float x, y, z, w; };
inline double2 make_double2(double a, double b) { return {a, b}; }
inline float2 make_float2(float a, float b) { return {a, b}; }
inline float4 make_float4(float a, float b, float c, float d) { return {a, b, c, d}; }
struct uint3v { unsigned x, y, z; };
extern thread_local uint3v threadIdx;
extern uint3v blockIdx;
extern std::barrier<> *g_cta_bar;
extern std::barrier<> *g_warp_bar[32];
extern unsigned g_warp_val[32][32];
inline void __syncthreads() { g_cta_bar->arrive_and_wait(); }
inline unsigned __reduce_max_sync(unsigned mask, unsigned v)
{
    const unsigned w = threadIdx.x / 32, l = threadIdx.x % 32;
    g_warp_val[w][l] = v;
    g_warp_bar[w]->arrive_and_wait();
    unsigned m = 0;
    for (int i = 0; i < 32; i++)
        if ((mask >> i) & 1) m = std::max(m, g_warp_val[w][i]);
    g_warp_bar[w]->arrive_and_wait();
    return m;
}
template <class T> inline T __ldg(const T *p) { return *p; }
template <class T> inline T __ldcs(const T *p) { return *p; }
template <class T> inline T __ldcg(const T *p) { return *p; }
template <class T> inline void __stcs(T *p, T v) { *p = v; }
inline unsigned atomicMax(unsigned *p, unsigned v)
{
    std::atomic_ref<unsigned> a(*p);
    unsigned o = a.load();
    while (o < v && !a.compare_exchange_weak(o, v)) {
    }
    return o;
}
inline int __ffs(int x) { return __builtin_ffs(x); }
inline int atomicAdd(int *p, int v) { return std::atomic_ref<int>(*p).fetch_add(v); }
inline int atomicExch(int *p, int v) { return std::atomic_ref<int>(*p).exchange(v); }
inline void __threadfence() { std::atomic_thread_fence(std::memory_order_seq_cst); }
inline void __nanosleep(unsigned) { std::this_thread::yield(); }
using std::fma;
using std::max;
using std::min;
inline long long min(long long a, long long b) { return a < b ? a : b; }
typedef int cudaError_t;
typedef void *cudaStream_t;
typedef void *cudaEvent_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaFuncAttributeMaxDynamicSharedMemorySize = 8 };
template <class F> inline int cudaFuncSetAttribute(F, int, int) { return 0; }
inline int cudaGetDevice(int *d) { *d = 0; return 0; }
inline int cudaGetLastError() { return 0; }

// ---- the runtime calls of the auxiliary kernels' file (fft_aux.cu), on host
// memory: allocations are malloc, copies memcpy, streams and events tokens,
// and a launch runs every thread of the grid in turn (those kernels use
// neither shared memory nor barriers).
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
extern dim3 blockDim, gridDim;
enum cudaMemcpyKind { cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
enum { cudaStreamNonBlocking = 1 };
inline int cudaSetDevice(int) { return 0; }
inline int cudaGetDeviceCount(int *n) { *n = 1; return 0; }
inline int cudaMalloc(void **p, size_t b) { *p = std::calloc(1, b); return *p ? 0 : 2; }
inline int cudaFree(void *p) { std::free(p); return 0; }
inline int cudaMallocHost(void **p, size_t b) { return cudaMalloc(p, b); }
inline int cudaFreeHost(void *p) { return cudaFree(p); }
inline int cudaMemsetAsync(void *p, int v, size_t b, cudaStream_t);
inline int cudaMemcpyAsync(void *d, const void *s, size_t b, cudaMemcpyKind, cudaStream_t)
{
    std::memmove(d, s, b);
    return 0;
}
inline int cudaMemcpy2DAsync(void *d, size_t dp, const void *s, size_t sp, size_t w, size_t h,
                             cudaMemcpyKind, cudaStream_t)
{
    for (size_t r = 0; r < h; r++) std::memmove((char *)d + r * dp, (const char *)s + r * sp, w);
    return 0;
}
inline int cudaStreamCreateWithFlags(cudaStream_t *s, int) { *s = (void *)1; return 0; }
inline int cudaStreamDestroy(cudaStream_t) { return 0; }
inline int cudaStreamSynchronize(cudaStream_t) { return 0; }
inline int cudaStreamWaitEvent(cudaStream_t, cudaEvent_t, int) { return 0; }
inline int cudaEventCreate(cudaEvent_t *e) { *e = (void *)1; return 0; }
inline int cudaEventDestroy(cudaEvent_t) { return 0; }
inline int cudaEventRecord(cudaEvent_t, cudaStream_t) { return 0; }
inline int cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) { *ms = 0; return 0; }
inline const char *cudaGetErrorString(int) { return "host stand-in"; }
// stream capture: while a capture is open, launches and memsets are recorded
// (their arguments copied) and a launched graph replays them in order
using emu_graph = std::vector<std::function<void()>>;
extern emu_graph *g_capture;
typedef emu_graph *cudaGraph_t;
typedef emu_graph *cudaGraphExec_t;
enum { cudaStreamCaptureModeThreadLocal = 1, cudaDevAttrMultiProcessorCount = 16 };
inline int cudaStreamBeginCapture(cudaStream_t, int)
{
    if (g_capture) return 1;
    g_capture = new emu_graph;
    return 0;
}
inline int cudaStreamEndCapture(cudaStream_t, cudaGraph_t *g)
{
    *g = g_capture;
    g_capture = nullptr;
    return *g ? 0 : 1;
}
inline int cudaGraphInstantiate(cudaGraphExec_t *x, cudaGraph_t g, int)
{
    *x = new emu_graph(*g);
    return 0;
}
inline int cudaMemsetAsync(void *p, int v, size_t b, cudaStream_t)
{
    if (g_capture) g_capture->push_back([p, v, b] { std::memset(p, v, b); });
    else std::memset(p, v, b);
    return 0;
}
inline int cudaGraphDestroy(cudaGraph_t g) { delete g; return 0; }
inline int cudaGraphExecDestroy(cudaGraphExec_t x) { delete x; return 0; }
inline int cudaGraphLaunch(cudaGraphExec_t x, cudaStream_t)
{
    for (auto &f : *x) f();
    return 0;
}
// one CTA at a time: a persistent grid runs as a single CTA, which takes the
// work items in their (topological) order
template <class K> inline int cudaOccupancyMaxActiveBlocksPerMultiprocessor(int *n, K, int, size_t)
{
    *n = 1;
    return 0;
}
inline int cudaDeviceGetAttribute(int *v, int, int) { *v = 1; return 0; }

template <class F> inline void emu_launch_now(dim3 g, dim3 b, F f)
{
    gridDim = g;
    blockDim = b;
    for (unsigned by = 0; by < g.y; by++)
        for (unsigned bx = 0; bx < g.x; bx++)
            for (unsigned tx = 0; tx < b.x; tx++) {
                blockIdx = {bx, by, 0};
                threadIdx = {tx, 0, 0};
                f();
            }
}
// a launch of a kernel that synchronises its CTA: each CTA in turn, all of
// its threads at once (one std::thread each), with the CTA and warp barriers
template <class F> inline void emu_cta_launch_now(dim3 g, dim3 b, F f)
{
    gridDim = g;
    blockDim = b;
    const int threads = (int)b.x;
    for (unsigned bx = 0; bx < g.x; bx++) {
        blockIdx = {bx, 0, 0};
        std::barrier<> cta(threads);
        g_cta_bar = &cta;
        std::barrier<> *warps[32] = {};
        for (int w = 0; w * 32 < threads; w++)
            g_warp_bar[w] = warps[w] = new std::barrier<>(std::min(32, threads - 32 * w));
        std::vector<std::thread> th;
        th.reserve(threads);
        for (int x = 0; x < threads; x++)
            th.emplace_back([&f, x] {
                threadIdx = {(unsigned)x, 0, 0};
                f();
            });
        for (auto &t : th) t.join();
        for (int w = 0; w * 32 < threads; w++) delete warps[w];
    }
}
template <class F> inline void emu_launch(dim3 g, dim3 b, F f)
{
    if (g_capture) g_capture->push_back([g, b, f] { emu_launch_now(g, b, f); });
    else emu_launch_now(g, b, f);
}
template <class F> inline void emu_cta_launch(dim3 g, dim3 b, F f)
{
    if (g_capture) g_capture->push_back([g, b, f] { emu_cta_launch_now(g, b, f); });
    else emu_cta_launch_now(g, b, f);
}
// device math the auxiliary kernels call, written from the definitions
inline void sincospi(double x, double *s, double *c)
{
    const long double a = (long double)x * 3.141592653589793238462643383279502884L;
    *s = (double)sinl(a);
    *c = (double)cosl(a);
}
inline float __double2float_rn(double x) { return (float)x; }
inline unsigned __brev(unsigned v)
{
    unsigned r = 0;
    for (int i = 0; i < 32; i++) r |= ((v >> i) & 1u) << (31 - i);
    return r;
}
