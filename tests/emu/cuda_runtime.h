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
#include <cstring>
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
using std::fma;
using std::max;
using std::min;
inline long long min(long long a, long long b) { return a < b ? a : b; }
typedef int cudaError_t;
typedef void *cudaStream_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaFuncAttributeMaxDynamicSharedMemorySize = 8 };
template <class F> inline int cudaFuncSetAttribute(F, int, int) { return 0; }
inline int cudaGetDevice(int *d) { *d = 0; return 0; }
inline int cudaGetLastError() { return 0; }
