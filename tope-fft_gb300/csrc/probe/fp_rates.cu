// Throughput probe: DFMA, DADD, FFMA, F64->F32 conversion. Independent chains, no memory in loop.
#include <cstdio>
#include <cuda_runtime.h>
#define ITERS 4096
template <int CH>
__global__ void k_dfma(double *out, double a, double b) {
  double x[CH];
  for (int i = 0; i < CH; i++) x[i] = threadIdx.x * 1e-9 + i;
  for (int it = 0; it < ITERS; it++) {
#pragma unroll
    for (int i = 0; i < CH; i++) x[i] = fma(x[i], a, b);
  }
  double s = 0; for (int i = 0; i < CH; i++) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <int CH>
__global__ void k_ffma(float *out, float a, float b) {
  float x[CH];
  for (int i = 0; i < CH; i++) x[i] = threadIdx.x * 1e-9f + i;
  for (int it = 0; it < ITERS; it++) {
#pragma unroll
    for (int i = 0; i < CH; i++) x[i] = fmaf(x[i], a, b);
  }
  float s = 0; for (int i = 0; i < CH; i++) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <int CH>
__global__ void k_cvt(float *out, double a) {
  double x[CH]; float y[CH];
  for (int i = 0; i < CH; i++) { x[i] = threadIdx.x * 1e-9 + i; y[i] = 0; }
  for (int it = 0; it < ITERS; it++) {
#pragma unroll
    for (int i = 0; i < CH; i++) { y[i] += __double2float_rn(x[i]); }
  }
  float s = 0; for (int i = 0; i < CH; i++) s += y[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
int main() {
  int dev = 0; cudaDeviceProp p; cudaGetDeviceProperties(&p, dev);
  printf("%s SMs=%d cc=%d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
  const int CH = 8, TPB = 256; int blocks = p.multiProcessorCount * 8;
  size_t n = (size_t)blocks * TPB;
  double *od; float *of; cudaMalloc(&od, n * 8); cudaMalloc(&of, n * 4);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1); float ms;
  for (int rep = 0; rep < 2; rep++) {
    cudaEventRecord(e0); k_dfma<CH><<<blocks, TPB>>>(od, 0.999999, 1e-7); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)n * ITERS * CH;
    printf("DFMA: %.3f ms  %.1f Ginstr/s  %.3f TFLOP/s  %.2f instr/clk/SM @2.07GHz\n", ms, ops / ms * 1e-6, 2 * ops / ms * 1e-9, ops / (ms * 1e-3) / p.multiProcessorCount / 2.07e9);
    cudaEventRecord(e0); k_ffma<CH><<<blocks, TPB>>>(of, 0.999999f, 1e-7f); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    printf("FFMA: %.3f ms  %.1f Ginstr/s  %.3f TFLOP/s  %.2f instr/clk/SM @2.07GHz\n", ms, ops / ms * 1e-6, 2 * ops / ms * 1e-9, ops / (ms * 1e-3) / p.multiProcessorCount / 2.07e9);
    cudaEventRecord(e0); k_cvt<CH><<<blocks, TPB>>>(of, 1.0); cudaEventRecord(e1);
    cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    printf("F64->F32 cvt(+FADD): %.3f ms  %.1f Ginstr/s  %.2f instr/clk/SM\n", ms, ops / ms * 1e-6, ops / (ms * 1e-3) / p.multiProcessorCount / 2.07e9);
  }
  cudaError_t err = cudaDeviceSynchronize();
  printf("status: %s\n", cudaGetErrorString(err));
  return err == cudaSuccess ? 0 : 1;
}
