// FP64 throughput probe (rocketgpu_fp64_peak): the denominator of the FP64 roofline of the
// complex128 transforms. Every thread runs kChains independent fused multiply-add chains, so
// the FP64 pipe (not latency) bounds it; grid = 8 CTAs of 256 threads per SM. Timed with CUDA
// events on the caller's stream after one warm-up launch.
#include <cuda_runtime.h>

#include "rg_error.hpp"
#include "rg_launch.hpp"

namespace rg {

namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;

__global__ void __launch_bounds__(256) fp64_fma_kernel(double *out, double seed) {
  double a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = seed + c + threadIdx.x * 1e-6;
  const double b = 1.0 - 1e-9, d = 1e-9;
#pragma unroll 4
  for (int i = 0; i < kIters; ++i)
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = fma(a[c], b, d);
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  if (s == -1.0) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // never true; keeps the chains live
}

}  // namespace

double fp64_peak_gflops(cudaStream_t st) {
  const int grid = sm_count() * 8, threads = 256;
  double *out = nullptr;  // one slot per thread (the store never happens, the buffer is real)
  RG_CUDA(cudaMalloc(&out, sizeof(double) * size_t(grid) * threads));
  cudaEvent_t e0, e1;
  RG_CUDA(cudaEventCreate(&e0));
  RG_CUDA(cudaEventCreate(&e1));
  fp64_fma_kernel<<<grid, threads, 0, st>>>(out, 1.0);
  RG_CUDA(cudaGetLastError());
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    RG_CUDA(cudaEventRecord(e0, st));
    fp64_fma_kernel<<<grid, threads, 0, st>>>(out, 1.0 + rep);
    RG_CUDA(cudaEventRecord(e1, st));
    RG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    RG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  RG_CUDA(cudaFree(out));
  const double flops = 2.0 * kChains * kIters * double(grid) * threads;
  return flops / (double(best) * 1e-3) / 1e9;
}

}  // namespace rg
