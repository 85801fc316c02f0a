// Bluestein tables built on the device (rg_plan.cpp get_blue): the chirp bk_j = e^{+i pi j^2 / n}
// and the scaled spectrum bkf = FFT_m(b) / m of its zero-padded symmetric extension b
// (b_j = bk_j for j < n, b_{m-j} = bk_j for 0 < j < n, 0 elsewhere), the reference's fftblue
// construction (rocket_fft/_pocketfft_hdronly.h:2744-2793). Everything is computed in double:
// the angle from the exact integer j^2 mod 2n through sincospi, the spectrum by the library's
// own complex128 FFT; each table is rounded once to the plan precision.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "rg_error.hpp"
#include "rg_exec.hpp"
#include "rg_exec_detail.hpp"
#include "rg_plan.hpp"

namespace rg {

namespace {

__global__ void __launch_bounds__(256) chirp_kernel(uint64_t n, uint64_t m, double2 *__restrict__ b, void *bk, int f64) {
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < m; j += uint64_t(gridDim.x) * blockDim.x) {
    // b_j: the chirp at index j (j < n), at index m - j (j > m - n), else 0
    const uint64_t i = j < n ? j : (m - j < n ? m - j : n);
    double2 v = make_double2(0.0, 0.0);
    if (i < n) {
      const uint64_t t = (i * i) % (2 * n);  // i < 2^27: i^2 < 2^54 fits
      double s, c;
      sincospi(double(t) / double(n), &s, &c);
      v = make_double2(c, s);
      if (j < n) {
        if (f64)
          reinterpret_cast<double2 *>(bk)[j] = v;
        else
          reinterpret_cast<float2 *>(bk)[j] = make_float2(float(c), float(s));
      }
    }
    b[j] = v;
  }
}

__global__ void __launch_bounds__(256) round_kernel(uint64_t m, const double2 *__restrict__ src, float2 *__restrict__ dst) {
  for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < m; j += uint64_t(gridDim.x) * blockDim.x)
    dst[j] = make_float2(float(src[j].x), float(src[j].y));
}

}  // namespace

void blue_tables_device(uint64_t n, uint64_t m, DType dt, void *bk, void *bkf) {
  RG_CHECK(n < (uint64_t(1) << 27), RG_ERR_UNSUPPORTED, "Bluestein length too large");
  // a private stream: the tables are complete when this returns, whatever stream the caller uses
  cudaStream_t st;
  RG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  try {
    DevBuf tmp(size_t(m) * sizeof(double2), st);
    double2 *b = static_cast<double2 *>(tmp.get());
    const unsigned grid = unsigned(std::min<uint64_t>(1024, (m + 255) / 256));
    chirp_kernel<<<grid, 256, 0, st>>>(n, m, b, bk, dt == DType::F64 ? 1 : 0);
    RG_CUDA(cudaGetLastError());
    const Side rows = detail::contiguous_rows(1, int64_t(m));
    if (dt == DType::F64) {
      detail::c2c_rows(DType::F64, int64_t(m), b, rows, bkf, rows, 1, false, false, 1.0 / double(m), st);
    } else {
      detail::c2c_rows(DType::F64, int64_t(m), b, rows, b, rows, 1, false, false, 1.0 / double(m), st);
      round_kernel<<<grid, 256, 0, st>>>(m, b, static_cast<float2 *>(bkf));
      RG_CUDA(cudaGetLastError());
    }
    RG_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    cudaStreamDestroy(st);
    throw;
  }
  RG_CUDA(cudaStreamDestroy(st));
}

}  // namespace rg
