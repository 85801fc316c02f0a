// N-d driver of the GB300 pocketfft path: the GPU counterpart of the reference's
// general_nd / general_r2c / general_c2r and the public c2c/r2c/c2r/dct/dst/r2r_* functions
// (rocket_fft/_pocketfft_hdronly.h:3568-4091).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "rg_plan.hpp"

namespace rg {

// Strided view of a device array; strides in elements of the array's own type
// (complex elements for complex arrays, reals for real arrays).
struct NdArray {
  void *data = nullptr;
  std::vector<int64_t> shape, stride;
};

using Axes = std::vector<uint64_t>;

// Two-axis plane kernels on or off (process-wide); returns the previous setting.
int set_plane_kernels(bool on);

void exec_c2c(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool forward,
              double fct, cudaStream_t st);
// bscale: extra scale of the interior half-spectrum bins along the last axis (0 < k < n/2):
// 1 for the transforms themselves, 2 for r2c as the adjoint of c2r, 0.5 for c2r as the
// adjoint of r2c (the Hermitian bin weighting).
void exec_r2c(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool forward,
              double fct, cudaStream_t st, double bscale = 1.0);
void exec_c2r(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool forward,
              double fct, cudaStream_t st, double bscale = 1.0);
void exec_c2c_sym(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool forward,
                  double fct, cudaStream_t st);

// Real-to-real transforms (rg_r2r.cu): DCT (cosine) / DST types 1-4, FFTPACK r2r, Hartley.
// adjoint: the transpose of the transform (DCT/DST-II <-> III with the element-0 weight of the
// transpose; types 1 and 4 are symmetric).
// DCT-II of a C-contiguous float32 n0 x n1 x n2 volume over its three axes (fct 1) whose last
// pass divides by the Neumann eigenvalues lam = lam0 | lam1 | lam2 as it stores (0 at the origin):
// the Poisson solver's DCT-II and eigenvalue divide in one. False (nothing done) when the last
// axis has no compile-time kernel.
bool dct2_eigdiv_3d(const float *in, float *out, int64_t n0, int64_t n1, int64_t n2, const float *lam,
                    cudaStream_t st);
void exec_dcst(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, int type, bool cosine,
               double fct, bool ortho, cudaStream_t st, bool adjoint = false);
void exec_r2r_fftpack(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool real2hermitian,
                      bool forward, double fct, cudaStream_t st);
void exec_hartley(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool genuine, double fct,
                  cudaStream_t st);

// out = in cyclically shifted by shifts[d] along every dimension d (rg_shift.cu); element size
// 1, 2, 4, 8 or 16 bytes; in and out distinct.
void roll(const NdArray &in, const NdArray &out, int64_t itemsize, const std::vector<int64_t> &shifts,
          cudaStream_t st);

// Device workspace from a per-device stream-ordered pool.
class DevBuf {
 public:
  DevBuf(size_t bytes, cudaStream_t st);
  ~DevBuf();
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  void *get() const { return p_; }

 private:
  void *p_ = nullptr;
  cudaStream_t st_;
};
void pool_trim();

}  // namespace rg
