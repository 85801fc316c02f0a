// Kernels of the spectral Poisson solver with Neumann boundaries on a 3-D grid (h = 1), the
// DCT-II/III application of the transform path (rocket-fft's scipy.fft.dctn/idctn of type 2 ->
// numba_dct; rocket_fft/overloads.py:1614-1633):
//
//   A u = f,  (A u)_i = sum over axes of (u_{i+1} - 2 u_i + u_{i-1}) with mirrored ghost cells
//   (u_{-1} = u_0, u_n = u_{n-1}); DCT-II diagonalises A with eigenvalues
//   lambda_k = sum over axes of (2 cos(pi k_a / n_a) - 2); mode 0 (lambda = 0) is set to 0.
//
// rocketgpu_poisson_eigdiv: X_k /= lambda_k in place (DCT-II coefficients, float or double).
// rocketgpu_poisson_update: u_hi + u_lo += delta (exact two-sum, rounding error into u_lo).
// rocketgpu_poisson_residual: r = f - A(u_hi + u_lo) in double, written as float for the next
//   single-precision solve, and sum(r^2).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/rocket_gpu.h"
#include "rg_error.hpp"
#include "rg_launch.hpp"

namespace {

struct Grid {
  int64_t n0, n1, n2;
};

template <typename T>
__global__ void __launch_bounds__(256) eigdiv_kernel(T *X, Grid g, const double *l0, const double *l1,
                                                     const double *l2) {
  const int64_t total = g.n0 * g.n1 * g.n2;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t k2 = i % g.n2, t = i / g.n2, k1 = t % g.n1, k0 = t / g.n1;
    const double lam = l0[k0] + l1[k1] + l2[k2];
    X[i] = i == 0 ? T(0) : T(double(X[i]) / lam);
  }
}

// The solution is carried as an unevaluated sum u_hi + u_lo (u_hi double, u_lo float, u_lo
// optional): corrections are added to u_hi by an exact two-sum whose rounding error goes to u_lo,
// so the iterate keeps more than a double's precision and the residual floor drops well below
// the 1e-12 target (a single double leaves a floor near 1e-12 on a 512^3 grid).
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// r = f - A(u_hi + u_lo): the hi second differences (a - c) + (b - c) are exact for a smooth
// iterate (neighbours within a factor of two, Sterbenz); the lo part only needs float accuracy.
__global__ void __launch_bounds__(256) residual_kernel(const double *uh, const float *ul, const double *f,
                                                       float *r32, Grid g, double *sum) {
  const int64_t total = g.n0 * g.n1 * g.n2;
  const int64_t s0 = g.n1 * g.n2, s1 = g.n2;
  double acc = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t k2 = i % g.n2, t = i / g.n2, k1 = t % g.n1, k0 = t / g.n1;
    // mirrored neighbours (Neumann): an out-of-range neighbour is the cell itself
    const int64_t m0 = k0 > 0 ? i - s0 : i, p0 = k0 + 1 < g.n0 ? i + s0 : i;
    const int64_t m1 = k1 > 0 ? i - s1 : i, p1 = k1 + 1 < g.n1 ? i + s1 : i;
    const int64_t m2 = k2 > 0 ? i - 1 : i, p2 = k2 + 1 < g.n2 ? i + 1 : i;
    const double c = uh[i];
    double Au = ((uh[m0] - c) + (uh[p0] - c)) + ((uh[m1] - c) + (uh[p1] - c)) + ((uh[m2] - c) + (uh[p2] - c));
    if (ul) {
      const float cl = ul[i];
      Au += double(((ul[m0] - cl) + (ul[p0] - cl)) + ((ul[m1] - cl) + (ul[p1] - cl)) + ((ul[m2] - cl) + (ul[p2] - cl)));
    }
    const double r = f[i] - Au;
    if (r32) r32[i] = float(r);
    acc += r * r;
  }
  // block reduction of sum(r^2)
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(sum, red[0]);
}

// u_hi + u_lo += delta: exact two-sum, rounding error into u_lo
__global__ void __launch_bounds__(256) update_kernel(double *uh, float *ul, const float *delta, int64_t total) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    double s, e;
    two_sum(uh[i], double(delta[i]), s, e);
    uh[i] = s;
    if (ul) ul[i] = float(double(ul[i]) + e);
  }
}

thread_local std::string t_err;

template <class F> int guarded(F f) {
  try {
    f();
    t_err.clear();
    return RG_OK;
  } catch (const rg::Error &e) {
    t_err = e.what();
    return e.code;
  } catch (const std::exception &e) {
    t_err = e.what();
    return RG_ERR_INTERNAL;
  }
}

unsigned grid_for(int64_t total) {
  int64_t b = (total + 255) / 256;
  return unsigned(std::min<int64_t>(b, 152 * 16));
}

}  // namespace

// X: C-contiguous n0 x n1 x n2 DCT-II coefficients (itemsize 4 or 8), divided in place by the
// Neumann eigenvalues lam0[k0] + lam1[k1] + lam2[k2] (device tables, lam = lam0|lam1|lam2 with
// lam_a[k] = 2 cos(pi k / n_a) - 2); mode (0,0,0) set to 0.
extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_eigdiv(void *X, int64_t itemsize, int64_t n0,
                                                                              int64_t n1, int64_t n2,
                                                                              const double *lam, void *stream) {
  return guarded([&] {
    RG_CHECK(itemsize == 4 || itemsize == 8, RG_ERR_ARG, "float32 or float64 coefficients required");
    RG_CHECK(n0 > 0 && n1 > 0 && n2 > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Grid g{n0, n1, n2};
    const unsigned b = grid_for(n0 * n1 * n2);
    if (itemsize == 4)
      eigdiv_kernel<float><<<b, 256, 0, st>>>(static_cast<float *>(X), g, lam, lam + n0, lam + n0 + n1);
    else
      eigdiv_kernel<double><<<b, 256, 0, st>>>(static_cast<double *>(X), g, lam, lam + n0, lam + n0 + n1);
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

// u_hi (+ u_lo) += delta by an exact two-sum (u_lo may be NULL: plain addition).
extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_update(double *u, float *u_lo,
                                                                              const float *delta, int64_t total,
                                                                              void *stream) {
  return guarded([&] {
    RG_CHECK(total > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    update_kernel<<<grid_for(total), 256, 0, st>>>(u, u_lo, delta, total);
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

// r = f - A (u + u_lo) (double, Neumann 7-point stencil, u_lo optional); r32 (optional)
// receives r as float. *sumsq (device double) is overwritten with sum(r^2).
extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_residual(
    const double *u, const float *u_lo, const double *f, float *r32, int64_t n0, int64_t n1, int64_t n2,
    double *sumsq, void *stream) {
  return guarded([&] {
    RG_CHECK(n0 > 0 && n1 > 0 && n2 > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RG_CUDA(cudaMemsetAsync(sumsq, 0, sizeof(double), st));
    Grid g{n0, n1, n2};
    residual_kernel<<<grid_for(n0 * n1 * n2), 256, 0, st>>>(u, u_lo, f, r32, g, sumsq);
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) const char *rocketgpu_poisson_last_error(void) {
  return t_err.c_str();
}
