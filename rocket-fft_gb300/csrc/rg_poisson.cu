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
// rocketgpu_poisson_residual: r = f - A(u_hi + u_lo) (the u_hi stencil in double), written as
//   float for the next single-precision solve, and sum(r^2).
// GB300 executes FP64 at a small fraction of its FP32 rate, so each kernel keeps in double only
// what the 1e-12 target needs: the exact u_hi differences and their sum, and u_hi itself.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/rocket_gpu.h"
#include "rg_common.cuh"
#include "rg_error.hpp"
#include "rg_exec.hpp"
#include "rg_launch.hpp"

namespace {

struct Grid {
  int64_t n0, n1, n2;
};

// Elementwise kernels walk their arrays in grid-stride steps of kIlp elements per thread (at
// i, i + stride, ...), all loads of a step issued before any use: with one load in flight per
// thread the conversions ran at 0.26-0.6 of the HBM copy bandwidth (latency-bound).
constexpr int kIlp = 4;

// Row sweep of the n0 x n1 x n2 grid (C order) for the elementwise and stencil kernels: a few
// CTAs per SM; at step t CTA b takes the ROWS rows (k0, k1) number t * G * ROWS + u * G + b
// (u < ROWS, G = gridDim.x), its threads run along the last axis, and the loads of all ROWS rows
// are issued before any use. All CTAs move through the volume together, a window of G * ROWS
// rows (a few planes), so a stencil's neighbours one plane away are recent L2 lines.
// Row number u of step t for this CTA, and its (k0, k1).
__device__ __forceinline__ int64_t sweep_row(int64_t t, int u, int rows_per_step) {
  return (t * rows_per_step + u) * int64_t(gridDim.x) + blockIdx.x;
}

// Grid of the stencil-shaped kernels: x = positions along the last axis (blockDim.x threads
// each), y = index along the middle axis, z = index along the first axis; no divisions.
// X /= lambda in X's own precision: the float32 spectral solve of the mixed-precision
// refinement only needs float accuracy, and GB300's FP64 rate would otherwise bound it (the
// eigenvalues are all <= 0, so their sum has no cancellation).
// V consecutive elements of a row per thread as one vector load/store (V = 16 / sizeof(T) when
// the rows allow it, else 1), ROWS rows per step: enough bytes in flight per SM for the copy
// bandwidth (an elementwise pass carries no reuse to hide latency with).
template <typename T, int V> struct Vec;
template <> struct Vec<float, 4> { using type = float4; };
template <> struct Vec<double, 2> { using type = double2; };

template <typename T, int V>
__global__ void __launch_bounds__(256, 4) eigdiv_kernel(T *X, Grid g, const T *l0, const T *l1, const T *l2) {
  constexpr int ROWS = V == 1 ? 8 : 4;
  const int64_t rows = g.n0 * g.n1;
  for (int64_t t = 0; t * gridDim.x * ROWS < rows; ++t) {
    T *base[ROWS];
    T lam01[ROWS];
#pragma unroll
    for (int u = 0; u < ROWS; ++u) {
      const int64_t row = sweep_row(t, u, ROWS);
      base[u] = row < rows ? X + row * g.n2 : nullptr;
      if (row < rows) {
        const int64_t k0 = row / g.n1;
        lam01[u] = l0[k0] + l1[row - k0 * g.n1];
      }
    }
    for (int64_t k2 = int64_t(threadIdx.x) * V; k2 < g.n2; k2 += int64_t(blockDim.x) * V) {
      T l2k[V];
#pragma unroll
      for (int v = 0; v < V; ++v) l2k[v] = l2[k2 + v];
      if constexpr (V == 1) {
        T x[ROWS];
#pragma unroll
        for (int u = 0; u < ROWS; ++u)
          if (base[u]) x[u] = base[u][k2];
#pragma unroll
        for (int u = 0; u < ROWS; ++u)
          if (base[u]) base[u][k2] = (base[u] == X && k2 == 0) ? T(0) : rg::eig_div<T>(x[u], lam01[u] + l2k[0]);
      } else {
        using VT = typename Vec<T, V>::type;
        VT x[ROWS];
#pragma unroll
        for (int u = 0; u < ROWS; ++u)
          if (base[u]) x[u] = *reinterpret_cast<const VT *>(base[u] + k2);
#pragma unroll
        for (int u = 0; u < ROWS; ++u) {
          if (base[u]) {
            T *e = reinterpret_cast<T *>(&x[u]);
#pragma unroll
            for (int v = 0; v < V; ++v) e[v] = rg::eig_div<T>(e[v], lam01[u] + l2k[v]);
            if (base[u] == X && k2 == 0) e[0] = T(0);
            *reinterpret_cast<VT *>(base[u] + k2) = x[u];
          }
        }
      }
    }
  }
}

// r = f - A(u_hi + u_lo): the hi second differences (a - c) + (b - c) are exact for a smooth
// iterate (neighbours within a factor of two, Sterbenz); the lo part only needs float accuracy.
// Neighbours come from L1/L2: a block row's planes above and below are recently read rows.
__global__ void __launch_bounds__(256) residual_kernel(const double *uh, const float *ul, const double *f,
                                                       float *r32, Grid g, double *sum) {
  const int64_t k2 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t k1 = blockIdx.y, k0 = blockIdx.z;
  const int64_t s0 = g.n1 * g.n2, s1 = g.n2;
  double acc = 0.0;
  if (k2 < g.n2) {
    const int64_t i = k0 * s0 + k1 * s1 + k2;
    // mirrored neighbours (Neumann): an out-of-range neighbour is the cell itself
    const int64_t m0 = k0 > 0 ? i - s0 : i, p0 = k0 + 1 < g.n0 ? i + s0 : i;
    const int64_t m1 = k1 > 0 ? i - s1 : i, p1 = k1 + 1 < g.n1 ? i + s1 : i;
    const int64_t m2 = k2 > 0 ? i - 1 : i, p2 = k2 + 1 < g.n2 ? i + 1 : i;
    const double c = uh[i];
    const double Au = ((uh[m0] - c) + (uh[p0] - c)) + ((uh[m1] - c) + (uh[p1] - c)) + ((uh[m2] - c) + (uh[p2] - c));
    // r = (f - A u_hi) - A u_lo: the second term is a small correction, float is enough for it
    // and for the float32 copy of r
    float r = float(f[i] - Au);
    if (ul) {
      const float cl = ul[i];
      r -= ((ul[m0] - cl) + (ul[p0] - cl)) + ((ul[m1] - cl) + (ul[p1] - cl)) + ((ul[m2] - cl) + (ul[p2] - cl));
    }
    if (r32) r32[i] = r;
    acc = double(r) * double(r);  // squared in double: no overflow for large right-hand sides
  }
  // block reduction of sum(r^2): warp shuffles, then one value per warp
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) t += red[w];
    atomicAdd(sum, t);
  }
}

// The solution is carried as an unevaluated sum u_hi + u_lo (u_hi double, u_lo float, u_lo
// optional): corrections are added to u_hi by an exact two-sum whose rounding error goes to u_lo,
// so the iterate keeps more than a double's precision and the residual floor drops well below
// the 1e-12 target (a single double leaves a floor near 1e-12 on a 512^3 grid).
// u_hi + u_lo += delta: exact sum in double (Dekker's fast two-sum on the operands ordered by
// magnitude, three double operations), rounding error added to u_lo in float
__global__ void __launch_bounds__(256) update_kernel(double *uh, float *ul, const float *delta, int64_t total) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    const double a = uh[i], b = double(delta[i]);
    const double s = a + b;
    const bool big_a = fabs(a) >= fabs(b);
    const double e = big_a ? b - (s - a) : a - (s - b);
    uh[i] = s;
    if (ul) ul[i] += float(e);
  }
}

// ---- fixed-point iterate --------------------------------------------------------------------
// u = U * 2^-e with U int64: the 7-point differences and their sum are exact integer arithmetic
// (GB300 runs int64 adds on its integer pipes and FP64 at about one operation per clock per SM),
// and only f - A u is formed in double. e is chosen from the first correction so that
// |U| < 2^62, which keeps 2^-e at about 2^-60 of max|u| -- the residual floor this leaves is
// well below the 1e-12 target.

// U += round(delta * 2^e) (assign: U = round(delta * 2^e), the first correction)
__global__ void __launch_bounds__(256) fx_update_kernel(long long *U, const float *delta, int64_t total, int e,
                                                        int assign) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i0 < total; i0 += kIlp * stride) {
    float d[kIlp];
    long long u[kIlp];
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      d[q] = i < total ? delta[i] : 0.f;
      u[q] = i < total && !assign ? U[i] : 0;
    }
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      if (i < total) U[i] = u[q] + __float2ll_rn(ldexpf(d[q], e));
    }
  }
}

// Float of an int64 through the two 32-bit halves of its magnitude (32-bit conversions, no
// FP64; splitting the magnitude rather than the two's-complement value avoids cancellation for
// small negative values): exact for |v| < 2^24, within one rounding of float otherwise.
__device__ __forceinline__ float ll_to_float(long long v) {
  const unsigned long long m = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const unsigned hi = unsigned(m >> 32), lo = unsigned(m & 0xffffffffull);
  const float a = hi ? fmaf(float(hi), 4294967296.0f, float(lo)) : float(lo);
  return v < 0 ? -a : a;
}

// R = F - A U exact in int64 (F = f on the iterate's fixed-point scale), r = R 2^-e + Frem
// written as float; sum(r^2) accumulated as sum((r 2^-k)^2) 2^2k, k from max |f|, so that float
// squares neither overflow nor underflow.
__global__ void __launch_bounds__(256) fx_residual_kernel(const long long *U, const long long *F, const float *Frem,
                                                          float *r32, Grid g, int e, int k, double *sum) {
  const int64_t k2 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t k1 = blockIdx.y, k0 = blockIdx.z;
  const int64_t s0 = g.n1 * g.n2, s1 = g.n2;
  float acc = 0.f;
  if (k2 < g.n2) {
    const int64_t i = k0 * s0 + k1 * s1 + k2;
    const int64_t m0 = k0 > 0 ? i - s0 : i, p0 = k0 + 1 < g.n0 ? i + s0 : i;
    const int64_t m1 = k1 > 0 ? i - s1 : i, p1 = k1 + 1 < g.n1 ? i + s1 : i;
    const int64_t m2 = k2 > 0 ? i - 1 : i, p2 = k2 + 1 < g.n2 ? i + 1 : i;
    // modulo-2^64 arithmetic: the intermediate sums may wrap, the result (f minus a second
    // difference, small) is exact
    const unsigned long long c = (unsigned long long)U[i];
    const unsigned long long au = ((unsigned long long)U[m0] + (unsigned long long)U[p0]) +
                                  ((unsigned long long)U[m1] + (unsigned long long)U[p1]) +
                                  ((unsigned long long)U[m2] + (unsigned long long)U[p2]) - 6ull * c;
    const long long R = (long long)((unsigned long long)F[i] - au);
    // f = F 2^-e + Frem: the remainder keeps f's bits below the fixed-point grid
    const float rf = ldexpf(ll_to_float(R), -e) + (Frem ? Frem[i] : 0.f);
    if (r32) r32[i] = rf;
    const float rs = ldexpf(rf, -k);
    acc = rs * rs;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ float red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) t += red[w];
    atomicAdd(sum, std::ldexp(double(t), 2 * k));
  }
}

// The same residual as a row sweep, for even n2 with 16-byte aligned rows: each thread takes
// two adjacent elements of a row (16-byte loads of U and F, 8-byte of Frem, an 8-byte store of
// r), the CTAs sweep the rows together (sweep_row: a stencil's neighbours one plane away are
// recent L2 lines), and each CTA adds its sum to *sum once. The one-element form issued a CTA
// and a double atomic per 256 elements (524,288 atomics on one address for 512^3).
__device__ __forceinline__ float fx_res_one(unsigned long long c, unsigned long long nb, long long f, float frem,
                                            int e) {
  // modulo-2^64 arithmetic: the intermediate sums may wrap, the result (f minus a second
  // difference, small) is exact
  const long long R = (long long)((unsigned long long)f - (nb - 6ull * c));
  return ldexpf(ll_to_float(R), -e) + frem;
}

__global__ void __launch_bounds__(256) fx_residual_rows_kernel(const long long *U, const long long *F,
                                                               const float *Frem, float *r32, Grid g, int e, int k,
                                                               double *sum) {
  const int64_t rows = g.n0 * g.n1, s0 = g.n1 * g.n2, s1 = g.n2;
  float acc = 0.f;
  for (int64_t t = 0; t * gridDim.x < rows; ++t) {
    const int64_t row = sweep_row(t, 0, 1);
    if (row >= rows) break;
    const int64_t k0 = row / g.n1, k1 = row - k0 * g.n1;
    const int64_t base = row * g.n2;
    const int64_t o0m = k0 > 0 ? -s0 : 0, o0p = k0 + 1 < g.n0 ? s0 : 0;
    const int64_t o1m = k1 > 0 ? -s1 : 0, o1p = k1 + 1 < g.n1 ? s1 : 0;
    for (int64_t k2 = 2 * int64_t(threadIdx.x); k2 < g.n2; k2 += 2 * int64_t(blockDim.x)) {
      const int64_t i = base + k2;
      const longlong2 c = *reinterpret_cast<const longlong2 *>(U + i);
      const longlong2 m0 = *reinterpret_cast<const longlong2 *>(U + i + o0m);
      const longlong2 p0 = *reinterpret_cast<const longlong2 *>(U + i + o0p);
      const longlong2 m1 = *reinterpret_cast<const longlong2 *>(U + i + o1m);
      const longlong2 p1 = *reinterpret_cast<const longlong2 *>(U + i + o1p);
      const long long left = k2 > 0 ? U[i - 1] : c.x;
      const long long right = k2 + 2 < g.n2 ? U[i + 2] : c.y;
      const longlong2 f = *reinterpret_cast<const longlong2 *>(F + i);
      const float2 fr = Frem ? *reinterpret_cast<const float2 *>(Frem + i) : make_float2(0.f, 0.f);
      typedef unsigned long long u64;
      const u64 nx = ((u64)m0.x + (u64)p0.x) + ((u64)m1.x + (u64)p1.x) + ((u64)left + (u64)c.y);
      const u64 ny = ((u64)m0.y + (u64)p0.y) + ((u64)m1.y + (u64)p1.y) + ((u64)c.x + (u64)right);
      const float rx = fx_res_one((u64)c.x, nx, f.x, fr.x, e), ry = fx_res_one((u64)c.y, ny, f.y, fr.y, e);
      if (r32) *reinterpret_cast<float2 *>(r32 + i) = make_float2(rx, ry);
      const float sx = ldexpf(rx, -k), sy = ldexpf(ry, -k);
      acc = fmaf(sx, sx, fmaf(sy, sy, acc));
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ float red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) t += double(red[w]);
    atomicAdd(sum, std::ldexp(t, 2 * k));
  }
}

// Sliding-window form, for rows of 64 .. 512 points (a multiple of 64): a CTA of n2 / 2 threads
// (two adjacent points each) walks a strip of STRIP rows k1 of one plane k0 and keeps the U values
// of rows k1 - 1, k1 and k1 + 1 in registers; the neighbours along the row come from the
// adjacent lanes by shuffles (a warp's edge lanes load theirs). Each U row is then read three
// times (its own plane's walk and the two neighbouring planes'), not seven. CTAs go through the
// planes in order, so the neighbouring planes' rows are recent L2 lines.
template <int STRIP>
__global__ void __launch_bounds__(256) fx_residual_window_kernel(const long long *U, const long long *F,
                                                                 const float *Frem, float *r32, Grid g, int e, int k,
                                                                 double *sum) {
  typedef unsigned long long u64;
  const int64_t s0 = g.n1 * g.n2, s1 = g.n2;
  const int64_t strips = (g.n1 + STRIP - 1) / STRIP;
  const int64_t k0 = int64_t(blockIdx.x) / strips, k1a = (int64_t(blockIdx.x) - k0 * strips) * STRIP;
  const int64_t k1b = k1a + STRIP < g.n1 ? k1a + STRIP : g.n1;
  const int64_t k2 = 2 * int64_t(threadIdx.x);  // n2 == 2 * blockDim.x
  const int64_t o0m = k0 > 0 ? -s0 : 0, o0p = k0 + 1 < g.n0 ? s0 : 0;
  const int64_t plane = k0 * s0 + k2;
  const unsigned lane = threadIdx.x & 31u;
  auto ldU = [&](int64_t r) { return *reinterpret_cast<const longlong2 *>(U + plane + r * s1); };
  longlong2 prev = ldU(k1a > 0 ? k1a - 1 : k1a), cur = ldU(k1a);
  float acc = 0.f;
  for (int64_t k1 = k1a; k1 < k1b; ++k1) {
    const int64_t i = plane + k1 * s1;
    const longlong2 next = ldU(k1 + 1 < g.n1 ? k1 + 1 : k1);
    const longlong2 m0 = *reinterpret_cast<const longlong2 *>(U + i + o0m);
    const longlong2 p0 = *reinterpret_cast<const longlong2 *>(U + i + o0p);
    const longlong2 f = *reinterpret_cast<const longlong2 *>(F + i);
    const float2 fr = Frem ? *reinterpret_cast<const float2 *>(Frem + i) : make_float2(0.f, 0.f);
    long long left = __shfl_up_sync(0xffffffffu, cur.y, 1);
    long long right = __shfl_down_sync(0xffffffffu, cur.x, 1);
    if (lane == 0) left = k2 > 0 ? U[i - 1] : cur.x;
    if (lane == 31) right = k2 + 2 < g.n2 ? U[i + 2] : cur.y;
    const u64 nx = ((u64)m0.x + (u64)p0.x) + ((u64)prev.x + (u64)next.x) + ((u64)left + (u64)cur.y);
    const u64 ny = ((u64)m0.y + (u64)p0.y) + ((u64)prev.y + (u64)next.y) + ((u64)cur.x + (u64)right);
    const float rx = fx_res_one((u64)cur.x, nx, f.x, fr.x, e), ry = fx_res_one((u64)cur.y, ny, f.y, fr.y, e);
    if (r32) *reinterpret_cast<float2 *>(r32 + i) = make_float2(rx, ry);
    const float sx = ldexpf(rx, -k), sy = ldexpf(ry, -k);
    acc = fmaf(sx, sx, fmaf(sy, sy, acc));
    prev = cur;
    cur = next;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ float red[8];
  if (lane == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) t += double(red[w]);
    atomicAdd(sum, std::ldexp(t, 2 * k));
  }
}

// The conversions between float64 and the fixed-point scale run on integer arithmetic over the
// bits of the doubles: GB300's FP64 pipe made the plain double versions (ldexp, rounding,
// subtraction, int64 <-> double conversions) the most expensive kernels of a solve.

// F = round(f 2^e) (half to even) and Frem = f - F 2^-e rounded to float, from the exponent and
// mantissa of f (|f| = M 2^ex): f 2^e = M 2^s, s = ex + e; for s < 0 the quotient M >> -s is
// rounded and the remainder r (|r| <= 2^(-s-1)) is exact, Frem = +-r 2^ex. Same values as
// __double2ll_rn(ldexp(f, e)) and float(f - ldexp(double(F), -e)) (that difference is exact).
// v 2^ex as a float rounded to nearest even, assembled from the normalised magnitude of v
// (correctly rounded, unlike the two-step ll_to_float); out of the normal range: ldexpf.
__device__ __forceinline__ float scaled_float(long long v, int ex) {
  if (v == 0) return 0.f;
  const unsigned sgn = v < 0 ? 0x80000000u : 0u;
  unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const int lz = __clzll((long long)a);
  a <<= lz;  // top bit at 63: |v| = a 2^-lz
  unsigned long long mant = a >> 40;
  const unsigned long long rb = a & ((1ull << 40) - 1), half = 1ull << 39;
  if (rb > half || (rb == half && (mant & 1ull))) ++mant;
  int E = 63 - lz + ex;  // |v| 2^ex = mant 2^(E - 23)
  if (mant >> 24) {
    mant >>= 1;
    ++E;
  }
  const int biased = E + 127;
  if (biased <= 0 || biased >= 255) return ldexpf(ll_to_float(v), ex);
  return __uint_as_float(sgn | unsigned(biased) << 23 | unsigned(mant & 0x7fffffull));
}

__device__ __forceinline__ void fixed_of(double f, int e, long long &F, float &rem) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(f);
  const bool neg = (b >> 63) != 0;
  const int E = int((b >> 52) & 0x7ffull);
  unsigned long long M = b & 0xfffffffffffffull;
  if (E != 0) M |= 1ull << 52;
  const int ex = (E != 0 ? E : 1) - 1075;
  const int s = ex + e;
  unsigned long long Fm = 0;
  long long r = 0;
  if (M != 0) {
    if (s >= 0) {
      Fm = M << s;  // exact; the caller keeps |F| < 2^62
    } else if (s <= -64) {
      r = (long long)M;  // M < 2^53 <= half of 2^-s: rounds to 0
    } else {
      const int t = -s;
      const unsigned long long q = M >> t, low = M & ((1ull << t) - 1), half = 1ull << (t - 1);
      const bool up = low > half || (low == half && (q & 1ull));
      Fm = q + (up ? 1ull : 0ull);
      r = (long long)(low - (up ? (1ull << t) : 0ull));  // two's complement: low - 2^t when up
    }
  }
  F = neg ? -(long long)Fm : (long long)Fm;
  rem = M == 0 ? (neg ? -0.f : 0.f) : scaled_float(neg ? -r : r, ex);  // -0.0 - 0.0 keeps its sign
}

__global__ void __launch_bounds__(256) fx_from_double_kernel(const double *f, long long *F, float *Frem, int64_t total,
                                                             int e) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i0 < total; i0 += kIlp * stride) {
    double x[kIlp];
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      x[q] = i < total ? f[i] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      if (i < total) {
        long long v;
        float rem;
        fixed_of(x[q], e, v, rem);
        F[i] = v;
        if (Frem) Frem[i] = rem;
      }
    }
  }
}

// The out-of-range fallbacks of the integer conversions below, kept out of line: inlined, the
// compiler evaluated them for every element (predicated), which put an FP64 conversion per
// element on GB300's FP64 pipe (85 % busy in the fixed-point to double conversion, 0.26 of the
// HBM copy bandwidth).
__device__ __noinline__ double scaled_double_slow(long long v, int e) { return ldexp(double(v), -e); }
__device__ __noinline__ float float_of_slow(double f) { return __double2float_rn(f); }

// v 2^-e as a double rounded to nearest even, assembled from the normalised magnitude of v
// (no FP64 operations); results outside the normal range fall back to the double path.
__device__ __forceinline__ double scaled_double(long long v, int e) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
  unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const int lz = __clzll((long long)a);
  a <<= lz;  // top bit at 63: |v| = a 2^-lz
  unsigned long long mant = a >> 11;
  const unsigned long long rb = a & 0x7ffull;
  if (rb > 0x400ull || (rb == 0x400ull && (mant & 1ull))) ++mant;
  int E = 63 - lz - e;  // |v| 2^-e = mant 2^(E - 52)
  if (mant >> 53) {
    mant >>= 1;
    ++E;
  }
  const int biased = E + 1023;
  if (biased <= 0 || biased >= 2047) return scaled_double_slow(v, e);
  return __longlong_as_double((long long)(sgn | (unsigned long long)biased << 52 | (mant & 0xfffffffffffffull)));
}

// out = (U - *m) 2^-e (m = 0 when NULL)
__global__ void __launch_bounds__(256) fx_to_double_kernel(const long long *U, double *out, int64_t total, int e,
                                                           const long long *m) {
  const long long shift = m ? *m : 0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i0 < total; i0 += kIlp * stride) {
    long long v[kIlp];
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      v[q] = i < total ? U[i] : 0;
    }
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      if (i < total) out[i] = scaled_double(v[q] - shift, e);
    }
  }
}

// Exact sum of the int64 iterate (128-bit accumulators), one partial per CTA.
__global__ void __launch_bounds__(256) fx_sum_kernel(const long long *U, int64_t total, unsigned long long *part) {
  __int128 acc = 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x)
    acc += U[i];
  __shared__ __int128 sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (int(threadIdx.x) < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const unsigned __int128 v = (unsigned __int128)sh[0];
    part[2 * blockIdx.x] = (unsigned long long)v;
    part[2 * blockIdx.x + 1] = (unsigned long long)(v >> 64);
  }
}

// m = the mean of U rounded to an integer (the division in double: within one unit of the
// exact rounding, 2^-e of the solution)
__global__ void fx_mean_kernel(const unsigned long long *part, int nparts, int64_t total, long long *m) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  __int128 S = 0;
  for (int b = 0; b < nparts; ++b)
    S += (__int128)(((unsigned __int128)part[2 * b + 1] << 64) | (unsigned __int128)part[2 * b]);
  const double hi = double((long long)(S >> 64)), lo = double((unsigned long long)S);
  *m = (long long)llrint((hi * 18446744073709551616.0 + lo) / double(total));
}

// max |x| over the bits (sign cleared, finite values order like their magnitudes), atomically
// into *out as the bits of a double
template <typename T>
__global__ void __launch_bounds__(256) absmax_kernel(const T *x, int64_t total, unsigned long long *out) {
  using B = typename std::conditional<sizeof(T) == 8, unsigned long long, unsigned>::type;
  constexpr B mask = B(~B(0)) >> 1;
  B mx = 0;
  const B *xb = reinterpret_cast<const B *>(x);  // the bits of the values
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i0 < total; i0 += kIlp * stride) {
    B b[kIlp];
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      b[q] = i < total ? xb[i] : B(0);
    }
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const B c = b[q] & mask;
      mx = c > mx ? c : mx;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const B y = __shfl_down_sync(0xffffffffu, mx, o);
    mx = y > mx ? y : mx;
  }
  __shared__ B red[8];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < int(blockDim.x >> 5); ++w) mx = red[w] > mx ? red[w] : mx;
    unsigned long long d;
    if constexpr (sizeof(T) == 8) {
      d = mx;
    } else {
      float fv;
      memcpy(&fv, &mx, 4);
      d = (unsigned long long)__double_as_longlong(double(fv));
    }
    atomicMax(out, d);
  }
}

// float(f) rounded to nearest even from the bits of f (no FP64 operation); out of float's
// normal range the conversion instruction
__device__ __forceinline__ float float_of(double f) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(f);
  const int E = int((b >> 52) & 0x7ffull) - 1023 + 127;
  if (E <= 0 || E >= 254) return float_of_slow(f);
  unsigned long long m = (b & 0xfffffffffffffull) >> 29;
  const unsigned long long rb = b & ((1ull << 29) - 1), half = 1ull << 28;
  unsigned e = unsigned(E);
  if (rb > half || (rb == half && (m & 1ull))) {
    if (++m >> 23) {  // the mantissa carried into the exponent
      m = 0;
      ++e;
    }
  }
  return __uint_as_float(unsigned(b >> 63) << 31 | e << 23 | unsigned(m));
}

// r32 = float(f), stats[0] = max |f| (as the bits of a double, atomic max), stats[1] += sum of
// float(f)^2 (float per thread, double per CTA): one pass over the right-hand side
__global__ void __launch_bounds__(256) prepare_kernel(const double *f, float *r32, int64_t total, double *stats) {
  unsigned long long mx = 0;
  float ss = 0.f;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i0 < total; i0 += kIlp * stride) {
    double v[kIlp];
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      v[q] = i < total ? f[i] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < kIlp; ++q) {
      const int64_t i = i0 + q * stride;
      if (i < total) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(v[q]) & 0x7fffffffffffffffull;
        mx = b > mx ? b : mx;
        const float x = float_of(v[q]);
        r32[i] = x;
        ss = fmaf(x, x, ss);
      }
    }
  }
  double ssd = double(ss);
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, mx, o);
    mx = y > mx ? y : mx;
    ssd += __shfl_down_sync(0xffffffffu, ssd, o);
  }
  __shared__ unsigned long long rm[8];
  __shared__ double rs[8];
  if ((threadIdx.x & 31) == 0) {
    rm[threadIdx.x >> 5] = mx;
    rs[threadIdx.x >> 5] = ssd;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < int(blockDim.x >> 5); ++w) {
      mx = rm[w] > mx ? rm[w] : mx;
      ssd += rs[w];
    }
    atomicMax(reinterpret_cast<unsigned long long *>(stats), mx);
    atomicAdd(stats + 1, ssd);
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

// CTAs of the row-sweep kernels: a few per SM, at most one per row
unsigned grid_rows(const Grid &g, int per_sm) {
  const int64_t want = int64_t(rg::sm_count()) * per_sm;
  return unsigned(std::max<int64_t>(1, std::min<int64_t>(want, g.n0 * g.n1)));
}

dim3 grid3(const Grid &g) {
  RG_CHECK(g.n1 < 65536 && g.n0 < 65536, RG_ERR_UNSUPPORTED, "grid extent beyond 65535 along the first two axes");
  return dim3(unsigned((g.n2 + 255) / 256), unsigned(g.n1), unsigned(g.n0));
}

}  // namespace

// X: C-contiguous n0 x n1 x n2 DCT-II coefficients (itemsize 4 or 8), divided in place by the
// Neumann eigenvalues lam0[k0] + lam1[k1] + lam2[k2] (device tables in X's precision,
// lam = lam0|lam1|lam2 with lam_a[k] = 2 cos(pi k / n_a) - 2); mode (0,0,0) set to 0.
extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_eigdiv(void *X, int64_t itemsize, int64_t n0,
                                                                              int64_t n1, int64_t n2,
                                                                              const void *lam, void *stream) {
  return guarded([&] {
    RG_CHECK(itemsize == 4 || itemsize == 8, RG_ERR_ARG, "float32 or float64 coefficients required");
    RG_CHECK(n0 > 0 && n1 > 0 && n2 > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Grid g{n0, n1, n2};
    const uint64_t bytes = uint64_t(2 * itemsize) * uint64_t(n0 * n1 * n2);
    // vector rows: n2 a multiple of the vector width and X 16-byte aligned
    const bool vec = n2 % (16 / itemsize) == 0 && reinterpret_cast<uintptr_t>(X) % 16 == 0;
    // threads: one per vector of a row (a multiple of 32, at most 256), so that none idles on
    // short rows (512 float32 points: 128 threads), and CTAs per SM in proportion
    const int64_t per_row = (n2 / (vec ? 16 / itemsize : 1) + 31) / 32 * 32;
    const int threads = int(std::min<int64_t>(256, std::max<int64_t>(32, per_row)));
    const unsigned b = grid_rows(g, 4 * 256 / threads);
    rg::profiled_launch(itemsize == 4 ? "poisson_eigdiv_f32" : "poisson_eigdiv_f64", bytes, st, [&] {
      if (itemsize == 4) {
        const float *l = static_cast<const float *>(lam);
        if (vec) eigdiv_kernel<float, 4><<<b, threads, 0, st>>>(static_cast<float *>(X), g, l, l + n0, l + n0 + n1);
        else eigdiv_kernel<float, 1><<<b, threads, 0, st>>>(static_cast<float *>(X), g, l, l + n0, l + n0 + n1);
      } else {
        const double *l = static_cast<const double *>(lam);
        if (vec) eigdiv_kernel<double, 2><<<b, threads, 0, st>>>(static_cast<double *>(X), g, l, l + n0, l + n0 + n1);
        else eigdiv_kernel<double, 1><<<b, threads, 0, st>>>(static_cast<double *>(X), g, l, l + n0, l + n0 + n1);
      }
    });
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_dct2_eigdiv(const float *in, float *out,
                                                                                   int64_t n0, int64_t n1,
                                                                                   int64_t n2, const float *lam,
                                                                                   void *stream) {
  return guarded([&] {
    RG_CHECK(n0 > 0 && n1 > 0 && n2 > 0, RG_ERR_ARG, "empty grid");
    RG_CHECK(rg::dct2_eigdiv_3d(in, out, n0, n1, n2, lam, static_cast<cudaStream_t>(stream)), RG_ERR_UNSUPPORTED,
             "no compile-time DCT-II kernel for the last axis");
  });
}

// u_hi (+ u_lo) += delta by an exact two-sum (u_lo may be NULL: plain addition).
extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_update(double *u, float *u_lo,
                                                                              const float *delta, int64_t total,
                                                                              void *stream) {
  return guarded([&] {
    RG_CHECK(total > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint64_t bytes = uint64_t(total) * (u_lo ? 28 : 20);
    rg::profiled_launch("poisson_update", bytes, st,
                        [&] { update_kernel<<<grid_for(total), 256, 0, st>>>(u, u_lo, delta, total); });
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
    const uint64_t bytes = uint64_t(n0 * n1 * n2) * (16 + (u_lo ? 4 : 0) + (r32 ? 4 : 0));
    rg::profiled_launch("poisson_residual", bytes, st,
                        [&] { residual_kernel<<<grid3(g), 256, 0, st>>>(u, u_lo, f, r32, g, sumsq); });
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

// Fixed-point iterate u = U * 2^-e (U int64, C-contiguous n0 x n1 x n2).
extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_update_fx(int64_t *U, const float *delta,
                                                                                 int64_t total, int32_t e,
                                                                                 void *stream) {
  return guarded([&] {
    RG_CHECK(total > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rg::profiled_launch("poisson_update_fx", uint64_t(total) * 20, st, [&] {
      fx_update_kernel<<<grid_for(total), 256, 0, st>>>(reinterpret_cast<long long *>(U), delta, total, e, 0);
    });
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_residual_fx(
    const int64_t *U, const int64_t *F, const float *Frem, int32_t e, int32_t k, float *r32, int64_t n0, int64_t n1,
    int64_t n2, double *sumsq, void *stream) {
  return guarded([&] {
    RG_CHECK(n0 > 0 && n1 > 0 && n2 > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RG_CUDA(cudaMemsetAsync(sumsq, 0, sizeof(double), st));
    Grid g{n0, n1, n2};
    const uint64_t bytes = uint64_t(n0 * n1 * n2) * (16 + (Frem ? 4 : 0) + (r32 ? 4 : 0));
    const bool rows_form = n2 % 2 == 0 && reinterpret_cast<uintptr_t>(U) % 16 == 0 &&
                           reinterpret_cast<uintptr_t>(F) % 16 == 0 && reinterpret_cast<uintptr_t>(Frem) % 8 == 0 &&
                           reinterpret_cast<uintptr_t>(r32) % 8 == 0;
    constexpr int kStrip = 32;
    const bool window_form = rows_form && n2 % 64 == 0 && n2 <= 512 && n0 * ((n1 + kStrip - 1) / kStrip) < (int64_t(1) << 31);
    rg::profiled_launch("poisson_residual_fx", bytes, st, [&] {
      if (window_form)
        fx_residual_window_kernel<kStrip><<<unsigned(n0 * ((n1 + kStrip - 1) / kStrip)), unsigned(n2 / 2), 0, st>>>(
            reinterpret_cast<const long long *>(U), reinterpret_cast<const long long *>(F), Frem, r32, g, e, k, sumsq);
      else if (rows_form)
        fx_residual_rows_kernel<<<grid_rows(g, 8), 256, 0, st>>>(reinterpret_cast<const long long *>(U),
                                                                 reinterpret_cast<const long long *>(F), Frem, r32,
                                                                 g, e, k, sumsq);
      else
        fx_residual_kernel<<<grid3(g), 256, 0, st>>>(reinterpret_cast<const long long *>(U),
                                                     reinterpret_cast<const long long *>(F), Frem, r32, g, e, k, sumsq);
    });
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_to_fx(const double *f, int32_t e, int64_t *F,
                                                                             float *Frem, int64_t total, void *stream) {
  return guarded([&] {
    RG_CHECK(total > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rg::profiled_launch("poisson_to_fx", uint64_t(total) * 20, st, [&] {
      fx_from_double_kernel<<<grid_for(total), 256, 0, st>>>(f, reinterpret_cast<long long *>(F), Frem, total, e);
    });
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_fx_to_double(const int64_t *U, int32_t e,
                                                                                    double *out, int64_t total,
                                                                                    void *stream) {
  return guarded([&] {
    RG_CHECK(total > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    fx_to_double_kernel<<<grid_for(total), 256, 0, st>>>(reinterpret_cast<const long long *>(U), out, total, e,
                                                         nullptr);
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_fx_to_double_zero_mean(const int64_t *U,
                                                                                              int32_t e, double *out,
                                                                                              int64_t total,
                                                                                              void *stream) {
  return guarded([&] {
    RG_CHECK(total > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned g = grid_for(total);
    rg::DevBuf work(size_t(2 * g + 1) * sizeof(unsigned long long), st);
    unsigned long long *part = static_cast<unsigned long long *>(work.get());
    long long *m = reinterpret_cast<long long *>(part + 2 * g);
    const long long *u = reinterpret_cast<const long long *>(U);
    rg::profiled_launch("poisson_fx_sum", uint64_t(total) * 8, st,
                        [&] { fx_sum_kernel<<<g, 256, 0, st>>>(u, total, part); });
    fx_mean_kernel<<<1, 32, 0, st>>>(part, int(g), total, m);
    rg::profiled_launch("poisson_fx_to_double", uint64_t(total) * 16, st,
                        [&] { fx_to_double_kernel<<<g, 256, 0, st>>>(u, out, total, e, m); });
    for (int i = 0; i < 3; ++i) rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_init_fx(int64_t *U, const float *delta,
                                                                               int64_t total, int32_t e,
                                                                               void *stream) {
  return guarded([&] {
    RG_CHECK(total > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rg::profiled_launch("poisson_init_fx", uint64_t(total) * 12, st, [&] {
      fx_update_kernel<<<grid_for(total), 256, 0, st>>>(reinterpret_cast<long long *>(U), delta, total, e, 1);
    });
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) int rocketgpu_poisson_prepare(const double *f, float *r32,
                                                                               int64_t total, double *stats,
                                                                               void *stream) {
  return guarded([&] {
    RG_CHECK(total > 0, RG_ERR_ARG, "empty grid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RG_CUDA(cudaMemsetAsync(stats, 0, 2 * sizeof(double), st));
    rg::profiled_launch("poisson_prepare", uint64_t(total) * 12, st,
                        [&] { prepare_kernel<<<grid_for(total), 256, 0, st>>>(f, r32, total, stats); });
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) int rocketgpu_abs_max(const void *x, int64_t itemsize, int64_t total,
                                                                       double *out, void *stream) {
  return guarded([&] {
    RG_CHECK(itemsize == 4 || itemsize == 8, RG_ERR_ARG, "float32 or float64 data");
    RG_CHECK(total >= 0, RG_ERR_ARG, "negative size");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    RG_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st));
    if (total == 0) return;
    unsigned long long *o = reinterpret_cast<unsigned long long *>(out);
    rg::profiled_launch("abs_max", uint64_t(total) * uint64_t(itemsize), st, [&] {
      if (itemsize == 8) absmax_kernel<double><<<grid_for(total), 256, 0, st>>>(static_cast<const double *>(x), total, o);
      else absmax_kernel<float><<<grid_for(total), 256, 0, st>>>(static_cast<const float *>(x), total, o);
    });
    rg::note_launch();
    RG_CUDA(cudaGetLastError());
  });
}

extern "C" __attribute__((visibility("default"))) const char *rocketgpu_poisson_last_error(void) {
  return t_err.c_str();
}
