// Tensor-core split-FP16 form of the DFT-16 stages (tcgen05, accumulators in tensor memory).
//
// A radix-16 butterfly is a 16 x 16 complex matrix-vector product, i.e. with complex numbers
// written as (re, im) pairs a 32 x 32 real one: Y = F x with
//     Re Y_q = sum_p cos(t) Re x_p + sin(t) Im x_p,   Im Y_q = sum_p -sin(t) Re x_p + cos(t) Im x_p,
//     t = 2 pi q p / 16.
// One MMA group computes 128 butterflies at once: D[128 x 32] = X[128 x 32] * F^T, rows of X =
// butterflies (one thread each), K order (Re x_0..15, Im x_0..15), N order (Re Y_0..15, Im
// Y_0..15). Each operand is split into an FP16 high part and an FP16 residual
// (x = x_hi + x_lo, F = F_hi + F_lo, 22 significant bits). Two FP32 accumulators per group:
// D1 = x_hi F_hi and D2 = x_hi F_lo + x_lo F_hi (the x_lo F_lo term, about 2^-22 of the product,
// is left out: a quarter fewer MMAs); the tensor core's accumulation
// does not round to nearest, so the large product is kept apart from the corrections and the
// two are added in SIMT code (Y = D1 + D2, one rounding). Each butterfly's inputs are first scaled by a
// power of two that puts their largest magnitude in [2^13, 2^14) (exact, undone on the
// outputs), which keeps x_hi and x_lo inside FP16's range.
//
// Twiddles, index arithmetic and the loads and stores stay in FP32 SIMT code; only the 16-point
// DFTs run on the tensor cores. Kernel: complex64 c2c of length 256 along a strided axis
// (column walk, 16 columns per CTA), the two passes 16 x 16 of the plain fixed-length kernel.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/rocket_gpu.h"
#include "rg_error.hpp"
#include "rg_fixed_kernel.cuh"
#include "rg_launch.hpp"
#include "rg_tc.cuh"

namespace rg {
namespace {

constexpr int kTcThreads = 256;  // = butterflies per pass of a 16-column tile of length 256
constexpr int kTcCols = 128;     // tensor-memory columns: two MMA groups x two accumulators x 32 f32
constexpr uint32_t kSbo = 512;   // 8 rows x 32 f16 of K
constexpr uint64_t kWaitNs = 1000000000ull;  // 1 s bound on every mbarrier wait

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase (false on timeout).
__device__ __forceinline__ bool mbar_wait_timed(uint64_t *mbar, uint32_t parity) {
  const uint64_t t0 = globaltimer();
  for (;;) {
    if (tc::mbar_wait(mbar, parity, 64)) return true;
    if (globaltimer() - t0 > kWaitNs) return false;
  }
}

// Shared layout of the tensor-core kernels (dynamic shared memory):
//   [0, 16K)   X_hi  256 rows x 32 f16, canonical K-major
//   [16K, 32K) X_lo
//   [32K, 34K) F_hi  32 rows (N) x 32 f16
//   [34K, 36K) F_lo
//   [36K, ...) exchange buffer of the two passes (complex64, padded rows)
constexpr uint32_t kOffXhi = 0, kOffXlo = 16384, kOffFhi = 32768, kOffFlo = 34816, kOffBuf = 36864;

struct TcShared {
  uint32_t tmem;
  uint32_t err;
  uint64_t mbar;
};

// Write one butterfly row (16 complex values, already scaled) as hi/lo FP16 operand rows.
__device__ __forceinline__ void put_row(unsigned char *sm, int row, const float2 (&v)[16]) {
  const uint32_t base = uint32_t((row >> 3) * kSbo + (row & 7) * 16);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    // chunk c: K = 8c .. 8c+7 -> c < 2: Re x_{8c..8c+7}; c >= 2: Im x_{8(c-2)..}
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int p = (c & 1) * 8 + 2 * h;
      const float a = c < 2 ? v[p].x : v[p].y;
      const float b = c < 2 ? v[p + 1].x : v[p + 1].y;
      const __half2 hh = __floats2half2_rn(a, b);
      const float2 hf = __half22float2(hh);
      const __half2 ll = __floats2half2_rn(a - hf.x, b - hf.y);
      hi[h] = *reinterpret_cast<const uint32_t *>(&hh);
      lo[h] = *reinterpret_cast<const uint32_t *>(&ll);
    }
    *reinterpret_cast<uint4 *>(sm + kOffXhi + base + c * tc::kLBO) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<uint4 *>(sm + kOffXlo + base + c * tc::kLBO) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
  }
}

// Power-of-two scale putting max |component| in [2^13, 2^14) (1 for an all-zero butterfly).
__device__ __forceinline__ float pow2_scale(const float2 (&v)[16]) {
  float m = 0.f;
#pragma unroll
  for (int k = 0; k < 16; ++k) m = fmaxf(m, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
  if (!(m > 0.f) || !(m < INFINITY)) return 1.f;
  const int ex = int((__float_as_uint(m) >> 23) & 0xFF);  // biased exponent (0 for subnormal)
  int sb = 267 - (ex == 0 ? 1 : ex);                       // biased exponent of 2^(13 - e)
  sb = sb > 254 ? 254 : sb;
  return __uint_as_float(uint32_t(sb) << 23);
}

// The MMAs of one pass and their commit. Group g (butterflies 128 g .. 128 g + 127) writes D1
// at tensor-memory column 64 g and D2 at 64 g + 32; K = 32 takes two K = 16 steps.
__device__ __forceinline__ void issue_pass(unsigned char *sm, uint32_t tmem, uint64_t *mbar) {
  const uint32_t base = tc::saddr(sm);
  constexpr uint32_t idesc = tc::idesc_f16_f32(128, 32);
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    const uint32_t d1 = tmem + uint32_t(64 * g), d2 = d1 + 32;
    const uint32_t xh = base + kOffXhi + uint32_t(g) * 16 * kSbo, xl = base + kOffXlo + uint32_t(g) * 16 * kSbo;
    const uint32_t fh = base + kOffFhi, fl = base + kOffFlo;
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
      const uint32_t ko = uint32_t(ks) * 2 * tc::kLBO;
      tc::mma_f16(d1, tc::smem_desc(xh + ko, tc::kLBO, kSbo), tc::smem_desc(fh + ko, tc::kLBO, kSbo), idesc, ks);
    }
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
      const uint32_t ko = uint32_t(ks) * 2 * tc::kLBO;
      tc::mma_f16(d2, tc::smem_desc(xh + ko, tc::kLBO, kSbo), tc::smem_desc(fl + ko, tc::kLBO, kSbo), idesc, ks);
      tc::mma_f16(d2, tc::smem_desc(xl + ko, tc::kLBO, kSbo), tc::smem_desc(fh + ko, tc::kLBO, kSbo), idesc, 1);
    }
  }
  tc::mma_commit(mbar);
}

// This thread's row of D1 + D2 for group g (lane = thread within the group).
__device__ __forceinline__ void read_pass(const TcShared &S, float (&d)[32]) {
  const int tid = threadIdx.x, warp = tid >> 5, g = tid >> 7;
  const uint32_t t = S.tmem + (uint32_t(32 * (warp & 3)) << 16) + uint32_t(64 * g);
  float e[32];
  tc::tmem_ld32(t, d);
  tc::tmem_ld32(t + 32, e);
#pragma unroll
  for (int n = 0; n < 32; ++n) d[n] += e[n];
}

// Load the split DFT-16 matrix (global [2][32][32] f16, rows n, K contiguous) into the
// canonical layout.
__device__ __forceinline__ void load_fmat(unsigned char *sm, const __half *fmat) {
  for (int e = threadIdx.x; e < 2 * 32 * 4; e += blockDim.x) {  // 16-byte chunks
    const int which = e / 128, rem = e % 128, n = rem / 4, c = rem % 4;
    const uint4 v = *reinterpret_cast<const uint4 *>(fmat + which * 1024 + n * 32 + c * 8);
    const uint32_t off = uint32_t((n >> 3) * kSbo + c * tc::kLBO + (n & 7) * 16);
    *reinterpret_cast<uint4 *>(sm + (which ? kOffFlo : kOffFhi) + off) = v;
  }
}

// One tensor-core DFT-16 of this thread's butterfly (all 256 threads call it together):
// scale, split into operand rows, MMA, read back, unscale. `phase` is the mbarrier parity.
__device__ __forceinline__ void tc_dft16(unsigned char *sm, TcShared &S, float2 (&v)[16], uint32_t phase) {
  const int tid = threadIdx.x;
  const float s = pow2_scale(v);
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = make_float2(v[k].x * s, v[k].y * s);
  put_row(sm, tid, v);
  tc::fence_smem_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (tid == 0) issue_pass(sm, S.tmem, &S.mbar);
  if (!mbar_wait_timed(&S.mbar, phase)) S.err = 1;
  tc::fence_after();
  float d[32];
  read_pass(S, d);
  const float inv = 1.f / s;
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = make_float2(d[q] * inv, d[16 + q] * inv);
}

using TcCfg = FxCfg<float, OP_C2C, 8, true>;
constexpr uint32_t kOffShared = kOffBuf + uint32_t(TcCfg::TB * TcCfg::PITCH * sizeof(float2));
constexpr size_t kTcSmem = kOffShared + sizeof(TcShared);

template <bool BWD>
__global__ void __launch_bounds__(kTcThreads) tc_c2c256_col_kernel(const __grid_constant__ KArgs a,
                                                                     const __half *__restrict__ fmat, int *err) {
  using C = TcCfg;
  constexpr int TB = C::TB, PS = C::PS, PITCH = C::PITCH;
  static_assert(TB == 16 && C::NT == kTcThreads, "tile");
  extern __shared__ __align__(16) unsigned char sm[];
  TcShared &S = *reinterpret_cast<TcShared *>(sm + kOffShared);
  float2 *buf = reinterpret_cast<float2 *>(sm + kOffBuf);
  const int tid = threadIdx.x;
  if (tid < 32) tc::tmem_alloc(&S.tmem, kTcCols);
  if (tid == 0) {
    tc::mbar_init(&S.mbar, 1);
    S.err = 0;
  }
  load_fmat(sm, fmat);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();

  const uint32_t row0 = uint32_t(blockIdx.x) * TB;
  const int rows = int(min(int64_t(TB), a.nrows - int64_t(row0)));
  const float2 *tw = reinterpret_cast<const float2 *>(a.core.tw);
  const int r = tid & (TB - 1), j = tid >> 4;  // column of the tile, butterfly within the column
  const bool live = r < rows;
  const bool scale = a.fct != 1.0;
  const float fct = float(a.fct);

  // pass 0: x[j + 16 k] -> Z[16 j + q]
  float2 v[16];
  if (live) {
    const float2 *p = reinterpret_cast<const float2 *>(a.in) + side_offset32(a.ld, row0 + uint32_t(r)) +
                      int64_t(j) * a.ld.axis_stride;
    const int64_t step = 16 * a.ld.axis_stride;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const float2 x = __ldg(p + k * step);
      v[k] = BWD ? make_float2(x.y, x.x) : x;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = make_float2(0.f, 0.f);
  }
  tc_dft16(sm, S, v, 0);
  {
    float2 *dp = buf + r * PITCH;
    const int b0 = 16 * j + j;  // position 16 j + q padded: 16 j + j + q
#pragma unroll
    for (int q = 0; q < 16; ++q) dp[b0 + q] = v[q];
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();

  // pass 1: Z[j + 16 k] * W_256^{j k} -> X[j + 16 q]
  {
    const float2 *sp = buf + r * PITCH;
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = sp[fx_pos<PS, 16>(j, k)];
    const float2 *t = tw + fx::tw_of(8, 1) + j;
#pragma unroll
    for (int k = 1; k < 16; ++k) v[k] = mul<float>(v[k], __ldg(t + (k - 1) * 16));
  }
  tc_dft16(sm, S, v, 1);
  if (live) {
    float2 *p = reinterpret_cast<float2 *>(a.out) + side_offset32(a.st, row0 + uint32_t(r)) +
                int64_t(j) * a.st.axis_stride;
    const int64_t step = 16 * a.st.axis_stride;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float2 x = BWD ? make_float2(v[q].y, v[q].x) : v[q];
      if (scale) x = make_float2(x.x * fct, x.y * fct);
      p[q * step] = x;
    }
  }
  tc::fence_before();
  __syncthreads();
  if (S.err) {
    // a wait gave up: give the outstanding MMAs one more bounded wait before freeing their
    // tensor memory, then report
    if (tid == 0) {
      mbar_wait_timed(&S.mbar, 1);
      atomicExch(err, 1);
    }
    __syncthreads();
  }
  if (tid < 32) tc::tmem_dealloc(S.tmem, kTcCols);
}

// Self-test of the tensor-core primitives: D = A B^T + A B2^T + A2 B^T for A, A2
// 256 x 32 and B, B2 32 x 32 (f16, row-major, K contiguous), D 256 x 32 f32 -- the exact
// operation sequence of one pass of the kernels above.
__global__ void __launch_bounds__(kTcThreads) tc_selftest_kernel(const __half *A, const __half *A2, const __half *B,
                                                                   const __half *B2, float *D, int *err) {
  extern __shared__ __align__(16) unsigned char sm[];
  TcShared &S = *reinterpret_cast<TcShared *>(sm + kOffBuf);
  const int tid = threadIdx.x;
  if (tid < 32) tc::tmem_alloc(&S.tmem, kTcCols);
  if (tid == 0) {
    tc::mbar_init(&S.mbar, 1);
    S.err = 0;
  }
  // A rows -> X_hi / X_lo, B rows -> F_hi / F_lo
  for (int c = 0; c < 4; ++c) {
    const uint32_t off = uint32_t((tid >> 3) * kSbo + c * tc::kLBO + (tid & 7) * 16);
    *reinterpret_cast<uint4 *>(sm + kOffXhi + off) = *reinterpret_cast<const uint4 *>(A + tid * 32 + c * 8);
    *reinterpret_cast<uint4 *>(sm + kOffXlo + off) = *reinterpret_cast<const uint4 *>(A2 + tid * 32 + c * 8);
  }
  if (tid < 32) {
    for (int c = 0; c < 4; ++c) {
      const uint32_t off = uint32_t((tid >> 3) * kSbo + c * tc::kLBO + (tid & 7) * 16);
      *reinterpret_cast<uint4 *>(sm + kOffFhi + off) = *reinterpret_cast<const uint4 *>(B + tid * 32 + c * 8);
      *reinterpret_cast<uint4 *>(sm + kOffFlo + off) = *reinterpret_cast<const uint4 *>(B2 + tid * 32 + c * 8);
    }
  }
  tc::fence_smem_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (tid == 0) issue_pass(sm, S.tmem, &S.mbar);
  if (!mbar_wait_timed(&S.mbar, 0)) S.err = 1;
  tc::fence_after();
  float d[32];
  read_pass(S, d);
  for (int n = 0; n < 32; ++n) D[tid * 32 + n] = d[n];
  tc::fence_before();
  __syncthreads();
  if (S.err) {
    if (tid == 0) {
      mbar_wait_timed(&S.mbar, 0);
      atomicExch(err, 1);
    }
    __syncthreads();
  }
  if (tid < 32) tc::tmem_dealloc(S.tmem, kTcCols);
}

// Per-device tables: the split DFT-16 matrix and an error flag.
struct TcTables {
  __half *fmat = nullptr;
  int *err = nullptr;
};

TcTables &tc_tables() {
  static std::mutex mu;
  static TcTables t[64];
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  TcTables &x = t[dev];
  if (!x.fmat) {
    std::vector<__half> h(2 * 32 * 32);
    const double pi = 3.14159265358979323846;
    for (int n = 0; n < 32; ++n)
      for (int k = 0; k < 32; ++k) {
        const int q = n & 15, p = k & 15;
        const double t = 2.0 * pi * double((q * p) & 15) / 16.0;
        double f;
        if (n < 16) f = k < 16 ? std::cos(t) : std::sin(t);
        else f = k < 16 ? -std::sin(t) : std::cos(t);
        const __half hi = __double2half(f);
        const __half lo = __double2half(f - double(__half2float(hi)));
        h[n * 32 + k] = hi;
        h[1024 + n * 32 + k] = lo;
      }
    RG_CUDA(cudaMalloc(&x.fmat, h.size() * sizeof(__half)));
    RG_CUDA(cudaMemcpy(x.fmat, h.data(), h.size() * sizeof(__half), cudaMemcpyHostToDevice));
    RG_CUDA(cudaMalloc(&x.err, sizeof(int)));
    RG_CUDA(cudaMemset(x.err, 0, sizeof(int)));
  }
  return x;
}

}  // namespace

// Tensor-core c2c of length 256 along a strided complex64 axis (column walk). Returns false if
// the job is not of that shape.
bool launch_tc_c2c(const KArgs &a, bool col, bool bwd, cudaStream_t st) {
  if (!col || a.core.L != 256) return false;
  TcTables &t = tc_tables();
  const void *fn = bwd ? reinterpret_cast<const void *>(&tc_c2c256_col_kernel<true>)
                       : reinterpret_cast<const void *>(&tc_c2c256_col_kernel<false>);
  set_smem_attr(fn, kTcSmem);
  const int64_t grid = (a.nrows + 15) / 16;
  RG_CHECK(grid < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "too many transforms in one call");
  if (bwd)
    tc_c2c256_col_kernel<true><<<unsigned(grid), kTcThreads, kTcSmem, st>>>(a, t.fmat, t.err);
  else
    tc_c2c256_col_kernel<false><<<unsigned(grid), kTcThreads, kTcSmem, st>>>(a, t.fmat, t.err);
  return true;
}

int tc_error_flag(cudaStream_t st) {
  TcTables &t = tc_tables();
  int h = 0;
  RG_CUDA(cudaMemcpyAsync(&h, t.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  RG_CUDA(cudaStreamSynchronize(st));
  return h;
}

void tc_selftest(const void *A, const void *A2, const void *B, const void *B2, float *D, cudaStream_t st) {
  TcTables &t = tc_tables();
  const void *fn = reinterpret_cast<const void *>(&tc_selftest_kernel);
  set_smem_attr(fn, kOffBuf + sizeof(TcShared));
  tc_selftest_kernel<<<1, kTcThreads, kOffBuf + sizeof(TcShared), st>>>(static_cast<const __half *>(A), static_cast<const __half *>(A2),
                                                     static_cast<const __half *>(B), static_cast<const __half *>(B2), D,
                                                     t.err);
  note_launch();
  RG_CUDA(cudaGetLastError());
}

}  // namespace rg
