// Shared host/device definitions for the GB300 pocketfft transform path.
//
// Everything that crosses the host->kernel boundary lives here as plain structs passed by
// value as kernel parameters (one launch = one "axis job": a batch of 1-D transforms along
// one axis of a strided array).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rg {

constexpr int kMaxPass = 20;    // radix passes of one on-chip FFT
constexpr int kMaxBatchDims = 6; // batch (non-transformed) dims after host-side collapsing

// Division by a runtime constant d (1 <= d < 2^31) for unsigned 32-bit numerators via a
// multiply-high: q = (umulhi(n, m) + n) >> s, the round-up method of Granlund & Montgomery
// (PLDI'94), with the add done in 64 bits so that no n < 2^32 overflows.
struct FastDiv {
  uint32_t d, m, s, pad_;
};

inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f{d, 0, 0, 0};
  uint32_t s = 0;
  while ((uint64_t(1) << s) < d) ++s;
  f.s = s;
  f.m = uint32_t(((uint64_t(1) << 32) * ((uint64_t(1) << s) - d)) / d + 1);
  return f;
}

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
  uint32_t hi = __umulhi(n, f.m);
  return uint32_t((uint64_t(hi) + n) >> f.s);
}
#endif

// One Stockham radix pass of an on-chip FFT of length L (see rg_fft.cuh).
struct PassDesc {
  int R;   // radix
  int Ns;  // product of the radices of the previous passes
  int LR;  // L / R butterflies per transform
  int tw;  // offset of this pass's twiddles in the core table: (R-1)*Ns entries
  FastDiv dNs, dLR;
};

// An on-chip FFT of length L as a sequence of radix passes.
struct FFTCore {
  int L;
  int npass;
  const void *tw;  // complex<T> twiddles, forward sign, all passes back to back
  PassDesc pass[kMaxPass];
};

// Global addressing of one side (load or store) of an axis job. Element (row g, position i)
// lives at  sum_d idx_d(g) * bstride[d] + i * axis_stride  (in units of the side's element
// type), where idx_d(g) decomposes the row number over bshape with dim 0 fastest.
struct Side {
  int64_t axis_stride;
  int64_t bshape[kMaxBatchDims];
  int64_t bstride[kMaxBatchDims];
  int nbd;
  int colmap;  // 1: consecutive threads walk consecutive rows (rows are adjacent in memory)
  FastDiv bdiv[kMaxBatchDims];  // reciprocals of bshape (set by the launcher for kernels that
                                // decompose 32-bit row numbers, rg_fixed_kernel.cuh)
};

// What the kernel does around the on-chip FFT.
enum Op : int {
  OP_C2C = 0,        // complex -> complex, length n = L
  OP_C2C_TW = 1,     // four-step first pass: C2C, then multiply element k of row g by
                     // W_N^{(g mod aux_n) * k}, N = L * aux_n
  OP_R2C_EVEN = 2,   // real n = 2L -> n/2+1 complex (half-length complex FFT + split)
  OP_R2C_ODD = 3,    // real n = L -> n/2+1 complex
  OP_C2R_EVEN = 4,   // n/2+1 complex -> real n = 2L
  OP_C2R_ODD = 5,    // n/2+1 complex -> real n = L
  OP_BLUE = 6,       // complex n -> complex n through a length-L (L >= 2n-1) convolution
  OP_DCT2 = 7, OP_DCT3 = 8, OP_DCT4_EVEN = 9, OP_DCT1 = 10, OP_DST1 = 11,
  OP_R2R_FFTPACK_R2H = 12, OP_R2R_FFTPACK_H2R = 13, OP_HARTLEY = 14,
  OP_DCT2_HALF = 15,  // DCT/DST-II of real n = 2L through the length-L complex FFT of the
                      // Makhoul-ordered input (r2c) and the post-twiddle (compile-time-L only)
  OP_DCT3_HALF = 16,  // DCT/DST-III of real n = 2L: pre-twiddled half spectrum, c2r (same)
  OP_COUNT = 17
};

constexpr int kFlagStream = 4;
// OP_DCT2_HALF row walk over the last axis of a C-contiguous n0 x n1 x n2 volume: divide every
// output by the Neumann eigenvalue lam0[k0] + lam1[k1] + lam2[k2] (aux3 = lam0 | lam1 | lam2,
// aux_s = n0, aux_n = n1; the (0, 0, 0) output set to 0) -- the Poisson solver's spectral divide
// fused into its DCT-II
constexpr int kFlagEigDiv = 8;
// The divide of the Poisson spectral step (the float32 preconditioner of an exact fixed-point
// refinement): in float32 the fast division (two ulp; an IEEE division per point cost the fused
// DCT-II pass 60 % more time), in float64 the IEEE one. The separate divide kernel uses the same
// function, so both routes give the same bits.
template <typename T> __device__ __forceinline__ T eig_div(T y, T lam) {
  if constexpr (sizeof(T) == 4) return __fdividef(y, lam);
  else return y / lam;
}

// L2 cache policy for a launch's input loads: evict-first when the launch reads its input once
// (kFlagStream), so that it does not push out of L2 the data the next launch reads; evict-normal
// otherwise. One policy register per thread, one load instruction for both cases.
__device__ __forceinline__ uint64_t input_policy(bool once) {
  uint64_t pol;
  if (once)
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  else
    asm("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
// Read-only global loads with an L2 cache policy.
__device__ __forceinline__ float ld_in(const float *p, uint64_t pol) {
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double ld_in(const double *p, uint64_t pol) {
  double v;
  asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ float2 ld_in(const float2 *p, uint64_t pol) {
  float2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ld_in(const double2 *p, uint64_t pol) {
  double2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(p), "l"(pol));
  return v;
}

struct KArgs {
  const void *in;
  void *out;
  Side ld, st;
  int64_t nrows;   // number of transforms in this launch
  int TB;          // transforms (rows) per CTA
  int n;           // logical transform length along the axis
  int nin, nout;   // elements per row read / written
  int pitch;       // shared-memory row pitch, in complex elements
  int ps;          // pad shift: shared index i is stored at i + (i >> ps)
  int conj_in;     // conjugate while loading (backward transforms run the forward core on
  int conj_out;    // conjugated data) / while storing
  int flags;       // bit 1 (op-specific) = sine transform (DST) for the fused DCT ops; bit 2 =
                   // the input is read once (out-of-place launch): loads evict-first (kFlagStream)
  double fct;      // scale applied to every output
  double bscale;   // r2c/c2r: extra scale of the interior half-spectrum bins 0 < k < n/2 (1 for
                   // the transforms; 2 / 0.5 for the adjoints of c2r / r2c)
  double e0;       // fused DCT-II: weight of output element 0; DCT-III: of input element 0
  const void *aux;   // op-specific table (split twiddles, chirp, ...)
  const void *aux2;  // op-specific second table (Bluestein spectrum, ...)
  int aux_n;         // op-specific integer (four-step: number of columns)
  int aux_s;         // op-specific integer (four-step: low-table split shift)
  const void *aux3;  // op-specific third table (kFlagEigDiv: the eigenvalues)
  FFTCore core;
};

}  // namespace rg
