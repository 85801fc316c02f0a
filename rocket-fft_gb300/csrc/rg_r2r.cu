// Real-to-real transforms on the GPU: DCT/DST types I-IV, r2r_fftpack and the separable and
// genuine Hartley transforms (the reference's T_dct1/T_dst1/T_dcst23/T_dcst4, ExecR2R,
// ExecHartley and r2r_genuine_hartley; rocket_fft/_pocketfft_hdronly.h:2918-3163, 3661-3705,
// 3854-3873, 4025-4091).
//
// Each axis job is: a pre kernel that forms, per row, a complex sequence of length M in a
// workspace; the complex FFT of length M (c2c_rows: on chip, four-step or Bluestein); a post
// kernel that forms the real outputs. The reductions (M per transform):
//   DCT-I   M = 2(n-1)  even extension,            y_k = Re W_k
//   DST-I   M = 2(n+1)  odd extension,             y_k = -Im W_{k+1}
//   DCT-II  M = n       v = (x_0, x_2, ..., x_3, x_1) (Makhoul), y_k = 2 Re(e^{-i pi k/2n} V_k)
//   DCT-III M = n       V_k = (x_k - i x_{n-k}) e^{i pi k/2n}, v = IDFT(V), y_2j = Re v_j,
//                       y_2j+1 = Re v_{n-1-j}
//   DCT-IV  M = 2n      W = DFT_2n(x_j e^{-i pi j/2n}), y_k = 2 Re(e^{-i pi (2k+1)/4n} W_k)
// DSTs of types II-IV follow the reference's sign flips and reversals around the cosine
// transform, and `ortho` scales the same elements as there (for DST-II/III the element the
// reference scales, which is the first one after its reversal / before its reversal). The
// FFTPACK r2r keeps the reference's half-complex order and its sign flips of entries 2,4,...
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>

#include "rg_error.hpp"
#include "rg_exec.hpp"
#include "rg_exec_detail.hpp"
#include "rg_fft.cuh"
#include "rg_launch.hpp"

namespace rg {

namespace {

enum R2RKind : int {
  K_DCT1 = 0, K_DST1, K_DCT2, K_DCT3, K_DCT4, K_R2HC, K_HC2R, K_HARTLEY
};

struct R2RArgs {
  const void *in;
  void *out;
  Side ld, st;        // real side of the user's array (ld for pre, st for post)
  int64_t nrows;
  int n;              // transform length
  int M;              // complex workspace length per row
  int cosine;         // DCT vs DST
  int neg;            // fftpack: negate entries 2,4,... (pre for r2hc, post for hc2r)
  double fct;
  double e0, e1;      // element weights: DCT-I input ends (e0) / output ends (e1); DCT-II output
                      // element 0 (e0); DCT-III input element 0 (e0). From `ortho`, or the
                      // transposes' weights for the adjoints.
  const void *wa;     // W_{4n}^k, k < n   (DCT-II/III/IV)
  const void *wb;     // W_{8n}^k, k < 2n  (DCT-IV)
};

__device__ __forceinline__ int64_t roff(const Side &s, int64_t g) {
  int64_t off = 0;
  for (int d = 0; d < s.nbd; ++d) {
    const int64_t q = g / s.bshape[d];
    off += (g - q * s.bshape[d]) * s.bstride[d];
    g = q;
  }
  return off;
}

// pre: user real row -> complex workspace row of length M
template <typename T, int K>
__global__ void __launch_bounds__(256) r2r_pre_kernel(const __grid_constant__ R2RArgs a) {
  const T *in = reinterpret_cast<const T *>(a.in);
  cx<T> *ws = reinterpret_cast<cx<T> *>(a.out);
  const int n = a.n, M = a.M;
  const T e0 = T(a.e0);
  for (int64_t g = blockIdx.y; g < a.nrows; g += gridDim.y) {
    const int64_t o = roff(a.ld, g);
    const int64_t s = a.ld.axis_stride;
    auto x = [&](int j) { return in[o + j * s]; };
    cx<T> *w = ws + g * M;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < M; j += gridDim.x * blockDim.x) {
      cx<T> v = mk<T>(T(0), T(0));
      if constexpr (K == K_DCT1) {
        const int src = j < n ? j : M - j;
        T val = x(src);
        if (src == 0 || src == n - 1) val *= e0;
        v.x = val;
      } else if constexpr (K == K_DST1) {
        if (j >= 1 && j <= n) v.x = x(j - 1);
        else if (j >= n + 2) v.x = -x(M - 1 - j);
      } else if constexpr (K == K_DCT2) {
        const int h = (n + 1) / 2;
        const int src = j < h ? 2 * j : 2 * (n - 1 - j) + 1;
        T val = x(src);
        if (!a.cosine && (src & 1)) val = -val;
        v.x = val;
      } else if constexpr (K == K_DCT3) {
        // x'' = x with x_0 scaled by sqrt2 (ortho), reversed for DST; V_j = (x''_j - i x''_{n-j}) e^{i pi j/2n}
        auto xpp = [&](int q) {
          const int src = a.cosine ? q : n - 1 - q;
          T val = x(src);
          if (src == 0) val *= e0;
          return val;
        };
        const T re = xpp(j), im = j == 0 ? T(0) : -xpp(n - j);
        const cx<T> t = reinterpret_cast<const cx<T> *>(a.wa)[j];  // e^{-i pi j/2n}
        v = cj<T>(mulc<T>(mk<T>(re, im), t));  // conj(V_j): the FFT then gives conj(IDFT)
      } else if constexpr (K == K_DCT4) {
        if (j < n) {
          const T val = a.cosine ? x(j) : x(n - 1 - j);
          v = scl<T>(reinterpret_cast<const cx<T> *>(a.wa)[j], val);  // x_j e^{-i pi j/2n}
        }
      } else if constexpr (K == K_R2HC || K == K_HARTLEY) {
        T val = x(j);
        if (a.neg && j >= 2 && (j & 1) == 0) val = -val;
        v.x = val;
      } else if constexpr (K == K_HC2R) {
        // Hermitian spectrum from half-complex t, conjugated (the FFT then gives conj(IDFT))
        if (j == 0) {
          v.x = x(0);
        } else if (2 * j < n) {
          v = mk<T>(x(2 * j - 1), -x(2 * j));
        } else if (2 * j == n) {
          v.x = x(n - 1);
        } else {
          const int k = n - j;
          v = mk<T>(x(2 * k - 1), x(2 * k));
        }
      }
      w[j] = v;
    }
  }
}

// post: complex spectrum row -> user real row
template <typename T, int K>
__global__ void __launch_bounds__(256) r2r_post_kernel(const __grid_constant__ R2RArgs a) {
  const cx<T> *ws = reinterpret_cast<const cx<T> *>(a.in);
  T *out = reinterpret_cast<T *>(a.out);
  const int n = a.n, M = a.M;
  const T fct = T(a.fct);
  const T e0 = T(a.e0), e1 = T(a.e1);
  for (int64_t g = blockIdx.y; g < a.nrows; g += gridDim.y) {
    const int64_t o = roff(a.st, g);
    const int64_t s = a.st.axis_stride;
    const cx<T> *W = ws + g * M;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
      T y;
      if constexpr (K == K_DCT1) {
        y = W[k].x * fct;
        if (k == 0 || k == n - 1) y *= e1;
      } else if constexpr (K == K_DST1) {
        y = -W[k + 1].y * fct;
      } else if constexpr (K == K_DCT2) {
        const int kk = a.cosine ? k : n - 1 - k;
        const cx<T> t = reinterpret_cast<const cx<T> *>(a.wa)[kk];
        y = T(2) * (W[kk].x * t.x - W[kk].y * t.y) * fct;
        if (k == 0) y *= e0;
      } else if constexpr (K == K_DCT3) {
        const int j = (k & 1) ? n - 1 - (k >> 1) : (k >> 1);
        y = W[j].x * fct;
        if (!a.cosine && (k & 1)) y = -y;
      } else if constexpr (K == K_DCT4) {
        const cx<T> t = reinterpret_cast<const cx<T> *>(a.wb)[2 * k + 1];  // e^{-i pi (2k+1)/4n}
        y = T(2) * (W[k].x * t.x - W[k].y * t.y) * fct;
        if (!a.cosine && (k & 1)) y = -y;
      } else if constexpr (K == K_R2HC) {
        if (k == 0) y = W[0].x;
        else if (k & 1) y = W[(k + 1) >> 1].x;
        else y = W[k >> 1].y;
        y *= fct;
      } else if constexpr (K == K_HC2R) {
        y = W[k].x * fct;
        if (a.neg && k >= 2 && (k & 1) == 0) y = -y;
      } else if constexpr (K == K_HARTLEY) {
        if (k == 0 || 2 * k == n) y = W[k].x;
        else if (2 * k < n) y = W[k].x + W[k].y;
        else y = W[n - k].x - W[n - k].y;
        y *= fct;
      }
      out[o + k * s] = y;
    }
  }
}

dim3 pw_grid(int64_t nrows, int per_row) {
  unsigned gx = unsigned((per_row + 255) / 256);
  if (gx > 4096) gx = 4096;
  int64_t gy = std::min<int64_t>(nrows, 16384 / int64_t(gx) + 1);
  if (gy > 65535) gy = 65535;
  return dim3(gx, unsigned(gy));
}

template <typename T> void launch_pre(int K, const R2RArgs &a, cudaStream_t st) {
  const dim3 g = pw_grid(a.nrows, a.M);
  switch (K) {
    case K_DCT1: r2r_pre_kernel<T, K_DCT1><<<g, 256, 0, st>>>(a); break;
    case K_DST1: r2r_pre_kernel<T, K_DST1><<<g, 256, 0, st>>>(a); break;
    case K_DCT2: r2r_pre_kernel<T, K_DCT2><<<g, 256, 0, st>>>(a); break;
    case K_DCT3: r2r_pre_kernel<T, K_DCT3><<<g, 256, 0, st>>>(a); break;
    case K_DCT4: r2r_pre_kernel<T, K_DCT4><<<g, 256, 0, st>>>(a); break;
    case K_R2HC: r2r_pre_kernel<T, K_R2HC><<<g, 256, 0, st>>>(a); break;
    case K_HC2R: r2r_pre_kernel<T, K_HC2R><<<g, 256, 0, st>>>(a); break;
    default: r2r_pre_kernel<T, K_HARTLEY><<<g, 256, 0, st>>>(a); break;
  }
  note_launch();
  RG_CUDA(cudaGetLastError());
}

template <typename T> void launch_post(int K, const R2RArgs &a, cudaStream_t st) {
  const dim3 g = pw_grid(a.nrows, a.n);
  switch (K) {
    case K_DCT1: r2r_post_kernel<T, K_DCT1><<<g, 256, 0, st>>>(a); break;
    case K_DST1: r2r_post_kernel<T, K_DST1><<<g, 256, 0, st>>>(a); break;
    case K_DCT2: r2r_post_kernel<T, K_DCT2><<<g, 256, 0, st>>>(a); break;
    case K_DCT3: r2r_post_kernel<T, K_DCT3><<<g, 256, 0, st>>>(a); break;
    case K_DCT4: r2r_post_kernel<T, K_DCT4><<<g, 256, 0, st>>>(a); break;
    case K_R2HC: r2r_post_kernel<T, K_R2HC><<<g, 256, 0, st>>>(a); break;
    case K_HC2R: r2r_post_kernel<T, K_HC2R><<<g, 256, 0, st>>>(a); break;
    default: r2r_post_kernel<T, K_HARTLEY><<<g, 256, 0, st>>>(a); break;
  }
  note_launch();
  RG_CUDA(cudaGetLastError());
}

// Fused DCT-II/III kernels can be switched off (ROCKET_GPU_FUSED_DCT=0) to compare against the
// three-kernel route.
bool fused_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("ROCKET_GPU_FUSED_DCT");
    return !(e && e[0] == '0');
  }();
  return on;
}

// One real-to-real axis job through a complex workspace.
void r2r_axis(DType dt, int K, int64_t n, const void *in, const Side &ld, void *out, const Side &sd,
              int64_t nrows, bool cosine, bool neg, double fct, double e0, double e1, cudaStream_t st) {
  int64_t M = n;
  if (K == K_DCT1) M = 2 * (n - 1);
  if (K == K_DST1) M = 2 * (n + 1);
  if (K == K_DCT4) M = 2 * n;
  RG_CHECK(M >= 1, RG_ERR_ARG, "zero-length FFT requested");
  RG_CHECK(M < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "transform length too large");
  if ((K == K_DCT2 || K == K_DCT3) && fused_enabled() && n % 2 == 0) {
    // one kernel, the reference's reduction (T_dcst23, rocket_fft/_pocketfft_hdronly.h:2987-3061:
    // a real FFT of the reordered input) on the half-length complex FFT: Makhoul reordering +
    // r2c split + post-twiddle (type II), pre-twiddled half spectrum + c2r merge + reordering
    // (type III); only compile-time-length kernels implement it
    detail::Job j{};
    j.dt = dt;
    j.op = K == K_DCT2 ? OP_DCT2_HALF : OP_DCT3_HALF;
    j.n = j.nin = j.nout = int(n);
    j.L = int(n / 2);
    j.Lsm = j.L + 1;
    j.in = in;
    j.out = out;
    j.ld = ld;
    j.st = sd;
    j.nrows = nrows;
    j.fct = fct;
    j.e0 = e0;
    j.flags = cosine ? 0 : 2;
    if (detail::fixed_job_ok(j)) {
      j.aux = get_roots(uint64_t(4 * n), uint64_t(n), dt);
      j.aux2 = get_roots(uint64_t(n), uint64_t(n / 4 + 1), dt);
      detail::run_job(j, st);
      return;
    }
  }
  if ((K == K_DCT2 || K == K_DCT3) && fused_enabled() && detail::fits_core(n, dt)) {
    // one kernel: the reordering / twiddles of the reduction fused into the on-chip FFT's load
    // and store phases
    detail::Job j{};
    j.dt = dt;
    j.op = K == K_DCT2 ? OP_DCT2 : OP_DCT3;
    j.n = j.L = j.Lsm = j.nin = j.nout = int(n);
    j.in = in;
    j.out = out;
    j.ld = ld;
    j.st = sd;
    j.nrows = nrows;
    j.fct = fct;
    j.e0 = e0;
    j.flags = cosine ? 0 : 2;
    j.aux = get_roots(uint64_t(4 * n), uint64_t(n), dt);
    detail::run_job(j, st);
    return;
  }
  DevBuf ws(size_t(nrows) * size_t(M) * cx_size(dt), st);
  R2RArgs a{};
  a.in = in;
  a.out = ws.get();
  a.ld = ld;
  a.st = sd;
  a.nrows = nrows;
  a.n = int(n);
  a.M = int(M);
  a.cosine = cosine;
  a.neg = neg;
  a.fct = fct;
  a.e0 = e0;
  a.e1 = e1;
  if (K == K_DCT2 || K == K_DCT3 || K == K_DCT4) a.wa = get_roots(uint64_t(4 * n), uint64_t(n), dt);
  if (K == K_DCT4) a.wb = get_roots(uint64_t(8 * n), uint64_t(2 * n), dt);
  if (dt == DType::F32)
    launch_pre<float>(K, a, st);
  else
    launch_pre<double>(K, a, st);
  const Side w = detail::contiguous_rows(nrows, M);
  detail::c2c_rows(dt, M, ws.get(), w, ws.get(), w, nrows, false, false, 1.0, st);
  a.in = ws.get();
  a.out = out;
  if (dt == DType::F32)
    launch_post<float>(K, a, st);
  else
    launch_post<double>(K, a, st);
}

// general_nd over the axes of a real array with a per-axis job (fct on the first axis only)
template <class F>
void real_nd(const NdArray &in, const NdArray &out, const Axes &axes, double fct, F job) {
  if (detail::any_zero(in.shape)) return;
  for (size_t k = 0; k < axes.size(); ++k) {
    const NdArray &src = k == 0 ? in : out;
    const int ax = int(axes[k]);
    const detail::Batch b = detail::make_batch(in.shape, src.stride, out.stride, ax);
    const Side ld = detail::make_side(src.stride[ax], b.shape, b.s_in);
    const Side sd = detail::make_side(out.stride[ax], b.shape, b.s_out);
    job(in.shape[ax], src.data, ld, out.data, sd, b.nrows, k == 0 ? fct : 1.0);
  }
}

// r2r_genuine_hartley combine: for every half-spectrum position p (C order) with mirror q,
// the state the reference's serial loop leaves (HDR:4080-4089): out[p] = re+im, out[q] = re-im,
// where a pair inside the half is written by its later member and a self-mirror ends as re-im.
struct GenArgs {
  const void *spec;  // C-contiguous half spectrum
  void *out;
  int ndim, last;
  uint32_t revmask;
  int64_t shape[kMaxDims], ostride[kMaxDims];
  int64_t half, total;
};

template <typename T> __global__ void __launch_bounds__(256) hartley_gen_kernel(const __grid_constant__ GenArgs a) {
  const cx<T> *sp = reinterpret_cast<const cx<T> *>(a.spec);
  T *out = reinterpret_cast<T *>(a.out);
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < a.total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    int64_t rem = idx, po = 0, qo = 0, qlin = 0, mul = 1;
    bool outside = false;
    for (int k = a.ndim - 1; k >= 0; --k) {
      const int64_t ext = (k == a.last) ? a.half : a.shape[k];
      const int64_t q0 = rem / ext;
      const int64_t pos = rem - q0 * ext;
      rem = q0;
      int64_t qp = pos;
      if ((a.revmask >> k) & 1u) qp = pos == 0 ? 0 : a.shape[k] - pos;
      if (k == a.last && qp >= a.half) outside = true;
      po += pos * a.ostride[k];
      qo += qp * a.ostride[k];
      qlin += qp * mul;
      mul *= ext;
    }
    const cx<T> v = sp[idx];
    if (outside || qlin < idx) {
      out[po] = v.x + v.y;
      out[qo] = v.x - v.y;
    } else if (qlin == idx) {
      out[po] = v.x - v.y;
    }
  }
}

}  // namespace

bool dct2_eigdiv_3d(const float *in, float *out, int64_t n0, int64_t n1, int64_t n2, const float *lam,
                    cudaStream_t st) {
  NdArray a, b;
  a.data = const_cast<float *>(in);
  b.data = out;
  a.shape = b.shape = {n0, n1, n2};
  a.stride = b.stride = {n1 * n2, n2, 1};
  const Axes axes = {0, 1, 2};
  // the last axis' job, checked before any work: it must run in the compile-time kernel
  const detail::Batch bl = detail::make_batch(b.shape, b.stride, b.stride, 2);
  detail::Job j{};
  j.dt = DType::F32;
  j.op = OP_DCT2_HALF;
  j.n = j.nin = j.nout = int(n2);
  j.L = int(n2 / 2);
  j.Lsm = j.L + 1;
  j.in = out;
  j.out = out;
  j.ld = detail::make_side(1, bl.shape, bl.s_in);
  j.st = detail::make_side(1, bl.shape, bl.s_out);
  j.nrows = bl.nrows;
  j.fct = 1.0;
  j.e0 = 1.0;
  j.flags = kFlagEigDiv;
  j.aux_n = int(n1);
  j.aux_s = int(n0);
  j.aux3 = lam;
  if (n2 % 2 != 0 || !fused_enabled() || n0 * n1 >= (int64_t(1) << 31) || bl.nrows != n0 * n1 ||
      !detail::fixed_job_ok(j))
    return false;
  j.aux = get_roots(uint64_t(4 * n2), uint64_t(n2), DType::F32);
  j.aux2 = get_roots(uint64_t(n2), uint64_t(n2 / 4 + 1), DType::F32);
  real_nd(a, b, {0, 1}, 1.0, [&](int64_t n, const void *src, const Side &ld, void *dst, const Side &sd, int64_t rows,
                                 double f) {
    r2r_axis(DType::F32, K_DCT2, n, src, ld, dst, sd, rows, true, false, f, 1.0, 1.0, st);
  });
  detail::run_job(j, st);
  return true;
}

void exec_dcst(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, int type, bool cosine,
               double fct, bool ortho, cudaStream_t st, bool adjoint) {
  const double r2 = 1.4142135623730951, h2 = 0.7071067811865476;
  int K = type == 1 ? (cosine ? K_DCT1 : K_DST1) : type == 2 ? K_DCT2 : type == 3 ? K_DCT3 : K_DCT4;
  // element weights of the reference's `ortho` (HDR:2931-2947, 3040-3045)
  double e0 = 1, e1 = 1;
  if (K == K_DCT1 && ortho) e0 = r2, e1 = h2;
  if (K == K_DCT2 && ortho) e0 = h2;
  if (K == K_DCT3 && ortho) e0 = r2;
  if (adjoint) {
    // transposes: DCT-II^T = DCT-III with input element 0 weighted 2 (sqrt2 with ortho);
    // DCT-III^T = DCT-II with output element 0 weighted 1/2 (1/sqrt2 with ortho);
    // DCT-I^T weights the input ends by 2 and the output ends by 1/2 (ortho DCT-I, DST-I and
    // types 4 are their own transposes)
    RG_CHECK(cosine || type == 1 || type == 4, RG_ERR_UNSUPPORTED, "adjoint of DST-II/III is not provided");
    if (K == K_DCT2) K = K_DCT3, e0 = ortho ? r2 : 2.0;
    else if (K == K_DCT3) K = K_DCT2, e0 = ortho ? h2 : 0.5;
    else if (K == K_DCT1 && !ortho) e0 = 2.0, e1 = 0.5;
  }
  real_nd(in, out, axes, fct, [&](int64_t n, const void *src, const Side &ld, void *dst, const Side &sd, int64_t rows,
                                  double f) { r2r_axis(dt, K, n, src, ld, dst, sd, rows, cosine, false, f, e0, e1, st); });
}

void exec_r2r_fftpack(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool r2h, bool forward,
                      double fct, cudaStream_t st) {
  // forward: r2hc, with entries 2,4,... of the input negated when !r2h;
  // backward: hc2r, with entries 2,4,... of the output negated when r2h
  const int K = forward ? K_R2HC : K_HC2R;
  const bool neg = forward ? !r2h : r2h;
  real_nd(in, out, axes, fct, [&](int64_t n, const void *src, const Side &ld, void *dst, const Side &sd, int64_t rows,
                                  double f) { r2r_axis(dt, K, n, src, ld, dst, sd, rows, true, neg, f, 1, 1, st); });
}

void exec_hartley(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool genuine, double fct,
                  cudaStream_t st) {
  if (detail::any_zero(in.shape) || axes.empty()) return;
  if (!genuine || axes.size() == 1) {
    real_nd(in, out, axes, fct, [&](int64_t n, const void *src, const Side &ld, void *dst, const Side &sd,
                                    int64_t rows, double f) {
      r2r_axis(dt, K_HARTLEY, n, src, ld, dst, sd, rows, true, false, f, 1, 1, st);
    });
    return;
  }
  // genuine: r2c over the axes into a C-contiguous half spectrum, then the mirror combine
  RG_CHECK(in.shape.size() <= size_t(kMaxDims), RG_ERR_UNSUPPORTED, "too many dimensions");
  const int last = int(axes.back());
  std::vector<int64_t> hs = in.shape;
  hs[last] = hs[last] / 2 + 1;
  int64_t total = 1;
  for (int64_t v : hs) total *= v;
  DevBuf tmp(size_t(total) * cx_size(dt), st);
  NdArray t;
  t.data = tmp.get();
  t.shape = hs;
  t.stride.assign(hs.size(), 1);
  for (int d = int(hs.size()) - 2; d >= 0; --d) t.stride[d] = t.stride[d + 1] * hs[d + 1];
  exec_r2c(dt, in, t, axes, true, fct, st);
  GenArgs g{};
  g.spec = tmp.get();
  g.out = out.data;
  g.ndim = int(in.shape.size());
  g.last = last;
  for (uint64_t a : axes) g.revmask |= 1u << a;
  for (int d = 0; d < g.ndim; ++d) {
    g.shape[d] = in.shape[d];
    g.ostride[d] = out.stride[d];
  }
  g.half = hs[last];
  g.total = total;
  int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 32);
  if (dt == DType::F32)
    hartley_gen_kernel<float><<<unsigned(blocks), 256, 0, st>>>(g);
  else
    hartley_gen_kernel<double><<<unsigned(blocks), 256, 0, st>>>(g);
  note_launch();
  RG_CUDA(cudaGetLastError());
}

}  // namespace rg
