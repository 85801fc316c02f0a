// Batched complex FFTs of uneven lengths in one persistent launch.
//
// A plan holds, for a list of lengths, one work item per transform. Each CTA of the persistent
// kernel takes items from an atomic counter (items sorted by estimated cost, largest first) and
// runs the whole transform itself:
//   DIRECT     n <= Lmax, 13-smooth: load, on-chip passes, store
//   FOUR       n = n1 * n2 (both <= Lmax): columns of length n1 through shared memory into a
//              workspace row (with the W_n^{j2 k1} twiddle), then rows of length n2 to the output
//   BLUE       other n: Bluestein with m = good_size(2n - 1) (on chip when m <= Lmax, else m
//              itself in two passes), chirp products and the spectrum product in between
// Inputs and outputs are flat concatenations of the rows. The plan owns its tables and the
// workspace (one region per item), so execution allocates nothing and can be captured in a CUDA
// graph. Lmax, the threads and register budget per CTA and the four-step split policy are
// chosen by timing the candidates on the plan's own lengths (rocketgpu_batch_create with
// autotune).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "rg_batch.hpp"
#include "rg_error.hpp"
#include "rg_exec_detail.hpp"
#include "rg_axis_kernel.cuh"
#include "rg_launch.hpp"

namespace rg {

namespace {

enum ItemType : int { IT_DIRECT = 0, IT_FOUR = 1, IT_BLUE_DIRECT = 2, IT_BLUE_FOUR = 3 };

struct Item {
  int type;
  int n, n1, n2, m;
  int core0, core1;          // FFTCore indices: DIRECT/BLUE_DIRECT: core0 (length n or m);
                             // FOUR/BLUE_FOUR: core0 = n1, core1 = n2
  int tw_shift;
  const void *tw_lo, *tw_hi; // split twiddles of W_N, N = n (FOUR) or m (BLUE_FOUR)
  const void *bk, *bkf;      // Bluestein chirp (n) and spectrum (m)
  int64_t in_off, out_off, ws_off;
};

struct BatchArgs {
  const Item *items;
  const FFTCore *cores;
  int count;
  const void *in;
  void *out;
  void *ws;
  int *counter;
  int conj;       // backward transform: conjugate on load and on store
  double fct;
  int Lmax, pitch, ps;
};

// Row pitch (complex elements) of a shared-memory row of length len: index i at i + (i >> ps),
// the pitch odd modulo the bank width (same rule as the axis kernels).
__device__ __forceinline__ int rowpitch(int len, int ps, int mod) {
  int p = len + ((len - 1) >> ps) + 1;
  p += (1 - p % mod + mod) % mod;
  return p;
}

template <typename T> struct K {
  const BatchArgs &a;
  cx<T> *s0, *s1;
  const T fct;
  const bool bwd;  // backward transform
  int pitch;  // pitch of the rows currently in shared memory
  static constexpr int kMod = 128 / int(sizeof(cx<T>));

  // rows of length len fitting the shared buffers (capacity: one padded row of Lmax)
  __device__ int rows_for(int len) {
    pitch = rowpitch(len, a.ps, kMod);
    return max(1, a.pitch / pitch);
  }

  // rows x len complex elements from global (row r at base + r*rstride + i*estride) into
  // shared buffer s0, optionally conjugated, optionally times conj(bk[i]) (i < n) / zero beyond.
  // Each thread issues kBatch loads before its first shared store, so that kBatch loads per
  // thread are in flight (one at a time leaves the pass bound by memory latency).
  static constexpr int kBatch = 8;
  __device__ void load(const cx<T> *base, int rows, int len, int64_t rstride, int64_t estride, bool conj_in,
                       const cx<T> *bk = nullptr, int nvalid = 1 << 30) {
    const int total = rows * len;
    const int nth = blockDim.x;
    for (int e0 = threadIdx.x; e0 < total; e0 += nth * kBatch) {
      cx<T> v[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * nth;
        v[u] = mk<T>(T(0), T(0));
        if (e < total) {
          const int r = e / len, i = e - r * len;
          if (i < nvalid) {
            v[u] = base[r * rstride + i * estride];
            if (conj_in) v[u].y = -v[u].y;
            if (bk) v[u] = mulc<T>(v[u], bk[i]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * nth;
        if (e < total) {
          const int r = e / len, i = e - r * len;
          s0[sidx(r, i, pitch, a.ps)] = v[u];
        }
      }
    }
    __syncthreads();
  }

  __device__ cx<T> *fft(int rows, const FFTCore &core) { return fft_rows<T>(s0, s1, rows, pitch, a.ps, core); }

  // rows x len from shared `res` to global (row r at base + r*rstride + i*estride); optional
  // four-step twiddle W_N^{(col0 + r) * i}; optional conj/fct; optional *bk (y = conj(F*bk), bk
  // indexed like the output: bk[r*rstride + i*estride]).
  // colwalk: consecutive threads take consecutive rows (rows adjacent in memory, rstride 1).
  // Elements at offsets r*rstride + i*estride >= lim are not stored.
  __device__ void store(const cx<T> *res, cx<T> *base, int rows, int len, int64_t rstride, int64_t estride,
                        bool conj_out, T scale, const cx<T> *lo = nullptr, const cx<T> *hi = nullptr, int shift = 0,
                        int col0 = 0, const cx<T> *bk = nullptr, int nvalid = 1 << 30, bool colwalk = false,
                        int64_t lim = INT64_MAX) {
    const int total = rows * len;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      int r, i;
      if (colwalk) {
        i = e / rows;
        r = e - i * rows;
      } else {
        r = e / len;
        i = e - r * len;
      }
      if (i >= nvalid || r * rstride + i * estride >= lim) continue;
      cx<T> v = res[sidx(r, i, pitch, a.ps)];
      if (lo) v = mul<T>(v, split_twiddle<T>(lo, hi, shift, uint32_t(col0 + r) * uint32_t(i)));
      if (bk) v = cj<T>(mul<T>(v, bk[r * rstride + i * estride]));
      v = mk<T>(v.x * scale, (conj_out ? -v.y : v.y) * scale);
      base[r * rstride + i * estride] = v;
    }
    __syncthreads();
  }

  // Columns c0 .. c0+rows-1 of src viewed as n1 x n2 (column j2 = c0 + r: elements j1 at
  // src[j1 * n2 + j2]) into shared buffer s0 as rows of length n1; the Bluestein chirp and
  // padding use the global index j = j1 * n2 + j2. Columns fastest: consecutive threads read
  // consecutive j2 of one j1 (coalesced); kBatch loads per thread in flight before the shared
  // stores.
  __device__ void load_cols(const cx<T> *src, int n1, int n2, int c0, int rows, bool conj_in, const cx<T> *bk_in,
                            int nvalid_in) {
    const int total = rows * n1;
    const int nth = blockDim.x;
    for (int e0 = threadIdx.x; e0 < total; e0 += nth * kBatch) {
      cx<T> v[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * nth;
        v[u] = mk<T>(T(0), T(0));
        if (e < total) {
          const int j1 = e / rows, r = e - j1 * rows;
          const int j = j1 * n2 + c0 + r;
          if (j < nvalid_in) {
            v[u] = src[j];
            if (conj_in) v[u].y = -v[u].y;
            if (bk_in) v[u] = mulc<T>(v[u], bk_in[j]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * nth;
        if (e < total) {
          const int j1 = e / rows, r = e - j1 * rows;
          s0[sidx(r, j1, pitch, a.ps)] = v[u];
        }
      }
    }
    __syncthreads();
  }

  // Bluestein convolution of length m = m1 * m2 in three passes over one workspace w (m
  // elements), y = conj(F(W) bk) * scale with W = conj(F(x conj(bk)) bkf) -- the same product
  // as two full four-step FFTs, with the inverse's row FFTs run in the same residency as the
  // forward's:
  //   columns j2:  DFT_m1 over j1 of x[j1 m2 + j2] conj(bk) (zero from n on), times
  //                W_m^{j2 k1}, to w[k1 m2 + j2]
  //   rows k1:     DFT_m2 over j2 gives F(a)[k1 + m1 k2] along the row; times bkf there,
  //                conjugated: W[k1 + m1 k2]; DFT_m2 over k2, times W_m^{q k1}, back to
  //                w[k1 m2 + q]
  //   columns q:   DFT_m1 over k1 gives F(W)[m2 p + q]; outputs j = m2 p + q < n to y, times bk,
  //                conjugated and scaled
  // (F(W)[m2 p + q] = sum_k1 W_m1^{p k1} W_m^{q k1} sum_k2 W[k1 + m1 k2] W_m2^{q k2}.)
  __device__ void blue_conv(const cx<T> *x, cx<T> *y, cx<T> *w, int n, int m1, int m2, const FFTCore &c1,
                            const FFTCore &c2, const cx<T> *lo, const cx<T> *hi, int shift, const cx<T> *bk,
                            const cx<T> *bkf, bool conj_in, bool conj_out, T scale) {
    const int tbA = rows_for(m1);
    for (int c0 = 0; c0 < m2; c0 += tbA) {
      const int rows = min(tbA, m2 - c0);
      load_cols(x, m1, m2, c0, rows, conj_in, bk, n);
      cx<T> *res = fft(rows, c1);
      store(res, w + c0, rows, m1, 1, m2, false, T(1), lo, hi, shift, c0, nullptr, 1 << 30, true);
    }
    __syncthreads();
    const int tbB = rows_for(m2);
    for (int k0 = 0; k0 < m1; k0 += tbB) {
      const int rows = min(tbB, m1 - k0);
      load(w + int64_t(k0) * m2, rows, m2, m2, 1, false);
      cx<T> *res = fft(rows, c2);
      // spectrum product into s0 (the next FFT's input); rows fastest, so that the bkf reads
      // (index k1 + m1 k2) are consecutive
      for (int e = threadIdx.x; e < rows * m2; e += blockDim.x) {
        const int i = e / rows, r = e - i * rows;
        const int si = sidx(r, i, pitch, a.ps);
        s0[si] = cj<T>(mul<T>(res[si], bkf[(k0 + r) + int64_t(m1) * i]));
      }
      __syncthreads();
      res = fft(rows, c2);
      store(res, w + int64_t(k0) * m2, rows, m2, m2, 1, false, T(1), lo, hi, shift, k0);
    }
    __syncthreads();
    rows_for(m1);
    for (int c0 = 0; c0 < m2; c0 += tbA) {
      const int rows = min(tbA, m2 - c0);
      load_cols(w, m1, m2, c0, rows, false, nullptr, 1 << 30);
      cx<T> *res = fft(rows, c1);
      store(res, y + c0, rows, m1, 1, m2, conj_out, scale, nullptr, nullptr, 0, 0, bk + c0, 1 << 30, true, n - c0);
    }
  }

  // dst = DFT_n(src) for n = n1 * n2 through `tmp` (column pass, then row pass)
  __device__ void four_step(const cx<T> *src, cx<T> *dst, cx<T> *tmp, int n1, int n2, const FFTCore &c1,
                            const FFTCore &c2, const cx<T> *lo, const cx<T> *hi, int shift, bool conj_in,
                            bool conj_out, T scale) {
    const int tbA = rows_for(n1);
    for (int c0 = 0; c0 < n2; c0 += tbA) {
      const int rows = min(tbA, n2 - c0);
      load_cols(src, n1, n2, c0, rows, conj_in, nullptr, 1 << 30);
      cx<T> *res = fft(rows, c1);
      store(res, tmp + c0, rows, n1, 1, n2, false, T(1), lo, hi, shift, c0, nullptr, 1 << 30, true);
    }
    __syncthreads();
    const int tbB = rows_for(n2);
    for (int k0 = 0; k0 < n1; k0 += tbB) {
      const int rows = min(tbB, n1 - k0);
      load(tmp + int64_t(k0) * n2, rows, n2, n2, 1, false);
      cx<T> *res = fft(rows, c2);
      store(res, dst + k0, rows, n2, 1, n1, conj_out, scale, nullptr, nullptr, 0, 0, nullptr, 1 << 30, true);
    }
  }
};

// Register budgets of the kernel instances: V = 0 up to 512 threads at one CTA per SM (128
// registers); V = 1 and 2 at 256 threads for 3 and 4 CTAs per SM (80 and 64 registers; single
// precision only, double precision spills at those budgets). The autotuner picks one.
constexpr int kBatchNT[3] = {512, 256, 256};
constexpr int kBatchMinB[3] = {1, 3, 4};

template <typename T, int V>
__global__ void __launch_bounds__(kBatchNT[V], kBatchMinB[V]) batch_kernel(const __grid_constant__ BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_item;
  cx<T> *s0 = reinterpret_cast<cx<T> *>(smraw);
  cx<T> *s1 = s0 + a.pitch;
  K<T> k{a, s0, s1, T(a.fct), a.conj != 0, a.pitch};
  const cx<T> *in = reinterpret_cast<const cx<T> *>(a.in);
  cx<T> *out = reinterpret_cast<cx<T> *>(a.out);
  cx<T> *ws = reinterpret_cast<cx<T> *>(a.ws);
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= a.count) break;
    const Item &I = a.items[it];
    const cx<T> *x = in + I.in_off;
    cx<T> *y = out + I.out_off;
    cx<T> *w = ws + I.ws_off;
    const cx<T> *lo = reinterpret_cast<const cx<T> *>(I.tw_lo), *hi = reinterpret_cast<const cx<T> *>(I.tw_hi);
    const cx<T> *bk = reinterpret_cast<const cx<T> *>(I.bk), *bkf = reinterpret_cast<const cx<T> *>(I.bkf);
    if (I.type == IT_DIRECT) {
      k.rows_for(I.n);
      k.load(x, 1, I.n, 0, 1, k.bwd);
      cx<T> *res = k.fft(1, a.cores[I.core0]);
      k.store(res, y, 1, I.n, 0, 1, k.bwd, k.fct);
    } else if (I.type == IT_FOUR) {
      k.four_step(x, y, w, I.n1, I.n2, a.cores[I.core0], a.cores[I.core1], lo, hi, I.tw_shift, k.bwd, k.bwd, k.fct);
    } else if (I.type == IT_BLUE_DIRECT) {
      // a = x conj(bk), padded to m; FFT; * bkf, conj; FFT; y = conj(F bk) (see OP_BLUE)
      k.rows_for(I.m);
      k.load(x, 1, I.m, 0, 1, k.bwd, bk, I.n);
      cx<T> *res = k.fft(1, a.cores[I.core0]);
      for (int i = threadIdx.x; i < I.m; i += blockDim.x) {
        const int si = sidx(0, i, k.pitch, a.ps);
        res[si] = cj<T>(mul<T>(res[si], bkf[i]));
      }
      __syncthreads();
      if (res != s0) {  // the next FFT starts from s0
        for (int i = threadIdx.x; i < I.m; i += blockDim.x) s0[sidx(0, i, k.pitch, a.ps)] = res[sidx(0, i, k.pitch, a.ps)];
        __syncthreads();
      }
      res = k.fft(1, a.cores[I.core0]);
      k.store(res, y, 1, I.n, 0, 1, k.bwd, k.fct, nullptr, nullptr, 0, 0, bk, I.n);
    } else {  // IT_BLUE_FOUR: workspace w holds m elements
      k.blue_conv(x, y, w, I.n, I.n1, I.n2, a.cores[I.core0], a.cores[I.core1], lo, hi, I.tw_shift, bk, bkf, k.bwd,
                  k.bwd, k.fct);
      __syncthreads();
    }
  }
}

size_t pitch_bytes(DType dt, int Lmax, int &pitch, int &ps) {
  ps = dt == DType::F32 ? 4 : 3;
  pitch = Lmax + ((Lmax - 1) >> ps) + 1;
  const int mod = 128 / int(cx_size(dt));
  while (pitch % mod != 1) ++pitch;
  return 2 * size_t(pitch) * cx_size(dt);
}

}  // namespace

struct BatchPlan {
  DType dt;
  bool forward;
  double fct;
  std::vector<int64_t> lengths;
  int64_t total = 0;  // sum of lengths
  // chosen configuration
  int Lmax = 4096, threads = 256, split = 0, variant = 0;
  std::string tune_log;
  // device state
  Item *d_items = nullptr;
  FFTCore *d_cores = nullptr;
  int *d_counter = nullptr;
  void *d_ws = nullptr;
  int count = 0;
  size_t smem = 0;
  int pitch = 0, ps = 0;
  int grid = 0;
  ~BatchPlan() {
    if (d_items) cudaFree(d_items);
    if (d_cores) cudaFree(d_cores);
    if (d_counter) cudaFree(d_counter);
    if (d_ws) cudaFree(d_ws);
  }
};

namespace {

bool onchip(int64_t n, int Lmax) { return n >= 1 && n <= Lmax && core_smooth(uint64_t(n)); }

// n = n1 * n2 with both on chip; policy 0: n1 as close to sqrt(n) as possible; policy 1: the
// smallest n1 that leaves n2 on chip (long contiguous rows in the second pass)
bool split(int64_t n, int Lmax, int policy, int &n1, int &n2) {
  int64_t best = 0;
  for (int64_t d = 1; d <= Lmax && d * d <= n * int64_t(Lmax); ++d) {
    if (n % d || !onchip(d, Lmax) || !onchip(n / d, Lmax)) continue;
    if (policy == 1) {
      best = d;
      break;
    }
    if (d * d <= n) best = d;
  }
  if (!best) return false;
  n1 = int(best);
  n2 = int(n / best);
  return true;
}

double cost(const Item &I) {
  switch (I.type) {
    case IT_DIRECT: return double(I.n);
    case IT_FOUR: return 3.0 * I.n;
    case IT_BLUE_DIRECT: return 2.0 * I.m;
    default: return 8.0 * I.m;
  }
}

const void *kernel_fn(DType dt, int variant) {
  if (dt != DType::F32) return reinterpret_cast<const void *>(&batch_kernel<double, 0>);
  switch (variant) {
    case 1: return reinterpret_cast<const void *>(&batch_kernel<float, 1>);
    case 2: return reinterpret_cast<const void *>(&batch_kernel<float, 2>);
    default: return reinterpret_cast<const void *>(&batch_kernel<float, 0>);
  }
}

// Build items, cores and workspace for one configuration (device memory owned by `p`).
void build(BatchPlan &p, int Lmax, int threads, int policy, int variant) {
  const DType dt = p.dt;
  RG_CHECK(variant >= 0 && variant < 3 && (variant == 0 || dt == DType::F32) && threads <= kBatchNT[variant],
           RG_ERR_INTERNAL, "batch kernel variant");
  p.Lmax = Lmax;
  p.threads = threads;
  p.split = policy;
  p.variant = variant;
  std::vector<Item> items;
  std::vector<FFTCore> cores;
  std::vector<int> core_len;
  auto core_id = [&](int L) {
    for (size_t i = 0; i < core_len.size(); ++i)
      if (core_len[i] == L) return int(i);
    cores.push_back(get_core(L, dt).core);
    core_len.push_back(L);
    return int(cores.size() - 1);
  };
  int64_t off = 0, wsoff = 0;
  for (int64_t n : p.lengths) {
    Item I{};
    I.n = int(n);
    I.in_off = I.out_off = off;
    I.ws_off = wsoff;
    if (onchip(n, Lmax)) {
      I.type = IT_DIRECT;
      I.core0 = core_id(int(n));
    } else if (core_smooth(uint64_t(n)) && split(n, Lmax, policy, I.n1, I.n2)) {
      I.type = IT_FOUR;
      I.core0 = core_id(I.n1);
      I.core1 = core_id(I.n2);
      const SplitTables t = get_split(uint64_t(n), dt);
      I.tw_lo = t.lo;
      I.tw_hi = t.hi;
      I.tw_shift = t.shift;
      wsoff += n;
    } else {
      const BlueTables &b = get_blue(uint64_t(n), dt);
      I.m = int(b.m);
      I.bk = b.bk;
      I.bkf = b.bkf;
      if (onchip(I.m, Lmax)) {
        I.type = IT_BLUE_DIRECT;
        I.core0 = core_id(I.m);
      } else {
        RG_CHECK(split(I.m, Lmax, policy, I.n1, I.n2), RG_ERR_UNSUPPORTED, "length too large for the batch kernel");
        I.type = IT_BLUE_FOUR;
        I.core0 = core_id(I.n1);
        I.core1 = core_id(I.n2);
        const SplitTables t = get_split(uint64_t(I.m), dt);
        I.tw_lo = t.lo;
        I.tw_hi = t.hi;
        I.tw_shift = t.shift;
        wsoff += int64_t(I.m);
      }
    }
    off += n;
    items.push_back(I);
  }
  std::stable_sort(items.begin(), items.end(), [](const Item &x, const Item &y) { return cost(x) > cost(y); });
  if (p.d_items) cudaFree(p.d_items);
  if (p.d_cores) cudaFree(p.d_cores);
  if (p.d_ws) cudaFree(p.d_ws);
  p.d_items = nullptr;
  p.d_cores = nullptr;
  p.d_ws = nullptr;
  RG_CUDA(cudaMalloc(&p.d_items, std::max<size_t>(items.size(), 1) * sizeof(Item)));
  RG_CUDA(cudaMemcpy(p.d_items, items.data(), items.size() * sizeof(Item), cudaMemcpyHostToDevice));
  RG_CUDA(cudaMalloc(&p.d_cores, std::max<size_t>(cores.size(), 1) * sizeof(FFTCore)));
  RG_CUDA(cudaMemcpy(p.d_cores, cores.data(), cores.size() * sizeof(FFTCore), cudaMemcpyHostToDevice));
  RG_CUDA(cudaMalloc(&p.d_ws, std::max<int64_t>(wsoff, 1) * cx_size(dt)));
  if (!p.d_counter) RG_CUDA(cudaMalloc(&p.d_counter, sizeof(int)));
  p.count = int(items.size());
  p.smem = pitch_bytes(dt, Lmax, p.pitch, p.ps);
  int dev = 0, sms = 0;
  RG_CUDA(cudaGetDevice(&dev));
  RG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const void *fn = kernel_fn(dt, variant);
  RG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(p.smem)));
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, p.smem));
  RG_CHECK(per_sm > 0, RG_ERR_UNSUPPORTED, "batch kernel does not fit on an SM");
  p.grid = sms * per_sm;
}

}  // namespace

void batch_exec(BatchPlan &p, const void *in, void *out, cudaStream_t st) {
  RG_CUDA(cudaMemsetAsync(p.d_counter, 0, sizeof(int), st));
  BatchArgs a{};
  a.items = p.d_items;
  a.cores = p.d_cores;
  a.count = p.count;
  a.in = in;
  a.out = out;
  a.ws = p.d_ws;
  a.counter = p.d_counter;
  a.conj = p.forward ? 0 : 1;
  a.fct = p.fct;
  a.Lmax = p.Lmax;
  a.pitch = p.pitch;
  a.ps = p.ps;
  if (p.dt != DType::F32)
    batch_kernel<double, 0><<<p.grid, p.threads, p.smem, st>>>(a);
  else if (p.variant == 1)
    batch_kernel<float, 1><<<p.grid, p.threads, p.smem, st>>>(a);
  else if (p.variant == 2)
    batch_kernel<float, 2><<<p.grid, p.threads, p.smem, st>>>(a);
  else
    batch_kernel<float, 0><<<p.grid, p.threads, p.smem, st>>>(a);
  note_launch();
  RG_CUDA(cudaGetLastError());
}

BatchPlan *batch_create(const int64_t *lengths, int64_t count, DType dt, bool forward, double fct, bool autotune) {
  RG_CHECK(count > 0, RG_ERR_ARG, "empty batch");
  std::unique_ptr<BatchPlan> p(new BatchPlan());
  p->dt = dt;
  p->forward = forward;
  p->fct = fct;
  for (int64_t i = 0; i < count; ++i) {
    RG_CHECK(lengths[i] >= 1 && lengths[i] < (int64_t(1) << 27), RG_ERR_ARG, "bad length in batch");
    p->lengths.push_back(lengths[i]);
    p->total += lengths[i];
  }
  struct Cand {
    int Lmax, threads, policy, variant;
  };
  // on-chip capacities whose two shared row buffers fit a CTA (8192: one CTA per SM, single
  // precision only); without the autotune, ROCKET_GPU_BATCH_LMAX picks one (default 4096)
  auto fits = [&](int Lmax) {
    int pitch = 0, ps = 0;
    return pitch_bytes(dt, Lmax, pitch, ps) <= max_smem_optin();
  };
  int lmax0 = 4096;
  if (const char *e = std::getenv("ROCKET_GPU_BATCH_LMAX")) {
    const int v = std::atoi(e);
    if ((v == 2048 || v == 4096 || v == 8192) && fits(v)) lmax0 = v;
  }
  // ROCKET_GPU_BATCH_TUNE=0 skips the autotune (the configuration then comes from the two
  // variables here); ROCKET_GPU_BATCH_CTAS (3 or 4, single precision) picks the 80- or
  // 64-register instance
  if (const char *e = std::getenv("ROCKET_GPU_BATCH_TUNE"))
    if (std::atoi(e) == 0) autotune = false;
  int var0 = 0;
  if (const char *e = std::getenv("ROCKET_GPU_BATCH_CTAS")) {
    const int v = std::atoi(e);
    if (dt == DType::F32 && (v == 3 || v == 4)) var0 = v - 2;
  }
  std::vector<Cand> cands = {{lmax0, 256, 0, var0}};
  if (autotune) {
    // every capacity x (threads, register budget) with the square-root split; then the other
    // split policy for the fastest of those
    cands.clear();
    for (int Lmax : {2048, 4096, 8192})
      if (fits(Lmax)) {
        cands.push_back({Lmax, 256, 0, 0});
        cands.push_back({Lmax, 512, 0, 0});
        if (dt == DType::F32) {
          cands.push_back({Lmax, 256, 0, 1});
          cands.push_back({Lmax, 256, 0, 2});
        }
      }
  }
  if (cands.size() == 1) {
    build(*p, cands[0].Lmax, cands[0].threads, cands[0].policy, cands[0].variant);
    return p.release();
  }
  // time every candidate on the plan's own lengths (random data, two runs each, best kept)
  void *din = nullptr, *dout = nullptr;
  const size_t bytes = size_t(p->total) * cx_size(dt);
  RG_CUDA(cudaMalloc(&din, bytes));
  RG_CUDA(cudaMalloc(&dout, bytes));
  RG_CUDA(cudaMemset(din, 0, bytes));
  cudaEvent_t e0, e1;
  RG_CUDA(cudaEventCreate(&e0));
  RG_CUDA(cudaEventCreate(&e1));
  std::ostringstream log;
  float best = 1e30f;
  Cand pick = cands[0];
  bool split_tried = false;
  try {
    for (size_t ci = 0; ci < cands.size(); ++ci) {
      const Cand c = cands[ci];
      build(*p, c.Lmax, c.threads, c.policy, c.variant);
      batch_exec(*p, din, dout, nullptr);  // warm-up
      float t = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {
        RG_CUDA(cudaEventRecord(e0, nullptr));
        batch_exec(*p, din, dout, nullptr);
        RG_CUDA(cudaEventRecord(e1, nullptr));
        RG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        RG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        t = std::min(t, ms);
      }
      log << "Lmax=" << c.Lmax << ",threads=" << c.threads << ",ctas=" << kBatchMinB[c.variant] << ",split=" << c.policy
          << ":" << t << "ms;";
      if (t < best) {
        best = t;
        pick = c;
      }
      if (ci + 1 == cands.size() && !split_tried) {
        split_tried = true;
        cands.push_back({pick.Lmax, pick.threads, 1, pick.variant});
      }
    }
  } catch (...) {
    cudaFree(din);
    cudaFree(dout);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaFree(din);
  cudaFree(dout);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  build(*p, pick.Lmax, pick.threads, pick.policy, pick.variant);
  log << "chosen Lmax=" << pick.Lmax << ",threads=" << pick.threads << ",ctas=" << kBatchMinB[pick.variant]
      << ",split=" << pick.policy;
  p->tune_log = log.str();
  return p.release();
}

void batch_destroy(BatchPlan *p) { delete p; }

std::string batch_info(const BatchPlan &p) {
  std::ostringstream s;
  int counts[4] = {0, 0, 0, 0};
  std::vector<Item> items(size_t(p.count));
  cudaMemcpy(items.data(), p.d_items, items.size() * sizeof(Item), cudaMemcpyDeviceToHost);
  for (const Item &I : items) counts[I.type]++;
  s << "{\"count\": " << p.count << ", \"elements\": " << p.total << ", \"Lmax\": " << p.Lmax
    << ", \"threads\": " << p.threads << ", \"min_ctas_per_sm\": " << kBatchMinB[p.variant]
    << ", \"split_policy\": " << p.split << ", \"grid\": " << p.grid
    << ", \"direct\": " << counts[0] << ", \"four_step\": " << counts[1] << ", \"bluestein_onchip\": " << counts[2]
    << ", \"bluestein_four_step\": " << counts[3] << ", \"tune\": \"" << p.tune_log << "\"}";
  return s.str();
}

}  // namespace rg
