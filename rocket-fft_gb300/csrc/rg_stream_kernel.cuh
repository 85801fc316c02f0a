// Persistent, software-pipelined axis kernel for power-of-two core lengths.
//
// The one-shot kernels (rg_axis_kernel.cuh, rg_pow2_kernel.cuh) give each CTA one tile of TB
// rows: load, compute, store, exit. Their loads are issued from registers, so an SM only has
// memory traffic in flight while its CTAs sit in the load phase, and the HBM pipe idles
// whenever the resident CTAs compute. This kernel decouples the two:
//
//  * grid = CTAs that fit at once (a multiple of the SM count); CTA b owns tiles
//    b, b + grid, b + 2 grid, ... (a tile = TB rows of one axis job);
//  * tile data is moved global -> shared with cp.async (LDGSTS: asynchronous, no registers
//    held), S - 1 tiles ahead of the one being computed, into a ring of S stage buffers;
//  * the radix passes run stage -> work -> stage ... in shared memory and the last pass writes
//    straight to global memory (C2C, C2R_EVEN) or, for R2C_EVEN, all passes and the split
//    run on chip followed by a staged store.
//
// The row offsets of a tile (both sides) are decomposed over the batch dims once per tile and
// kept in a ring of S + 1 slots, one tile ahead of the loads that use them.
//
// Ops: C2C (conjugation on load / store, fct), R2C_EVEN, C2R_EVEN (with the interior-bin scale
// of the adjoints). Loads are 8- or 16-byte copies of whole complex units, or for R2C_EVEN
// inputs that are not pair-aligned, two copies of one real each. Shared layout per stage: TB
// rows of `pitch` complex slots, element i of row r at r * pitch + i + (i >> ps).
#pragma once
#include "rg_pow2_kernel.cuh"

namespace rg {

struct StreamParams {
  int pair_ok;  // R2C_EVEN: (x_2i, x_2i+1) may be copied as one unit (contiguous, aligned)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return uint32_t(__cvta_generic_to_shared(p));
}

template <int BYTES> __device__ __forceinline__ void cp_async(uint32_t dst, const void *src) {
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// One radix-R Stockham pass reading shared memory (optionally conjugating), writing shared
// memory or global memory (DST_GLOBAL: C2C / C2R_EVEN output through the row offsets `ro`).
template <typename T, int OP, int R, int DST, int MAP>
__device__ __forceinline__ void sk_pass(const KArgs &a, int TB, int lTB, int rows, const cx<T> *__restrict__ src,
                                        cx<T> *__restrict__ dst, const int64_t *ro, const PassDesc &pd,
                                        const cx<T> *__restrict__ tw, bool cin) {
  const int pitch = a.pitch, ps = a.ps;
  const int LR = pd.LR, Ns = pd.Ns;
  const int lLR = 31 - __clz(LR), lNs = 31 - __clz(Ns);
  const int nbf = (MAP == MAP_COL ? TB : rows) * LR;
  for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
    int r, j;
    if (MAP == MAP_COL) {
      r = bf & (TB - 1);
      j = bf >> lTB;
      if (r >= rows) continue;
    } else {
      r = bf >> lLR;
      j = bf & (LR - 1);
    }
    cx<T> v[R];
    const cx<T> *sr = src + r * pitch;
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int i = j + k * LR;
      v[k] = sr[i + (i >> ps)];
    }
    if (cin) {
#pragma unroll
      for (int k = 0; k < R; ++k) v[k].y = -v[k].y;
    }
    const int m = j & (Ns - 1);
    if (Ns > 1) {
      const cx<T> *t = tw + pd.tw + m;
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = mul<T>(v[k], t[(k - 1) << lNs]);
    }
    dft<T, R>(v);
    const int base = ((j - m) * R) + m;
    if constexpr (DST == DST_GLOBAL) {
      const int64_t off = ro[r], s = a.st.axis_stride;
      const T fct = T(a.fct);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int i = base + (k << lNs);
        const cx<T> x = v[k];
        if constexpr (OP == OP_C2R_EVEN) {
          // (x_2i, x_2i+1) = (Re F_i, -Im F_i) * fct
          T *out = reinterpret_cast<T *>(a.out);
          const T re = x.x * fct, im = -x.y * fct;
          if (s == 1 && (reinterpret_cast<uintptr_t>(out + off) & (sizeof(cx<T>) - 1)) == 0) {
            reinterpret_cast<cx<T> *>(out + off)[i] = mk<T>(re, im);
          } else {
            out[off + 2 * i * s] = re;
            out[off + (2 * i + 1) * s] = im;
          }
        } else {
          reinterpret_cast<cx<T> *>(a.out)[off + i * s] = mk<T>(x.x * fct, (a.conj_out ? -x.y : x.y) * fct);
        }
      }
    } else {
      cx<T> *dr = dst + r * pitch;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int i = base + (k << lNs);
        dr[i + (i >> ps)] = v[k];
      }
    }
  }
  __syncthreads();
}

template <typename T, int OP, int DST, int MAP>
__device__ __forceinline__ void sk_dispatch(const KArgs &a, int TB, int lTB, int rows, const cx<T> *src, cx<T> *dst,
                                            const int64_t *ro, const PassDesc &pd, const cx<T> *tw, bool cin) {
  switch (pd.R) {
    case 16: sk_pass<T, OP, 16, DST, MAP>(a, TB, lTB, rows, src, dst, ro, pd, tw, cin); break;
    case 8: sk_pass<T, OP, 8, DST, MAP>(a, TB, lTB, rows, src, dst, ro, pd, tw, cin); break;
    case 4: sk_pass<T, OP, 4, DST, MAP>(a, TB, lTB, rows, src, dst, ro, pd, tw, cin); break;
    default: sk_pass<T, OP, 2, DST, MAP>(a, TB, lTB, rows, src, dst, ro, pd, tw, cin); break;
  }
}

template <typename T, int OP>
__device__ __forceinline__ void sk_last(const KArgs &a, int TB, int lTB, int rows, const cx<T> *src, const int64_t *ro,
                                        const PassDesc &pd, const cx<T> *tw, bool cin) {
  if (a.st.colmap)
    sk_dispatch<T, OP, DST_GLOBAL, MAP_COL>(a, TB, lTB, rows, src, nullptr, ro, pd, tw, cin);
  else
    sk_dispatch<T, OP, DST_GLOBAL, MAP_ROW>(a, TB, lTB, rows, src, nullptr, ro, pd, tw, cin);
}

template <typename T, int OP, int S>
__global__ void __launch_bounds__(512) stream_kernel(const __grid_constant__ KArgs a, FastDiv dIn, FastDiv dOut,
                                                     StreamParams sp) {
  static_assert(OP == OP_C2C || OP == OP_R2C_EVEN || OP == OP_C2R_EVEN, "op");
  extern __shared__ __align__(16) unsigned char smraw[];
  const int TB = a.TB, lTB = 31 - __clz(a.TB);
  const int pitch = a.pitch, ps = a.ps;
  const size_t tile = size_t(TB) * pitch;
  cx<T> *stage0 = reinterpret_cast<cx<T> *>(smraw);
  cx<T> *work = stage0 + S * tile;
  int64_t *roff = reinterpret_cast<int64_t *>(work + tile);  // [S + 1][2][TB]
  const int64_t ntiles = (a.nrows + TB - 1) / TB;
  const int tid = threadIdx.x, nth = blockDim.x;
  const int L = a.core.L;
  const int np = a.core.npass;
  const cx<T> *tw = reinterpret_cast<const cx<T> *>(a.core.tw);
  const int64_t gstep = gridDim.x;

  // row offsets of local tile `it` into slot it % (S + 1)
  auto fill_roff = [&](int64_t it) {
    const int64_t t = int64_t(blockIdx.x) + it * gstep;
    if (t >= ntiles) return;
    int64_t *ri = roff + (it % (S + 1)) * 2 * TB;
    for (int r = tid; r < TB; r += nth) {
      const int64_t g = t * TB + r;
      if (g < a.nrows) {
        ri[r] = side_offset(a.ld, g);
        ri[TB + r] = side_offset(a.st, g);
      }
    }
  };
  // cp.async of local tile `it` into stage it % S (one commit group per call, possibly empty)
  auto issue = [&](int64_t it) {
    const int64_t t = int64_t(blockIdx.x) + it * gstep;
    if (t < ntiles) {
      const int rows = int(min(int64_t(TB), a.nrows - t * TB));
      const int64_t *ri = roff + (it % (S + 1)) * 2 * TB;
      const uint32_t sbase = smem_u32(stage0 + (it % S) * tile);
      const int units = a.nin;
      const int total = TB * units;
      const int64_t s = a.ld.axis_stride;
      for (int e = tid; e < total; e += nth) {
        int r, i;
        if (a.ld.colmap) {
          i = e >> lTB;
          r = e & (TB - 1);
        } else {
          r = int(fdiv(uint32_t(e), dIn));
          i = e - r * units;
        }
        if (r >= rows) continue;
        const uint32_t d = sbase + uint32_t(sidx(r, i, pitch, ps)) * uint32_t(sizeof(cx<T>));
        if constexpr (OP == OP_R2C_EVEN) {
          const T *in = reinterpret_cast<const T *>(a.in) + ri[r];
          if (sp.pair_ok) {
            cp_async<sizeof(cx<T>)>(d, in + 2 * i);
          } else {
            cp_async<sizeof(T)>(d, in + 2 * i * s);
            cp_async<sizeof(T)>(d + uint32_t(sizeof(T)), in + (2 * i + 1) * s);
          }
        } else {
          cp_async<sizeof(cx<T>)>(d, reinterpret_cast<const cx<T> *>(a.in) + ri[r] + i * s);
        }
      }
    }
    cp_async_commit();
  };

  // prologue: offsets of tiles 0..S-1, loads of tiles 0..S-2
  for (int q = 0; q < S; ++q) fill_roff(q);
  __syncthreads();
  for (int q = 0; q < S - 1; ++q) issue(q);

  for (int64_t it = 0;; ++it) {
    const int64_t t = int64_t(blockIdx.x) + it * gstep;
    if (t >= ntiles) break;
    issue(it + S - 1);
    cp_async_wait<S - 1>();
    fill_roff(it + S);  // slot of tile it - 1, whose last reads ended before the previous barrier
    __syncthreads();

    const int rows = int(min(int64_t(TB), a.nrows - t * TB));
    const int64_t *ro = roff + (it % (S + 1)) * 2 * TB + TB;
    cx<T> *sb = stage0 + (it % S) * tile;

    if constexpr (OP == OP_C2C) {
      const bool cin = a.conj_in != 0;
      if (np == 1) {
        sk_last<T, OP>(a, TB, lTB, rows, sb, ro, a.core.pass[0], tw, cin);
      } else {
        sk_dispatch<T, OP, DST_SMEM, MAP_ROW>(a, TB, lTB, rows, sb, work, ro, a.core.pass[0], tw, cin);
        cx<T> *cur = work, *nxt = sb;
        for (int p = 1; p < np - 1; ++p) {
          sk_dispatch<T, OP, DST_SMEM, MAP_ROW>(a, TB, lTB, rows, cur, nxt, ro, a.core.pass[p], tw, false);
          cx<T> *x = cur;
          cur = nxt;
          nxt = x;
        }
        sk_last<T, OP>(a, TB, lTB, rows, cur, ro, a.core.pass[np - 1], tw, false);
      }
    } else if constexpr (OP == OP_C2R_EVEN) {
      // Hermitian merge of the raw X_0..X_L in the stage into conj(Z_0..Z_{L-1}), in place
      const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);
      const int half = L / 2 + 1;
      const bool cin = a.conj_in != 0;
      const T bsc = T(a.bscale);
      auto fetch = [&](int r, int i) {
        cx<T> x = sb[sidx(r, i, pitch, ps)];
        if (cin) x.y = -x.y;
        if (i == 0 || i == L) x.y = T(0);
        else x = scl<T>(x, bsc);
        return x;
      };
      for (int e = tid; e < rows * half; e += nth) {
        const int r = e / half;
        const int k = e - r * half;
        if (k == 0) {
          const cx<T> x0 = fetch(r, 0), xl = fetch(r, L);
          const cx<T> A = add<T>(x0, cj<T>(xl)), B = sub<T>(x0, cj<T>(xl));
          sb[sidx(r, 0, pitch, ps)] = cj<T>(add<T>(A, mposi<T>(B)));
        } else {
          const int kc = L - k;
          const cx<T> xk = fetch(r, k), xc = fetch(r, kc);
          const cx<T> A = add<T>(xk, cj<T>(xc)), B = sub<T>(xk, cj<T>(xc));
          const cx<T> u = mposi<T>(mulc<T>(B, w[k]));
          sb[sidx(r, k, pitch, ps)] = cj<T>(add<T>(A, u));
          if (kc != k) sb[sidx(r, kc, pitch, ps)] = sub<T>(A, u);
        }
      }
      __syncthreads();
      if (np == 1) {
        sk_last<T, OP>(a, TB, lTB, rows, sb, ro, a.core.pass[0], tw, false);
      } else {
        sk_dispatch<T, OP, DST_SMEM, MAP_ROW>(a, TB, lTB, rows, sb, work, ro, a.core.pass[0], tw, false);
        cx<T> *cur = work, *nxt = sb;
        for (int p = 1; p < np - 1; ++p) {
          sk_dispatch<T, OP, DST_SMEM, MAP_ROW>(a, TB, lTB, rows, cur, nxt, ro, a.core.pass[p], tw, false);
          cx<T> *x = cur;
          cur = nxt;
          nxt = x;
        }
        sk_last<T, OP>(a, TB, lTB, rows, cur, ro, a.core.pass[np - 1], tw, false);
      }
    } else {  // OP_R2C_EVEN
      cx<T> *cur = sb, *nxt = work;
      for (int p = 0; p < np; ++p) {
        sk_dispatch<T, OP, DST_SMEM, MAP_ROW>(a, TB, lTB, rows, cur, nxt, ro, a.core.pass[p], tw, false);
        cx<T> *x = cur;
        cur = nxt;
        nxt = x;
      }
      // split Z_0..Z_{L-1} into X_0..X_L, in place
      const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);
      const int half = L / 2 + 1;
      for (int e = tid; e < rows * half; e += nth) {
        const int r = e / half;
        const int k = e - r * half;
        if (k == 0) {
          const cx<T> z0 = cur[sidx(r, 0, pitch, ps)];
          cur[sidx(r, 0, pitch, ps)] = mk<T>(z0.x + z0.y, T(0));
          cur[sidx(r, L, pitch, ps)] = mk<T>(z0.x - z0.y, T(0));
        } else {
          const int kc = L - k;
          const cx<T> zk = cur[sidx(r, k, pitch, ps)], zc = cj<T>(cur[sidx(r, kc, pitch, ps)]);
          const cx<T> E = scl<T>(add<T>(zk, zc), T(0.5));
          const cx<T> O = mnegi<T>(scl<T>(sub<T>(zk, zc), T(0.5)));
          const cx<T> u = mul<T>(w[k], O);
          cur[sidx(r, k, pitch, ps)] = add<T>(E, u);
          if (kc != k) cur[sidx(r, kc, pitch, ps)] = cj<T>(sub<T>(E, u));
        }
      }
      __syncthreads();
      const int units = L + 1;
      const int64_t s = a.st.axis_stride;
      const T fct = T(a.fct);
      const T bsc = T(a.bscale);
      const bool cout = a.conj_out != 0;
      for (int e = tid; e < TB * units; e += nth) {
        int r, i;
        if (a.st.colmap) {
          i = e >> lTB;
          r = e & (TB - 1);
        } else {
          r = int(fdiv(uint32_t(e), dOut));
          i = e - r * units;
        }
        if (r >= rows) continue;
        cx<T> x = cur[sidx(r, i, pitch, ps)];
        if (i != 0 && i != L) x = scl<T>(x, bsc);
        reinterpret_cast<cx<T> *>(a.out)[ro[r] + i * s] = mk<T>(x.x * fct, (cout ? -x.y : x.y) * fct);
      }
      __syncthreads();
    }
  }
  cp_async_wait<0>();  // no copy may outlive the CTA (all remaining groups are empty)
}

}  // namespace rg
