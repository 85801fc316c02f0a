// Axis-job kernel specialised for power-of-two core lengths (all passes radix 16/8/4/2).
//
// Differences from the generic axis_kernel (rg_axis_kernel.cuh):
//  * every division is a shift or a mask (L, L/R, Ns and the rows-per-CTA TB are powers of 2);
//  * the first radix pass reads its butterfly inputs straight from global memory and the last
//    pass writes its outputs straight to global memory, so a two-pass length (e.g. 256 =
//    16 x 16) touches shared memory once instead of three times. Butterflies are assigned to
//    threads row-fastest ("column" walk, rows adjacent in memory) or position-fastest ("row"
//    walk, contiguous axis) per pass so that these global accesses coalesce;
//  * ops: C2C, C2C_TW (four-step first pass), R2C_EVEN (staged split + store), C2R_EVEN
//    (staged load + merge).
#pragma once
#include "rg_axis_kernel.cuh"

namespace rg {

struct P2 {  // per-CTA constants
  int TB, lTB, rows, pitch, ps;
};

enum : int { SRC_SMEM = 0, SRC_GLOBAL = 1 };
enum : int { DST_SMEM = 0, DST_GLOBAL = 1 };
enum : int { MAP_ROW = 0, MAP_COL = 1 };

template <typename T, int OP, int R, int SRC, int DST, int MAP>
__device__ __forceinline__ void p2_pass(const KArgs &a, const P2 &c, const cx<T> *__restrict__ src,
                                        cx<T> *__restrict__ dst, const int64_t *roff_in,
                                        const int64_t *roff_out, const int *rowaux, const PassDesc &pd,
                                        const cx<T> *__restrict__ tw, int lLR, int lNs) {
  const int LR = pd.LR;
  const int Ns = pd.Ns;
  const int nbf = (MAP == MAP_COL ? c.TB : c.rows) * LR;
  const bool cin = a.conj_in != 0, cout = a.conj_out != 0;
  const T fct = T(a.fct);
  for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
    int r, j;
    if (MAP == MAP_COL) {
      r = bf & (c.TB - 1);
      j = bf >> c.lTB;
      if (r >= c.rows) continue;
    } else {
      r = bf >> lLR;
      j = bf & (LR - 1);
    }
    cx<T> v[R];
    if constexpr (SRC == SRC_GLOBAL) {
      const int64_t off = roff_in[r], s = a.ld.axis_stride;
#pragma unroll
      for (int k = 0; k < R; ++k) v[k] = load_unit<T, OP>(a.in, off, j + k * LR, s);
      if (OP == OP_C2C || OP == OP_C2C_TW) {
        if (cin) {
#pragma unroll
          for (int k = 0; k < R; ++k) v[k].y = -v[k].y;
        }
      }
    } else {
      const cx<T> *sr = src + r * c.pitch;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int i = j + k * LR;
        v[k] = sr[i + (i >> c.ps)];
      }
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
      const int64_t off = roff_out[r], s = a.st.axis_stride;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int i = base + (k << lNs);
        cx<T> x = v[k];
        if constexpr (OP == OP_C2C_TW) {
          x = mul<T>(x, split_twiddle<T>(reinterpret_cast<const cx<T> *>(a.aux),
                                         reinterpret_cast<const cx<T> *>(a.aux2), a.aux_s,
                                         uint32_t(rowaux[r]) * uint32_t(i)));
        }
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
          reinterpret_cast<cx<T> *>(a.out)[off + i * s] = mk<T>(x.x * fct, (cout ? -x.y : x.y) * fct);
        }
      }
    } else {
      cx<T> *dr = dst + r * c.pitch;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int i = base + (k << lNs);
        dr[i + (i >> c.ps)] = v[k];
      }
    }
  }
  __syncthreads();
}

template <typename T, int OP, int SRC, int DST, int MAP>
__device__ __forceinline__ void p2_dispatch(const KArgs &a, const P2 &c, const cx<T> *src, cx<T> *dst,
                                            const int64_t *ri, const int64_t *ro, const int *ra,
                                            const PassDesc &pd, const cx<T> *tw) {
  const int lLR = 31 - __clz(pd.LR), lNs = 31 - __clz(pd.Ns);
  switch (pd.R) {
    case 16: p2_pass<T, OP, 16, SRC, DST, MAP>(a, c, src, dst, ri, ro, ra, pd, tw, lLR, lNs); break;
    case 8: p2_pass<T, OP, 8, SRC, DST, MAP>(a, c, src, dst, ri, ro, ra, pd, tw, lLR, lNs); break;
    case 4: p2_pass<T, OP, 4, SRC, DST, MAP>(a, c, src, dst, ri, ro, ra, pd, tw, lLR, lNs); break;
    default: p2_pass<T, OP, 2, SRC, DST, MAP>(a, c, src, dst, ri, ro, ra, pd, tw, lLR, lNs); break;
  }
}

template <typename T, int OP>
__global__ void __launch_bounds__(512) pow2_kernel(const __grid_constant__ KArgs a, FastDiv dTB, FastDiv dIn,
                                                   FastDiv dOut) {
  static_assert(OP == OP_C2C || OP == OP_C2C_TW || OP == OP_R2C_EVEN || OP == OP_C2R_EVEN, "op");
  pdl_begin();
  extern __shared__ __align__(16) unsigned char smraw[];
  P2 c;
  c.TB = a.TB;
  c.lTB = 31 - __clz(a.TB);
  c.pitch = a.pitch;
  c.ps = a.ps;
  cx<T> *sm = reinterpret_cast<cx<T> *>(smraw);
  cx<T> *sm1 = sm + size_t(c.TB) * c.pitch;
  int64_t *roff_in = reinterpret_cast<int64_t *>(smraw + 2 * sizeof(cx<T>) * size_t(c.TB) * c.pitch);
  int64_t *roff_out = roff_in + c.TB;
  int *rowaux = reinterpret_cast<int *>(roff_out + c.TB);
  const int64_t row0 = int64_t(blockIdx.x) * c.TB;
  c.rows = int(min(int64_t(c.TB), a.nrows - row0));
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int r = tid; r < c.rows; r += nth) {
    roff_in[r] = side_offset(a.ld, row0 + r);
    roff_out[r] = side_offset(a.st, row0 + r);
    if (OP == OP_C2C_TW) rowaux[r] = int((row0 + r) % a.aux_n);
  }
  __syncthreads();
  const int L = a.core.L;
  const cx<T> *tw = reinterpret_cast<const cx<T> *>(a.core.tw);
  const int np = a.core.npass;

  cx<T> *cur = sm, *nxt = sm1;
  int p = 0;
  if constexpr (OP == OP_C2R_EVEN) {
    // staged Hermitian load + merge into conj(Z) (as the generic kernel)
    const int units = L + 1;
    const int64_t s = a.ld.axis_stride;
    for (int e = tid; e < c.TB * units; e += nth) {
      int r, i;
      walk(e, a.ld.colmap, c.TB, dTB, units, dIn, r, i);
      if (r >= c.rows) continue;
      cx<T> x = __ldg(reinterpret_cast<const cx<T> *>(a.in) + roff_in[r] + i * s);
      if (a.conj_in) x.y = -x.y;
      if (i == 0 || i == L) x.y = T(0);
      else x = scl<T>(x, T(a.bscale));
      sm[sidx(r, i, c.pitch, c.ps)] = x;
    }
    __syncthreads();
    const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);
    const int half = L / 2 + 1;
    for (int e = tid; e < c.rows * half; e += nth) {
      const int r = e / half;
      const int k = e - r * half;
      if (k == 0) {
        const cx<T> x0 = sm[sidx(r, 0, c.pitch, c.ps)], xl = sm[sidx(r, L, c.pitch, c.ps)];
        const cx<T> A = add<T>(x0, cj<T>(xl)), B = sub<T>(x0, cj<T>(xl));
        sm[sidx(r, 0, c.pitch, c.ps)] = cj<T>(add<T>(A, mposi<T>(B)));
      } else {
        const int kc = L - k;
        const cx<T> xk = sm[sidx(r, k, c.pitch, c.ps)], xc = sm[sidx(r, kc, c.pitch, c.ps)];
        const cx<T> A = add<T>(xk, cj<T>(xc)), B = sub<T>(xk, cj<T>(xc));
        const cx<T> u = mposi<T>(mulc<T>(B, w[k]));
        sm[sidx(r, k, c.pitch, c.ps)] = cj<T>(add<T>(A, u));
        if (kc != k) sm[sidx(r, kc, c.pitch, c.ps)] = sub<T>(A, u);
      }
    }
    __syncthreads();
  } else {
    // first pass straight from global memory
    const int map = a.ld.colmap ? MAP_COL : MAP_ROW;
    const bool last_direct = (np == 1) && (OP != OP_R2C_EVEN) && (a.ld.colmap == a.st.colmap);
    if (last_direct) {
      if (map == MAP_COL)
        p2_dispatch<T, OP, SRC_GLOBAL, DST_GLOBAL, MAP_COL>(a, c, nullptr, nullptr, roff_in, roff_out, rowaux, a.core.pass[0], tw);
      else
        p2_dispatch<T, OP, SRC_GLOBAL, DST_GLOBAL, MAP_ROW>(a, c, nullptr, nullptr, roff_in, roff_out, rowaux, a.core.pass[0], tw);
      return;
    }
    if (map == MAP_COL)
      p2_dispatch<T, OP, SRC_GLOBAL, DST_SMEM, MAP_COL>(a, c, nullptr, cur, roff_in, roff_out, rowaux, a.core.pass[0], tw);
    else
      p2_dispatch<T, OP, SRC_GLOBAL, DST_SMEM, MAP_ROW>(a, c, nullptr, cur, roff_in, roff_out, rowaux, a.core.pass[0], tw);
    p = 1;
  }
  // middle passes in shared memory (ping-pong)
  const int last_smem = (OP == OP_R2C_EVEN) ? np : np - 1;  // passes [p, last_smem) stay on chip
  for (; p < last_smem; ++p) {
    p2_dispatch<T, OP, SRC_SMEM, DST_SMEM, MAP_ROW>(a, c, cur, nxt, roff_in, roff_out, rowaux, a.core.pass[p], tw);
    cx<T> *t = cur;
    cur = nxt;
    nxt = t;
  }
  if constexpr (OP == OP_R2C_EVEN) {
    // split into X_0..X_L, then a staged store (as the generic kernel)
    const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);
    const int half = L / 2 + 1;
    for (int e = tid; e < c.rows * half; e += nth) {
      const int r = e / half;
      const int k = e - r * half;
      if (k == 0) {
        const cx<T> z0 = cur[sidx(r, 0, c.pitch, c.ps)];
        cur[sidx(r, 0, c.pitch, c.ps)] = mk<T>(z0.x + z0.y, T(0));
        cur[sidx(r, L, c.pitch, c.ps)] = mk<T>(z0.x - z0.y, T(0));
      } else {
        const int kc = L - k;
        const cx<T> zk = cur[sidx(r, k, c.pitch, c.ps)], zc = cj<T>(cur[sidx(r, kc, c.pitch, c.ps)]);
        const cx<T> E = scl<T>(add<T>(zk, zc), T(0.5));
        const cx<T> O = mnegi<T>(scl<T>(sub<T>(zk, zc), T(0.5)));
        const cx<T> t = mul<T>(w[k], O);
        cur[sidx(r, k, c.pitch, c.ps)] = add<T>(E, t);
        if (kc != k) cur[sidx(r, kc, c.pitch, c.ps)] = cj<T>(sub<T>(E, t));
      }
    }
    __syncthreads();
    const int units = L + 1;
    const int64_t s = a.st.axis_stride;
    const T fct = T(a.fct);
    const bool cout = a.conj_out != 0;
    constexpr int kBatch = 8;
    for (int e0 = tid; e0 < c.TB * units; e0 += nth * kBatch) {
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * nth;
        if (e >= c.TB * units) break;
        int r, i;
        walk(e, a.st.colmap, c.TB, dTB, units, dOut, r, i);
        if (r >= c.rows) continue;
        cx<T> x = cur[sidx(r, i, c.pitch, c.ps)];
        if (i != 0 && i != L) x = scl<T>(x, T(a.bscale));
        reinterpret_cast<cx<T> *>(a.out)[roff_out[r] + i * s] = mk<T>(x.x * fct, (cout ? -x.y : x.y) * fct);
      }
    }
  } else {
    // last pass straight to global memory
    if (a.st.colmap)
      p2_dispatch<T, OP, SRC_SMEM, DST_GLOBAL, MAP_COL>(a, c, cur, nullptr, roff_in, roff_out, rowaux, a.core.pass[np - 1], tw);
    else
      p2_dispatch<T, OP, SRC_SMEM, DST_GLOBAL, MAP_ROW>(a, c, cur, nullptr, roff_in, roff_out, rowaux, a.core.pass[np - 1], tw);
  }
}

}  // namespace rg
