// Axis-job kernel compiled for one power-of-two core length L = 2^E.
//
// The runtime-parameterised kernels (rg_axis_kernel.cuh, rg_pow2_kernel.cuh) carry every
// radix and pass shape in one binary and compute shared-memory and twiddle indices at run
// time; on GB300 they are bound by instruction issue (integer index arithmetic and
// instruction-cache misses), not by HBM. Here the pass schedule (the same radices as the host
// core plan, core_radices in rg_plan.cpp), the rows per CTA (TB), the thread count, the
// shared-memory pitch and every per-pass index are compile-time constants, so a butterfly's
// shared and twiddle accesses are immediate offsets from one base address and the kernel
// holds only the code of its own passes.
//
// Walks: COL = rows are adjacent columns of a strided axis (threads run across rows, TB rows
// give one 128-byte segment per position); ROW = rows are contiguous along the axis (threads
// run along the row). Both sides of the job walk the same way.
//
// Flows (pass 0 reads global memory directly, the last pass of C2C / C2R_EVEN writes it; one
// shared buffer A per CTA, passes in between run in place: all reads, barrier, all writes):
//   C2C       global -> A [-> A ...] -> global; backward = the forward core applied to
//             (im, re)-swapped data, swapped back on store (swap(F(swap(x))) = conj(F(conj(x))))
//   R2C_EVEN  real pairs -> A -> ... (all passes on chip), split into X_0..X_L, staged store
//   C2R_EVEN  staged Hermitian load, merge into conj(Z), passes, real pairs to global
//   DCT2/3    (DCT/DST types II and III by Makhoul's n-point complex FFT) staged load with the
//             reordering / pre-twiddle, passes, post-twiddle / un-reordering on the last store
#pragma once
#include "rg_axis_kernel.cuh"
#include "rg_pdl.cuh"

namespace rg {
namespace fx {

// radices of a power-of-two core 2^e, identical to core_radices(): 16^a, then 2/4/8, with
// 16^(a-1) * 8 * 4 instead of 16^a * 2
__host__ __device__ constexpr int np_of(int e) {
  return (e % 4 == 1 && e / 4 >= 1) ? e / 4 + 1 : e / 4 + (e % 4 ? 1 : 0);
}
__host__ __device__ constexpr int radix_of(int e, int p) {
  return (e % 4 == 1 && e / 4 >= 1) ? (p < e / 4 - 1 ? 16 : p == e / 4 - 1 ? 8 : 4)
         : (p < e / 4 ? 16 : e % 4 == 1 ? 2 : e % 4 == 2 ? 4 : 8);
}
__host__ __device__ constexpr int ns_of(int e, int p) {
  int n = 1;
  for (int q = 0; q < p; ++q) n *= radix_of(e, q);
  return n;
}
// offset of pass p's twiddles in the core table; the table has no entries for pass 0 (Ns = 1)
__host__ __device__ constexpr int tw_of(int e, int p) {
  int t = 0;
  for (int q = 1; q < p; ++q) t += (radix_of(e, q) - 1) * ns_of(e, q);
  return t;
}
// padded row pitch (as row_pitch() on the host): index i at i + (i >> ps), pitch = 1 mod the
// number of elements per 128-byte bank line
__host__ __device__ constexpr int pitch_of(int lsm, int ps, int esz) {
  int p = lsm + ((lsm - 1) >> ps) + 1;
  while (p % (128 / esz) != 1) ++p;
  return p;
}
// Column walk: lanes run across the TB rows first, then along the positions. A warp's shared
// access is served one 128-byte line of lanes at a time (16 complex64 or 8 complex128 lanes),
// which covers TB rows x line / TB positions when TB < line: lane (r, j) lands on slot
// pitch * r + j of the line, so the pitch must be line / TB modulo the line for the slots to be
// distinct (1 when TB >= line).
__host__ __device__ constexpr int pitch_col(int lsm, int ps, int esz, int TB) {
  const int line = 128 / esz;
  const int want = TB < line ? line / TB : 1;
  int p = lsm + ((lsm - 1) >> ps) + 1;
  while (p % line != want) ++p;
  return p;
}
__host__ __device__ constexpr int clampi(int x, int lo, int hi) { return x < lo ? lo : x > hi ? hi : x; }
// Row walk: when a bank line's worth of lanes spans several rows (g = L / 16 lanes per row in
// the first pass and the staged loops, g < elements per bank line), rows start g slots apart
// modulo the bank line so that the rows of one wavefront use disjoint banks.
__host__ __device__ constexpr int pitch_row(int lsm, int ps, int esz, int L) {
  const int line = 128 / esz;
  const int g = L / 16 < line ? L / 16 : line;
  const int want = g >= line ? 1 : g;
  int p = lsm + ((lsm - 1) >> ps) + 1;
  while (p % line != want) ++p;
  return p;
}

}  // namespace fx

template <typename T, int OP, int E, bool COL> struct FxCfg {
  static constexpr int L = 1 << E;
  static constexpr int NP = fx::np_of(E);
  static constexpr int ESZ = int(2 * sizeof(T));
  static constexpr int PS = sizeof(T) == 4 ? 4 : 3;
  static constexpr int LSM = (OP == OP_C2C || OP == OP_DCT2 || OP == OP_DCT3) ? L : L + 1;
  static constexpr int TB = COL ? (sizeof(T) == 4 ? (L <= 256 ? 16 : 8) : (L <= 256 ? 8 : 4))
                                : ((sizeof(T) == 4 ? 4096 : 2048) / L > 1 ? (sizeof(T) == 4 ? 4096 : 2048) / L : 1);
  static constexpr int PITCH = COL ? fx::pitch_col(LSM, PS, ESZ, TB) : fx::pitch_row(LSM, PS, ESZ, L);
  static constexpr int NT = fx::clampi(TB * L / 16, 64, 512);
  static constexpr int NBUF = OP == OP_C2C && NP == 1 ? 0 : 1;  // middle passes run in place
  static constexpr size_t SMEM = size_t(NBUF) * TB * PITCH * ESZ;
  // CTAs per SM the register allocation leaves room for (float32): 48 registers a thread up to
  // 256 threads, 64 at 512. Left to itself the allocator kept 54-128 registers for the ILP of the
  // butterflies and the DCT pre/post steps, and the register file then held these memory-bound
  // passes to 2-4 CTAs per SM. Measured on GB300 (256^3 / 512^3 inputs, L2-cold): r2c L=128 rows
  // 36.5 -> 33.0 us, DCT-III half length 512^3 416 -> 278 us, batched r2c of 2^12 points 0.51 ->
  // 0.65 of the HBM copy bandwidth; the slowest change was +2 % (a strided L=256 c2c pass).
  static constexpr int MINB = sizeof(T) != 4 ? 1 : NT >= 512 ? 2 : NT == 256 ? 5 : NT == 128 ? 10 : 21;
  static_assert(NT % TB == 0 && NT / TB >= 1, "threads per row");
};

// Row offset of row g (< 2^32) through 32-bit reciprocal divisions.
__device__ __forceinline__ int64_t side_offset32(const Side &s, uint32_t g) {
  int64_t off = 0;
  for (int d = 0; d < s.nbd; ++d) {
    const uint32_t q = d + 1 < s.nbd ? fdiv(g, s.bdiv[d]) : 0u;
    off += int64_t(g - q * uint32_t(s.bshape[d])) * s.bstride[d];
    g = q;
  }
  return off;
}

// Padded shared position of element i = j + k * STEP (k compile-time): linear in k whenever
// STEP is a multiple of the pad period.
template <int PS, int STEP> __device__ __forceinline__ int fx_pos(int j, int k) {
  if constexpr (STEP % (1 << PS) == 0) {
    return j + (j >> PS) + k * (STEP + (STEP >> PS));
  } else {
    const int i = j + k * STEP;
    return i + (i >> PS);
  }
}

enum : int { FX_SMEM = 0, FX_GLOBAL = 1 };

// Butterfly bf of pass p: its row and position.
template <int TB, int LR, bool COL> __device__ __forceinline__ void fx_rj(int bf, int &r, int &j) {
  if constexpr (COL) {
    r = bf & (TB - 1);
    j = bf / TB;
  } else {
    r = bf / LR;
    j = bf & (LR - 1);
  }
}

// Inputs of butterfly (r, j) of pass p: gathered from global memory (pass 0) or shared memory,
// twiddled and transformed in registers.
template <typename T, int OP, int E, int P, bool COL, bool BWD, int SRC, typename C = FxCfg<T, OP, E, COL>>
__device__ __forceinline__ void fx_compute(const KArgs &a, uint32_t row0, int r, int j, const cx<T> *__restrict__ src,
                                           const cx<T> *__restrict__ tw, bool pair_ok,
                                           cx<T> (&v)[fx::radix_of(E, P)]) {
  constexpr int L = C::L, R = fx::radix_of(E, P), LR = L / R, NS = fx::ns_of(E, P), TWO = fx::tw_of(E, P);
  constexpr int PS = C::PS, PITCH = C::PITCH;
  if constexpr (SRC == FX_GLOBAL) {
    const int64_t s = a.ld.axis_stride;
    const int64_t off = side_offset32(a.ld, row0 + uint32_t(r));
    const uint64_t once = input_policy((a.flags & kFlagStream) != 0);
    if constexpr (OP == OP_R2C_EVEN) {
      const T *in = reinterpret_cast<const T *>(a.in) + off;
      if (pair_ok) {
        const cx<T> *p = reinterpret_cast<const cx<T> *>(in) + j;
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = ld_in(p + k * LR, once);
      } else {
        const T *p = in + 2 * int64_t(j) * s;
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = mk<T>(ld_in(p + 2 * k * LR * s, once), ld_in(p + (2 * k * LR + 1) * s, once));
      }
    } else {
      const cx<T> *p = reinterpret_cast<const cx<T> *>(a.in) + off + int64_t(j) * s;
      const int64_t step = int64_t(LR) * s;
#pragma unroll
      for (int k = 0; k < R; ++k) v[k] = ld_in(p + k * step, once);
      if constexpr (BWD) {
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = mk<T>(v[k].y, v[k].x);
      }
    }
  } else {
    const cx<T> *sp = src + r * PITCH;
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = sp[fx_pos<PS, LR>(j, k)];
  }
  if constexpr (NS > 1) {
    const cx<T> *t = tw + TWO + (j & (NS - 1));
#pragma unroll
    for (int k = 1; k < R; ++k) v[k] = mul<T>(v[k], __ldg(t + (k - 1) * NS));
  }
  dft<T, R>(v);
}

// Outputs of butterfly (r, j) of pass p: to shared memory, or (last pass of C2C / C2R_EVEN)
// to global memory with the op's output conversion.
template <typename T, int OP, int E, int P, bool COL, bool BWD, int DST, typename C = FxCfg<T, OP, E, COL>>
__device__ __forceinline__ void fx_emit(const KArgs &a, uint32_t row0, int r, int j, cx<T> *__restrict__ dst,
                                        bool scale, bool pair_ok, const cx<T> (&v)[fx::radix_of(E, P)]) {
  constexpr int R = fx::radix_of(E, P), NS = fx::ns_of(E, P);
  constexpr int PS = C::PS, PITCH = C::PITCH;
  const int m = j & (NS - 1);
  const int base = (j - m) * R + m;
  if constexpr (DST == FX_GLOBAL) {
    const int64_t s = a.st.axis_stride;
    const int64_t off = side_offset32(a.st, row0 + uint32_t(r));
    const T fct = T(a.fct);
    if constexpr (OP == OP_DCT2) {
      // y_pos = 2 Re(e^{-i pi kk / 2n} V_kk) * fct, pos = kk (DCT) or n-1-kk (DST); pos 0 x e0
      constexpr int L = C::L;
      T *out = reinterpret_cast<T *>(a.out) + off;
      const cx<T> *tw2 = reinterpret_cast<const cx<T> *>(a.aux);
      const bool sine = (a.flags & 2) != 0;
      const T e0 = T(a.e0);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int kk = base + k * NS;
        const cx<T> t = __ldg(tw2 + kk);
        T y = T(2) * (v[k].x * t.x - v[k].y * t.y) * fct;
        const int pos = sine ? L - 1 - kk : kk;
        if (pos == 0) y *= e0;
        out[pos * s] = y;
      }
    } else if constexpr (OP == OP_DCT3) {
      // y_2j = Re v_j (j < n/2), y_2(n-1-j)+1 = Re v_j (j >= n/2); DST: odd outputs negated
      constexpr int L = C::L;
      T *out = reinterpret_cast<T *>(a.out) + off;
      const bool sine = (a.flags & 2) != 0;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int jj = base + k * NS;
        const bool odd = jj >= L / 2;
        const int pos = odd ? 2 * (L - 1 - jj) + 1 : 2 * jj;
        const T y = v[k].x * fct;
        out[pos * s] = (sine && odd) ? -y : y;
      }
    } else if constexpr (OP == OP_DCT3_HALF) {
      // v_2i = Re F_i, v_2i+1 = -Im F_i (c2r of the half spectrum), then y_2j = v_j (j < n/2),
      // y_2(n-1-j)+1 = v_j (j >= n/2); DST: odd outputs negated. n = 2L.
      constexpr int N = 2 * C::L;
      T *out = reinterpret_cast<T *>(a.out) + off;
      const bool sine = (a.flags & 2) != 0;
      auto put = [&](int jj, T y) {
        const bool odd = jj >= N / 2;
        const int pos = odd ? 2 * (N - 1 - jj) + 1 : 2 * jj;
        out[pos * s] = (sine && odd) ? -y : y;
      };
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int i = base + k * NS;
        put(2 * i, v[k].x * fct);
        put(2 * i + 1, -v[k].y * fct);
      }
    } else if constexpr (OP == OP_C2R_EVEN) {
      // (x_2i, x_2i+1) = (Re F_i, -Im F_i) * fct
      T *out = reinterpret_cast<T *>(a.out) + off;
      if (pair_ok) {
        cx<T> *p = reinterpret_cast<cx<T> *>(out) + base;
#pragma unroll
        for (int k = 0; k < R; ++k) p[k * NS] = scale ? mk<T>(v[k].x * fct, -v[k].y * fct) : mk<T>(v[k].x, -v[k].y);
      } else {
        T *p = out + 2 * int64_t(base) * s;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          p[2 * k * NS * s] = v[k].x * fct;
          p[(2 * k * NS + 1) * s] = -v[k].y * fct;
        }
      }
    } else {
      cx<T> *p = reinterpret_cast<cx<T> *>(a.out) + off + int64_t(base) * s;
      const int64_t step = int64_t(NS) * s;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        cx<T> x = BWD ? mk<T>(v[k].y, v[k].x) : v[k];
        if (scale) x = scl<T>(x, fct);
        p[k * step] = x;
      }
    }
  } else {
    cx<T> *dp = dst + r * PITCH;
    if constexpr (NS % (1 << PS) == 0) {
      const int b0 = base + (base >> PS);
#pragma unroll
      for (int k = 0; k < R; ++k) dp[b0 + k * (NS + (NS >> PS))] = v[k];
    } else if constexpr (NS == 1 && ((1 << PS) % R) == 0) {
      const int b0 = base + (base >> PS);  // base = R * j: the R outputs share one pad block
#pragma unroll
      for (int k = 0; k < R; ++k) dp[b0 + k] = v[k];
    } else {
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int i = base + k * NS;
        dp[i + (i >> PS)] = v[k];
      }
    }
  }
}

// One radix pass p of the compile-time schedule. Rows r >= rows (tail tile) are skipped.
// INPL: source and destination are the same shared buffer; every butterfly of the CTA reads
// its inputs (and transforms them) before a barrier, then all write. C: the geometry (rows per
// CTA, threads, shared pitch); FxCfg for the axis kernels, the plane kernels bring their own.
template <typename T, int OP, int E, int P, bool COL, bool BWD, int SRC, int DST, bool INPL = false,
          typename C = FxCfg<T, OP, E, COL>>
__device__ __forceinline__ void fx_pass(const KArgs &a, uint32_t row0, int rows, const cx<T> *src, cx<T> *dst,
                                        const cx<T> *__restrict__ tw, bool scale, bool pair_ok) {
  constexpr int L = C::L, R = fx::radix_of(E, P), LR = L / R;
  constexpr int TB = C::TB, NT = C::NT;
  constexpr int NBF = TB * LR;
  constexpr int ITER = (NBF + NT - 1) / NT;
  if constexpr (!INPL) {
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
      const int bf = int(threadIdx.x) + it * NT;
      if (NBF % NT != 0 && bf >= NBF) break;
      int r, j;
      fx_rj<TB, LR, COL>(bf, r, j);
      if (r >= rows) continue;
      cx<T> v[R];
      fx_compute<T, OP, E, P, COL, BWD, SRC, C>(a, row0, r, j, src, tw, pair_ok, v);
      fx_emit<T, OP, E, P, COL, BWD, DST, C>(a, row0, r, j, dst, scale, pair_ok, v);
    }
  } else {
    static_assert(SRC == FX_SMEM && DST == FX_SMEM, "in-place passes stay on chip");
    cx<T> v[ITER][R];
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
      const int bf = int(threadIdx.x) + it * NT;
      int r, j;
      fx_rj<TB, LR, COL>(bf, r, j);
      if ((NBF % NT == 0 || bf < NBF) && r < rows) fx_compute<T, OP, E, P, COL, BWD, SRC, C>(a, row0, r, j, src, tw, pair_ok, v[it]);
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
      const int bf = int(threadIdx.x) + it * NT;
      int r, j;
      fx_rj<TB, LR, COL>(bf, r, j);
      if ((NBF % NT == 0 || bf < NBF) && r < rows) fx_emit<T, OP, E, P, COL, BWD, DST, C>(a, row0, r, j, dst, scale, pair_ok, v[it]);
    }
  }
}

// The split of one unit of the last R2C_EVEN pass: v1, v2 are the DFT outputs of the
// butterflies j1 = u and j2 = NS - u (u = 0: j1 = 0, j2 = NS / 2), whose outputs Z_{j + q NS}
// hold both members of every pair (k, L - k); put(k, X_k) receives every bin 0 <= k <= L once.
//     X_k = E + W_2L^k O,  X_{L-k} = conj(E - W_2L^k O),  E = (Z_k + conj Z_{L-k}) / 2,
//     O = -i (Z_k - conj Z_{L-k}) / 2,   X_0 = Re Z_0 + Im Z_0,  X_L = Re Z_0 - Im Z_0.
template <typename T, int L, int R, int NS, typename Put>
__device__ __forceinline__ void fx_split_unit(int u, const cx<T> (&v1)[R], const cx<T> (&v2)[R],
                                              const cx<T> *__restrict__ w, Put &&put) {
  const int j2 = u == 0 ? NS / 2 : NS - u;
  // Slot q of a unit: the pair (ka, L - ka), ka <= L / 2, from za = Z_ka, zb = Z_{L-ka}:
  //   u >= 1, q < R/2:   (u + q NS, v1[q], v2[R-1-q]);  q >= R/2: (j2 + (R-1-q) NS, v2[R-1-q], v1[q])
  //   u = 0:   q = 0: (0, v1[0], v1[0]) -- the split formula then gives X_0 and X_L;
  //            1 <= q < R/2: (q NS, v1[q], v1[R-q]);  q = R/2: (L/2, v1[R/2], v1[R/2]), one output;
  //            R/2 < q <= R: (NS/2 + (q-R/2-1) NS, v2[q-R/2-1], v2[R-1-(q-R/2-1)])
  // All lanes run the same R + 1 slots (the last only for u = 0); operands are selected, not
  // branched on, so the unit-0 lanes of a warp do not diverge.
  const bool u0 = u == 0;
#pragma unroll
  for (int q = 0; q <= R; ++q) {
    // general unit
    int kg = 0;
    cx<T> zag = v1[0], zbg = v1[0];
    if (q < R / 2) {
      kg = u + q * NS;
      zag = v1[q];
      zbg = v2[R - 1 - q];
    } else if (q < R) {
      kg = j2 + (R - 1 - q) * NS;
      zag = v2[R - 1 - q];
      zbg = v1[q];
    }
    // unit 0
    int k0;
    cx<T> za0, zb0;
    bool two0 = true;
    if (q == 0) {
      k0 = 0;
      za0 = v1[0];
      zb0 = v1[0];
    } else if (q < R / 2) {
      k0 = q * NS;
      za0 = v1[q];
      zb0 = v1[R - q];
    } else if (q == R / 2) {
      k0 = L / 2;
      za0 = v1[R / 2];
      zb0 = v1[R / 2];
      two0 = false;
    } else {
      const int qq = q - R / 2 - 1;
      k0 = NS / 2 + qq * NS;
      za0 = v2[qq];
      zb0 = v2[R - 1 - qq];
    }
    const int ka = u0 ? k0 : kg;
    const cx<T> za = u0 ? za0 : zag, zb = u0 ? zb0 : zbg;
    const bool two = u0 ? two0 : true;
    if (u0 || q < R) {
      const cx<T> zc = cj<T>(zb);
      const cx<T> Ev = scl<T>(add<T>(za, zc), T(0.5));
      const cx<T> O = mnegi<T>(scl<T>(sub<T>(za, zc), T(0.5)));
      const cx<T> t = mul<T>(__ldg(w + ka), O);
      put(ka, add<T>(Ev, t));
      if (two) put(L - ka, cj<T>(sub<T>(Ev, t)));
    }
  }
}

// Last pass of R2C_EVEN with the split fused in (last radix <= 8). Unit (r, u) transforms the
// butterflies j1 = u and j2 = NS - u of row r (fx_split_unit) and stores X straight to global
// memory.
template <typename T, int E, bool COL>
__device__ __forceinline__ void fx_r2c_last_split(const KArgs &a, uint32_t row0, int rows, const cx<T> *buf,
                                                  const cx<T> *__restrict__ tw) {
  using C = FxCfg<T, OP_R2C_EVEN, E, COL>;
  constexpr int L = C::L, P = C::NP - 1, R = fx::radix_of(E, P), LR = L / R, NS = fx::ns_of(E, P);
  constexpr int TWO = fx::tw_of(E, P);
  static_assert(NS == LR && R <= 8 && R >= 2, "last pass");
  constexpr int TB = C::TB, NT = C::NT, PS = C::PS, PITCH = C::PITCH;
  constexpr int UPR = LR / 2;  // units per row
  constexpr int NU = TB * UPR;
  constexpr int ITER = (NU + NT - 1) / NT;
  const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);
  const int64_t s = a.st.axis_stride;
  const T fct = T(a.fct), bsc = T(a.bscale);
  const bool cout = a.conj_out != 0;
  const bool plain = a.fct == 1.0 && a.bscale == 1.0 && !cout;
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int unit = int(threadIdx.x) + it * NT;
    if (NU % NT != 0 && unit >= NU) break;
    int r, u;
    if constexpr (COL) {
      r = unit & (TB - 1);
      u = unit / TB;
    } else {
      r = unit / UPR;
      u = unit % UPR;
    }
    if (r >= rows) continue;
    const int j1 = u, j2 = u == 0 ? NS / 2 : NS - u;
    cx<T> v1[R], v2[R];
    {
      const cx<T> *sp = buf + r * PITCH;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        v1[k] = sp[fx_pos<PS, LR>(j1, k)];
        v2[k] = sp[fx_pos<PS, LR>(j2, k)];
      }
      const cx<T> *t1 = tw + TWO + j1, *t2 = tw + TWO + j2;
#pragma unroll
      for (int k = 1; k < R; ++k) {
        v1[k] = mul<T>(v1[k], __ldg(t1 + (k - 1) * NS));
        v2[k] = mul<T>(v2[k], __ldg(t2 + (k - 1) * NS));
      }
      dft<T, R>(v1);
      dft<T, R>(v2);
    }
    cx<T> *p = reinterpret_cast<cx<T> *>(a.out) + side_offset32(a.st, row0 + uint32_t(r));
    fx_split_unit<T, L, R, NS>(u, v1, v2, w, [&](int i, cx<T> x) {
      if (!plain) {
        if (i != 0 && i != L) x = scl<T>(x, bsc);
        x = mk<T>(x.x * fct, (cout ? -x.y : x.y) * fct);
      }
      p[i * s] = x;
    });
  }
}

// Passes 1 .. NP-2 in place in buffer A (the first reads global memory or A, the last writes
// global memory or stays in A).
template <typename T, int OP, int E, bool COL, bool BWD, int P, int PEND, typename C = FxCfg<T, OP, E, COL>>
__device__ __forceinline__ void fx_middle(const KArgs &a, uint32_t row0, int rows, cx<T> *buf, const cx<T> *tw,
                                          bool scale, bool pair_ok) {
  if constexpr (P < PEND) {
    fx_pass<T, OP, E, P, COL, BWD, FX_SMEM, FX_SMEM, true, C>(a, row0, rows, buf, buf, tw, scale, pair_ok);
    __syncthreads();
    fx_middle<T, OP, E, COL, BWD, P + 1, PEND, C>(a, row0, rows, buf, tw, scale, pair_ok);
  }
}

template <typename T, int OP, int E, bool COL, bool BWD>
__global__ void __launch_bounds__(FxCfg<T, OP, E, COL>::NT, FxCfg<T, OP, E, COL>::MINB)
    fixed_kernel(const __grid_constant__ KArgs a, int pair_ok_i) {
  pdl_begin();
  using C = FxCfg<T, OP, E, COL>;
  constexpr int L = C::L, NP = C::NP, TB = C::TB, NT = C::NT, PS = C::PS, PITCH = C::PITCH;
  constexpr int TPR = NT / TB;  // threads per row in the staged loops
  extern __shared__ __align__(16) unsigned char smraw[];
  cx<T> *buf = reinterpret_cast<cx<T> *>(smraw);
  const uint32_t row0 = uint32_t(blockIdx.x) * TB;
  const int rows = int(min(int64_t(TB), a.nrows - int64_t(row0)));
  const cx<T> *tw = reinterpret_cast<const cx<T> *>(a.core.tw);
  const bool scale = a.fct != 1.0;
  const bool pair_ok = pair_ok_i != 0;
  const int tid = threadIdx.x;
  // staged loops: thread -> (row, first element), TPR threads per row
  const int sr = COL ? (tid & (TB - 1)) : tid / TPR;
  const int si0 = COL ? tid / TB : tid % TPR;
  const uint64_t once = input_policy((a.flags & kFlagStream) != 0);

  if constexpr (OP == OP_C2C) {
    if constexpr (NP == 1) {
      fx_pass<T, OP, E, 0, COL, BWD, FX_GLOBAL, FX_GLOBAL>(a, row0, rows, nullptr, nullptr, tw, scale, pair_ok);
    } else {
      fx_pass<T, OP, E, 0, COL, BWD, FX_GLOBAL, FX_SMEM>(a, row0, rows, nullptr, buf, tw, scale, pair_ok);
      __syncthreads();
      fx_middle<T, OP, E, COL, BWD, 1, NP - 1>(a, row0, rows, buf, tw, scale, pair_ok);
      fx_pass<T, OP, E, NP - 1, COL, BWD, FX_SMEM, FX_GLOBAL>(a, row0, rows, buf, nullptr, tw, scale, pair_ok);
    }
  } else if constexpr (OP == OP_R2C_EVEN) {
    fx_pass<T, OP, E, 0, COL, false, FX_GLOBAL, FX_SMEM>(a, row0, rows, nullptr, buf, tw, scale, pair_ok);
    __syncthreads();
    if constexpr (NP >= 2 && fx::radix_of(E, NP - 1) <= 8) {
      fx_middle<T, OP, E, COL, false, 1, NP - 1>(a, row0, rows, buf, tw, scale, pair_ok);
      fx_r2c_last_split<T, E, COL>(a, row0, rows, buf, tw);
    } else {
      fx_middle<T, OP, E, COL, false, 1, NP>(a, row0, rows, buf, tw, scale, pair_ok);
      // split Z_0..Z_{L-1} into X_0..X_L in place
      const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);
      constexpr int HALF = L / 2 + 1;
      for (int e = tid; e < rows * HALF; e += NT) {
        const int r = e / HALF;
        const int k = e - r * HALF;
        cx<T> *row = buf + r * PITCH;
        if (k == 0) {
          const cx<T> z0 = row[0];
          row[0] = mk<T>(z0.x + z0.y, T(0));
          row[L + (L >> PS)] = mk<T>(z0.x - z0.y, T(0));
        } else {
          const int kc = L - k;
          const cx<T> zk = row[k + (k >> PS)], zc = cj<T>(row[kc + (kc >> PS)]);
          const cx<T> Ev = scl<T>(add<T>(zk, zc), T(0.5));
          const cx<T> O = mnegi<T>(scl<T>(sub<T>(zk, zc), T(0.5)));
          const cx<T> u = mul<T>(__ldg(w + k), O);
          row[k + (k >> PS)] = add<T>(Ev, u);
          if (kc != k) row[kc + (kc >> PS)] = cj<T>(sub<T>(Ev, u));
        }
      }
      __syncthreads();
      // staged store of L + 1 bins per row; bins 0 and L carry no interior-bin scale
      constexpr int UNITS = L + 1;
      const int64_t s = a.st.axis_stride;
      const T fct = T(a.fct), bsc = T(a.bscale);
      const bool cout = a.conj_out != 0;
      const bool plain = !scale && a.bscale == 1.0 && !cout;
      if (sr < rows) {
        cx<T> *p = reinterpret_cast<cx<T> *>(a.out) + side_offset32(a.st, row0 + uint32_t(sr));
        const cx<T> *row = buf + sr * PITCH;
        if (plain) {
#pragma unroll 4
          for (int i = si0; i < UNITS; i += TPR) p[i * s] = row[i + (i >> PS)];
        } else {
          for (int i = si0; i < UNITS; i += TPR) {
            cx<T> x = row[i + (i >> PS)];
            if (i != 0 && i != L) x = scl<T>(x, bsc);
            p[i * s] = mk<T>(x.x * fct, (cout ? -x.y : x.y) * fct);
          }
        }
      }
    }
  } else if constexpr (OP == OP_DCT2 || OP == OP_DCT3) {
    const int64_t s = a.ld.axis_stride;
    const bool sine = (a.flags & 2) != 0;
    if constexpr (OP == OP_DCT2) {
      // Makhoul order: v_m = x_2m, v_{n-1-m} = x_2m+1 (DST: odd inputs negated), as complex
      // numbers with zero imaginary part; the thread loads the pairs m = first + q * TPR
      constexpr int HP = L / 2, NQ = (HP + TPR - 1) / TPR;
      if (sr < rows) {
        const T *p = reinterpret_cast<const T *>(a.in) + side_offset32(a.ld, row0 + uint32_t(sr));
        cx<T> xv[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int m = si0 + q * TPR;
          if (HP % TPR == 0 || m < HP) {
            if (pair_ok) xv[q] = ld_in(reinterpret_cast<const cx<T> *>(p) + m, once);
            else xv[q] = mk<T>(ld_in(p + 2 * m * s, once), ld_in(p + (2 * m + 1) * s, once));
          }
        }
        cx<T> *row = buf + sr * PITCH;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int m = si0 + q * TPR;
          if (HP % TPR == 0 || m < HP) {
            const int mc = L - 1 - m;
            row[m + (m >> PS)] = mk<T>(xv[q].x, T(0));
            row[mc + (mc >> PS)] = mk<T>(sine ? -xv[q].y : xv[q].y, T(0));
          }
        }
      }
    } else {
      // conj(V_i), V_i = (x''_i - i x''_{n-i}) e^{i pi i / 2n}, x''_q = x_q (DCT) or x_{n-1-q}
      // (DST), x''_n = 0; input element 0 weighted e0
      constexpr int NQ = (L + TPR - 1) / TPR;
      if (sr < rows) {
        const T *p = reinterpret_cast<const T *>(a.in) + side_offset32(a.ld, row0 + uint32_t(sr));
        const cx<T> *tw3 = reinterpret_cast<const cx<T> *>(a.aux);
        const T e0 = T(a.e0);
        cx<T> xv[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int i = si0 + q * TPR;
          if (L % TPR == 0 || i < L) {
            const int sa = sine ? L - 1 - i : i;
            const T xa = ld_in(p + sa * s, once);
            const T xb = i == 0 ? T(0) : ld_in(p + (sine ? i - 1 : L - i) * s, once);
            xv[q] = mk<T>(xa, xb);
          }
        }
        cx<T> *row = buf + sr * PITCH;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int i = si0 + q * TPR;
          if (L % TPR == 0 || i < L) {
            cx<T> x = xv[q];
            if (sine ? i == L - 1 : i == 0) x.x *= e0;
            if (sine && i == 1) x.y *= e0;
            const cx<T> t = __ldg(tw3 + i);  // e^{-i pi i / 2n}
            row[i + (i >> PS)] = cj<T>(mulc<T>(mk<T>(x.x, -x.y), t));
          }
        }
      }
    }
    __syncthreads();
    fx_middle<T, OP, E, COL, false, 0, NP - 1>(a, row0, rows, buf, tw, scale, pair_ok);
    fx_pass<T, OP, E, NP - 1, COL, false, FX_SMEM, FX_GLOBAL>(a, row0, rows, buf, nullptr, tw, scale, pair_ok);
  } else if constexpr (OP == OP_DCT2_HALF) {
    // y = DCT-II (DST-II) of real n = 2L: v = Makhoul order of x (v_m = x_2m, v_{n-1-m} =
    // x_2m+1, DST: odd inputs negated) as L complex pairs z_j = (v_2j, v_2j+1); X = r2c(v) by
    // the length-L FFT and the split; y_p = 2 Re(e^{-i pi k / 2n} X_k) fct, k = p (DCT) or n-1-p
    // (DST), X_k = conj X_{n-k} for k > n/2; y_0 weighted e0.
    constexpr int N = 2 * L;
    const int64_t s = a.ld.axis_stride;
    const bool sine = (a.flags & 2) != 0;
    {
      constexpr int HP = N / 2, NQ = (HP + TPR - 1) / TPR;
      if (sr < rows) {
        const T *p = reinterpret_cast<const T *>(a.in) + side_offset32(a.ld, row0 + uint32_t(sr));
        cx<T> xv[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int m = si0 + q * TPR;
          if (HP % TPR == 0 || m < HP) {
            if (pair_ok) xv[q] = ld_in(reinterpret_cast<const cx<T> *>(p) + m, once);
            else xv[q] = mk<T>(ld_in(p + 2 * m * s, once), ld_in(p + (2 * m + 1) * s, once));
          }
        }
        T *row = reinterpret_cast<T *>(buf + sr * PITCH);
        auto vput = [&](int i, T val) {  // v_i -> component (i & 1) of z_{i/2}
          const int jz = i >> 1;
          row[2 * (jz + (jz >> PS)) + (i & 1)] = val;
        };
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int m = si0 + q * TPR;
          if (HP % TPR == 0 || m < HP) {
            vput(m, xv[q].x);
            vput(N - 1 - m, sine ? -xv[q].y : xv[q].y);
          }
        }
      }
    }
    __syncthreads();
    fx_middle<T, OP, E, COL, false, 0, NP>(a, row0, rows, buf, tw, scale, pair_ok);
    // split and post-twiddle fused: the thread takes the pairs (k, L - k), k = first + q * TPR
    // <= L / 2, of its row, forms X_k and X_{L-k} from Z_k and Z_{L-k} and stores the four
    // outputs they give: with z = t_k X_k, y_k = 2 Re z and y_{N-k} = -2 Im z (t_{N-k} =
    // -i conj t_k), the same for L - k; k = 0 gives y_0 and y_L from X_0 = Re Z_0 + Im Z_0 and
    // X_L = Re Z_0 - Im Z_0 (both real). Output position p = kk (DCT) or N-1-kk (DST); y at p = 0
    // weighted e0.
    {
      constexpr int HP2 = L / 2 + 1, NQ = (HP2 + TPR - 1) / TPR;
      const int64_t so = a.st.axis_stride;
      const T fct2 = T(2) * T(a.fct), e0 = T(a.e0);
      const cx<T> *t2 = reinterpret_cast<const cx<T> *>(a.aux);   // e^{-i pi k / 2n}, k <= L used
      const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux2);    // W_n^k, k <= L / 2
      if (sr < rows) {
        T *p = reinterpret_cast<T *>(a.out) + side_offset32(a.st, row0 + uint32_t(sr));
        const cx<T> *row = buf + sr * PITCH;
        // kFlagEigDiv: row g = k0 n1 + k1; the same float operations as the separate divide
        const bool eig = (a.flags & kFlagEigDiv) != 0;
        const T *lam2 = nullptr;
        T lam01 = T(0);
        bool origin = false;
        if (eig) {
          const T *lam = reinterpret_cast<const T *>(a.aux3);
          const uint32_t g = row0 + uint32_t(sr), n1 = uint32_t(a.aux_n);
          const uint32_t k0 = g / n1, k1 = g - k0 * n1;
          lam01 = lam[k0] + lam[a.aux_s + k1];
          lam2 = lam + a.aux_s + n1;
          origin = g == 0;
        }
        auto put = [&](int kk, T y) {
          const int pos = sine ? N - 1 - kk : kk;
          y = pos == 0 ? y * e0 : y;
          if (eig) y = (origin && pos == 0) ? T(0) : eig_div<T>(y, lam01 + lam2[pos]);
          p[pos * so] = y;
        };
        auto emit = [&](int k, cx<T> X) {  // 0 < k < L
          const cx<T> z = mul<T>(__ldg(t2 + k), X);
          put(k, z.x * fct2);
          put(N - k, -z.y * fct2);
        };
#pragma unroll 2
        for (int q = 0; q < NQ; ++q) {
          const int k = si0 + q * TPR;
          if (HP2 % TPR == 0 || k < HP2) {
            if (k == 0) {
              const cx<T> z0 = row[0];
              put(0, (z0.x + z0.y) * fct2);
              put(L, (z0.x - z0.y) * __ldg(t2 + L).x * fct2);
            } else {
              const int kc = L - k;
              const cx<T> zk = row[k + (k >> PS)], zc = cj<T>(row[kc + (kc >> PS)]);
              const cx<T> Ev = scl<T>(add<T>(zk, zc), T(0.5));
              const cx<T> O = mnegi<T>(scl<T>(sub<T>(zk, zc), T(0.5)));
              const cx<T> u = mul<T>(__ldg(w + k), O);
              emit(k, add<T>(Ev, u));
              if (kc != k) emit(kc, cj<T>(sub<T>(Ev, u)));
            }
          }
        }
      }
    }
  } else if constexpr (OP == OP_DCT3_HALF) {
    // y = DCT-III (DST-III) of real n = 2L: V_k = (x''_k - i x''_{n-k}) e^{i pi k / 2n} for
    // k = 0..L (x''_q = x_q (DCT) or x_{n-1-q} (DST), x''_n = 0, input element 0 weighted e0)
    // is the half spectrum of the real sequence v; the fused load builds V_i and V_{L-i} and
    // merges them into conj(Z) (as C2R_EVEN, no conjugation), the passes and the last store
    // give v and its DCT order.
    constexpr int N = 2 * L;
    constexpr int HP = L / 2 + 1;
    constexpr int NQ = (HP + TPR - 1) / TPR;
    const bool sine = (a.flags & 2) != 0;
    if (sr < rows) {
      const int64_t s = a.ld.axis_stride;
      const T *p = reinterpret_cast<const T *>(a.in) + side_offset32(a.ld, row0 + uint32_t(sr));
      const cx<T> *t2 = reinterpret_cast<const cx<T> *>(a.aux);   // e^{-i pi k / 2n}
      const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux2);   // e^{-2 pi i k / n}
      const T e0 = T(a.e0);
      auto xdd = [&](int q) -> T {  // x''_q
        if (q >= N) return T(0);
        const int src = sine ? N - 1 - q : q;
        T v = ld_in(p + src * s, once);
        if (src == 0) v *= e0;
        return v;
      };
      auto V = [&](int k) {  // conj(t_k) (x''_k - i x''_{n-k}); imaginary part of bins 0, L zeroed
        const cx<T> t = __ldg(t2 + k);
        cx<T> r = mulc<T>(mk<T>(xdd(k), -xdd(N - k)), t);
        if (k == 0 || k == L) r.y = T(0);
        return r;
      };
      cx<T> *row = buf + sr * PITCH;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const int i = si0 + q * TPR;
        if (HP % TPR == 0 || i < HP) {
          const cx<T> x = V(i), y = V(L - i);
          const cx<T> A = add<T>(x, cj<T>(y)), B = sub<T>(x, cj<T>(y));
          if (i == 0) {
            row[0] = cj<T>(add<T>(A, mposi<T>(B)));
          } else {
            const int kc = L - i;
            const cx<T> U = mposi<T>(mulc<T>(B, __ldg(w + i)));
            row[i + (i >> PS)] = cj<T>(add<T>(A, U));
            if (kc != i) row[kc + (kc >> PS)] = sub<T>(A, U);
          }
        }
      }
    }
    __syncthreads();
    fx_middle<T, OP, E, COL, false, 0, NP - 1>(a, row0, rows, buf, tw, scale, pair_ok);
    fx_pass<T, OP, E, NP - 1, COL, false, FX_SMEM, FX_GLOBAL>(a, row0, rows, buf, nullptr, tw, scale, pair_ok);
  } else {  // OP_C2R_EVEN
    // staged Hermitian load fused with the merge: the thread takes the pairs (i, L - i),
    // i = first + q * TPR <= L / 2, loads both bins (all loads issued before any use), applies
    // the input conversion (conjugation, zero imaginary parts of bins 0 and L, interior-bin
    // scale) and writes conj(Z_i) and conj(Z_{L-i}):
    //     A = X_i + conj X_{L-i},  B = X_i - conj X_{L-i},  U = i B conj(W_2L^i),
    //     conj Z_i = conj(A + U),  conj Z_{L-i} = A - U   (i = 0: conj Z_0 = conj(A + i B)).
    constexpr int HP = L / 2 + 1;
    constexpr int NQ = (HP + TPR - 1) / TPR;
    if (sr < rows) {
      const int64_t s = a.ld.axis_stride;
      const bool cin = a.conj_in != 0;
      const T bsc = T(a.bscale);
      const cx<T> *p = reinterpret_cast<const cx<T> *>(a.in) + side_offset32(a.ld, row0 + uint32_t(sr));
      const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);
      cx<T> xa[NQ], xb[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const int i = si0 + q * TPR;
        if (HP % TPR == 0 || i < HP) {
          xa[q] = ld_in(p + i * s, once);
          xb[q] = ld_in(p + (L - i) * s, once);
        }
      }
      auto fix = [&](int i, cx<T> x) {
        if (cin) x.y = -x.y;
        if (i == 0 || i == L) x.y = T(0);
        else x = scl<T>(x, bsc);
        return x;
      };
      cx<T> *row = buf + sr * PITCH;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const int i = si0 + q * TPR;
        if (HP % TPR == 0 || i < HP) {
          const cx<T> x = fix(i, xa[q]), y = fix(L - i, xb[q]);
          const cx<T> A = add<T>(x, cj<T>(y)), B = sub<T>(x, cj<T>(y));
          if (i == 0) {
            row[0] = cj<T>(add<T>(A, mposi<T>(B)));
          } else {
            const int kc = L - i;
            const cx<T> U = mposi<T>(mulc<T>(B, __ldg(w + i)));
            row[i + (i >> PS)] = cj<T>(add<T>(A, U));
            if (kc != i) row[kc + (kc >> PS)] = sub<T>(A, U);
          }
        }
      }
    }
    __syncthreads();
    fx_middle<T, OP, E, COL, false, 0, NP - 1>(a, row0, rows, buf, tw, scale, pair_ok);
    fx_pass<T, OP, E, NP - 1, COL, false, FX_SMEM, FX_GLOBAL>(a, row0, rows, buf, nullptr, tw, scale, pair_ok);
  }
}

}  // namespace rg
