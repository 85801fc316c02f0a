// Two-axis real transforms of whole planes in one thread-block cluster.
//
// A multi-axis r2c runs the real transform along the last axis and then complex transforms
// along the others (rocket_fft/_pocketfft_hdronly.h:3955-3975); c2r runs them in the reverse
// order (3995-4023). Done one axis at a time, each axis is a full read and write of the volume
// in HBM. Here the last axis (real length n2 = 2H, contiguous) and the axis before it in the
// axis list (length L1, any stride) are done in ONE pass: every plane (the L1 x n2 real
// elements for one index of the remaining dimensions) is held on chip by a cluster of CL
// CTAs, and the transposition between the two axes goes through distributed shared memory.
//
// Forward (r2c, then c2c along the outer axis):
//   row phase     CTA c transforms rows c*RB .. c*RB+RB-1 of the plane: the length-H complex
//                 FFT of the real pairs (first pass reads HBM, middle passes in place), the
//                 last pass fused with the real split (fx_split_unit), whose bins go straight
//                 into the shared memory of the CTA that owns their column (mapa +
//                 st.shared::cluster).
//   column phase  CTA c owns half-spectrum columns c*SB .. c*SB+SB-1 and runs the length-L1
//                 complex FFT down each (all passes on chip, the last one stores to HBM).
// Columns 0 and H (the DC and Nyquist bins of every row) are real, so they travel packed as
// one complex column W = X_0 + i X_H; after its column FFT the two spectra are separated,
//     Y_0[k] = (F[k] + conj F[-k]) / 2,   Y_H[k] = -i (F[k] - conj F[-k]) / 2,
// which makes exactly H columns, SB = H / CL per CTA.
//
// Inverse (c2c backward along the outer axis, then c2r): the column phase loads the CTA's
// columns (column 0 as the Hermitian parts of input columns 0 and H packed into one,
// W = A_h + i B_h with A_h[k] = (A[k] + conj A[-k]) / 2, whose backward FFT is
// Re G_0 + i Re G_H -- exactly the parts of bins 0 and H that the c2r reads), the last column
// pass writes every element into the row owner's shared memory, and the row phase merges the
// half spectrum into the length-H complex sequence (as the C2R_EVEN kernel) and stores real
// pairs to HBM.
//
// Both phases share one shared buffer (the row and column layouts alias): a cluster barrier
// separates the last local reads of one layout from the first remote writes of the other, and
// a second barrier makes the remote writes visible. Every thread of every CTA executes both
// barriers (no early exit), and no CTA touches another's shared memory after the second.
#pragma once
#include "rg_fixed_kernel.cuh"
#include "rg_pdl.cuh"

namespace rg {
namespace pl {

__device__ __forceinline__ uint32_t cta_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t remote(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::
          : "memory");
}
__device__ __forceinline__ void st_remote(uint32_t a, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void st_remote(uint32_t a, double2 v) {
  asm volatile("st.shared::cluster.v2.f64 [%0], {%1, %2};" ::"r"(a), "d"(v.x), "d"(v.y) : "memory");
}
__device__ __forceinline__ void st_remote1(uint32_t a, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}
__device__ __forceinline__ void st_remote1(uint32_t a, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}

}  // namespace pl

// Geometry of one phase, in the form the fixed-kernel passes take (fx_pass's C).
template <typename T, int E, bool COL, int TB_, int NT_> struct PlaneSub {
  static constexpr int L = 1 << E;
  static constexpr int ESZ = int(2 * sizeof(T));
  static constexpr int PS = sizeof(T) == 4 ? 4 : 3;
  static constexpr int PITCH = COL ? fx::pitch_of(L, PS, ESZ) : fx::pitch_row(L, PS, ESZ, L);
  static constexpr int TB = TB_;
  static constexpr int NT = NT_;
};

template <typename T, int E1_, int E2, int CL_> struct PlaneCfg {
  static constexpr int E1 = E1_, CL = CL_;
  static constexpr int L1 = 1 << E1;                // outer-axis length
  static constexpr int EH = E2 - 1, H = 1 << EH;    // complex half length of the real rows
  static constexpr int RB = L1 / CL;                // plane rows per CTA (row phase)
  static constexpr int SB = H / CL;                 // half-spectrum columns per CTA
  static constexpr int NT = 256;
  static constexpr int MINB = 3;                    // CTAs per SM the register budget allows
  static constexpr int ESZ = int(2 * sizeof(T));
  using Row = PlaneSub<T, EH, false, RB, NT>;
  using Col = PlaneSub<T, E1, true, SB, NT>;
  static constexpr int NPR = fx::np_of(EH), NPC = fx::np_of(E1);
  static constexpr size_t SMEM =
      size_t(RB * Row::PITCH > SB * Col::PITCH ? RB * Row::PITCH : SB * Col::PITCH) * ESZ;
  static_assert(RB >= 1 && SB >= 1 && (SB & (SB - 1)) == 0 && (RB & (RB - 1)) == 0, "plane split");
  static_assert(NPR >= 2 && fx::radix_of(EH, NPR - 1) <= 8 && fx::radix_of(EH, NPR - 1) >= 2,
                "row length: the real split is fused into a last pass of radix 2..8");
};

// Forward: the last row pass with the real split, bins to the column owners.
template <typename T, typename P>
__device__ __forceinline__ void plane_split_to_slots(const KArgs &ar, uint32_t rank, const cx<T> *buf,
                                                     const cx<T> *__restrict__ tw) {
  using Row = typename P::Row;
  using Col = typename P::Col;
  constexpr int EH = P::EH, L = P::H, PP = P::NPR - 1;
  constexpr int R = fx::radix_of(EH, PP), LR = L / R, NS = fx::ns_of(EH, PP), TWO = fx::tw_of(EH, PP);
  static_assert(NS == LR, "last pass");
  constexpr int NT = P::NT, UPR = LR / 2, NU = P::RB * UPR, ITER = (NU + NT - 1) / NT;
  constexpr int ESZ = P::ESZ;
  const cx<T> *w = reinterpret_cast<const cx<T> *>(ar.aux);
  cx<T> v1[ITER][R], v2[ITER][R];
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int unit = int(threadIdx.x) + it * NT;
    if (NU % NT == 0 || unit < NU) {
      const int r = unit / UPR, u = unit % UPR;
      const int j1 = u, j2 = u == 0 ? NS / 2 : NS - u;
      const cx<T> *sp = buf + r * Row::PITCH;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        v1[it][k] = sp[fx_pos<Row::PS, LR>(j1, k)];
        v2[it][k] = sp[fx_pos<Row::PS, LR>(j2, k)];
      }
      const cx<T> *t1 = tw + TWO + j1, *t2 = tw + TWO + j2;
#pragma unroll
      for (int k = 1; k < R; ++k) {
        v1[it][k] = mul<T>(v1[it][k], __ldg(t1 + (k - 1) * NS));
        v2[it][k] = mul<T>(v2[it][k], __ldg(t2 + (k - 1) * NS));
      }
      dft<T, R>(v1[it]);
      dft<T, R>(v2[it]);
    }
  }
  pl::cluster_sync();  // every CTA has read its row layout: the column layout may be written
  const uint32_t sbase = uint32_t(__cvta_generic_to_shared(buf));
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int unit = int(threadIdx.x) + it * NT;
    if (NU % NT == 0 || unit < NU) {
      const int r = unit / UPR, u = unit % UPR;
      const int jg = int(rank) * P::RB + r;  // row of the plane = element of the column FFT
      const int pos = jg + (jg >> Col::PS);
      fx_split_unit<T, L, R, NS>(u, v1[it], v2[it], w, [&](int i, cx<T> x) {
        if (i == 0 || i == L) {  // packed column: X_0 in .x, X_H in .y of column slot 0, CTA 0
          const uint32_t off = uint32_t(pos * ESZ + (i == L ? int(sizeof(T)) : 0));
          pl::st_remote1(pl::remote(sbase + off, 0), x.x);
        } else {
          const int o = i / P::SB, kl = i % P::SB;
          pl::st_remote(pl::remote(sbase + uint32_t((kl * Col::PITCH + pos) * ESZ), uint32_t(o)), x);
        }
      });
    }
  }
}

template <typename T, int E1, int E2, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(PlaneCfg<T, E1, E2, CL>::NT, PlaneCfg<T, E1, E2, CL>::MINB)
    plane_r2c_kernel(const __grid_constant__ KArgs ar, const __grid_constant__ KArgs ac) {
  pdl_begin();
  using P = PlaneCfg<T, E1, E2, CL>;
  using Row = typename P::Row;
  using Col = typename P::Col;
  extern __shared__ __align__(16) unsigned char smraw[];
  cx<T> *buf = reinterpret_cast<cx<T> *>(smraw);
  const uint32_t rank = pl::cta_rank();
  const uint32_t plane = blockIdx.x / CL;
  const cx<T> *twr = reinterpret_cast<const cx<T> *>(ar.core.tw);
  const cx<T> *twc = reinterpret_cast<const cx<T> *>(ac.core.tw);
  // row phase: real pairs of rows plane*L1 + rank*RB .. (+RB) -> length-H FFT -> split
  const uint32_t row0 = plane * P::L1 + rank * P::RB;
  fx_pass<T, OP_R2C_EVEN, P::EH, 0, false, false, FX_GLOBAL, FX_SMEM, false, Row>(ar, row0, P::RB, nullptr, buf,
                                                                                  twr, false, true);
  __syncthreads();
  fx_middle<T, OP_R2C_EVEN, P::EH, false, false, 1, P::NPR - 1, Row>(ar, row0, P::RB, buf, twr, false, true);
  plane_split_to_slots<T, P>(ar, rank, buf, twr);
  pl::cluster_sync();  // all columns are in place
  // column phase: columns plane*H + rank*SB .. (+SB), length L1, the last pass to HBM
  const uint32_t col0 = plane * P::H + rank * P::SB;
  const bool scale = ac.fct != 1.0;
  fx_middle<T, OP_C2C, E1, true, false, 0, P::NPC - 1, Col>(ac, col0, P::SB, buf, twc, false, true);
  fx_pass<T, OP_C2C, E1, P::NPC - 1, true, false, FX_SMEM, FX_GLOBAL, false, Col>(ac, col0, P::SB, buf, nullptr,
                                                                                   twc, scale, true);
  if (rank == 0) {
    // separate the packed column: F = FFT(X_0 + i X_H) -> output columns 0 and H
    __syncthreads();  // the column-0 stores of this CTA are visible to its threads
    constexpr int NPAIR = P::L1 / 2 + 1, NQ = (NPAIR + P::NT - 1) / P::NT;
    const int64_t s = ac.st.axis_stride;
    cx<T> *c0 = reinterpret_cast<cx<T> *>(ac.out) + side_offset32(ac.st, col0);
    cx<T> *cH = c0 + int64_t(P::H) * ac.st.bstride[0];
    cx<T> f1[NQ], f2[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int k1 = int(threadIdx.x) + q * P::NT;
      if (k1 < NPAIR) {
        const int k2 = (P::L1 - k1) & (P::L1 - 1);
        f1[q] = __ldcg(c0 + k1 * s);
        f2[q] = __ldcg(c0 + k2 * s);
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int k1 = int(threadIdx.x) + q * P::NT;
      if (k1 < NPAIR) {
        const int k2 = (P::L1 - k1) & (P::L1 - 1);
        const cx<T> g = cj<T>(f2[q]);
        const cx<T> y0 = scl<T>(add<T>(f1[q], g), T(0.5));
        const cx<T> yh = mnegi<T>(scl<T>(sub<T>(f1[q], g), T(0.5)));
        c0[k1 * s] = y0;
        cH[k1 * s] = yh;
        if (k2 != k1) {
          c0[k2 * s] = cj<T>(y0);
          cH[k2 * s] = cj<T>(yh);
        }
      }
    }
  }
}

// Inverse: the last column pass, every element to the shared memory of its row's owner.
template <typename T, typename P>
__device__ __forceinline__ void plane_cols_to_rows(const KArgs &ac, uint32_t rank, const cx<T> *buf,
                                                   const cx<T> *__restrict__ tw) {
  using Row = typename P::Row;
  using Col = typename P::Col;
  constexpr int E1 = P::E1, L = P::L1, PP = P::NPC - 1;
  constexpr int R = fx::radix_of(E1, PP), LR = L / R, NS = fx::ns_of(E1, PP);
  constexpr int TB = P::SB, NT = P::NT, NBF = TB * LR, ITER = (NBF + NT - 1) / NT;
  constexpr int ESZ = P::ESZ;
  cx<T> v[ITER][R];
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int bf = int(threadIdx.x) + it * NT;
    if (NBF % NT == 0 || bf < NBF) {
      int r, j;
      fx_rj<TB, LR, true>(bf, r, j);
      fx_compute<T, OP_C2C, E1, PP, true, false, FX_SMEM, Col>(ac, 0, r, j, buf, tw, true, v[it]);
    }
  }
  pl::cluster_sync();  // every CTA has read its column layout: the row layout may be written
  const uint32_t sbase = uint32_t(__cvta_generic_to_shared(buf));
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int bf = int(threadIdx.x) + it * NT;
    if (NBF % NT == 0 || bf < NBF) {
      int r, j;
      fx_rj<TB, LR, true>(bf, r, j);
      const int m = j & (NS - 1);
      const int base = (j - m) * R + m;
      const int k = int(rank) * P::SB + r;  // half-spectrum column = element of the row
      const int kpos = k + (k >> Row::PS);
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const int jj = base + q * NS;  // plane row
        const int o = jj / P::RB, jl = jj % P::RB;
        const cx<T> x = mk<T>(v[it][q].y, v[it][q].x);  // undo the load-side swap: backward FFT
        pl::st_remote(pl::remote(sbase + uint32_t((jl * Row::PITCH + kpos) * ESZ), uint32_t(o)), x);
      }
    }
  }
}

template <typename T, int E1, int E2, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(PlaneCfg<T, E1, E2, CL>::NT, PlaneCfg<T, E1, E2, CL>::MINB)
    plane_c2r_kernel(const __grid_constant__ KArgs ar, const __grid_constant__ KArgs ac) {
  pdl_begin();
  using P = PlaneCfg<T, E1, E2, CL>;
  using Row = typename P::Row;
  using Col = typename P::Col;
  extern __shared__ __align__(16) unsigned char smraw[];
  cx<T> *buf = reinterpret_cast<cx<T> *>(smraw);
  const uint32_t rank = pl::cta_rank();
  const uint32_t plane = blockIdx.x / CL;
  const cx<T> *twr = reinterpret_cast<const cx<T> *>(ar.core.tw);
  const cx<T> *twc = reinterpret_cast<const cx<T> *>(ac.core.tw);
  const int tid = threadIdx.x;
  // column phase: staged load of columns plane*H + rank*SB .. (+SB), (im, re)-swapped so that
  // the forward passes give the backward transform
  const uint32_t col0 = plane * P::H + rank * P::SB;
  {
    constexpr int JS = P::NT / P::SB, NQ = P::L1 / JS;
    static_assert(P::NT % P::SB == 0 && P::L1 % JS == 0, "column staging");
    const int kl = tid & (P::SB - 1), j0 = tid / P::SB;
    const int64_t s = ac.ld.axis_stride;
    const cx<T> *col = reinterpret_cast<const cx<T> *>(ac.in) + side_offset32(ac.ld, col0 + uint32_t(kl));
    cx<T> *dst = buf + kl * Col::PITCH;
    cx<T> xv[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) xv[q] = __ldg(col + (j0 + q * JS) * s);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int jj = j0 + q * JS;
      dst[jj + (jj >> Col::PS)] = mk<T>(xv[q].y, xv[q].x);
    }
  }
  if (rank == 0) {
    // packed column 0: W[k] = A_h[k] + i B_h[k] from A (input column 0, staged above) and
    // B (input column H); thread k1 owns the pair (k1, -k1), A_h[-k1] = conj A_h[k1]
    __syncthreads();
    constexpr int NPAIR = P::L1 / 2 + 1, NQ = (NPAIR + P::NT - 1) / P::NT;
    const int64_t s = ac.ld.axis_stride;
    const cx<T> *colH = reinterpret_cast<const cx<T> *>(ac.in) + side_offset32(ac.ld, col0) +
                        int64_t(P::H) * ac.ld.bstride[0];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int k1 = tid + q * P::NT;
      if (k1 < NPAIR) {
        const int k2 = (P::L1 - k1) & (P::L1 - 1);
        const int p1 = k1 + (k1 >> Col::PS), p2 = k2 + (k2 >> Col::PS);
        const cx<T> b1 = __ldg(colH + k1 * s), b2 = __ldg(colH + k2 * s);
        const cx<T> a1s = buf[p1], a2s = buf[p2];
        const cx<T> a1 = mk<T>(a1s.y, a1s.x), a2 = mk<T>(a2s.y, a2s.x);
        const cx<T> ah = scl<T>(add<T>(a1, cj<T>(a2)), T(0.5)), bh = scl<T>(add<T>(b1, cj<T>(b2)), T(0.5));
        const cx<T> w1 = add<T>(ah, mposi<T>(bh));              // W[k1]
        const cx<T> w2 = add<T>(cj<T>(ah), mposi<T>(cj<T>(bh)));  // W[-k1]
        buf[p1] = mk<T>(w1.y, w1.x);
        if (k2 != k1) buf[p2] = mk<T>(w2.y, w2.x);
      }
    }
  }
  __syncthreads();
  fx_middle<T, OP_C2C, E1, true, false, 0, P::NPC - 1, Col>(ac, col0, P::SB, buf, twc, false, true);
  plane_cols_to_rows<T, P>(ac, rank, buf, twc);
  pl::cluster_sync();  // all rows are in place
  // row phase: merge X_0..X_H of each row into conj(Z) (as the C2R_EVEN load), H-point FFT,
  // real pairs to HBM. Entry 0 holds (Re G_0, Re G_H), the real parts of bins 0 and H.
  {
    constexpr int L = P::H, HP = L / 2 + 1, PS = Row::PS;
    const cx<T> *w = reinterpret_cast<const cx<T> *>(ar.aux);
    for (int e = tid; e < P::RB * HP; e += P::NT) {
      const int r = e / HP, i = e - r * HP;
      cx<T> *row = buf + r * Row::PITCH;
      if (i == 0) {
        const cx<T> e0 = row[0];
        const cx<T> A = mk<T>(e0.x + e0.y, T(0)), B = mk<T>(e0.x - e0.y, T(0));
        row[0] = cj<T>(add<T>(A, mposi<T>(B)));
      } else {
        const int kc = L - i;
        const cx<T> x = row[i + (i >> PS)], y = row[kc + (kc >> PS)];
        const cx<T> A = add<T>(x, cj<T>(y)), B = sub<T>(x, cj<T>(y));
        const cx<T> U = mposi<T>(mulc<T>(B, __ldg(w + i)));
        row[i + (i >> PS)] = cj<T>(add<T>(A, U));
        if (kc != i) row[kc + (kc >> PS)] = sub<T>(A, U);
      }
    }
  }
  __syncthreads();
  const uint32_t row0 = plane * P::L1 + rank * P::RB;
  const bool scale = ar.fct != 1.0;
  fx_middle<T, OP_C2R_EVEN, P::EH, false, false, 0, P::NPR - 1, Row>(ar, row0, P::RB, buf, twr, scale, true);
  fx_pass<T, OP_C2R_EVEN, P::EH, P::NPR - 1, false, false, FX_SMEM, FX_GLOBAL, false, Row>(ar, row0, P::RB, buf,
                                                                                          nullptr, twr, scale, true);
}

}  // namespace rg
