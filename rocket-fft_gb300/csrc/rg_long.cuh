// Long power-of-two complex64 transforms (2^14 .. 2^24 points) and float32 real transforms
// whose half length is in that range, in one persistent launch.
//
// The on-chip kernels hold a whole transform in one CTA (up to 8192 points). Past that the
// reference runs its radix passes over the whole row in memory (cfftp::pass_all,
// rocket_fft/_pocketfft_hdronly.h:1690-1740); here the row is factored as n = n1 * n2 (the
// four-step form of the same DFT) and split into two phases of on-chip FFTs:
//
//   phase A  x viewed as n1 rows x n2 columns (x[j1 n2 + j2]): for each column j2, an FFT of
//            length n1 over j1, times W_n^{j2 k1}, into Y[k1 n2 + j2]
//   phase B  for each row k1 of Y, an FFT of length n2 over j2, into X[k1 + n1 k2]
//
// A phase-A tile is C = TT / n1 adjacent columns of one transform (its HBM reads are C-element
// segments, two columns per 16-byte load); a phase-B tile is D = TT / n2 adjacent rows of Y
// (its HBM writes are D-element segments, two rows per 16-byte store). Both phases read their
// first radix pass straight from global memory into registers and write their last pass straight
// back; the passes in between run in place in one shared buffer.
//
// Y is the only intermediate, and it is kept in L2: transforms go through in groups of G
// (G * n * 8 bytes of Y per group), and each group has its own region of a ring of nbuf Y
// buffers. Every tile is a ticket taken from an atomic counter, in the order
//     look = 1:  A0 A1 B0 A2 B1 ... A(g) B(g-1) ... B(last)      (nbuf >= 2)
//     look = 0:  A0 B0 A1 B1 ...                                  (nbuf == 1)
// A B(g) tile first waits until every A(g) tile is done; an A(g) tile waits until every
// B(g - nbuf) tile has released its Y buffer. A CTA only ever waits on tickets below its own,
// which running CTAs hold, so the launch always makes progress. Every wait is bounded (2 s of
// %globaltimer): past it the CTA sets the error word and every CTA leaves its loop.
// Y is written and read through L2 only (st/ld .cg), and a phase-B tile discards the Y lines it
// has consumed (discard.global.L2), so dead intermediate data is never written back to HBM.
//
// Real transforms of n = 2m points run the complex transform of length m on the real pairs
// z_j = x_2j + i x_2j+1 (the reference's rfftp for even n reaches the same spectrum by its own
// real radix passes, HDR:1836-2717). The split X_k = (Z_k + conj Z_{m-k}) / 2
// - i W_n^k (Z_k - conj Z_{m-k}) / 2 needs Z_k and Z_{m-k} together: with k = k1 + n1 k2,
// m - k = (n1 - k1) + n1 (n2 - 1 - k2), so an r2c phase-B tile holds D/2 rows k1 and their
// mirror rows n1 - k1 (tile 0: rows 0 and n1/2, which mirror onto themselves, and rows
// 1 .. D/2-1 with their mirrors), runs every pass on chip and stores X_k and X_{m-k} from each
// pair. c2r is the mirror image: its phase-A tile holds columns j2 and n2 - j2, merges the
// Hermitian half spectrum into conj(Z) as it loads, and phase B stores conj of the result as
// the real pairs.
#pragma once
#include "rg_fixed_kernel.cuh"

namespace rg {

struct LongArgs {
  const void *in;
  void *out;
  Side ld, st;        // batch decomposition of transform b (both sides: axis stride 1)
  int64_t batch;      // transforms
  void *ybuf;         // nbuf * G * n complex elements
  int *ctr;           // [0] ticket, [1] error, [2] unused, [3, 3+ng) A done, [3+ng, 3+2ng) B done
  int *errw;          // per-device error word: set when a wait gave up
  int G, ngroups, nbuf, look;
  int tiles;          // tiles per phase and group (G * n / TT)
  int conj_in, conj_out;
  float fct;
  const void *twA, *twB;  // core twiddle tables of the lengths n1 and n2
  const void *lo, *hi;    // split table of W_n (n: the complex length)
  int shift;
  const void *lo2, *hi2;  // real transforms: split table of W_{2n}
  int shift2;
  int flags;              // bit 0: discard consumed Y lines; bit 1: evict-first output stores
};

enum : int { LG_C2C = 0, LG_R2C = 1, LG_C2R = 2 };

constexpr int kLongDiscard = 1;
constexpr int kLongEvictOut = 2;

namespace lg {

// shared index of position pos of a line: one pad slot per 32 positions
__host__ __device__ constexpr int sp(int pos) { return pos + (pos >> 5); }

// Line pitch in shared slots for lines of length L accessed in the first / last pass by lanes
// that run across `pairs` pairs of adjacent lines first (two lines per lane): lane (pair q, j)
// lands on slot 2 q pitch + (a function of j taking 16 / pairs consecutive values), so the
// pitch must be 8 / pairs modulo 8 for the 32 lanes to fill each of the 16 eight-byte slots of
// a wavefront exactly twice.
__host__ __device__ constexpr int pitch(int L, int pairs) {
  int p = sp(L - 1) + 1;
  const int want = pairs >= 2 && pairs <= 8 ? 8 / pairs : -1;
  if (want >= 0)
    while (p % 8 != want) ++p;
  return p;
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Wait until *p >= need. Returns 1 (and sets *err) after 2 s, or at once when another CTA has
// set *err.
__device__ __forceinline__ int wait_count(const int *p, int need, int *err) {
  if (ld_acquire(p) >= need) return 0;
  const uint64_t t0 = globaltimer();
  for (;;) {
    __nanosleep(128);
    if (ld_acquire(p) >= need) return 0;
    if (ld_relaxed(err) != 0) return 1;
    if (globaltimer() - t0 > 2000000000ull) {
      atomicExch(err, 1);
      return 1;
    }
  }
}

__device__ __forceinline__ float4 ld_x(const float4 *p, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_x(float4 *p, float4 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void discard_l2(const void *p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

}  // namespace lg

// Compile-time geometry: n1 = 2^E1 (phase-A length), n2 = 2^E2, tile of TT = 2^ET elements.
template <int E1, int E2, int ET> struct LgCfg {
  static constexpr int N1 = 1 << E1, N2 = 1 << E2, TT = 1 << ET;
  static constexpr int C = TT / N1, D = TT / N2;  // columns per A tile, rows per B tile
  static constexpr int NT = TT / 32;              // threads: one pair of radix-16 butterflies each
  static constexpr int PA = lg::pitch(N1, C / 2), PB = lg::pitch(N2, D / 2);
  static constexpr int SLOTS = C * PA > D * PB ? C * PA : D * PB;
  // the tile, then two control words (ticket, wait failure): no static shared memory, so the
  // dynamic size may be raised to the device's opt-in maximum
  static constexpr size_t SMEM = size_t(SLOTS) * 8 + 16;
  static_assert(C >= 2 && D >= 2 && C <= 32 && D <= 32, "tile shape");
  static_assert(fx::radix_of(E1, 0) == 16 && fx::radix_of(E2, 0) == 16, "first pass radix 16");
};

// ---- passes over lines of length 2^E held in shared memory (line l at sm + l * PITCH) ----

// Middle pass P, in place: all butterflies read (and transform) before a barrier, then write.
template <int E, int P, int M, int NT, int PITCH>
__device__ __forceinline__ void lg_middle(float2 *sm, const float2 *__restrict__ tw) {
  constexpr int L = 1 << E, R = fx::radix_of(E, P), LR = L / R, NS = fx::ns_of(E, P), TWO = fx::tw_of(E, P);
  constexpr int UNITS = M * LR, ITER = (UNITS + NT - 1) / NT;
  static_assert(UNITS % NT == 0, "whole iterations");
  float2 v[ITER][R];
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int u = int(threadIdx.x) + it * NT;
    const int line = u / LR, j = u % LR;
    const float2 *s = sm + line * PITCH;
#pragma unroll
    for (int k = 0; k < R; ++k) v[it][k] = s[lg::sp(j + k * LR)];
    if constexpr (NS > 1) {
      const float2 *t = tw + TWO + (j & (NS - 1));
#pragma unroll
      for (int k = 1; k < R; ++k) v[it][k] = mul<float>(v[it][k], __ldg(t + (k - 1) * NS));
    }
    dft<float, R>(v[it]);
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int u = int(threadIdx.x) + it * NT;
    const int line = u / LR, j = u % LR;
    const int m = j & (NS - 1), base = (j - m) * R + m;
    float2 *s = sm + line * PITCH;
#pragma unroll
    for (int k = 0; k < R; ++k) s[lg::sp(base + k * NS)] = v[it][k];
  }
  __syncthreads();
}

template <int E, int M, int NT, int PITCH, int P, int PEND>
__device__ __forceinline__ void lg_middles(float2 *sm, const float2 *__restrict__ tw) {
  if constexpr (P < PEND) {
    lg_middle<E, P, M, NT, PITCH>(sm, tw);
    lg_middles<E, M, NT, PITCH, P + 1, PEND>(sm, tw);
  }
}

// Last-pass butterfly j of the line pair (l0, l0 + 1): inputs from shared memory, twiddled,
// transformed; output k lands at position j + k * NS of the transform.
template <int E, int PITCH>
__device__ __forceinline__ void lg_last_pair(const float2 *sm, const float2 *__restrict__ tw, int l0, int j,
                                             float2 (&a)[fx::radix_of(E, fx::np_of(E) - 1)],
                                             float2 (&b)[fx::radix_of(E, fx::np_of(E) - 1)]) {
  constexpr int L = 1 << E, P = fx::np_of(E) - 1, R = fx::radix_of(E, P), LR = L / R, NS = fx::ns_of(E, P);
  constexpr int TWO = fx::tw_of(E, P);
  static_assert(NS == LR, "last pass");
  const float2 *s0 = sm + l0 * PITCH, *s1 = s0 + PITCH;
#pragma unroll
  for (int k = 0; k < R; ++k) {
    a[k] = s0[lg::sp(j + k * LR)];
    b[k] = s1[lg::sp(j + k * LR)];
  }
  if constexpr (NS > 1) {
    const float2 *t = tw + TWO + j;
#pragma unroll
    for (int k = 1; k < R; ++k) {
      const float2 w = __ldg(t + (k - 1) * NS);
      a[k] = mul<float>(a[k], w);
      b[k] = mul<float>(b[k], w);
    }
  }
  dft<float, R>(a);
  dft<float, R>(b);
}

// ---- paired lines of the real transforms ----

// Line l of pair tile t over a dimension of length NL with H = LINES / 2 primary lines: lines
// [0, H) are the rows (or columns) t H + l, line LINES-1-i their mirror NL - (t H + i); tile 0
// holds 0 .. H-1, its mirrors NL-1 .. NL-H+1 on lines LINES-2 .. H, and NL/2 on line LINES-1.
template <int NL, int LINES>
__device__ __forceinline__ int pair_index(int t, int l) {
  constexpr int H = LINES / 2;
  if (l < H) return t * H + l;
  if (t == 0 && l == LINES - 1) return NL / 2;
  return NL - t * H - (LINES - 1 - l);
}

// Unit (i, q) of a pair tile (i < H primary lines, q < len positions): where its first element
// sits (line la, position pa, transform index ka = pair_index * stride + pa * ...), and its
// partner (line lb, position pb). Tile 0, line 0 splits its positions between the self-mirrored
// lines 0 (positions q < len/2, partner len - q) and LINES-1 (positions q - len/2, partner
// len-1-(q - len/2)); the unit at line 0, position len/2 (its own partner) is left to
// pair_self_unit.
template <int LINES, int LEN>
__device__ __forceinline__ void pair_unit(int t, int i, int q, int &la, int &pa, int &lb, int &pb) {
  if (t == 0 && i == 0) {
    if (q < LEN / 2) {
      la = 0;
      pa = q;
      lb = 0;
      pb = (LEN - q) & (LEN - 1);
    } else {
      la = LINES - 1;
      pa = q - LEN / 2;
      lb = LINES - 1;
      pb = LEN - 1 - pa;
    }
  } else {
    la = i;
    pa = q;
    lb = LINES - 1 - i;
    pb = LEN - 1 - q;
  }
}

// ---- phase A: C columns of one transform ----

template <int KIND, int E1, int E2, int ET>
__device__ __forceinline__ void lg_phase_a(const LongArgs &a, float2 *sm, const float2 *__restrict__ x,
                                           float2 *__restrict__ y, int part) {
  using Cf = LgCfg<E1, E2, ET>;
  constexpr int N1 = Cf::N1, N2 = Cf::N2, C = Cf::C, NT = Cf::NT, PA = Cf::PA;
  constexpr int CP = C / 2;
  const float2 *tw = reinterpret_cast<const float2 *>(a.twA);
  if constexpr (KIND != LG_C2R) {
    // first pass: radix 16 straight from global memory, two columns per 16-byte load
    constexpr int R = 16, LR = N1 / R, UNITS = CP * LR;
    static_assert(UNITS == NT, "one unit per thread");
    const int u = int(threadIdx.x);
    const int cp = u % CP, j = u / CP;
    const uint64_t pol = input_policy(true);
    const float4 *p = reinterpret_cast<const float4 *>(x + part * C + int64_t(j) * N2 + 2 * cp);
    constexpr int64_t STEP = int64_t(LR) * N2 / 2;
    float2 va[R], vb[R];
    float4 q[R];
#pragma unroll
    for (int k = 0; k < R; ++k) q[k] = lg::ld_x(p + k * STEP, pol);
    const float sgn = a.conj_in ? -1.f : 1.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
      va[k] = make_float2(q[k].x, q[k].y * sgn);
      vb[k] = make_float2(q[k].z, q[k].w * sgn);
    }
    dft<float, R>(va);
    dft<float, R>(vb);
    float2 *l0 = sm + (2 * cp) * PA, *l1 = l0 + PA;
#pragma unroll
    for (int k = 0; k < R; ++k) {
      l0[lg::sp(j * R + k)] = va[k];
      l1[lg::sp(j * R + k)] = vb[k];
    }
    __syncthreads();
    lg_middles<E1, C, NT, PA, 1, fx::np_of(E1) - 1>(sm, tw);
  } else {
    // c2r: merge the half spectrum X (m + 1 elements, m = n1 n2) of columns j2 and n2 - j2
    // into conj(Z) on chip, then every pass but the last in shared memory
    constexpr int64_t M = int64_t(N1) * N2;
    constexpr int H = C / 2;
    const float2 *lo2 = reinterpret_cast<const float2 *>(a.lo2), *hi2 = reinterpret_cast<const float2 *>(a.hi2);
    const float sgn = a.conj_in ? -1.f : 1.f;
    const uint64_t pol = input_policy(true);
    auto ldX = [&](int64_t j) {
      float2 v;
      asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(x + j), "l"(pol));
      v.y *= sgn;
      if (j == 0 || j == M) v.y = 0.f;
      return v;
    };
    // conj(Z_ja) = conj(A + u), conj(Z_{m-ja}) = A - u,  A = X_ja + conj X_{m-ja},
    // u = i (X_ja - conj X_{m-ja}) conj(W_2m^ja)
    auto merge = [&](int la, int pa, int lb, int pb, int64_t ja, bool two) {
      const float2 xa = ldX(ja), xb = ldX(M - ja);
      const float2 A = add<float>(xa, cj<float>(xb)), B = sub<float>(xa, cj<float>(xb));
      const float2 w = split_twiddle<float>(lo2, hi2, a.shift2, uint32_t(ja));
      const float2 uu = mposi<float>(mulc<float>(B, w));
      sm[la * PA + lg::sp(pa)] = cj<float>(add<float>(A, uu));
      if (two) sm[lb * PA + lg::sp(pb)] = sub<float>(A, uu);
    };
    const int t = part;
    for (int u = int(threadIdx.x); u < H * N1; u += NT) {
      const int i = u % H, j1 = u / H;
      int la, pa, lb, pb;
      pair_unit<C, N1>(t, i, j1, la, pa, lb, pb);
      const int64_t ja = int64_t(pa) * N2 + pair_index<N2, C>(t, la);
      merge(la, pa, lb, pb, ja, ja != 0);
    }
    if (t == 0 && threadIdx.x == 0) merge(0, N1 / 2, 0, N1 / 2, M / 2, false);
    __syncthreads();
    lg_middles<E1, C, NT, PA, 0, fx::np_of(E1) - 1>(sm, tw);
  }
  // last pass: outputs k1 = j + k * NS, times W_n^{j2 k1}, to Y[k1][j2]
  {
    constexpr int P = fx::np_of(E1) - 1, R = fx::radix_of(E1, P), LR = N1 / R, NS = LR;
    constexpr int UNITS = CP * LR, ITER = UNITS / NT;
    static_assert(UNITS % NT == 0, "whole iterations");
    const float2 *lo = reinterpret_cast<const float2 *>(a.lo), *hi = reinterpret_cast<const float2 *>(a.hi);
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
      const int u = int(threadIdx.x) + it * NT;
      const int cp = u % CP, j = u / CP;
      float2 va[R], vb[R];
      lg_last_pair<E1, PA>(sm, tw, 2 * cp, j, va, vb);
      if constexpr (KIND != LG_C2R) {
        // two adjacent columns per 16-byte store
        const uint32_t c0 = uint32_t(part * C + 2 * cp);
        float2 *yc = y + part * C + 2 * cp;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          const uint32_t k1 = uint32_t(j + k * NS);
          const float2 wa = split_twiddle<float>(lo, hi, a.shift, c0 * k1);
          const float2 wb = split_twiddle<float>(lo, hi, a.shift, c0 * k1 + k1);
          const float2 ra = mul<float>(va[k], wa), rb = mul<float>(vb[k], wb);
          __stcg(reinterpret_cast<float4 *>(yc + int64_t(k1) * N2), make_float4(ra.x, ra.y, rb.x, rb.y));
        }
      } else {
        // paired columns need not be adjacent: one 8-byte store per column
        const uint32_t ca = uint32_t(pair_index<N2, C>(part, 2 * cp)), cb = uint32_t(pair_index<N2, C>(part, 2 * cp + 1));
#pragma unroll
        for (int k = 0; k < R; ++k) {
          const uint32_t k1 = uint32_t(j + k * NS);
          __stcg(y + int64_t(k1) * N2 + ca, mul<float>(va[k], split_twiddle<float>(lo, hi, a.shift, ca * k1)));
          __stcg(y + int64_t(k1) * N2 + cb, mul<float>(vb[k], split_twiddle<float>(lo, hi, a.shift, cb * k1)));
        }
      }
    }
  }
}

// ---- phase B: D rows of Y ----

template <int KIND, int E1, int E2, int ET>
__device__ __forceinline__ void lg_phase_b(const LongArgs &a, float2 *sm, const float2 *__restrict__ yg,
                                           float2 *__restrict__ X, int part) {
  using Cf = LgCfg<E1, E2, ET>;
  constexpr int N1 = Cf::N1, N2 = Cf::N2, D = Cf::D, NT = Cf::NT, PB = Cf::PB;
  const float2 *tw = reinterpret_cast<const float2 *>(a.twB);
  // row of Y held by line r
  auto yrow = [&](int r) -> const float2 * {
    const int k1 = KIND == LG_R2C ? pair_index<N1, D>(part, r) : part * D + r;
    return yg + int64_t(k1) * N2;
  };
  // first pass: radix 16 from Y (L2), two adjacent butterflies per 16-byte load
  {
    constexpr int R = 16, LR = N2 / R, JP = LR / 2, UNITS = D * JP;
    static_assert(UNITS == NT, "one unit per thread");
    const int u = int(threadIdx.x);
    const int r = u / JP, jp = u % JP;
    const float4 *p = reinterpret_cast<const float4 *>(yrow(r) + 2 * jp);
    float4 q[R];
#pragma unroll
    for (int k = 0; k < R; ++k) q[k] = __ldcg(p + k * (LR / 2));
    float2 va[R], vb[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      va[k] = make_float2(q[k].x, q[k].y);
      vb[k] = make_float2(q[k].z, q[k].w);
    }
    dft<float, R>(va);
    dft<float, R>(vb);
    float2 *l = sm + r * PB;
    const int j0 = 2 * jp;
#pragma unroll
    for (int k = 0; k < R; ++k) {
      l[lg::sp(j0 * R + k)] = va[k];
      l[lg::sp((j0 + 1) * R + k)] = vb[k];
    }
  }
  __syncthreads();
  if (a.flags & kLongDiscard) {
    // every line of this tile's rows of Y has been read: drop them from L2 unwritten
    constexpr int LPR = N2 * 8 / 128;  // 128-byte lines per row
    for (int i = int(threadIdx.x); i < D * LPR; i += NT)
      lg::discard_l2(reinterpret_cast<const char *>(yrow(i / LPR)) + (i % LPR) * 128);
  }
  const float fct = a.fct;
  const float sgn = a.conj_out ? -fct : fct;
  const uint64_t pol = input_policy((a.flags & kLongEvictOut) != 0);
  if constexpr (KIND != LG_R2C) {
    lg_middles<E2, D, NT, PB, 1, fx::np_of(E2) - 1>(sm, tw);
    // last pass: outputs k2 = j + k * NS of rows (2rp, 2rp + 1) to X[2rp + k2 n1] (16-byte stores)
    constexpr int P = fx::np_of(E2) - 1, R = fx::radix_of(E2, P), LR = N2 / R, NS = LR;
    constexpr int RP = D / 2, UNITS = RP * LR, ITER = UNITS / NT;
    static_assert(UNITS % NT == 0, "whole iterations");
    float2 *Xt = X + part * D;
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
      const int u = int(threadIdx.x) + it * NT;
      const int rp = u % RP, j = u / RP;
      float2 va[R], vb[R];
      lg_last_pair<E2, PB>(sm, tw, 2 * rp, j, va, vb);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int64_t k2 = j + k * NS;
        lg::st_x(reinterpret_cast<float4 *>(Xt + 2 * rp + k2 * N1),
                 make_float4(va[k].x * fct, va[k].y * sgn, vb[k].x * fct, vb[k].y * sgn), pol);
      }
    }
  } else {
    // r2c: every pass on chip, then the split of each row pair into X_k and X_{m-k}
    lg_middles<E2, D, NT, PB, 1, fx::np_of(E2)>(sm, tw);
    constexpr int64_t M = int64_t(N1) * N2;
    constexpr int H = D / 2;
    const float2 *lo2 = reinterpret_cast<const float2 *>(a.lo2), *hi2 = reinterpret_cast<const float2 *>(a.hi2);
    auto put = [&](int64_t k, float2 v) {
      float2 *p = X + k;
      const float vy = v.y * sgn;
      asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x * fct), "f"(vy), "l"(pol)
                   : "memory");
    };
    auto split = [&](int la, int pa, int lb, int pb, int64_t ka, bool two) {
      const float2 za = sm[la * PB + lg::sp(pa)], zc = cj<float>(sm[lb * PB + lg::sp(pb)]);
      const float2 Ev = scl<float>(add<float>(za, zc), 0.5f);
      const float2 O = mnegi<float>(scl<float>(sub<float>(za, zc), 0.5f));
      const float2 t = mul<float>(split_twiddle<float>(lo2, hi2, a.shift2, uint32_t(ka)), O);
      put(ka, add<float>(Ev, t));
      if (two) put(M - ka, cj<float>(sub<float>(Ev, t)));
    };
    for (int u = int(threadIdx.x); u < H * N2; u += NT) {
      const int i = u % H, k2 = u / H;
      int la, pa, lb, pb;
      pair_unit<D, N2>(part, i, k2, la, pa, lb, pb);
      split(la, pa, lb, pb, pair_index<N1, D>(part, la) + int64_t(N1) * pa, true);
    }
    if (part == 0 && threadIdx.x == 0) split(0, N2 / 2, 0, N2 / 2, M / 2, false);
  }
}

// ---- the persistent kernel ----

// Ticket block -> (group, phase).
__device__ __forceinline__ void lg_decode(int blk, int ng, int look, int &g, bool &isA) {
  if (look == 0) {
    g = blk >> 1;
    isA = (blk & 1) == 0;
  } else if (blk == 0) {
    g = 0;
    isA = true;
  } else if (blk == 2 * ng - 1) {
    g = ng - 1;
    isA = false;
  } else if (blk & 1) {
    g = (blk + 1) >> 1;
    isA = true;
  } else {
    g = (blk >> 1) - 1;
    isA = false;
  }
}

// KIND: LG_C2C (complex in, complex out), LG_R2C (real in, n/2+1 complex out), LG_C2R. Row
// offsets from the sides are in units of the side's element (float for real rows).
template <int KIND, int E1, int E2, int ET>
__global__ void __launch_bounds__(LgCfg<E1, E2, ET>::NT, 512 / LgCfg<E1, E2, ET>::NT)
    long_kernel(const __grid_constant__ LongArgs a) {
  using Cf = LgCfg<E1, E2, ET>;
  constexpr int64_t n = int64_t(1) << (E1 + E2);
  constexpr int TPA = Cf::N2 / Cf::C;  // A tiles per transform
  constexpr int TPB = Cf::N1 / Cf::D;  // B tiles per transform
  static_assert(TPA == TPB, "equal tile counts");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  extern __shared__ __align__(16) unsigned char smraw[];
  float2 *sm = reinterpret_cast<float2 *>(smraw);
  int &s_t = *reinterpret_cast<int *>(smraw + size_t(Cf::SLOTS) * 8);
  int &s_fail = *(&s_t + 1);
  const int N = a.tiles;
  const int total = 2 * a.ngroups * N;
  int *doneA = a.ctr + 3, *doneB = a.ctr + 3 + a.ngroups;
  for (;;) {
    if (threadIdx.x == 0) s_t = atomicAdd(a.ctr, 1);
    __syncthreads();
    const int t = s_t;
    if (t >= total) break;
    const int blk = t / N, tile = t - blk * N;
    int g;
    bool isA;
    lg_decode(blk, a.ngroups, a.look, g, isA);
    if (threadIdx.x == 0) {
      int fail = 0;
      if (isA) {
        if (g >= a.nbuf) fail = lg::wait_count(doneB + (g - a.nbuf), N, a.ctr + 1);
      } else {
        fail = lg::wait_count(doneA + g, N, a.ctr + 1);
      }
      s_fail = fail;
    }
    __syncthreads();
    if (s_fail) {
      if (threadIdx.x == 0) atomicOr(a.errw, 1);
      break;
    }
    const int bl = tile / TPA, part = tile - bl * TPA;
    const int64_t b = int64_t(g) * a.G + bl;
    if (b < a.batch) {
      float2 *ybase = reinterpret_cast<float2 *>(a.ybuf) + (int64_t(g % a.nbuf) * a.G + bl) * n;
      if (isA) {
        const float2 *x;
        if constexpr (KIND == LG_R2C)
          x = reinterpret_cast<const float2 *>(reinterpret_cast<const float *>(a.in) + side_offset(a.ld, b));
        else
          x = reinterpret_cast<const float2 *>(a.in) + side_offset(a.ld, b);
        lg_phase_a<KIND, E1, E2, ET>(a, sm, x, ybase, part);
      } else {
        float2 *X;
        if constexpr (KIND == LG_C2R)
          X = reinterpret_cast<float2 *>(reinterpret_cast<float *>(a.out) + side_offset(a.st, b));
        else
          X = reinterpret_cast<float2 *>(a.out) + side_offset(a.st, b);
        lg_phase_b<KIND, E1, E2, ET>(a, sm, ybase, X, part);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(isA ? doneA + g : doneB + g, 1);
    }
  }
}

}  // namespace rg
