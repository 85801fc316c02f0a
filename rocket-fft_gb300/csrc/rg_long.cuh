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
// segments: lanes run across the columns first); a phase-B tile is D = TT / n2 adjacent rows of
// Y (its HBM writes are D-element segments). Each thread runs one first-pass butterfly (radix
// 16, at most 64 registers, TT / 16 threads; radix 32 for phases of 2^9 or 2^10 points, at most
// 128 registers, TT / 32 threads, where a radix-16 first pass of the other phase of a complex
// transform takes two butterflies per thread) and the later passes' butterflies in turn. Both phases
// read their first radix pass straight from global memory into registers and write their last
// pass straight back; the passes in between run in place in one shared buffer, whose line pitch
// and padding period are chosen at compile time to minimise shared-memory wavefronts over the
// kernel's access patterns. Phase A's four-step twiddle is a per-butterfly table lookup times a
// factor from a per-tile table in shared memory.
//
// Y is the only intermediate, and it is kept in L2: transforms go through in groups of G
// (G * n * 8 bytes of Y per group), and group g uses slot g mod S of a ring of S Y buffers.
// Every tile is a ticket taken from an atomic counter; phase A runs `look` groups ahead of
// phase B, the tickets in the order
//     A0 .. A(look-1), then A(g) B(g-look) for g = look .. ng-1, then the remaining B
// A B(g) tile first waits until every A(g) tile is done; an A(g) tile waits until every
// B(g - S) tile has released its slot (S >= look + 1). A CTA waits only on tickets below its
// own; the lowest unfinished ticket is held by a running CTA and waits on nothing unfinished,
// so the launch always makes progress (a CTA holds its next ticket while it works on the
// current one, which keeps that true). Every wait is bounded (2 s of %globaltimer): past it the
// CTA sets the error word and every CTA leaves its loop.
// Y is written and read through L2 only (st/ld .cg), and a phase-B tile discards the Y lines it
// has consumed (discard.global.L2), so dead intermediate data is never written back to HBM.
//
// Real transforms of n = 2m points run the complex transform of length m on the real pairs
// z_j = x_2j + i x_2j+1 (the reference's rfftp for even n reaches the same spectrum by its own
// real radix passes, HDR:1836-2717). The split X_k = (Z_k + conj Z_{m-k}) / 2
// - i W_n^k (Z_k - conj Z_{m-k}) / 2 needs Z_k and Z_{m-k} together: with k = k1 + n1 k2,
// m - k = (n1 - k1) + n1 (n2 - 1 - k2), so an r2c phase-B tile holds D/2 rows k1 and their
// mirror rows n1 - k1 (tile 0: rows 0 and n1/2, which mirror onto themselves, and rows
// 1 .. D/2-1 with their mirrors) and stores X_k and X_{m-k} from each pair: past tile 0 the last
// pass runs a row's butterfly and the mirror row's mirrored butterfly in lanes l and l + 16 of
// one warp, which exchange their halves by shuffle; tile 0 splits from shared memory. c2r is
// the mirror image: its phase-A tile holds columns j2 and n2 - j2, merges the Hermitian half
// spectrum into conj(Z) as it loads (past tile 0 in the first pass's registers, the same lane
// pairing), and phase B stores conj of the result as the real pairs.
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
  int G, ngroups, nbuf, look;  // nbuf: ring slots S
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

// shared index of position pos of a line: one pad slot per 2^PS positions (PS = 3, 4 or 5,
// chosen per phase together with the line pitch)
__host__ __device__ constexpr int spad(int pos, int ps) { return pos + (pos >> ps); }

// The real transforms' paired passes (the r2c split after phase B's last pass, the c2r merge
// before phase A's first): lane l of warp w, iteration it, in a tile of `lines` lines with `nb`
// butterflies each. Lane l < 16 takes primary line i at butterfly j, lane l + 16 the mirror
// line lines-1-i at butterfly nb-1-j, so that output (r2c) or input (c2r) R-1-k of the one is
// the mirror element of the other's k.
__host__ __device__ constexpr void pair_lane(int w, int it, int warps, int l, int lines, int nb, int &line, int &j) {
  const int h = lines / 2, v = (w + it * warps) * 16 + (l & 15), i = v % h, q = v / h;
  line = l >= 16 ? lines - 1 - i : i;
  j = l >= 16 ? nb - 1 - q : q;
}

// spad(base + k * STEP, PS) as the base's index plus a compile-time offset, for the runs the
// passes use: STEP a multiple of 2^PS (any base); STEP 16 with PS 5 and base % 32 < 16; STEP 1
// with base a multiple of 16 (the first-pass writes, base = 16 j, k < 16); else spad().
template <int STEP, int PS> __device__ __forceinline__ int sp_k(int base, int k) {
  if constexpr (STEP % (1 << PS) == 0) return base + (base >> PS) + k * (STEP + (STEP >> PS));
  else if constexpr (PS == 5 && STEP == 16) return base + (base >> 5) + 16 * k + (k >> 1);
  else if constexpr (STEP == 1 && PS == 5) return base + (base >> 5) + k;
  else if constexpr (STEP == 1) return base + (base >> PS) + k + (k >> PS);
  else return spad(base + k * STEP, PS);
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

// evict-last L2 policy: the intermediate stays in L2 between the phases
__device__ __forceinline__ uint64_t keep_policy() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void st_keep(float2 *p, float2 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_out(float2 *p, float2 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void discard_l2(const void *p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

}  // namespace lg

// Shared-memory wavefronts of the lanes of the first warps over one tile phase whose M lines of
// length 2^E sit `pitch` slots apart (padding period 2^ps): the first pass's writes, every middle
// pass's reads and writes and the last pass's reads, each with its lane-to-(line, position)
// mapping. `a_side`: the first and last passes run lanes across the lines first (phase A: the
// columns; phase B: only its last pass). A warp's 8-byte accesses are served one half-warp at a
// time, 16 slots (128 bytes) per wavefront; this count matched the bank conflicts ncu measured
// on GB300 (2^14 points: 6.3 M modelled, 6.4 M measured excess store wavefronts).
namespace lg {
constexpr int wave(const int (&slot)[32]) {
  int total = 0;
  for (int h = 0; h < 2; ++h) {
    int cnt[16] = {}, worst = 0;
    for (int l = 16 * h; l < 16 * h + 16; ++l) {
      const int b = slot[l] & 15;
      if (++cnt[b] > worst) worst = cnt[b];
    }
    total += worst;
  }
  return total;
}
// Radix schedule of a phase of length 2^E: r0 = 16, the on-chip kernels' schedule (radix-16
// passes, the last one 16, 8, 4 or 2); r0 = 32 (E = 8 .. 10): two passes, 32 x 2^(E-5).
constexpr int np(int E, int r0) { return r0 == 32 ? 2 : fx::np_of(E); }
constexpr int radix(int E, int r0, int p) { return r0 == 32 ? (p == 0 ? 32 : (1 << E) / 32) : fx::radix_of(E, p); }
constexpr int ns(int E, int r0, int p) { return r0 == 32 ? (p == 0 ? 1 : 32) : fx::ns_of(E, p); }
// offset of pass p's twiddles in the phase's table (r0 = 32: the table of get_pass_tw)
constexpr int twoff(int E, int r0, int p) { return r0 == 32 ? 0 : fx::tw_of(E, p); }
// First-pass radix of a phase of 2^E points: 32 for 2^RG_LONG_R32_MIN .. 2^10, else 16. For 2^9
// and 2^10 the 32 x 2^(E-5) schedule has two passes instead of three (one shared-memory round
// trip and two barriers fewer per tile): measured on GB300 with both phases so, c2c 2^18 .. 2^20
// +11 %, r2c 2^21 +6 %. Taking 2^8 phases as 32 x 8 too (same pass count) measured -3 to -8 %
// except c2c 2^17 (+4 %), so the default range starts at 2^9. A CTA whose phases take radix 32
// and 16 runs TT / 32 threads; its radix-16 first pass then takes two butterflies per thread.
#ifndef RG_LONG_R32_MIN
#define RG_LONG_R32_MIN 9
#endif
constexpr int phase_radix(int E) { return E >= RG_LONG_R32_MIN && E <= 10 ? 32 : 16; }
// The first-pass radix of phase A (phase_a) or B of a shape of kind `kind`. Where only one phase
// takes radix 32 (2^8 x 2^9, 2^10 x 2^11), the complex transforms mix the two (c2c 2^17 +2.5 %,
// 2^21 +7 %) and the real ones keep radix 16 in both (mixed, r2c 2^18 measured 6 % slower).
constexpr int first_radix(int kind, int E1, int E2, bool phase_a) {
  const int ra = phase_radix(E1), rb = phase_radix(E2);
  if (ra != rb && kind != LG_C2C) return 16;
  return phase_a ? ra : rb;
}

// pair: the real transforms' paired lines instead, for phase A's first pass (c2r, a_side) or
// phase B's last pass (r2c): lane l < 16 of a warp on primary line i at butterfly j, lane l + 16
// on the mirror line M-1-i at the mirrored butterfly.
constexpr int phase_waves(int E, int M, int NT, int pitch, bool a_side, int ps, int r0, bool pair) {
  const int L = 1 << E, NP = np(E, r0);
  const bool pair_first = pair && a_side, pair_last = pair && !a_side;
  int total = 0;
  for (int w = 0; w < NT / 32 && w < 4; ++w) {
    int slot[32] = {};
    // first pass (radix r0, output position r0 j + k)
    for (int it = 0; it < (M * (L / r0)) / NT; ++it)
      for (int k = 0; k < r0; ++k) {
        for (int l = 0; l < 32; ++l) {
          const int u = 32 * w + l + it * NT;
          int line = a_side ? u % M : u / (L / r0), j = a_side ? u / M : u % (L / r0);
          if (pair_first) pair_lane(w, it, NT / 32, l, M, L / r0, line, j);
          slot[l] = line * pitch + spad(r0 * j + k, ps);
        }
        total += wave(slot);
      }
    for (int p = 1; p < NP; ++p) {
      const int R = radix(E, r0, p), LR = L / R, NS = ns(E, r0, p);
      for (int it = 0; it < (M * LR) / NT; ++it)
        for (int k = 0; k < R; ++k) {
          for (int l = 0; l < 32; ++l) {  // reads
            const int u = 32 * w + l + it * NT;
            const bool last = p == NP - 1;
            int line = last ? u % M : u / LR, j = last ? u / M : u % LR;
            if (last && pair_last) pair_lane(w, it, NT / 32, l, M, NS, line, j);
            slot[l] = line * pitch + spad(j + k * LR, ps);
          }
          total += wave(slot);
          if (p < NP - 1) {
            for (int l = 0; l < 32; ++l) {  // writes of a middle pass
              const int u = 32 * w + l + it * NT;
              const int line = u / LR, j = u % LR, m = j & (NS - 1);
              slot[l] = line * pitch + spad((j - m) * R + m + k * NS, ps);
            }
            total += wave(slot);
          }
        }
    }
  }
  return total;
}
// For padding period 2^ps: the pitch (>= the padded line length, within 16 slots of it) with
// the fewest wavefronts, as cost * 2^16 + pitch.
constexpr int best_pitch(int E, int M, int NT, bool a_side, int ps, int r0, bool pair = false) {
  const int base = spad((1 << E) - 1, ps) + 1;
  int best = base, cost = 1 << 14;
  for (int p = base; p < base + 16; ++p) {
    const int c = phase_waves(E, M, NT, p, a_side, ps, r0, pair);
    if (c < cost) {
      cost = c;
      best = p;
    }
  }
  return (cost << 16) + best;
}
// Of three such choices (periods 32, 16, 8), the one with the fewest wavefronts, as
// log2 period * 2^16 + pitch; ties keep the longer period (less padding).
constexpr int pick_layout(int c5, int c4, int c3) {
  const int k5 = c5 >> 16, k4 = c4 >> 16, k3 = c3 >> 16;
  if (k5 <= k4 && k5 <= k3) return (5 << 16) + (c5 & 0xffff);
  if (k4 <= k3) return (4 << 16) + (c4 & 0xffff);
  return (3 << 16) + (c3 & 0xffff);
}
}  // namespace lg

// Compile-time geometry of kind KIND: n1 = 2^E1 (phase-A length), n2 = 2^E2, tile of TT = 2^ET
// elements.
template <int E1, int E2, int ET, int KIND> struct LgCfg {
  static constexpr int N1 = 1 << E1, N2 = 1 << E2, TT = 1 << ET;
  static constexpr int C = TT / N1, D = TT / N2;  // columns per A tile, rows per B tile
  static constexpr int R0A = lg::first_radix(KIND, E1, E2, true), R0B = lg::first_radix(KIND, E1, E2, false);
  static constexpr int RMAX = R0A > R0B ? R0A : R0B;
  static constexpr int NT = TT / RMAX;            // threads: one radix-RMAX butterfly each
  // CTAs per SM the registers are sized for: 64 registers a thread at 16 points per thread, 128
  // at 32
  static constexpr int MINB = RMAX == 32 ? 512 / NT : 1024 / NT;
  // shared layout of each phase: padding period and line pitch (each candidate period searched
  // in a constant of its own, within the compiler's constant-evaluation budget)
  static constexpr bool PAIRA = KIND == LG_C2R;  // c2r: phase A's first pass on column pairs
  static constexpr int A5 = lg::best_pitch(E1, C, NT, true, 5, R0A, PAIRA);
  static constexpr int A4 = lg::best_pitch(E1, C, NT, true, 4, R0A, PAIRA);
  static constexpr int A3 = lg::best_pitch(E1, C, NT, true, 3, R0A, PAIRA);
  static constexpr bool PAIRB = KIND == LG_R2C;  // r2c: phase B's last pass on line pairs
  static constexpr int B5 = lg::best_pitch(E2, D, NT, false, 5, R0B, PAIRB);
  static constexpr int B4 = lg::best_pitch(E2, D, NT, false, 4, R0B, PAIRB);
  static constexpr int B3 = lg::best_pitch(E2, D, NT, false, 3, R0B, PAIRB);
  static constexpr int LA = lg::pick_layout(A5, A4, A3), LB = lg::pick_layout(B5, B4, B3);
  static constexpr int PA = LA & 0xffff, PB = LB & 0xffff;  // line pitches (slots)
  static constexpr int SA = LA >> 16, SB = LB >> 16;        // padding periods (log2)
  static constexpr int SLOTS = C * PA > D * PB ? C * PA : D * PB;
  // radix of phase A's last pass, and its per-tile factors W_n^{col k NS} (k = 1 .. RA-1, one
  // per column of the tile)
  static constexpr int RA = lg::radix(E1, R0A, lg::np(E1, R0A) - 1);
  static constexpr int FTAB = (RA - 1) * C;
  // the tile, the factor table, then two control words (ticket, wait failure): no static
  // shared memory, so the dynamic size may be raised to the device's opt-in maximum
  static constexpr size_t CTRL = size_t(SLOTS + FTAB) * 8;
  static constexpr size_t SMEM = CTRL + 16;
  static_assert(C >= 2 && D >= 2 && C <= 32 && D <= 32, "tile shape");
  static_assert(lg::radix(E1, R0A, 0) == R0A && lg::radix(E2, R0B, 0) == R0B, "first pass radix");
};

// ---- passes over lines of length 2^E held in shared memory (line l at sm + l * PITCH) ----

// Middle pass P, in place: all butterflies read (and transform) before a barrier, then write.
template <int E, int R0, int P, int M, int NT, int PITCH, int PS>
__device__ __forceinline__ void lg_middle(float2 *sm, const float2 *__restrict__ tw) {
  constexpr int L = 1 << E, R = lg::radix(E, R0, P), LR = L / R, NS = lg::ns(E, R0, P), TWO = lg::twoff(E, R0, P);
  constexpr int UNITS = M * LR, ITER = (UNITS + NT - 1) / NT;
  static_assert(UNITS % NT == 0, "whole iterations");
  float2 v[ITER][R];
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int u = int(threadIdx.x) + it * NT;
    const int line = u / LR, j = u % LR;
    const float2 *s = sm + line * PITCH;
#pragma unroll
    for (int k = 0; k < R; ++k) v[it][k] = s[lg::sp_k<LR, PS>(j, k)];
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
    for (int k = 0; k < R; ++k) s[lg::sp_k<NS, PS>(base, k)] = v[it][k];
  }
  __syncthreads();
}

template <int E, int R0, int M, int NT, int PITCH, int PS, int P, int PEND>
__device__ __forceinline__ void lg_middles(float2 *sm, const float2 *__restrict__ tw) {
  if constexpr (P < PEND) {
    lg_middle<E, R0, P, M, NT, PITCH, PS>(sm, tw);
    lg_middles<E, R0, M, NT, PITCH, PS, P + 1, PEND>(sm, tw);
  }
}

// Pass P in place like lg_middle, but with the lanes across the M lines first (butterfly j of
// line u % M): the pattern of the passes that read or write global memory, for which the
// layout is chosen. The real transforms run their on-chip first (c2r, phase A) or last (r2c,
// phase B) pass this way; along the lines, one pad slot per 8 positions puts lanes 0 and 15 of
// a half-warp on one bank. Measured on GB300 (2^15-point real rows): r2c bank conflicts
// 5.1 M -> 1.0 M per launch (launch -3 %), c2r +5-8 % at 2^15 and 2^16.
template <int E, int R0, int P, int M, int NT, int PITCH, int PS>
__device__ __forceinline__ void lg_pass_across(float2 *sm, const float2 *__restrict__ tw) {
  constexpr int L = 1 << E, R = lg::radix(E, R0, P), LR = L / R, NS = lg::ns(E, R0, P), TWO = lg::twoff(E, R0, P);
  constexpr int UNITS = M * LR, ITER = UNITS / NT;
  static_assert(UNITS % NT == 0, "whole iterations");
  float2 v[ITER][R];
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int u = int(threadIdx.x) + it * NT;
    const int line = u % M, j = u / M;
    const float2 *s = sm + line * PITCH;
#pragma unroll
    for (int k = 0; k < R; ++k) v[it][k] = s[lg::sp_k<LR, PS>(j, k)];
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
    const int line = u % M, j = u / M;
    const int m = j & (NS - 1), base = (j - m) * R + m;
    float2 *s = sm + line * PITCH;
#pragma unroll
    for (int k = 0; k < R; ++k) s[lg::sp_k<NS, PS>(base, k)] = v[it][k];
  }
  __syncthreads();
}

// Last-pass butterfly j of line l: inputs from shared memory, twiddled, transformed; output k
// lands at position j + k * NS of the transform.
template <int E, int R0, int PITCH, int PS>
__device__ __forceinline__ void lg_last_one(const float2 *sm, const float2 *__restrict__ tw, int l, int j,
                                            float2 (&a)[lg::radix(E, R0, lg::np(E, R0) - 1)]) {
  constexpr int L = 1 << E, P = lg::np(E, R0) - 1, R = lg::radix(E, R0, P), LR = L / R, NS = lg::ns(E, R0, P);
  constexpr int TWO = lg::twoff(E, R0, P);
  static_assert(NS == LR, "last pass");
  const float2 *s0 = sm + l * PITCH;
#pragma unroll
  for (int k = 0; k < R; ++k) a[k] = s0[lg::sp_k<LR, PS>(j, k)];
  if constexpr (NS > 1) {
    const float2 *t = tw + TWO + j;
#pragma unroll
    for (int k = 1; k < R; ++k) a[k] = mul<float>(a[k], __ldg(t + (k - 1) * NS));
  }
  dft<float, R>(a);
}

// ---- paired lines of the real transforms ----

// Line l of pair tile t over a dimension of length NL with H = LINES / 2 primary lines: lines
// [0, H) are the rows (or columns) t H + l, line LINES-1-i their mirror NL - (t H + i); tile 0
// holds 0 .. H-1, its mirrors NL-1 .. NL-H+1 on lines LINES-2 .. H, and NL/2 on line LINES-1.
template <int NL, int LINES>
__host__ __device__ __forceinline__ int pair_index(int t, int l) {
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
  using Cf = LgCfg<E1, E2, ET, KIND>;
  constexpr int N1 = Cf::N1, N2 = Cf::N2, C = Cf::C, NT = Cf::NT, PA = Cf::PA, SA = Cf::SA;
  const float2 *tw = reinterpret_cast<const float2 *>(a.twA);
  const float2 *lo = reinterpret_cast<const float2 *>(a.lo), *hi = reinterpret_cast<const float2 *>(a.hi);
  // The four-step twiddle of output k1 = j + k NS of column col, W_n^{col k1}, is applied as
  // W_n^{col j} (one table lookup per butterfly) times W_n^{col k NS} from a per-tile table in
  // shared memory: looked up per element, the scattered lo-table reads of a warp (one sector per
  // lane) were most of the kernel's L1 wavefronts. Visible to the last pass after the first
  // pass's barrier.
  float2 *ftab = sm + Cf::SLOTS;
  {
    constexpr int NS = N1 / Cf::RA;  // the last pass's stride (= its butterflies per line)
    for (int i = int(threadIdx.x); i < Cf::FTAB; i += NT) {
      const int kk = i / C + 1, cc = i - (kk - 1) * C;
      const int col = KIND == LG_C2R ? pair_index<N2, C>(part, cc) : part * C + cc;
      ftab[i] = split_twiddle<float>(lo, hi, a.shift, uint32_t(col) * uint32_t(kk * NS));
    }
  }
  if constexpr (KIND != LG_C2R) {
    // first pass: radix R0A straight from global memory (IT butterflies per thread, all loads
    // first); lanes run across the C columns first
    constexpr int R = Cf::R0A, LR = N1 / R, UNITS = C * LR, IT = UNITS / NT;
    static_assert(UNITS % NT == 0, "whole first-pass units per thread");
    const uint64_t pol = input_policy(true);
    constexpr int64_t STEP = int64_t(LR) * N2;
    float2 v[IT][R];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const int u = int(threadIdx.x) + it * NT;
      const int c = u % C, j = u / C;
      const float2 *p = x + part * C + int64_t(j) * N2 + c;
#pragma unroll
      for (int k = 0; k < R; ++k) v[it][k] = ld_in(p + k * STEP, pol);
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const int u = int(threadIdx.x) + it * NT;
      const int c = u % C, j = u / C;
      if (a.conj_in) {
#pragma unroll
        for (int k = 0; k < R; ++k) v[it][k].y = -v[it][k].y;
      }
      dft<float, R>(v[it]);
      float2 *l0 = sm + c * PA;
#pragma unroll
      for (int k = 0; k < R; ++k) l0[lg::sp_k<1, SA>(j * R, k)] = v[it][k];
    }
    __syncthreads();
    lg_middles<E1, Cf::R0A, C, NT, PA, SA, 1, lg::np(E1, Cf::R0A) - 1>(sm, tw);
  } else {
    // c2r: merge the half spectrum X (m + 1 elements, m = n1 n2) of columns j2 and n2 - j2
    // into conj(Z) on chip, then every pass but the last
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
    // conj(Z_ja) = conj(A + u) into za, conj(Z_{m-ja}) = A - u into zb,  A = X_ja + conj X_{m-ja},
    // u = i (X_ja - conj X_{m-ja}) conj(W_2m^ja)
    auto merge = [&](int64_t ja, float2 &za, float2 &zb) {
      const float2 xa = ldX(ja), xb = ldX(M - ja);
      const float2 A = add<float>(xa, cj<float>(xb)), B = sub<float>(xa, cj<float>(xb));
      const float2 w = split_twiddle<float>(lo2, hi2, a.shift2, uint32_t(ja));
      const float2 uu = mposi<float>(mulc<float>(B, w));
      za = cj<float>(add<float>(A, uu));
      zb = sub<float>(A, uu);
    };
    const int t = part;
    if (t != 0) {
      // The merge straight into the first pass: lane l < 16 of a warp runs butterfly j of primary
      // column line i, lane l + 16 butterfly LR-1-j of the mirror line C-1-i, whose input R-1-k
      // is the mirror element (index m - j) of the lane's input k. Each lane merges the pairs of
      // its inputs k < R/2 and hands the partner its half by shuffle (no shared-memory round trip
      // and no barrier before the pass). The layout's pitch is chosen for this pattern
      // (LgCfg::PAIRA).
      constexpr int R = Cf::R0A, LR = N1 / R;
      constexpr int WARPS = NT / 32, ITER = H * LR / (WARPS * 16);
      static_assert((H * LR) % (WARPS * 16) == 0 && R % 2 == 0, "whole pair iterations");
      for (int it = 0; it < ITER; ++it) {
        int line, jj;
        lg::pair_lane(int(threadIdx.x) >> 5, it, WARPS, int(threadIdx.x) & 31, C, LR, line, jj);
        const int64_t jb = int64_t(jj) * N2 + pair_index<N2, C>(t, line);
        float2 z[R];
#pragma unroll
        for (int k = 0; k < R / 2; ++k) merge(jb + int64_t(k) * LR * N2, z[k], z[R - 1 - k]);
        // z[R-1-k] (k < R/2) holds the partner's input R-1-k: swap those halves
#pragma unroll
        for (int k = R / 2; k < R; ++k) {
          z[k].x = __shfl_xor_sync(0xffffffffu, z[k].x, 16);
          z[k].y = __shfl_xor_sync(0xffffffffu, z[k].y, 16);
        }
        dft<float, R>(z);
        float2 *l0 = sm + line * PA;
#pragma unroll
        for (int k = 0; k < R; ++k) l0[lg::sp_k<1, SA>(jj * R, k)] = z[k];
      }
      __syncthreads();
    } else {
      // tile 0 (columns 0 and n2/2 mirror onto themselves): merge into shared memory, then the
      // first pass with the lanes across the columns
      auto merge_sm = [&](int la, int pa, int lb, int pb, int64_t ja, bool two) {
        float2 za, zb;
        merge(ja, za, zb);
        sm[la * PA + lg::spad(pa, SA)] = za;
        if (two) sm[lb * PA + lg::spad(pb, SA)] = zb;
      };
      constexpr int MERGE_IT = H * N1 / NT;
      static_assert((H * N1) % NT == 0 && NT % H == 0, "whole merge iterations");
#pragma unroll 4
      for (int it = 0; it < MERGE_IT; ++it) {
        const int u = int(threadIdx.x) + it * NT;
        const int i = u % H, j1 = u / H;
        int la, pa, lb, pb;
        pair_unit<C, N1>(0, i, j1, la, pa, lb, pb);
        const int64_t ja = int64_t(pa) * N2 + pair_index<N2, C>(0, la);
        merge_sm(la, pa, lb, pb, ja, ja != 0);
      }
      if (threadIdx.x == 0) merge_sm(0, N1 / 2, 0, N1 / 2, M / 2, false);
      __syncthreads();
      lg_pass_across<E1, Cf::R0A, 0, C, NT, PA, SA>(sm, tw);
    }
    lg_middles<E1, Cf::R0A, C, NT, PA, SA, 1, lg::np(E1, Cf::R0A) - 1>(sm, tw);
  }
  // last pass: outputs k1 = j + k * NS, times W_n^{j2 k1}, to Y[k1][j2]; lanes across the C
  // columns first (L2-resident stores, kept there with an evict-last policy)
  {
    constexpr int P = lg::np(E1, Cf::R0A) - 1, R = lg::radix(E1, Cf::R0A, P), LR = N1 / R, NS = LR;
    constexpr int UNITS = C * LR, ITER = UNITS / NT;
    static_assert(UNITS % NT == 0, "whole iterations");
    static_assert(R == Cf::RA, "factor table radix");
    const uint64_t keep = lg::keep_policy();
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
      const int u = int(threadIdx.x) + it * NT;
      const int c = u % C, j = u / C;
      float2 v[R];
      lg_last_one<E1, Cf::R0A, PA, SA>(sm, tw, c, j, v);
      const int col = KIND == LG_C2R ? pair_index<N2, C>(part, c) : part * C + c;
      float2 *yc = y + col;
      const float2 wj = split_twiddle<float>(lo, hi, a.shift, uint32_t(col) * uint32_t(j));
      lg::st_keep(yc + int64_t(j) * N2, mul<float>(v[0], wj), keep);
#pragma unroll
      for (int k = 1; k < R; ++k) {
        const float2 w = mul<float>(wj, ftab[(k - 1) * C + c]);
        lg::st_keep(yc + int64_t(j + k * NS) * N2, mul<float>(v[k], w), keep);
      }
    }
  }
}

// ---- phase B: D rows of Y ----

template <int KIND, int E1, int E2, int ET>
__device__ __forceinline__ void lg_phase_b(const LongArgs &a, float2 *sm, const float2 *__restrict__ yg,
                                           float2 *__restrict__ X, int part) {
  using Cf = LgCfg<E1, E2, ET, KIND>;
  constexpr int N1 = Cf::N1, N2 = Cf::N2, D = Cf::D, NT = Cf::NT, PB = Cf::PB, SB = Cf::SB;
  const float2 *tw = reinterpret_cast<const float2 *>(a.twB);
  // row of Y held by line r
  auto yrow = [&](int r) -> const float2 * {
    const int k1 = KIND == LG_R2C ? pair_index<N1, D>(part, r) : part * D + r;
    return yg + int64_t(k1) * N2;
  };
  // first pass: radix R0B from Y (L2; IT butterflies per thread, all loads first); lanes along
  // the row
  {
    constexpr int R = Cf::R0B, LR = N2 / R, UNITS = D * LR, IT = UNITS / NT;
    static_assert(UNITS % NT == 0, "whole first-pass units per thread");
    float2 v[IT][R];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const int u = int(threadIdx.x) + it * NT;
      const int r = u / LR, j = u % LR;
      const float2 *p = yrow(r) + j;
#pragma unroll
      for (int k = 0; k < R; ++k) v[it][k] = __ldcg(p + k * LR);
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const int u = int(threadIdx.x) + it * NT;
      const int r = u / LR, j = u % LR;
      dft<float, R>(v[it]);
      float2 *l = sm + r * PB;
#pragma unroll
      for (int k = 0; k < R; ++k) l[lg::sp_k<1, SB>(j * R, k)] = v[it][k];
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
    lg_middles<E2, Cf::R0B, D, NT, PB, SB, 1, lg::np(E2, Cf::R0B) - 1>(sm, tw);
    // last pass: outputs k2 = j + k * NS of row r to X[r + k2 n1]; lanes across the D rows first
    constexpr int P = lg::np(E2, Cf::R0B) - 1, R = lg::radix(E2, Cf::R0B, P), LR = N2 / R, NS = LR;
    constexpr int UNITS = D * LR, ITER = UNITS / NT;
    static_assert(UNITS % NT == 0, "whole iterations");
    float2 *Xt = X + part * D;
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
      const int u = int(threadIdx.x) + it * NT;
      const int r = u % D, j = u / D;
      float2 v[R];
      lg_last_one<E2, Cf::R0B, PB, SB>(sm, tw, r, j, v);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int64_t k2 = j + k * NS;
        lg::st_out(Xt + r + k2 * N1, make_float2(v[k].x * fct, v[k].y * sgn), pol);
      }
    }
  } else {
    // r2c: every pass but the last on chip, then the last pass and the split of each row pair
    // into X_k and X_{m-k}
    constexpr int NPB = lg::np(E2, Cf::R0B);
    lg_middles<E2, Cf::R0B, D, NT, PB, SB, 1, NPB - 1>(sm, tw);
    constexpr int64_t M = int64_t(N1) * N2;
    constexpr int H = D / 2;
    const float2 *lo2 = reinterpret_cast<const float2 *>(a.lo2), *hi2 = reinterpret_cast<const float2 *>(a.hi2);
    auto put = [&](int64_t k, float2 v) {
      float2 *p = X + k;
      const float vy = v.y * sgn;
      asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x * fct), "f"(vy), "l"(pol)
                   : "memory");
    };
    // X_ka and (two) X_{m-ka} from za = Z_ka and zb = Z_{m-ka}
    auto split = [&](float2 za, float2 zb, int64_t ka, bool two) {
      const float2 zc = cj<float>(zb);
      const float2 Ev = scl<float>(add<float>(za, zc), 0.5f);
      const float2 O = mnegi<float>(scl<float>(sub<float>(za, zc), 0.5f));
      const float2 t = mul<float>(split_twiddle<float>(lo2, hi2, a.shift2, uint32_t(ka)), O);
      put(ka, add<float>(Ev, t));
      if (two) put(M - ka, cj<float>(sub<float>(Ev, t)));
    };
    if (part != 0) {
      // The last pass straight into the split: lane l < 16 of a warp runs butterfly j of primary
      // line i, lane l + 16 butterfly NS-1-j of the mirror line D-1-i, whose output R-1-k is the
      // mirror element (index m - k) of the lane's output k. Each lane splits the pairs of its
      // outputs k < R/2; the partner's half comes by shuffle (no shared-memory round trip and
      // no barrier). The layout's pitch is chosen for this pattern (LgCfg::PAIRB).
      constexpr int P = NPB - 1, R = lg::radix(E2, Cf::R0B, P), NS = N2 / R;
      constexpr int WARPS = NT / 32, ITER = H * NS / (WARPS * 16);
      static_assert((H * NS) % (WARPS * 16) == 0 && R % 2 == 0, "whole pair iterations");
      for (int it = 0; it < ITER; ++it) {
        int line, jj;
        lg::pair_lane(int(threadIdx.x) >> 5, it, WARPS, int(threadIdx.x) & 31, D, NS, line, jj);
        float2 z[R];
        lg_last_one<E2, Cf::R0B, PB, SB>(sm, tw, line, jj, z);
        const int64_t kb = pair_index<N1, D>(part, line) + int64_t(N1) * jj;
#pragma unroll
        for (int k = 0; k < R / 2; ++k) {
          const float2 zb = make_float2(__shfl_xor_sync(0xffffffffu, z[R - 1 - k].x, 16),
                                        __shfl_xor_sync(0xffffffffu, z[R - 1 - k].y, 16));
          split(z[k], zb, kb + int64_t(N1) * NS * k, true);
        }
      }
    } else {
      // tile 0 (rows 0 and n1/2 mirror onto themselves): the last pass in place with the lanes
      // across the rows, then the split from shared memory
      lg_pass_across<E2, Cf::R0B, NPB - 1, D, NT, PB, SB>(sm, tw);
      auto at = [&](int l, int pos) { return sm[l * PB + lg::spad(pos, SB)]; };
      // H divides NT: a thread keeps its line pair i and steps through positions
      constexpr int SPLIT_IT = H * N2 / NT;
      static_assert((H * N2) % NT == 0 && NT % H == 0, "whole split iterations");
#pragma unroll 4
      for (int it = 0; it < SPLIT_IT; ++it) {
        const int u = int(threadIdx.x) + it * NT;
        const int i = u % H, k2 = u / H;
        int la, pa, lb, pb;
        pair_unit<D, N2>(0, i, k2, la, pa, lb, pb);
        split(at(la, pa), at(lb, pb), pair_index<N1, D>(0, la) + int64_t(N1) * pa, true);
      }
      if (threadIdx.x == 0) split(at(0, N2 / 2), at(0, N2 / 2), M / 2, false);
    }
  }
}

// ---- the persistent kernel ----

// Ticket block -> (group, phase), for lookahead `look` (0 <= look <= ng).
__host__ __device__ __forceinline__ void lg_decode(int blk, int ng, int look, int &g, bool &isA) {
  if (blk < look) {
    g = blk;
    isA = true;
  } else if (blk < 2 * ng - look) {
    const int k = blk - look;
    isA = (k & 1) == 0;
    g = isA ? look + (k >> 1) : (k >> 1);
  } else {
    g = blk - ng;
    isA = false;
  }
}

__device__ __forceinline__ void red_release_add(int *p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// KIND: LG_C2C (complex in, complex out), LG_R2C (real in, n/2+1 complex out), LG_C2R. Row
// offsets from the sides are in units of the side's element (float for real rows).
template <int KIND, int E1, int E2, int ET>
__global__ void __launch_bounds__(LgCfg<E1, E2, ET, KIND>::NT, LgCfg<E1, E2, ET, KIND>::MINB)
    long_kernel(const __grid_constant__ LongArgs a) {
  using Cf = LgCfg<E1, E2, ET, KIND>;
  constexpr int64_t n = int64_t(1) << (E1 + E2);
  constexpr int TPA = Cf::N2 / Cf::C;  // A tiles per transform
  constexpr int TPB = Cf::N1 / Cf::D;  // B tiles per transform
  static_assert(TPA == TPB, "equal tile counts");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  extern __shared__ __align__(16) unsigned char smraw[];
  float2 *sm = reinterpret_cast<float2 *>(smraw);
  int &s_t = *reinterpret_cast<int *>(smraw + Cf::CTRL);
  int &s_fail = *(&s_t + 1);
  const int N = a.tiles;
  const int total = 2 * a.ngroups * N;
  int *doneA = a.ctr + 3, *doneB = a.ctr + 3 + a.ngroups;
  int next = 0;  // thread 0: the ticket after the current one, taken while the current one runs
  if (threadIdx.x == 0) next = atomicAdd(a.ctr, 1);
  for (;;) {
    if (threadIdx.x == 0) {
      s_t = next;
      if (next < total) next = atomicAdd(a.ctr, 1);
    }
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
    // every thread's stores of this tile precede the count (barrier, then a release reduction)
    if (threadIdx.x == 0) red_release_add(isA ? doneA + g : doneB + g, 1);
  }
}

}  // namespace rg
