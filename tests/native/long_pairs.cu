// Host-compiled check of the long kernel's paired passes for the real transforms
// (rocket-fft_gb300/csrc/rg_long.cuh), for every instantiated shape and every tile past the
// first, with the kernel's own lane rule (lg::pair_lane) and line-to-row map (pair_index):
//  * r2c phase B: the last pass's butterflies cover each (line, position) of the tile once; the
//    output R-1-k of lane l ^ 16 is the mirror element (index m - ka) of lane l's output k; the
//    pairs a lane splits (its k < R/2) write every X index of the tile exactly once; and, for two
//    shapes (the layout search is costly to evaluate at compile time), the pass's shared reads
//    take one wavefront per half-warp under the layout LgCfg picks;
//  * c2r phase A: the merge's pairs fill each (column line, position) input of the first pass
//    once, and the element a lane merges for its partner is that partner's input R-1-k.
// Exit status 0 when every check holds.
#include <cstdio>
#include <set>
#include <vector>

#include "rg_long_launch.cuh"

using namespace rg;

namespace {

int failures = 0;

void fail(const char *what, int e1, int e2, int et, int t) {
  if (failures < 20) std::printf("FAIL %s: shape (%d, %d, %d), tile %d\n", what, e1, e2, et, t);
  ++failures;
}

template <int E1, int E2, int ET, bool WAVES> void check_r2c() {
  using Cf = LgCfg<E1, E2, ET, LG_R2C>;
  constexpr int N1 = Cf::N1, N2 = Cf::N2, D = Cf::D, NT = Cf::NT;
  constexpr int P = lg::np(E2, Cf::R0B) - 1, R = lg::radix(E2, Cf::R0B, P), NS = N2 / R;
  constexpr int H = D / 2, WARPS = NT / 32, ITER = H * NS / (WARPS * 16);
  constexpr long long M = static_cast<long long>(N1) * N2;
  static_assert((H * NS) % (WARPS * 16) == 0, "whole pair iterations");
  for (int t = 1; t < N1 / D; ++t) {
    std::vector<int> seen(D * N2, 0);
    std::set<long long> outs, expect;
    for (int i = 0; i < H; ++i)
      for (int k2 = 0; k2 < N2; ++k2) {
        const long long ka = pair_index<N1, D>(t, i) + static_cast<long long>(N1) * k2;
        expect.insert(ka);
        expect.insert(M - ka);
      }
    for (int w = 0; w < WARPS; ++w)
      for (int it = 0; it < ITER; ++it) {
        int line[32], jj[32];
        for (int l = 0; l < 32; ++l) lg::pair_lane(w, it, WARPS, l, D, NS, line[l], jj[l]);
        for (int k = 0; k < R; ++k) {
          int slot[32];
          for (int l = 0; l < 32; ++l) {
            const int pos = jj[l] + k * NS;
            if (line[l] < 0 || line[l] >= D || jj[l] < 0 || jj[l] >= NS) {
              fail("r2c lane out of the tile", E1, E2, ET, t);
              return;
            }
            seen[line[l] * N2 + pos]++;
            if constexpr (WAVES) slot[l] = line[l] * Cf::PB + lg::spad(pos, Cf::SB);
          }
          if constexpr (WAVES)
            if (lg::wave(slot) != 2) fail("r2c last-pass read not conflict-free", E1, E2, ET, t);
        }
        for (int l = 0; l < 32; ++l) {
          const int q = l ^ 16;
          const long long kb = pair_index<N1, D>(t, line[l]) + static_cast<long long>(N1) * jj[l];
          const long long kq = pair_index<N1, D>(t, line[q]) + static_cast<long long>(N1) * jj[q];
          for (int k = 0; k < R / 2; ++k) {
            const long long ka = kb + static_cast<long long>(N1) * NS * k;
            const long long kp = kq + static_cast<long long>(N1) * NS * (R - 1 - k);
            if (ka + kp != M) fail("r2c partner is not the mirror element", E1, E2, ET, t);
            if (ka <= 0 || ka >= M) fail("r2c index out of range", E1, E2, ET, t);
            if (!outs.insert(ka).second || !outs.insert(M - ka).second) fail("r2c output written twice", E1, E2, ET, t);
          }
        }
      }
    for (int s : seen)
      if (s != 1) {
        fail("r2c position not read exactly once", E1, E2, ET, t);
        break;
      }
    if (outs != expect) fail("r2c outputs differ from the tile's", E1, E2, ET, t);
  }
}

template <int E1, int E2, int ET> void check_c2r() {
  using Cf = LgCfg<E1, E2, ET, LG_C2R>;
  constexpr int N1 = Cf::N1, N2 = Cf::N2, C = Cf::C, NT = Cf::NT, R = Cf::R0A, LR = N1 / R;
  constexpr int H = C / 2, WARPS = NT / 32, ITER = H * LR / (WARPS * 16);
  constexpr long long M = static_cast<long long>(N1) * N2;
  static_assert((H * LR) % (WARPS * 16) == 0, "whole pair iterations");
  for (int t = 1; t < N2 / C; ++t) {
    std::vector<int> seen(C * N1, 0);
    for (int w = 0; w < WARPS; ++w)
      for (int it = 0; it < ITER; ++it) {
        int line[32], jj[32];
        for (int l = 0; l < 32; ++l) lg::pair_lane(w, it, WARPS, l, C, LR, line[l], jj[l]);
        for (int l = 0; l < 32; ++l) {
          if (line[l] < 0 || line[l] >= C || jj[l] < 0 || jj[l] >= LR) {
            fail("c2r lane out of the tile", E1, E2, ET, t);
            return;
          }
          const int q = l ^ 16;
          const long long jb = static_cast<long long>(jj[l]) * N2 + pair_index<N2, C>(t, line[l]);
          for (int k = 0; k < R; ++k) {
            const int pos = jj[l] + k * LR;
            seen[line[l] * N1 + pos]++;
            if (k >= R / 2) continue;
            // the element merged for input k, and the partner's input R-1-k (its mirror)
            const long long ja = jb + static_cast<long long>(k) * LR * N2;
            if (ja != static_cast<long long>(pos) * N2 + pair_index<N2, C>(t, line[l]))
              fail("c2r element index", E1, E2, ET, t);
            const long long ep = static_cast<long long>(jj[q] + (R - 1 - k) * LR) * N2 + pair_index<N2, C>(t, line[q]);
            if (M - ja != ep) fail("c2r partner input is not the mirror element", E1, E2, ET, t);
            if (ja <= 0 || ja >= M) fail("c2r index out of range", E1, E2, ET, t);
          }
        }
      }
    for (int s : seen)
      if (s != 1) {
        fail("c2r input not filled exactly once", E1, E2, ET, t);
        break;
      }
  }
}

}  // namespace

int main() {
  int shapes = 0;
#define X(a, b, c)          \
  check_r2c<a, b, c, false>(); \
  check_c2r<a, b, c>();        \
  ++shapes;
  RG_LONG_SHAPES(X)
#undef X
  // 32 lines of 8-point last butterflies, and 8 lines of 32-point ones
  check_r2c<7, 7, 12, true>();
  check_r2c<10, 10, 13, true>();
  std::printf("%d shapes, %d failures\n", shapes, failures);
  return failures != 0;
}
