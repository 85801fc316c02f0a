// Host-compiled check of the long kernel's tile schedule (rocket-fft_gb300/csrc/rg_long.cuh:
// lg_decode and the waits of long_kernel) for the group / ring / lookahead choices the host
// makes (rocket-fft_gb300/csrc/rg_long.cu: ring slots S in 1 .. min(16, groups), lookahead in
// 0 .. min(S - 1, groups)):
//  * the tickets hold, per group, one block of phase-A tiles and one of phase-B tiles;
//  * every tile waits only on tiles of lower tickets (B(g) on all of A(g); A(g), g >= S, on all
//    of B(g - S), which last used its ring slot);
//  * persistent CTAs that each hold their current ticket and the next one, run under random
//    interleavings, always finish every tile (no deadlock), and no phase-A tile writes a ring
//    slot while a phase-B tile of another group that reads it is unfinished or running.
// Exit status 0 when every check holds.
#include <cstdio>
#include <random>
#include <vector>

#include "rg_long_launch.cuh"

using namespace rg;

namespace {

int failures = 0;

void fail(const char *what, int ng, int nbuf, int look, int tiles, int ctas) {
  if (failures < 20)
    std::printf("FAIL %s: groups %d, slots %d, lookahead %d, tiles %d, CTAs %d\n", what, ng, nbuf, look, tiles,
                ctas);
  ++failures;
}

struct Tile {
  int g;
  bool isA;
};

Tile decode(int t, int tiles, int ng, int look) {
  Tile r{};
  lg_decode(t / tiles, ng, look, r.g, r.isA);
  return r;
}

// the lowest and highest ticket of group g's phase (A or B)
void block_of(int g, bool isA, int ng, int look, int tiles, int &lo, int &hi) {
  lo = 1 << 30;
  hi = -1;
  for (int t = 0; t < 2 * ng * tiles; ++t) {
    const Tile d = decode(t, tiles, ng, look);
    if (d.g == g && d.isA == isA) {
      lo = t < lo ? t : lo;
      hi = t > hi ? t : hi;
    }
  }
}

void check_static(int ng, int nbuf, int look, int tiles) {
  const int total = 2 * ng * tiles;
  std::vector<int> countA(ng, 0), countB(ng, 0);
  for (int t = 0; t < total; ++t) {
    const Tile d = decode(t, tiles, ng, look);
    if (d.g < 0 || d.g >= ng) {
      fail("ticket decodes to no group", ng, nbuf, look, tiles, 0);
      return;
    }
    (d.isA ? countA : countB)[d.g]++;
  }
  for (int g = 0; g < ng; ++g)
    if (countA[g] != tiles || countB[g] != tiles) fail("group phase without exactly its tiles", ng, nbuf, look, tiles, 0);
  for (int g = 0; g < ng; ++g) {
    int aLo, aHi, bLo, bHi;
    block_of(g, true, ng, look, tiles, aLo, aHi);
    block_of(g, false, ng, look, tiles, bLo, bHi);
    if (aHi - aLo != tiles - 1 || bHi - bLo != tiles - 1) fail("phase tiles not one block", ng, nbuf, look, tiles, 0);
    if (aHi >= bLo) fail("B(g) waits on a later ticket", ng, nbuf, look, tiles, 0);
    if (g >= nbuf) {
      int pLo, pHi;
      block_of(g - nbuf, false, ng, look, tiles, pLo, pHi);
      if (pHi >= aLo) fail("A(g) waits on a later ticket", ng, nbuf, look, tiles, 0);
    }
  }
}

void simulate(int ng, int nbuf, int look, int tiles, int ctas, unsigned seed) {
  const int total = 2 * ng * tiles;
  std::mt19937 rng(seed);
  std::vector<int> doneA(ng, 0), doneB(ng, 0), startedA(ng, 0), runningB(ng, 0);
  // per CTA: 4 = not started, 0 = taking tickets, 1 = waiting on its tile, 2 = running it,
  // 3 = left the loop
  std::vector<int> state(ctas, 4), cur(ctas, -1), next(ctas, -1);
  int counter = 0, finished = 0, exited = 0;
  std::vector<int> ready;
  for (int step = 0; step < 100 * total + 1000; ++step) {
    ready.clear();
    for (int c = 0; c < ctas; ++c) {
      if (state[c] == 3) continue;
      if (state[c] == 0 || state[c] == 2 || state[c] == 4) {
        ready.push_back(c);
        continue;
      }
      // the waits of long_kernel: A(g) on every B(g - S) tile, B(g) on every A(g) tile
      const Tile d = decode(cur[c], tiles, ng, look);
      const bool ok = d.isA ? (d.g < nbuf || doneB[d.g - nbuf] == tiles) : doneA[d.g] == tiles;
      if (ok) ready.push_back(c);
    }
    if (ready.empty()) break;
    const int c = ready[rng() % ready.size()];
    if (state[c] == 4) {  // the CTA starts: its first ticket
      next[c] = counter++;
      state[c] = 0;
    } else if (state[c] == 0) {  // s_t = next; next = atomicAdd(ticket) while next < total
      cur[c] = next[c];
      if (next[c] < total) next[c] = counter++;
      if (cur[c] >= total) {
        state[c] = 3;
        ++exited;
      } else {
        state[c] = 1;
      }
    } else if (state[c] == 1) {  // the wait is over: the tile starts
      const Tile d = decode(cur[c], tiles, ng, look);
      if (d.isA) {
        // the slot g % S must hold no unfinished reader of another group
        for (int h = d.g % nbuf; h < ng; h += nbuf)
          if (h != d.g && h < d.g && (doneB[h] != tiles || runningB[h] != 0))
            fail("A tile overwrites a ring slot still read", ng, nbuf, look, tiles, ctas);
        startedA[d.g]++;
      } else {
        for (int h = d.g % nbuf; h < ng; h += nbuf)
          if (h > d.g && startedA[h] != 0) fail("B tile reads a ring slot already rewritten", ng, nbuf, look, tiles, ctas);
        runningB[d.g]++;
      }
      state[c] = 2;
    } else {  // the tile finishes and is counted
      const Tile d = decode(cur[c], tiles, ng, look);
      if (d.isA) {
        doneA[d.g]++;
      } else {
        runningB[d.g]--;
        doneB[d.g]++;
      }
      ++finished;
      state[c] = 0;
    }
  }
  if (finished != total || exited != ctas) fail("tiles left unfinished (deadlock)", ng, nbuf, look, tiles, ctas);
}

}  // namespace

int main() {
  int configs = 0;
  for (int ng = 1; ng <= 12; ++ng)
    for (int nbuf = 1; nbuf <= (ng < 16 ? ng : 16); ++nbuf)
      for (int look = 0; look <= (nbuf - 1 < ng ? nbuf - 1 : ng); ++look)
        for (int tiles : {1, 3}) {
          check_static(ng, nbuf, look, tiles);
          for (int ctas : {1, 2, 5, 13})
            for (unsigned seed = 1; seed <= 3; ++seed) simulate(ng, nbuf, look, tiles, ctas, seed * 7919u + ng);
          ++configs;
        }
  std::printf("%d schedules, %d failures\n", configs, failures);
  return failures != 0;
}
