// Host side of the long complex64 / float32 real transforms (rg_long.cuh): the split
// n = n1 * n2 and tile size per length, the group size and Y ring, the per-call counters, and
// the launch.
#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "rg_error.hpp"
#include "rg_exec.hpp"
#include "rg_launch.hpp"
#include "rg_long_launch.cuh"
#include "rg_plan.hpp"

namespace rg {

namespace {

int env_int(const char *name, int dflt) {
  const char *e = std::getenv(name);
  return e && *e ? std::atoi(e) : dflt;
}

// Per-device error word the long kernels raise when a wait gives up (read and cleared by
// long_error_flag).
int *error_word() {
  static std::mutex mu;
  static int *words[64] = {};
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (!words[dev & 63]) {
    RG_CUDA(cudaMalloc(&words[dev & 63], sizeof(int)));
    RG_CUDA(cudaMemset(words[dev & 63], 0, sizeof(int)));
  }
  return words[dev & 63];
}

struct Shape {
  int e1, e2, et;
};

// Split and tile per log2 length. n1 <= n2, so that phase A (which reads the input from HBM)
// gets the wider segments. Tiles of 32 columns / rows (256-byte segments) for n1, n2 <= 2^8
// and 2^11 x 2^11, else 2^13 elements (64 KB of shared memory), 2^14 (128 KB) from 2^23 up,
// where 2^13 would leave two-element segments. Measured on GB300 (256 MiB batches): the
// one-step-larger tile gained 5-10 % at 2^14, 2^15 and 2^22 and lost 3-15 % at 2^16 .. 2^21.
// ROCKET_GPU_LONG_ET_SHIFT (-2 .. 1) takes other tiles where such an instance exists.
Shape shape_for(int e) {
  Shape s{0, 0, 0};
  switch (e) {
    case 14: s = {7, 7, 12}; break;
    case 15: s = {7, 8, 12}; break;
    case 16: s = {8, 8, 12}; break;
    case 17: s = {8, 9, 12}; break;
    case 18: s = {9, 9, 13}; break;
    case 19: s = {9, 10, 13}; break;
    case 20: s = {10, 10, 13}; break;
    case 21: s = {10, 11, 13}; break;
    case 22: s = {11, 11, 14}; break;
    case 23: s = {11, 12, 14}; break;
    case 24: s = {12, 12, 14}; break;
    default: return s;
  }
  const int shift = env_int("ROCKET_GPU_LONG_ET_SHIFT", 0);
  if (shift != 0 && shift >= -2 && shift <= 1 && long_shape_instantiated(s.e1, s.e2, s.et + shift)) s.et += shift;
  return s;
}

bool strides_multiple(const Side &s, int64_t q) {
  for (int d = 0; d < s.nbd; ++d)
    if (s.bstride[d] % q != 0) return false;
  return true;
}

bool pow2_in(int64_t n, int lo, int hi) {
  return n >= (int64_t(1) << lo) && n <= (int64_t(1) << hi) && (n & (n - 1)) == 0;
}

int log2_of(int64_t n) {
  int e = 0;
  while ((int64_t(1) << e) < n) ++e;
  return e;
}

// One launch of kind KIND for `nrows` transforms of complex length m (the half length of the
// real transforms).
template <int KIND>
void run_long(int64_t m, const void *in, const Side &ld, void *out, const Side &sd, int64_t nrows, bool cin,
              bool cout, double fct, const char *name, uint64_t bytes, cudaStream_t st) {
  const DType dt = DType::F32;
  const Shape s = shape_for(log2_of(m));
  RG_CHECK(s.e1 + s.e2 == log2_of(m), RG_ERR_INTERNAL, "no long-transform shape for this length");
  const int64_t tt = int64_t(1) << s.et;
  const int64_t ybytes = m * int64_t(cx_size(dt));
  // group: about ROCKET_GPU_LONG_GROUP_MB (32) MiB of Y; ring: as many groups as fit in
  // ROCKET_GPU_LONG_YMB (96) MiB, at most 8 (ROCKET_GPU_LONG_NBUF overrides); phase A runs
  // S - 2 groups ahead of phase B (ROCKET_GPU_LONG_LOOK overrides, at most S - 1). Measured on
  // GB300 (2^14 .. 2^22 points): 32 / 96 MiB ran 15-25 % faster than 8 / 64 MiB.
  const int64_t want = int64_t(env_int("ROCKET_GPU_LONG_GROUP_MB", 32)) << 20;
  const int64_t budget = int64_t(env_int("ROCKET_GPU_LONG_YMB", 96)) << 20;
  const int64_t G = std::max<int64_t>(1, std::min<int64_t>(nrows, want / ybytes));
  const int64_t ng = (nrows + G - 1) / G;
  int64_t nbuf = std::max<int64_t>(1, std::min<int64_t>(8, budget / (G * ybytes)));
  // one group of 64 MiB (2^23 complex points) fills the default ring: a second slot up to a
  // 128 MiB ring lets phase A of the next transform overlap phase B of this one (measured on
  // GB300: c2c 2^23 and r2c 2^24 +10-11 %)
  if (nbuf < 2 && !std::getenv("ROCKET_GPU_LONG_YMB") && 2 * G * ybytes <= (int64_t(128) << 20)) nbuf = 2;
  const int nenv = env_int("ROCKET_GPU_LONG_NBUF", 0);
  if (nenv >= 1 && nenv <= 16) nbuf = nenv;
  nbuf = std::min<int64_t>(nbuf, ng);
  int64_t look = std::max<int64_t>(0, nbuf - 2);
  const int lenv = env_int("ROCKET_GPU_LONG_LOOK", -1);
  if (lenv >= 0) look = lenv;
  look = std::min<int64_t>({look, nbuf - 1, ng});
  const int64_t tiles = G * m / tt;
  const int64_t tickets = 2 * ng * tiles;
  RG_CHECK(tickets < (int64_t(1) << 31) && ng < (int64_t(1) << 28), RG_ERR_UNSUPPORTED,
           "too many transforms in one call");
  // counters first (256-byte aligned block), then the Y ring
  const size_t ctr_bytes = (size_t(3 + 2 * ng) * sizeof(int) + 255) / 256 * 256;
  DevBuf ws(ctr_bytes + size_t(nbuf) * size_t(G) * size_t(ybytes), st);
  RG_CUDA(cudaMemsetAsync(ws.get(), 0, size_t(3 + 2 * ng) * sizeof(int), st));
  LongArgs a{};
  a.in = in;
  a.out = out;
  a.ld = ld;
  a.st = sd;
  a.batch = nrows;
  a.ctr = static_cast<int *>(ws.get());
  a.ybuf = static_cast<char *>(ws.get()) + ctr_bytes;
  a.errw = error_word();
  a.G = int(G);
  a.ngroups = int(ng);
  a.nbuf = int(nbuf);
  a.look = int(look);
  a.tiles = int(tiles);
  a.conj_in = cin ? 1 : 0;
  a.conj_out = cout ? 1 : 0;
  a.fct = float(fct);
  // pass twiddles of each phase's schedule (rg_long.cuh, lg::radix)
  a.twA = lg::first_radix(KIND, s.e1, s.e2, true) == 32 ? get_pass_tw(1 << s.e1, 32, dt) : get_core(1 << s.e1, dt).core.tw;
  a.twB = lg::first_radix(KIND, s.e1, s.e2, false) == 32 ? get_pass_tw(1 << s.e2, 32, dt) : get_core(1 << s.e2, dt).core.tw;
  const SplitTables sp = get_split(uint64_t(m), dt);
  a.lo = sp.lo;
  a.hi = sp.hi;
  a.shift = sp.shift;
  if (KIND != LG_C2C) {
    const SplitTables sp2 = get_split(uint64_t(2 * m), dt);
    a.lo2 = sp2.lo;
    a.hi2 = sp2.hi;
    a.shift2 = sp2.shift;
  }
  a.flags = (env_int("ROCKET_GPU_LONG_DISCARD", 1) ? kLongDiscard : 0) |
            (env_int("ROCKET_GPU_LONG_EVICT_OUT", 1) ? kLongEvictOut : 0);
  profiled_launch(name, bytes, st, [&] {
    RG_CHECK(long_dispatch<KIND>(s.e1, s.e2, s.et, a, tickets, st), RG_ERR_INTERNAL,
             "long-transform kernel not instantiated");
  });
}

}  // namespace

bool long_enabled() {
  static const bool on = env_int("ROCKET_GPU_LONG", 1) != 0;
  return on;
}

bool long_c2c_ok(DType dt, int64_t n, const void *in, const Side &ld, const void *out, const Side &sd) {
  if (dt != DType::F32 || !long_enabled() || !pow2_in(n, 14, 24)) return false;
  if (ld.axis_stride != 1 || sd.axis_stride != 1 || !strides_multiple(ld, 2) || !strides_multiple(sd, 2)) return false;
  return reinterpret_cast<uintptr_t>(in) % 16 == 0 && reinterpret_cast<uintptr_t>(out) % 16 == 0;
}

void long_c2c(DType, int64_t n, const void *in, const Side &ld, void *out, const Side &sd, int64_t nrows,
              bool cin, bool cout, double fct, cudaStream_t st) {
  run_long<LG_C2C>(n, in, ld, out, sd, nrows, cin, cout, fct, "long_c2c_f32", 2 * uint64_t(nrows) * uint64_t(n) * 8, st);
}

// Real rows of n = 2m points, m = 2^14 .. 2^23: the real side contiguous, its rows 16-byte
// aligned (two complex pairs per access); the half-spectrum side contiguous along the axis.
bool long_real_ok(DType dt, int64_t n, const void *real, const Side &rs, const Side &cs, double bscale) {
  if (dt != DType::F32 || !long_enabled() || bscale != 1.0 || n % 2 != 0 || !pow2_in(n / 2, 14, 23)) return false;
  if (rs.axis_stride != 1 || cs.axis_stride != 1 || !strides_multiple(rs, 4)) return false;
  return reinterpret_cast<uintptr_t>(real) % 16 == 0;
}

void long_r2c(int64_t n, const void *in, const Side &ld, void *out, const Side &sd, int64_t nrows, bool cout,
              double fct, cudaStream_t st) {
  const uint64_t bytes = uint64_t(nrows) * (uint64_t(n) * 4 + uint64_t(n / 2 + 1) * 8);
  run_long<LG_R2C>(n / 2, in, ld, out, sd, nrows, false, cout, fct, "long_r2c_f32", bytes, st);
}

void long_c2r(int64_t n, const void *in, const Side &ld, void *out, const Side &sd, int64_t nrows, bool cin,
              double fct, cudaStream_t st) {
  const uint64_t bytes = uint64_t(nrows) * (uint64_t(n) * 4 + uint64_t(n / 2 + 1) * 8);
  // phase B stores conj of the inverse transform as the real pairs (Re, -Im)
  run_long<LG_C2R>(n / 2, in, ld, out, sd, nrows, cin, true, fct, "long_c2r_f32", bytes, st);
}

int long_error_flag(cudaStream_t st) {
  int *w = error_word();
  int h = 0;
  RG_CUDA(cudaMemcpyAsync(&h, w, sizeof(int), cudaMemcpyDeviceToHost, st));
  RG_CUDA(cudaStreamSynchronize(st));
  if (h) RG_CUDA(cudaMemsetAsync(w, 0, sizeof(int), st));
  return h;
}

}  // namespace rg
