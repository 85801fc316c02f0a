// N-d driver: turns a (shape, strides, axes) request into axis jobs and each axis job into
// one kernel (length fits on chip), a four-step pair (long smooth lengths) or a Bluestein
// sequence (lengths with a prime factor above 13).
//
// Semantics follow the reference's drivers (rocket_fft/_pocketfft_hdronly.h):
//   c2c      general_nd 3568-3607: axes in the given order, the first reads `in`, later ones
//            work in place on `out`; fct is applied once (here: by the first axis job).
//   r2c      3955-3975: r2c along axes.back(), then c2c in place over the other axes.
//   c2r      3995-4023: c2c over axes[:-1] into a C-contiguous temporary, then c2r along
//            axes.back() with fct.
//   c2c_sym  rocket_fft/_pocketfft_numba.cpp:111-143: r2c into the full-size output, then
//            Hermitian completion (rg_launch.hpp MirrorArgs).
#include "rg_exec.hpp"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "rg_error.hpp"
#include "rg_exec_detail.hpp"
#include "rg_launch.hpp"
#include "rg_plane.hpp"

namespace rg {

// ---------------------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------------------

static cudaMemPool_t device_pool() {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    RG_CUDA(cudaMemPoolCreate(&pools[dev], &props));
    uint64_t thresh = UINT64_MAX;  // keep freed blocks for reuse
    RG_CUDA(cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &thresh));
  }
  return pools[dev];
}

DevBuf::DevBuf(size_t bytes, cudaStream_t st) : st_(st) {
  if (bytes == 0) bytes = 16;
  RG_CUDA(cudaMallocFromPoolAsync(&p_, bytes, device_pool(), st));
}

DevBuf::~DevBuf() {
  if (p_) cudaFreeAsync(p_, st_);
}

void pool_trim() { cudaMemPoolTrimTo(device_pool(), 0); }

// ---------------------------------------------------------------------------------------
// batch geometry
// ---------------------------------------------------------------------------------------

namespace detail {

Batch make_batch(const std::vector<int64_t> &shape, const std::vector<int64_t> &s_in,
                 const std::vector<int64_t> &s_out, int axis) {
  struct D {
    int64_t n, a, b;
  };
  std::vector<D> ds;
  for (int d = 0; d < int(shape.size()); ++d)
    if (d != axis && shape[d] > 1) ds.push_back({shape[d], s_in[d], s_out[d]});
  std::stable_sort(ds.begin(), ds.end(), [](const D &x, const D &y) {
    return std::llabs(x.a) + std::llabs(x.b) < std::llabs(y.a) + std::llabs(y.b);
  });
  std::vector<D> m;
  for (const D &d : ds) {
    if (!m.empty() && m.back().a * m.back().n == d.a && m.back().b * m.back().n == d.b)
      m.back().n *= d.n;
    else
      m.push_back(d);
  }
  Batch b;
  for (const D &d : m) {
    b.shape.push_back(d.n);
    b.s_in.push_back(d.a);
    b.s_out.push_back(d.b);
    b.nrows *= d.n;
  }
  return b;
}

Side make_side(int64_t axis_stride, const std::vector<int64_t> &shape,
               const std::vector<int64_t> &strides) {
  Side s{};
  RG_CHECK(shape.size() <= size_t(kMaxBatchDims), RG_ERR_UNSUPPORTED,
           "too many non-mergeable batch dimensions");
  s.axis_stride = axis_stride;
  s.nbd = int(shape.size());
  for (size_t d = 0; d < shape.size(); ++d) {
    s.bshape[d] = shape[d];
    s.bstride[d] = strides[d];
  }
  return s;
}

// prepend a batch dim (fastest) to a side
Side with_inner(const Side &s, int64_t n, int64_t stride, int64_t new_axis_stride) {
  RG_CHECK(s.nbd + 1 <= kMaxBatchDims, RG_ERR_UNSUPPORTED, "too many batch dimensions");
  Side r{};
  r.axis_stride = new_axis_stride;
  r.nbd = s.nbd + 1;
  r.bshape[0] = n;
  r.bstride[0] = stride;
  for (int d = 0; d < s.nbd; ++d) {
    r.bshape[d + 1] = s.bshape[d];
    r.bstride[d + 1] = s.bstride[d];
  }
  return r;
}

void set_colmap(Side &s) {
  s.colmap = (s.nbd > 0 && std::llabs(s.bstride[0]) < std::llabs(s.axis_stride)) ? 1 : 0;
}

Side contiguous_rows(int64_t nrows, int64_t len) {
  Side s{};
  s.axis_stride = 1;
  if (nrows > 1) {
    s.nbd = 1;
    s.bshape[0] = nrows;
    s.bstride[0] = len;
  }
  return s;
}

// Shared-memory geometry of an on-chip job: two ping-pong buffers of TB rows, each row
// padded (index i stored at i + (i >> ps)) and the row pitch made odd modulo the bank width
// so that column walks across rows do not conflict.
int row_pitch(DType dt, int Lsm, int &ps) {
  const int esz = int(cx_size(dt));
  ps = dt == DType::F32 ? 4 : 3;
  int pitch = Lsm + ((Lsm - 1) >> ps) + 1;
  const int mod = 128 / esz;
  while (pitch % mod != 1) ++pitch;
  return pitch;
}

size_t smem_bytes(DType dt, int TB, int pitch) {
  return 2 * size_t(TB) * pitch * cx_size(dt) + size_t(TB) * 20 + 16;
}

bool fits_core(int64_t L, DType dt) {
  if (L < 1 || L > kMaxCore || !core_smooth(uint64_t(L))) return false;
  int ps;
  const int pitch = row_pitch(dt, int(L) + 1, ps);
  return smem_bytes(dt, 1, pitch) <= max_smem_optin();
}

struct Geo {
  int TB, threads, pitch, ps;
  size_t smem;
};

// Rows per CTA, threads and shared memory for an on-chip job of core length L whose
// shared rows need Lsm complex slots. `pow2tb` keeps TB a power of two (the power-of-two
// kernel indexes rows with masks).
Geo choose_geo(DType dt, int L, int Lsm, bool col, int64_t nrows, bool pow2tb) {
  Geo g{};
  g.pitch = row_pitch(dt, Lsm, g.ps);
  const size_t maxsm = max_smem_optin();
  int TB;
  if (col)
    TB = dt == DType::F32 ? 16 : 8;
  else
    TB = std::max(1, (dt == DType::F32 ? 4096 : 2048) / L);
  if (int64_t(TB) > nrows && !(pow2tb && col)) TB = int(std::max<int64_t>(1, nrows));
  if (pow2tb)
    while (TB & (TB - 1)) TB &= TB - 1;
  // at most ~80 KB per CTA so that at least two CTAs share an SM
  const size_t budget_soft = 80 * 1024;
  for (;;) {
    const size_t smem = smem_bytes(dt, TB, g.pitch);
    if (smem <= (TB == 1 ? maxsm : std::min(maxsm, budget_soft))) {
      const int64_t work = int64_t(TB) * L / (dt == DType::F32 ? 16 : 8);
      g.TB = TB;
      g.threads = int(std::min<int64_t>(kMaxThreads, std::max<int64_t>(64, (work + 31) / 32 * 32)));
      g.smem = smem;
      return g;
    }
    if (TB == 1) throw Error(RG_ERR_INTERNAL, "no launch geometry for length " + std::to_string(L));
    TB = pow2tb ? TB / 2 : (TB > 4 ? TB - TB / 4 : TB - 1);
  }
}

// The power-of-two kernel can be switched off (ROCKET_GPU_POW2=0) to compare against the
// generic kernel.
bool pow2_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("ROCKET_GPU_POW2");
    return !(e && e[0] == '0');
  }();
  return on;
}



// The persistent pipelined kernel (rg_stream_kernel.cuh) can be switched off
// (ROCKET_GPU_STREAM=0); ROCKET_GPU_STREAM_S picks its stage count (2..4, default 2).
bool stream_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("ROCKET_GPU_STREAM");
    return e && e[0] == '1';
  }();
  return on;
}
// Out-of-place launches read their input once: the compile-time-L kernels load it evict-first
// (kFlagStream) so that it does not displace from L2 the data the next pass of the same
// transform reads. ROCKET_GPU_LDCS=0 loads it like any other data.
bool stream_loads_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("ROCKET_GPU_LDCS");
    return !(e && e[0] == '0');
  }();
  return on;
}

// L2 size of the current device, bytes (cached per device).
int64_t l2_bytes() {
  static std::atomic<int64_t> cache[64] = {};
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  std::atomic<int64_t> &c = cache[dev & 63];
  int64_t v = c.load(std::memory_order_relaxed);
  if (v == 0) {
    int b = 0;
    RG_CUDA(cudaDeviceGetAttribute(&b, cudaDevAttrL2CacheSize, dev));
    v = std::max<int64_t>(1, b);
    c.store(v, std::memory_order_relaxed);
  }
  return v;
}

// Evict-first input loads pay when the launch's output, which the next pass reads, can stay in
// L2: an out-of-place launch whose output takes at most 3/4 of it (measured on GB300: the
// 256^3 round trip, 67.6 MB spectra, 3.3 % faster; the 64 x 1024^2 rfftn, 269 MB, 0.8 % slower
// with the hint, so larger outputs load normally).
bool stream_loads(const Job &j) {
  if (j.in == j.out || !stream_loads_enabled()) return false;
  const bool real_out = j.op == OP_C2R_EVEN || j.op == OP_C2R_ODD || j.op == OP_DCT2 || j.op == OP_DCT3 ||
                        j.op == OP_DCT4_EVEN || j.op == OP_DCT1 || j.op == OP_DST1 || j.op == OP_R2R_FFTPACK_R2H ||
                        j.op == OP_R2R_FFTPACK_H2R || j.op == OP_HARTLEY || j.op == OP_DCT2_HALF ||
                        j.op == OP_DCT3_HALF;
  const int64_t out_bytes = j.nrows * int64_t(j.nout) * int64_t(real_out ? real_size(j.dt) : cx_size(j.dt));
  return 4 * out_bytes <= 3 * l2_bytes();
}

// The compile-time-L kernels (rg_fixed_kernel.cuh) can be switched off (ROCKET_GPU_FIXED=0).
bool fixed_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("ROCKET_GPU_FIXED");
    return !(e && e[0] == '0');
  }();
  return on;
}

// The plane kernels (rg_plane.cuh) are off unless ROCKET_GPU_PLANE=1 or set_plane_kernels(true):
// on GB300 they measured slower than the axis-by-axis kernels.
static std::atomic<int> g_plane{-1};
bool plane_enabled() {
  int v = g_plane.load(std::memory_order_relaxed);
  if (v < 0) {
    const char *e = std::getenv("ROCKET_GPU_PLANE");
    int want = (e && e[0] == '1') ? 1 : 0;
    g_plane.compare_exchange_strong(v, want);
    v = g_plane.load(std::memory_order_relaxed);
  }
  return v != 0;
}

// Reciprocals of the batch extents for 32-bit row decomposition; false if an extent does not
// fit the reciprocal range.
bool set_fastdivs(Side &s) {
  for (int d = 0; d < s.nbd; ++d) {
    if (s.bshape[d] <= 0 || s.bshape[d] >= (int64_t(1) << 31)) return false;
    s.bdiv[d] = make_fastdiv(uint32_t(s.bshape[d]));
  }
  return true;
}
int stream_stages() {
  static const int s = [] {
    const char *e = std::getenv("ROCKET_GPU_STREAM_S");
    const int v = e ? std::atoi(e) : 2;
    return v < 2 ? 2 : v > 4 ? 4 : v;
  }();
  return s;
}

// Geometry of the pipelined kernel: tiles of about 32 KB (4096 complex64 / 2048 complex128
// elements), 16 (8) rows for a column walk so that a tile row is one 128-byte segment, one
// radix-16 butterfly per thread, stages + 1 tile buffers and S + 1 slots of row offsets.
// Returns false when no tile fits in shared memory.
bool stream_geo(const Job &j, bool col, int stages, Geo &g) {
  const int esz = int(cx_size(j.dt));
  g.pitch = row_pitch(j.dt, j.Lsm, g.ps);
  const int target = j.dt == DType::F32 ? 4096 : 2048;
  int TB = col ? (j.dt == DType::F32 ? 16 : 8) : std::max(1, target / j.L);
  while (TB & (TB - 1)) TB &= TB - 1;
  const size_t maxsm = max_smem_optin();
  for (;;) {
    const size_t smem = size_t(stages + 1) * TB * g.pitch * esz + size_t(stages + 1) * 2 * TB * 8;
    if (smem <= maxsm) {
      g.TB = TB;
      g.smem = smem;
      const int64_t bf = int64_t(TB) * j.L / 16;
      g.threads = int(std::min<int64_t>(512, std::max<int64_t>(64, (bf + 31) / 32 * 32)));
      return true;
    }
    if (TB == 1 || (col && TB <= 4)) return false;
    TB /= 2;
  }
}

bool fixed_job_ok(const Job &j) {
  if (!(j.L >= 64 && (j.L & (j.L - 1)) == 0) || !pow2_enabled() || !fixed_enabled() || stream_enabled()) return false;
  Side ld = j.ld, sd = j.st;
  set_colmap(ld);
  set_colmap(sd);
  if (ld.colmap != sd.colmap || j.nrows >= (int64_t(1) << 31)) return false;
  if (!set_fastdivs(ld) || !set_fastdivs(sd)) return false;
  if (j.op == OP_C2C && j.cin != j.cout) return false;
  return j.L <= (ld.colmap ? 1024 : 8192);
}

void run_job(const Job &j, cudaStream_t st) {
  if (j.nrows <= 0) return;
  const CoreTables &ct = get_core(j.L, j.dt);
  Side ld = j.ld, sd = j.st;
  set_colmap(ld);
  set_colmap(sd);
  // power-of-two kernel: L = 2^k >= 2, ops with a direct first or last pass; a single pass
  // whose two sides walk differently stays on the generic kernel
  const bool pow2_op = j.op == OP_C2C || j.op == OP_C2C_TW || j.op == OP_R2C_EVEN || j.op == OP_C2R_EVEN;
  const bool pow2 = pow2_op && j.L >= 2 && (j.L & (j.L - 1)) == 0 && pow2_enabled() &&
                    !((j.op == OP_C2C || j.op == OP_C2C_TW) && ct.core.npass == 1 && ld.colmap != sd.colmap);
  // pipelined kernel: element-aligned sources (cp.async copies whole complex units)
  const size_t csz = cx_size(j.dt);
  bool stream = pow2 && stream_enabled() && (j.op == OP_C2C || j.op == OP_R2C_EVEN || j.op == OP_C2R_EVEN) &&
                j.L >= 16;
  int pair_ok = 0;
  if (stream) {
    const uintptr_t base = reinterpret_cast<uintptr_t>(j.in);
    if (j.op == OP_R2C_EVEN) {
      bool even = ld.axis_stride == 1 && base % csz == 0;
      for (int d = 0; d < ld.nbd; ++d) even = even && (ld.bstride[d] % 2 == 0);
      pair_ok = even ? 1 : 0;
      stream = base % real_size(j.dt) == 0;
    } else {
      stream = base % csz == 0;
    }
  }
  Geo g{};
  const int stages = stream_stages();
  if (stream) stream = stream_geo(j, ld.colmap != 0, stages, g);
  if (!stream) g = choose_geo(j.dt, j.L, j.Lsm, ld.colmap || sd.colmap, j.nrows, pow2);
  KArgs a{};
  a.in = j.in;
  a.out = j.out;
  a.ld = ld;
  a.st = sd;
  a.nrows = j.nrows;
  a.TB = g.TB;
  a.n = j.n;
  a.nin = j.nin;
  a.nout = j.nout;
  a.pitch = g.pitch;
  a.ps = g.ps;
  a.conj_in = j.cin;
  a.conj_out = j.cout;
  a.fct = j.fct;
  a.aux = j.aux;
  a.aux2 = j.aux2;
  a.aux3 = j.aux3;
  a.aux_n = j.aux_n;
  a.aux_s = j.aux_s;
  a.bscale = j.bscale;
  a.e0 = j.e0;
  a.flags = j.flags | (stream_loads(j) ? kFlagStream : 0);
  a.core = ct.core;
  const size_t smem = g.smem;
  LaunchCfg cfg;
  const int64_t grid = (j.nrows + g.TB - 1) / g.TB;
  RG_CHECK(grid < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "too many transforms in one call");
  cfg.grid = unsigned(grid);
  cfg.threads = g.threads;
  cfg.smem = smem;
  cfg.pow2 = pow2;
  if (stream) {
    cfg.stages = stages;
    cfg.pair_ok = pair_ok;
  }
  // compile-time-L kernel: power-of-two L, both sides walking alike, 32-bit row numbers,
  // C2C conjugating on both sides or neither
  const bool pow2L = j.L >= 2 && (j.L & (j.L - 1)) == 0 && pow2_enabled();
  const bool fixed_op = j.op == OP_C2C || j.op == OP_R2C_EVEN || j.op == OP_C2R_EVEN || j.op == OP_DCT2 ||
                        j.op == OP_DCT3 || j.op == OP_DCT2_HALF || j.op == OP_DCT3_HALF;
  if (pow2L && !stream && fixed_enabled() && fixed_op && ld.colmap == sd.colmap &&
      j.nrows < (int64_t(1) << 31) && (j.op != OP_C2C || j.cin == j.cout) && set_fastdivs(a.ld) &&
      set_fastdivs(a.st)) {
    cfg.fixed = true;
    cfg.col = ld.colmap != 0;
    cfg.bwd = j.op == OP_C2C && j.cin;
    const size_t rsz = real_size(j.dt);
    if (j.op == OP_R2C_EVEN || j.op == OP_DCT2 || j.op == OP_DCT2_HALF) {
      bool ok = ld.axis_stride == 1 && reinterpret_cast<uintptr_t>(j.in) % (2 * rsz) == 0;
      for (int d = 0; d < ld.nbd; ++d) ok = ok && ld.bstride[d] % 2 == 0;
      cfg.pair_ok = ok ? 1 : 0;
    } else if (j.op == OP_C2R_EVEN) {
      bool ok = sd.axis_stride == 1 && reinterpret_cast<uintptr_t>(j.out) % (2 * rsz) == 0;
      for (int d = 0; d < sd.nbd; ++d) ok = ok && sd.bstride[d] % 2 == 0;
      cfg.pair_ok = ok ? 1 : 0;
    }
  }
  RG_CHECK(cfg.fixed || (j.op != OP_DCT2_HALF && j.op != OP_DCT3_HALF), RG_ERR_INTERNAL,
           "half-length DCT job without a fixed-length kernel");
  launch_axis(j.dt, j.op, a, cfg, st);
}

void pointwise(DType dt, int op, const void *in, const Side &ld, void *out, const Side &sd,
               int64_t nrows, int nout, int n, bool cin, bool cout, double fct, const void *aux,
               const void *aux2, cudaStream_t st, double bscale = 1.0) {
  PwArgs p{};
  p.in = in;
  p.out = out;
  p.ld = ld;
  p.st = sd;
  p.nrows = nrows;
  p.nout = nout;
  p.n = n;
  p.conj_in = cin;
  p.conj_out = cout;
  p.fct = fct;
  p.bscale = bscale;
  p.aux = aux;
  p.aux2 = aux2;
  launch_pointwise(dt, op, p, st);
}

// Split n = n1 * n2 with both halves on chip, n1 as close to sqrt(n) as possible.
bool four_step_split(DType dt, int64_t n, int64_t &n1, int64_t &n2) {
  int64_t best = 0;
  for (int64_t d = 1; d * d <= n; ++d)
    if (n % d == 0 && fits_core(d, dt) && fits_core(n / d, dt)) best = d;
  if (!best) return false;
  n1 = best;
  n2 = n / best;
  return true;
}

// ---------------------------------------------------------------------------------------
// complex transforms of a batch of rows (any length)
// ---------------------------------------------------------------------------------------

void c2c_rows(DType dt, int64_t n, const void *in, const Side &ld, void *out, const Side &sd,
              int64_t nrows, bool cin, bool cout, double fct, cudaStream_t st);

void c2c_four_step(DType dt, int64_t n, int64_t n1, int64_t n2, const void *in, const Side &ld,
                   void *out, const Side &sd, int64_t nrows, bool cin, bool cout, double fct,
                   cudaStream_t st) {
  DevBuf ws(size_t(nrows) * size_t(n) * cx_size(dt), st);
  const SplitTables tw = get_split(uint64_t(n), dt);
  // pass A: columns j2 of length n1 (stride n2), twiddle W_n^{j2 k1}, into ws[row][k1][j2]
  Job a{};
  a.dt = dt;
  a.op = OP_C2C_TW;
  a.n = a.L = a.Lsm = a.nin = a.nout = int(n1);
  a.in = in;
  a.out = ws.get();
  a.ld = with_inner(ld, n2, ld.axis_stride, ld.axis_stride * n2);
  Side wsrows = contiguous_rows(nrows, n);
  a.st = with_inner(wsrows, n2, 1, n2);
  a.nrows = nrows * n2;
  a.cin = cin;
  a.cout = false;
  a.fct = 1.0;
  a.aux = tw.lo;
  a.aux2 = tw.hi;
  a.aux_s = tw.shift;
  a.aux_n = int(n2);
  run_job(a, st);
  // pass B: rows k1 of length n2 from ws, output element k2 to out[k2*n1 + k1]
  Job b{};
  b.dt = dt;
  b.op = OP_C2C;
  b.n = b.L = b.Lsm = b.nin = b.nout = int(n2);
  b.in = ws.get();
  b.out = out;
  b.ld = with_inner(wsrows, n1, n2, 1);
  b.st = with_inner(sd, n1, sd.axis_stride, sd.axis_stride * n1);
  b.nrows = nrows * n1;
  b.cin = false;
  b.cout = cout;
  b.fct = fct;
  run_job(b, st);
}

void c2c_bluestein_large(DType dt, int64_t n, const void *in, const Side &ld, void *out,
                         const Side &sd, int64_t nrows, bool cin, bool cout, double fct,
                         cudaStream_t st) {
  const BlueTables &bt = get_blue(uint64_t(n), dt);
  const int64_t m = int64_t(bt.m);
  DevBuf ws(size_t(nrows) * size_t(m) * cx_size(dt), st);
  const Side wrows = contiguous_rows(nrows, m);
  pointwise(dt, PW_BLUE_PRE, in, ld, ws.get(), wrows, nrows, int(m), int(n), cin, false, 1.0, bt.bk,
            bt.bkf, st);
  c2c_rows(dt, m, ws.get(), wrows, ws.get(), wrows, nrows, false, false, 1.0, st);
  pointwise(dt, PW_BLUE_MID, ws.get(), wrows, ws.get(), wrows, nrows, int(m), int(n), false, false,
            1.0, bt.bk, bt.bkf, st);
  c2c_rows(dt, m, ws.get(), wrows, ws.get(), wrows, nrows, false, false, 1.0, st);
  pointwise(dt, PW_BLUE_POST, ws.get(), wrows, out, sd, nrows, int(n), int(n), false, cout, fct,
            bt.bk, bt.bkf, st);
}

void c2c_rows(DType dt, int64_t n, const void *in, const Side &ld, void *out, const Side &sd,
              int64_t nrows, bool cin, bool cout, double fct, cudaStream_t st) {
  RG_CHECK(n < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "transform length too large");
  if (fits_core(n, dt)) {
    Job j{};
    j.dt = dt;
    j.op = OP_C2C;
    j.n = j.L = j.Lsm = j.nin = j.nout = int(n);
    j.in = in;
    j.out = out;
    j.ld = ld;
    j.st = sd;
    j.nrows = nrows;
    j.cin = cin;
    j.cout = cout;
    j.fct = fct;
    run_job(j, st);
    return;
  }
  if (long_c2c_ok(dt, n, in, ld, out, sd)) {
    long_c2c(dt, n, in, ld, out, sd, nrows, cin, cout, fct, st);
    return;
  }
  int64_t n1, n2;
  if (core_smooth(uint64_t(n)) && four_step_split(dt, n, n1, n2)) {
    c2c_four_step(dt, n, n1, n2, in, ld, out, sd, nrows, cin, cout, fct, st);
    return;
  }
  RG_CHECK(core_smooth(uint64_t(n)) == false, RG_ERR_UNSUPPORTED,
           "transform length too large for a two-pass decomposition");
  const uint64_t m = blue_length(uint64_t(n));
  if (fits_core(int64_t(m), dt)) {
    const BlueTables &bt = get_blue(uint64_t(n), dt);
    Job j{};
    j.dt = dt;
    j.op = OP_BLUE;
    j.n = int(n);
    j.L = j.Lsm = int(m);
    j.nin = j.nout = int(n);
    j.in = in;
    j.out = out;
    j.ld = ld;
    j.st = sd;
    j.nrows = nrows;
    j.cin = cin;
    j.cout = cout;
    j.fct = fct;
    j.aux = bt.bk;
    j.aux2 = bt.bkf;
    run_job(j, st);
    return;
  }
  c2c_bluestein_large(dt, n, in, ld, out, sd, nrows, cin, cout, fct, st);
}

// real -> half-complex along rows; conj_out conjugates (reference: forward=false)
void r2c_rows(DType dt, int64_t n, const void *in, const Side &ld, void *out, const Side &sd,
              int64_t nrows, bool cout, double fct, cudaStream_t st, double bscale) {
  RG_CHECK(n < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "transform length too large");
  if (n % 2 == 0 && fits_core(n / 2, dt)) {
    const int L = int(n / 2);
    Job j{};
    j.dt = dt;
    j.op = OP_R2C_EVEN;
    j.n = int(n);
    j.L = L;
    j.Lsm = L + 1;
    j.nin = L;  // real pairs
    j.nout = L + 1;
    j.in = in;
    j.out = out;
    j.ld = ld;
    j.st = sd;
    j.nrows = nrows;
    j.cin = false;
    j.cout = cout;
    j.fct = fct;
    j.bscale = bscale;
    j.aux = get_roots(uint64_t(n), uint64_t(L / 2 + 1), dt);
    run_job(j, st);
    return;
  }
  if (n % 2 == 1 && fits_core(n, dt)) {
    Job j{};
    j.dt = dt;
    j.op = OP_R2C_ODD;
    j.bscale = bscale;
    j.n = j.L = j.Lsm = j.nin = int(n);
    j.nout = int(n / 2 + 1);
    j.in = in;
    j.out = out;
    j.ld = ld;
    j.st = sd;
    j.nrows = nrows;
    j.cin = false;
    j.cout = cout;
    j.fct = fct;
    run_job(j, st);
    return;
  }
  if (long_real_ok(dt, n, in, ld, sd, bscale)) {
    long_r2c(n, in, ld, out, sd, nrows, cout, fct, st);
    return;
  }
  // general length: full complex transform of the real row, keep bins 0..n/2
  DevBuf ws(size_t(nrows) * size_t(n) * cx_size(dt), st);
  const Side w = contiguous_rows(nrows, n);
  pointwise(dt, PW_R2C_PACK, in, ld, ws.get(), w, nrows, int(n), int(n), false, false, 1.0, nullptr,
            nullptr, st);
  c2c_rows(dt, n, ws.get(), w, ws.get(), w, nrows, false, false, 1.0, st);
  pointwise(dt, PW_R2C_TAKE, ws.get(), w, out, sd, nrows, int(n / 2 + 1), int(n), false, cout, fct,
            nullptr, nullptr, st, bscale);
}

// half-complex -> real along rows; conj_in conjugates the input (reference: forward=true)
void c2r_rows(DType dt, int64_t n, const void *in, const Side &ld, void *out, const Side &sd,
              int64_t nrows, bool cin, double fct, cudaStream_t st, double bscale) {
  RG_CHECK(n < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "transform length too large");
  if (n % 2 == 0 && fits_core(n / 2, dt)) {
    const int L = int(n / 2);
    Job j{};
    j.dt = dt;
    j.op = OP_C2R_EVEN;
    j.n = int(n);
    j.L = L;
    j.Lsm = L + 1;
    j.nin = L + 1;
    j.nout = L;  // real pairs
    j.in = in;
    j.out = out;
    j.ld = ld;
    j.st = sd;
    j.nrows = nrows;
    j.cin = cin;
    j.cout = false;
    j.fct = fct;
    j.bscale = bscale;
    j.aux = get_roots(uint64_t(n), uint64_t(L / 2 + 1), dt);
    run_job(j, st);
    return;
  }
  if (n % 2 == 1 && fits_core(n, dt)) {
    Job j{};
    j.dt = dt;
    j.op = OP_C2R_ODD;
    j.bscale = bscale;
    j.n = j.L = j.Lsm = int(n);
    j.nin = int(n / 2 + 1);
    j.nout = int(n);
    j.in = in;
    j.out = out;
    j.ld = ld;
    j.st = sd;
    j.nrows = nrows;
    j.cin = cin;
    j.cout = false;
    j.fct = fct;
    run_job(j, st);
    return;
  }
  if (long_real_ok(dt, n, out, sd, ld, bscale)) {
    long_c2r(n, in, ld, out, sd, nrows, cin, fct, st);
    return;
  }
  DevBuf ws(size_t(nrows) * size_t(n) * cx_size(dt), st);
  const Side w = contiguous_rows(nrows, n);
  pointwise(dt, PW_C2R_BUILD, in, ld, ws.get(), w, nrows, int(n), int(n), cin, false, 1.0, nullptr,
            nullptr, st, bscale);
  c2c_rows(dt, n, ws.get(), w, ws.get(), w, nrows, false, false, 1.0, st);
  pointwise(dt, PW_C2R_TAKE, ws.get(), w, out, sd, nrows, int(n), int(n), false, false, fct, nullptr,
            nullptr, st);
}

// ---------------------------------------------------------------------------------------
// two-axis plane jobs (rg_plane.cuh): the last axis (real, contiguous) and the axis before it
// in the axis list, one cluster per plane
// ---------------------------------------------------------------------------------------

int log2_exact(int64_t n) {
  if (n < 1 || (n & (n - 1))) return -1;
  int e = 0;
  while ((int64_t(1) << e) < n) ++e;
  return e;
}

struct PlaneGeo {
  int a1 = -1, last = -1, E1 = 0, E2 = 0;
  int64_t L1 = 0, n2 = 0, H = 0, nplanes = 0;
  Batch b;  // the dimensions other than a1 and last (strides: complex side, real side)
};

// Plane geometry of an r2c (real = in, cplx = out) or c2r (cplx = in, real = out) request,
// false when no plane kernel applies: the real side must hold contiguous, aligned pairs along
// the last axis, the complex side unit stride along it.
bool plane_geo(DType dt, const NdArray &real, const NdArray &cplx, const Axes &axes, PlaneGeo &g) {
  if (axes.size() < 2 || !plane_enabled() || !fixed_enabled() || !pow2_enabled() || stream_enabled() ||
      tc_split_enabled())
    return false;
  g.last = int(axes.back());
  g.a1 = int(axes[axes.size() - 2]);
  if (g.a1 == g.last) return false;
  g.n2 = real.shape[g.last];
  g.L1 = real.shape[g.a1];
  g.E1 = int(log2_exact(g.L1));
  g.E2 = int(log2_exact(g.n2));
  if (g.E1 < 0 || g.E2 < 0 || plane_cluster(dt, g.E1, g.E2) == 0) return false;
  g.H = g.n2 / 2;
  if (real.stride[g.last] != 1 || cplx.stride[g.last] != 1) return false;
  if (reinterpret_cast<uintptr_t>(real.data) % (2 * real_size(dt)) != 0 || real.stride[g.a1] % 2 != 0) return false;
  std::vector<int64_t> shape = real.shape;
  shape[g.a1] = 1;
  g.b = make_batch(shape, cplx.stride, real.stride, g.last);
  for (int64_t sr : g.b.s_out)
    if (sr % 2 != 0) return false;
  if (g.b.shape.size() + 1 > size_t(kMaxBatchDims)) return false;
  g.nplanes = g.b.nrows;
  return g.nplanes * g.L1 < (int64_t(1) << 31) && g.nplanes * g.H < (int64_t(1) << 31);
}

// r2c along `last` then c2c along `a1`, in -> out, fct applied once. True if it ran.
bool plane_r2c(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, double fct, cudaStream_t st) {
  PlaneGeo g;
  if (!plane_geo(dt, in, out, axes, g)) return false;
  KArgs ar{}, ac{};
  ar.in = in.data;
  ar.ld = with_inner(make_side(1, g.b.shape, g.b.s_out), g.L1, in.stride[g.a1], 1);
  ar.nrows = g.L1 * g.nplanes;
  ar.core = get_core(int(g.H), dt).core;
  ar.aux = get_roots(uint64_t(g.n2), uint64_t(g.H / 2 + 1), dt);
  ar.fct = 1.0;
  ac.out = out.data;
  ac.st = with_inner(make_side(out.stride[g.a1], g.b.shape, g.b.s_in), g.H, out.stride[g.last], out.stride[g.a1]);
  ac.nrows = g.H * g.nplanes;
  ac.core = get_core(int(g.L1), dt).core;
  ac.fct = fct;
  if (!set_fastdivs(ar.ld) || !set_fastdivs(ac.st)) return false;
  const uint64_t bytes = uint64_t(g.nplanes * g.L1) * (uint64_t(g.n2) * real_size(dt) + uint64_t(g.H + 1) * cx_size(dt));
  bool ran = false;
  profiled_launch(dt == DType::F32 ? "plane_r2c_f32" : "plane_r2c_f64", bytes, st,
                  [&] { ran = launch_plane(dt, false, g.E1, g.E2, ar, ac, g.nplanes, st); });
  RG_CHECK(ran, RG_ERR_INTERNAL, "plane kernel instance missing");
  return true;
}

// c2c backward along `a1` then c2r along `last`, src -> out with fct. True if it ran.
bool plane_c2r(DType dt, const NdArray &src, const NdArray &out, const Axes &axes, double fct, cudaStream_t st) {
  PlaneGeo g;
  if (!plane_geo(dt, out, src, axes, g)) return false;
  KArgs ar{}, ac{};
  ac.in = src.data;
  ac.ld = with_inner(make_side(src.stride[g.a1], g.b.shape, g.b.s_in), g.H, src.stride[g.last], src.stride[g.a1]);
  ac.nrows = g.H * g.nplanes;
  ac.core = get_core(int(g.L1), dt).core;
  ac.fct = 1.0;
  ar.out = out.data;
  ar.st = with_inner(make_side(1, g.b.shape, g.b.s_out), g.L1, out.stride[g.a1], 1);
  ar.nrows = g.L1 * g.nplanes;
  ar.core = get_core(int(g.H), dt).core;
  ar.aux = get_roots(uint64_t(g.n2), uint64_t(g.H / 2 + 1), dt);
  ar.fct = fct;
  if (!set_fastdivs(ac.ld) || !set_fastdivs(ar.st)) return false;
  const uint64_t bytes = uint64_t(g.nplanes * g.L1) * (uint64_t(g.n2) * real_size(dt) + uint64_t(g.H + 1) * cx_size(dt));
  bool ran = false;
  profiled_launch(dt == DType::F32 ? "plane_c2r_f32" : "plane_c2r_f64", bytes, st,
                  [&] { ran = launch_plane(dt, true, g.E1, g.E2, ar, ac, g.nplanes, st); });
  RG_CHECK(ran, RG_ERR_INTERNAL, "plane kernel instance missing");
  return true;
}

bool any_zero(const std::vector<int64_t> &shape) {
  for (int64_t s : shape)
    if (s == 0) return true;
  return false;
}

}  // namespace detail

using namespace detail;

int set_plane_kernels(bool on) {
  const int prev = plane_enabled() ? 1 : 0;
  g_plane.store(on ? 1 : 0, std::memory_order_relaxed);
  return prev;
}

// ---------------------------------------------------------------------------------------
// public driver
// ---------------------------------------------------------------------------------------

void exec_c2c(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool forward,
              double fct, cudaStream_t st) {
  if (any_zero(out.shape)) return;
  for (size_t k = 0; k < axes.size(); ++k) {
    const NdArray &src = k == 0 ? in : out;
    const int ax = int(axes[k]);
    const Batch b = make_batch(out.shape, src.stride, out.stride, ax);
    const Side ld = make_side(src.stride[ax], b.shape, b.s_in);
    const Side sd = make_side(out.stride[ax], b.shape, b.s_out);
    c2c_rows(dt, out.shape[ax], src.data, ld, out.data, sd, b.nrows, !forward, !forward,
             k == 0 ? fct : 1.0, st);
  }
}

void exec_r2c(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool forward,
              double fct, cudaStream_t st, double bscale) {
  if (any_zero(in.shape) || axes.empty()) return;
  const int last = int(axes.back());
  if (forward && bscale == 1.0 && plane_r2c(dt, in, out, axes, fct, st)) {
    // the last two axes in one pass; the rest in place
    if (axes.size() > 2) {
      NdArray o = out;
      o.shape = in.shape;
      o.shape[last] = in.shape[last] / 2 + 1;
      exec_c2c(dt, o, o, Axes(axes.begin(), axes.end() - 2), forward, 1.0, st);
    }
    return;
  }
  const Batch b = make_batch(in.shape, in.stride, out.stride, last);
  const Side ld = make_side(in.stride[last], b.shape, b.s_in);
  const Side sd = make_side(out.stride[last], b.shape, b.s_out);
  r2c_rows(dt, in.shape[last], in.data, ld, out.data, sd, b.nrows, !forward, fct, st, bscale);
  if (axes.size() > 1) {
    NdArray o = out;
    o.shape = in.shape;
    o.shape[last] = in.shape[last] / 2 + 1;
    exec_c2c(dt, o, o, Axes(axes.begin(), axes.end() - 1), forward, 1.0, st);
  }
}

void exec_c2r(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool forward,
              double fct, cudaStream_t st, double bscale) {
  if (any_zero(out.shape) || axes.empty()) return;
  const int last = int(axes.back());
  std::vector<int64_t> shape_in = out.shape;
  shape_in[last] = out.shape[last] / 2 + 1;
  if (axes.size() == 1) {
    const Batch b = make_batch(out.shape, in.stride, out.stride, last);
    const Side ld = make_side(in.stride[last], b.shape, b.s_in);
    const Side sd = make_side(out.stride[last], b.shape, b.s_out);
    c2r_rows(dt, out.shape[last], in.data, ld, out.data, sd, b.nrows, forward, fct, st, bscale);
    return;
  }
  if (!forward && bscale == 1.0) {
    // the last two axes in one pass (after the other axes, into a temporary, if any)
    NdArray src = in;
    src.shape = shape_in;
    if (axes.size() == 2 && plane_c2r(dt, src, out, axes, fct, st)) return;
    NdArray t;  // C-contiguous temporary for the other axes
    t.shape = shape_in;
    t.stride.assign(shape_in.size(), 1);
    for (int d = int(shape_in.size()) - 2; d >= 0; --d) t.stride[d] = t.stride[d + 1] * shape_in[d + 1];
    PlaneGeo g;
    if (axes.size() > 2 && plane_geo(dt, out, t, axes, g)) {
      int64_t total = 1;
      for (int64_t s : shape_in) total *= s;
      DevBuf tmp(size_t(total) * cx_size(dt), st);
      t.data = tmp.get();
      exec_c2c(dt, src, t, Axes(axes.begin(), axes.end() - 2), forward, 1.0, st);
      RG_CHECK(plane_c2r(dt, t, out, axes, fct, st), RG_ERR_INTERNAL, "plane geometry changed");
      return;
    }
  }
  // C-contiguous complex temporary with the input's shape
  int64_t total = 1;
  for (int64_t s : shape_in) total *= s;
  DevBuf tmp(size_t(total) * cx_size(dt), st);
  NdArray t;
  t.data = tmp.get();
  t.shape = shape_in;
  t.stride.assign(shape_in.size(), 1);
  for (int d = int(shape_in.size()) - 2; d >= 0; --d) t.stride[d] = t.stride[d + 1] * shape_in[d + 1];
  NdArray src = in;
  src.shape = shape_in;
  exec_c2c(dt, src, t, Axes(axes.begin(), axes.end() - 1), forward, 1.0, st);
  const Batch b = make_batch(out.shape, t.stride, out.stride, last);
  const Side ld = make_side(t.stride[last], b.shape, b.s_in);
  const Side sd = make_side(out.stride[last], b.shape, b.s_out);
  c2r_rows(dt, out.shape[last], t.data, ld, out.data, sd, b.nrows, forward, fct, st, bscale);
}

void exec_c2c_sym(DType dt, const NdArray &in, const NdArray &out, const Axes &axes, bool forward,
                  double fct, cudaStream_t st) {
  if (any_zero(in.shape) || axes.empty()) return;
  exec_r2c(dt, in, out, axes, forward, fct, st);
  MirrorArgs m{};
  RG_CHECK(in.shape.size() <= size_t(kMaxDims), RG_ERR_UNSUPPORTED, "too many dimensions");
  m.data = out.data;
  m.ndim = int(in.shape.size());
  m.last = int(axes.back());
  for (uint64_t a : axes) m.revmask |= 1u << a;
  m.half = in.shape[m.last] / 2 + 1;
  m.total = 1;
  for (int d = 0; d < m.ndim; ++d) {
    m.shape[d] = in.shape[d];
    m.stride[d] = out.stride[d];
    m.total *= d == m.last ? m.half : in.shape[d];
  }
  launch_mirror(dt, m, st);
}

}  // namespace rg
