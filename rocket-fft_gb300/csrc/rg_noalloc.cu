// Allocation-free complex FFT: rocketgpu_c2c_noalloc (declared in include/rocket_gpu.h).
//
// Some callers cannot allocate device memory while they run: code inside a memory-capped or
// pre-partitioned CUDA context, real-time loops that must not take the allocator's locks or
// risk an out-of-memory failure midway, and hosts whose allocator belongs to another runtime
// (a framework caching allocator that does not want a second one beside it). The regular
// entry points allocate: plan tables are cudaMalloc'ed into the plan cache, and long
// transforms take their four-step workspace from a stream-ordered pool. This entry point
// allocates nothing: its tables and workspace live in one file-scope device array of
// kScratchBytes (32 MiB), which every GPU that loads the library holds until the process
// exits.
//
// Rules of use:
//  * device arrays only (host arrays would need staging buffers), complex64 or complex128;
//  * every transformed length must be 13-smooth (no Bluestein), on chip (<= 8192) or a
//    four-step product of two on-chip lengths; tables plus the largest four-step workspace
//    (rows * n * itemsize) must fit in kScratchBytes, otherwise the call returns
//    RG_ERR_UNSUPPORTED with a message naming the limit and does nothing;
//  * the array is shared by all calls and keeps the last call's contents; each call rewrites
//    the part it reads before reading it (a kernel computes the tables into it from parameters
//    passed by value, the workspace is fully written by the four-step first pass), so nothing
//    needs to start at zero and no host memory is read by the GPU. Calls whose GPU work
//    overlaps (different streams, or different host threads without ordering) race on it;
//  * the first call in a CUDA context of a device looks up the array's device address in that
//    context (cudaGetSymbolAddress); make that first call before any stream capture. Arrays
//    must live on the current device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rocket_gpu.h"
#include "rg_error.hpp"
#include "rg_launch.hpp"
#include "rg_plan.hpp"

static constexpr size_t kScratchBytes = size_t(32) << 20;  // 32 MiB

// The scratch array. In host code its name is only a host-side stand-in for the symbol, never
// a device address: the kernels receive the address cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

constexpr size_t kAlign = 256;

// The driver's current context, through the runtime's driver entry point (no link against the
// driver library); nullptr when the entry point is unavailable.
void *current_context() {
  using Fn = int (*)(void **);
  static Fn fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return Fn(nullptr);
    }
    return reinterpret_cast<Fn>(f);
  }();
  void *ctx = nullptr;
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}

// Device address of the scratch array in the current device and context. A __device__ array
// has one instance per context, so the address is looked up once per (device, context); when
// the context cannot be identified it is looked up on every call (the lookup allocates nothing).
void *scratch_address() {
  struct Ent {
    int dev;
    void *ctx, *addr;
  };
  static std::mutex mu;
  static std::vector<Ent> cache;
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  void *ctx = current_context();  // nullptr before the runtime has made a context current
  std::lock_guard<std::mutex> lk(mu);
  if (ctx)
    for (const Ent &e : cache)
      if (e.dev == dev && e.ctx == ctx) return e.addr;
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) rg::cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
  if (ctx) cache.push_back({dev, ctx, p});
  return p;
}

thread_local int t_status = RG_OK;

using rg::DType;
using rg::Error;

struct Arr {
  char *data;
  int64_t itemsize;
  std::vector<int64_t> shape, stride;  // stride in elements
};

// 1: device (or managed) memory of the current device; 0: not device memory; -1: device
// memory of another device.
int device_memory(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) return 0;
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  return at.type == cudaMemoryTypeManaged || at.device == dev ? 1 : -1;
}

Arr parse(uint64_t ndim, const rocketgpu_arystruct_t *a, const char *name) {
  RG_CHECK(a != nullptr, RG_ERR_ARG, std::string(name) + " is NULL");
  Arr r{static_cast<char *>(a->data), a->itemsize, std::vector<int64_t>(ndim), std::vector<int64_t>(ndim)};
  RG_CHECK(r.itemsize == 8 || r.itemsize == 16, RG_ERR_ARG, "complex64 or complex128 arrays required");
  for (uint64_t i = 0; i < ndim; ++i) {
    r.shape[i] = a->shape_and_strides[i];
    const int64_t bs = a->shape_and_strides[ndim + i];
    RG_CHECK(r.shape[i] >= 0, RG_ERR_ARG, "negative extent");
    RG_CHECK(bs % r.itemsize == 0, RG_ERR_UNSUPPORTED, "strides must be multiples of the item size");
    r.stride[i] = bs / r.itemsize;
  }
  return r;
}

// ---- on-device layout: [tables...][workspace], every block 256-byte aligned -------------

// One block of twiddles W_N^t = e^{-2 pi i t / N} in the scratch array: entry i has
// t = (i mod ns) * (i / ns + 1) (the radix-pass layout: (k - 1) * Ns + m -> m k) when ns > 0,
// else t = i * step (split tables).
struct TwSeg {
  uint64_t off;   // byte offset in the scratch array
  uint64_t N, step;
  uint32_t count, ns;
};
constexpr int kMaxSegs = 40;
struct TwFill {
  TwSeg seg[kMaxSegs];
  int nseg, f64;
};

// Computes the tables on the device from the descriptors (kernel parameters, passed by value):
// the angle 2 pi t / N as sincospi(2t / N) in double (2t and N exact in double), rounded once
// to the transform precision. One CTA row per descriptor.
__global__ void __launch_bounds__(256) noalloc_tables(unsigned char *base, const __grid_constant__ TwFill f) {
  const TwSeg sg = f.seg[blockIdx.y];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < sg.count; i += gridDim.x * blockDim.x) {
    uint64_t t = sg.ns ? uint64_t(i % sg.ns) * uint64_t(i / sg.ns + 1) : uint64_t(i) * sg.step;
    t %= sg.N;
    double sn, cs;
    sincospi(double(2 * t) / double(sg.N), &sn, &cs);
    if (f.f64)
      reinterpret_cast<double2 *>(base + sg.off)[i] = make_double2(cs, -sn);
    else
      reinterpret_cast<float2 *>(base + sg.off)[i] = make_float2(float(cs), float(-sn));
  }
}

struct Arena {
  DType dt;
  size_t bytes = 0;  // tables so far
  std::vector<TwSeg> segs;
  size_t ws_bytes = 0;

  // room for `count` entries; returns the block's byte offset
  size_t put(uint64_t count, uint64_t N, uint32_t ns, uint64_t step) {
    const size_t off = (bytes + kAlign - 1) / kAlign * kAlign;
    bytes = off + std::max<size_t>(count, 1) * rg::cx_size(dt);
    if (count > 0) segs.push_back({off, N, step, uint32_t(count), ns});
    return off;
  }
  size_t tables_bytes() const { return (bytes + kAlign - 1) / kAlign * kAlign; }

  void fill(unsigned char *base, cudaStream_t st) const {
    for (size_t s0 = 0; s0 < segs.size(); s0 += kMaxSegs) {
      TwFill f{};
      f.nseg = int(std::min<size_t>(kMaxSegs, segs.size() - s0));
      f.f64 = dt == DType::F64 ? 1 : 0;
      uint32_t most = 1;
      for (int k = 0; k < f.nseg; ++k) {
        f.seg[k] = segs[s0 + size_t(k)];
        most = std::max(most, f.seg[k].count);
      }
      const unsigned gx = std::min<unsigned>(64, (most + 255) / 256);
      noalloc_tables<<<dim3(gx, unsigned(f.nseg)), 256, 0, st>>>(base, f);
      rg::note_launch();
      RG_CUDA(cudaGetLastError());
    }
  }
};

// Pass descriptors + twiddles of an on-chip FFT of length L (Stockham radix passes, the
// same schedule the cached plans use); core.tw is filled in once the arena has an address.
struct CoreRef {
  rg::FFTCore core;
  size_t off;
};

CoreRef add_core(Arena &ar, int L) {
  CoreRef c{};
  const std::vector<int> rad = rg::core_radices(L);
  RG_CHECK(int(rad.size()) <= rg::kMaxPass, RG_ERR_UNSUPPORTED, "too many passes");
  c.core.L = L;
  c.core.npass = int(rad.size());
  // the passes' twiddles back to back: pass p with Ns > 1 holds W_{Ns R}^{m k} at
  // (k - 1) Ns + m, from entry pd.tw on
  int Ns = 1, total = 0;
  for (int p = 0; p < c.core.npass; ++p) {
    rg::PassDesc &pd = c.core.pass[p];
    pd.R = rad[p];
    pd.Ns = Ns;
    pd.LR = L / pd.R;
    pd.tw = total;
    pd.dNs = rg::make_fastdiv(uint32_t(Ns));
    pd.dLR = rg::make_fastdiv(uint32_t(pd.LR));
    if (Ns > 1) total += (pd.R - 1) * Ns;
    Ns *= pd.R;
  }
  c.off = (ar.bytes + kAlign - 1) / kAlign * kAlign;  // the block's start (entries follow per pass)
  for (int p = 0; p < c.core.npass; ++p) {
    const rg::PassDesc &pd = c.core.pass[p];
    if (pd.Ns == 1) continue;
    const uint64_t cnt = uint64_t(pd.R - 1) * pd.Ns;
    ar.segs.push_back({c.off + size_t(pd.tw) * rg::cx_size(ar.dt), uint64_t(pd.Ns) * pd.R, 0, uint32_t(cnt),
                       uint32_t(pd.Ns)});
  }
  ar.bytes = c.off + std::max<size_t>(total, 1) * rg::cx_size(ar.dt);
  return c;
}

struct SplitRef {
  size_t lo, hi;
  int shift;
};

SplitRef add_split(Arena &ar, uint64_t N) {
  int bits = 0;
  while ((uint64_t(1) << bits) < N) ++bits;
  const int shift = (bits + 1) / 2;
  const uint64_t nlo = uint64_t(1) << shift, nhi = (N + nlo - 1) / nlo;
  SplitRef s{};
  s.lo = ar.put(nlo, N, 0, 1);    // W_N^t, t < 2^shift
  s.hi = ar.put(nhi, N, 0, nlo);  // W_N^{t 2^shift}
  s.shift = shift;
  return s;
}

// ---- geometry (same rules as the allocating driver) -------------------------------------

constexpr int kMaxCore = 8192;

int row_pitch(DType dt, int Lsm, int &ps) {
  const int esz = int(rg::cx_size(dt));
  ps = dt == DType::F32 ? 4 : 3;
  int pitch = Lsm + ((Lsm - 1) >> ps) + 1;
  while (pitch % (128 / esz) != 1) ++pitch;
  return pitch;
}

size_t smem_bytes(DType dt, int TB, int pitch) { return 2 * size_t(TB) * pitch * rg::cx_size(dt) + size_t(TB) * 20 + 16; }

bool on_chip(int64_t L, DType dt) {
  if (L < 1 || L > kMaxCore || !rg::core_smooth(uint64_t(L))) return false;
  int ps;
  return smem_bytes(dt, 1, row_pitch(dt, int(L) + 1, ps)) <= rg::max_smem_optin();
}

bool split2(DType dt, int64_t n, int64_t &n1, int64_t &n2) {
  int64_t best = 0;
  for (int64_t d = 1; d * d <= n; ++d)
    if (n % d == 0 && on_chip(d, dt) && on_chip(n / d, dt)) best = d;
  if (!best) return false;
  n1 = best;
  n2 = n / best;
  return true;
}

struct Batch {
  std::vector<int64_t> shape, si, so;
  int64_t rows = 1;
};

Batch batch_of(const Arr &src, const Arr &dst, int axis) {
  struct D {
    int64_t n, a, b;
  };
  std::vector<D> ds;
  for (int d = 0; d < int(dst.shape.size()); ++d)
    if (d != axis && dst.shape[d] > 1) ds.push_back({dst.shape[d], src.stride[d], dst.stride[d]});
  std::stable_sort(ds.begin(), ds.end(), [](const D &x, const D &y) {
    return std::llabs(x.a) + std::llabs(x.b) < std::llabs(y.a) + std::llabs(y.b);
  });
  Batch b;
  for (const D &d : ds) {
    if (!b.shape.empty() && b.si.back() * b.shape.back() == d.a && b.so.back() * b.shape.back() == d.b) {
      b.shape.back() *= d.n;
    } else {
      b.shape.push_back(d.n);
      b.si.push_back(d.a);
      b.so.push_back(d.b);
    }
    b.rows *= d.n;
  }
  return b;
}

rg::Side side(int64_t axis_stride, const std::vector<int64_t> &shape, const std::vector<int64_t> &st,
              int64_t inner_n = 0, int64_t inner_stride = 0) {
  rg::Side s{};
  const int extra = inner_n ? 1 : 0;
  RG_CHECK(int(shape.size()) + extra <= rg::kMaxBatchDims, RG_ERR_UNSUPPORTED, "too many batch dimensions");
  s.axis_stride = axis_stride;
  s.nbd = int(shape.size()) + extra;
  if (extra) {
    s.bshape[0] = inner_n;
    s.bstride[0] = inner_stride;
  }
  for (size_t d = 0; d < shape.size(); ++d) {
    s.bshape[d + extra] = shape[d];
    s.bstride[d + extra] = st[d];
  }
  s.colmap = (s.nbd > 0 && std::llabs(s.bstride[0]) < std::llabs(s.axis_stride)) ? 1 : 0;
  return s;
}

void launch_c2c(DType dt, int op, const rg::FFTCore &core, const void *in, const rg::Side &ld, void *out,
                const rg::Side &sd, int64_t nrows, bool cin, bool cout, double fct, const void *aux,
                const void *aux2, int aux_n, int aux_s, cudaStream_t st) {
  if (nrows <= 0) return;
  const int L = core.L;
  int ps = 0;
  const int pitch = row_pitch(dt, L, ps);
  const bool col = ld.colmap || sd.colmap;
  int TB = col ? (dt == DType::F32 ? 16 : 8) : std::max(1, (dt == DType::F32 ? 4096 : 2048) / L);
  if (int64_t(TB) > nrows) TB = int(std::max<int64_t>(1, nrows));
  const size_t maxsm = rg::max_smem_optin();
  while (TB > 1 && smem_bytes(dt, TB, pitch) > std::min<size_t>(maxsm, col ? 160 * 1024 : 112 * 1024)) --TB;
  RG_CHECK(smem_bytes(dt, TB, pitch) <= maxsm, RG_ERR_INTERNAL, "no launch geometry");
  rg::KArgs a{};
  a.in = in;
  a.out = out;
  a.ld = ld;
  a.st = sd;
  a.nrows = nrows;
  a.TB = TB;
  a.n = a.nin = a.nout = L;
  a.pitch = pitch;
  a.ps = ps;
  a.conj_in = cin;
  a.conj_out = cout;
  a.fct = fct;
  a.aux = aux;
  a.aux2 = aux2;
  a.aux_n = aux_n;
  a.aux_s = aux_s;
  a.core = core;
  rg::LaunchCfg cfg;
  const int64_t grid = (nrows + TB - 1) / TB;
  RG_CHECK(grid < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "too many transforms in one call");
  cfg.grid = unsigned(grid);
  const int64_t work = int64_t(TB) * L / (dt == DType::F32 ? 16 : 8);
  cfg.threads = int(std::min<int64_t>(rg::kMaxThreads, std::max<int64_t>(64, (work + 31) / 32 * 32)));
  cfg.smem = smem_bytes(dt, TB, pitch);
  cfg.pow2 = false;
  rg::launch_axis(dt, op, a, cfg, st);
}

struct AxisPlan {
  int axis;
  int64_t n, n1 = 0, n2 = 0;
  CoreRef c0, c1;  // on chip: c0; four-step: c0 = n1 (columns), c1 = n2 (rows)
  SplitRef tw{};
  size_t ws = 0;   // workspace bytes
};

void run(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
         rocketgpu_arystruct_t *axes, bool forward, double fct, cudaStream_t st) {
  const Arr in = parse(ndim, ain, "ain"), out = parse(ndim, aout, "aout");
  RG_CHECK(in.itemsize == out.itemsize, RG_ERR_ARG, "input and output dtypes differ");
  RG_CHECK(in.shape == out.shape, RG_ERR_ARG, "input and output shapes differ");
  const DType dt = in.itemsize == 16 ? DType::F64 : DType::F32;
  RG_CHECK(axes != nullptr && axes->itemsize == 8, RG_ERR_ARG, "axes must be a 64-bit integer array");
  std::vector<uint64_t> ax(static_cast<size_t>(axes->nitems));
  for (size_t i = 0; i < ax.size(); ++i)
    std::memcpy(&ax[i], static_cast<const char *>(axes->data) + int64_t(i) * axes->shape_and_strides[1], 8);
  for (uint64_t a : ax) RG_CHECK(a < ndim, RG_ERR_ARG, "bad axis number");
  for (int64_t s : in.shape)
    if (s == 0) return;
  if (ax.empty()) return;
  const int din = device_memory(in.data), dout = device_memory(out.data);
  RG_CHECK(din != 0 && dout != 0, RG_ERR_UNSUPPORTED,
           "rocketgpu_c2c_noalloc takes device arrays only (host arrays need staging buffers)");
  RG_CHECK(din == 1 && dout == 1, RG_ERR_ARG,
           "rocketgpu_c2c_noalloc: the arrays live on another device than the current one");
  RG_CHECK(reinterpret_cast<uintptr_t>(in.data) % uintptr_t(in.itemsize) == 0 &&
               reinterpret_cast<uintptr_t>(out.data) % uintptr_t(out.itemsize) == 0,
           RG_ERR_UNSUPPORTED, "device data must be aligned to its item size");

  Arena ar;
  ar.dt = dt;
  std::vector<AxisPlan> plans;
  for (uint64_t a : ax) {
    AxisPlan p;
    p.axis = int(a);
    p.n = in.shape[a];
    RG_CHECK(p.n < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "transform length too large");
    int64_t rows = 1;
    for (size_t d = 0; d < in.shape.size(); ++d)
      if (d != a) rows *= in.shape[d];
    if (on_chip(p.n, dt)) {
      p.c0 = add_core(ar, int(p.n));
    } else if (rg::core_smooth(uint64_t(p.n)) && split2(dt, p.n, p.n1, p.n2)) {
      p.c0 = add_core(ar, int(p.n1));
      p.c1 = add_core(ar, int(p.n2));
      p.tw = add_split(ar, uint64_t(p.n));
      p.ws = size_t(rows) * size_t(p.n) * rg::cx_size(dt);
    } else {
      throw Error(RG_ERR_UNSUPPORTED, "rocketgpu_c2c_noalloc: length " + std::to_string(p.n) +
                                          " has a prime factor above 13 or exceeds two on-chip passes");
    }
    ar.ws_bytes = std::max(ar.ws_bytes, p.ws);
    plans.push_back(p);
  }
  const size_t need = ar.tables_bytes() + ar.ws_bytes;
  RG_CHECK(need <= kScratchBytes, RG_ERR_UNSUPPORTED,
           "rocketgpu_c2c_noalloc needs " + std::to_string(need) + " bytes of scratch; the maximum is " +
               std::to_string(kScratchBytes) + " bytes (32 MiB)");

  char *base = static_cast<char *>(scratch_address());
  ar.fill(reinterpret_cast<unsigned char *>(base), st);
  void *ws = base + ar.tables_bytes();

  for (size_t k = 0; k < plans.size(); ++k) {
    AxisPlan &p = plans[k];
    const Arr &src = k == 0 ? in : out;
    const Batch b = batch_of(src, out, p.axis);
    const double f = k == 0 ? fct : 1.0;
    if (p.ws == 0) {
      rg::FFTCore core = p.c0.core;
      core.tw = base + p.c0.off;
      launch_c2c(dt, rg::OP_C2C, core, src.data, side(src.stride[p.axis], b.shape, b.si), out.data,
                 side(out.stride[p.axis], b.shape, b.so), b.rows, !forward, !forward, f, nullptr, nullptr, 1, 0, st);
      continue;
    }
    // four-step: columns of length n1 (stride n2) with the W_n^{j2 k1} twiddle into ws, then
    // rows of length n2 from ws into the transposed output positions
    rg::FFTCore cA = p.c0.core, cB = p.c1.core;
    cA.tw = base + p.c0.off;
    cB.tw = base + p.c1.off;
    const int64_t n = p.n, n1 = p.n1, n2 = p.n2, rows = b.rows;
    const int64_t sa = src.stride[p.axis], so = out.stride[p.axis];
    const std::vector<int64_t> wshape = rows > 1 ? std::vector<int64_t>{rows} : std::vector<int64_t>{};
    const std::vector<int64_t> wstride = rows > 1 ? std::vector<int64_t>{n} : std::vector<int64_t>{};
    launch_c2c(dt, rg::OP_C2C_TW, cA, src.data, side(sa * n2, b.shape, b.si, n2, sa), ws,
               side(n2, wshape, wstride, n2, 1), rows * n2, !forward, false, 1.0, base + p.tw.lo, base + p.tw.hi,
               int(n2), p.tw.shift, st);
    launch_c2c(dt, rg::OP_C2C, cB, ws, side(1, wshape, wstride, n1, n2), out.data,
               side(so * n1, b.shape, b.so, n1, so), rows * n1, false, !forward, f, nullptr, nullptr, 1, 0, st);
  }
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int rocketgpu_c2c_noalloc(
    uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
    bool forward, double fct, uint64_t /*nthreads*/, void *stream, char *errbuf, size_t errlen) {
  std::string msg;
  try {
    run(ndim, ain, aout, axes, forward, fct, static_cast<cudaStream_t>(stream));
    t_status = RG_OK;
  } catch (const rg::Error &e) {
    t_status = e.code;
    msg = e.what();
  } catch (const std::exception &e) {
    t_status = RG_ERR_INTERNAL;
    msg = e.what();
  } catch (...) {
    t_status = RG_ERR_INTERNAL;
    msg = "unknown error";
  }
  if (errbuf && errlen > 0) {
    const size_t n = std::min(errlen - 1, msg.size());
    std::memcpy(errbuf, msg.data(), n);
    errbuf[n] = '\0';
  }
  return t_status;
}
