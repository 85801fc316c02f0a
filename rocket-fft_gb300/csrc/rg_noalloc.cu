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
//    the part it reads before reading it (tables are uploaded, the workspace is fully written
//    by the four-step first pass), so nothing needs to start at zero. Calls whose GPU work
//    overlaps (different streams, or different host threads without ordering) race on it;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress)
//    for that device; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <complex>
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

// Device address of the scratch array for the current device (looked up once per device).
void *scratch_address() {
  static std::mutex mu;
  static void *addr[64] = {};
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  RG_CHECK(dev >= 0 && dev < 64, RG_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) rg::cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
    addr[dev] = p;
  }
  return addr[dev];
}

thread_local int t_status = RG_OK;

using rg::DType;
using rg::Error;

struct Arr {
  char *data;
  int64_t itemsize;
  std::vector<int64_t> shape, stride;  // stride in elements
};

bool is_device(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
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

struct Arena {
  DType dt;
  std::vector<unsigned char> host;  // table bytes, uploaded in one copy
  size_t ws_bytes = 0;

  size_t put(const std::vector<std::complex<double>> &v) {
    size_t off = (host.size() + kAlign - 1) / kAlign * kAlign;
    const size_t es = rg::cx_size(dt);
    host.resize(off + std::max<size_t>(v.size(), 1) * es, 0);
    for (size_t i = 0; i < v.size(); ++i) {
      if (dt == DType::F64) {
        const double d[2] = {v[i].real(), v[i].imag()};
        std::memcpy(&host[off + i * 16], d, 16);
      } else {
        const float f[2] = {float(v[i].real()), float(v[i].imag())};
        std::memcpy(&host[off + i * 8], f, 8);
      }
    }
    return off;
  }
  size_t tables_bytes() const { return (host.size() + kAlign - 1) / kAlign * kAlign; }
};

std::complex<double> wfwd(uint64_t t, uint64_t N) {
  double c, s;
  rg::unit_root(t, N, c, s);
  return {c, -s};
}

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
  std::vector<std::complex<double>> tw;
  c.core.L = L;
  c.core.npass = int(rad.size());
  int Ns = 1;
  for (int p = 0; p < c.core.npass; ++p) {
    rg::PassDesc &pd = c.core.pass[p];
    pd.R = rad[p];
    pd.Ns = Ns;
    pd.LR = L / pd.R;
    pd.tw = int(tw.size());
    pd.dNs = rg::make_fastdiv(uint32_t(Ns));
    pd.dLR = rg::make_fastdiv(uint32_t(pd.LR));
    if (Ns > 1)
      for (int k = 1; k < pd.R; ++k)
        for (int m = 0; m < Ns; ++m) tw.push_back(wfwd(uint64_t(m) * k, uint64_t(Ns) * pd.R));
    Ns *= pd.R;
  }
  c.off = ar.put(tw);
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
  std::vector<std::complex<double>> lo(nlo), hi(nhi);
  for (uint64_t t = 0; t < nlo; ++t) lo[t] = wfwd(t, N);
  for (uint64_t t = 0; t < nhi; ++t) hi[t] = wfwd(t * nlo, N);
  SplitRef s{};
  s.lo = ar.put(lo);
  s.hi = ar.put(hi);
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
  RG_CHECK(is_device(in.data) && is_device(out.data), RG_ERR_UNSUPPORTED,
           "rocketgpu_c2c_noalloc takes device arrays only (host arrays need staging buffers)");
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
  if (!ar.host.empty())
    RG_CUDA(cudaMemcpyAsync(base, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice, st));
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
