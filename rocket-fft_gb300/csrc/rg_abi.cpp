// extern "C" entry points: the drop-in replacement of rocket_fft/_pocketfft_numba.cpp.
//
// Each numba_* function parses numba array structs (shapes, BYTE strides), validates them,
// stages host arrays through device memory when needed, and runs the N-d driver on the
// calling thread's stream. Errors never escape as exceptions: they become a status code and
// a thread-local message (rocketgpu_last_status / rocketgpu_last_error).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rocket_gpu.h"
#include "rg_batch.hpp"
#include "rg_error.hpp"
#include "rg_exec.hpp"
#include "rg_launch.hpp"
#include "rg_plan.hpp"

#define RG_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

thread_local int t_status = RG_OK;
thread_local std::string t_msg;
thread_local cudaStream_t t_stream = nullptr;

template <class F> int guarded(F &&f) {
  try {
    f();
    t_status = RG_OK;
    t_msg.clear();
  } catch (const rg::Error &e) {
    t_status = e.code;
    t_msg = e.what();
  } catch (const std::bad_alloc &) {
    t_status = RG_ERR_NOMEM;
    t_msg = "host allocation failed";
  } catch (const std::exception &e) {
    t_status = RG_ERR_INTERNAL;
    t_msg = e.what();
  } catch (...) {
    t_status = RG_ERR_INTERNAL;
    t_msg = "unknown error";
  }
  return t_status;
}

using rg::DType;
using rg::Error;
using rg::NdArray;

struct Desc {
  void *data;
  int64_t itemsize;
  std::vector<int64_t> shape, bstride;  // byte strides
};

Desc parse(uint64_t ndim, const rocketgpu_arystruct_t *a, const char *name) {
  RG_CHECK(a != nullptr, RG_ERR_ARG, std::string(name) + " is NULL");
  Desc d;
  d.data = a->data;
  d.itemsize = a->itemsize;
  d.shape.resize(ndim);
  d.bstride.resize(ndim);
  for (uint64_t i = 0; i < ndim; ++i) {
    d.shape[i] = a->shape_and_strides[i];
    d.bstride[i] = a->shape_and_strides[ndim + i];
    RG_CHECK(d.shape[i] >= 0, RG_ERR_ARG, std::string(name) + ": negative extent");
  }
  return d;
}

bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes at{};
  const cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Page-locked host memory (cudaHostAlloc / cudaHostRegister, e.g. torch pin_memory): copies
// from it run asynchronously on the copy engines, which the pipelines below rely on.
bool is_pinned_host(const void *p) {
  if (!p) return false;
  cudaPointerAttributes at{};
  const cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

bool any_zero(const std::vector<int64_t> &s) {
  for (int64_t v : s)
    if (v == 0) return true;
  return false;
}

std::vector<uint64_t> parse_axes(const rocketgpu_arystruct_t *ax, uint64_t ndim) {
  RG_CHECK(ax != nullptr, RG_ERR_ARG, "axes is NULL");
  RG_CHECK(ax->itemsize == 8, RG_ERR_ARG, "axes must be a 64-bit integer array");
  const int64_t n = ax->nitems;
  RG_CHECK(n >= 0, RG_ERR_ARG, "bad axes size");
  std::vector<uint64_t> axes(static_cast<size_t>(n));
  if (n == 0) return axes;
  const int64_t stride = ax->shape_and_strides[1];  // 1-D: [extent, byte stride]
  const char *base = static_cast<const char *>(ax->data);
  if (is_device_ptr(base)) {
    std::vector<char> host(size_t((n - 1) * std::llabs(stride) + 8));
    RG_CHECK(stride > 0, RG_ERR_ARG, "device axes must have a positive stride");
    RG_CUDA(cudaMemcpy(host.data(), base, host.size(), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; ++i) std::memcpy(&axes[size_t(i)], host.data() + i * stride, 8);
  } else {
    for (int64_t i = 0; i < n; ++i) std::memcpy(&axes[size_t(i)], base + i * stride, 8);
  }
  for (uint64_t a : axes) RG_CHECK(a < ndim, RG_ERR_ARG, "bad axis number");
  return axes;
}

// A device view of one argument: either the caller's device array, or a staged copy of a
// host array (copied in on construction if `copy_in`, copied back by copy_out()).
class Staged {
 public:
  Staged(const Desc &d, bool copy_in_always, cudaStream_t st) : d_(d), st_(st) {
    for (size_t i = 0; i < d.shape.size(); ++i)
      RG_CHECK(d.bstride[i] % d.itemsize == 0, RG_ERR_UNSUPPORTED,
               "strides must be multiples of the item size");
    view_.shape = d.shape;
    view_.stride.resize(d.shape.size());
    for (size_t i = 0; i < d.shape.size(); ++i) view_.stride[i] = d.bstride[i] / d.itemsize;
    if (any_zero(d.shape) || d.data == nullptr) {
      view_.data = d.data;
      return;
    }
    device_ = is_device_ptr(d.data);
    if (device_) {
      RG_CHECK(reinterpret_cast<uintptr_t>(d.data) % uintptr_t(d.itemsize) == 0, RG_ERR_UNSUPPORTED,
               "device data must be aligned to its item size");
      view_.data = d.data;
      return;
    }
    int64_t lo = 0, hi = 0, count = 1;
    for (size_t i = 0; i < d.shape.size(); ++i) {
      const int64_t ext = (d.shape[i] - 1) * d.bstride[i];
      if (ext < 0) lo += ext; else hi += ext;
      count *= d.shape[i];
    }
    span_lo_ = lo;
    span_ = size_t(hi - lo + d.itemsize);
    buf_.reset(new rg::DevBuf(span_, st));
    view_.data = static_cast<char *>(buf_->get()) - lo;
    const bool dense = span_ == size_t(count * d.itemsize);
    if (copy_in_always || !dense)
      RG_CUDA(cudaMemcpyAsync(buf_->get(), static_cast<char *>(d.data) + lo, span_,
                              cudaMemcpyHostToDevice, st));
  }
  void copy_out() {
    if (!buf_) return;
    RG_CUDA(cudaMemcpyAsync(static_cast<char *>(d_.data) + span_lo_, buf_->get(), span_,
                            cudaMemcpyDeviceToHost, st_));
  }
  bool staged() const { return bool(buf_); }
  const NdArray &view() const { return view_; }
  // share another staged view's device memory when both describe the same host array
  void alias(const Staged &o) {
    view_.data = o.view_.data;
    buf_.reset();
  }

 private:
  Desc d_;
  cudaStream_t st_;
  NdArray view_;
  bool device_ = false;
  int64_t span_lo_ = 0;
  size_t span_ = 0;
  std::unique_ptr<rg::DevBuf> buf_;
};

// Runs body(in_view, out_view) with host arrays staged, then copies results back.
template <class Body>
void with_views(const Desc &din, const Desc &dout, Body body) {
  cudaStream_t st = t_stream;
  Staged sin(din, true, st);
  const bool inplace = din.data == dout.data && din.bstride == dout.bstride &&
                       din.itemsize == dout.itemsize && sin.staged();
  Staged sout(dout, false, st);
  if (inplace) sout.alias(sin);
  body(sin.view(), sout.view(), st);
  if (sin.staged() || sout.staged()) {
    if (inplace)
      sin.copy_out();
    else
      sout.copy_out();
    RG_CUDA(cudaStreamSynchronize(st));
  }
}

// ---- host arrays, r2c / c2r over three or more axes: copies overlapped with the passes ----
//
// A host call stages its arrays through the GPU, so it is bound by the host link. For r2c the
// passes over every axis but the outermost only need the planes they work on: the input goes in
// as slabs of planes on a copy stream, and each slab is transformed as soon as it has arrived;
// then the outermost axis runs over the whole array and the result goes out. For c2r the
// outermost axis runs first (in place on the staging copy), then each slab of planes takes the
// remaining passes and goes out on the copy stream while the next slab is transformed. Dense
// C-order arrays only, the outermost axis transformed first (axes[0] == 0, three or more axes).

// Side streams of the current device: 0 = host-to-device copies, 1 = device-to-host copies,
// 2 and 3 = compute of the batch slabs below.
enum SideStream { kCopyIn = 0, kCopyOut = 1, kCompute0 = 2, kSideStreams = 4 };
cudaStream_t side_stream(int which) {
  static std::mutex mu;
  static cudaStream_t streams[64][kSideStreams] = {};
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  RG_CHECK(dev >= 0 && dev < 64, RG_ERR_UNSUPPORTED, "device index above 63");
  std::lock_guard<std::mutex> lk(mu);
  cudaStream_t &s = streams[dev][which];
  if (!s) RG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  return s;
}

// Slab count limit of the host-array pipelines: ROCKET_GPU_SLABS (0 = whole-array staging
// always), default 4.
int64_t max_slabs() {
  static const int64_t k = [] {
    const char *e = std::getenv("ROCKET_GPU_SLABS");
    return e ? std::max<int64_t>(0, std::atoll(e)) : int64_t(4);
  }();
  return k;
}

bool dense_c(const Desc &d) {
  int64_t acc = d.itemsize;
  for (int i = int(d.shape.size()) - 1; i >= 0; --i) {
    if (d.shape[i] != 1 && d.bstride[i] != acc) return false;
    acc *= d.shape[i];
  }
  return true;
}

NdArray dense_view(void *data, std::vector<int64_t> shape) {
  NdArray v;
  v.data = data;
  v.shape = std::move(shape);
  v.stride.assign(v.shape.size(), 1);
  for (int i = int(v.shape.size()) - 2; i >= 0; --i) v.stride[i] = v.stride[i + 1] * v.shape[i + 1];
  return v;
}

bool pipeline_ok(const Desc &din, const Desc &dout, const std::vector<uint64_t> &ax) {
  if (max_slabs() == 0) return false;
  if (ax.size() < 3 || ax[0] != 0 || din.shape.empty() || din.shape[0] < 2) return false;
  for (size_t i = 1; i < ax.size(); ++i)
    if (ax[i] == 0) return false;
  if (!dense_c(din) || !dense_c(dout) || !din.data || !dout.data) return false;
  // page-locked only: with pageable arrays the slab copies were slower than whole-array
  // staging (256^3 float32 r2c 892 vs 847 us, c2r 952 vs 847 us)
  return is_pinned_host(din.data) && is_pinned_host(dout.data);
}

// Events for the pipelines, created once per thread and device and reused by every call.
class EventCache {
 public:
  cudaEvent_t get(size_t i) {
    int dev = 0;
    RG_CUDA(cudaGetDevice(&dev));
    std::vector<cudaEvent_t> &v = per_dev_[dev & 63];
    while (v.size() <= i) {
      cudaEvent_t e;
      RG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      v.push_back(e);
    }
    return v[i];
  }

 private:
  std::vector<cudaEvent_t> per_dev_[64];
};
thread_local EventCache t_events;

// Makes `st` wait for everything enqueued on the side streams when an error unwinds the call,
// so that the staging buffers (freed in st's order) outlive the work that uses them. A call
// that completes joins through its last device-to-host copy instead (dismiss()).
struct JoinSides {
  cudaStream_t st;
  std::vector<cudaStream_t> sides;
  bool active = true;
  void dismiss() { active = false; }
  ~JoinSides() {
    if (!active) return;
    for (cudaStream_t s : sides) {
      cudaEvent_t e;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) continue;
      if (cudaEventRecord(e, s) == cudaSuccess) cudaStreamWaitEvent(st, e, 0);
      cudaEventDestroy(e);
    }
  }
};

// View of columns [j0, j0 + nj) of dimension 1 of a dense C-order array (all other dims whole).
NdArray column_chunk(void *base, const std::vector<int64_t> &shape, int64_t itemsize, int64_t j0, int64_t nj) {
  NdArray v = dense_view(base, shape);
  v.data = static_cast<char *>(base) + j0 * v.stride[1] * itemsize;
  v.shape[1] = nj;
  return v;
}

// Slab and column-chunk counts of the three-axis pipelines.
int64_t slab_count(int64_t n0) { return std::max<int64_t>(1, std::min<int64_t>(2 * max_slabs(), n0)); }
int64_t chunk_count(int64_t n1) { return std::max<int64_t>(1, std::min<int64_t>(max_slabs(), n1)); }

// r2c (forward, fct) of host din into host dout, pipelined as described above: slabs of planes
// in (copy-in stream) and through the passes over every axis but the outermost; then the
// outermost axis in column chunks along dimension 1, each chunk copied out (a 2-D copy on the
// copy-out stream) while the next one is transformed.
void pipelined_r2c(DType dt, const Desc &din, const Desc &dout, const std::vector<uint64_t> &ax, bool forward,
                   double fct) {
  cudaStream_t st = t_stream, cin = side_stream(kCopyIn), cout = side_stream(kCopyOut);
  const int64_t n0 = din.shape[0], n1 = dout.shape[1];
  const int64_t plane_in = din.bstride[0], plane_out = dout.bstride[0];
  rg::DevBuf bin(size_t(n0 * plane_in), st), bout(size_t(n0 * plane_out), st);
  JoinSides join{st, {cin, cout}};
  size_t ne = 0;
  cudaEvent_t ready = t_events.get(ne++);
  RG_CUDA(cudaEventRecord(ready, st));  // the buffers exist in st's order
  RG_CUDA(cudaStreamWaitEvent(cin, ready, 0));
  const int64_t K = slab_count(n0), per = (n0 + K - 1) / K;
  const rg::Axes rest(ax.begin() + 1, ax.end());
  for (int64_t c0 = 0; c0 < n0; c0 += per) {
    const int64_t cn = std::min(per, n0 - c0);
    RG_CUDA(cudaMemcpyAsync(static_cast<char *>(bin.get()) + c0 * plane_in,
                            static_cast<const char *>(din.data) + c0 * plane_in, size_t(cn * plane_in),
                            cudaMemcpyHostToDevice, cin));
    cudaEvent_t arrived = t_events.get(ne++);
    RG_CUDA(cudaEventRecord(arrived, cin));
    RG_CUDA(cudaStreamWaitEvent(st, arrived, 0));
    std::vector<int64_t> si = din.shape, so = dout.shape;
    si[0] = so[0] = cn;
    rg::exec_r2c(dt, dense_view(static_cast<char *>(bin.get()) + c0 * plane_in, si),
                 dense_view(static_cast<char *>(bout.get()) + c0 * plane_out, so), rest, forward, fct, st);
  }
  const int64_t KC = chunk_count(n1), cper = (n1 + KC - 1) / KC;
  const int64_t row = plane_out / n1;  // bytes of one index of dimension 1
  for (int64_t j0 = 0; j0 < n1; j0 += cper) {
    const int64_t nj = std::min(cper, n1 - j0);
    const NdArray v = column_chunk(bout.get(), dout.shape, dout.itemsize, j0, nj);
    rg::exec_c2c(dt, v, v, rg::Axes{0}, forward, 1.0, st);
    cudaEvent_t done = t_events.get(ne++);
    RG_CUDA(cudaEventRecord(done, st));
    RG_CUDA(cudaStreamWaitEvent(cout, done, 0));
    RG_CUDA(cudaMemcpy2DAsync(static_cast<char *>(dout.data) + j0 * row, size_t(plane_out),
                              static_cast<char *>(bout.get()) + j0 * row, size_t(plane_out), size_t(nj * row),
                              size_t(n0), cudaMemcpyDeviceToHost, cout));
  }
  cudaEvent_t fin = t_events.get(ne++);
  RG_CUDA(cudaEventRecord(fin, cout));
  RG_CUDA(cudaStreamWaitEvent(st, fin, 0));
  join.dismiss();
  RG_CUDA(cudaEventSynchronize(fin));
}

// c2r (forward, fct) of host din into host dout, pipelined as described above: the input in
// column chunks along dimension 1 (2-D copies on the copy-in stream), each chunk through the
// outermost axis as soon as it has arrived (in place on the staging copy); then slabs of planes
// through the remaining passes, each copied out while the next is transformed.
void pipelined_c2r(DType dt, const Desc &din, const Desc &dout, const std::vector<uint64_t> &ax, bool forward,
                   double fct) {
  cudaStream_t st = t_stream, cin = side_stream(kCopyIn), cout = side_stream(kCopyOut);
  const int64_t n0 = dout.shape[0], n1 = din.shape[1];
  const int64_t plane_in = din.bstride[0], plane_out = dout.bstride[0];
  rg::DevBuf bin(size_t(n0 * plane_in), st), bout(size_t(n0 * plane_out), st);
  JoinSides join{st, {cin, cout}};
  size_t ne = 0;
  cudaEvent_t ready = t_events.get(ne++);
  RG_CUDA(cudaEventRecord(ready, st));
  RG_CUDA(cudaStreamWaitEvent(cin, ready, 0));
  const int64_t KC = chunk_count(n1), cper = (n1 + KC - 1) / KC;
  const int64_t row = plane_in / n1;
  for (int64_t j0 = 0; j0 < n1; j0 += cper) {
    const int64_t nj = std::min(cper, n1 - j0);
    RG_CUDA(cudaMemcpy2DAsync(static_cast<char *>(bin.get()) + j0 * row, size_t(plane_in),
                              static_cast<const char *>(din.data) + j0 * row, size_t(plane_in), size_t(nj * row),
                              size_t(n0), cudaMemcpyHostToDevice, cin));
    cudaEvent_t arrived = t_events.get(ne++);
    RG_CUDA(cudaEventRecord(arrived, cin));
    RG_CUDA(cudaStreamWaitEvent(st, arrived, 0));
    const NdArray v = column_chunk(bin.get(), din.shape, din.itemsize, j0, nj);
    rg::exec_c2c(dt, v, v, rg::Axes{0}, forward, 1.0, st);  // in place on the staging copy
  }
  const int64_t K = slab_count(n0), per = (n0 + K - 1) / K;
  const rg::Axes rest(ax.begin() + 1, ax.end());
  for (int64_t c0 = 0; c0 < n0; c0 += per) {
    const int64_t cn = std::min(per, n0 - c0);
    std::vector<int64_t> si = din.shape, so = dout.shape;
    si[0] = so[0] = cn;
    rg::exec_c2r(dt, dense_view(static_cast<char *>(bin.get()) + c0 * plane_in, si),
                 dense_view(static_cast<char *>(bout.get()) + c0 * plane_out, so), rest, forward, fct, st);
    cudaEvent_t done = t_events.get(ne++);
    RG_CUDA(cudaEventRecord(done, st));
    RG_CUDA(cudaStreamWaitEvent(cout, done, 0));
    RG_CUDA(cudaMemcpyAsync(static_cast<char *>(dout.data) + c0 * plane_out,
                            static_cast<char *>(bout.get()) + c0 * plane_out, size_t(cn * plane_out),
                            cudaMemcpyDeviceToHost, cout));
  }
  cudaEvent_t fin = t_events.get(ne++);
  RG_CUDA(cudaEventRecord(fin, cout));
  RG_CUDA(cudaStreamWaitEvent(st, fin, 0));
  join.dismiss();
  RG_CUDA(cudaEventSynchronize(fin));
}

// ---- host arrays with a batch dimension: copy-in, compute and copy-out overlapped ----
//
// When the outermost dimension is not transformed, its slabs are independent transforms. A
// host call then runs as a three-stage pipeline: slab i is copied in on the copy-in stream,
// transformed on one of two compute streams as soon as it has arrived, and copied out on the
// copy-out stream, while slab i+1 is copied in and slab i-1 copied out; the two link
// directions run at once. Dense C-order host arrays only (every slab is one contiguous range
// of both arrays), and only when the copies are large enough to matter.

bool slabs_ok(const Desc &din, const Desc &dout, const std::vector<uint64_t> &ax) {
  if (din.shape.empty() || din.shape[0] < 2 || dout.shape.empty() || dout.shape[0] != din.shape[0]) return false;
  for (uint64_t a : ax)
    if (a == 0) return false;
  if (!din.data || !dout.data || !dense_c(din) || !dense_c(dout)) return false;
  const int64_t bytes = din.shape[0] * din.bstride[0] + dout.shape[0] * dout.bstride[0];
  if (bytes < (int64_t(2) << 20)) return false;
  // pageable memory is copied through the driver's staging buffers, synchronously with the
  // host: smaller copies only add overhead there (measured 310 us whole vs 499 us in 4 slabs
  // for 256 x 4096 complex128)
  return is_pinned_host(din.data) && is_pinned_host(dout.data);
}

template <class Body>
void pipelined_slabs(const Desc &din, const Desc &dout, Body body) {
  cudaStream_t st = t_stream, cin = side_stream(kCopyIn), cout = side_stream(kCopyOut);
  cudaStream_t comp[2] = {side_stream(kCompute0), side_stream(kCompute0 + 1)};
  const int64_t n0 = din.shape[0];
  const int64_t plane_in = din.bstride[0], plane_out = dout.bstride[0];
  const bool inplace = din.data == dout.data && plane_in == plane_out && din.itemsize == dout.itemsize;
  rg::DevBuf bin(size_t(n0 * plane_in), st);
  std::unique_ptr<rg::DevBuf> bout_own;
  if (!inplace) bout_own.reset(new rg::DevBuf(size_t(n0 * plane_out), st));
  char *dev_in = static_cast<char *>(bin.get());
  char *dev_out = inplace ? dev_in : static_cast<char *>(bout_own->get());
  JoinSides join{st, {cin, cout, comp[0], comp[1]}};
  // ordering: st (buffers exist) -> copy-in of slab i -> compute of slab i -> copy-out of slab
  // i -> st (buffers are freed); every side stream's work hangs off this chain
  size_t ne = 0;
  cudaEvent_t ready = t_events.get(ne++);
  RG_CUDA(cudaEventRecord(ready, st));
  RG_CUDA(cudaStreamWaitEvent(cin, ready, 0));
  // about 4 MiB of input per slab, 2..max_slabs() slabs
  const int64_t want = std::min<int64_t>(max_slabs(), std::max<int64_t>(2, n0 * plane_in / (int64_t(4) << 20)));
  const int64_t K = std::min(want, n0), per = (n0 + K - 1) / K;
  int slab = 0;
  for (int64_t c0 = 0; c0 < n0; c0 += per, ++slab) {
    const int64_t cn = std::min(per, n0 - c0);
    RG_CUDA(cudaMemcpyAsync(dev_in + c0 * plane_in, static_cast<const char *>(din.data) + c0 * plane_in,
                            size_t(cn * plane_in), cudaMemcpyHostToDevice, cin));
    cudaEvent_t arrived = t_events.get(ne++);
    RG_CUDA(cudaEventRecord(arrived, cin));
    cudaStream_t cs = comp[slab % 2];
    RG_CUDA(cudaStreamWaitEvent(cs, arrived, 0));
    std::vector<int64_t> si = din.shape, so = dout.shape;
    si[0] = so[0] = cn;
    body(dense_view(dev_in + c0 * plane_in, si), dense_view(dev_out + c0 * plane_out, so), cs);
    cudaEvent_t done = t_events.get(ne++);
    RG_CUDA(cudaEventRecord(done, cs));
    RG_CUDA(cudaStreamWaitEvent(cout, done, 0));
    RG_CUDA(cudaMemcpyAsync(static_cast<char *>(dout.data) + c0 * plane_out, dev_out + c0 * plane_out,
                            size_t(cn * plane_out), cudaMemcpyDeviceToHost, cout));
  }
  cudaEvent_t fin = t_events.get(ne++);
  RG_CUDA(cudaEventRecord(fin, cout));
  RG_CUDA(cudaStreamWaitEvent(st, fin, 0));
  join.dismiss();
  RG_CUDA(cudaEventSynchronize(fin));
}

// Runs body(in_view, out_view, stream) on device views of the arguments: the batch-slab
// pipeline for large host arrays with an untransformed outer dimension, else whole arrays
// staged (or used in place when they are device arrays).
template <class Body>
void run_views(const Desc &din, const Desc &dout, const std::vector<uint64_t> &ax, Body body) {
  if (max_slabs() >= 2 && slabs_ok(din, dout, ax))
    pipelined_slabs(din, dout, body);
  else
    with_views(din, dout, body);
}

void check_same_shape(const Desc &a, const Desc &b) {
  RG_CHECK(a.shape == b.shape, RG_ERR_ARG, "input and output shapes differ");
}

void check_half_shape(const Desc &full, const Desc &half, const std::vector<uint64_t> &axes) {
  RG_CHECK(full.shape.size() == half.shape.size(), RG_ERR_ARG, "rank mismatch");
  const uint64_t last = axes.back();
  for (size_t i = 0; i < full.shape.size(); ++i) {
    const int64_t want = i == last ? full.shape[i] / 2 + 1 : full.shape[i];
    RG_CHECK(half.shape[i] == want, RG_ERR_ARG,
             "half-spectrum shape must equal the real shape with the last axis n/2+1");
  }
}

DType complex_dtype(int64_t itemsize) {
  RG_CHECK(itemsize == 8 || itemsize == 16, RG_ERR_ARG, "complex arrays must be complex64 or complex128");
  return itemsize == 16 ? DType::F64 : DType::F32;
}
DType real_dtype(int64_t itemsize) {
  RG_CHECK(itemsize == 4 || itemsize == 8, RG_ERR_ARG, "real arrays must be float32 or float64");
  return itemsize == 8 ? DType::F64 : DType::F32;
}

int do_c2c(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
           rocketgpu_arystruct_t *axes, bool forward, double fct) {
  return guarded([&] {
    const Desc din = parse(ndim, ain, "ain"), dout = parse(ndim, aout, "aout");
    const DType dt = complex_dtype(din.itemsize);
    RG_CHECK(dout.itemsize == din.itemsize, RG_ERR_ARG, "input and output dtypes differ");
    check_same_shape(din, dout);
    const auto ax = parse_axes(axes, ndim);
    if (any_zero(din.shape) || ax.empty()) return;
    run_views(din, dout, ax, [&](const NdArray &i, const NdArray &o, cudaStream_t st) {
      rg::exec_c2c(dt, i, o, ax, forward, fct, st);
    });
  });
}

int do_r2c(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
           rocketgpu_arystruct_t *axes, bool forward, double fct, bool sym, double bscale = 1.0) {
  return guarded([&] {
    const Desc din = parse(ndim, ain, "ain"), dout = parse(ndim, aout, "aout");
    const DType dt = real_dtype(din.itemsize);
    RG_CHECK(dout.itemsize == 2 * din.itemsize, RG_ERR_ARG, "output must be the matching complex dtype");
    const auto ax = parse_axes(axes, ndim);
    RG_CHECK(!ax.empty(), RG_ERR_ARG, "at least one axis is required");
    if (sym)
      check_same_shape(din, dout);
    else
      check_half_shape(din, dout, ax);
    if (any_zero(din.shape)) return;
    if (!sym && bscale == 1.0 && pipeline_ok(din, dout, ax)) {
      pipelined_r2c(dt, din, dout, ax, forward, fct);
      return;
    }
    run_views(din, dout, ax, [&](const NdArray &i, const NdArray &o, cudaStream_t st) {
      if (sym)
        rg::exec_c2c_sym(dt, i, o, ax, forward, fct, st);
      else
        rg::exec_r2c(dt, i, o, ax, forward, fct, st, bscale);
    });
  });
}

int do_c2r(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
           rocketgpu_arystruct_t *axes, bool forward, double fct, double bscale = 1.0) {
  return guarded([&] {
    const Desc din = parse(ndim, ain, "ain"), dout = parse(ndim, aout, "aout");
    const DType dt = complex_dtype(din.itemsize);
    RG_CHECK(2 * dout.itemsize == din.itemsize, RG_ERR_ARG, "output must be the matching real dtype");
    const auto ax = parse_axes(axes, ndim);
    RG_CHECK(!ax.empty(), RG_ERR_ARG, "at least one axis is required");
    check_half_shape(dout, din, ax);
    if (any_zero(dout.shape)) return;
    if (bscale == 1.0 && pipeline_ok(din, dout, ax)) {
      pipelined_c2r(dt, din, dout, ax, forward, fct);
      return;
    }
    run_views(din, dout, ax, [&](const NdArray &i, const NdArray &o, cudaStream_t st) {
      rg::exec_c2r(dt, i, o, ax, forward, fct, st, bscale);
    });
  });
}

// Real in, real out, same shape and dtype (dct/dst/r2r_fftpack/Hartley).
template <class Body> int do_real(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                                  rocketgpu_arystruct_t *axes, Body body) {
  return guarded([&] {
    const Desc din = parse(ndim, ain, "ain"), dout = parse(ndim, aout, "aout");
    const DType dt = real_dtype(din.itemsize);
    RG_CHECK(dout.itemsize == din.itemsize, RG_ERR_ARG, "input and output dtypes differ");
    check_same_shape(din, dout);
    const auto ax = parse_axes(axes, ndim);
    if (any_zero(din.shape) || ax.empty()) return;
    run_views(din, dout, ax, [&](const NdArray &i, const NdArray &o, cudaStream_t st) { body(dt, i, o, ax, st); });
  });
}

int do_dcst(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
            rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho, bool cosine,
            bool adjoint = false) {
  if (type < 1 || type > 4)  // checked before anything else, as the reference (HDR:3896-3897, 3919-3920)
    return guarded([&] { throw Error(RG_ERR_ARG, cosine ? "invalid DCT type" : "invalid DST type"); });
  return do_real(ndim, ain, aout, axes, [&](DType dt, const NdArray &i, const NdArray &o, const rg::Axes &ax,
                                            cudaStream_t st) {
    rg::exec_dcst(dt, i, o, ax, int(type), cosine, fct, ortho, st, adjoint);
  });
}

}  // namespace

// ---------------------------------------------------------------------------------------
// drop-in entry points
// ---------------------------------------------------------------------------------------

RG_EXPORT uint64_t numba_good_size(uint64_t target, bool real) {
  uint64_t r = 0;
  guarded([&] { r = real ? rg::good_size_real(target) : rg::good_size_cmplx(target); });
  return r;
}

RG_EXPORT int numba_c2c_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                           rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t) {
  return do_c2c(ndim, ain, aout, axes, forward, fct);
}
RG_EXPORT void numba_c2c(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                         rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads) {
  numba_c2c_st(ndim, ain, aout, axes, forward, fct, nthreads);
}

RG_EXPORT int numba_r2c_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                           rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t) {
  return do_r2c(ndim, ain, aout, axes, forward, fct, false);
}
RG_EXPORT void numba_r2c(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                         rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads) {
  numba_r2c_st(ndim, ain, aout, axes, forward, fct, nthreads);
}

RG_EXPORT int numba_c2c_sym_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                               rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes, bool forward,
                               double fct, uint64_t) {
  return do_r2c(ndim, ain, aout, axes, forward, fct, true);
}
RG_EXPORT void numba_c2c_sym(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                             rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads) {
  numba_c2c_sym_st(ndim, ain, aout, axes, forward, fct, nthreads);
}

RG_EXPORT int numba_c2r_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                           rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t) {
  return do_c2r(ndim, ain, aout, axes, forward, fct);
}
RG_EXPORT void numba_c2r(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                         rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads) {
  numba_c2r_st(ndim, ain, aout, axes, forward, fct, nthreads);
}

RG_EXPORT int numba_dct_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                           rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho, uint64_t) {
  return do_dcst(ndim, ain, aout, axes, type, fct, ortho, true);
}
RG_EXPORT void numba_dct(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                         rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho,
                         uint64_t nthreads) {
  numba_dct_st(ndim, ain, aout, axes, type, fct, ortho, nthreads);
}
RG_EXPORT int numba_dst_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                           rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho, uint64_t) {
  return do_dcst(ndim, ain, aout, axes, type, fct, ortho, false);
}
RG_EXPORT void numba_dst(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                         rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho,
                         uint64_t nthreads) {
  numba_dst_st(ndim, ain, aout, axes, type, fct, ortho, nthreads);
}
RG_EXPORT int numba_r2r_fftpack_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                                   rocketgpu_arystruct_t *axes, bool real2hermitian, bool forward, double fct,
                                   uint64_t) {
  return do_real(ndim, ain, aout, axes, [&](DType dt, const NdArray &i, const NdArray &o, const rg::Axes &ax,
                                            cudaStream_t st) {
    rg::exec_r2r_fftpack(dt, i, o, ax, real2hermitian, forward, fct, st);
  });
}
RG_EXPORT void numba_r2r_fftpack(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                 rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                                 bool real2hermitian, bool forward, double fct, uint64_t nthreads) {
  numba_r2r_fftpack_st(ndim, ain, aout, axes, real2hermitian, forward, fct, nthreads);
}
RG_EXPORT int numba_r2r_separable_hartley_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                             rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes, double fct,
                                             uint64_t) {
  return do_real(ndim, ain, aout, axes, [&](DType dt, const NdArray &i, const NdArray &o, const rg::Axes &ax,
                                            cudaStream_t st) { rg::exec_hartley(dt, i, o, ax, false, fct, st); });
}
RG_EXPORT void numba_r2r_separable_hartley(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                           rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                                           double fct, uint64_t nthreads) {
  numba_r2r_separable_hartley_st(ndim, ain, aout, axes, fct, nthreads);
}
RG_EXPORT int numba_r2r_genuine_hartley_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                           rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes, double fct,
                                           uint64_t) {
  return do_real(ndim, ain, aout, axes, [&](DType dt, const NdArray &i, const NdArray &o, const rg::Axes &ax,
                                            cudaStream_t st) { rg::exec_hartley(dt, i, o, ax, true, fct, st); });
}
RG_EXPORT void numba_r2r_genuine_hartley(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                         rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                                         double fct, uint64_t nthreads) {
  numba_r2r_genuine_hartley_st(ndim, ain, aout, axes, fct, nthreads);
}

// ---------------------------------------------------------------------------------------
// adjoints (no reference counterpart; used by the torch.autograd wrappers)
// ---------------------------------------------------------------------------------------

// Adjoint of numba_r2c(., forward, fct): c2r in the opposite direction with the interior bins
// of the last axis halved. ain is the half spectrum (cotangent), aout the real gradient.
RG_EXPORT int rocketgpu_r2c_adjoint_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                       rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes, bool forward,
                                       double fct, uint64_t) {
  return do_c2r(ndim, ain, aout, axes, !forward, fct, 0.5);
}

// Adjoint of numba_c2r(., forward, fct): r2c in the opposite direction with the interior bins
// of the last axis doubled. ain is the real cotangent, aout the half-spectrum gradient.
RG_EXPORT int rocketgpu_c2r_adjoint_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                       rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes, bool forward,
                                       double fct, uint64_t) {
  return do_r2c(ndim, ain, aout, axes, !forward, fct, false, 2.0);
}

// Adjoint (transpose) of numba_dct(., type, fct, ortho).
RG_EXPORT int rocketgpu_dct_adjoint_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                       rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes, uint64_t type,
                                       double fct, bool ortho, uint64_t) {
  return do_dcst(ndim, ain, aout, axes, type, fct, ortho, true, true);
}

// ---------------------------------------------------------------------------------------
// batched uneven lengths (no reference counterpart)
// ---------------------------------------------------------------------------------------

RG_EXPORT void *rocketgpu_batch_create(const int64_t *lengths, int64_t count, int64_t itemsize, bool forward,
                                       double fct, int autotune) {
  rg::BatchPlan *p = nullptr;
  guarded([&] {
    RG_CHECK(lengths != nullptr, RG_ERR_ARG, "lengths is NULL");
    const DType dt = complex_dtype(itemsize);
    p = rg::batch_create(lengths, count, dt, forward, fct, autotune != 0);
  });
  return p;
}

RG_EXPORT int rocketgpu_batch_exec(void *plan, const void *in, void *out, void *stream) {
  return guarded([&] {
    RG_CHECK(plan != nullptr, RG_ERR_ARG, "plan is NULL");
    RG_CHECK(is_device_ptr(in) && is_device_ptr(out), RG_ERR_UNSUPPORTED, "batch buffers must be device memory");
    rg::batch_exec(*static_cast<rg::BatchPlan *>(plan), in, out, static_cast<cudaStream_t>(stream));
  });
}

RG_EXPORT int rocketgpu_batch_info(void *plan, char *buf, size_t len) {
  std::string info;
  const int st = guarded([&] {
    RG_CHECK(plan != nullptr, RG_ERR_ARG, "plan is NULL");
    info = rg::batch_info(*static_cast<rg::BatchPlan *>(plan));
  });
  if (buf && len > 0) {
    const size_t n = std::min(len - 1, info.size());
    std::memcpy(buf, info.data(), n);
    buf[n] = '\0';
  }
  return st;
}

RG_EXPORT void rocketgpu_batch_destroy(void *plan) {
  guarded([&] { rg::batch_destroy(static_cast<rg::BatchPlan *>(plan)); });
}

// ---------------------------------------------------------------------------------------
// runtime control
// ---------------------------------------------------------------------------------------

RG_EXPORT int rocketgpu_last_status(void) { return t_status; }

RG_EXPORT int rocketgpu_last_error(char *buf, size_t len) {
  if (buf && len > 0) {
    const size_t n = std::min(len - 1, t_msg.size());
    std::memcpy(buf, t_msg.data(), n);
    buf[n] = '\0';
  }
  return t_status;
}

RG_EXPORT void rocketgpu_set_stream(void *stream) { t_stream = static_cast<cudaStream_t>(stream); }
RG_EXPORT void *rocketgpu_get_stream(void) { return t_stream; }

RG_EXPORT uint64_t rocketgpu_plan_cache_entries(void) { return rg::cache_entries(); }
RG_EXPORT uint64_t rocketgpu_plan_cache_bytes(void) { return rg::cache_bytes(); }
RG_EXPORT int rocketgpu_plan_cache_clear(void) {
  return guarded([] {
    rg::cache_clear();
    rg::pool_trim();
  });
}

RG_EXPORT uint64_t rocketgpu_launch_count(void) { return rg::launch_count(); }

RG_EXPORT int rocketgpu_set_tc_split(int on) { return rg::set_tc_split(on != 0); }

RG_EXPORT int rocketgpu_set_plane_kernels(int on) { return rg::set_plane_kernels(on != 0); }

RG_EXPORT int rocketgpu_roll(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                             const int64_t *shifts) {
  return guarded([&] {
    const Desc din = parse(ndim, ain, "ain"), dout = parse(ndim, aout, "aout");
    RG_CHECK(din.itemsize == dout.itemsize, RG_ERR_ARG, "input and output dtypes differ");
    check_same_shape(din, dout);
    RG_CHECK(shifts != nullptr || ndim == 0, RG_ERR_ARG, "shifts is NULL");
    if (any_zero(din.shape)) return;
    const std::vector<int64_t> sh(shifts, shifts + ndim);
    with_views(din, dout, [&](const NdArray &i, const NdArray &o, cudaStream_t st) {
      rg::roll(i, o, din.itemsize, sh, st);
    });
  });
}

RG_EXPORT int rocketgpu_tc_error(void *stream) {
  int flag = 0;
  const int st = guarded([&] { flag = rg::tc_error_flag(static_cast<cudaStream_t>(stream)); });
  return st == RG_OK ? flag : -st;
}

RG_EXPORT int rocketgpu_fp64_peak(double *gflops, void *stream) {
  return guarded([&] {
    RG_CHECK(gflops != nullptr, RG_ERR_ARG, "gflops is NULL");
    *gflops = rg::fp64_peak_gflops(static_cast<cudaStream_t>(stream));
  });
}

RG_EXPORT int rocketgpu_long_error(void *stream) {
  int flag = 0;
  const int st = guarded([&] { flag = rg::long_error_flag(static_cast<cudaStream_t>(stream)); });
  return st == RG_OK ? flag : -st;
}

RG_EXPORT int rocketgpu_tc_selftest(const void *A, const void *A2, const void *B, const void *B2, float *D,
                                    void *stream) {
  return guarded([&] {
    RG_CHECK(A && A2 && B && B2 && D, RG_ERR_ARG, "null operand");
    rg::tc_selftest(A, A2, B, B2, D, static_cast<cudaStream_t>(stream));
  });
}

RG_EXPORT void rocketgpu_profile_enable(int on) { rg::profile_enable(on != 0); }

RG_EXPORT int rocketgpu_profile_read(rocketgpu_kstat_t *out, int max) {
  int n = 0;
  guarded([&] {
    const auto stats = rg::profile_read();
    for (const auto &k : stats) {
      if (n >= max) break;
      std::memcpy(out[n].name, k.name, sizeof(out[n].name));
      out[n].launches = k.launches;
      out[n].total_ms = k.total_ms;
      out[n].bytes = k.bytes;
      ++n;
    }
  });
  return n;
}

RG_EXPORT void rocketgpu_profile_reset(void) {
  guarded([] { rg::profile_reset(); });
}

RG_EXPORT const char *rocketgpu_version(void) { return "rocket-fft_gb300 0.1.0 (sm_103a)"; }
