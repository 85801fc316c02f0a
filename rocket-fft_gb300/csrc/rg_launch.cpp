// Precision dispatch and launch bookkeeping.
#include "rg_launch.hpp"

#include <atomic>
#include <cstdlib>
#include <functional>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rg_error.hpp"

namespace rg {

void launch_axis_f32(int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st);
bool launch_fixed_f32(int op, const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st);
bool launch_fixed_f64(int op, const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st);
void launch_axis_f64(int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st);
void launch_pw_f32(int op, const PwArgs &a, cudaStream_t st);
void launch_pw_f64(int op, const PwArgs &a, cudaStream_t st);
void launch_mirror_f32(const MirrorArgs &a, cudaStream_t st);
void launch_mirror_f64(const MirrorArgs &a, cudaStream_t st);

static std::atomic<uint64_t> g_launches{0};
static std::atomic<int> g_tc{0};

// Programmatic dependent launch of the chained kernels (rg_pdl.cuh); ROCKET_GPU_PDL=0 turns it off.
bool pdl_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("ROCKET_GPU_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

bool tc_split_enabled() { return g_tc.load(std::memory_order_relaxed) != 0; }
int set_tc_split(bool on) { return g_tc.exchange(on ? 1 : 0); }

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------------------------------
// event-based per-kernel profile: when enabled, every launch is bracketed by two CUDA events
// on its own stream and its algorithmic bytes (one read of its input rows plus one write of
// its output rows) are recorded; profile_read() synchronises and aggregates per kernel name.
// ---------------------------------------------------------------------------------------

namespace {
struct ProfRec {
  std::string name;
  uint64_t bytes;
  cudaEvent_t a, b;
};
std::atomic<bool> g_prof{false};
std::mutex g_pmu;
std::vector<ProfRec> g_pending;
std::map<std::string, KernelStat> g_agg;

const char *axis_name(int op) {
  switch (op) {
    case OP_C2C: return "axis_c2c";
    case OP_C2C_TW: return "axis_c2c_twiddle";
    case OP_R2C_EVEN: return "axis_r2c_even";
    case OP_R2C_ODD: return "axis_r2c_odd";
    case OP_C2R_EVEN: return "axis_c2r_even";
    case OP_C2R_ODD: return "axis_c2r_odd";
    case OP_BLUE: return "axis_bluestein";
    case OP_DCT2: return "axis_dct2";
    case OP_DCT3: return "axis_dct3";
    case OP_DCT2_HALF: return "axis_dct2_half";
    case OP_DCT3_HALF: return "axis_dct3_half";
    default: return "axis_other";
  }
}
const char *pw_name(int op) {
  switch (op) {
    case PW_BLUE_PRE: return "pw_blue_pre";
    case PW_BLUE_MID: return "pw_blue_mid";
    case PW_BLUE_POST: return "pw_blue_post";
    case PW_R2C_PACK: return "pw_r2c_pack";
    case PW_R2C_TAKE: return "pw_r2c_take";
    case PW_C2R_BUILD: return "pw_c2r_build";
    case PW_C2R_TAKE: return "pw_c2r_take";
    default: return "pw_other";
  }
}

template <class F> void timed(const std::string &name, uint64_t bytes, cudaStream_t st, F launch) {
  if (!g_prof.load(std::memory_order_relaxed)) {
    launch();
    return;
  }
  ProfRec r{name, bytes, nullptr, nullptr};
  RG_CUDA(cudaEventCreate(&r.a));
  RG_CUDA(cudaEventCreate(&r.b));
  RG_CUDA(cudaEventRecord(r.a, st));
  launch();
  RG_CUDA(cudaEventRecord(r.b, st));
  std::lock_guard<std::mutex> lk(g_pmu);
  g_pending.push_back(r);
}

uint64_t axis_bytes(DType dt, int op, const KArgs &a) {
  const uint64_t c = cx_size(dt), r = real_size(dt);
  // units: real pairs for the even-length real ops, single reals for the odd ones
  const bool real_io = op == OP_DCT2 || op == OP_DCT3 || op == OP_DCT2_HALF || op == OP_DCT3_HALF;
  const uint64_t in_unit = op == OP_R2C_EVEN ? 2 * r : (op == OP_R2C_ODD || real_io) ? r : c;
  const uint64_t out_unit = op == OP_C2R_EVEN ? 2 * r : (op == OP_C2R_ODD || real_io) ? r : c;
  return uint64_t(a.nrows) * (uint64_t(a.nin) * in_unit + uint64_t(a.nout) * out_unit);
}
}  // namespace

void profile_enable(bool on) { g_prof.store(on); }

void profiled_launch(const char *name, uint64_t bytes, cudaStream_t st, const std::function<void()> &launch) {
  timed(name, bytes, st, launch);
}

std::vector<KernelStat> profile_read() {
  std::lock_guard<std::mutex> lk(g_pmu);
  for (ProfRec &r : g_pending) {
    RG_CUDA(cudaEventSynchronize(r.b));
    float ms = 0.f;
    RG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    KernelStat &k = g_agg[r.name];
    std::strncpy(k.name, r.name.c_str(), sizeof(k.name) - 1);
    k.launches += 1;
    k.total_ms += ms;
    k.bytes += r.bytes;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_pending.clear();
  std::vector<KernelStat> out;
  for (auto &kv : g_agg) out.push_back(kv.second);
  return out;
}

void profile_reset() {
  profile_read();
  std::lock_guard<std::mutex> lk(g_pmu);
  g_agg.clear();
}

void launch_axis(DType dt, int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st) {
  if (cfg.grid == 0) return;
  if (cfg.fixed && dt == DType::F32 && op == OP_C2C && cfg.col && a.core.L == 256 && tc_split_enabled()) {
    timed("axis_c2c_tc_f32", axis_bytes(dt, op, a), st, [&] {
      RG_CHECK(launch_tc_c2c(a, cfg.col, cfg.bwd, st), RG_ERR_INTERNAL, "tensor-core kernel rejected its job");
      note_launch();
      RG_CUDA(cudaGetLastError());
    });
    return;
  }
  const std::string name = std::string(axis_name(op)) + (dt == DType::F32 ? "_f32" : "_f64");
  timed(name, axis_bytes(dt, op, a), st, [&] {
    if (cfg.fixed) {
      const bool done = dt == DType::F32 ? launch_fixed_f32(op, a, cfg.col, cfg.bwd, cfg.pair_ok, st)
                                         : launch_fixed_f64(op, a, cfg.col, cfg.bwd, cfg.pair_ok, st);
      if (done) {
        note_launch();
        RG_CUDA(cudaGetLastError());
        return;
      }
    }
    if (dt == DType::F32)
      launch_axis_f32(op, a, cfg, st);
    else
      launch_axis_f64(op, a, cfg, st);
  });
}

void launch_pointwise(DType dt, int op, const PwArgs &a, cudaStream_t st) {
  const std::string name = std::string(pw_name(op)) + (dt == DType::F32 ? "_f32" : "_f64");
  timed(name, uint64_t(a.nrows) * uint64_t(a.nout) * 2 * cx_size(dt), st, [&] {
    if (dt == DType::F32)
      launch_pw_f32(op, a, st);
    else
      launch_pw_f64(op, a, st);
  });
}

void launch_mirror(DType dt, const MirrorArgs &a, cudaStream_t st) {
  timed(std::string("mirror") + (dt == DType::F32 ? "_f32" : "_f64"), uint64_t(a.total) * 2 * cx_size(dt), st,
        [&] {
          if (dt == DType::F32)
            launch_mirror_f32(a, st);
          else
            launch_mirror_f64(a, st);
        });
}

void set_smem_attr(const void *fn, size_t smem) {
  if (smem <= 48 * 1024) return;
  static std::mutex mu;
  static std::vector<std::pair<const void *, int>> done;
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  for (auto &p : done)
    if (p.first == fn && p.second == dev) return;
  RG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(max_smem_optin())));
  done.emplace_back(fn, dev);
}

int64_t resident_ctas(const void *fn, int threads, size_t smem) {
  struct Ent {
    const void *fn;
    int threads, dev;
    size_t smem;
    int64_t ctas;
  };
  static std::mutex mu;
  static std::vector<Ent> cache;
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lk(mu);
    for (const Ent &e : cache)
      if (e.fn == fn && e.threads == threads && e.smem == smem && e.dev == dev) return e.ctas;
  }
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  const int64_t ctas = int64_t(per_sm) * sm_count();
  std::lock_guard<std::mutex> lk(mu);
  cache.push_back({fn, threads, dev, smem, ctas});
  return ctas;
}

int sm_count() {
  static int cache[64] = {};
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && cache[dev]) return cache[dev];
  int v = 0;
  RG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
  if (dev < 64) cache[dev] = v;
  return v;
}

size_t max_smem_optin() {
  int dev = 0, v = 0;
  RG_CUDA(cudaGetDevice(&dev));
  RG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  return size_t(v);
}

}  // namespace rg
