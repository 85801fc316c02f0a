// Precision dispatch and launch bookkeeping.
#include "rg_launch.hpp"

#include <atomic>

#include "rg_error.hpp"

namespace rg {

void launch_axis_f32(int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st);
void launch_axis_f64(int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st);
void launch_pw_f32(int op, const PwArgs &a, cudaStream_t st);
void launch_pw_f64(int op, const PwArgs &a, cudaStream_t st);
void launch_mirror_f32(const MirrorArgs &a, cudaStream_t st);
void launch_mirror_f64(const MirrorArgs &a, cudaStream_t st);

static std::atomic<uint64_t> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

void launch_axis(DType dt, int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st) {
  if (cfg.grid == 0) return;
  if (dt == DType::F32)
    launch_axis_f32(op, a, cfg, st);
  else
    launch_axis_f64(op, a, cfg, st);
}

void launch_pointwise(DType dt, int op, const PwArgs &a, cudaStream_t st) {
  if (dt == DType::F32)
    launch_pw_f32(op, a, st);
  else
    launch_pw_f64(op, a, st);
}

void launch_mirror(DType dt, const MirrorArgs &a, cudaStream_t st) {
  if (dt == DType::F32)
    launch_mirror_f32(a, st);
  else
    launch_mirror_f64(a, st);
}

size_t max_smem_optin() {
  int dev = 0, v = 0;
  RG_CUDA(cudaGetDevice(&dev));
  RG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  return size_t(v);
}

}  // namespace rg
