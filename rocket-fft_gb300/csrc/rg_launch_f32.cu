// Single-precision (complex64 / float32) instantiations of the transform kernels.
#include "rg_launch_impl.cuh"

namespace rg {
void launch_axis_f32(int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st) {
  launch_axis_typed<float>(op, a, cfg, st);
}
void launch_pw_f32(int op, const PwArgs &a, cudaStream_t st) { launch_pw_typed<float>(op, a, st); }
void launch_mirror_f32(const MirrorArgs &a, cudaStream_t st) { launch_mirror_typed<float>(a, st); }
}  // namespace rg
