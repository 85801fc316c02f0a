// Double-precision (complex128 / float64) instantiations of the transform kernels.
#include "rg_launch_impl.cuh"

namespace rg {
void launch_axis_f64(int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st) {
  launch_axis_typed<double>(op, a, cfg, st);
}
void launch_pw_f64(int op, const PwArgs &a, cudaStream_t st) { launch_pw_typed<double>(op, a, st); }
void launch_mirror_f64(const MirrorArgs &a, cudaStream_t st) { launch_mirror_typed<double>(a, st); }
}  // namespace rg
