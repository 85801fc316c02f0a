// Single-precision instances of the compile-time-L axis kernels.
#include "rg_fixed_launch.cuh"

namespace rg {
bool launch_fixed_f32(int op, const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st) {
  return launch_fixed_typed<float>(op, a, col, bwd, pair_ok, st);
}
}  // namespace rg
