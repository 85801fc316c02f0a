// Instances of the long-transform kernel for kind LG_R2C (rg_long.cuh, rg_long_launch.cuh).
#include "rg_long_launch.cuh"

namespace rg {

template <> bool long_dispatch<LG_R2C>(int e1, int e2, int et, LongArgs &a, int64_t tickets, cudaStream_t st) {
  constexpr int KIND_ = LG_R2C;
  RG_LONG_SHAPES(RG_LONG_CASE)

  return false;
}

}  // namespace rg
