// Double-precision instances of the compile-time-L axis kernels: c2c, and the dispatcher.
#include "rg_fixed_launch.cuh"

namespace rg {
RG_FIXED_OP_INSTANCE(double, OP_C2C)
template <> bool launch_fixed_op<double, OP_R2C_EVEN>(const KArgs &, bool, bool, int, cudaStream_t);
template <> bool launch_fixed_op<double, OP_C2R_EVEN>(const KArgs &, bool, bool, int, cudaStream_t);
template <> bool launch_fixed_op<double, OP_DCT2>(const KArgs &, bool, bool, int, cudaStream_t);
template <> bool launch_fixed_op<double, OP_DCT3>(const KArgs &, bool, bool, int, cudaStream_t);
template <> bool launch_fixed_op<double, OP_DCT2_HALF>(const KArgs &, bool, bool, int, cudaStream_t);
template <> bool launch_fixed_op<double, OP_DCT3_HALF>(const KArgs &, bool, bool, int, cudaStream_t);

bool launch_fixed_f64(int op, const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st) {
  return launch_fixed_typed<double>(op, a, col, bwd, pair_ok, st);
}
}  // namespace rg
