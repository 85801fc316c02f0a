// Single-precision instances of the compile-time-L axis kernels: even-length r2c and c2r.
#include "rg_fixed_launch.cuh"

namespace rg {
RG_FIXED_OP_INSTANCE(float, OP_R2C_EVEN)
RG_FIXED_OP_INSTANCE(float, OP_C2R_EVEN)
}  // namespace rg
