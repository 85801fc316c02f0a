// Single-precision instances of the compile-time-L axis kernels: DCT/DST types II and III.
#include "rg_fixed_launch.cuh"

namespace rg {
RG_FIXED_OP_INSTANCE(float, OP_DCT2)
RG_FIXED_OP_INSTANCE(float, OP_DCT3)
}  // namespace rg
