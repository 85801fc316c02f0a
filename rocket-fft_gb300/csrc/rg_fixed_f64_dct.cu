// Double-precision instances of the compile-time-L axis kernels: DCT/DST types II and III.
#include "rg_fixed_launch.cuh"

namespace rg {
RG_FIXED_OP_INSTANCE(double, OP_DCT2)
RG_FIXED_OP_INSTANCE(double, OP_DCT3)
}  // namespace rg
