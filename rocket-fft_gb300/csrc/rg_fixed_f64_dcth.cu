// Double-precision instances of the compile-time-L axis kernels: DCT/DST types II and III through
// the half-length FFT.
#include "rg_fixed_launch.cuh"

namespace rg {
RG_FIXED_OP_INSTANCE(double, OP_DCT2_HALF)
RG_FIXED_OP_INSTANCE(double, OP_DCT3_HALF)
}  // namespace rg
