// Launchers of the compile-time-L kernels (rg_fixed_kernel.cuh), instantiated per precision by
// rg_fixed_f32.cu / rg_fixed_f64.cu for L = 64 ... 4096 (row walk) and L = 64 ... 1024
// (column walk).
#pragma once
#include "rg_error.hpp"
#include "rg_fixed_kernel.cuh"
#include "rg_launch.hpp"

namespace rg {

template <typename T, int OP, int E, bool COL, bool BWD>
void fx_launch(const KArgs &a, int pair_ok, cudaStream_t st) {
  using C = FxCfg<T, OP, E, COL>;
  const void *fn = reinterpret_cast<const void *>(&fixed_kernel<T, OP, E, COL, BWD>);
  set_smem_attr(fn, C::SMEM);
  const int64_t grid = (a.nrows + C::TB - 1) / C::TB;
  RG_CHECK(grid < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "too many transforms in one call");
  fixed_kernel<T, OP, E, COL, BWD><<<unsigned(grid), C::NT, C::SMEM, st>>>(a, pair_ok);
}

template <typename T, int OP, bool COL, bool BWD>
bool fx_by_length(int E, const KArgs &a, int pair_ok, cudaStream_t st) {
  switch (E) {
    case 6: fx_launch<T, OP, 6, COL, BWD>(a, pair_ok, st); return true;
    case 7: fx_launch<T, OP, 7, COL, BWD>(a, pair_ok, st); return true;
    case 8: fx_launch<T, OP, 8, COL, BWD>(a, pair_ok, st); return true;
    case 9: fx_launch<T, OP, 9, COL, BWD>(a, pair_ok, st); return true;
    case 10: fx_launch<T, OP, 10, COL, BWD>(a, pair_ok, st); return true;
    default: break;
  }
  if constexpr (!COL) {
    switch (E) {
      case 11: fx_launch<T, OP, 11, COL, BWD>(a, pair_ok, st); return true;
      case 12: fx_launch<T, OP, 12, COL, BWD>(a, pair_ok, st); return true;
      default: break;
    }
  }
  return false;
}

// True when an instance exists for (op, L, walk, direction) and was launched.
template <typename T> bool launch_fixed_typed(int op, const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st) {
  int E = 0;
  while ((1 << E) < a.core.L) ++E;
  if ((1 << E) != a.core.L) return false;
  switch (op) {
    case OP_C2C:
      if (col) return bwd ? fx_by_length<T, OP_C2C, true, true>(E, a, pair_ok, st)
                          : fx_by_length<T, OP_C2C, true, false>(E, a, pair_ok, st);
      return bwd ? fx_by_length<T, OP_C2C, false, true>(E, a, pair_ok, st)
                 : fx_by_length<T, OP_C2C, false, false>(E, a, pair_ok, st);
    case OP_R2C_EVEN:
      return col ? fx_by_length<T, OP_R2C_EVEN, true, false>(E, a, pair_ok, st)
                 : fx_by_length<T, OP_R2C_EVEN, false, false>(E, a, pair_ok, st);
    case OP_C2R_EVEN:
      return col ? fx_by_length<T, OP_C2R_EVEN, true, false>(E, a, pair_ok, st)
                 : fx_by_length<T, OP_C2R_EVEN, false, false>(E, a, pair_ok, st);
    default: return false;
  }
}

}  // namespace rg
