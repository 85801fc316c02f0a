// Launchers of the compile-time-L kernels (rg_fixed_kernel.cuh) for L = 64 ... 8192 (row walk)
// and L = 64 ... 1024 (column walk); instantiated per precision and op family in
// rg_fixed_{f32,f64}{,_real,_dct}.cu.
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
  launch_pdl(&fixed_kernel<T, OP, E, COL, BWD>, dim3(unsigned(grid)), dim3(C::NT), C::SMEM, st, a, pair_ok);
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
      case 13: fx_launch<T, OP, 13, COL, BWD>(a, pair_ok, st); return true;
      default: break;
    }
  }
  return false;
}

// Instances of one op (both walks and, for c2c, both directions); defined in the per-op
// translation units so that they compile in parallel.
template <typename T, int OP> bool launch_fixed_op(const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st);

template <typename T, int OP>
bool launch_fixed_op_impl(int E, const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st) {
  if constexpr (OP == OP_C2C) {
    if (col) return bwd ? fx_by_length<T, OP, true, true>(E, a, pair_ok, st) : fx_by_length<T, OP, true, false>(E, a, pair_ok, st);
    return bwd ? fx_by_length<T, OP, false, true>(E, a, pair_ok, st) : fx_by_length<T, OP, false, false>(E, a, pair_ok, st);
  } else {
    return col ? fx_by_length<T, OP, true, false>(E, a, pair_ok, st) : fx_by_length<T, OP, false, false>(E, a, pair_ok, st);
  }
}

#define RG_FIXED_OP_INSTANCE(T, OP)                                                                          \
  template <>                                                                                                \
  bool launch_fixed_op<T, OP>(const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st) {           \
    int E = 0;                                                                                               \
    while ((1 << E) < a.core.L) ++E;                                                                         \
    if ((1 << E) != a.core.L) return false;                                                                  \
    return launch_fixed_op_impl<T, OP>(E, a, col, bwd, pair_ok, st);                                         \
  }

// True when an instance exists for (op, L, walk, direction) and was launched.
template <typename T> bool launch_fixed_typed(int op, const KArgs &a, bool col, bool bwd, int pair_ok, cudaStream_t st) {
  switch (op) {
    case OP_C2C: return launch_fixed_op<T, OP_C2C>(a, col, bwd, pair_ok, st);
    case OP_R2C_EVEN: return launch_fixed_op<T, OP_R2C_EVEN>(a, col, bwd, pair_ok, st);
    case OP_C2R_EVEN: return launch_fixed_op<T, OP_C2R_EVEN>(a, col, bwd, pair_ok, st);
    case OP_DCT2: return launch_fixed_op<T, OP_DCT2>(a, col, bwd, pair_ok, st);
    case OP_DCT3: return launch_fixed_op<T, OP_DCT3>(a, col, bwd, pair_ok, st);
    case OP_DCT2_HALF: return launch_fixed_op<T, OP_DCT2_HALF>(a, col, bwd, pair_ok, st);
    case OP_DCT3_HALF: return launch_fixed_op<T, OP_DCT3_HALF>(a, col, bwd, pair_ok, st);
    default: return false;
  }
}

}  // namespace rg
