// Host check (no GPU): the compile-time pass schedule of the fixed-length kernels
// (rg_fixed_kernel.cuh: radices, Ns, twiddle-table offsets) equals the host core plan
// (core_radices in rg_plan.cpp and the table layout of get_core) for every power of two up to
// 2^16, and every instantiated configuration fits the 227 KB shared-memory budget.
#include <cstdio>
#include <vector>

#include "rg_fixed_kernel.cuh"
#include "rg_plan.hpp"

// The planner's Bluestein tables are built by the library's kernels (rg_plan_dev.cu), which this
// host-only check does not link; it builds no Bluestein plan.
namespace rg {
void blue_tables_device(uint64_t, uint64_t, DType, void *, void *) {}
}  // namespace rg

template <typename T, int OP, int E, bool COL> int check_cfg() {
  using C = rg::FxCfg<T, OP, E, COL>;
  if (C::SMEM > 227 * 1024) {
    std::printf("smem %zu too large: E=%d col=%d\n", C::SMEM, E, int(COL));
    return 1;
  }
  return 0;
}

template <typename T, int OP, bool COL> int check_all() {
  int bad = check_cfg<T, OP, 6, COL>() + check_cfg<T, OP, 7, COL>() + check_cfg<T, OP, 8, COL>() +
            check_cfg<T, OP, 9, COL>() + check_cfg<T, OP, 10, COL>();
  if (!COL) bad += check_cfg<T, OP, 11, COL>() + check_cfg<T, OP, 12, COL>() + check_cfg<T, OP, 13, COL>();
  return bad;
}

int main() {
  int bad = 0;
  for (int e = 1; e <= 16; ++e) {
    const std::vector<int> r = rg::core_radices(1 << e);
    if (int(r.size()) != rg::fx::np_of(e)) {
      std::printf("pass count differs at L=2^%d\n", e);
      ++bad;
      continue;
    }
    int ns = 1, tw = 0;
    for (int p = 0; p < int(r.size()); ++p) {
      if (r[p] != rg::fx::radix_of(e, p) || ns != rg::fx::ns_of(e, p) || tw != rg::fx::tw_of(e, p)) {
        std::printf("pass %d of L=2^%d differs\n", p, e);
        ++bad;
      }
      if (ns > 1) tw += (r[p] - 1) * ns;
      ns *= r[p];
    }
  }
  bad += check_all<float, rg::OP_C2C, false>() + check_all<float, rg::OP_C2C, true>();
  bad += check_all<float, rg::OP_R2C_EVEN, false>() + check_all<float, rg::OP_R2C_EVEN, true>();
  bad += check_all<float, rg::OP_C2R_EVEN, false>() + check_all<float, rg::OP_C2R_EVEN, true>();
  bad += check_all<double, rg::OP_C2C, false>() + check_all<double, rg::OP_C2C, true>();
  bad += check_all<double, rg::OP_R2C_EVEN, false>() + check_all<double, rg::OP_R2C_EVEN, true>();
  bad += check_all<double, rg::OP_C2R_EVEN, false>() + check_all<double, rg::OP_C2R_EVEN, true>();
  std::printf("%d mismatches\n", bad);
  return bad ? 1 : 0;
}
