// Launch of one plane-kernel instance (shared by the per-precision translation units).
#pragma once
#include "rg_error.hpp"
#include "rg_launch.hpp"
#include "rg_plane.cuh"

namespace rg {

template <typename T, int E1, int E2, int CL>
void plane_launch(bool inverse, const KArgs &ar, const KArgs &ac, int64_t nplanes, cudaStream_t st) {
  using P = PlaneCfg<T, E1, E2, CL>;
  const int64_t grid = nplanes * CL;
  RG_CHECK(grid < (int64_t(1) << 31), RG_ERR_UNSUPPORTED, "too many planes in one call");
  if (inverse) {
    const void *fn = reinterpret_cast<const void *>(&plane_c2r_kernel<T, E1, E2, CL>);
    set_smem_attr(fn, P::SMEM);
    launch_pdl(&plane_c2r_kernel<T, E1, E2, CL>, dim3(unsigned(grid)), dim3(P::NT), P::SMEM, st, ar, ac);
  } else {
    const void *fn = reinterpret_cast<const void *>(&plane_r2c_kernel<T, E1, E2, CL>);
    set_smem_attr(fn, P::SMEM);
    launch_pdl(&plane_r2c_kernel<T, E1, E2, CL>, dim3(unsigned(grid)), dim3(P::NT), P::SMEM, st, ar, ac);
  }
  note_launch();
  RG_CUDA(cudaGetLastError());
}

// The instances: (E1, E2, cluster size) with the plane (L1 x n2/2 complex elements) at most
// about 70 KB per CTA, so that three CTAs share an SM.
#define RG_PLANE_CASES(X) \
  X(7, 7, 2)              \
  X(7, 8, 2)              \
  X(8, 7, 2)              \
  X(8, 8, 4)              \
  X(9, 8, 8)

#define RG_PLANE_CASES_F64(X) \
  X(7, 7, 2)                  \
  X(7, 8, 4)                  \
  X(8, 7, 4)                  \
  X(8, 8, 8)

}  // namespace rg
