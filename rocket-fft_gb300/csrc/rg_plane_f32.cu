// Plane-kernel instances, float.
#include "rg_plane.hpp"
#include "rg_plane_impl.cuh"

namespace rg {

int plane_cluster_f32(int E1, int E2) {
#define RG_CL(a, b, c) \
  if (E1 == a && E2 == b) return c;
  RG_PLANE_CASES(RG_CL)
#undef RG_CL
  return 0;
}

bool launch_plane_f32(bool inverse, int E1, int E2, const KArgs &ar, const KArgs &ac, int64_t nplanes,
                     cudaStream_t st) {
#define RG_GO(a, b, c)                                                  \
  if (E1 == a && E2 == b) {                                             \
    plane_launch<float, a, b, c>(inverse, ar, ac, nplanes, st);         \
    return true;                                                        \
  }
  RG_PLANE_CASES(RG_GO)
#undef RG_GO
  return false;
}

}  // namespace rg
