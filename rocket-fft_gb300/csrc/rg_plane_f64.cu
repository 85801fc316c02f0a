// Plane-kernel instances, double.
#include "rg_plane.hpp"
#include "rg_plane_impl.cuh"

namespace rg {

int plane_cluster_f64(int E1, int E2) {
#define RG_CL(a, b, c) \
  if (E1 == a && E2 == b) return c;
  RG_PLANE_CASES_F64(RG_CL)
#undef RG_CL
  return 0;
}

bool launch_plane_f64(bool inverse, int E1, int E2, const KArgs &ar, const KArgs &ac, int64_t nplanes,
                     cudaStream_t st) {
#define RG_GO(a, b, c)                                                  \
  if (E1 == a && E2 == b) {                                             \
    plane_launch<double, a, b, c>(inverse, ar, ac, nplanes, st);         \
    return true;                                                        \
  }
  RG_PLANE_CASES_F64(RG_GO)
#undef RG_GO
  return false;
}

int plane_cluster_f32(int E1, int E2);
bool launch_plane_f32(bool inverse, int E1, int E2, const KArgs &ar, const KArgs &ac, int64_t nplanes,
                      cudaStream_t st);

int plane_cluster(DType dt, int E1, int E2) {
  return dt == DType::F32 ? plane_cluster_f32(E1, E2) : plane_cluster_f64(E1, E2);
}

bool launch_plane(DType dt, bool inverse, int E1, int E2, const KArgs &ar, const KArgs &ac, int64_t nplanes,
                  cudaStream_t st) {
  return dt == DType::F32 ? launch_plane_f32(inverse, E1, E2, ar, ac, nplanes, st)
                          : launch_plane_f64(inverse, E1, E2, ar, ac, nplanes, st);
}

}  // namespace rg
