// Host side of the plane kernels (rg_plane.cuh): two-axis r2c / c2r of whole planes in one
// thread-block cluster.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "rg_common.cuh"
#include "rg_plan.hpp"

namespace rg {

// Cluster size of the instance for (precision, log2 outer length E1, log2 real row length E2),
// 0 when there is none.
int plane_cluster(DType dt, int E1, int E2);

// Launch one instance over `nplanes` planes: forward = r2c along the rows then c2c along the
// outer axis (ar: row-phase loads, ac: column-phase stores, fct), inverse = the backward
// c2c then c2r (ac: column-phase loads, ar: row-phase stores, fct). False when no instance.
bool launch_plane(DType dt, bool inverse, int E1, int E2, const KArgs &ar, const KArgs &ac, int64_t nplanes,
                  cudaStream_t st);

}  // namespace rg
