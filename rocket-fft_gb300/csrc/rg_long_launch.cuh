// Launch of the long-transform kernels (rg_long.cuh) and the list of instantiated shapes
// (log2 n1, log2 n2, log2 tile): one translation unit per kind (rg_long_{c2c,r2c,c2r}.cu)
// instantiates them, rg_long.cu chooses the shape and calls long_dispatch.
#pragma once
#include <algorithm>

#include "rg_error.hpp"
#include "rg_launch.hpp"
#include "rg_long.cuh"

namespace rg {

template <int KIND, int E1, int E2, int ET>
void launch_long(LongArgs &a, int64_t tickets, cudaStream_t st) {
  using Cf = LgCfg<E1, E2, ET, KIND>;
  const void *fn = reinterpret_cast<const void *>(&long_kernel<KIND, E1, E2, ET>);
  set_smem_attr(fn, Cf::SMEM);
  const int64_t res = resident_ctas(fn, Cf::NT, Cf::SMEM);
  RG_CHECK(res > 0, RG_ERR_INTERNAL, "long transform kernel does not fit on an SM");
  const unsigned grid = unsigned(std::min<int64_t>(tickets, res));
  long_kernel<KIND, E1, E2, ET><<<grid, Cf::NT, Cf::SMEM, st>>>(a);
  note_launch();
  RG_CUDA(cudaGetLastError());
}

// X(E1, E2, ET): every instantiated shape; the real kinds stop at half length 2^23
#define RG_LONG_SHAPES(X)                                                                          \
  X(7, 7, 10) X(7, 7, 11) X(7, 8, 10) X(7, 8, 11) X(8, 8, 11) X(8, 8, 12) X(8, 9, 11) X(8, 9, 12) \
  X(9, 9, 11) X(9, 9, 12) X(9, 9, 13) X(9, 10, 11) X(9, 10, 12) X(9, 10, 13) X(10, 10, 11)        \
  X(10, 10, 12) X(10, 10, 13) X(10, 11, 12) X(10, 11, 13) X(11, 11, 12) X(11, 11, 13)             \
  X(11, 11, 14) X(11, 12, 13) X(11, 12, 14) X(7, 7, 12) X(7, 8, 12)
#define RG_LONG_SHAPES_C2C_ONLY(X) X(12, 12, 13) X(12, 12, 14)

inline bool long_shape_instantiated(int e1, int e2, int et) {
#define RG_LONG_HAS(A, B, T) \
  if (e1 == A && e2 == B && et == T) return true;
  RG_LONG_SHAPES(RG_LONG_HAS)
  RG_LONG_SHAPES_C2C_ONLY(RG_LONG_HAS)
#undef RG_LONG_HAS
  return false;
}

// Launch kind KIND with shape (e1, e2, et); false when no such instance exists.
template <int KIND> bool long_dispatch(int e1, int e2, int et, LongArgs &a, int64_t tickets, cudaStream_t st);
template <> bool long_dispatch<LG_C2C>(int, int, int, LongArgs &, int64_t, cudaStream_t);
template <> bool long_dispatch<LG_R2C>(int, int, int, LongArgs &, int64_t, cudaStream_t);
template <> bool long_dispatch<LG_C2R>(int, int, int, LongArgs &, int64_t, cudaStream_t);

#define RG_LONG_CASE(A, B, T)                   \
  if (e1 == A && e2 == B && et == T) {          \
    launch_long<KIND_, A, B, T>(a, tickets, st); \
    return true;                                \
  }

}  // namespace rg
