// Internal building blocks of the N-d driver (rg_exec.cpp), shared with the real-to-real
// transforms (rg_r2r.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "rg_common.cuh"
#include "rg_plan.hpp"

namespace rg {
namespace detail {

// Non-transformed dims of one axis job: sorted by stride (fastest first), merged where both
// sides are contiguous across them.
struct Batch {
  std::vector<int64_t> shape, s_in, s_out;
  int64_t nrows = 1;
};
Batch make_batch(const std::vector<int64_t> &shape, const std::vector<int64_t> &s_in,
                 const std::vector<int64_t> &s_out, int axis);
Side make_side(int64_t axis_stride, const std::vector<int64_t> &shape, const std::vector<int64_t> &strides);
Side with_inner(const Side &s, int64_t n, int64_t stride, int64_t new_axis_stride);
Side contiguous_rows(int64_t nrows, int64_t len);
bool fits_core(int64_t L, DType dt);
bool any_zero(const std::vector<int64_t> &shape);

// One on-chip axis job (a single kernel launch).
struct Job {
  DType dt;
  int op;
  int n;     // logical length
  int L;     // core length
  int Lsm;   // shared slots per row
  int nin, nout;
  const void *in;
  void *out;
  Side ld, st;
  int64_t nrows;
  bool cin, cout;
  double fct;
  const void *aux = nullptr, *aux2 = nullptr, *aux3 = nullptr;
  int aux_n = 1, aux_s = 0;
  double bscale = 1.0;  // interior half-spectrum bin scale (r2c/c2r adjoints)
  double e0 = 1.0;      // fused DCT ops: element-0 weight
  int flags = 0;        // fused DCT ops: bit 1 = DST
};
void run_job(const Job &j, cudaStream_t st);
// True when run_job hands job j to a compile-time-length kernel instance (power-of-two L in the
// instantiated range for its walk, both sides walking alike, 32-bit row numbers, specialised
// kernels enabled). Ops that exist only there (OP_DCT2_HALF, OP_DCT3_HALF) need it.
bool fixed_job_ok(const Job &j);

// Complex transforms of `nrows` rows of length n (any n: on chip, four-step or Bluestein),
// the forward core on data conjugated on load (cin) and store (cout), scaled by fct.
void c2c_rows(DType dt, int64_t n, const void *in, const Side &ld, void *out, const Side &sd,
              int64_t nrows, bool cin, bool cout, double fct, cudaStream_t st);

}  // namespace detail
}  // namespace rg
