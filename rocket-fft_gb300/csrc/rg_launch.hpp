// Kernel launch layer: typed entry points into the axis-job kernel and the row-wise
// pointwise kernels, plus a process-wide launch counter.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <vector>

#include "rg_common.cuh"
#include "rg_plan.hpp"

namespace rg {

struct LaunchCfg {
  unsigned grid;
  int threads;
  size_t smem;
  bool pow2 = false;  // use the power-of-two specialised kernel (rg_pow2_kernel.cuh)
  int stages = 0;     // > 0: persistent pipelined kernel (rg_stream_kernel.cuh) with this many
                      // stage buffers; `grid` is then the tile count (the launch caps it at
                      // the CTAs that fit on the device at once)
  int pair_ok = 0;    // R2C_EVEN input / C2R_EVEN output: real pairs are contiguous and aligned
  bool fixed = false; // prefer the compile-time-L kernel (rg_fixed_kernel.cuh) when one exists
  bool col = false;   // fixed kernel: both sides walk across rows
  bool bwd = false;   // fixed kernel, C2C: conjugate on load and store
};

// Launch axis_kernel<T, op> with the given configuration.
void launch_axis(DType dt, int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st);

// Row-wise elementwise kernels used around multi-kernel transforms. For each row g and
// output element i (0 <= i < nout) the op reads the input row through `ld` and writes
// through `st` (both Side descriptors with the row decomposition of the axis kernel).
enum PwOp : int {
  PW_BLUE_PRE = 0,   // out[i] = i < n ? conj?(x_i) * conj(bk_i) : 0            (i < m)
  PW_BLUE_MID = 1,   // out[i] = conj(in_i * bkf_i)                             (i < m)
  PW_BLUE_POST = 2,  // out[i] = conj?(conj(in_i * bk_i)) * fct                 (i < n)
  PW_R2C_PACK = 3,   // out[i] = (x_i, 0)                                       (i < n)
  PW_R2C_TAKE = 4,   // out[i] = conj?(in_i) * fct, imag of bins 0, n/2 zeroed  (i <= n/2)
  PW_C2R_BUILD = 5,  // out = conj of the Hermitian extension of conj?(X)       (i < n)
  PW_C2R_TAKE = 6,   // out[i] = Re(in_i) * fct (real output)                   (i < n)
  PW_COUNT = 7
};

struct PwArgs {
  const void *in;
  void *out;
  Side ld, st;
  int64_t nrows;
  int nout;        // output elements per row
  int n;           // logical transform length
  int conj_in, conj_out;
  double fct;
  double bscale;  // interior half-spectrum bin scale (PW_R2C_TAKE, PW_C2R_BUILD)
  const void *aux, *aux2;
};

void launch_pointwise(DType dt, int op, const PwArgs &a, cudaStream_t st);

// Hermitian completion for c2c_sym: over every position p of the half-spectrum (last
// transformed axis cut to n/2+1, C order), q = mirror(p) (i -> (n_i - i) mod n_i on the
// transformed axes). out[q] = conj(out[p]) when q lies outside the half, or when it lies
// inside and comes at or after p in C order -- the serial rev_iter loop of the reference's
// numba_c2c_sym (rocket_fft/_pocketfft_numba.cpp:111-143) leaves exactly this state.
constexpr int kMaxDims = 16;
struct MirrorArgs {
  void *data;
  int ndim, last;
  uint32_t revmask;          // bit d set: axis d is transformed
  int64_t shape[kMaxDims];   // full shape
  int64_t stride[kMaxDims];  // complex-element strides
  int64_t half;              // n_last / 2 + 1
  int64_t total;             // product of the half shape
};
void launch_mirror(DType dt, const MirrorArgs &a, cudaStream_t st);

// Largest dynamic shared memory a CTA may use on the current device.
size_t max_smem_optin();
// Allow a kernel the large shared-memory carve-out (once per kernel and device).
void set_smem_attr(const void *fn, size_t smem);
// Streaming multiprocessors of the current device.
int sm_count();

// Tensor-core split-FP16 form (rg_tc_kernel.cu).
bool tc_split_enabled();
int set_tc_split(bool on);
bool launch_tc_c2c(const KArgs &a, bool col, bool bwd, cudaStream_t st);
int tc_error_flag(cudaStream_t st);
void tc_selftest(const void *A, const void *A2, const void *B, const void *B2, float *D, cudaStream_t st);

// Long power-of-two complex64 transforms, 2^14 .. 2^24 points (rg_long.cu): true when a batch of
// rows with these sides can take the two-phase persistent kernel.
bool long_c2c_ok(DType dt, int64_t n, const void *in, const Side &ld, const void *out, const Side &sd);
void long_c2c(DType dt, int64_t n, const void *in, const Side &ld, void *out, const Side &sd, int64_t nrows,
              bool cin, bool cout, double fct, cudaStream_t st);
// float32 real rows of n = 2m points, m = 2^14 .. 2^23, through the same kernel on the real pairs.
bool long_real_ok(DType dt, int64_t n, const void *real, const Side &rs, const Side &cs, double bscale);
void long_r2c(int64_t n, const void *in, const Side &ld, void *out, const Side &sd, int64_t nrows, bool cout,
              double fct, cudaStream_t st);
void long_c2r(int64_t n, const void *in, const Side &ld, void *out, const Side &sd, int64_t nrows, bool cin,
              double fct, cudaStream_t st);
// 1 if a long-transform kernel gave up waiting on another CTA since the last call (cleared).
int long_error_flag(cudaStream_t st);

// FP64 fused multiply-add throughput of the current device, GFLOP/s (rg_probe.cu).
double fp64_peak_gflops(cudaStream_t st);

uint64_t launch_count();
void note_launch();

// Per-kernel profile (see rocketgpu_profile_* in include/rocket_gpu.h).
struct KernelStat {
  char name[48] = {0};
  uint64_t launches = 0;
  double total_ms = 0;
  uint64_t bytes = 0;
};
void profile_enable(bool on);
// Run `launch` (one kernel launch on `st`) under the profile when it is enabled, recording
// `bytes` algorithmic bytes for kernel `name`.
void profiled_launch(const char *name, uint64_t bytes, cudaStream_t st, const std::function<void()> &launch);
std::vector<KernelStat> profile_read();
void profile_reset();

}  // namespace rg
