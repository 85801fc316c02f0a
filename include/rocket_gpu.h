/*
 * rocket_gpu.h — C ABI of the GB300 pocketfft transform path.
 *
 * The ten `numba_*` entry points keep the names, argument order and argument types of the
 * reference's C shim rocket_fft/_pocketfft_numba.cpp (cited per function below), so the
 * reference's Numba intrinsics (rocket_fft/pocketfft.py:32-128) can bind them unchanged.
 * Array arguments use numba's array-struct layout; shapes are element counts and strides are
 * BYTES, as in the reference. `data` may be a device pointer (CUDA allocation, managed or
 * device memory) or a host pointer; host arrays are staged through device memory on the
 * current stream and the call returns after the result is back on the host.
 *
 * The reference returns void and reports nothing (its C++ exceptions cross the C ABI, which is
 * undefined behaviour). Here every void entry point records a status and message that
 * rocketgpu_last_status()/rocketgpu_last_error() return for the calling thread, and every
 * function has an `int`-returning `_st` twin. `nthreads` is accepted and ignored: the GPU grid
 * replaces the reference's CPU thread pool.
 */
#ifndef ROCKET_GPU_H
#define ROCKET_GPU_H

#include <stddef.h>
#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* numba's array struct (numba/_arraystruct.h, not vendored by the reference either):
 * shape_and_strides holds ndim extents followed by ndim byte strides. */
typedef struct rocketgpu_arystruct {
  void *meminfo;
  void *parent;
  int64_t nitems;
  int64_t itemsize;
  void *data;
  int64_t shape_and_strides[1]; /* really [2 * ndim] */
} rocketgpu_arystruct_t;

/* status codes */
#define RG_OK 0
#define RG_ERR_ARG 1         /* bad shape, stride, axis, dtype or type argument */
#define RG_ERR_UNSUPPORTED 2 /* valid request outside what this build implements */
#define RG_ERR_CUDA 3        /* a CUDA runtime call failed */
#define RG_ERR_NOMEM 4       /* device memory exhausted */
#define RG_ERR_INTERNAL 5

/* ---- drop-in entry points (same signatures as the reference) ---- */

/* rocket_fft/_pocketfft_numba.cpp:25-29 */
uint64_t numba_good_size(uint64_t target, bool real);

/* rocket_fft/_pocketfft_numba.cpp:31-49 (c2c), :91-109 (r2c), :111-143 (c2c_sym),
 * :145-163 (c2r) */
void numba_c2c(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
               rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);
void numba_r2c(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
               rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);
void numba_c2c_sym(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                   rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);
void numba_c2r(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
               rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);

/* rocket_fft/_pocketfft_numba.cpp:51-69 (dct), :71-89 (dst) */
void numba_dct(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
               rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho,
               uint64_t nthreads);
void numba_dst(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
               rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho,
               uint64_t nthreads);

/* rocket_fft/_pocketfft_numba.cpp:165-183 */
void numba_r2r_fftpack(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                       rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                       bool real2hermitian, bool forward, double fct, uint64_t nthreads);

/* rocket_fft/_pocketfft_numba.cpp:185-203 (separable), :205-223 (genuine) */
void numba_r2r_separable_hartley(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                 rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                                 double fct, uint64_t nthreads);
void numba_r2r_genuine_hartley(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                               rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                               double fct, uint64_t nthreads);

/* ---- status-returning twins (no reference counterpart: the reference returns void) ---- */
int numba_c2c_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                 rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);
int numba_r2c_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                 rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);
int numba_c2c_sym_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                     rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes, bool forward,
                     double fct, uint64_t nthreads);
int numba_c2r_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                 rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);
int numba_dct_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                 rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho,
                 uint64_t nthreads);
int numba_dst_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                 rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho,
                 uint64_t nthreads);
int numba_r2r_fftpack_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                         rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                         bool real2hermitian, bool forward, double fct, uint64_t nthreads);
int numba_r2r_separable_hartley_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                   rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                                   double fct, uint64_t nthreads);
int numba_r2r_genuine_hartley_st(uint64_t ndim, const rocketgpu_arystruct_t *ain,
                                 rocketgpu_arystruct_t *aout, rocketgpu_arystruct_t *axes,
                                 double fct, uint64_t nthreads);

/* ---- adjoints for automatic differentiation (no reference counterpart) ----
 * Same arguments as the transform whose adjoint they compute; ain is the cotangent of that
 * transform's output, aout receives the cotangent of its input.
 *   rocketgpu_r2c_adjoint_st: adjoint of numba_r2c -- a c2r in the opposite direction with the
 *     interior half-spectrum bins (0 < k < n/2) of the last axis halved; ain half spectrum,
 *     aout real.
 *   rocketgpu_c2r_adjoint_st: adjoint of numba_c2r -- an r2c in the opposite direction with
 *     those bins doubled; ain real, aout half spectrum.
 *   rocketgpu_dct_adjoint_st: transpose of numba_dct (types 1-4). */
int rocketgpu_r2c_adjoint_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                             rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);
int rocketgpu_c2r_adjoint_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                             rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads);
int rocketgpu_dct_adjoint_st(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                             rocketgpu_arystruct_t *axes, uint64_t type, double fct, bool ortho,
                             uint64_t nthreads);

/* ---- spectral Poisson solver kernels (no reference counterpart; the DCT-II/III application of
 * the transform path). Grids are C-contiguous n0 x n1 x n2, h = 1, Neumann boundaries (mirrored
 * ghost cells); the DCT-II diagonalises the 7-point Laplacian with eigenvalues
 * lam0[k0] + lam1[k1] + lam2[k2], lam_a[k] = 2 cos(pi k / n_a) - 2.
 *   rocketgpu_poisson_eigdiv: X /= lambda in place (float or double, itemsize 4/8; the table lam =
 *     lam0|lam1|lam2 is in the same precision as X, arithmetic in that precision: float32 by the
 *     fast division, within two ulp), mode 0 set to 0; lam = the three device tables back to
 *     back (n0+n1+n2 values).
 *   rocketgpu_poisson_update: u += delta with an exact two-sum whose rounding error goes to the
 *     float u_lo (u_lo may be NULL).
 *   rocketgpu_poisson_residual: r = f - A (u + u_lo) in double (u_lo may be NULL), written as
 *     float to r32 (if not NULL); sum(r^2) to *sumsq (device).
 *   rocketgpu_poisson_to_fx / _update_fx / _residual_fx / _fx_to_double: the same refinement
 *     with the iterate and the right-hand side in fixed point, u = U * 2^-e, f = F * 2^-e + Frem
 *     (U, F int64, Frem float, may be NULL): F = round(f * 2^e), Frem = f - F 2^-e;
 *     U += round(delta * 2^e); r = 2^-e (F - A U) + Frem, exact in integers until the final
 *     rounding to float (r32 if not NULL; sum(r^2) to *sumsq, squares formed
 *     as (r 2^-k)^2 with k the caller's estimate of log2 max|f|); out = U * 2^-e. The caller
 *     picks e so that |U| and |F| stay below 2^62.
 * All return a status; rocketgpu_poisson_last_error gives the calling thread's message. */
int rocketgpu_poisson_eigdiv(void *X, int64_t itemsize, int64_t n0, int64_t n1, int64_t n2, const void *lam,
                             void *stream);
/* out = rocketgpu_poisson_eigdiv applied to the DCT-II (fct 1) of the float32 volume in over all
 * three axes, the divide done by the last axis' pass as it stores (results identical to the two
 * calls; in and out C-contiguous, distinct or equal). Returns RG_ERR_UNSUPPORTED, having done
 * nothing, when the last axis has no compile-time kernel (n2 odd, n2 / 2 not a power of two in
 * the instantiated range): the caller then makes the two calls. */
int rocketgpu_poisson_dct2_eigdiv(const float *in, float *out, int64_t n0, int64_t n1, int64_t n2, const float *lam,
                                  void *stream);
int rocketgpu_poisson_update(double *u, float *u_lo, const float *delta, int64_t total, void *stream);
int rocketgpu_poisson_residual(const double *u, const float *u_lo, const double *f, float *r32, int64_t n0,
                               int64_t n1, int64_t n2, double *sumsq, void *stream);
int rocketgpu_poisson_update_fx(int64_t *U, const float *delta, int64_t total, int32_t e, void *stream);
int rocketgpu_poisson_to_fx(const double *f, int32_t e, int64_t *F, float *Frem, int64_t total, void *stream);
int rocketgpu_poisson_residual_fx(const int64_t *U, const int64_t *F, const float *Frem, int32_t e, int32_t k,
                                  float *r32, int64_t n0, int64_t n1, int64_t n2, double *sumsq, void *stream);
int rocketgpu_poisson_fx_to_double(const int64_t *U, int32_t e, double *out, int64_t total, void *stream);
/* out = (U - m) 2^-e with m = the mean of U rounded to an integer (exact 128-bit sum): the
 * zero-mean solution, without FP64 arithmetic per element. Workspace from the library's pool. */
int rocketgpu_poisson_fx_to_double_zero_mean(const int64_t *U, int32_t e, double *out, int64_t total, void *stream);
/* *out (device double) = max |x| over total float32 (itemsize 4) or float64 (8) elements of a
 * device array, by integer comparison of the bits. */
int rocketgpu_abs_max(const void *x, int64_t itemsize, int64_t total, double *out, void *stream);
/* U = round(delta 2^e): the first correction of the fixed-point iterate (no read of U). */
int rocketgpu_poisson_init_fx(int64_t *U, const float *delta, int64_t total, int32_t e, void *stream);
/* One pass over the right-hand side f (float64): r32 = float(f) rounded to nearest even,
 * stats[0] = max |f|, stats[1] = sum of float(f)^2 (device doubles). */
int rocketgpu_poisson_prepare(const double *f, float *r32, int64_t total, double *stats, void *stream);
const char *rocketgpu_poisson_last_error(void);

/* ---- batched uneven-length complex FFTs (no reference counterpart) ----
 * One plan for `count` transforms of the given lengths (complex64: itemsize 8, complex128: 16),
 * all forward or all backward, scaled by fct. Rows are stored back to back in flat device
 * buffers (row i starts at sum of lengths[0..i-1]). Execution is one persistent kernel launch
 * (plus a 4-byte counter reset) that allocates nothing, so it can be captured in a CUDA graph.
 * With autotune, rocketgpu_batch_create times the candidate schedules (on-chip capacity per CTA,
 * threads per CTA, four-step split policy) on these lengths and keeps the fastest;
 * rocketgpu_batch_info returns the choice and the timings as JSON. create returns NULL on error
 * (rocketgpu_last_error has the message). */
void *rocketgpu_batch_create(const int64_t *lengths, int64_t count, int64_t itemsize, bool forward, double fct,
                             int autotune);
int rocketgpu_batch_exec(void *plan, const void *in, void *out, void *stream);
int rocketgpu_batch_info(void *plan, char *buf, size_t len);
void rocketgpu_batch_destroy(void *plan);

/* ---- runtime control (no reference counterpart) ---- */

/* Status and message of the calling thread's most recent call (RG_OK / "" after success).
 * rocketgpu_last_error copies at most len-1 bytes plus a terminating NUL and returns the
 * status. */
int rocketgpu_last_status(void);
int rocketgpu_last_error(char *buf, size_t len);

/* The CUDA stream (cudaStream_t) the calling thread's transforms are issued on; NULL is the
 * legacy default stream. Device-array calls return without synchronising. */
void rocketgpu_set_stream(void *stream);
void *rocketgpu_get_stream(void);

/* Plan cache: number of cached plans, device bytes they hold, and a clear that must not run
 * concurrently with transforms. */
uint64_t rocketgpu_plan_cache_entries(void);
uint64_t rocketgpu_plan_cache_bytes(void);
int rocketgpu_plan_cache_clear(void);

/* Kernel launches issued by this library since load (all threads). */
uint64_t rocketgpu_launch_count(void);

/* Event-based per-kernel profile. While enabled, every kernel launch is bracketed by CUDA
 * events on its stream; rocketgpu_profile_read synchronises them and returns per-kernel-name
 * aggregates (launches, summed device milliseconds, summed algorithmic bytes = one read of the
 * launch's input rows plus one write of its output rows). Returns the number of entries
 * written (at most max). */
typedef struct rocketgpu_kstat {
  char name[48];
  uint64_t launches;
  double total_ms;
  uint64_t bytes;
} rocketgpu_kstat_t;
void rocketgpu_profile_enable(int on);
int rocketgpu_profile_read(rocketgpu_kstat_t *out, int max);
void rocketgpu_profile_reset(void);

/* Allocation-free complex FFT. No counterpart in the reference: it exists for callers that
 * cannot allocate device memory while they run (memory-capped or pre-partitioned contexts,
 * real-time loops that must not take the allocator's locks or fail on out-of-memory midway,
 * hosts whose device allocator belongs to another runtime). Same transform and arguments as
 * numba_c2c_st for DEVICE arrays of complex64/complex128, issued on `stream` (NULL = legacy
 * default stream); every length must be 13-smooth (on chip up to 8192, or a two-pass
 * product). It calls no cudaMalloc/cudaFree or any allocating library routine: plan tables and
 * the long-length workspace live in one 32 MiB static device array (held by every GPU that
 * loads the library until exit); requests that need more return RG_ERR_UNSUPPORTED without
 * doing any work. All calls share the array: calls whose GPU work overlaps race. The first call
 * on a device looks the array's address up (cudaGetSymbolAddress); make it before any stream
 * capture. Returns a status; a message (if any) is copied to errbuf (at most errlen-1 bytes
 * plus NUL; errbuf may be NULL). */
int rocketgpu_c2c_noalloc(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                          rocketgpu_arystruct_t *axes, bool forward, double fct, uint64_t nthreads,
                          void *stream, char *errbuf, size_t errlen);

/* Tensor-core split-FP16 form (no counterpart in the reference; a precision form of the same
 * transforms). While enabled (process-wide), complex64 transforms of length 256 along strided
 * axes run their two radix-16 stages as tcgen05 matrix products on FP16 hi/lo operand splits
 * with FP32 accumulation (about 22 significant bits per product); every other job keeps the
 * plain FP32 kernels. rocketgpu_set_tc_split returns the previous setting.
 * rocketgpu_tc_error returns 1 if a tensor-core kernel gave up waiting for its matrix products
 * since the library was loaded (0 otherwise, negative status on failure).
 * rocketgpu_tc_selftest computes D = A B^T + A B2^T + A2 B^T on the tensor cores through the
 * same operand layout, descriptors and tensor-memory path as the transform kernels: A, A2
 * 256 x 32, B, B2 32 x 32 float16 (row-major, device), D 256 x 32 float32 (device). */
int rocketgpu_set_tc_split(int on);
int rocketgpu_tc_error(void *stream);

/* Long power-of-two complex64 transforms (2^14 .. 2^24 points; no reference counterpart: the
 * reference runs such rows through cfftp::pass_all, rocket_fft/_pocketfft_hdronly.h:1690-1740)
 * run as one persistent launch whose CTAs wait on each other's tiles, each wait bounded to 2 s.
 * rocketgpu_long_error returns 1 if such a wait gave up since the previous call (and clears the
 * flag), 0 otherwise, a negative status on failure. Synchronises `stream`. */
int rocketgpu_long_error(void *stream);

/* Measurement aid (no reference counterpart): FP64 fused multiply-add throughput of the current
 * device in GFLOP/s, from a kernel of independent FMA chains timed with CUDA events on `stream`
 * (best of three launches) -- the FP64 roofline of the complex128 transforms. */
int rocketgpu_fp64_peak(double *gflops, void *stream);

/* Two-axis plane kernels (no reference counterpart; off unless switched on here or by
 * ROCKET_GPU_PLANE=1). While on, an r2c over two or more axes whose last axis (contiguous, even
 * power-of-two length) and the axis before it fit one of the compiled plane sizes runs those
 * two axes in one pass, one thread-block cluster per plane with the transposition through
 * distributed shared memory; c2r likewise. Measured slower than the axis-by-axis kernels on
 * GB300, kept as a tested alternative. Returns the previous setting. */
int rocketgpu_set_plane_kernels(int on);
int rocketgpu_tc_selftest(const void *A, const void *A2, const void *B, const void *B2, float *D, void *stream);

/* N-d cyclic shift, numpy.roll semantics over every dimension: out[(i_d + shifts[d]) mod n_d] =
 * in[i_d] (shifts: host array of ndim entries, any sign). The fftshift/ifftshift helpers of the
 * reference's NumPy/SciPy layer (rocket_fft/overloads.py:1251-1310, via np.roll). Any element
 * size of 1-16 bytes; in and out must be distinct arrays of the same shape; device arrays in
 * place, host arrays staged. Returns a status. */
int rocketgpu_roll(uint64_t ndim, const rocketgpu_arystruct_t *ain, rocketgpu_arystruct_t *aout,
                   const int64_t *shifts);

/* Library version string. */
const char *rocketgpu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ROCKET_GPU_H */
