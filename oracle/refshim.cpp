// Test infrastructure only: not part of the product.
//
// C shim over the reference's own pocketfft header (rocket_fft/_pocketfft_hdronly.h),
// compiled in place from the reference tree by oracle/Makefile into oracle/_ref/.
// It exports the same ten functions as rocket_fft/_pocketfft_numba.cpp:25-223, renamed
// with a `ref_` prefix, taking the same numba array-struct layout. The reference's
// own C++ file cannot be compiled here because it includes numba's private headers
// (_pocketfft_numba.cpp:5-6) and numba is not installed, so the layout is re-declared.
//
// A `long double` instantiation of c2c/r2c/c2r/dct/dst (ref_ld_*) provides a
// higher-than-FP64 answer for the tolerance tests: pocketfft computes its twiddles
// in `Thigh` = long double when T0 is long double (HDR:470).
#include <cstddef>
#include <cstdint>
#include <complex>
typedef std::ptrdiff_t npy_intp;
#include "_pocketfft_hdronly.h"

extern "C" {
typedef struct {
  void *meminfo;
  void *parent;
  npy_intp nitems;
  npy_intp itemsize;
  void *data;
  npy_intp shape_and_strides[1];
} arystruct_t;
}

using pocketfft::axes_view_t;
using pocketfft::shape_view_t;
using pocketfft::stride_view_t;
using pocketfft::detail::ndarr;
using pocketfft::detail::rev_iter;
using pocketfft::detail::util;

#define EXPORT extern "C" __attribute__((visibility("default")))

namespace {
struct Views {
  shape_view_t shape_in, shape_out;
  stride_view_t sin, sout;
  axes_view_t axes;
  Views(uint64_t ndim, const arystruct_t *ain, const arystruct_t *aout, const arystruct_t *ax)
      : shape_in(ain->shape_and_strides, ndim), shape_out(aout->shape_and_strides, ndim),
        sin(&ain->shape_and_strides[ndim], ndim), sout(&aout->shape_and_strides[ndim], ndim),
        axes(reinterpret_cast<const uint64_t *>(ax->data), uint64_t(ax->nitems)) {}
};
// The reference throws C++ exceptions across its C ABI (undefined behaviour there);
// here they become a status code so the tests can check which inputs are errors.
template <class F> int guarded(F f) {
  try {
    f();
    return 0;
  } catch (...) {
    return 1;
  }
}
} // namespace

EXPORT uint64_t ref_good_size(uint64_t target, bool real) {
  return real ? util::good_size_real(target) : util::good_size_cmplx(target);
}

EXPORT int ref_c2c(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout, arystruct_t *axes,
                   bool forward, double fct, uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 16)
      pocketfft::c2c<double>(v.shape_in, v.sin, v.sout, v.axes, forward,
                             (std::complex<double> *)ain->data, (std::complex<double> *)aout->data,
                             fct, nthreads);
    else
      pocketfft::c2c<float>(v.shape_in, v.sin, v.sout, v.axes, forward,
                            (std::complex<float> *)ain->data, (std::complex<float> *)aout->data,
                            float(fct), nthreads);
  });
}

template <class T>
static void c2c_sym_impl(const Views &v, const arystruct_t *ain, arystruct_t *aout, bool forward,
                         double fct, uint64_t nthreads) {
  auto in = (const T *)ain->data;
  auto out = (std::complex<T> *)aout->data;
  pocketfft::r2c<T>(v.shape_in, v.sin, v.sout, v.axes, forward, in, out, T(fct), nthreads);
  ndarr<std::complex<T>> ares(out, v.shape_in, v.sout);
  rev_iter iter(ares, v.axes);
  while (iter.remaining() > 0) {
    auto val = ares[iter.ofs()];
    ares[iter.rev_ofs()] = std::conj(val);
    iter.advance();
  }
}

EXPORT int ref_r2c(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout, arystruct_t *axes,
                   bool forward, double fct, uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 8)
      pocketfft::r2c<double>(v.shape_in, v.sin, v.sout, v.axes, forward, (const double *)ain->data,
                             (std::complex<double> *)aout->data, fct, nthreads);
    else
      pocketfft::r2c<float>(v.shape_in, v.sin, v.sout, v.axes, forward, (const float *)ain->data,
                            (std::complex<float> *)aout->data, float(fct), nthreads);
  });
}

EXPORT int ref_c2c_sym(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout,
                       arystruct_t *axes, bool forward, double fct, uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 8)
      c2c_sym_impl<double>(v, ain, aout, forward, fct, nthreads);
    else
      c2c_sym_impl<float>(v, ain, aout, forward, fct, nthreads);
  });
}

EXPORT int ref_c2r(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout, arystruct_t *axes,
                   bool forward, double fct, uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 16)
      pocketfft::c2r<double>(v.shape_out, v.sin, v.sout, v.axes, forward,
                             (const std::complex<double> *)ain->data, (double *)aout->data, fct,
                             nthreads);
    else
      pocketfft::c2r<float>(v.shape_out, v.sin, v.sout, v.axes, forward,
                            (const std::complex<float> *)ain->data, (float *)aout->data,
                            float(fct), nthreads);
  });
}

EXPORT int ref_dct(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout, arystruct_t *axes,
                   uint64_t type, double fct, bool ortho, uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 8)
      pocketfft::dct<double>(v.shape_in, v.sin, v.sout, v.axes, int(type),
                             (const double *)ain->data, (double *)aout->data, fct, ortho,
                             nthreads);
    else
      pocketfft::dct<float>(v.shape_in, v.sin, v.sout, v.axes, int(type), (const float *)ain->data,
                            (float *)aout->data, float(fct), ortho, nthreads);
  });
}

EXPORT int ref_dst(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout, arystruct_t *axes,
                   uint64_t type, double fct, bool ortho, uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 8)
      pocketfft::dst<double>(v.shape_in, v.sin, v.sout, v.axes, int(type),
                             (const double *)ain->data, (double *)aout->data, fct, ortho,
                             nthreads);
    else
      pocketfft::dst<float>(v.shape_in, v.sin, v.sout, v.axes, int(type), (const float *)ain->data,
                            (float *)aout->data, float(fct), ortho, nthreads);
  });
}

EXPORT int ref_r2r_fftpack(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout,
                           arystruct_t *axes, bool real2hermitian, bool forward, double fct,
                           uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 8)
      pocketfft::r2r_fftpack<double>(v.shape_in, v.sin, v.sout, v.axes, real2hermitian, forward,
                                     (const double *)ain->data, (double *)aout->data, fct,
                                     nthreads);
    else
      pocketfft::r2r_fftpack<float>(v.shape_in, v.sin, v.sout, v.axes, real2hermitian, forward,
                                    (const float *)ain->data, (float *)aout->data, float(fct),
                                    nthreads);
  });
}

EXPORT int ref_r2r_separable_hartley(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout,
                                     arystruct_t *axes, double fct, uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 8)
      pocketfft::r2r_separable_hartley<double>(v.shape_in, v.sin, v.sout, v.axes,
                                               (const double *)ain->data, (double *)aout->data,
                                               fct, nthreads);
    else
      pocketfft::r2r_separable_hartley<float>(v.shape_in, v.sin, v.sout, v.axes,
                                              (const float *)ain->data, (float *)aout->data,
                                              float(fct), nthreads);
  });
}

EXPORT int ref_r2r_genuine_hartley(uint64_t ndim, const arystruct_t *ain, arystruct_t *aout,
                                   arystruct_t *axes, double fct, uint64_t nthreads) {
  Views v(ndim, ain, aout, axes);
  return guarded([&] {
    if (ain->itemsize == 8)
      pocketfft::r2r_genuine_hartley<double>(v.shape_in, v.sin, v.sout, v.axes,
                                             (const double *)ain->data, (double *)aout->data, fct,
                                             nthreads);
    else
      pocketfft::r2r_genuine_hartley<float>(v.shape_in, v.sin, v.sout, v.axes,
                                            (const float *)ain->data, (float *)aout->data,
                                            float(fct), nthreads);
  });
}

// ---- long double (80-bit on x86) instantiations: the higher-precision answer ----
// Arrays are passed as contiguous long double buffers with byte strides.
EXPORT int ref_ld_c2c(uint64_t ndim, const npy_intp *shape, const npy_intp *sin,
                      const npy_intp *sout, uint64_t naxes, const uint64_t *axes, bool forward,
                      long double fct, const void *in, void *out) {
  return guarded([&] {
    pocketfft::c2c<long double>(shape_view_t(shape, ndim), stride_view_t(sin, ndim),
                                stride_view_t(sout, ndim), axes_view_t(axes, naxes), forward,
                                (const std::complex<long double> *)in,
                                (std::complex<long double> *)out, fct, 1);
  });
}

EXPORT int ref_ld_r2c(uint64_t ndim, const npy_intp *shape, const npy_intp *sin,
                      const npy_intp *sout, uint64_t naxes, const uint64_t *axes, bool forward,
                      long double fct, const void *in, void *out) {
  return guarded([&] {
    pocketfft::r2c<long double>(shape_view_t(shape, ndim), stride_view_t(sin, ndim),
                                stride_view_t(sout, ndim), axes_view_t(axes, naxes), forward,
                                (const long double *)in, (std::complex<long double> *)out, fct,
                                1);
  });
}

EXPORT int ref_ld_c2r(uint64_t ndim, const npy_intp *shape_out, const npy_intp *sin,
                      const npy_intp *sout, uint64_t naxes, const uint64_t *axes, bool forward,
                      long double fct, const void *in, void *out) {
  return guarded([&] {
    pocketfft::c2r<long double>(shape_view_t(shape_out, ndim), stride_view_t(sin, ndim),
                                stride_view_t(sout, ndim), axes_view_t(axes, naxes), forward,
                                (const std::complex<long double> *)in, (long double *)out, fct,
                                1);
  });
}

EXPORT int ref_ld_dcst(uint64_t ndim, const npy_intp *shape, const npy_intp *sin,
                       const npy_intp *sout, uint64_t naxes, const uint64_t *axes, bool cosine,
                       uint64_t type, long double fct, bool ortho, const void *in, void *out) {
  return guarded([&] {
    if (cosine)
      pocketfft::dct<long double>(shape_view_t(shape, ndim), stride_view_t(sin, ndim),
                                  stride_view_t(sout, ndim), axes_view_t(axes, naxes), int(type),
                                  (const long double *)in, (long double *)out, fct, ortho, 1);
    else
      pocketfft::dst<long double>(shape_view_t(shape, ndim), stride_view_t(sin, ndim),
                                  stride_view_t(sout, ndim), axes_view_t(axes, naxes), int(type),
                                  (const long double *)in, (long double *)out, fct, ortho, 1);
  });
}
