// N-d cyclic shift (numpy.roll / fftshift / ifftshift semantics): out[(i_d + shift_d) mod n_d] =
// in[i_d] for every dimension d, any element size of 1..16 bytes, any strides. The index map
// behind the fftshift/ifftshift helpers of the NumPy/SciPy-level front end
// (rocket_fft/overloads.py:1251-1310 implement them with np.roll).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "rg_error.hpp"
#include "rg_exec.hpp"
#include "rg_launch.hpp"

namespace rg {
namespace {

constexpr int kMaxRollDims = 16;

struct RollArgs {
  const unsigned char *in;
  unsigned char *out;
  int ndim;
  int64_t total;
  int64_t shape[kMaxRollDims];
  int64_t sin[kMaxRollDims], sout[kMaxRollDims];  // byte strides
  int64_t shift[kMaxRollDims];                     // in [0, n_d)
};

template <int B> struct Unit { unsigned char b[B]; };
template <> struct Unit<4> { uint32_t v; };
template <> struct Unit<8> { uint2 v; };
template <> struct Unit<16> { uint4 v; };

template <int B>
__global__ void __launch_bounds__(256) roll_kernel(const __grid_constant__ RollArgs a) {
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < a.total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    int64_t rem = idx, oi = 0, oo = 0;
    for (int d = a.ndim - 1; d >= 0; --d) {
      const int64_t n = a.shape[d];
      const int64_t q = rem / n, i = rem - q * n;
      rem = q;
      int64_t j = i + a.shift[d];
      if (j >= n) j -= n;
      oi += i * a.sin[d];
      oo += j * a.sout[d];
    }
    *reinterpret_cast<Unit<B> *>(a.out + oo) = *reinterpret_cast<const Unit<B> *>(a.in + oi);
  }
}

}  // namespace

void roll(const NdArray &in, const NdArray &out, int64_t itemsize, const std::vector<int64_t> &shifts,
          cudaStream_t st) {
  RG_CHECK(in.shape.size() <= size_t(kMaxRollDims), RG_ERR_UNSUPPORTED, "too many dimensions");
  RollArgs a{};
  a.in = static_cast<const unsigned char *>(in.data);
  a.out = static_cast<unsigned char *>(out.data);
  a.ndim = int(in.shape.size());
  a.total = 1;
  for (int d = 0; d < a.ndim; ++d) {
    const int64_t n = in.shape[d];
    a.shape[d] = n;
    a.sin[d] = in.stride[d] * itemsize;
    a.sout[d] = out.stride[d] * itemsize;
    a.shift[d] = n > 0 ? ((shifts[size_t(d)] % n) + n) % n : 0;
    a.total *= n;
  }
  if (a.total == 0) return;
  RG_CHECK(in.data != out.data, RG_ERR_ARG, "roll needs distinct input and output arrays");
  const int64_t blocks = std::min<int64_t>((a.total + 255) / 256, 152 * 32);
  switch (itemsize) {
    case 1: roll_kernel<1><<<unsigned(blocks), 256, 0, st>>>(a); break;
    case 2: roll_kernel<2><<<unsigned(blocks), 256, 0, st>>>(a); break;
    case 4: roll_kernel<4><<<unsigned(blocks), 256, 0, st>>>(a); break;
    case 8: roll_kernel<8><<<unsigned(blocks), 256, 0, st>>>(a); break;
    case 16: roll_kernel<16><<<unsigned(blocks), 256, 0, st>>>(a); break;
    default: throw Error(RG_ERR_UNSUPPORTED, "roll: item size must be 1, 2, 4, 8 or 16 bytes");
  }
  note_launch();
  RG_CUDA(cudaGetLastError());
}

}  // namespace rg
