// Typed launch helpers, included once per precision by rg_launch_f32.cu / rg_launch_f64.cu.
#pragma once
#include <algorithm>
#include <atomic>
#include <mutex>

#include "rg_axis_kernel.cuh"
#include "rg_pow2_kernel.cuh"
#include "rg_stream_kernel.cuh"
#include "rg_error.hpp"
#include "rg_launch.hpp"
#include "rg_pdl.cuh"

namespace rg {

inline void ensure_smem_attr(const void *fn, size_t smem) { set_smem_attr(fn, smem); }

// Persistent pipelined kernel: grid = min(tiles, CTAs resident at once).
template <typename T, int OP, int S>
void launch_stream_s(const KArgs &a, const LaunchCfg &cfg, const FastDiv &dIn, const FastDiv &dOut,
                     cudaStream_t st) {
  const void *fn = reinterpret_cast<const void *>(&stream_kernel<T, OP, S>);
  ensure_smem_attr(fn, cfg.smem);
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, cfg.threads, cfg.smem));
  RG_CHECK(per_sm > 0, RG_ERR_INTERNAL, "stream kernel does not fit on an SM");
  const int64_t cap = int64_t(per_sm) * sm_count();
  const unsigned grid = unsigned(std::min<int64_t>(cfg.grid, cap));
  StreamParams sp{cfg.pair_ok};
  stream_kernel<T, OP, S><<<grid, cfg.threads, cfg.smem, st>>>(a, dIn, dOut, sp);
}

template <typename T, int OP>
void launch_axis_t(const KArgs &a, const LaunchCfg &cfg, cudaStream_t st) {
  const FastDiv dTB = make_fastdiv(uint32_t(a.TB));
  const FastDiv dIn = make_fastdiv(uint32_t(a.nin > 0 ? a.nin : 1));
  const FastDiv dOut = make_fastdiv(uint32_t(a.nout > 0 ? a.nout : 1));
  if constexpr (OP == OP_C2C || OP == OP_R2C_EVEN || OP == OP_C2R_EVEN) {
    if (cfg.stages > 0) {
      switch (cfg.stages) {
        case 2: launch_stream_s<T, OP, 2>(a, cfg, dIn, dOut, st); break;
        case 3: launch_stream_s<T, OP, 3>(a, cfg, dIn, dOut, st); break;
        default: launch_stream_s<T, OP, 4>(a, cfg, dIn, dOut, st); break;
      }
      note_launch();
      RG_CUDA(cudaGetLastError());
      return;
    }
  }
  if constexpr (OP == OP_C2C || OP == OP_C2C_TW || OP == OP_R2C_EVEN || OP == OP_C2R_EVEN) {
    if (cfg.pow2) {
      const void *fn = reinterpret_cast<const void *>(&pow2_kernel<T, OP>);
      ensure_smem_attr(fn, cfg.smem);
      launch_pdl(&pow2_kernel<T, OP>, dim3(cfg.grid), dim3(cfg.threads), cfg.smem, st, a, dTB, dIn, dOut);
      note_launch();
      RG_CUDA(cudaGetLastError());
      return;
    }
  }
  const void *fn = reinterpret_cast<const void *>(&axis_kernel<T, OP>);
  ensure_smem_attr(fn, cfg.smem);
  launch_pdl(&axis_kernel<T, OP>, dim3(cfg.grid), dim3(cfg.threads), cfg.smem, st, a, dTB, dIn, dOut);
  note_launch();
  RG_CUDA(cudaGetLastError());
}

template <typename T> void launch_axis_typed(int op, const KArgs &a, const LaunchCfg &cfg, cudaStream_t st) {
  switch (op) {
    case OP_C2C: launch_axis_t<T, OP_C2C>(a, cfg, st); break;
    case OP_C2C_TW: launch_axis_t<T, OP_C2C_TW>(a, cfg, st); break;
    case OP_R2C_EVEN: launch_axis_t<T, OP_R2C_EVEN>(a, cfg, st); break;
    case OP_R2C_ODD: launch_axis_t<T, OP_R2C_ODD>(a, cfg, st); break;
    case OP_C2R_EVEN: launch_axis_t<T, OP_C2R_EVEN>(a, cfg, st); break;
    case OP_C2R_ODD: launch_axis_t<T, OP_C2R_ODD>(a, cfg, st); break;
    case OP_BLUE: launch_axis_t<T, OP_BLUE>(a, cfg, st); break;
    case OP_DCT2: launch_axis_t<T, OP_DCT2>(a, cfg, st); break;
    case OP_DCT3: launch_axis_t<T, OP_DCT3>(a, cfg, st); break;
    default: throw Error(RG_ERR_INTERNAL, "launch_axis: unknown op");
  }
}

// ---------------------------------------------------------------------------------------
// pointwise row kernels
// ---------------------------------------------------------------------------------------

template <typename T, int OP>
__global__ void __launch_bounds__(256) pointwise_kernel(const __grid_constant__ PwArgs a) {
  pdl_begin();
  const int n = a.n;
  const T fct = T(a.fct);
  for (int64_t g = blockIdx.y; g < a.nrows; g += gridDim.y) {
    const int64_t oi = side_offset(a.ld, g);
    const int64_t oo = side_offset(a.st, g);
    const int64_t si = a.ld.axis_stride, so = a.st.axis_stride;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nout; i += gridDim.x * blockDim.x) {
      if constexpr (OP == PW_BLUE_PRE) {
        const cx<T> *in = reinterpret_cast<const cx<T> *>(a.in);
        cx<T> v = mk<T>(T(0), T(0));
        if (i < n) {
          v = in[oi + i * si];
          if (a.conj_in) v.y = -v.y;
          v = mulc<T>(v, reinterpret_cast<const cx<T> *>(a.aux)[i]);
        }
        reinterpret_cast<cx<T> *>(a.out)[oo + i * so] = v;
      } else if constexpr (OP == PW_BLUE_MID) {
        const cx<T> v = reinterpret_cast<const cx<T> *>(a.in)[oi + i * si];
        reinterpret_cast<cx<T> *>(a.out)[oo + i * so] =
            cj<T>(mul<T>(v, reinterpret_cast<const cx<T> *>(a.aux2)[i]));
      } else if constexpr (OP == PW_BLUE_POST) {
        const cx<T> v = reinterpret_cast<const cx<T> *>(a.in)[oi + i * si];
        cx<T> y = cj<T>(mul<T>(v, reinterpret_cast<const cx<T> *>(a.aux)[i]));
        y = mk<T>(y.x * fct, (a.conj_out ? -y.y : y.y) * fct);
        reinterpret_cast<cx<T> *>(a.out)[oo + i * so] = y;
      } else if constexpr (OP == PW_R2C_PACK) {
        const T x = reinterpret_cast<const T *>(a.in)[oi + i * si];
        reinterpret_cast<cx<T> *>(a.out)[oo + i * so] = mk<T>(x, T(0));
      } else if constexpr (OP == PW_R2C_TAKE) {
        cx<T> v = reinterpret_cast<const cx<T> *>(a.in)[oi + i * si];
        if (i == 0 || 2 * i == n) v.y = T(0);
        else v = scl<T>(v, T(a.bscale));
        reinterpret_cast<cx<T> *>(a.out)[oo + i * so] = mk<T>(v.x * fct, (a.conj_out ? -v.y : v.y) * fct);
      } else if constexpr (OP == PW_C2R_BUILD) {
        const cx<T> *in = reinterpret_cast<const cx<T> *>(a.in);
        cx<T> w;
        if (2 * i <= n) {
          cx<T> x = in[oi + i * si];
          if (a.conj_in) x.y = -x.y;
          if (i == 0 || 2 * i == n) x.y = T(0);
          else x = scl<T>(x, T(a.bscale));
          w = cj<T>(x);
        } else {
          cx<T> x = in[oi + (n - i) * si];
          if (a.conj_in) x.y = -x.y;
          w = scl<T>(x, T(a.bscale));
        }
        reinterpret_cast<cx<T> *>(a.out)[oo + i * so] = w;
      } else if constexpr (OP == PW_C2R_TAKE) {
        const cx<T> v = reinterpret_cast<const cx<T> *>(a.in)[oi + i * si];
        reinterpret_cast<T *>(a.out)[oo + i * so] = v.x * fct;
      }
    }
  }
}

template <typename T, int OP> void launch_pw_t(const PwArgs &a, cudaStream_t st) {
  if (a.nrows <= 0 || a.nout <= 0) return;
  const int threads = 256;
  unsigned gx = unsigned((a.nout + threads - 1) / threads);
  if (gx > 4096) gx = 4096;
  int64_t gy = a.nrows;
  const int64_t target = 16384 / int64_t(gx) + 1;  // enough CTAs to fill the GPU
  if (gy > target) gy = target;
  if (gy > 65535) gy = 65535;
  launch_pdl(&pointwise_kernel<T, OP>, dim3(gx, unsigned(gy)), dim3(threads), 0, st, a);
  note_launch();
  RG_CUDA(cudaGetLastError());
}

template <typename T> void launch_pw_typed(int op, const PwArgs &a, cudaStream_t st) {
  switch (op) {
    case PW_BLUE_PRE: launch_pw_t<T, PW_BLUE_PRE>(a, st); break;
    case PW_BLUE_MID: launch_pw_t<T, PW_BLUE_MID>(a, st); break;
    case PW_BLUE_POST: launch_pw_t<T, PW_BLUE_POST>(a, st); break;
    case PW_R2C_PACK: launch_pw_t<T, PW_R2C_PACK>(a, st); break;
    case PW_R2C_TAKE: launch_pw_t<T, PW_R2C_TAKE>(a, st); break;
    case PW_C2R_BUILD: launch_pw_t<T, PW_C2R_BUILD>(a, st); break;
    case PW_C2R_TAKE: launch_pw_t<T, PW_C2R_TAKE>(a, st); break;
    default: throw Error(RG_ERR_INTERNAL, "launch_pointwise: unknown op");
  }
}

// ---------------------------------------------------------------------------------------
// Hermitian mirror for c2c_sym
// ---------------------------------------------------------------------------------------

template <typename T> __global__ void __launch_bounds__(256) mirror_kernel(const __grid_constant__ MirrorArgs a) {
  pdl_begin();
  cx<T> *d = reinterpret_cast<cx<T> *>(a.data);
  for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < a.total;
       idx += int64_t(gridDim.x) * blockDim.x) {
    int64_t rem = idx, po = 0, qo = 0, qlin = 0, mul = 1;
    bool outside = false;
    for (int k = a.ndim - 1; k >= 0; --k) {
      const int64_t ext = (k == a.last) ? a.half : a.shape[k];
      const int64_t q0 = rem / ext;
      const int64_t pos = rem - q0 * ext;
      rem = q0;
      int64_t qp = pos;
      if ((a.revmask >> k) & 1u) qp = pos == 0 ? 0 : a.shape[k] - pos;
      if (k == a.last && qp >= a.half) outside = true;
      po += pos * a.stride[k];
      qo += qp * a.stride[k];
      qlin += qp * mul;
      mul *= ext;
    }
    if (outside || qlin >= idx) {
      const cx<T> v = d[po];
      d[qo] = cj<T>(v);
    }
  }
}

template <typename T> void launch_mirror_typed(const MirrorArgs &a, cudaStream_t st) {
  if (a.total <= 0) return;
  int64_t blocks = (a.total + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  launch_pdl(&mirror_kernel<T>, dim3(unsigned(blocks)), dim3(256), 0, st, a);
  note_launch();
  RG_CUDA(cudaGetLastError());
}

}  // namespace rg
