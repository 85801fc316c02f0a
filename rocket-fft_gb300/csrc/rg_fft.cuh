// On-chip mixed-radix FFT for sm_103a: complex helpers, forward butterflies, and the
// Stockham radix pass over rows held in shared memory.
//
// Formulation (one pass of radix R over a length-L row, Ns = product of earlier radices):
//   butterfly j in [0, L/R):  m = j mod Ns
//     v_k = a[j + k*L/R] * W_{Ns*R}^{m*k}             (k = 0..R-1, W_N = e^{-2 pi i / N})
//     y   = DFT_R(v)
//     b[(j - m)*R + m + k*Ns] = y_k
// Reads are unit-stride across consecutive j (conflict-free after padding); the result is in
// natural order after the last pass (self-sorting, no bit reversal). The core only computes
// the forward transform; backward transforms conjugate on load and on store.
//
// This plays the role of the reference's cfftp::pass_all (rocket_fft/_pocketfft_hdronly.h:
// 1690-1740) and its passN butterflies (HDR:1079-1688); the decomposition is a GPU Stockham
// autosort instead of FFTPACK's in-place ping-pong, so the arithmetic order differs and only
// the results (within rounding) match.
#pragma once
#include "rg_common.cuh"

namespace rg {

template <typename T> struct CxT;
template <> struct CxT<float> { using type = float2; };
template <> struct CxT<double> { using type = double2; };
template <typename T> using cx = typename CxT<T>::type;

template <typename T> __host__ __device__ __forceinline__ cx<T> mk(T r, T i) {
  cx<T> z;
  z.x = r;
  z.y = i;
  return z;
}
template <typename T> __host__ __device__ __forceinline__ cx<T> add(cx<T> a, cx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __host__ __device__ __forceinline__ cx<T> sub(cx<T> a, cx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __host__ __device__ __forceinline__ cx<T> mul(cx<T> a, cx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> __host__ __device__ __forceinline__ cx<T> mulc(cx<T> a, cx<T> b) {
  return mk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T> __host__ __device__ __forceinline__ cx<T> scl(cx<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
template <typename T> __host__ __device__ __forceinline__ cx<T> cj(cx<T> a) { return mk<T>(a.x, -a.y); }
// a * (-i)
template <typename T> __host__ __device__ __forceinline__ cx<T> mnegi(cx<T> a) { return mk<T>(a.y, -a.x); }
// a * i
template <typename T> __host__ __device__ __forceinline__ cx<T> mposi(cx<T> a) { return mk<T>(-a.y, a.x); }

// cos(2 pi t / R) and sin(2 pi t / R), 1 <= t <= (R-1)/2, correctly rounded to double.
__host__ __device__ __forceinline__ constexpr double kcos(int R, int t) {
  return R == 3 ? -0.5
       : R == 5 ? (t == 1 ? 0.30901699437494745 : -0.8090169943749475)
       : R == 7 ? (t == 1 ? 0.6234898018587335 : t == 2 ? -0.2225209339563144 : -0.9009688679024191)
       : R == 11 ? (t == 1 ? 0.8412535328311812 : t == 2 ? 0.41541501300188644
                  : t == 3 ? -0.14231483827328514 : t == 4 ? -0.6548607339452851 : -0.9594929736144974)
       : /* 13 */ (t == 1 ? 0.8854560256532099 : t == 2 ? 0.5680647467311558
                  : t == 3 ? 0.12053668025532305 : t == 4 ? -0.3546048870425356
                  : t == 5 ? -0.7485107481711011 : -0.970941817426052);
}
__host__ __device__ __forceinline__ constexpr double ksin(int R, int t) {
  return R == 3 ? 0.8660254037844386
       : R == 5 ? (t == 1 ? 0.9510565162951535 : 0.5877852522924731)
       : R == 7 ? (t == 1 ? 0.7818314824680298 : t == 2 ? 0.9749279121818236 : 0.4338837391175581)
       : R == 11 ? (t == 1 ? 0.5406408174555976 : t == 2 ? 0.9096319953545183
                  : t == 3 ? 0.9898214418809327 : t == 4 ? 0.7557495743542583 : 0.28173255684142967)
       : /* 13 */ (t == 1 ? 0.46472317204376856 : t == 2 ? 0.8229838658936564
                  : t == 3 ? 0.992708874098054 : t == 4 ? 0.9350162426854148
                  : t == 5 ? 0.6631226582407952 : 0.23931566428755777);
}

constexpr double kSqrtHalf = 0.7071067811865476;
constexpr double kCos8 = 0.9238795325112867;  // cos(pi/8)
constexpr double kSin8 = 0.3826834323650898;  // sin(pi/8)

// cos(pi s / 16) and sin(pi s / 16), 1 <= s <= 7, correctly rounded to double
__host__ __device__ __forceinline__ constexpr double kc16(int s) {
  return s == 1 ? 0.9807852804032304 : s == 2 ? 0.9238795325112867 : s == 3 ? 0.8314696123025452
       : s == 4 ? 0.7071067811865476 : s == 5 ? 0.5555702330196022 : s == 6 ? 0.3826834323650898
       : 0.19509032201612828;
}
__host__ __device__ __forceinline__ constexpr double ks16(int s) { return kc16(8 - s); }

template <typename T> __host__ __device__ __forceinline__ void dft4(cx<T> &a0, cx<T> &a1, cx<T> &a2, cx<T> &a3) {
  cx<T> t0 = add<T>(a0, a2), t1 = sub<T>(a0, a2), t2 = add<T>(a1, a3), t3 = mnegi<T>(sub<T>(a1, a3));
  a0 = add<T>(t0, t2);
  a2 = sub<T>(t0, t2);
  a1 = add<T>(t1, t3);
  a3 = sub<T>(t1, t3);
}

// multiply by W_16^e for the exponents that occur in the 4x4 split
template <typename T, int E> __host__ __device__ __forceinline__ cx<T> w16(cx<T> a) {
  const T c = T(kCos8), s = T(kSin8), r = T(kSqrtHalf);
  if constexpr (E == 0) return a;
  else if constexpr (E == 1) return mk<T>(a.x * c + a.y * s, a.y * c - a.x * s);    // (c, -s)
  else if constexpr (E == 2) return mk<T>((a.x + a.y) * r, (a.y - a.x) * r);        // (r, -r)
  else if constexpr (E == 3) return mk<T>(a.x * s + a.y * c, a.y * s - a.x * c);    // (s, -c)
  else if constexpr (E == 4) return mnegi<T>(a);                                      // -i
  else if constexpr (E == 6) return mk<T>((a.y - a.x) * r, -(a.x + a.y) * r);       // (-r, -r)
  else return mk<T>(-a.x * c - a.y * s, a.x * s - a.y * c);                         // E == 9: (-c, s)
}

// multiply by W_32^S = cos(pi S / 16) - i sin(pi S / 16), 0 <= S < 16
template <typename T, int S> __host__ __device__ __forceinline__ cx<T> w32(cx<T> a) {
  if constexpr (S == 0) {
    return a;
  } else if constexpr (S == 8) {
    return mnegi<T>(a);
  } else {
    constexpr double c = S < 8 ? kc16(S) : -kc16(16 - S);
    constexpr double sn = S < 8 ? ks16(S) : ks16(16 - S);
    return mk<T>(a.x * T(c) + a.y * T(sn), a.y * T(c) - a.x * T(sn));
  }
}
// the radix-2 combination of a 32-point DFT: y_s = e_s + W_32^s o_s, y_{s+16} = e_s - W_32^s o_s
template <typename T, int S> __host__ __device__ __forceinline__ void dft32_join(cx<T> *v, const cx<T> *e, const cx<T> *o) {
  if constexpr (S < 16) {
    const cx<T> t = w32<T, S>(o[S]);
    v[S] = add<T>(e[S], t);
    v[S + 16] = sub<T>(e[S], t);
    dft32_join<T, S + 1>(v, e, o);
  }
}

template <typename T, int R> __host__ __device__ __forceinline__ void dft_odd(cx<T> *v) {
  // v[k], v[R-k] are replaced by their sum and difference in place; outputs y_q, y_{R-q}
  // are accumulated pairwise and written back once every pair has been consumed, so the
  // live set is the R inputs plus one output pair per q (kept in the upper half of v only
  // after the sums/differences it overwrites are no longer needed).
  constexpr int H = (R - 1) / 2;
  const cx<T> x0 = v[0];
  cx<T> y0 = x0;
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    const cx<T> a = v[k], b = v[R - k];
    v[k] = add<T>(a, b);      // s_k
    v[R - k] = sub<T>(a, b);  // d_k
    y0 = add<T>(y0, v[k]);
  }
  cx<T> out[R - 1];
#pragma unroll
  for (int q = 1; q <= H; ++q) {
    cx<T> re = x0, im = mk<T>(T(0), T(0));
#pragma unroll
    for (int k = 1; k <= H; ++k) {
      const int t = (q * k) % R;
      const int tt = t <= H ? t : R - t;  // cos symmetric, sin antisymmetric
      const T c = T(kcos(R, tt));
      const T sn = t <= H ? T(ksin(R, tt)) : -T(ksin(R, tt));
      re = mk<T>(re.x + v[k].x * c, re.y + v[k].y * c);
      im = mk<T>(im.x + v[R - k].x * sn, im.y + v[R - k].y * sn);
    }
    out[q - 1] = mk<T>(re.x + im.y, re.y - im.x);      // y_q = re - i*im
    out[R - 1 - q] = mk<T>(re.x - im.y, re.y + im.x);  // y_{R-q} = re + i*im
  }
  v[0] = y0;
#pragma unroll
  for (int q = 1; q < R; ++q) v[q] = out[q - 1];
}

// Forward DFT of R points held in registers, natural order in and out.
template <typename T, int R> __host__ __device__ __forceinline__ void dft(cx<T> *v) {
  if constexpr (R == 2) {
    cx<T> t = v[0];
    v[0] = add<T>(t, v[1]);
    v[1] = sub<T>(t, v[1]);
  } else if constexpr (R == 4) {
    dft4<T>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    cx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    cx<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<T>(e0, e1, e2, e3);
    dft4<T>(o0, o1, o2, o3);
    const T r = T(kSqrtHalf);
    o1 = mk<T>((o1.x + o1.y) * r, (o1.y - o1.x) * r);
    o2 = mnegi<T>(o2);
    o3 = mk<T>((o3.y - o3.x) * r, -(o3.x + o3.y) * r);
    v[0] = add<T>(e0, o0); v[4] = sub<T>(e0, o0);
    v[1] = add<T>(e1, o1); v[5] = sub<T>(e1, o1);
    v[2] = add<T>(e2, o2); v[6] = sub<T>(e2, o2);
    v[3] = add<T>(e3, o3); v[7] = sub<T>(e3, o3);
  } else if constexpr (R == 16) {
    // a_{4p+q}: DFT4 over p for each q, twiddle W16^{qs}, DFT4 over q; y_{s+4t}
    dft4<T>(v[0], v[4], v[8], v[12]);
    dft4<T>(v[1], v[5], v[9], v[13]);
    dft4<T>(v[2], v[6], v[10], v[14]);
    dft4<T>(v[3], v[7], v[11], v[15]);
    v[5] = w16<T, 1>(v[5]);  v[9] = w16<T, 2>(v[9]);  v[13] = w16<T, 3>(v[13]);
    v[6] = w16<T, 2>(v[6]);  v[10] = w16<T, 4>(v[10]); v[14] = w16<T, 6>(v[14]);
    v[7] = w16<T, 3>(v[7]);  v[11] = w16<T, 6>(v[11]); v[15] = w16<T, 9>(v[15]);
    // now v[4s+q] holds b[q][s]
    dft4<T>(v[0], v[1], v[2], v[3]);
    dft4<T>(v[4], v[5], v[6], v[7]);
    dft4<T>(v[8], v[9], v[10], v[11]);
    dft4<T>(v[12], v[13], v[14], v[15]);
    // v[4s+t] holds y_{s+4t}: transpose the 4x4 index
    cx<T> t;
    t = v[1]; v[1] = v[4]; v[4] = t;
    t = v[2]; v[2] = v[8]; v[8] = t;
    t = v[3]; v[3] = v[12]; v[12] = t;
    t = v[6]; v[6] = v[9]; v[9] = t;
    t = v[7]; v[7] = v[13]; v[13] = t;
    t = v[11]; v[11] = v[14]; v[14] = t;
  } else if constexpr (R == 32) {
    // even and odd points through two 16-point DFTs, then one radix-2 step
    cx<T> e[16], o[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      e[j] = v[2 * j];
      o[j] = v[2 * j + 1];
    }
    dft<T, 16>(e);
    dft<T, 16>(o);
    dft32_join<T, 0>(v, e, o);
  } else {
    dft_odd<T, R>(v);
  }
}

// Shared-memory index of element i of row r.
__device__ __forceinline__ int sidx(int r, int i, int pitch, int ps) { return r * pitch + i + (i >> ps); }

// One radix-R pass over `rows` rows: shared buffer src -> shared buffer dst (ping-pong), one
// butterfly live per thread at a time, barrier at the end.
template <typename T, int R>
__device__ __forceinline__ void fft_pass(const cx<T> *__restrict__ src, cx<T> *__restrict__ dst, int rows,
                                         int pitch, int ps, const PassDesc &pd,
                                         const cx<T> *__restrict__ tw) {
  const int LR = pd.LR;
  const int nbf = rows * LR;
  for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
    const int r = int(fdiv(uint32_t(bf), pd.dLR));
    const int j = bf - r * LR;
    const cx<T> *s = src + r * pitch;
    cx<T> v[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int i = j + k * LR;
      v[k] = s[i + (i >> ps)];
    }
    int m = 0;
    if (pd.Ns > 1) {
      m = j - int(fdiv(uint32_t(j), pd.dNs)) * pd.Ns;
      const cx<T> *t = tw + pd.tw + m;
#pragma unroll
      for (int k = 1; k < R; ++k) v[k] = mul<T>(v[k], t[(k - 1) * pd.Ns]);
    }
    dft<T, R>(v);
    cx<T> *d = dst + r * pitch;
    const int base = (j - m) * R + m;
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int i = base + k * pd.Ns;
      d[i + (i >> ps)] = v[k];
    }
  }
  __syncthreads();
}

// All passes of the core over `rows` rows (forward transform, natural order). The data
// starts in buf[0]; returns the buffer that holds the result.
template <typename T>
__device__ __forceinline__ cx<T> *fft_rows(cx<T> *buf0, cx<T> *buf1, int rows, int pitch, int ps,
                                           const FFTCore &core) {
  const cx<T> *tw = reinterpret_cast<const cx<T> *>(core.tw);
  cx<T> *src = buf0, *dst = buf1;
  for (int p = 0; p < core.npass; ++p) {
    const PassDesc &pd = core.pass[p];
    switch (pd.R) {
      case 16: fft_pass<T, 16>(src, dst, rows, pitch, ps, pd, tw); break;
      case 8: fft_pass<T, 8>(src, dst, rows, pitch, ps, pd, tw); break;
      case 4: fft_pass<T, 4>(src, dst, rows, pitch, ps, pd, tw); break;
      case 2: fft_pass<T, 2>(src, dst, rows, pitch, ps, pd, tw); break;
      case 3: fft_pass<T, 3>(src, dst, rows, pitch, ps, pd, tw); break;
      case 5: fft_pass<T, 5>(src, dst, rows, pitch, ps, pd, tw); break;
      case 7: fft_pass<T, 7>(src, dst, rows, pitch, ps, pd, tw); break;
      case 11: fft_pass<T, 11>(src, dst, rows, pitch, ps, pd, tw); break;
      case 13: fft_pass<T, 13>(src, dst, rows, pitch, ps, pd, tw); break;
      default: break;  // the planner only emits the radices above
    }
    cx<T> *t = src;
    src = dst;
    dst = t;
  }
  return src;
}

}  // namespace rg
