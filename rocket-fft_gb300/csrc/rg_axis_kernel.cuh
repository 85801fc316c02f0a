// The axis-job kernel: a batch of 1-D transforms along one axis of a strided array.
//
// One CTA owns TB rows (transforms). Phases, separated by barriers:
//   1. row offsets:  decompose each row number over the batch dims (both sides)
//   2. load:         global -> shared, coalesced either along the axis (rows are long and
//                    contiguous) or across rows (rows are adjacent columns of a strided axis);
//                    op-specific input conversion (real pairs, Hermitian half, chirp, sign)
//   3. pre-op:       e.g. the c2r even-length Hermitian merge
//   4. on-chip FFT:  Stockham radix passes (rg_fft.cuh)
//   5. post-op:      e.g. the r2c even-length split, the Bluestein spectrum product + 2nd FFT
//   6. store:        shared -> global with conjugation, scaling, four-step twiddles
//
// It replaces the reference's per-thread gather -> plan.exec -> scatter loop of general_nd /
// general_r2c / general_c2r (rocket_fft/_pocketfft_hdronly.h:3568-3607, 3723-3852): rows
// processed as SIMD lanes there are processed as CTA rows here.
#pragma once
#include "rg_pdl.cuh"
#include "rg_fft.cuh"

namespace rg {

__device__ __forceinline__ int64_t side_offset(const Side &s, int64_t g) {
  int64_t off = 0;
  for (int d = 0; d < s.nbd; ++d) {
    const int64_t q = g / s.bshape[d];
    off += (g - q * s.bshape[d]) * s.bstride[d];
    g = q;
  }
  return off;
}

// Map loop counter e to (row r, element i) for a row-major walk (i fastest) or a
// column walk (r fastest).
__device__ __forceinline__ void walk(int e, int colmap, int TB, const FastDiv &dTB, int units,
                                     const FastDiv &dUnits, int &r, int &i) {
  if (colmap) {
    i = int(fdiv(uint32_t(e), dTB));
    r = e - i * TB;
  } else {
    r = int(fdiv(uint32_t(e), dUnits));
    i = e - r * units;
  }
}

// W_N^t from the split table: lo[t & mask] * hi[t >> shift]
template <typename T>
__device__ __forceinline__ cx<T> split_twiddle(const cx<T> *__restrict__ lo, const cx<T> *__restrict__ hi,
                                               int shift, uint32_t t) {
  const cx<T> a = lo[t & ((1u << shift) - 1u)];
  const cx<T> b = hi[t >> shift];
  return mul<T>(a, b);
}

// One input unit of an op: a complex element, or for the even-length real transforms the
// real pair (x_2i, x_2i+1) read as one 8/16-byte access when the row is contiguous and aligned.
template <typename T, int OP>
__device__ __forceinline__ cx<T> load_unit(const void *base, int64_t off, int i, int64_t s) {
  if constexpr (OP == OP_R2C_EVEN) {
    const T *in = reinterpret_cast<const T *>(base);
    if (s == 1 && (reinterpret_cast<uintptr_t>(in + off) & (sizeof(cx<T>) - 1)) == 0)
      return __ldg(reinterpret_cast<const cx<T> *>(in + off) + i);
    return mk<T>(__ldg(in + off + 2 * i * s), __ldg(in + off + (2 * i + 1) * s));
  } else if constexpr (OP == OP_R2C_ODD) {
    return mk<T>(__ldg(reinterpret_cast<const T *>(base) + off + i * s), T(0));
  } else {
    return __ldg(reinterpret_cast<const cx<T> *>(base) + off + i * s);
  }
}

template <typename T, int OP>
__global__ void __launch_bounds__(512) axis_kernel(const __grid_constant__ KArgs a, FastDiv dTB,
                                                   FastDiv dIn, FastDiv dOut) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char smraw[];
  const int TB = a.TB;
  const int pitch = a.pitch, ps = a.ps;
  cx<T> *sm = reinterpret_cast<cx<T> *>(smraw);           // ping-pong buffer 0 (loads land here)
  cx<T> *sm1 = sm + size_t(TB) * pitch;                    // ping-pong buffer 1
  int64_t *roff_in = reinterpret_cast<int64_t *>(smraw + 2 * sizeof(cx<T>) * size_t(TB) * pitch);
  int64_t *roff_out = roff_in + TB;
  int *rowaux = reinterpret_cast<int *>(roff_out + TB);

  const int64_t row0 = int64_t(blockIdx.x) * TB;
  const int rows = int(min(int64_t(TB), a.nrows - row0));
  const int tid = threadIdx.x, nth = blockDim.x;
  const bool cin = a.conj_in != 0, cout = a.conj_out != 0;
  const T fct = T(a.fct);
  const T bsc = T(a.bscale);

  for (int r = tid; r < rows; r += nth) {
    roff_in[r] = side_offset(a.ld, row0 + r);
    roff_out[r] = side_offset(a.st, row0 + r);
    if (OP == OP_C2C_TW) rowaux[r] = int((row0 + r) % a.aux_n);
  }
  __syncthreads();

  const int L = a.core.L;

  // ---------------- load ----------------
  // Each thread gathers kBatch independent elements into registers before writing any of
  // them to shared memory, so that kBatch global loads are in flight per thread.
  {
    constexpr int kBatch = 8;
    const int units = a.nin;
    const int total = TB * units;
    const int64_t s = a.ld.axis_stride;
    for (int e0 = tid; e0 < total; e0 += nth * kBatch) {
      cx<T> v[kBatch];
      int rr[kBatch], ii[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * nth;
        rr[u] = -1;
        if (e < total) {
          int r, i;
          walk(e, a.ld.colmap, TB, dTB, units, dIn, r, i);
          if (r < rows) {
            rr[u] = r;
            ii[u] = i;
            if constexpr (OP == OP_DCT2) {
              v[u] = mk<T>(__ldg(reinterpret_cast<const T *>(a.in) + roff_in[r] + i * s), T(0));
            } else if constexpr (OP == OP_DCT3) {
              // (x''_i, x''_{n-i}) with x''_q = x_q (DCT) or x_{n-1-q} (DST); x''_n = 0
              const T *in = reinterpret_cast<const T *>(a.in) + roff_in[r];
              const int n = a.n;
              const bool sine = (a.flags & 2) != 0;
              const int sa = sine ? n - 1 - i : i;
              const T xa = __ldg(in + sa * s);
              const T xb = i == 0 ? T(0) : __ldg(in + (sine ? i - 1 : n - i) * s);
              v[u] = mk<T>(xa, xb);
            } else {
              v[u] = load_unit<T, OP>(a.in, roff_in[r], i, s);
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        if (rr[u] < 0) continue;
        const int r = rr[u], i = ii[u];
        cx<T> x = v[u];
        if constexpr (OP == OP_C2C || OP == OP_C2C_TW) {
          if (cin) x.y = -x.y;
          sm[sidx(r, i, pitch, ps)] = x;
        } else if constexpr (OP == OP_BLUE) {
          // a_j = x_j * conj(bk_j), zero-padded to L below
          if (cin) x.y = -x.y;
          sm[sidx(r, i, pitch, ps)] = mulc<T>(x, reinterpret_cast<const cx<T> *>(a.aux)[i]);
        } else if constexpr (OP == OP_R2C_EVEN || OP == OP_R2C_ODD) {
          sm[sidx(r, i, pitch, ps)] = x;  // (x_2j, x_2j+1) or (x_j, 0)
        } else if constexpr (OP == OP_C2R_EVEN) {
          // units = L+1 Hermitian bins; imaginary parts of bins 0 and L are ignored
          if (cin) x.y = -x.y;
          if (i == 0 || i == L) x.y = T(0);
          else x = scl<T>(x, bsc);
          sm[sidx(r, i, pitch, ps)] = x;
        } else if constexpr (OP == OP_DCT2) {
          // Makhoul order: x_2j -> j, x_2j+1 -> n-1-j; DST: odd inputs negated
          const int n = a.n;
          const int j = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
          if ((a.flags & 2) && (i & 1)) x.x = -x.x;
          sm[sidx(r, j, pitch, ps)] = x;
        } else if constexpr (OP == OP_DCT3) {
          // conj(V_i), V_i = (x''_i - i x''_{n-i}) e^{i pi i / 2n}; input element 0 weighted e0
          const int n = a.n;
          const bool sine = (a.flags & 2) != 0;
          const T e0 = T(a.e0);
          if (sine ? i == n - 1 : i == 0) x.x *= e0;
          if (sine && i == 1) x.y *= e0;
          const cx<T> t = reinterpret_cast<const cx<T> *>(a.aux)[i];  // e^{-i pi i / 2n}
          sm[sidx(r, i, pitch, ps)] = cj<T>(mulc<T>(mk<T>(x.x, -x.y), t));
        } else if constexpr (OP == OP_C2R_ODD) {
          // units = (n+1)/2 bins; build conj of the full Hermitian spectrum:
          //   W_0 = Re X_0, W_i = conj(X_i), W_{n-i} = X_i
          if (cin) x.y = -x.y;
          if (i == 0) {
            sm[sidx(r, 0, pitch, ps)] = mk<T>(x.x, T(0));
          } else {
            x = scl<T>(x, bsc);
            sm[sidx(r, i, pitch, ps)] = cj<T>(x);
            sm[sidx(r, L - i, pitch, ps)] = x;
          }
        }
      }
    }
    if constexpr (OP == OP_BLUE) {
      // zero padding j in [n, L)
      const int n = a.n;
      const int padn = L - n;
      for (int e = tid; e < TB * padn; e += nth) {
        const int r = e / padn;
        const int i = n + (e - r * padn);
        if (r < rows) sm[sidx(r, i, pitch, ps)] = mk<T>(T(0), T(0));
      }
    }
  }
  __syncthreads();

  // ---------------- pre-op ----------------
  if constexpr (OP == OP_C2R_EVEN) {
    // Z_k = A + u, Z_{L-k} = conj(A - u), A = X_k + conj(X_{L-k}), B = X_k - conj(X_{L-k}),
    // u = i * conj(W_n^k) * B; the core then transforms conj(Z).
    const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);  // W_n^k, k = 0..L/2
    const int half = L / 2 + 1;
    for (int e = tid; e < TB * half; e += nth) {
      const int r = e / half;
      const int k = e - r * half;
      if (r >= rows) continue;
      if (k == 0) {
        const cx<T> x0 = sm[sidx(r, 0, pitch, ps)], xl = sm[sidx(r, L, pitch, ps)];
        const cx<T> A = add<T>(x0, cj<T>(xl)), B = sub<T>(x0, cj<T>(xl));
        sm[sidx(r, 0, pitch, ps)] = cj<T>(add<T>(A, mposi<T>(B)));
      } else {
        const int kc = L - k;
        const cx<T> xk = sm[sidx(r, k, pitch, ps)], xc = sm[sidx(r, kc, pitch, ps)];
        const cx<T> A = add<T>(xk, cj<T>(xc)), B = sub<T>(xk, cj<T>(xc));
        const cx<T> u = mposi<T>(mulc<T>(B, w[k]));
        sm[sidx(r, k, pitch, ps)] = cj<T>(add<T>(A, u));
        if (kc != k) sm[sidx(r, kc, pitch, ps)] = sub<T>(A, u);  // conj(conj(A - u))
      }
    }
    __syncthreads();
  }

  // ---------------- FFT ----------------
  cx<T> *res = fft_rows<T>(sm, sm1, rows, pitch, ps, a.core);

  // ---------------- post-op ----------------
  if constexpr (OP == OP_R2C_EVEN) {
    // X_k = E + t, X_{L-k} = conj(E - t), E = (Z_k + conj Z_{L-k})/2, O = (Z_k - conj Z_{L-k})/(2i),
    // t = W_n^k O; X_0 = Re Z_0 + Im Z_0, X_L = Re Z_0 - Im Z_0.
    const cx<T> *w = reinterpret_cast<const cx<T> *>(a.aux);
    const int half = L / 2 + 1;
    for (int e = tid; e < TB * half; e += nth) {
      const int r = e / half;
      const int k = e - r * half;
      if (r >= rows) continue;
      if (k == 0) {
        const cx<T> z0 = res[sidx(r, 0, pitch, ps)];
        res[sidx(r, 0, pitch, ps)] = mk<T>(z0.x + z0.y, T(0));
        res[sidx(r, L, pitch, ps)] = mk<T>(z0.x - z0.y, T(0));
      } else {
        const int kc = L - k;
        const cx<T> zk = res[sidx(r, k, pitch, ps)], zc = cj<T>(res[sidx(r, kc, pitch, ps)]);
        const cx<T> E = scl<T>(add<T>(zk, zc), T(0.5));
        const cx<T> O = mnegi<T>(scl<T>(sub<T>(zk, zc), T(0.5)));
        const cx<T> t = mul<T>(w[k], O);
        res[sidx(r, k, pitch, ps)] = add<T>(E, t);
        if (kc != k) res[sidx(r, kc, pitch, ps)] = cj<T>(sub<T>(E, t));
      }
    }
    __syncthreads();
  } else if constexpr (OP == OP_BLUE) {
    // C = conj(A * bkf); then forward FFT again gives conj(conv)
    const cx<T> *bkf = reinterpret_cast<const cx<T> *>(a.aux2);
    for (int e = tid; e < TB * L; e += nth) {
      const int r = e / L;
      const int i = e - r * L;
      if (r >= rows) continue;
      const int si = sidx(r, i, pitch, ps);
      res[si] = cj<T>(mul<T>(res[si], bkf[i]));
    }
    __syncthreads();
    res = fft_rows<T>(res, res == sm ? sm1 : sm, rows, pitch, ps, a.core);
  }

  // ---------------- store ----------------
  {
    constexpr int kBatch = 8;
    const int units = a.nout;
    const int total = TB * units;
    const int64_t s = a.st.axis_stride;
    for (int e0 = tid; e0 < total; e0 += nth * kBatch) {
      cx<T> v[kBatch];
      int rr[kBatch], ii[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int e = e0 + u * nth;
        rr[u] = -1;
        if (e < total) {
          int r, i;
          walk(e, a.st.colmap, TB, dTB, units, dOut, r, i);
          if (r < rows) {
            rr[u] = r;
            ii[u] = i;
            if constexpr (OP == OP_DCT2) {
              // y_k = 2 Re(e^{-i pi k'/2n} V_k'), k' = k (DCT) or n-1-k (DST); element 0 weighted
              const int n = a.n;
              const int kk = (a.flags & 2) ? n - 1 - i : i;
              const cx<T> V = res[sidx(r, kk, pitch, ps)];
              const cx<T> t = reinterpret_cast<const cx<T> *>(a.aux)[kk];
              T y = T(2) * (V.x * t.x - V.y * t.y) * fct;
              if (i == 0) y *= T(a.e0);
              v[u] = mk<T>(y, T(0));
              continue;
            } else if constexpr (OP == OP_DCT3) {
              // y_2j = Re v_j, y_2j+1 = Re v_{n-1-j}; DST: odd outputs negated
              const int n = a.n;
              const int j = (i & 1) ? n - 1 - (i >> 1) : (i >> 1);
              T y = res[sidx(r, j, pitch, ps)].x * fct;
              if ((a.flags & 2) && (i & 1)) y = -y;
              v[u] = mk<T>(y, T(0));
              continue;
            }
            cx<T> x = res[sidx(r, i, pitch, ps)];
            if constexpr (OP == OP_C2C_TW) {
              x = mul<T>(x, split_twiddle<T>(reinterpret_cast<const cx<T> *>(a.aux),
                                             reinterpret_cast<const cx<T> *>(a.aux2), a.aux_s,
                                             uint32_t(rowaux[r]) * uint32_t(i)));
            } else if constexpr (OP == OP_BLUE) {
              // y = conj(F) * conj(bk) = conj(F * bk)
              x = cj<T>(mul<T>(x, reinterpret_cast<const cx<T> *>(a.aux)[i]));
            } else if constexpr (OP == OP_R2C_ODD) {
              if (i == 0) x.y = T(0);
              else x = scl<T>(x, bsc);
            } else if constexpr (OP == OP_R2C_EVEN) {
              if (i != 0 && i != L) x = scl<T>(x, bsc);
            } else if constexpr (OP == OP_C2R_EVEN) {
              x.y = -x.y;  // (x_2i, x_2i+1) = (Re F_i, -Im F_i)
            }
            if constexpr (OP == OP_C2R_EVEN || OP == OP_C2R_ODD) {
              v[u] = mk<T>(x.x * fct, x.y * fct);
            } else {
              v[u] = mk<T>(x.x * fct, (cout ? -x.y : x.y) * fct);
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        if (rr[u] < 0) continue;
        const int64_t off = roff_out[rr[u]];
        const int i = ii[u];
        if constexpr (OP == OP_C2R_EVEN) {
          T *out = reinterpret_cast<T *>(a.out);
          if (s == 1 && (reinterpret_cast<uintptr_t>(out + off) & (sizeof(cx<T>) - 1)) == 0) {
            reinterpret_cast<cx<T> *>(out + off)[i] = v[u];
          } else {
            out[off + 2 * i * s] = v[u].x;
            out[off + (2 * i + 1) * s] = v[u].y;
          }
        } else if constexpr (OP == OP_C2R_ODD || OP == OP_DCT2 || OP == OP_DCT3) {
          reinterpret_cast<T *>(a.out)[off + i * s] = v[u].x;
        } else {
          reinterpret_cast<cx<T> *>(a.out)[off + i * s] = v[u];
        }
      }
    }
  }
}

}  // namespace rg
