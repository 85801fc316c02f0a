// Test infrastructure only: not part of the product.
//
// CPU restatement of the reference's pocketfft transform path (rocket-fft 0.3.1,
// rocket_fft/_pocketfft_hdronly.h = "HDR", rocket_fft/_pocketfft_numba.cpp = "SHIM"), used as
// the oracle where the reference itself cannot run (the GPU host has no reference tree), and
// as the timed CPU baseline there. Exported functions mirror SHIM's ten entry points
// (prefix `port_`, int status instead of void).
//
// What follows the reference step by step (cited per function): the size utilities
// (good_size, largest_prime_factor, cost_guess), the packed-vs-Bluestein decision, the
// Bluestein construction, the FFTPACK half-complex layout, the DCT/DST reductions, fct
// placement, the N-d axis loop and the Hermitian fills of c2c_sym / genuine Hartley.
// What differs: the complex radix passes are a Stockham formulation (radix 4, 2, 3, 5 and a
// generic odd radix) instead of FFTPACK's pass2..pass11/passg, and the real transform is a
// half-length complex FFT plus a split instead of rfftp's radf/radb passes. Those produce
// the same transforms up to rounding.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <tuple>
#include <vector>

namespace port {

using u64 = uint64_t;
using i64 = int64_t;

template <class T> struct C {
  T r, i;
};
template <class T> inline C<T> operator+(C<T> a, C<T> b) { return {a.r + b.r, a.i + b.i}; }
template <class T> inline C<T> operator-(C<T> a, C<T> b) { return {a.r - b.r, a.i - b.i}; }
template <class T> inline C<T> operator*(C<T> a, C<T> b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
template <class T> inline C<T> operator*(C<T> a, T s) { return {a.r * s, a.i * s}; }
template <class T> inline C<T> conj(C<T> a) { return {a.r, -a.i}; }
// multiply by conj(b) when `cj`
template <class T> inline C<T> mulx(C<T> a, C<T> b, bool cj) { return cj ? a * conj(b) : a * b; }

// ---------------------------------------------------------------------------------------
// size utilities (HDR:546-650)
// ---------------------------------------------------------------------------------------

// Smallest number >= n that is 2^a * (product of `odd`): enumerate the odd part, lift by 2.
static u64 smooth_ceil(u64 n, std::initializer_list<u64> odd) {
  u64 best = 1;
  while (best < n) best <<= 1;
  std::vector<u64> primes(odd);
  std::vector<std::pair<u64, size_t>> todo{{1, 0}};
  while (!todo.empty()) {
    auto [v, first] = todo.back();
    todo.pop_back();
    u64 x = v;
    while (x < n) x *= 2;
    best = std::min(best, x);
    for (size_t p = first; p < primes.size(); ++p)
      if (v <= best / primes[p]) todo.push_back({v * primes[p], p});
  }
  return best;
}
u64 good_size_cmplx(u64 n) { return n <= 12 ? n : smooth_ceil(n, {3, 5, 7, 11}); }  // HDR:589-619
u64 good_size_real(u64 n) { return n <= 6 ? n : smooth_ceil(n, {3, 5}); }             // HDR:622-650

u64 largest_prime_factor(u64 n) {  // HDR:548-565
  u64 res = 1;
  while ((n & 1) == 0) {
    res = 2;
    n >>= 1;
  }
  for (u64 x = 3; x * x <= n; x += 2)
    while (n % x == 0) {
      res = x;
      n /= x;
    }
  return n > 1 ? n : res;
}

double cost_guess(u64 n) {  // HDR:567-586: sum of factors, larger primes penalised by 1.1
  const double lfp = 1.1;
  const u64 ni = n;
  double result = 0.;
  while ((n & 1) == 0) {
    result += 2;
    n >>= 1;
  }
  for (u64 x = 3; x * x <= n; x += 2)
    while (n % x == 0) {
      result += (x <= 5) ? double(x) : lfp * double(x);
      n /= x;
    }
  if (n > 1) result += (n <= 5) ? double(n) : lfp * double(n);
  return result * double(ni);
}

// e^{+2 pi i t / N} in double: integer octant reduction, then cos/sin of an angle <= pi/4.
static void root(u64 t, u64 N, double &c, double &s) {
  t %= N;
  const unsigned __int128 t8 = (unsigned __int128)t * 8;
  const u64 oct = u64(t8 / N);
  const u64 rem = u64(t8 % N);
  const double q = 0.78539816339744830962 * (double((oct & 1) ? N - rem : rem) / double(N));
  double a = std::cos(q), b = std::sin(q);
  if (oct & 1) std::swap(a, b);
  switch (oct >> 1) {
    case 0: c = a; s = b; break;
    case 1: c = -b; s = a; break;
    case 2: c = -a; s = -b; break;
    default: c = b; s = -a; break;
  }
}
template <class T> static C<T> unit(u64 t, u64 N) {  // e^{+2 pi i t/N}
  double c, s;
  root(t, N, c, s);
  return {T(c), T(s)};
}

// ---------------------------------------------------------------------------------------
// packed complex FFT (role of cfftp, HDR:1060-1830): Stockham passes
// ---------------------------------------------------------------------------------------

template <class T> class CPack {
 public:
  explicit CPack(u64 n) : n_(n) {
    if (n == 0) throw std::runtime_error("zero-length FFT requested");
    u64 len = n;
    while (len % 4 == 0) {
      fac_.push_back(4);
      len /= 4;
    }
    if (len % 2 == 0) {
      fac_.insert(fac_.begin(), 2);
      len /= 2;
    }
    for (u64 d = 3; d * d <= len; d += 2)
      while (len % d == 0) {
        fac_.push_back(d);
        len /= d;
      }
    if (len > 1) fac_.push_back(len);
    u64 ns = 1;
    for (u64 R : fac_) {
      off_.push_back(tw_.size());
      for (u64 k = 1; k < R; ++k)
        for (u64 m = 0; m < ns; ++m) tw_.push_back(unit<T>(m * k, ns * R));  // e^{+}
      if (R > 5) {
        roots_off_.push_back(rt_.size());
        for (u64 t = 0; t < R; ++t) rt_.push_back(unit<T>(t, R));
      } else {
        roots_off_.push_back(0);
      }
      ns *= R;
    }
  }
  u64 length() const { return n_; }

  // forward: exponent -2 pi i (pocketfft's fwd=true); scale by fct at the end
  void exec(C<T> *c, T fct, bool fwd) const {
    if (n_ == 1) {
      c[0] = c[0] * fct;
      return;
    }
    std::vector<C<T>> buf(n_);
    C<T> *a = c, *b = buf.data();
    u64 ns = 1;
    for (size_t p = 0; p < fac_.size(); ++p) {
      pass(fac_[p], ns, a, b, tw_.data() + off_[p], rt_.data() + roots_off_[p], fwd);
      std::swap(a, b);
      ns *= fac_[p];
    }
    if (a != c) {
      for (u64 i = 0; i < n_; ++i) c[i] = a[i] * fct;
    } else if (fct != T(1)) {
      for (u64 i = 0; i < n_; ++i) c[i] = c[i] * fct;
    }
  }

 private:
  void pass(u64 R, u64 ns, const C<T> *x, C<T> *y, const C<T> *tw, const C<T> *rt, bool fwd) const {
    const u64 L = n_ / R;
    const bool cj = fwd;  // forward uses conj(e^{+}) = e^{-}
    C<T> v[64];
    std::vector<C<T>> vb;
    C<T> *vv = v;
    if (R > 64) {
      vb.resize(2 * R);
      vv = vb.data();
    }
    for (u64 b0 = 0; b0 < L; b0 += ns) {
      for (u64 m = 0; m < ns; ++m) {
        const u64 j = b0 + m;
        for (u64 k = 0; k < R; ++k) vv[k] = x[j + k * L];
        if (ns > 1)
          for (u64 k = 1; k < R; ++k) vv[k] = mulx(vv[k], tw[(k - 1) * ns + m], cj);
        C<T> *out = y + b0 * R + m;
        switch (R) {
          case 2: {
            out[0] = vv[0] + vv[1];
            out[ns] = vv[0] - vv[1];
            break;
          }
          case 4: {
            const C<T> t0 = vv[0] + vv[2], t1 = vv[0] - vv[2], t2 = vv[1] + vv[3];
            C<T> t3 = vv[1] - vv[3];
            t3 = fwd ? C<T>{t3.i, -t3.r} : C<T>{-t3.i, t3.r};  // * (-i) or * (+i)
            out[0] = t0 + t2;
            out[2 * ns] = t0 - t2;
            out[ns] = t1 + t3;
            out[3 * ns] = t1 - t3;
            break;
          }
          case 3: {
            const T c1 = T(-0.5), s1 = T(fwd ? -0.86602540378443864676 : 0.86602540378443864676);
            const C<T> s = vv[1] + vv[2], d = vv[1] - vv[2];
            const C<T> a = vv[0] + s * c1;
            const C<T> b = {-d.i * s1, d.r * s1};  // i * s1 * d
            out[0] = vv[0] + s;
            out[ns] = a + b;
            out[2 * ns] = a - b;
            break;
          }
          case 5: {
            const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);
            const T sg = fwd ? T(-1) : T(1);
            const T s1 = sg * T(0.95105651629515357212), s2 = sg * T(0.58778525229247312917);
            const C<T> sa = vv[1] + vv[4], da = vv[1] - vv[4], sb = vv[2] + vv[3], db = vv[2] - vv[3];
            const C<T> a1 = vv[0] + sa * c1 + sb * c2, a2 = vv[0] + sa * c2 + sb * c1;
            const C<T> e1 = da * s1 + db * s2, e2 = da * s2 - db * s1;
            const C<T> b1 = {-e1.i, e1.r}, b2 = {-e2.i, e2.r};
            out[0] = vv[0] + sa + sb;
            out[ns] = a1 + b1;
            out[4 * ns] = a1 - b1;
            out[2 * ns] = a2 + b2;
            out[3 * ns] = a2 - b2;
            break;
          }
          default: {  // generic radix: y_q = sum_k v_k w^{qk}
            for (u64 q = 0; q < R; ++q) {
              C<T> acc = vv[0];
              u64 e = 0;
              for (u64 k = 1; k < R; ++k) {
                e += q;
                if (e >= R) e -= R;
                acc = acc + mulx(vv[k], rt[e], cj);
              }
              out[q * ns] = acc;
            }
          }
        }
      }
    }
  }

  u64 n_;
  std::vector<u64> fac_;
  std::vector<size_t> off_, roots_off_;
  std::vector<C<T>> tw_, rt_;
};

// ---------------------------------------------------------------------------------------
// Bluestein (restates fftblue, HDR:2723-2828)
// ---------------------------------------------------------------------------------------

template <class T> class Blue {
 public:
  explicit Blue(u64 n) : n_(n), n2_(good_size_cmplx(2 * n - 1)), plan_(n2_), bk_(n), bkf_(n2_) {
    // bk[m] = e^{+i pi m^2 / n}, the exponent accumulated modulo 2n (HDR:2773-2780)
    bk_[0] = {T(1), T(0)};
    u64 coeff = 0;
    for (u64 m = 1; m < n; ++m) {
      coeff += 2 * m - 1;
      if (coeff >= 2 * n) coeff -= 2 * n;
      bk_[m] = unit<T>(coeff, 2 * n);
    }
    // zero-padded, symmetric, normalised, transformed (HDR:2783-2792)
    std::vector<C<T>> t(n2_, C<T>{T(0), T(0)});
    const T xn2 = T(1) / T(n2_);
    t[0] = bk_[0] * xn2;
    for (u64 m = 1; m < n; ++m) t[m] = t[n2_ - m] = bk_[m] * xn2;
    plan_.exec(t.data(), T(1), true);
    bkf_ = t;
  }
  u64 length() const { return n_; }

  void exec(C<T> *c, T fct, bool fwd) const {  // HDR:2732-2762
    std::vector<C<T>> a(n2_, C<T>{T(0), T(0)});
    for (u64 m = 0; m < n_; ++m) a[m] = mulx(c[m], bk_[m], fwd);
    plan_.exec(a.data(), T(1), true);
    for (u64 m = 0; m < n2_; ++m) a[m] = mulx(a[m], bkf_[m], !fwd);
    plan_.exec(a.data(), T(1), false);
    for (u64 m = 0; m < n_; ++m) c[m] = mulx(a[m], bk_[m], fwd) * fct;
  }

 private:
  u64 n_, n2_;
  CPack<T> plan_;
  std::vector<C<T>> bk_, bkf_;
};

// decision of pocketfft_c / pocketfft_r (HDR:2843-2861, 2885-2903)
static bool use_bluestein(u64 n, double factor) {
  const u64 tmp = (n < 50) ? 0 : largest_prime_factor(n);
  if (tmp * tmp <= n) return false;
  const double comp1 = factor * cost_guess(n);
  const double comp2 = 2 * cost_guess(good_size_cmplx(2 * n - 1)) * 1.5;
  return comp2 < comp1;
}

template <class T> class CPlan {
 public:
  explicit CPlan(u64 n) : n_(n) {
    if (n == 0) throw std::runtime_error("zero-length FFT requested");
    if (use_bluestein(n, 1.0))
      blue_.reset(new Blue<T>(n));
    else
      pack_.reset(new CPack<T>(n));
  }
  u64 length() const { return n_; }
  void exec(C<T> *c, T fct, bool fwd) const { pack_ ? pack_->exec(c, fct, fwd) : blue_->exec(c, fct, fwd); }

 private:
  u64 n_;
  std::unique_ptr<CPack<T>> pack_;
  std::unique_ptr<Blue<T>> blue_;
};

// ---------------------------------------------------------------------------------------
// real FFT in FFTPACK half-complex order (role of rfftp/pocketfft_r, HDR:1836-2717, 2876-2912)
//   r2hc:  [x_0..x_{n-1}] -> [X0.r, X1.r, X1.i, X2.r, X2.i, ..., (X_{n/2}.r if n even)]
//   hc2r:  the reverse direction, unnormalised (x_j = sum_k X_k e^{+2 pi i jk/n})
// ---------------------------------------------------------------------------------------

template <class T> class RPlan {
 public:
  explicit RPlan(u64 n) : n_(n) {
    if (n == 0) throw std::runtime_error("zero-length FFT requested");
    if (n % 2 == 0 && !use_bluestein(n, 0.5)) {
      half_.reset(new CPlan<T>(n / 2));
      for (u64 k = 0; k <= n / 2; ++k) w_.push_back(unit<T>(k, n));  // e^{+2 pi i k/n}
    } else {
      full_.reset(new CPlan<T>(n));
    }
  }
  u64 length() const { return n_; }

  void exec(T *c, T fct, bool r2hc) const {
    const u64 n = n_;
    if (n == 1) {
      c[0] *= fct;
      return;
    }
    if (full_) {
      std::vector<C<T>> z(n);
      if (r2hc) {
        for (u64 j = 0; j < n; ++j) z[j] = {c[j], T(0)};
        full_->exec(z.data(), fct, true);
        pack(z.data(), c);
      } else {
        unpack_full(c, z.data());
        full_->exec(z.data(), fct, false);
        for (u64 j = 0; j < n; ++j) c[j] = z[j].r;
      }
      return;
    }
    const u64 L = n / 2;
    std::vector<C<T>> z(L + 1);
    if (r2hc) {
      for (u64 j = 0; j < L; ++j) z[j] = {c[2 * j], c[2 * j + 1]};
      half_->exec(z.data(), T(1), true);
      // split: X_k = E + W^k O, E = (Z_k + conj Z_{L-k})/2, O = (Z_k - conj Z_{L-k})/(2i)
      std::vector<C<T>> X(L + 1);
      X[0] = {z[0].r + z[0].i, T(0)};
      X[L] = {z[0].r - z[0].i, T(0)};
      for (u64 k = 1; k <= L / 2; ++k) {
        const C<T> a = z[k], b = conj(z[L - k]);
        const C<T> E = (a + b) * T(0.5);
        const C<T> d = (a - b) * T(0.5);
        const C<T> O = {d.i, -d.r};
        const C<T> t = O * conj(w_[k]);  // W_n^k = e^{-2 pi i k/n}
        X[k] = E + t;
        X[L - k] = conj(E - t);
      }
      for (u64 k = 0; k <= L; ++k) X[k] = X[k] * fct;
      pack(X.data(), c);
    } else {
      std::vector<C<T>> X(L + 1);
      X[0] = {c[0], T(0)};
      for (u64 k = 1; k < L; ++k) X[k] = {c[2 * k - 1], c[2 * k]};
      X[L] = {c[n - 1], T(0)};
      // merge: Z_k = A + u, A = X_k + conj X_{L-k}, u = i conj(W^k) (X_k - conj X_{L-k})
      for (u64 k = 0; k < L; ++k) {
        const C<T> xk = X[k], xc = conj(X[L - k]);
        const C<T> A = xk + xc, B = xk - xc;
        const C<T> t = B * w_[k];  // conj(W_n^k) = e^{+2 pi i k/n}
        z[k] = A + C<T>{-t.i, t.r};
      }
      half_->exec(z.data(), fct, false);
      for (u64 j = 0; j < L; ++j) {
        c[2 * j] = z[j].r;
        c[2 * j + 1] = z[j].i;
      }
    }
  }

 private:
  void pack(const C<T> *X, T *c) const {
    c[0] = X[0].r;
    u64 i = 1, k = 1;
    for (; i + 1 < n_; i += 2, ++k) {
      c[i] = X[k].r;
      c[i + 1] = X[k].i;
    }
    if (i < n_) c[i] = X[k].r;
  }
  void unpack_full(const T *c, C<T> *z) const {
    const u64 n = n_;
    z[0] = {c[0], T(0)};
    u64 i = 1, k = 1;
    for (; i + 1 < n; i += 2, ++k) {
      z[k] = {c[i], c[i + 1]};
      z[n - k] = {c[i], -c[i + 1]};
    }
    if (i < n) z[k] = {c[i], T(0)};
  }

  u64 n_;
  std::unique_ptr<CPlan<T>> half_, full_;
  std::vector<C<T>> w_;
};

// ---------------------------------------------------------------------------------------
// sine/cosine transforms (restate T_dct1, T_dst1, T_dcst23, T_dcst4; HDR:2918-3163)
// ---------------------------------------------------------------------------------------

constexpr double kSqrt2 = 1.414213562373095048801688724209698;

template <class T> class Dct1 {  // HDR:2918-2955: rfft of the even extension, length 2(n-1)
 public:
  explicit Dct1(u64 n) : fft_(2 * (n - 1)) {}
  u64 length() const { return fft_.length() / 2 + 1; }
  void exec(T *c, T fct, bool ortho, int, bool) const {
    const u64 N = fft_.length(), n = N / 2 + 1;
    const T s2 = T(kSqrt2);
    if (ortho) {
      c[0] *= s2;
      c[n - 1] *= s2;
    }
    std::vector<T> t(N);
    t[0] = c[0];
    for (u64 i = 1; i < n; ++i) t[i] = t[N - i] = c[i];
    fft_.exec(t.data(), fct, true);
    c[0] = t[0];
    for (u64 i = 1; i < n; ++i) c[i] = t[2 * i - 1];
    if (ortho) {
      c[0] *= s2 * T(0.5);
      c[n - 1] *= s2 * T(0.5);
    }
  }

 private:
  RPlan<T> fft_;
};

template <class T> class Dst1 {  // HDR:2957-2985: rfft of the odd extension, length 2(n+1)
 public:
  explicit Dst1(u64 n) : fft_(2 * (n + 1)) {}
  u64 length() const { return fft_.length() / 2 - 1; }
  void exec(T *c, T fct, bool, int, bool) const {
    const u64 N = fft_.length(), n = N / 2 - 1;
    std::vector<T> t(N);
    t[0] = t[n + 1] = c[0] * T(0);
    for (u64 i = 0; i < n; ++i) {
      t[i + 1] = c[i];
      t[N - 1 - i] = -c[i];
    }
    fft_.exec(t.data(), fct, true);
    for (u64 i = 0; i < n; ++i) c[i] = -t[2 * i + 2];
  }

 private:
  RPlan<T> fft_;
};

template <class T> class Dcst23 {  // HDR:2987-3061
 public:
  explicit Dcst23(u64 n) : fft_(n), tw_(n) {
    for (u64 i = 0; i < n; ++i) tw_[i] = unit<T>(i + 1, 4 * n).r;  // cos(2 pi (i+1) / 4n)
  }
  u64 length() const { return fft_.length(); }
  void exec(T *c, T fct, bool ortho, int type, bool cosine) const {
    const u64 N = length(), NS2 = (N + 1) / 2;
    const T s2 = T(kSqrt2);
    if (type == 2) {
      if (!cosine)
        for (u64 k = 1; k < N; k += 2) c[k] = -c[k];
      c[0] *= 2;
      if ((N & 1) == 0) c[N - 1] *= 2;
      for (u64 k = 1; k + 1 < N; k += 2) {  // MPINPLACE(c[k+1], c[k]): (a, b) <- (a-b, a+b)
        const T a = c[k + 1], b = c[k];
        c[k + 1] = a - b;
        c[k] = a + b;
      }
      fft_.exec(c, fct, false);
      for (u64 k = 1, kc = N - 1; k < NS2; ++k, --kc) {
        const T t1 = tw_[k - 1] * c[kc] + tw_[kc - 1] * c[k];
        const T t2 = tw_[k - 1] * c[k] - tw_[kc - 1] * c[kc];
        c[k] = T(0.5) * (t1 + t2);
        c[kc] = T(0.5) * (t1 - t2);
      }
      if ((N & 1) == 0) c[NS2] *= tw_[NS2 - 1];
      if (!cosine)
        for (u64 k = 0, kc = N - 1; k < kc; ++k, --kc) std::swap(c[k], c[kc]);
      if (ortho) c[0] *= s2 * T(0.5);
    } else {
      if (ortho) c[0] *= s2;
      if (!cosine)
        for (u64 k = 0, kc = N - 1; k < NS2; ++k, --kc) std::swap(c[k], c[kc]);
      for (u64 k = 1, kc = N - 1; k < NS2; ++k, --kc) {
        const T t1 = c[k] + c[kc], t2 = c[k] - c[kc];
        c[k] = tw_[k - 1] * t2 + tw_[kc - 1] * t1;
        c[kc] = tw_[k - 1] * t1 - tw_[kc - 1] * t2;
      }
      if ((N & 1) == 0) c[NS2] *= 2 * tw_[NS2 - 1];
      fft_.exec(c, fct, true);
      for (u64 k = 1; k + 1 < N; k += 2) {  // MPINPLACE(c[k], c[k+1]): (a, b) <- (a-b, a+b)
        const T a = c[k], b = c[k + 1];
        c[k] = a - b;
        c[k + 1] = a + b;
      }
      if (!cosine)
        for (u64 k = 1; k < N; k += 2) c[k] = -c[k];
    }
  }

 private:
  RPlan<T> fft_;
  std::vector<T> tw_;
};

template <class T> class Dcst4 {  // HDR:3063-3163
 public:
  explicit Dcst4(u64 n) : N_(n) {
    if (n & 1) {
      rfft_.reset(new RPlan<T>(n));
    } else {
      fft_.reset(new CPlan<T>(n / 2));
      for (u64 i = 0; i < n / 2; ++i) C2_.push_back(conj(unit<T>(8 * i + 1, 16 * n)));
    }
  }
  u64 length() const { return N_; }
  void exec(T *c, T fct, bool, int, bool cosine) const {
    const u64 N = N_, n2 = N / 2;
    if (!cosine)
      for (u64 k = 0, kc = N - 1; k < n2; ++k, --kc) std::swap(c[k], c[kc]);
    if (N & 1) {
      // odd length: the index shuffle and sign pattern of the reference (derived there from
      // FFTW's apply_re11) around a real FFT of length N
      std::vector<T> y(N);
      {
        u64 i = 0, m = n2;
        for (; m < N; ++i, m += 4) y[i] = c[m];
        for (; m < 2 * N; ++i, m += 4) y[i] = -c[2 * N - m - 1];
        for (; m < 3 * N; ++i, m += 4) y[i] = -c[m - 2 * N];
        for (; m < 4 * N; ++i, m += 4) y[i] = c[4 * N - m - 1];
        for (; i < N; ++i, m += 4) y[i] = c[m - 4 * N];
      }
      rfft_->exec(y.data(), fct, true);
      auto sgn = [](u64 i) { return (i & 2) ? -T(kSqrt2) : T(kSqrt2); };
      c[n2] = y[0] * sgn(n2 + 1);
      u64 i = 0, i1 = 1, k = 1;
      for (; k < n2; ++i, ++i1, k += 2) {
        c[i] = y[2 * k - 1] * sgn(i1) + y[2 * k] * sgn(i);
        c[N - i1] = y[2 * k - 1] * sgn(N - i) - y[2 * k] * sgn(N - i1);
        c[n2 - i1] = y[2 * k + 1] * sgn(n2 - i) - y[2 * k + 2] * sgn(n2 - i1);
        c[n2 + i1] = y[2 * k + 1] * sgn(n2 + i + 2) + y[2 * k + 2] * sgn(n2 + i1);
      }
      if (k == n2) {
        c[i] = y[2 * k - 1] * sgn(i + 1) + y[2 * k] * sgn(i);
        c[N - i1] = y[2 * k - 1] * sgn(i + 2) + y[2 * k] * sgn(i1);
      }
    } else {
      // even length: half-length complex FFT between two twiddle multiplies
      std::vector<C<T>> y(n2);
      for (u64 i = 0; i < n2; ++i) y[i] = C<T>{c[2 * i], c[N - 1 - i * 2]} * C2_[i];
      fft_->exec(y.data(), fct, true);
      for (u64 i = 0, ic = n2 - 1; i < n2; ++i, --ic) {
        c[2 * i] = 2 * (y[i].r * C2_[i].r - y[i].i * C2_[i].i);
        c[2 * i + 1] = -2 * (y[ic].i * C2_[ic].r + y[ic].r * C2_[ic].i);
      }
    }
    if (!cosine)
      for (u64 k = 1; k < N; k += 2) c[k] = -c[k];
  }

 private:
  u64 N_;
  std::unique_ptr<CPlan<T>> fft_;
  std::unique_ptr<RPlan<T>> rfft_;
  std::vector<C<T>> C2_;
};

// ---------------------------------------------------------------------------------------
// plan cache (role of get_plan, HDR:3169-3223; unbounded, mutex-protected)
// ---------------------------------------------------------------------------------------

template <class P> std::shared_ptr<P> get_plan(u64 n) {
  static std::mutex mu;
  static std::map<u64, std::shared_ptr<P>> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(n);
  if (it != cache.end()) return it->second;
  auto p = std::make_shared<P>(n);
  cache.emplace(n, p);
  return p;
}

// ---------------------------------------------------------------------------------------
// N-d iteration (role of multi_iter / general_nd, HDR:3272-3353, 3568-3607)
// ---------------------------------------------------------------------------------------

struct View {
  char *d;
  std::vector<i64> shape, stride;  // byte strides
};

// thread count rule of util::thread_count (HDR:712-723)
static u64 thread_count(u64 nthreads, const std::vector<i64> &shape, size_t axis) {
  if (nthreads == 1) return 1;
  u64 size = 1;
  for (i64 s : shape) size *= u64(s);
  u64 parallel = size / u64(shape[axis]);
  if (shape[axis] < 1000) parallel /= 4;
  const u64 mx = nthreads == 0 ? std::max(1u, std::thread::hardware_concurrency()) : nthreads;
  return std::max<u64>(1, std::min(parallel, mx));
}

// Calls f(in_offset, out_offset) for every row along `axis` (C order of the other dims),
// spreading rows over threads.
template <class F>
static void for_rows(const std::vector<i64> &shape, const std::vector<i64> &sin, const std::vector<i64> &sout,
                     size_t axis, u64 nthreads, F f) {
  const size_t nd = shape.size();
  u64 rows = 1;
  for (size_t d = 0; d < nd; ++d)
    if (d != axis) rows *= u64(shape[d]);
  const u64 nt = thread_count(nthreads, shape, axis);
  auto work = [&](u64 lo, u64 hi) {
    for (u64 r = lo; r < hi; ++r) {
      u64 rem = r;
      i64 oi = 0, oo = 0;
      for (size_t dd = nd; dd-- > 0;) {
        if (dd == axis) continue;
        const u64 pos = rem % u64(shape[dd]);
        rem /= u64(shape[dd]);
        oi += i64(pos) * sin[dd];
        oo += i64(pos) * sout[dd];
      }
      f(oi, oo);
    }
  };
  if (nt <= 1) {
    work(0, rows);
    return;
  }
  std::vector<std::thread> th;
  for (u64 t = 0; t < nt; ++t) {
    const u64 lo = rows * t / nt, hi = rows * (t + 1) / nt;
    th.emplace_back(work, lo, hi);
  }
  for (auto &x : th) x.join();
}

static bool any_zero(const std::vector<i64> &s) {
  for (i64 v : s)
    if (v == 0) return true;
  return false;
}

template <class T>
static void c2c_nd(const View &in, const View &out, const std::vector<u64> &axes, bool fwd, T fct, u64 nth) {
  if (any_zero(in.shape)) return;
  for (size_t k = 0; k < axes.size(); ++k) {
    const View &src = k == 0 ? in : out;
    const size_t ax = axes[k];
    const u64 n = u64(in.shape[ax]);
    auto plan = get_plan<CPlan<T>>(n);
    const i64 si = src.stride[ax], so = out.stride[ax];
    const T f = k == 0 ? fct : T(1);
    for_rows(in.shape, src.stride, out.stride, ax, nth, [&](i64 oi, i64 oo) {
      std::vector<C<T>> buf(n);
      for (u64 j = 0; j < n; ++j) {
        const T *p = reinterpret_cast<const T *>(src.d + oi + i64(j) * si);
        buf[j] = {p[0], p[1]};
      }
      plan->exec(buf.data(), f, fwd);
      for (u64 j = 0; j < n; ++j) {
        T *p = reinterpret_cast<T *>(out.d + oo + i64(j) * so);
        p[0] = buf[j].r;
        p[1] = buf[j].i;
      }
    });
  }
}

// general_r2c (HDR:3723-3779): halfcomplex to complex, conjugated when !forward
template <class T>
static void r2c_axis(const View &in, const View &out, size_t ax, bool fwd, T fct, u64 nth) {
  const u64 n = u64(in.shape[ax]);
  auto plan = get_plan<RPlan<T>>(n);
  const i64 si = in.stride[ax], so = out.stride[ax];
  for_rows(in.shape, in.stride, out.stride, ax, nth, [&](i64 oi, i64 oo) {
    std::vector<T> t(n);
    for (u64 j = 0; j < n; ++j) t[j] = *reinterpret_cast<const T *>(in.d + oi + i64(j) * si);
    plan->exec(t.data(), fct, true);
    auto put = [&](u64 k, T re, T im) {
      T *p = reinterpret_cast<T *>(out.d + oo + i64(k) * so);
      p[0] = re;
      p[1] = fwd ? im : -im;
    };
    put(0, t[0], T(0));
    u64 i = 1, k = 1;
    for (; i + 1 < n; i += 2, ++k) put(k, t[i], t[i + 1]);
    if (i < n) put(k, t[i], T(0));
  });
}

// general_c2r (HDR:3780-3852): imaginary parts negated when forward
template <class T>
static void c2r_axis(const View &in, const View &out, size_t ax, bool fwd, T fct, u64 nth) {
  const u64 n = u64(out.shape[ax]);
  auto plan = get_plan<RPlan<T>>(n);
  const i64 si = in.stride[ax], so = out.stride[ax];
  for_rows(out.shape, in.stride, out.stride, ax, nth, [&](i64 oi, i64 oo) {
    std::vector<T> t(n);
    auto get = [&](u64 k) { return reinterpret_cast<const T *>(in.d + oi + i64(k) * si); };
    t[0] = get(0)[0];
    u64 i = 1, k = 1;
    for (; i + 1 < n; i += 2, ++k) {
      t[i] = get(k)[0];
      t[i + 1] = fwd ? -get(k)[1] : get(k)[1];
    }
    if (i < n) t[i] = get(k)[0];
    plan->exec(t.data(), fct, false);
    for (u64 j = 0; j < n; ++j) *reinterpret_cast<T *>(out.d + oo + i64(j) * so) = t[j];
  });
}

template <class T>
static void r2c_nd(const View &in, const View &out, const std::vector<u64> &axes, bool fwd, T fct, u64 nth) {
  if (any_zero(in.shape)) return;
  const size_t last = axes.back();
  View o = out;
  o.shape = in.shape;
  o.shape[last] = in.shape[last] / 2 + 1;
  r2c_axis(in, o, last, fwd, fct, nth);
  if (axes.size() > 1) c2c_nd<T>(o, o, std::vector<u64>(axes.begin(), axes.end() - 1), fwd, T(1), nth);
}

template <class T>
static void c2r_nd(const View &in, const View &out, const std::vector<u64> &axes, bool fwd, T fct, u64 nth) {
  if (any_zero(out.shape)) return;
  const size_t last = axes.back();
  View i2 = in;
  i2.shape = out.shape;
  i2.shape[last] = out.shape[last] / 2 + 1;
  if (axes.size() == 1) {
    c2r_axis(i2, out, last, fwd, fct, nth);
    return;
  }
  // c2c over the other axes into a C-contiguous temporary (HDR:4009-4020)
  u64 total = 1;
  for (i64 s : i2.shape) total *= u64(s);
  std::vector<C<T>> tmp(total);
  View t{reinterpret_cast<char *>(tmp.data()), i2.shape, std::vector<i64>(i2.shape.size())};
  i64 acc = sizeof(C<T>);
  for (size_t d = i2.shape.size(); d-- > 0;) {
    t.stride[d] = acc;
    acc *= i2.shape[d];
  }
  c2c_nd<T>(i2, t, std::vector<u64>(axes.begin(), axes.end() - 1), fwd, T(1), nth);
  c2r_axis(t, out, last, fwd, fct, nth);
}

// Serial walk over the half-shape in C order with the mirrored position (role of rev_iter,
// HDR:3383-3444): for axes in `axes` index i maps to (n - i) mod n.
template <class F>
static void mirror_walk(const std::vector<i64> &shape, const std::vector<i64> &sa, const std::vector<i64> &sb,
                        const std::vector<u64> &axes, F f) {
  const size_t nd = shape.size(), last = axes.back();
  std::vector<char> rev(nd, 0);
  for (u64 a : axes) rev[a] = 1;
  std::vector<i64> half = shape;
  half[last] = shape[last] / 2 + 1;
  u64 total = 1;
  for (i64 h : half) total *= u64(h);
  std::vector<i64> pos(nd, 0);
  for (u64 idx = 0; idx < total; ++idx) {
    i64 pa = 0, pb = 0, pr = 0;
    for (size_t d = 0; d < nd; ++d) {
      const i64 q = rev[d] ? (pos[d] == 0 ? 0 : shape[d] - pos[d]) : pos[d];
      pa += pos[d] * sa[d];
      pb += pos[d] * sb[d];
      pr += q * sb[d];
    }
    f(pa, pb, pr);
    for (size_t d = nd; d-- > 0;) {
      if (++pos[d] < half[d]) break;
      pos[d] = 0;
    }
  }
}

template <class T>
static void c2c_sym(const View &in, const View &out, const std::vector<u64> &axes, bool fwd, T fct, u64 nth) {
  if (any_zero(in.shape)) return;
  r2c_nd<T>(in, out, axes, fwd, fct, nth);
  mirror_walk(in.shape, out.stride, out.stride, axes, [&](i64, i64 p, i64 q) {
    const T *a = reinterpret_cast<const T *>(out.d + p);
    const T re = a[0], im = a[1];
    T *b = reinterpret_cast<T *>(out.d + q);
    b[0] = re;
    b[1] = -im;
  });
}

// ExecDcst (HDR:3707-3721) + dct/dst (HDR:3891-3935)
template <class T, class P>
static void dcst_nd(const View &in, const View &out, const std::vector<u64> &axes, int type, bool cosine,
                    T fct, bool ortho, u64 nth) {
  for (size_t k = 0; k < axes.size(); ++k) {
    const View &src = k == 0 ? in : out;
    const size_t ax = axes[k];
    const u64 n = u64(in.shape[ax]);
    auto plan = get_plan<P>(n);
    const i64 si = src.stride[ax], so = out.stride[ax];
    const T f = k == 0 ? fct : T(1);
    for_rows(in.shape, src.stride, out.stride, ax, nth, [&](i64 oi, i64 oo) {
      std::vector<T> t(n);
      for (u64 j = 0; j < n; ++j) t[j] = *reinterpret_cast<const T *>(src.d + oi + i64(j) * si);
      plan->exec(t.data(), f, ortho, type, cosine);
      for (u64 j = 0; j < n; ++j) *reinterpret_cast<T *>(out.d + oo + i64(j) * so) = t[j];
    });
  }
}

template <class T>
static void dcst(const View &in, const View &out, const std::vector<u64> &axes, int type, bool cosine, T fct,
                 bool ortho, u64 nth) {
  if (type < 1 || type > 4) throw std::invalid_argument("invalid DCT/DST type");
  if (any_zero(in.shape)) return;
  if (type == 1) {
    if (cosine)
      dcst_nd<T, Dct1<T>>(in, out, axes, type, cosine, fct, ortho, nth);
    else
      dcst_nd<T, Dst1<T>>(in, out, axes, type, cosine, fct, ortho, nth);
  } else if (type == 4) {
    dcst_nd<T, Dcst4<T>>(in, out, axes, type, cosine, fct, ortho, nth);
  } else {
    dcst_nd<T, Dcst23<T>>(in, out, axes, type, cosine, fct, ortho, nth);
  }
}

// ExecR2R (HDR:3854-3873) + r2r_fftpack (HDR:4025-4040)
template <class T>
static void r2r_fftpack(const View &in, const View &out, const std::vector<u64> &axes, bool r2h, bool fwd,
                        T fct, u64 nth) {
  if (any_zero(in.shape)) return;
  for (size_t k = 0; k < axes.size(); ++k) {
    const View &src = k == 0 ? in : out;
    const size_t ax = axes[k];
    const u64 n = u64(in.shape[ax]);
    auto plan = get_plan<RPlan<T>>(n);
    const i64 si = src.stride[ax], so = out.stride[ax];
    const T f = k == 0 ? fct : T(1);
    for_rows(in.shape, src.stride, out.stride, ax, nth, [&](i64 oi, i64 oo) {
      std::vector<T> t(n);
      for (u64 j = 0; j < n; ++j) t[j] = *reinterpret_cast<const T *>(src.d + oi + i64(j) * si);
      if (!r2h && fwd)
        for (u64 i = 2; i < n; i += 2) t[i] = -t[i];
      plan->exec(t.data(), f, fwd);
      if (r2h && !fwd)
        for (u64 i = 2; i < n; i += 2) t[i] = -t[i];
      for (u64 j = 0; j < n; ++j) *reinterpret_cast<T *>(out.d + oo + i64(j) * so) = t[j];
    });
  }
}

// ExecHartley + copy_hartley (HDR:3661-3705) + r2r_separable_hartley (HDR:4042-4056)
template <class T>
static void hartley_sep(const View &in, const View &out, const std::vector<u64> &axes, T fct, u64 nth) {
  if (any_zero(in.shape)) return;
  for (size_t k = 0; k < axes.size(); ++k) {
    const View &src = k == 0 ? in : out;
    const size_t ax = axes[k];
    const u64 n = u64(in.shape[ax]);
    auto plan = get_plan<RPlan<T>>(n);
    const i64 si = src.stride[ax], so = out.stride[ax];
    const T f = k == 0 ? fct : T(1);
    for_rows(in.shape, src.stride, out.stride, ax, nth, [&](i64 oi, i64 oo) {
      std::vector<T> t(n);
      for (u64 j = 0; j < n; ++j) t[j] = *reinterpret_cast<const T *>(src.d + oi + i64(j) * si);
      plan->exec(t.data(), f, true);
      auto at = [&](u64 j) -> T & { return *reinterpret_cast<T *>(out.d + oo + i64(j) * so); };
      at(0) = t[0];
      u64 i = 1, i1 = 1, i2 = n - 1;
      for (; i + 1 < n; i += 2, ++i1, --i2) {
        at(i1) = t[i] + t[i + 1];
        at(i2) = t[i] - t[i + 1];
      }
      if (i < n) at(i1) = t[i];
    });
  }
}

// r2r_genuine_hartley (HDR:4058-4091): r2c into a temporary, then re+im / re-im placed at
// the position and its mirror
template <class T>
static void hartley_gen(const View &in, const View &out, const std::vector<u64> &axes, T fct, u64 nth) {
  if (any_zero(in.shape)) return;
  if (axes.size() == 1) return hartley_sep<T>(in, out, axes, fct, nth);
  const size_t last = axes.back();
  std::vector<i64> ts = in.shape;
  ts[last] = ts[last] / 2 + 1;
  u64 total = 1;
  for (i64 s : ts) total *= u64(s);
  std::vector<C<T>> tmp(total);
  View t{reinterpret_cast<char *>(tmp.data()), ts, std::vector<i64>(ts.size())};
  i64 acc = sizeof(C<T>);
  for (size_t d = ts.size(); d-- > 0;) {
    t.stride[d] = acc;
    acc *= ts[d];
  }
  r2c_nd<T>(in, t, axes, true, fct, nth);
  mirror_walk(in.shape, t.stride, out.stride, axes, [&](i64 pt, i64 po, i64 pr) {
    const T *v = reinterpret_cast<const T *>(t.d + pt);
    *reinterpret_cast<T *>(out.d + po) = v[0] + v[1];
    *reinterpret_cast<T *>(out.d + pr) = v[0] - v[1];
  });
}

}  // namespace port

// ---------------------------------------------------------------------------------------
// C ABI, numba array-struct layout (as SHIM)
// ---------------------------------------------------------------------------------------

extern "C" {
typedef struct {
  void *meminfo;
  void *parent;
  int64_t nitems;
  int64_t itemsize;
  void *data;
  int64_t shape_and_strides[1];
} port_arystruct_t;
}

namespace {
using port::i64;
using port::u64;
using port::View;

View view(const port_arystruct_t *a, u64 ndim) {
  View v{static_cast<char *>(a->data), std::vector<i64>(ndim), std::vector<i64>(ndim)};
  for (u64 i = 0; i < ndim; ++i) {
    v.shape[i] = a->shape_and_strides[i];
    v.stride[i] = a->shape_and_strides[ndim + i];
  }
  return v;
}
std::vector<u64> axes_of(const port_arystruct_t *a) {
  const u64 *p = static_cast<const u64 *>(a->data);
  return std::vector<u64>(p, p + a->nitems);
}
template <class F> int guarded(F f) {
  try {
    f();
    return 0;
  } catch (...) {
    return 1;
  }
}
}  // namespace

#define PORT_EXPORT extern "C" __attribute__((visibility("default")))

PORT_EXPORT uint64_t port_good_size(uint64_t n, bool real) {
  return real ? port::good_size_real(n) : port::good_size_cmplx(n);
}

PORT_EXPORT int port_c2c(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout, port_arystruct_t *axes,
                         bool forward, double fct, u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 16)
      port::c2c_nd<double>(i, o, axes_of(axes), forward, fct, nthreads);
    else
      port::c2c_nd<float>(i, o, axes_of(axes), forward, float(fct), nthreads);
  });
}

PORT_EXPORT int port_r2c(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout, port_arystruct_t *axes,
                         bool forward, double fct, u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 8)
      port::r2c_nd<double>(i, o, axes_of(axes), forward, fct, nthreads);
    else
      port::r2c_nd<float>(i, o, axes_of(axes), forward, float(fct), nthreads);
  });
}

PORT_EXPORT int port_c2c_sym(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout,
                             port_arystruct_t *axes, bool forward, double fct, u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 8)
      port::c2c_sym<double>(i, o, axes_of(axes), forward, fct, nthreads);
    else
      port::c2c_sym<float>(i, o, axes_of(axes), forward, float(fct), nthreads);
  });
}

PORT_EXPORT int port_c2r(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout, port_arystruct_t *axes,
                         bool forward, double fct, u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 16)
      port::c2r_nd<double>(i, o, axes_of(axes), forward, fct, nthreads);
    else
      port::c2r_nd<float>(i, o, axes_of(axes), forward, float(fct), nthreads);
  });
}

PORT_EXPORT int port_dct(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout, port_arystruct_t *axes,
                         u64 type, double fct, bool ortho, u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 8)
      port::dcst<double>(i, o, axes_of(axes), int(type), true, fct, ortho, nthreads);
    else
      port::dcst<float>(i, o, axes_of(axes), int(type), true, float(fct), ortho, nthreads);
  });
}

PORT_EXPORT int port_dst(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout, port_arystruct_t *axes,
                         u64 type, double fct, bool ortho, u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 8)
      port::dcst<double>(i, o, axes_of(axes), int(type), false, fct, ortho, nthreads);
    else
      port::dcst<float>(i, o, axes_of(axes), int(type), false, float(fct), ortho, nthreads);
  });
}

PORT_EXPORT int port_r2r_fftpack(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout,
                                 port_arystruct_t *axes, bool real2hermitian, bool forward, double fct,
                                 u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 8)
      port::r2r_fftpack<double>(i, o, axes_of(axes), real2hermitian, forward, fct, nthreads);
    else
      port::r2r_fftpack<float>(i, o, axes_of(axes), real2hermitian, forward, float(fct), nthreads);
  });
}

PORT_EXPORT int port_r2r_separable_hartley(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout,
                                           port_arystruct_t *axes, double fct, u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 8)
      port::hartley_sep<double>(i, o, axes_of(axes), fct, nthreads);
    else
      port::hartley_sep<float>(i, o, axes_of(axes), float(fct), nthreads);
  });
}

PORT_EXPORT int port_r2r_genuine_hartley(u64 ndim, const port_arystruct_t *ain, port_arystruct_t *aout,
                                         port_arystruct_t *axes, double fct, u64 nthreads) {
  return guarded([&] {
    const View i = view(ain, ndim), o = view(aout, ndim);
    if (ain->itemsize == 8)
      port::hartley_gen<double>(i, o, axes_of(axes), fct, nthreads);
    else
      port::hartley_gen<float>(i, o, axes_of(axes), float(fct), nthreads);
  });
}
