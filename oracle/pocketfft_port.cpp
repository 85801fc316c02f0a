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
// What differs: the complex radix passes are a Stockham formulation (radix 8, 4, 2, 3, 5 and a
// generic odd radix, in cfftp's factor order) instead of FFTPACK's pass2..pass11/passg, and the
// real transform is a half-length complex FFT plus a split instead of rfftp's radf/radb passes.
// Those produce the same transforms up to rounding. Rows run several at a time in 16-byte lane
// vectors, as the reference's SIMD path does, so the port is also a fair CPU timing baseline.
#include <algorithm>
#include <condition_variable>
#include <functional>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <tuple>
#include <type_traits>
#include <vector>

#include <unistd.h>

namespace port {

using u64 = uint64_t;
using i64 = int64_t;

template <class T> struct C {
  T r, i;
};
// Complex numbers of scalars (plan tables) or of lane vectors (the data of several rows at
// once); the operators below are generic over both.
template <class D> inline C<D> operator+(C<D> a, C<D> b) { return {a.r + b.r, a.i + b.i}; }
template <class D> inline C<D> operator-(C<D> a, C<D> b) { return {a.r - b.r, a.i - b.i}; }
template <class T> inline C<T> operator*(C<T> a, C<T> b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
template <class T> inline C<T> operator*(C<T> a, T s) { return {a.r * s, a.i * s}; }
template <class D> inline C<D> conj(C<D> a) { return {a.r, -a.i}; }
// data times a real scalar
template <class D, class S> inline C<D> scale(C<D> a, S s) { return {a.r * s, a.i * s}; }
// data times a table entry w, or times conj(w) when CJ
template <bool CJ, class D, class T> inline C<D> tmul(C<D> a, C<T> w) {
  if constexpr (CJ)
    return {a.r * w.r + a.i * w.i, a.i * w.r - a.r * w.i};
  else
    return {a.r * w.r - a.i * w.i, a.r * w.i + a.i * w.r};
}

// Scratch array of n elements from a per-thread pool that is kept across calls, as the
// reference keeps one temporary per thread for all rows (HDR:3471-3494): one pool per call site
// (`slot`), so that nested users never share one; 64-byte aligned, contents undefined (every
// element is written before it is read). Reusing the memory matters beyond the allocation
// cost: a fresh block per row group made power-of-two strided gathers 2x slower.
enum Slot { kRows = 0, kRealZ, kRealX, kPass, kBlue, kDcst, kGenV, kGenS, kGenD, kSlots };
template <class X> class Scratch {
 public:
  Scratch(size_t n, Slot slot) {
    thread_local std::vector<char> pools[kSlots];
    std::vector<char> &p = pools[slot];
    const size_t need = n * sizeof(X) + 64;
    if (p.size() < need) p.resize(need);
    p_ = reinterpret_cast<X *>((reinterpret_cast<uintptr_t>(p.data()) + 63) & ~uintptr_t(63));
  }
  X &operator[](size_t i) { return p_[i]; }
  const X &operator[](size_t i) const { return p_[i]; }
  X *data() { return p_; }

 private:
  X *p_;
};

// Rows are transformed W at a time in 16-byte lane vectors (GCC vector extensions: SSE2 on
// x86-64, NEON on AArch64, no -march needed), as the reference's multi-row SIMD path does
// (HDR:3455-3470, 3585-3595); leftover rows go through the same code with W = 1.
template <class T> struct VecOf;
template <> struct VecOf<float> { using type = float __attribute__((vector_size(16))); };
template <> struct VecOf<double> { using type = double __attribute__((vector_size(16))); };
template <class T> constexpr int kLanes = int(16 / sizeof(T));
template <class T, int W> struct Lanes {
  using D = std::conditional_t<W == 1, T, typename VecOf<T>::type>;
  static T get(const D &v, int l) {
    if constexpr (W == 1) {
      (void)l;
      return v;
    } else {
      return v[l];
    }
  }
  static void set(D &v, int l, T x) {
    if constexpr (W == 1) {
      (void)l;
      v = x;
    } else {
      v[l] = x;
    }
  }
};

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

// e^{+2 pi i t / N} for many t < N at one N: two tables of about sqrt(N) roots each (by
// root()), hi_j = e^{2 pi i j S / N} and lo_j = e^{2 pi i j / N}, S the power of two at or
// above sqrt(N); a root is the double-precision product hi_{t / S} lo_{t mod S}, rounded once
// to T. O(sqrt(N)) cos/sin calls instead of one per twiddle, as the reference's table method
// (HDR:466-544).
class Roots {
 public:
  explicit Roots(u64 N) : N_(N), shift_(0) {
    while ((u64(1) << shift_) * (u64(1) << shift_) < N) ++shift_;
    const u64 S = u64(1) << shift_;
    for (u64 j = 0; j < S; ++j) lo_.push_back(dbl(j));
    for (u64 j = 0; j * S < N; ++j) hi_.push_back(dbl(j * S));
  }
  template <class T> C<T> get(u64 t) const {
    const C<double> a = hi_[t >> shift_], b = lo_[t & ((u64(1) << shift_) - 1)];
    return {T(a.r * b.r - a.i * b.i), T(a.r * b.i + a.i * b.r)};
  }

 private:
  C<double> dbl(u64 t) const {
    double c, s;
    root(t, N_, c, s);
    return {c, s};
  }
  u64 N_;
  int shift_;
  std::vector<C<double>> lo_, hi_;
};

// ---------------------------------------------------------------------------------------
// packed complex FFT (role of cfftp, HDR:1060-1830): Stockham passes
// ---------------------------------------------------------------------------------------

template <class T> class CPack {
 public:
  explicit CPack(u64 n) : n_(n) {
    if (n == 0) throw std::runtime_error("zero-length FFT requested");
    // factor order of cfftp::factorize (HDR:1750-1778): 8s, 4s, one 2 moved to the front, odd
    u64 len = n;
    while (len % 8 == 0) {
      fac_.push_back(8);
      len /= 8;
    }
    while (len % 4 == 0) {
      fac_.push_back(4);
      len /= 4;
    }
    if (len % 2 == 0) {
      len /= 2;
      fac_.push_back(2);
      std::swap(fac_.front(), fac_.back());
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
      const Roots roots(ns * R);
      for (u64 k = 1; k < R; ++k)
        for (u64 m = 0; m < ns; ++m) tw_.push_back(roots.get<T>(m * k));  // e^{+2 pi i m k / (ns R)}
      if (!specialised(R)) {  // odd radices: the roots of unity of order R
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
  template <class D> void exec(C<D> *c, T fct, bool fwd) const { fwd ? run<true>(c, fct) : run<false>(c, fct); }

 private:
  static bool specialised(u64 R) { return R == 2 || R == 3 || R == 4 || R == 5 || R == 8; }
  static bool odd_unrolled(u64 R) { return R == 7 || R == 11 || R == 13; }

  template <bool FWD, class D> void run(C<D> *c, T fct) const {
    if (n_ == 1) {
      c[0] = scale(c[0], fct);
      return;
    }
    // out of place passes: c -> s1, then s1 <-> s2, the last one back into c (two or more passes)
    const size_t np = fac_.size();
    Scratch<C<D>> buf((np > 2 ? 2 : 1) * n_, kPass);
    C<D> *s1 = buf.data(), *s2 = np > 2 ? s1 + n_ : nullptr;
    const C<D> *a = c;
    u64 ns = 1;
    for (size_t p = 0; p < np; ++p) {
      C<D> *b = p + 1 == np && np > 1 ? c : (p % 2 == 0 ? s1 : s2);
      const u64 R = fac_[p];
      const C<T> *tw = tw_.data() + off_[p];
      const C<T> *rt = rt_.data() + roots_off_[p];
      switch (R) {
        case 2: pass<FWD, 2>(ns, a, b, tw, [](C<D>(&v)[2]) { dft2(v); }); break;
        case 3: pass<FWD, 3>(ns, a, b, tw, [](C<D>(&v)[3]) { dft3<FWD>(v); }); break;
        case 4: pass<FWD, 4>(ns, a, b, tw, [](C<D>(&v)[4]) { dft4<FWD>(v); }); break;
        case 5: pass<FWD, 5>(ns, a, b, tw, [](C<D>(&v)[5]) { dft5<FWD>(v); }); break;
        case 8: pass<FWD, 8>(ns, a, b, tw, [](C<D>(&v)[8]) { dft8<FWD>(v); }); break;
        case 7: pass<FWD, 7>(ns, a, b, tw, [rt](C<D>(&v)[7]) { dft_odd<FWD, 7>(v, rt); }); break;
        case 11: pass<FWD, 11>(ns, a, b, tw, [rt](C<D>(&v)[11]) { dft_odd<FWD, 11>(v, rt); }); break;
        case 13: pass<FWD, 13>(ns, a, b, tw, [rt](C<D>(&v)[13]) { dft_odd<FWD, 13>(v, rt); }); break;
        default: passg<FWD>(R, ns, a, b, tw, rt);
      }
      a = b;
      ns *= R;
    }
    if (a != c) {  // a single pass
      for (u64 i = 0; i < n_; ++i) c[i] = scale(a[i], fct);
    } else if (fct != T(1)) {
      for (u64 i = 0; i < n_; ++i) c[i] = scale(c[i], fct);
    }
  }

  // One Stockham pass of radix R: butterfly (b0, m) reads x[j + k L] (j = b0 + m), twiddles
  // input k by (conj when forward) e^{+2 pi i m k / (ns R)}, writes y[b0 R + m + q ns].
  template <bool FWD, int R, class D, class Bfly>
  void pass(u64 ns, const C<D> *__restrict__ x, C<D> *__restrict__ y, const C<T> *__restrict__ tw, Bfly bfly) const {
    const u64 L = n_ / R;
    for (u64 b0 = 0; b0 < L; b0 += ns) {
      for (u64 m = 0; m < ns; ++m) {
        const u64 j = b0 + m;
        C<D> v[R];
        for (int k = 0; k < R; ++k) v[k] = x[j + k * L];
        if (ns > 1)
          for (int k = 1; k < R; ++k) v[k] = tmul<FWD>(v[k], tw[(k - 1) * ns + m]);
        bfly(v);
        C<D> *out = y + b0 * R + m;
        for (int q = 0; q < R; ++q) out[q * ns] = v[q];
      }
    }
  }

  // generic odd radix R: with s_k = v_k + v_{R-k}, d_k = v_k - v_{R-k} (k = 1..(R-1)/2) and
  // theta = 2 pi q k / R, y_q = A_q -+ i B_q and y_{R-q} = A_q +- i B_q (upper signs forward),
  // A_q = v_0 + sum_k s_k cos theta, B_q = sum_k d_k sin theta; y_0 = v_0 + sum_k s_k
  template <bool FWD, class D>
  void passg(u64 R, u64 ns, const C<D> *x, C<D> *y, const C<T> *tw, const C<T> *rt) const {
    const u64 L = n_ / R, H = (R - 1) / 2;
    Scratch<C<D>> v(R, kGenV), sk(H + 1, kGenS), dk(H + 1, kGenD);
    for (u64 b0 = 0; b0 < L; b0 += ns) {
      for (u64 m = 0; m < ns; ++m) {
        const u64 j = b0 + m;
        for (u64 k = 0; k < R; ++k) v[k] = x[j + k * L];
        if (ns > 1)
          for (u64 k = 1; k < R; ++k) v[k] = tmul<FWD>(v[k], tw[(k - 1) * ns + m]);
        C<D> y0 = v[0];
        for (u64 k = 1; k <= H; ++k) {
          sk[k] = v[k] + v[R - k];
          dk[k] = v[k] - v[R - k];
          y0 = y0 + sk[k];
        }
        C<D> *out = y + b0 * R + m;
        out[0] = y0;
        for (u64 q = 1; q <= H; ++q) {
          C<D> A = v[0], B = {D{}, D{}};
          u64 e = 0;
          for (u64 k = 1; k <= H; ++k) {
            e += q;
            if (e >= R) e -= R;
            A = A + scale(sk[k], rt[e].r);
            B = B + scale(dk[k], rt[e].i);
          }
          const C<D> iB = {-B.i, B.r};  // i B
          out[q * ns] = FWD ? A - iB : A + iB;
          out[(R - q) * ns] = FWD ? A + iB : A - iB;
        }
      }
    }
  }

  // multiply by -i (forward) or +i (backward)
  template <bool FWD, class D> static C<D> rot90(C<D> a) {
    if constexpr (FWD)
      return {a.i, -a.r};
    else
      return {-a.i, a.r};
  }
  template <class D> static void dft2(C<D> (&v)[2]) {
    const C<D> a = v[0];
    v[0] = a + v[1];
    v[1] = a - v[1];
  }
  template <bool FWD, class D> static void dft3(C<D> (&v)[3]) {
    const T c1 = T(-0.5), s1 = T(FWD ? -0.86602540378443864676 : 0.86602540378443864676);
    const C<D> s = v[1] + v[2], d = v[1] - v[2];
    const C<D> a = v[0] + scale(s, c1);
    const C<D> b = {-d.i * s1, d.r * s1};  // i * s1 * d
    v[0] = v[0] + s;
    v[1] = a + b;
    v[2] = a - b;
  }
  template <bool FWD, class D> static void dft4(C<D> (&v)[4]) {
    const C<D> t0 = v[0] + v[2], t1 = v[0] - v[2], t2 = v[1] + v[3];
    const C<D> t3 = rot90<FWD>(v[1] - v[3]);
    v[0] = t0 + t2;
    v[2] = t0 - t2;
    v[1] = t1 + t3;
    v[3] = t1 - t3;
  }
  template <bool FWD, class D> static void dft5(C<D> (&v)[5]) {
    const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);
    const T sg = FWD ? T(-1) : T(1);
    const T s1 = sg * T(0.95105651629515357212), s2 = sg * T(0.58778525229247312917);
    const C<D> sa = v[1] + v[4], da = v[1] - v[4], sb = v[2] + v[3], db = v[2] - v[3];
    const C<D> a1 = v[0] + scale(sa, c1) + scale(sb, c2), a2 = v[0] + scale(sa, c2) + scale(sb, c1);
    const C<D> e1 = scale(da, s1) + scale(db, s2), e2 = scale(da, s2) - scale(db, s1);
    const C<D> b1 = {-e1.i, e1.r}, b2 = {-e2.i, e2.r};
    v[0] = v[0] + sa + sb;
    v[1] = a1 + b1;
    v[4] = a1 - b1;
    v[2] = a2 + b2;
    v[3] = a2 - b2;
  }
  // radix 8 as two radix-4 transforms (even / odd inputs) and the eighth-root rotations
  template <bool FWD, class D> static void dft8(C<D> (&v)[8]) {
    C<D> a[4] = {v[0], v[2], v[4], v[6]}, b[4] = {v[1], v[3], v[5], v[7]};
    dft4<FWD>(a);
    dft4<FWD>(b);
    const T h = T(0.70710678118654752440084436210484904);
    const C<D> x1 = b[1], x3 = b[3];
    if constexpr (FWD) {  // b_q *= e^{-2 pi i q / 8}
      b[1] = {(x1.r + x1.i) * h, (x1.i - x1.r) * h};
      b[3] = {(x3.i - x3.r) * h, -(x3.r + x3.i) * h};
    } else {  // b_q *= e^{+2 pi i q / 8}
      b[1] = {(x1.r - x1.i) * h, (x1.r + x1.i) * h};
      b[3] = {-(x3.r + x3.i) * h, (x3.r - x3.i) * h};
    }
    b[2] = rot90<FWD>(b[2]);
    for (int q = 0; q < 4; ++q) {
      v[q] = a[q] + b[q];
      v[q + 4] = a[q] - b[q];
    }
  }

  // odd radix R unrolled at compile time: the pairing of passg with R fixed (rt = the roots of
  // order R); same operations in the same order, so the same results as the generic pass
  template <bool FWD, int R, class D> static void dft_odd(C<D> (&v)[R], const C<T> *rt) {
    constexpr int H = (R - 1) / 2;
    C<D> sk[H + 1], dk[H + 1], out[R];
    C<D> y0 = v[0];
    for (int k = 1; k <= H; ++k) {
      sk[k] = v[k] + v[R - k];
      dk[k] = v[k] - v[R - k];
      y0 = y0 + sk[k];
    }
    out[0] = y0;
    for (int q = 1; q <= H; ++q) {
      C<D> A = v[0], B = {D{}, D{}};
      for (int k = 1; k <= H; ++k) {
        const int e = (q * k) % R;
        A = A + scale(sk[k], rt[e].r);
        B = B + scale(dk[k], rt[e].i);
      }
      const C<D> iB = {-B.i, B.r};
      out[q] = FWD ? A - iB : A + iB;
      out[R - q] = FWD ? A + iB : A - iB;
    }
    for (int q = 0; q < R; ++q) v[q] = out[q];
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
    const Roots roots(2 * n);
    u64 coeff = 0;
    for (u64 m = 1; m < n; ++m) {
      coeff += 2 * m - 1;
      if (coeff >= 2 * n) coeff -= 2 * n;
      bk_[m] = roots.get<T>(coeff);
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

  template <class D> void exec(C<D> *c, T fct, bool fwd) const { fwd ? run<true>(c, fct) : run<false>(c, fct); }

 private:
  template <bool FWD, class D> void run(C<D> *c, T fct) const {  // HDR:2732-2762
    Scratch<C<D>> a(n2_, kBlue);
    std::fill(a.data() + n_, a.data() + n2_, C<D>{D{}, D{}});  // zero padding
    for (u64 m = 0; m < n_; ++m) a[m] = tmul<FWD>(c[m], bk_[m]);
    plan_.exec(a.data(), T(1), true);
    for (u64 m = 0; m < n2_; ++m) a[m] = tmul<!FWD>(a[m], bkf_[m]);
    plan_.exec(a.data(), T(1), false);
    for (u64 m = 0; m < n_; ++m) c[m] = scale(tmul<FWD>(a[m], bk_[m]), fct);
  }

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
  template <class D> void exec(C<D> *c, T fct, bool fwd) const {
    pack_ ? pack_->exec(c, fct, fwd) : blue_->exec(c, fct, fwd);
  }

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
      const Roots roots(n);
      for (u64 k = 0; k <= n / 2; ++k) w_.push_back(roots.get<T>(k));  // e^{+2 pi i k/n}
    } else {
      full_.reset(new CPlan<T>(n));
    }
  }
  u64 length() const { return n_; }

  template <class D> void exec(D *c, T fct, bool r2hc) const {
    const u64 n = n_;
    if (n == 1) {
      c[0] = c[0] * fct;
      return;
    }
    if (full_) {
      Scratch<C<D>> z(n, kRealZ);
      if (r2hc) {
        for (u64 j = 0; j < n; ++j) z[j] = {c[j], D{}};
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
    Scratch<C<D>> z(L + 1, kRealZ);
    if (r2hc) {
      for (u64 j = 0; j < L; ++j) z[j] = {c[2 * j], c[2 * j + 1]};
      half_->exec(z.data(), T(1), true);
      // split: X_k = E + W^k O, E = (Z_k + conj Z_{L-k})/2, O = (Z_k - conj Z_{L-k})/(2i)
      Scratch<C<D>> X(L + 1, kRealX);
      X[0] = {z[0].r + z[0].i, D{}};
      X[L] = {z[0].r - z[0].i, D{}};
      for (u64 k = 1; k <= L / 2; ++k) {
        const C<D> a = z[k], b = conj(z[L - k]);
        const C<D> E = scale(a + b, T(0.5));
        const C<D> d = scale(a - b, T(0.5));
        const C<D> O = {d.i, -d.r};
        const C<D> t = tmul<true>(O, w_[k]);  // W_n^k = e^{-2 pi i k/n}
        X[k] = E + t;
        X[L - k] = conj(E - t);
      }
      if (fct != T(1))
        for (u64 k = 0; k <= L; ++k) X[k] = scale(X[k], fct);
      pack(X.data(), c);
    } else {
      Scratch<C<D>> X(L + 1, kRealX);
      X[0] = {c[0], D{}};
      for (u64 k = 1; k < L; ++k) X[k] = {c[2 * k - 1], c[2 * k]};
      X[L] = {c[n - 1], D{}};
      // merge: Z_k = A + u, A = X_k + conj X_{L-k}, u = i conj(W^k) (X_k - conj X_{L-k})
      for (u64 k = 0; k < L; ++k) {
        const C<D> xk = X[k], xc = conj(X[L - k]);
        const C<D> A = xk + xc, B = xk - xc;
        const C<D> t = tmul<false>(B, w_[k]);  // conj(W_n^k) = e^{+2 pi i k/n}
        z[k] = A + C<D>{-t.i, t.r};
      }
      half_->exec(z.data(), fct, false);
      for (u64 j = 0; j < L; ++j) {
        c[2 * j] = z[j].r;
        c[2 * j + 1] = z[j].i;
      }
    }
  }

 private:
  template <class D> void pack(const C<D> *X, D *c) const {
    c[0] = X[0].r;
    u64 i = 1, k = 1;
    for (; i + 1 < n_; i += 2, ++k) {
      c[i] = X[k].r;
      c[i + 1] = X[k].i;
    }
    if (i < n_) c[i] = X[k].r;
  }
  template <class D> void unpack_full(const D *c, C<D> *z) const {
    const u64 n = n_;
    z[0] = {c[0], D{}};
    u64 i = 1, k = 1;
    for (; i + 1 < n; i += 2, ++k) {
      z[k] = {c[i], c[i + 1]};
      z[n - k] = {c[i], -c[i + 1]};
    }
    if (i < n) z[k] = {c[i], D{}};
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
  template <class D> void exec(D *c, T fct, bool ortho, int, bool) const {
    const u64 N = fft_.length(), n = N / 2 + 1;
    const T s2 = T(kSqrt2);
    if (ortho) {
      c[0] *= s2;
      c[n - 1] *= s2;
    }
    Scratch<D> t(N, kDcst);
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
  template <class D> void exec(D *c, T fct, bool, int, bool) const {
    const u64 N = fft_.length(), n = N / 2 - 1;
    Scratch<D> t(N, kDcst);
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
    const Roots roots(4 * n);
    for (u64 i = 0; i < n; ++i) tw_[i] = roots.get<T>(i + 1).r;  // cos(2 pi (i+1) / 4n)
  }
  u64 length() const { return fft_.length(); }
  template <class D> void exec(D *c, T fct, bool ortho, int type, bool cosine) const {
    const u64 N = length(), NS2 = (N + 1) / 2;
    const T s2 = T(kSqrt2);
    if (type == 2) {
      if (!cosine)
        for (u64 k = 1; k < N; k += 2) c[k] = -c[k];
      c[0] *= T(2);
      if ((N & 1) == 0) c[N - 1] *= T(2);
      for (u64 k = 1; k + 1 < N; k += 2) {  // MPINPLACE(c[k+1], c[k]): (a, b) <- (a-b, a+b)
        const D a = c[k + 1], b = c[k];
        c[k + 1] = a - b;
        c[k] = a + b;
      }
      fft_.exec(c, fct, false);
      for (u64 k = 1, kc = N - 1; k < NS2; ++k, --kc) {
        const D t1 = tw_[k - 1] * c[kc] + tw_[kc - 1] * c[k];
        const D t2 = tw_[k - 1] * c[k] - tw_[kc - 1] * c[kc];
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
        const D t1 = c[k] + c[kc], t2 = c[k] - c[kc];
        c[k] = tw_[k - 1] * t2 + tw_[kc - 1] * t1;
        c[kc] = tw_[k - 1] * t1 - tw_[kc - 1] * t2;
      }
      if ((N & 1) == 0) c[NS2] *= T(2) * tw_[NS2 - 1];
      fft_.exec(c, fct, true);
      for (u64 k = 1; k + 1 < N; k += 2) {  // MPINPLACE(c[k], c[k+1]): (a, b) <- (a-b, a+b)
        const D a = c[k], b = c[k + 1];
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
      const Roots roots(16 * n);
      for (u64 i = 0; i < n / 2; ++i) C2_.push_back(conj(roots.get<T>(8 * i + 1)));
    }
  }
  u64 length() const { return N_; }
  template <class D> void exec(D *c, T fct, bool, int, bool cosine) const {
    const u64 N = N_, n2 = N / 2;
    if (!cosine)
      for (u64 k = 0, kc = N - 1; k < n2; ++k, --kc) std::swap(c[k], c[kc]);
    if (N & 1) {
      // odd length: the index shuffle and sign pattern of the reference (derived there from
      // FFTW's apply_re11) around a real FFT of length N
      Scratch<D> y(N, kDcst);
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
      Scratch<C<D>> y(n2, kDcst);
      for (u64 i = 0; i < n2; ++i) y[i] = tmul<false>(C<D>{c[2 * i], c[N - 1 - i * 2]}, C2_[i]);
      fft_->exec(y.data(), fct, true);
      for (u64 i = 0, ic = n2 - 1; i < n2; ++i, --ic) {
        c[2 * i] = T(2) * (y[i].r * C2_[i].r - y[i].i * C2_[i].i);
        c[2 * i + 1] = T(-2) * (y[ic].i * C2_[ic].r + y[ic].r * C2_[ic].i);
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
static u64 thread_count(u64 nthreads, const std::vector<i64> &shape, size_t axis, u64 vlen) {
  if (nthreads == 1) return 1;
  u64 size = 1;
  for (i64 s : shape) size *= u64(s);
  u64 parallel = size / (u64(shape[axis]) * vlen);
  if (shape[axis] < 1000) parallel /= 4;
  const u64 mx = nthreads == 0 ? std::max(1u, std::thread::hardware_concurrency()) : nthreads;
  return std::max<u64>(1, std::min(parallel, mx));
}

// Persistent worker threads for the row loops (the reference keeps a thread pool too,
// HDR:760-960): run(nt, fn) calls fn(0..nt-1), index 0 on the calling thread, and returns when
// all are done. One job at a time; a child process after fork() builds its own pool.
class Pool {
 public:
  static Pool &get() {
    static Pool *pool = nullptr;
    static pid_t owner = 0;
    if (pool == nullptr || owner != getpid()) {  // the parent's workers do not exist after fork
      pool = new Pool();
      owner = getpid();
    }
    return *pool;
  }
  void run(u64 nt, const std::function<void(u64)> &fn) {
    std::lock_guard<std::mutex> job(job_mu_);
    {
      std::unique_lock<std::mutex> lk(mu_);
      while (workers_.size() + 1 < nt) workers_.emplace_back([this] { loop(); });
      fn_ = &fn;
      count_ = nt;
      next_ = 1;
      left_ = nt - 1;
      ++gen_;
    }
    cv_.notify_all();
    fn(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [&] { return left_ == 0; });
    fn_ = nullptr;
  }

 private:
  void loop() {
    u64 seen = 0;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      cv_.wait(lk, [&] { return gen_ != seen; });
      seen = gen_;
      while (fn_ != nullptr && next_ < count_) {
        const u64 i = next_++;
        const std::function<void(u64)> *fn = fn_;
        lk.unlock();
        (*fn)(i);
        lk.lock();
        if (--left_ == 0) done_.notify_all();
      }
    }
  }
  std::mutex job_mu_, mu_;
  std::condition_variable cv_, done_;
  std::vector<std::thread> workers_;
  const std::function<void(u64)> *fn_ = nullptr;
  u64 count_ = 0, next_ = 0, left_ = 0, gen_ = 0;
};

// Calls f(in_offsets, out_offsets, G, lanes) for the rows along `axis` (C order of the other
// dims): G groups of W consecutive rows (lanes = integral_constant<int, W>, G <= gmax) while W
// rows remain in a thread's share, then single rows (lanes = integral_constant<int, 1>, G = 1).
// Rows are spread over threads.
constexpr int kMaxRows = 64;
template <int W, class F>
static void for_rows(const std::vector<i64> &shape, const std::vector<i64> &sin, const std::vector<i64> &sout,
                     size_t axis, u64 nthreads, int gmax, F f) {
  const size_t nd = shape.size();
  u64 rows = 1;
  for (size_t d = 0; d < nd; ++d)
    if (d != axis) rows *= u64(shape[d]);
  const u64 nt = thread_count(nthreads, shape, axis, W);
  auto offsets = [&](u64 r, i64 &oi, i64 &oo) {
    u64 rem = r;
    oi = oo = 0;
    for (size_t dd = nd; dd-- > 0;) {
      if (dd == axis) continue;
      const u64 pos = rem % u64(shape[dd]);
      rem /= u64(shape[dd]);
      oi += i64(pos) * sin[dd];
      oo += i64(pos) * sout[dd];
    }
  };
  auto work = [&](u64 lo, u64 hi) {
    i64 oi[kMaxRows], oo[kMaxRows];
    u64 r = lo;
    if constexpr (W > 1) {
      while (r + W <= hi) {
        const int G = int(std::min<u64>(u64(gmax), (hi - r) / W));
        for (int l = 0; l < G * W; ++l) offsets(r + u64(l), oi[l], oo[l]);
        f(oi, oo, G, std::integral_constant<int, W>{});
        r += u64(G) * W;
      }
    }
    for (; r < hi; ++r) {
      offsets(r, oi[0], oo[0]);
      f(oi, oo, 1, std::integral_constant<int, 1>{});
    }
  };
  if (nt <= 1) {
    work(0, rows);
    return;
  }
  Pool::get().run(nt, [&](u64 t) { work(rows * t / nt, rows * (t + 1) / nt); });
}

// Groups of W rows taken per call: one for a contiguous axis; for a strided one enough that the
// rows cover 128 contiguous bytes, so that every cache line gathered from (or scattered to) the
// array is used whole at once, before the other rows' lines can evict it (with power-of-two
// strides all of a row's elements fall into one cache set).
template <int W> static int groups_for(i64 si, i64 so, size_t elem) {
  if (si == i64(elem) && so == i64(elem)) return 1;
  return std::max(1, std::min(kMaxRows / W, int(128 / (W * elem))));
}

// Real rows: gather G groups of W rows (element j of row g W + l at base[g W + l] + j * stride)
// into lane vectors t[g n + j], and scatter them back.
template <class T, int W>
static void gather_real(typename Lanes<T, W>::D *t, const char *d, const i64 *base, i64 stride, u64 n, int G) {
  for (u64 j = 0; j < n; ++j)
    for (int g = 0; g < G; ++g) {
      typename Lanes<T, W>::D v;
      for (int l = 0; l < W; ++l)
        Lanes<T, W>::set(v, l, *reinterpret_cast<const T *>(d + base[g * W + l] + i64(j) * stride));
      t[size_t(g) * n + j] = v;
    }
}
template <class T, int W>
static void scatter_real(const typename Lanes<T, W>::D *t, char *d, const i64 *base, i64 stride, u64 n, int G) {
  for (u64 j = 0; j < n; ++j)
    for (int g = 0; g < G; ++g) {
      const typename Lanes<T, W>::D v = t[size_t(g) * n + j];
      for (int l = 0; l < W; ++l) *reinterpret_cast<T *>(d + base[g * W + l] + i64(j) * stride) = Lanes<T, W>::get(v, l);
    }
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
    const int gmax = groups_for<kLanes<T>>(si, so, sizeof(C<T>));
    for_rows<kLanes<T>>(in.shape, src.stride, out.stride, ax, nth, gmax,
                        [&](const i64 *oi, const i64 *oo, int G, auto lanes) {
      constexpr int W = decltype(lanes)::value;
      using LN = Lanes<T, W>;
      Scratch<C<typename LN::D>> buf(size_t(G) * n, kRows);
      for (u64 j = 0; j < n; ++j)  // lanes composed in registers, one store per vector
        for (int g = 0; g < G; ++g) {
          typename LN::D re, im;
          for (int l = 0; l < W; ++l) {
            const C<T> x = *reinterpret_cast<const C<T> *>(src.d + oi[g * W + l] + i64(j) * si);
            LN::set(re, l, x.r);
            LN::set(im, l, x.i);
          }
          buf[size_t(g) * n + j] = {re, im};
        }
      for (int g = 0; g < G; ++g) plan->exec(buf.data() + size_t(g) * n, f, fwd);
      for (u64 j = 0; j < n; ++j)
        for (int g = 0; g < G; ++g) {
          const C<typename LN::D> v = buf[size_t(g) * n + j];
          for (int l = 0; l < W; ++l)
            *reinterpret_cast<C<T> *>(out.d + oo[g * W + l] + i64(j) * so) = C<T>{LN::get(v.r, l), LN::get(v.i, l)};
        }
    });
  }
}

// general_r2c (HDR:3723-3779): halfcomplex to complex, conjugated when !forward
template <class T>
static void r2c_axis(const View &in, const View &out, size_t ax, bool fwd, T fct, u64 nth) {
  const u64 n = u64(in.shape[ax]), nout = n / 2 + 1;
  auto plan = get_plan<RPlan<T>>(n);
  const i64 si = in.stride[ax], so = out.stride[ax];
  const int gmax = groups_for<kLanes<T>>(si == i64(sizeof(T)) ? i64(sizeof(C<T>)) : si, so, sizeof(C<T>));
  for_rows<kLanes<T>>(in.shape, in.stride, out.stride, ax, nth, gmax,
                      [&](const i64 *oi, const i64 *oo, int G, auto lanes) {
    constexpr int W = decltype(lanes)::value;
    using LN = Lanes<T, W>;
    Scratch<typename LN::D> t(size_t(G) * n, kRows);
    gather_real<T, W>(t.data(), in.d, oi, si, n, G);
    for (int g = 0; g < G; ++g) plan->exec(t.data() + size_t(g) * n, fct, true);
    // bin k from the half-complex row: (t_0, 0), (t_{2k-1}, t_{2k}), and (t_{n-1}, 0) at k = n/2
    // for even n
    auto put = [&](u64 k, int g, int l) {
      const typename LN::D *row = t.data() + size_t(g) * n;
      const T re = LN::get(row[k == 0 ? 0 : 2 * k - 1], l);
      const T im = (k == 0 || 2 * k >= n) ? T(0) : LN::get(row[2 * k], l);
      T *p = reinterpret_cast<T *>(out.d + oo[g * W + l] + i64(k) * so);
      p[0] = re;
      p[1] = fwd ? im : -im;
    };
    if (so == i64(sizeof(C<T>))) {  // contiguous output rows: one row after the other
      for (int g = 0; g < G; ++g)
        for (int l = 0; l < W; ++l)
          for (u64 k = 0; k < nout; ++k) put(k, g, l);
    } else {  // strided: bin by bin across the rows
      for (u64 k = 0; k < nout; ++k)
        for (int g = 0; g < G; ++g)
          for (int l = 0; l < W; ++l) put(k, g, l);
    }
  });
}

// general_c2r (HDR:3780-3852): imaginary parts negated when forward
template <class T>
static void c2r_axis(const View &in, const View &out, size_t ax, bool fwd, T fct, u64 nth) {
  const u64 n = u64(out.shape[ax]), nin = n / 2 + 1;
  auto plan = get_plan<RPlan<T>>(n);
  const i64 si = in.stride[ax], so = out.stride[ax];
  const int gmax = groups_for<kLanes<T>>(si, so == i64(sizeof(T)) ? i64(sizeof(C<T>)) : so, sizeof(C<T>));
  for_rows<kLanes<T>>(out.shape, in.stride, out.stride, ax, nth, gmax,
                      [&](const i64 *oi, const i64 *oo, int G, auto lanes) {
    constexpr int W = decltype(lanes)::value;
    using LN = Lanes<T, W>;
    Scratch<typename LN::D> t(size_t(G) * n, kRows);
    // half-complex row from the bins: t_0 = Re X_0, (t_{2k-1}, t_{2k}) = X_k, t_{n-1} = Re X_{n/2}
    // for even n
    auto get = [&](u64 k, int g, int l) {
      typename LN::D *row = t.data() + size_t(g) * n;
      const T *p = reinterpret_cast<const T *>(in.d + oi[g * W + l] + i64(k) * si);
      if (k == 0) {
        LN::set(row[0], l, p[0]);
      } else {
        LN::set(row[2 * k - 1], l, p[0]);
        if (2 * k < n) LN::set(row[2 * k], l, fwd ? -p[1] : p[1]);
      }
    };
    if (si == i64(sizeof(C<T>))) {  // contiguous input rows: one row after the other
      for (int g = 0; g < G; ++g)
        for (int l = 0; l < W; ++l)
          for (u64 k = 0; k < nin; ++k) get(k, g, l);
    } else {  // strided: bin by bin across the rows
      for (u64 k = 0; k < nin; ++k)
        for (int g = 0; g < G; ++g)
          for (int l = 0; l < W; ++l) get(k, g, l);
    }
    for (int g = 0; g < G; ++g) plan->exec(t.data() + size_t(g) * n, fct, false);
    scatter_real<T, W>(t.data(), out.d, oo, so, n, G);
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
  std::unique_ptr<C<T>[]> tmp(new C<T>[total]);  // every element is written by the c2c below
  View t{reinterpret_cast<char *>(tmp.get()), i2.shape, std::vector<i64>(i2.shape.size())};
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
    const int gmax = groups_for<kLanes<T>>(si, so, sizeof(T));
    for_rows<kLanes<T>>(in.shape, src.stride, out.stride, ax, nth, gmax,
                        [&](const i64 *oi, const i64 *oo, int G, auto lanes) {
      constexpr int W = decltype(lanes)::value;
      Scratch<typename Lanes<T, W>::D> t(size_t(G) * n, kRows);
      gather_real<T, W>(t.data(), src.d, oi, si, n, G);
      for (int g = 0; g < G; ++g) plan->exec(t.data() + size_t(g) * n, f, ortho, type, cosine);
      scatter_real<T, W>(t.data(), out.d, oo, so, n, G);
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
    const int gmax = groups_for<kLanes<T>>(si, so, sizeof(T));
    for_rows<kLanes<T>>(in.shape, src.stride, out.stride, ax, nth, gmax,
                        [&](const i64 *oi, const i64 *oo, int G, auto lanes) {
      constexpr int W = decltype(lanes)::value;
      Scratch<typename Lanes<T, W>::D> t(size_t(G) * n, kRows);
      gather_real<T, W>(t.data(), src.d, oi, si, n, G);
      for (int g = 0; g < G; ++g) {
        typename Lanes<T, W>::D *row = t.data() + size_t(g) * n;
        if (!r2h && fwd)
          for (u64 i = 2; i < n; i += 2) row[i] = -row[i];
        plan->exec(row, f, fwd);
        if (r2h && !fwd)
          for (u64 i = 2; i < n; i += 2) row[i] = -row[i];
      }
      scatter_real<T, W>(t.data(), out.d, oo, so, n, G);
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
    const int gmax = groups_for<kLanes<T>>(si, so, sizeof(T));
    for_rows<kLanes<T>>(in.shape, src.stride, out.stride, ax, nth, gmax,
                        [&](const i64 *oi, const i64 *oo, int G, auto lanes) {
      constexpr int W = decltype(lanes)::value;
      using LN = Lanes<T, W>;
      Scratch<typename LN::D> t(size_t(G) * n, kRows);
      gather_real<T, W>(t.data(), src.d, oi, si, n, G);
      for (int g = 0; g < G; ++g) plan->exec(t.data() + size_t(g) * n, f, true);
      // out_0 = t_0, out_k = t_{2k-1} + t_{2k}, out_{n-k} = t_{2k-1} - t_{2k}, and
      // out_{n/2} = t_{n-1} for even n
      for (u64 k = 0; k <= n / 2; ++k)
        for (int g = 0; g < G; ++g) {
          const typename LN::D *row = t.data() + size_t(g) * n;
          for (int l = 0; l < W; ++l) {
            auto at = [&](u64 j) -> T & { return *reinterpret_cast<T *>(out.d + oo[g * W + l] + i64(j) * so); };
            if (k == 0) {
              at(0) = LN::get(row[0], l);
            } else if (2 * k < n) {
              const T a = LN::get(row[2 * k - 1], l), b = LN::get(row[2 * k], l);
              at(k) = a + b;
              at(n - k) = a - b;
            } else {
              at(k) = LN::get(row[2 * k - 1], l);
            }
          }
        }
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
