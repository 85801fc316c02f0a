// Host-side check of the radix butterflies used by the GPU kernels (rocket-fft_gb300/csrc/
// rg_fft.cuh): each forward DFT_R against a naive long-double DFT of the same inputs. Built
// by tests/test_native.py with nvcc as a host program; needs no GPU.
#include <cmath>
#include <cstdio>
#include <random>

#include "rg_fft.cuh"

template <typename T, int R> double check(std::mt19937_64 &g) {
  std::normal_distribution<double> nd;
  rg::cx<T> v[R];
  long double re[R], im[R];
  for (int k = 0; k < R; ++k) {
    v[k] = rg::mk<T>(T(nd(g)), T(nd(g)));
    re[k] = v[k].x;
    im[k] = v[k].y;
  }
  rg::dft<T, R>(v);
  const long double pi = 3.141592653589793238462643383279502884L;
  long double num = 0, den = 0;
  for (int q = 0; q < R; ++q) {
    long double sr = 0, si = 0;
    for (int k = 0; k < R; ++k) {
      const long double a = -2 * pi * ((q * k) % R) / R;
      sr += re[k] * cosl(a) - im[k] * sinl(a);
      si += re[k] * sinl(a) + im[k] * cosl(a);
    }
    num += (sr - v[q].x) * (sr - v[q].x) + (si - v[q].y) * (si - v[q].y);
    den += sr * sr + si * si;
  }
  return double(sqrtl(num / den));
}

template <typename T> int run(const char *name, double tol) {
  std::mt19937_64 g(7);
  int bad = 0;
  auto one = [&](int R, double e) {
    printf("%s R=%d rel_l2=%.3e\n", name, R, e);
    if (!(e <= tol)) ++bad;
  };
  for (int rep = 0; rep < 3; ++rep) {
    one(2, check<T, 2>(g));
    one(3, check<T, 3>(g));
    one(4, check<T, 4>(g));
    one(5, check<T, 5>(g));
    one(7, check<T, 7>(g));
    one(8, check<T, 8>(g));
    one(11, check<T, 11>(g));
    one(13, check<T, 13>(g));
    one(16, check<T, 16>(g));
  }
  return bad;
}

int main() {
  int bad = run<float>("f32", 1e-6) + run<double>("f64", 1e-15);
  printf("%s\n", bad ? "FAIL" : "OK");
  return bad ? 1 : 0;
}
