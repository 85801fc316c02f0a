// Host-side planner: sizes, factorisations, FP64 tables, per-device plan cache.
#include "rg_plan.hpp"

#include <cmath>
#include <complex>
#include <map>
#include <mutex>
#include <stdexcept>
#include <tuple>

#include "rg_error.hpp"

namespace rg {

// ---------------------------------------------------------------------------------------
// sizes
// ---------------------------------------------------------------------------------------

// Smallest number >= n whose prime factors all lie in `primes` (ascending, starting with 2).
// Same contract as the reference's util::good_size_cmplx / good_size_real
// (rocket_fft/_pocketfft_hdronly.h:589-650): n below the small threshold is returned as is.
// The search here is a plain enumeration of the odd smooth part; every power of two times it
// that is >= n is a candidate and the minimum wins.
static uint64_t smallest_smooth_at_least(uint64_t n, const std::vector<uint64_t> &odd_primes) {
  // best starts at the next power of two >= n (always smooth)
  uint64_t best = 1;
  while (best < n) best <<= 1;
  // enumerate odd smooth numbers o < best recursively; for each, scale by 2^k up to >= n
  std::vector<uint64_t> stack{1};
  std::vector<size_t> start{0};
  while (!stack.empty()) {
    const uint64_t o = stack.back();
    const size_t first = start.back();
    stack.pop_back();
    start.pop_back();
    uint64_t x = o;
    while (x < n) x <<= 1;
    if (x < best) best = x;
    for (size_t p = first; p < odd_primes.size(); ++p) {
      const uint64_t q = odd_primes[p];
      if (o > best / q) break;  // o*q >= best can not improve
      stack.push_back(o * q);
      start.push_back(p);
    }
  }
  return best;
}

uint64_t good_size_cmplx(uint64_t n) {
  if (n <= 12) return n;
  return smallest_smooth_at_least(n, {3, 5, 7, 11});
}

uint64_t good_size_real(uint64_t n) {
  if (n <= 6) return n;
  return smallest_smooth_at_least(n, {3, 5});
}

uint64_t largest_prime_factor(uint64_t n) {
  uint64_t res = 1;
  while (n > 1 && (n & 1) == 0) {
    res = 2;
    n >>= 1;
  }
  for (uint64_t x = 3; x * x <= n; x += 2)
    while (n % x == 0) {
      res = x;
      n /= x;
    }
  if (n > 1) res = n;
  return res;
}

bool core_smooth(uint64_t n) {
  if (n == 0) return false;
  for (uint64_t p : {2, 3, 5, 7, 11, 13})
    while (n % p == 0) n /= p;
  return n == 1;
}

std::vector<int> core_radices(int L) {
  std::vector<int> r;
  int e = 0, rest = L;
  while ((rest & 1) == 0) {
    rest >>= 1;
    ++e;
  }
  // 2^e = 16^a * {1, 8*4 (or 2 when a == 0), 4, 8}
  const int a = e / 4, b = e % 4;
  if (b == 1 && a >= 1) {
    for (int i = 0; i < a - 1; ++i) r.push_back(16);
    r.push_back(8);
    r.push_back(4);
  } else {
    for (int i = 0; i < a; ++i) r.push_back(16);
    if (b == 1) r.push_back(2);
    if (b == 2) r.push_back(4);
    if (b == 3) r.push_back(8);
  }
  for (int p : {3, 5, 7, 11, 13})
    while (rest % p == 0) {
      r.push_back(p);
      rest /= p;
    }
  if (rest != 1) throw Error(RG_ERR_INTERNAL, "core_radices: length not 13-smooth");
  return r;
}

void unit_root(uint64_t t, uint64_t N, double &c, double &s) {
  t %= N;
  // 8 t / N selects the octant; reduce to an angle in [0, pi/4]
  const unsigned __int128 t8 = (unsigned __int128)t * 8;
  uint64_t oct = uint64_t(t8 / N);
  const uint64_t rem = uint64_t(t8 - (unsigned __int128)oct * N);  // 8t - oct*N in [0, N)
  // angle = (pi/4) * (oct + rem/N); within the octant use x = rem/N or 1 - rem/N
  const double pi4 = 0.78539816339744830962;
  double cc, ss;
  if ((oct & 1) == 0) {
    const double x = pi4 * (double(rem) / double(N));
    cc = std::cos(x);
    ss = std::sin(x);
  } else {
    const double x = pi4 * (double(N - rem) / double(N));
    cc = std::sin(x);
    ss = std::cos(x);
  }
  // now (cc, ss) = (cos, sin) of the angle reduced to the first quadrant of octant pair
  switch (oct >> 1) {
    case 0: c = cc; s = ss; break;
    case 1: c = -ss; s = cc; break;
    case 2: c = -cc; s = -ss; break;
    default: c = ss; s = -cc; break;
  }
}

uint64_t blue_length(uint64_t n) { return good_size_cmplx(2 * n - 1); }

// ---------------------------------------------------------------------------------------
// device table cache
// ---------------------------------------------------------------------------------------

namespace {

struct Key {
  int dev, dt, kind;
  uint64_t a, b;
  bool operator<(const Key &o) const {
    return std::tie(dev, dt, kind, a, b) < std::tie(o.dev, o.dt, o.kind, o.a, o.b);
  }
};

struct Entry {
  std::vector<void *> dptrs;
  size_t bytes = 0;
  std::shared_ptr<void> obj;  // the typed plan object
};

std::mutex g_mu;
std::map<Key, Entry> g_cache;
size_t g_bytes = 0;

int current_device() {
  int d = 0;
  RG_CUDA(cudaGetDevice(&d));
  return d;
}

// upload a vector of std::complex<double> converted to the plan's precision
void *upload(const std::vector<std::complex<double>> &v, DType dt, size_t &bytes) {
  const size_t n = v.size();
  const size_t nb = std::max<size_t>(n, 1) * cx_size(dt);
  void *d = nullptr;
  RG_CUDA(cudaMalloc(&d, nb));
  if (dt == DType::F64) {
    RG_CUDA(cudaMemcpy(d, v.data(), n * 16, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> f(2 * n);
    for (size_t i = 0; i < n; ++i) {
      f[2 * i] = float(v[i].real());
      f[2 * i + 1] = float(v[i].imag());
    }
    RG_CUDA(cudaMemcpy(d, f.data(), n * 8, cudaMemcpyHostToDevice));
  }
  bytes += nb;
  return d;
}

std::complex<double> wfwd(uint64_t t, uint64_t N) {  // e^{-2 pi i t / N}
  double c, s;
  unit_root(t, N, c, s);
  return {c, -s};
}

template <class Obj, class Build> std::shared_ptr<Obj> cached(const Key &k, Build build) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_cache.find(k);
  if (it != g_cache.end()) return std::static_pointer_cast<Obj>(it->second.obj);
  Entry e;
  auto obj = std::make_shared<Obj>();
  build(*obj, e);
  e.obj = obj;
  g_bytes += e.bytes;
  g_cache.emplace(k, std::move(e));
  return obj;
}

}  // namespace

static std::shared_ptr<CoreTables> core_ptr(int L, DType dt) {
  Key k{current_device(), int(dt), 1, uint64_t(L), 0};
  return cached<CoreTables>(k, [&](CoreTables &ct, Entry &e) {
    const std::vector<int> rad = core_radices(L);
    if (int(rad.size()) > kMaxPass) throw Error(RG_ERR_INTERNAL, "too many passes");
    std::vector<std::complex<double>> tw;
    FFTCore &c = ct.core;
    c.L = L;
    c.npass = int(rad.size());
    int Ns = 1;
    for (int p = 0; p < c.npass; ++p) {
      PassDesc &pd = c.pass[p];
      pd.R = rad[p];
      pd.Ns = Ns;
      pd.LR = L / pd.R;
      pd.tw = int(tw.size());
      pd.dNs = make_fastdiv(uint32_t(Ns));
      pd.dLR = make_fastdiv(uint32_t(pd.LR));
      if (Ns > 1)
        for (int kk = 1; kk < pd.R; ++kk)
          for (int m = 0; m < Ns; ++m) tw.push_back(wfwd(uint64_t(m) * kk, uint64_t(Ns) * pd.R));
      Ns *= pd.R;
    }
    void *d = upload(tw, dt, e.bytes);
    e.dptrs.push_back(d);
    c.tw = d;
  });
}

// Entries are only dropped by cache_clear(), which callers must not run concurrently with
// transforms; until then the returned references stay valid.
const CoreTables &get_core(int L, DType dt) { return *core_ptr(L, dt); }

const void *get_roots(uint64_t n, uint64_t count, DType dt) {
  struct Roots {
    const void *d;
  };
  Key k{current_device(), int(dt), 2, n, count};
  auto r = cached<Roots>(k, [&](Roots &o, Entry &e) {
    std::vector<std::complex<double>> v(count);
    for (uint64_t i = 0; i < count; ++i) v[i] = wfwd(i, n);
    void *d = upload(v, dt, e.bytes);
    e.dptrs.push_back(d);
    o.d = d;
  });
  return r->d;
}

const void *get_pass_tw(int L, int R0, DType dt) {
  struct Tw {
    const void *d;
  };
  Key k{current_device(), int(dt), 5, uint64_t(L), uint64_t(R0)};
  auto r = cached<Tw>(k, [&](Tw &o, Entry &e) {
    std::vector<std::complex<double>> v;
    for (int kk = 1; kk < L / R0; ++kk)
      for (int m = 0; m < R0; ++m) v.push_back(wfwd(uint64_t(m) * kk, uint64_t(L)));
    void *d = upload(v, dt, e.bytes);
    e.dptrs.push_back(d);
    o.d = d;
  });
  return r->d;
}

SplitTables get_split(uint64_t N, DType dt) {
  Key k{current_device(), int(dt), 3, N, 0};
  auto r = cached<SplitTables>(k, [&](SplitTables &o, Entry &e) {
    int bits = 0;
    while ((uint64_t(1) << bits) < N) ++bits;
    const int shift = (bits + 1) / 2;
    const uint64_t nlo = uint64_t(1) << shift;
    const uint64_t nhi = (N + nlo - 1) / nlo;
    std::vector<std::complex<double>> lo(nlo), hi(nhi);
    for (uint64_t t = 0; t < nlo; ++t) lo[t] = wfwd(t, N);
    for (uint64_t t = 0; t < nhi; ++t) hi[t] = wfwd(t * nlo, N);
    o.lo = upload(lo, dt, e.bytes);
    o.hi = upload(hi, dt, e.bytes);
    o.shift = shift;
    e.dptrs.push_back(const_cast<void *>(o.lo));
    e.dptrs.push_back(const_cast<void *>(o.hi));
  });
  return *r;
}

const BlueTables &get_blue(uint64_t n, DType dt) {
  const Key k{current_device(), int(dt), 4, n, 0};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(k);
    if (it != g_cache.end()) return *std::static_pointer_cast<BlueTables>(it->second.obj);
  }
  // built outside the cache lock: the device construction runs the library's own FFT, which
  // takes plans from this cache
  const uint64_t m = blue_length(n);
  auto obj = std::make_shared<BlueTables>();
  Entry e;
  void *bk = nullptr, *bkf = nullptr;
  RG_CUDA(cudaMalloc(&bk, std::max<uint64_t>(n, 1) * cx_size(dt)));
  if (cudaMalloc(&bkf, std::max<uint64_t>(m, 1) * cx_size(dt)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(bk);
    throw Error(RG_ERR_NOMEM, "cudaMalloc failed for Bluestein tables");
  }
  try {
    blue_tables_device(n, m, dt, bk, bkf);
  } catch (...) {
    cudaFree(bk);
    cudaFree(bkf);
    throw;
  }
  obj->n = n;
  obj->m = m;
  obj->bk = bk;
  obj->bkf = bkf;
  e.dptrs = {bk, bkf};
  e.bytes = size_t(n + m) * cx_size(dt);
  e.obj = obj;
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_cache.find(k);
  if (it != g_cache.end()) {  // another thread built the same tables meanwhile
    cudaFree(bk);
    cudaFree(bkf);
    return *std::static_pointer_cast<BlueTables>(it->second.obj);
  }
  g_bytes += e.bytes;
  g_cache.emplace(k, std::move(e));
  return *obj;
}

void cache_clear() {
  std::lock_guard<std::mutex> lk(g_mu);
  RG_CUDA(cudaDeviceSynchronize());
  for (auto &kv : g_cache)
    for (void *p : kv.second.dptrs) cudaFree(p);
  g_cache.clear();
  g_bytes = 0;
}

size_t cache_entries() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_cache.size();
}

size_t cache_bytes() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_bytes;
}

}  // namespace rg
