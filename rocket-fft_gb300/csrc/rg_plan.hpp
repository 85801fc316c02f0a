// Host-side planner for the GB300 pocketfft path: sizes, factorisations, FP64-accurate
// twiddle/chirp tables and a thread-safe, per-device plan cache.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "rg_common.cuh"

namespace rg {

enum class DType { F32 = 0, F64 = 1 };
inline size_t real_size(DType t) { return t == DType::F32 ? 4 : 8; }
inline size_t cx_size(DType t) { return 2 * real_size(t); }

// ---- sizes (rocket_fft/_pocketfft_hdronly.h:546-650) ----
uint64_t good_size_cmplx(uint64_t n);   // smallest 2^a 3^b 5^c 7^d 11^e >= n (n <= 12 -> n)
uint64_t good_size_real(uint64_t n);    // smallest 2^a 3^b 5^c >= n (n <= 6 -> n)
uint64_t largest_prime_factor(uint64_t n);

// Radices the on-chip core implements.
bool core_smooth(uint64_t n);                         // all prime factors in {2,3,5,7,11,13}
std::vector<int> core_radices(int L);                 // pass order for an on-chip FFT of length L

constexpr int kMaxThreads = 512; // threads per CTA of the axis kernel
constexpr int kMaxCore = 8192;   // longest on-chip transform (complex elements)

// e^{+2 pi i t / N}, accurate to about one ulp in double (octant reduction on integers).
void unit_root(uint64_t t, uint64_t N, double &c, double &s);

// Device tables, cached per (device, dtype, kind, parameters). Pointers stay valid for the
// life of the process (the cache owns them; a bounded number of entries is kept).
struct CoreTables {
  FFTCore core;     // with core.tw pointing to device memory
};
const CoreTables &get_core(int L, DType dt);

// W_n^k (forward sign) for k = 0..count-1
const void *get_roots(uint64_t n, uint64_t count, DType dt);

// Twiddles of the second pass of the two-pass schedule R0 x L / R0: entry (k - 1) R0 + m is
// W_L^{m k} (m < R0, 1 <= k < L / R0), the layout of a core table's pass with Ns = R0.
const void *get_pass_tw(int L, int R0, DType dt);

struct SplitTables {
  const void *lo, *hi;
  int shift;
};
// W_N^t = lo[t & (2^shift - 1)] * hi[t >> shift], forward sign, t < N
SplitTables get_split(uint64_t N, DType dt);

struct BlueTables {
  uint64_t n, m;
  const void *bk;   // e^{+i pi j^2 / n}, j < n
  const void *bkf;  // FFT_m(zero-padded symmetric bk) / m, m entries
};
const BlueTables &get_blue(uint64_t n, DType dt);

// Fill device tables bk (n entries) and bkf (m entries) in the precision dt (rg_plan_dev.cu);
// synchronous.
void blue_tables_device(uint64_t n, uint64_t m, DType dt, void *bk, void *bkf);

// Smallest 13-smooth length usable as the Bluestein convolution length for n.
uint64_t blue_length(uint64_t n);

// Plan-cache maintenance (exposed through the C ABI)
void cache_clear();
size_t cache_entries();
size_t cache_bytes();

}  // namespace rg
