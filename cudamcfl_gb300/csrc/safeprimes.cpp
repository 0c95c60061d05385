/*
 * Multipliers of the base-2^32 multiply-with-carry generator
 * (rand_MWC_co, CUDAMCFLrng.cu:17-23).  The reference reads them from
 * safeprimes_base32.txt (CUDAMCFLrng.cu:44-70), which it does not ship; this
 * file regenerates the list from its defining property: a is usable when
 * p = a*2^32 - 1 and (p-1)/2 = a*2^31 - 1 are both prime, which makes the
 * generator's period (a*2^32 - 2)/2.  The list is ordered from 2^32-1
 * downwards.  Entry 0 seeds the reference-style init_RNG and entries
 * 1..32768 are the per-stream multipliers; the engine's photon-indexed
 * streams use entries 1..32768.
 *
 * Primality: Miller-Rabin with the seven bases {2, 325, 9375, 28178, 450775,
 * 9780504, 1795265022}, which is deterministic for all 64-bit integers
 * (Sinclair, 2011), after trial division by the primes below 256.
 */
#include <cstdint>
#include <mutex>
#include <vector>

#include "mcfl_internal.h"

namespace mcfl {
namespace {

using u128 = unsigned __int128;

uint64_t mul_mod(uint64_t a, uint64_t b, uint64_t n) { return (uint64_t)((u128)a * b % n); }

uint64_t pow_mod(uint64_t b, uint64_t e, uint64_t n) {
  uint64_t r = 1;
  b %= n;
  for (; e; e >>= 1) {
    if (e & 1) r = mul_mod(r, b, n);
    b = mul_mod(b, b, n);
  }
  return r;
}

bool strong_probable_prime(uint64_t n, uint64_t base, uint64_t d, int s) {
  base %= n;
  if (base == 0) return true;
  uint64_t x = pow_mod(base, d, n);
  if (x == 1 || x == n - 1) return true;
  for (int i = 1; i < s; ++i) {
    x = mul_mod(x, x, n);
    if (x == n - 1) return true;
  }
  return false;
}

const std::vector<uint32_t> &small_primes() {
  static std::vector<uint32_t> p = [] {
    std::vector<uint32_t> v;
    for (uint32_t c = 3; c < 256; c += 2) {
      bool ok = true;
      for (uint32_t q : v)
        if (c % q == 0) { ok = false; break; }
      if (ok) v.push_back(c);
    }
    return v;
  }();
  return p;
}

bool is_prime(uint64_t n) {
  if (n < 2) return false;
  if ((n & 1) == 0) return n == 2;
  for (uint32_t q : small_primes()) {
    if (n == q) return true;
    if (n % q == 0) return false;
  }
  uint64_t d = n - 1;
  int s = 0;
  while ((d & 1) == 0) { d >>= 1; ++s; }
  static const uint64_t bases[7] = {2, 325, 9375, 28178, 450775, 9780504, 1795265022};
  for (uint64_t b : bases)
    if (!strong_probable_prime(n, b, d, s)) return false;
  return true;
}

} // namespace

bool mwc_multiplier_valid(uint32_t a) {
  const uint64_t q = ((uint64_t)a << 31) - 1, p = ((uint64_t)a << 32) - 1;
  return is_prime(q) && is_prime(p);
}

std::vector<uint32_t> mwc_multipliers(size_t count) {
  std::vector<uint32_t> out;
  out.reserve(count);
  for (uint64_t a = 0xFFFFFFFFull; a > 1 && out.size() < count; --a)
    if (mwc_multiplier_valid((uint32_t)a)) out.push_back((uint32_t)a);
  return out;
}

const std::vector<uint32_t> &mwc_table() {
  static std::once_flag once;
  static std::vector<uint32_t> table;
  std::call_once(once, [] { table = mwc_multipliers(kMwcTableEntries + 1); });
  return table;
}

} // namespace mcfl
