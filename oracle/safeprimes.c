/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or
 * runs this file; tests, smoke() and bench.py's CPU-baseline leg use it as a
 * checker.
 *
 * Generator of multiply-with-carry (MWC) multipliers in the text format that
 * the reference's init_RNG() reads (CUDAMCFLrng.cu:31-90): one line per
 * multiplier, three unsigned 32-bit integers "%u %u %u".  Line 1 is the
 * multiplier of the seeding generator ("begin", CUDAMCFLrng.cu:52); lines
 * 2..n+1 are the per-stream multipliers (CUDAMCFLrng.cu:67-70).
 *
 * The reference ships no multiplier file (safeprimes_base32.txt is listed as
 * missing), so the table is regenerated from the published criterion of the
 * base-2^32 MWC generator used by CUDAMC/CUDAMCML: a multiplier a is valid
 * when both a*2^32-1 and a*2^31-1 are prime (a*2^32-1 is then a safe prime
 * and the generator's period is (a*2^32-2)/2).  Candidates are taken
 * downwards from 2^32-1, after a sieve by the odd primes below 2^12, and are
 * confirmed with the deterministic Miller-Rabin test for 64-bit integers
 * (bases 2..37 are a proof for n < 3.3e24).
 *
 * Columns 2 and 3 of each line are the high and low 32-bit words of the
 * Sophie Germain prime a*2^31-1.  The reference reads and discards them
 * (tmp1, tmp2 at CUDAMCFLrng.cu:52,69).
 *
 * The product carries its own, independently written generator
 * (cudamcfl_gb300/csrc/safeprimes.cpp); tests check the two agree.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

static uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t m) {
  return (uint64_t)(((u128)a * b) % m);
}

static uint64_t powmod64(uint64_t b, uint64_t e, uint64_t m) {
  uint64_t r = 1;
  b %= m;
  while (e) {
    if (e & 1) r = mulmod64(r, b, m);
    b = mulmod64(b, b, m);
    e >>= 1;
  }
  return r;
}

/* Deterministic Miller-Rabin for odd n > 37. */
static int is_prime_u64(uint64_t n) {
  static const uint64_t bases[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  uint64_t d = n - 1;
  int s = 0;
  while ((d & 1) == 0) { d >>= 1; ++s; }
  for (int i = 0; i < 12; ++i) {
    uint64_t x = powmod64(bases[i], d, n);
    if (x == 1 || x == n - 1) continue;
    int composite = 1;
    for (int r = 1; r < s; ++r) {
      x = mulmod64(x, x, n);
      if (x == n - 1) { composite = 0; break; }
    }
    if (composite) return 0;
  }
  return 1;
}

/* Fills out[0..count) with valid multipliers, largest first. Returns count
 * found (always count unless the 32-bit range is exhausted). */
int oracle_safeprime_multipliers(uint32_t *out, int count) {
  enum { NSMALL = 600 };
  uint32_t small[NSMALL];
  uint32_t bad1[NSMALL], bad2[NSMALL]; /* a mod r that makes a*2^32-1 / a*2^31-1 divisible by r */
  int ns = 0;
  for (uint32_t r = 3; r < 4096 && ns < NSMALL; r += 2) {
    int pr = 1;
    for (uint32_t q = 3; q * q <= r; q += 2)
      if (r % q == 0) { pr = 0; break; }
    if (!pr) continue;
    /* a*2^32 == 1 (mod r)  <=>  a == inv(2^32) (mod r) */
    uint64_t t32 = powmod64(2, 32, r), t31 = powmod64(2, 31, r);
    small[ns] = r;
    bad1[ns] = (uint32_t)powmod64(t32, r - 2, r);
    bad2[ns] = (uint32_t)powmod64(t31, r - 2, r);
    ++ns;
  }
  const uint32_t BLOCK = 1u << 16;
  unsigned char *flag = (unsigned char *)malloc(BLOCK);
  int found = 0;
  uint64_t hi = 0xFFFFFFFFull; /* block covers a in (hi-BLOCK, hi] */
  while (found < count && hi > BLOCK) {
    uint64_t lo = hi - BLOCK + 1;
    memset(flag, 1, BLOCK);
    for (int i = 0; i < ns; ++i) {
      uint32_t r = small[i];
      uint32_t lom = (uint32_t)(lo % r);
      for (int k = 0; k < 2; ++k) {
        uint32_t bad = k ? bad2[i] : bad1[i];
        uint32_t first = (bad + r - lom) % r;
        for (uint64_t j = first; j < BLOCK; j += r) flag[j] = 0;
      }
    }
    for (int64_t j = BLOCK - 1; j >= 0 && found < count; --j) {
      if (!flag[j]) continue;
      uint64_t a = lo + (uint64_t)j;
      uint64_t q = (a << 31) - 1, p = (a << 32) - 1;
      if (is_prime_u64(q) && is_prime_u64(p)) out[found++] = (uint32_t)a;
    }
    hi = lo - 1;
  }
  free(flag);
  return found;
}

int oracle_write_safeprimes(const char *path, int count) {
  uint32_t *a = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)count);
  int n = oracle_safeprime_multipliers(a, count);
  FILE *f = fopen(path, "w");
  if (!f) { free(a); return -1; }
  for (int i = 0; i < n; ++i) {
    uint64_t q = ((uint64_t)a[i] << 31) - 1;
    fprintf(f, "%u %u %u\n", a[i], (uint32_t)(q >> 32), (uint32_t)q);
  }
  fclose(f);
  free(a);
  return n == count ? 0 : -2;
}

#ifdef SAFEPRIMES_MAIN
int main(int argc, char **argv) {
  int n = argc > 2 ? atoi(argv[2]) : 32769;
  const char *path = argc > 1 ? argv[1] : "safeprimes_base32.txt";
  return oracle_write_safeprimes(path, n) ? 1 : 0;
}
#endif
