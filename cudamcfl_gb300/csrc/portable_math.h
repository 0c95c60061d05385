/*
 * Bit-reproducible single-precision primitives of the photon transport.
 *
 * Every function here is written with IEEE-754 basic operations (add, sub,
 * mul, div, sqrt, conversions) only, each rounded once to nearest-even.  A
 * translation unit that compiles it without floating-point contraction (nvcc
 * -fmad=false -prec-div=true -prec-sqrt=true -ftz=false; gcc
 * -ffp-contract=off) therefore computes the same bits on an sm_103a GPU and
 * on any IEEE host CPU.  The exact-math transport kernel and the CPU oracle
 * both use this header; that is what makes their tallies comparable bit for
 * bit.
 *
 * The transcendental functions replace the fast-math intrinsics the reference
 * transport calls (__logf in the step length and the Gaussian beam radius,
 * CUDAMCFLtransport.cu:290,512; __sincosf in the azimuth, :517,603; __cosf in
 * the isotropic launch, :477).  They are written from the series of the
 * functions themselves, with no library code:
 *   log: x = 2^e m with m in [sqrt(1/2), sqrt(2)), f = (m-1)/(m+1),
 *        log m = 2 atanh f = 2 (f + f^3/3 + f^5/5 + f^7/7 + f^9/9 + f^11/11),
 *        |f| < 0.1716, truncation below 1e-10 relative; e ln 2 is added with
 *        ln 2 split into a 16-bit head and a tail (Cody-Waite).
 *   sin/cos: Cody-Waite reduction of x by pi/2 with a three-part constant,
 *        then the Taylor series of sin (to r^9) and cos (to r^10) on
 *        |r| <= pi/4, truncation below 2e-9.
 * Domain: plog for positive normal floats; psincos for |x| < 2^10.  Both are
 * within a few ulp of the true function (test_portable_math_accuracy in
 * tests/test_cpu_basics.py).
 */
#ifndef MCFL_PORTABLE_MATH_H
#define MCFL_PORTABLE_MATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define MCFL_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#include <string.h>
#define MCFL_HD static inline
#endif

MCFL_HD uint32_t mcfl_f2bits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

MCFL_HD float mcfl_bits2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

/* ---------------- conversions with the CUDA intrinsics' meaning ---------- */

/* float -> uint32, saturating (NaN and negatives -> 0, >= 2^32 -> 2^32-1). */
#if !defined(__CUDA_ARCH__)
static inline uint32_t mcfl_sat_u32_host(float r) {
  if (!(r > 0.0f)) return 0u;
  if (r >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)r;
}
#endif

MCFL_HD uint32_t mcfl_f2u_rz(float f) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rz(f);
#else
  return mcfl_sat_u32_host(truncf(f));
#endif
}

MCFL_HD uint32_t mcfl_f2u_ru(float f) {
#if defined(__CUDA_ARCH__)
  return __float2uint_ru(f);
#else
  return mcfl_sat_u32_host(ceilf(f));
#endif
}

MCFL_HD uint32_t mcfl_f2u_rn(float f) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rn(f);
#else
  return mcfl_sat_u32_host(nearbyintf(f));
#endif
}

/* uint32 -> float rounded toward zero: keep the leading 24 significant bits. */
MCFL_HD float mcfl_u2f_rz(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint2float_rz(u);
#else
  if (u < (1u << 24)) return (float)u;
  int drop = 8 - __builtin_clz(u);
  return (float)(u & ~((1u << drop) - 1u));
#endif
}

MCFL_HD float mcfl_u2f_rn(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint2float_rn(u);
#else
  return (float)u;
#endif
}

MCFL_HD float mcfl_i2f_rn(int i) {
#if defined(__CUDA_ARCH__)
  return __int2float_rn(i);
#else
  return (float)i;
#endif
}

MCFL_HD float mcfl_rint(float x) {
#if defined(__CUDA_ARCH__)
  return rintf(x);
#else
  return nearbyintf(x);
#endif
}

/* ---------------- natural logarithm ---------------- */

MCFL_HD float mcfl_plogf(float x) {
  const float LN2_HI = 0x1.62e4p-1f;       /* 16 significant bits: e*LN2_HI is exact */
  const float LN2_LO = 0x1.7f7d1cp-20f;
  const float SQRT2 = 0x1.6a09e6p+0f;
  uint32_t b = mcfl_f2bits(x);
  int e = (int)((b >> 23) & 0xffu) - 127;
  float m = mcfl_bits2f((b & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
  if (m > SQRT2) {
    m = m * 0.5f; /* exact */
    e = e + 1;
  }
  float f = (m - 1.0f) / (m + 1.0f); /* m - 1 is exact (Sterbenz) */
  float f2 = f * f;
  float p = 0x1.745d18p-4f;            /* 1/11 */
  p = p * f2 + 0x1.c71c72p-4f;         /* 1/9 */
  p = p * f2 + 0x1.24924ap-3f;         /* 1/7 */
  p = p * f2 + 0x1.99999ap-3f;         /* 1/5 */
  p = p * f2 + 0x1.555556p-2f;         /* 1/3 */
  p = p * f2;
  float tf = f + f;
  float lm = tf + tf * p;
  float fe = mcfl_i2f_rn(e);
  return fe * LN2_HI + (lm + fe * LN2_LO);
}

/* ---------------- sine and cosine ---------------- */

MCFL_HD void mcfl_psincosf(float x, float *s, float *c) {
  const float TWO_OVER_PI = 0x1.45f306p-1f;
  const float PIO2_1 = 0x1.922p+0f;          /* 13 significant bits */
  const float PIO2_2 = -0x1.2aefp-18f;
  const float PIO2_3 = 0x1.68c234p-39f;
  float q = mcfl_rint(x * TWO_OVER_PI);
  int qi = (int)q;
  float r = x - q * PIO2_1;
  r = r - q * PIO2_2;
  r = r - q * PIO2_3;
  float r2 = r * r;
  float ps = 0x1.71de3ap-19f;        /* 1/9! */
  ps = ps * r2 - 0x1.a01a02p-13f;    /* 1/7! */
  ps = ps * r2 + 0x1.111112p-7f;     /* 1/5! */
  ps = ps * r2 - 0x1.555556p-3f;     /* 1/3! */
  float sr = r + (r * r2) * ps;
  float pc = -0x1.27e4fcp-22f;       /* 1/10! */
  pc = pc * r2 + 0x1.a01a02p-16f;    /* 1/8! */
  pc = pc * r2 - 0x1.6c16c2p-10f;    /* 1/6! */
  pc = pc * r2 + 0x1.555556p-5f;     /* 1/4! */
  pc = pc * r2 - 0.5f;
  float cr = 1.0f + r2 * pc;
  switch (qi & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}

MCFL_HD float mcfl_pcosf(float x) {
  float s, c;
  mcfl_psincosf(x, &s, &c);
  return c;
}

/* ---------------- photon-indexed MWC stream set-up ---------------- */

/* SplitMix64 finaliser (Steele, Lea & Flood 2014; constants as published). */
MCFL_HD uint64_t mcfl_splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Key of one photon stream family (a job, or one phase of a run). */
MCFL_HD uint64_t mcfl_stream_key(uint64_t seed, uint64_t stream_tag) {
  return mcfl_splitmix64(seed ^ mcfl_splitmix64(stream_tag));
}

/* MWC state (carry in the high word) and multiplier for photon k of a stream
 * family.  The multiplier is one of 2^15 table entries; the state satisfies
 * the validity rules of CUDAMCFLrng.cu:60,72 (x != 0, carry < a-1, low word
 * != 2^32-1). */
MCFL_HD void mcfl_photon_stream(uint64_t key, uint64_t k, const uint32_t *table32768, uint64_t *x, uint32_t *a) {
  uint64_t h1 = mcfl_splitmix64(key + k);
  uint64_t h2 = mcfl_splitmix64(h1);
  uint32_t m = table32768[h1 >> 49];
  uint32_t c = (uint32_t)(((h2 >> 32) * (uint64_t)(m - 1u)) >> 32); /* [0, m-2] */
  uint32_t lo = (uint32_t)h2;
  if (lo == 0xFFFFFFFFu) lo = 0xFFFFFFFEu;
  if (c == 0u && lo == 0u) lo = 1u;
  *x = ((uint64_t)c << 32) | lo;
  *a = m;
}

#endif
