/*
 * ORACLE / TEST INFRASTRUCTURE ONLY (see oracle/README.md).
 *
 * Host shim that lets g++ compile the reference's own device code
 * (CUDAMCFLtransport.cu, CUDAMCFLrng.cu, CUDAMCFLio.cu, CUDAMCFLmem.cu) for
 * the CPU, unmodified, as a stand-in for the "emu" build that nvcc no longer
 * offers (Compile_emu:1 uses -deviceemu, removed from nvcc).  It is
 * force-included (-include) before the reference sources.
 *
 * Every CUDA intrinsic the reference calls is given its documented IEEE
 * meaning: conversions round as their suffix says and saturate like the
 * hardware (NaN and negatives to 0, overflow to the type maximum); the
 * fast-math intrinsics (__logf, __cosf, __sincosf, __fdividef, rsqrtf) map to
 * the C library.  Device memory calls map to host memory.  Kernels become
 * plain functions run over virtual (blockIdx, threadIdx) pairs that the
 * driver sets.
 */
#ifndef MCFL_REF_SHIM_H
#define MCFL_REF_SHIM_H

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define __device__
#define __global__
#define __constant__
#define __host__
#define __align__(n) __attribute__((aligned(n)))

struct mcfl_shim_dim3 { unsigned int x, y, z; };
extern thread_local mcfl_shim_dim3 blockIdx;
extern thread_local mcfl_shim_dim3 threadIdx;

static inline void __syncthreads(void) {}

/* ---- float -> unsigned int, saturating, with the named rounding ---- */
static inline unsigned int mcfl_sat_u32(double v) {
  if (!(v > 0.0)) return 0u; /* NaN, -0, negatives */
  if (v >= 4294967295.0) return 0xFFFFFFFFu;
  return (unsigned int)v;
}
static inline unsigned int __float2uint_rz(float f) { return mcfl_sat_u32(truncf(f)); }
static inline unsigned int __float2uint_ru(float f) { return mcfl_sat_u32(ceilf(f)); }
static inline unsigned int __float2uint_rn(float f) { return mcfl_sat_u32(nearbyintf(f)); }

/* ---- integer -> float ---- */
static inline float __int2float_rn(int i) { return (float)i; }
static inline float __uint2float_rn(unsigned int u) { return (float)u; }
static inline float __uint2float_rz(unsigned int u) {
  /* keep the leading 24 significant bits: exact, i.e. round toward zero */
  if (u < (1u << 24)) return (float)u;
  int lz = __builtin_clz(u);
  int drop = 8 - lz; /* bits beyond a 24-bit significand */
  return (float)(u & ~((1u << drop) - 1u));
}

/* ---- fast-math intrinsics -> IEEE / libm ---- */
/* glibc declares __logf/__cosf/__sincosf itself, hence the macros; the
 * helpers take float arguments like the CUDA intrinsics do. */
static inline float mcfl_shim_fdividef(float a, float b) { return a / b; }
static inline float mcfl_shim_logf(float x) { return logf(x); }
static inline float mcfl_shim_cosf(float x) { return cosf(x); }
static inline void mcfl_shim_sincosf(float x, float *s, float *c) { *s = sinf(x); *c = cosf(x); }
static inline float mcfl_shim_fsqrt_rn(float x) { return sqrtf(x); }
static inline float mcfl_shim_rsqrtf(float x) { return 1.0f / sqrtf(x); }
#define __fdividef(a, b) mcfl_shim_fdividef((a), (b))
#define __logf(x) mcfl_shim_logf(x)
#define __cosf(x) mcfl_shim_cosf(x)
#define __sincosf(x, s, c) mcfl_shim_sincosf((x), (s), (c))
#define __fsqrt_rn(x) mcfl_shim_fsqrt_rn(x)
#define rsqrtf(x) mcfl_shim_rsqrtf(x)

/* ---- 64-bit atomics used by the tallies ---- */
static inline unsigned long long atomicAdd(unsigned long long *p, unsigned long long v) {
  return __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
}

/* ---- CUDA runtime calls of CUDAMCFLmem.cu -> host memory ---- */
typedef int cudaError_t;
enum { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };
static inline cudaError_t cudaMalloc(void **p, size_t n) {
  *p = calloc(n ? n : 1, 1);
  return *p ? 0 : 2;
}
static inline cudaError_t cudaFree(void *p) { free(p); return 0; }
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, int) {
  if (n) memcpy(d, s, n);
  return 0;
}
static inline cudaError_t cudaMemset(void *d, int v, size_t n) {
  if (n) memset(d, v, n);
  return 0;
}
/* Like the runtime, a copy larger than the symbol fails and copies nothing. */
#define cudaMemcpyToSymbol(sym, src, n) \
  ((size_t)(n) <= sizeof(sym) ? (memcpy((void *)&(sym), (src), (n)), 0) : 11)

#endif
