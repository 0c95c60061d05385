/*
 * Small FP64 and integer kernels around the transport: the emission-source
 * list of the two-phase fluorescence scheme and the final normalisations.
 * Built with -fmad=false so every double operation rounds once, as the CPU
 * oracle's do.
 *
 * Emission list.  The reference runs one full simulation per voxel whose
 * label has albedof < 1 and weights its images by
 *   eY (1 - albedof) PHD_v / (N_v (2^32-1)),  PHD_v = fhd_v / ((2^32-1) N)
 * (CUDAMCFLmain.cu:550-577).  Here every such voxel with a non-zero weight
 * becomes an entry of one emission job; its weight is kept as the 64-bit
 * fixed-point integer q_v = rint(eY (1 - albedof) PHD_v f_v 2^40) (f_v the
 * optional fluorophore map), and exits add weight x q_v into 128-bit integer
 * images, so the emission images stay order-independent integers until the
 * FP64 normalisation.  The list keeps increasing voxel order: entry i holds
 * photons [i N_v, (i+1) N_v) of the emission job.
 */
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <utility>

#include "engine_types.h"

namespace {

constexpr int kPrepThreads = 256;
constexpr int kPrepPerThread = 16;
constexpr int kPrepTile = kPrepThreads * kPrepPerThread;

__device__ __forceinline__ uint64_t voxel_weight_q(uint32_t v, const uint8_t *labels, const float2 *fl,
                                                   const unsigned long long *fhd, const float *fmap,
                                                   unsigned long long photons) {
  const float2 f = fl[labels[v]]; /* eY, albedof */
  if (!(f.y < 1.0f)) return 0ull;
  const double fx = (double)fhd[v] / (double)(0xFFFFFFFFull * photons);
  double wv = (double)f.x * (double)(1 - f.y) * fx;
  if (fmap) wv = wv * (double)fmap[v];
  const double qs = rint(wv * 0x1p40);
  if (!(qs > 0.0)) return 0ull;
  return qs >= 18446744073709551615.0 ? 0xFFFFFFFFFFFFFFFFull : (uint64_t)qs;
}

__global__ void __launch_bounds__(kPrepThreads) prep_count(const uint8_t *labels, const float2 *fl,
                                                           const unsigned long long *fhd, const float *fmap,
                                                           uint32_t total, unsigned long long photons,
                                                           uint32_t *block_counts) {
  __shared__ uint32_t warp_sums[kPrepThreads / 32];
  const uint32_t base = blockIdx.x * kPrepTile + threadIdx.x * kPrepPerThread;
  uint32_t c = 0;
  for (int i = 0; i < kPrepPerThread; ++i) {
    const uint32_t v = base + i;
    if (v < total && voxel_weight_q(v, labels, fl, fhd, fmap, photons) != 0ull) ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w = 0; w < kPrepThreads / 32; ++w) s += warp_sums[w];
    block_counts[blockIdx.x] = s;
  }
}

/* Single block: exclusive scan of the block counts in place; writes the
 * list length, the emission job's photon count and its ticket end. */
__global__ void __launch_bounds__(1024) prep_scan(uint32_t *block_counts, uint32_t nblocks, uint32_t per_voxel,
                                                  unsigned long long *list_len, McflJob *job,
                                                  unsigned long long *ticket_end) {
  __shared__ unsigned long long part[1024];
  const uint32_t per = (nblocks + 1023) / 1024;
  const uint32_t b0 = threadIdx.x * per;
  unsigned long long s = 0;
  for (uint32_t i = 0; i < per; ++i)
    if (b0 + i < nblocks) s += block_counts[b0 + i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    unsigned long long v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0ull;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned long long run = threadIdx.x ? part[threadIdx.x - 1] : 0ull;
  for (uint32_t i = 0; i < per; ++i)
    if (b0 + i < nblocks) {
      const uint32_t c = block_counts[b0 + i];
      block_counts[b0 + i] = (uint32_t)run;
      run += c;
    }
  if (threadIdx.x == 1023) {
    const unsigned long long n = part[1023];
    *list_len = n;
    job->photons = n * per_voxel;
    *ticket_end = n * per_voxel;
  }
}

__global__ void __launch_bounds__(kPrepThreads) prep_scatter(const uint8_t *labels, const float2 *fl,
                                                             const unsigned long long *fhd, const float *fmap,
                                                             uint32_t total, unsigned long long photons,
                                                             const uint32_t *block_offsets, uint32_t *vox,
                                                             uint64_t *q) {
  __shared__ uint32_t warp_sums[kPrepThreads / 32];
  const uint32_t base = blockIdx.x * kPrepTile + threadIdx.x * kPrepPerThread;
  uint64_t qs[kPrepPerThread];
  uint32_t c = 0;
  for (int i = 0; i < kPrepPerThread; ++i) {
    const uint32_t v = base + i;
    qs[i] = v < total ? voxel_weight_q(v, labels, fl, fhd, fmap, photons) : 0ull;
    if (qs[i]) ++c;
  }
  /* exclusive scan of c over the block, in thread order */
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = c;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (unsigned)o) incl += v;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  uint32_t woff = 0;
  for (unsigned w = 0; w < warp; ++w) woff += warp_sums[w];
  uint32_t off = block_offsets[blockIdx.x] + woff + incl - c;
  for (int i = 0; i < kPrepPerThread; ++i)
    if (qs[i]) {
      vox[off] = base + i;
      q[off] = qs[i];
      ++off;
    }
}

__global__ void normalize_u64(const unsigned long long *raw, double *out, size_t n, double scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (double)raw[i] / scale;
}

/* raw[i] / scales[i / seg_len]: one normalisation per job of a batch */
__global__ void normalize_segments(const unsigned long long *raw, double *out, size_t seg_len, size_t n,
                                   const double *scales) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (double)raw[i] / scales[i / seg_len];
}

__global__ void normalize_phd(const unsigned long long *raw, double *out, size_t n, unsigned long long photons) {
  const double den = (double)(0xFFFFFFFFull * photons);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (double)raw[i] / den;
}

__global__ void normalize_128(const unsigned long long *raw, double *out, size_t n, double norm) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v = (double)raw[2 * i + 1] * 18446744073709551616.0 + (double)raw[2 * i];
    out[i] = v * 0x1p-40 / norm;
  }
}

int grid_for(size_t n) {
  size_t g = (n + 255) / 256;
  return (int)(g > 4096 ? 4096 : (g ? g : 1));
}

} // namespace

namespace mcfl {
size_t emission_prep_blocks(uint32_t total) { return (total + kPrepTile - 1) / kPrepTile; }
} // namespace mcfl

extern "C" cudaError_t mcfl_launch_emission_prep(const uint8_t *labels, const float2 *fl,
                                                 const unsigned long long *fhd, const float *fmap, uint32_t total,
                                                 unsigned long long photons_exc, uint32_t per_voxel,
                                                 uint32_t *block_counts, uint32_t *vox, uint64_t *q,
                                                 unsigned long long *list_len, McflJob *job,
                                                 unsigned long long *ticket_end, cudaStream_t s) {
  const uint32_t nb = (uint32_t)mcfl::emission_prep_blocks(total);
  prep_count<<<nb, kPrepThreads, 0, s>>>(labels, fl, fhd, fmap, total, photons_exc, block_counts);
  prep_scan<<<1, 1024, 0, s>>>(block_counts, nb, per_voxel, list_len, job, ticket_end);
  prep_scatter<<<nb, kPrepThreads, 0, s>>>(labels, fl, fhd, fmap, total, photons_exc, block_counts, vox, q);
  return cudaGetLastError();
}

extern "C" cudaError_t mcfl_launch_normalize_u64(const unsigned long long *raw, double *out, size_t n, double scale,
                                                 cudaStream_t s) {
  normalize_u64<<<grid_for(n), 256, 0, s>>>(raw, out, n, scale);
  return cudaGetLastError();
}

extern "C" cudaError_t mcfl_launch_normalize_segments(const unsigned long long *raw, double *out, size_t seg_len,
                                                      size_t n_seg, const double *scales, cudaStream_t s) {
  const size_t n = seg_len * n_seg;
  normalize_segments<<<grid_for(n), 256, 0, s>>>(raw, out, seg_len, n, scales);
  return cudaGetLastError();
}

extern "C" cudaError_t mcfl_launch_normalize_phd(const unsigned long long *raw, double *out, size_t n,
                                                 unsigned long long photons, cudaStream_t s) {
  normalize_phd<<<grid_for(n), 256, 0, s>>>(raw, out, n, photons);
  return cudaGetLastError();
}

extern "C" cudaError_t mcfl_launch_normalize_128(const unsigned long long *raw, double *out, size_t n, double norm,
                                                 cudaStream_t s) {
  normalize_128<<<grid_for(n), 256, 0, s>>>(raw, out, n, norm);
  return cudaGetLastError();
}

/* ------------------------------------------------ free-radius map
 * For voxel-boundary stepping: the free radius of a voxel is the largest
 * r <= MCFL_FREE_MAX such that every voxel of the grid within Chebyshev
 * distance r of it carries its label (the transport kernel clips the cube
 * to the grid).  It is 0 next to a different label (26 neighbours inside the
 * grid); elsewhere it is the Chebyshev distance to the nearest such voxel,
 * capped.  Built by Jacobi
 * relaxation: after k sweeps of r = min(r, 1 + min over the 26 neighbours)
 * every radius up to k is exact, so MCFL_FREE_MAX - 1 sweeps give the capped
 * map.  Packed with the label as label | r << 8, one 2-byte load per voxel
 * crossing. */

namespace {

constexpr int kFreeThreads = 256;

__global__ void free_init(const uint8_t *__restrict__ labels, int nx, int ny, int nz, uint8_t *__restrict__ r) {
  const size_t n = (size_t)nx * ny * nz;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((size_t)nx * ny));
    bool edge = false;
    const uint8_t l = labels[i];
    for (int c = 0; c < 27 && !edge; ++c) {
      const int u = x + c % 3 - 1, v = y + (c / 3) % 3 - 1, w = z + c / 9 - 1;
      if (u < 0 || v < 0 || w < 0 || u >= nx || v >= ny || w >= nz) continue;
      edge = labels[(size_t)u + (size_t)nx * ((size_t)v + (size_t)ny * w)] != l;
    }
    r[i] = edge ? 0 : MCFL_FREE_MAX;
  }
}

__global__ void free_relax(const uint8_t *__restrict__ in, int nx, int ny, int nz, uint8_t *__restrict__ out) {
  const size_t n = (size_t)nx * ny * nz;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    int r = in[i];
    if (r != 0) {
      const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((size_t)nx * ny));
      for (int c = 0; c < 27; ++c) {
        const int u = x + c % 3 - 1, v = y + (c / 3) % 3 - 1, w = z + c / 9 - 1;
        if (u < 0 || v < 0 || w < 0 || u >= nx || v >= ny || w >= nz) continue;
        r = min(r, 1 + (int)in[(size_t)u + (size_t)nx * ((size_t)v + (size_t)ny * w)]);
      }
    }
    out[i] = (uint8_t)r;
  }
}

__global__ void free_pack(const uint8_t *__restrict__ labels, const uint8_t *__restrict__ r, size_t n,
                          uint16_t *__restrict__ lab16) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    lab16[i] = (uint16_t)(labels[i] | (r[i] << 8));
}

} // namespace

extern "C" cudaError_t mcfl_launch_free_map(const uint8_t *labels, int nx, int ny, int nz, uint8_t *tmp,
                                           uint16_t *lab16, cudaStream_t s) {
  const size_t n = (size_t)nx * ny * nz;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t want = (n + kFreeThreads - 1) / kFreeThreads;
  const int blocks = (int)std::min<size_t>(want, (size_t)(sms > 0 ? sms : 1) * 8);
  uint8_t *a = tmp, *b = tmp + n;
  free_init<<<blocks, kFreeThreads, 0, s>>>(labels, nx, ny, nz, a);
  for (int k = 1; k < MCFL_FREE_MAX; ++k) {
    free_relax<<<blocks, kFreeThreads, 0, s>>>(a, nx, ny, nz, b);
    std::swap(a, b);
  }
  free_pack<<<blocks, kFreeThreads, 0, s>>>(labels, a, n, lab16);
  return cudaGetLastError();
}
