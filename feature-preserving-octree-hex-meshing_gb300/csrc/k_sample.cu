// k_sample.cu -- area-uniform random samples of a triangle mesh on the device, for the uniform-
// sample Hausdorff mode (the vertex-sampled metric of metro_hausdorff.cpp:358-506 evaluated at n
// samples per surface instead of at the vertices).
//
// Sample i of a surface draws three uniform variates u0, u1, u2 from a counter-based generator
// (SplitMix64 of Steele, Lea & Flood 2014, on the 64-bit counters seed + 3i + k), picks the face
// whose cumulative-area interval holds u0 * total area (first face with cdf > u0 * total), and
// places the point at barycentric weights (1 - sqrt(u1), sqrt(u1) (1 - u2), sqrt(u1) u2): the
// same draw for the same (seed, i, surface) on any device, in any launch configuration.
#include <cub/device/device_scan.cuh>

#include "hexopt_common.cuh"
#include "hexopt_kernels.h"

namespace hexopt {

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double unit53(uint64_t z) { return double(z >> 11) * (1.0 / 9007199254740992.0); }

__global__ void k_tri_area(const double *V, const int32_t *F, int64_t nf, double *area) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const double *a = V + 3 * (int64_t)F[3 * f], *b = V + 3 * (int64_t)F[3 * f + 1], *c = V + 3 * (int64_t)F[3 * f + 2];
  const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  const double n0 = e1[1] * e2[2] - e1[2] * e2[1], n1 = e1[2] * e2[0] - e1[0] * e2[2], n2 = e1[0] * e2[1] - e1[1] * e2[0];
  area[f] = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
}

__global__ void k_sample_surface(const double *V, const int32_t *F, const double *cdf, int64_t nf, int64_t n,
                                 uint64_t seed, double *P) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t base = seed + 3ull * (uint64_t)i;
  const double u0 = unit53(splitmix64(base)), u1 = unit53(splitmix64(base + 1)), u2 = unit53(splitmix64(base + 2));
  const double t = u0 * cdf[nf - 1];
  int64_t lo = 0, hi = nf - 1;  // first face with cdf > t
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (cdf[mid] > t) hi = mid;
    else lo = mid + 1;
  }
  const double r1 = sqrt(u1), w0 = 1 - r1, w1 = r1 * (1 - u2), w2 = r1 * u2;
  const double *a = V + 3 * (int64_t)F[3 * lo], *b = V + 3 * (int64_t)F[3 * lo + 1], *c = V + 3 * (int64_t)F[3 * lo + 2];
#pragma unroll
  for (int d = 0; d < 3; d++) P[3 * i + d] = w0 * a[d] + w1 * b[d] + w2 * c[d];
}

size_t sample_scratch_bytes(int64_t nf) {
  size_t tb = 0;
  cub::DeviceScan::InclusiveSum(nullptr, tb, (const double *)nullptr, (double *)nullptr, (int)nf, (cudaStream_t)0);
  return (((size_t)nf * 16 + 255) & ~(size_t)255) + tb;
}

cudaError_t sample_surface(const double *V, const int32_t *F, int64_t nf, int64_t n, uint64_t seed, double *P,
                           void *scratch, size_t scratch_bytes, cudaStream_t st) {
  if (nf <= 0 || n <= 0) return cudaSuccess;
  double *area = static_cast<double *>(scratch), *cdf = area + nf;
  const size_t used = ((size_t)nf * 16 + 255) & ~(size_t)255;
  size_t tb = scratch_bytes - used;
  k_tri_area<<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(V, F, nf, area);
  cudaError_t e = cub::DeviceScan::InclusiveSum(static_cast<char *>(scratch) + used, tb, area, cdf, (int)nf, st);
  if (e != cudaSuccess) return e;
  k_sample_surface<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(V, F, cdf, nf, n, seed, P);
  return cudaGetLastError();
}

}  // namespace hexopt
