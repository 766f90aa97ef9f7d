// k_order.cu -- Morton ordering of a batch's vertex and hex streams on upload, and the gathers
// that move per-vertex / per-hex arrays between the caller's order and the device order.
//
// Keys are (mesh << 32 | 30-bit Morton code) of the vertex position / hex centroid quantised in
// its mesh's bounding box, so one radix sort of the whole batch keeps every mesh's items
// contiguous (in mesh order) and spatially coherent inside the mesh: the hex kernels' corner
// gathers and scatters then hit L2 lines that neighbouring hexes share, whatever order the caller
// numbered its mesh in.
#include <cub/device/device_radix_sort.cuh>

#include "hexopt_common.cuh"
#include "hexopt_kernels.h"

namespace hexopt {

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}
__device__ __forceinline__ uint32_t morton30(const double p[3], const double *box) {
  uint32_t q[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double ext = box[3 + d] - box[d];
    const double t = ext > 0 ? (p[d] - box[d]) / ext : 0.0;
    q[d] = (uint32_t)fmin(fmax(t * 1024.0, 0.0), 1023.0);
  }
  return (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
}
// mesh of a global item: offsets[m] <= i < offsets[m + 1] (n_meshes + 1 offsets)
__device__ __forceinline__ int mesh_of(const int64_t *offsets, int n_meshes, int64_t i) {
  int lo = 0, hi = n_meshes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// vertex keys from the caller's rows (n x 3); box: 6 doubles per mesh
__global__ void k_vertex_keys(const double *rows, int64_t n, const int64_t *voff, int n_meshes, const double *box,
                              unsigned long long *keys, int32_t *vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int m = mesh_of(voff, n_meshes, i);
  const double p[3] = {rows[3 * i], rows[3 * i + 1], rows[3 * i + 2]};
  keys[i] = ((unsigned long long)m << 32) | morton30(p, box + 6 * m);
  vals[i] = (int32_t)i;
}
// hex keys from the centroids (caller's hexes: mesh-local corner ids, 8 per hex)
__global__ void k_hex_keys(const double *rows, const uint32_t *H, int64_t nh, const int64_t *hoff, const int64_t *voff,
                           int n_meshes, const double *box, unsigned long long *keys, int32_t *vals) {
  const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nh) return;
  const int m = mesh_of(hoff, n_meshes, h);
  double c[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int64_t v = voff[m] + H[8 * h + k];
#pragma unroll
    for (int d = 0; d < 3; d++) c[d] += rows[3 * v + d];
  }
#pragma unroll
  for (int d = 0; d < 3; d++) c[d] *= 0.125;
  keys[h] = ((unsigned long long)m << 32) | morton30(c, box + 6 * m);
  vals[h] = (int32_t)h;
}
__global__ void k_invert_perm(const int32_t *new2old, int64_t n, int32_t *old2new) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) old2new[new2old[i]] = (int32_t)i;
}
// hexv (AoSoA) of the device order from the caller's hexes
__global__ void k_hex_perm(const uint32_t *H, const int32_t *hnew2old, const int32_t *vold2new, int64_t nh,
                           const int64_t *hoff, const int64_t *voff, int n_meshes, uint32_t *hexv) {
  const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nh) return;
  const int64_t o = hnew2old[h];
  const int m = mesh_of(hoff, n_meshes, o);
#pragma unroll
  for (int c = 0; c < 8; c++) hexv[hex_idx(h, c)] = (uint32_t)vold2new[voff[m] + H[8 * o + c]];
}
// dst[i] = src[perm[i]] for rows of `width` doubles (perm null = identity)
__global__ void k_gather_rows(const double *src, const int32_t *perm, int64_t n, int width, double *dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s = perm ? perm[i] : i;
  for (int k = 0; k < width; k++) dst[i * width + k] = src[s * width + k];
}
// X (AoS4) of the device order from caller rows: X[i] = rows[new2old[i]]
__global__ void k_rows_to_aos4_perm(const double *rows, const int32_t *new2old, int64_t n, double *X) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s = new2old ? new2old[i] : i;
  X[4 * i] = rows[3 * s]; X[4 * i + 1] = rows[3 * s + 1]; X[4 * i + 2] = rows[3 * s + 2]; X[4 * i + 3] = 0;
}
// caller rows from X (AoS4): rows[old] = X[old2new[old]]
__global__ void k_aos4_to_rows_perm(const double *X, const int32_t *old2new, int64_t n, double *rows) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s = old2new ? old2new[i] : i;
  rows[3 * i] = X[4 * s]; rows[3 * i + 1] = X[4 * s + 1]; rows[3 * i + 2] = X[4 * s + 2];
}

static unsigned grid_of(int64_t n) { return (unsigned)((n + 255) / 256); }

cudaError_t order_batch(const double *rows, const uint32_t *H, int64_t NV, int64_t NH, const int64_t *voff_d,
                        const int64_t *hoff_d, int n_meshes, const double *box_d, int32_t *vnew2old, int32_t *vold2new,
                        int32_t *hnew2old, int32_t *hold2new, void *scratch, size_t scratch_bytes, cudaStream_t st) {
  // scratch: keys_in, keys_out (8 B each per item), vals_in (4 B) and cub's workspace
  const int64_t n = NV > NH ? NV : NH;
  char *sp = static_cast<char *>(scratch);
  auto *k_in = reinterpret_cast<unsigned long long *>(sp);
  auto *k_out = k_in + n;
  auto *v_in = reinterpret_cast<int32_t *>(k_out + n);
  size_t used = (size_t)n * 20;
  used = (used + 255) & ~(size_t)255;  // cub's workspace on a 256-byte boundary
  void *tmp = sp + used;
  size_t tmp_bytes = scratch_bytes - used;
  k_vertex_keys<<<grid_of(NV), 256, 0, st>>>(rows, NV, voff_d, n_meshes, box_d, k_in, v_in);
  cudaError_t e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, v_in, vnew2old, (int)NV, 0, 64, st);
  if (e != cudaSuccess) return e;
  k_invert_perm<<<grid_of(NV), 256, 0, st>>>(vnew2old, NV, vold2new);
  k_hex_keys<<<grid_of(NH), 256, 0, st>>>(rows, H, NH, hoff_d, voff_d, n_meshes, box_d, k_in, v_in);
  e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, v_in, hnew2old, (int)NH, 0, 64, st);
  if (e != cudaSuccess) return e;
  k_invert_perm<<<grid_of(NH), 256, 0, st>>>(hnew2old, NH, hold2new);
  return cudaGetLastError();
}
size_t order_scratch_bytes(int64_t NV, int64_t NH) {
  const int64_t n = NV > NH ? NV : NH;
  size_t tb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tb, (unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                  (int32_t *)nullptr, (int32_t *)nullptr, (int)n, 0, 64, (cudaStream_t)0);
  return (((size_t)n * 20 + 255) & ~(size_t)255) + tb;
}
void launch_hex_perm(const uint32_t *H, const int32_t *hnew2old, const int32_t *vold2new, int64_t nh, const int64_t *hoff,
                     const int64_t *voff, int n_meshes, uint32_t *hexv, cudaStream_t st) {
  if (nh > 0) k_hex_perm<<<grid_of(nh), 256, 0, st>>>(H, hnew2old, vold2new, nh, hoff, voff, n_meshes, hexv);
}
void launch_gather_rows(const double *src, const int32_t *perm, int64_t n, int width, double *dst, cudaStream_t st) {
  if (n > 0) k_gather_rows<<<grid_of(n), 256, 0, st>>>(src, perm, n, width, dst);
}
void launch_rows_to_aos4_perm(const double *rows, const int32_t *new2old, int64_t n, double *X, cudaStream_t st) {
  if (n > 0) k_rows_to_aos4_perm<<<grid_of(n), 256, 0, st>>>(rows, new2old, n, X);
}
void launch_aos4_to_rows_perm(const double *X, const int32_t *old2new, int64_t n, double *rows, cudaStream_t st) {
  if (n > 0) k_aos4_to_rows_perm<<<grid_of(n), 256, 0, st>>>(X, old2new, n, rows);
}

}  // namespace hexopt
