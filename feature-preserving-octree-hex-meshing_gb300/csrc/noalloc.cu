// noalloc.cu -- hexopt_point_face_distance_noalloc: the point-to-surface distance of
// hexopt_point_face_distance (min over faces of vcg's PointDistanceEP, metro_hausdorff's sample
// distance) on caller-owned device arrays, with every piece of scratch -- the triangle soup, the
// LBVH and its build buffers, the radix-sort workspace, the status word -- carved out of one
// file-scope static device array instead of allocated.
//
// Why: cudaMalloc / cudaFree are not free to call everywhere.  cudaFree synchronises the whole
// device, so a caller interleaving this query with latency-sensitive work on other streams
// stalls them all; a caller running under a fixed device-memory budget (a pre-sized pool that
// owns the rest of HBM) cannot have a library take memory behind it; and a caller sitting in a
// tight per-iteration loop does not want allocator traffic every call.  Such callers pass
// device pointers and a stream and get no allocation at all after the first call on a device.
//
// Limits and rules:
//  * capacity: kScratchBytes (80 MiB) per device, enough for a surface of up to kMaxFaces
//    (262,144) triangles; larger surfaces are rejected with an error naming both sizes.  The
//    number of query points is not limited (points and distances stay in the caller's arrays).
//  * set-up: the first call on a device resolves the scratch's address (cudaGetSymbolAddress,
//    checked), which loads this file's module and with it the 80 MiB array; a caller that must
//    not see that happen mid-stream makes one call (any size, e.g. one point) beforehand.
//    That holds under CUDA's lazy module loading (the default).  With CUDA_MODULE_LOADING=EAGER
//    the module, and the 80 MiB with it, is loaded on every device when a context first loads
//    this library, whether or not this entry point is ever called.
//  * one scratch per device, shared by every call: calls that overlap in time on one device --
//    from two streams or two host threads -- race on it and give wrong results.  Serialise them
//    (one stream, or an event between them).  The call itself is synchronous on `stream`.
//  * zeroing: the refit counters and the status word must start at zero; the call clears them
//    with cudaMemsetAsync on `stream` before use, so nothing is assumed about the array between
//    calls.
#include <cuda_runtime.h>
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/hexopt_gpu.h"
#include "hexopt_bvh.h"

using namespace hexopt;

namespace {

constexpr size_t kScratchBytes = size_t(80) << 20;
constexpr int64_t kMaxFaces = int64_t(1) << 18;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

void *g_base[kMaxDevices];
std::mutex g_mu;

void set_err(char *buf, size_t len, const char *fmt, ...) {
  if (!buf || len == 0) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, len, fmt, ap);
  va_end(ap);
}

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// Triangle soup (9 doubles per face) from the caller's vertices and faces; an out-of-range
// vertex id sets status bit 1 and writes zeros instead of reading.
__global__ void k_gather_tris(const double *V, int64_t nv, const int32_t *F, int64_t nf, double *tri, int *status) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  for (int c = 0; c < 3; c++) {
    const int32_t v = F[3 * f + c];
    const bool ok = v >= 0 && v < nv;
    if (!ok) atomicOr(status, 1);
    for (int d = 0; d < 3; d++) tri[9 * f + 3 * c + d] = ok ? V[3 * (int64_t)v + d] : 0.0;
  }
}

// Bounding box of the face centroids (the Morton frame), one block: centroid (a + b + c) / 3 per
// axis, as the allocating build computes it, so both builds make the same tree.
__global__ void __launch_bounds__(1024) k_centroid_box(const double *tri, int64_t nf, double *box6) {
  __shared__ double s[6][32];
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t f = threadIdx.x; f < nf; f += blockDim.x)
    for (int c = 0; c < 3; c++) {
      const double cen = (tri[9 * f + c] + tri[9 * f + 3 + c] + tri[9 * f + 6 + c]) / 3;
      lo[c] = fmin(lo[c], cen);
      hi[c] = fmax(hi[c], cen);
    }
  for (int o = 16; o > 0; o >>= 1)
    for (int c = 0; c < 3; c++) {
      lo[c] = fmin(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = fmax(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (lane == 0)
    for (int c = 0; c < 3; c++) { s[c][w] = lo[c]; s[3 + c][w] = hi[c]; }
  __syncthreads();
  if (w == 0) {
    for (int c = 0; c < 3; c++) {
      lo[c] = lane < nw ? s[c][lane] : INFINITY;
      hi[c] = lane < nw ? s[3 + c][lane] : -INFINITY;
    }
    for (int o = 16; o > 0; o >>= 1)
      for (int c = 0; c < 3; c++) {
        lo[c] = fmin(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
        hi[c] = fmax(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
      }
    if (lane == 0)
      for (int c = 0; c < 3; c++) { box6[c] = lo[c]; box6[3 + c] = hi[c]; }
  }
}

// Scratch layout for nf faces (offsets from the 256-byte aligned base, each 256-byte aligned).
struct Layout {
  size_t tri, keys, keys2, child, parent, box, leaf_face, counters, node, leafd, box6, status, sort, end;
};

Layout layout(int64_t nf, size_t sort_bytes) {
  const size_t n = (size_t)nf, ni = (size_t)std::max<int64_t>(nf - 1, 1), nn = 2 * n - 1;
  Layout L;
  size_t o = 0;
  L.tri = o; o = up256(o + sizeof(double) * 9 * n);
  L.keys = o; o = up256(o + sizeof(unsigned long long) * n);
  L.keys2 = o; o = up256(o + sizeof(unsigned long long) * n);
  L.child = o; o = up256(o + sizeof(int32_t) * 2 * ni);
  L.parent = o; o = up256(o + sizeof(int32_t) * nn);
  L.box = o; o = up256(o + sizeof(float) * 6 * nn);
  L.leaf_face = o; o = up256(o + sizeof(int32_t) * n);
  L.counters = o; o = up256(o + sizeof(unsigned) * ni);
  L.node = o; o = up256(o + sizeof(float4) * 4 * ni);
  L.leafd = o; o = up256(o + sizeof(float4) * 3 * n);
  L.box6 = o; o = up256(o + sizeof(double) * 6);
  L.status = o; o = up256(o + sizeof(int));
  L.sort = o; o = up256(o + sort_bytes);
  L.end = o;
  return L;
}

}  // namespace

#define NA_CK(call, what)                                                                               \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess) {                                                                           \
      set_err(err, err_len, "point_face_distance_noalloc: %s: %s", what, cudaGetErrorString(e_));      \
      rc = HEXOPT_ERR_CUDA;                                                                            \
      goto done;                                                                                       \
    }                                                                                                  \
  } while (0)

extern "C" int hexopt_point_face_distance_noalloc(int device, void *stream, int64_t np, const double *P_dev,
                                                  int64_t nv, const double *V_dev, int64_t nf,
                                                  const int32_t *F_dev, double *dist_dev, char *err,
                                                  size_t err_len) {
  if (err && err_len) err[0] = 0;
  if (device < 0 || device >= kMaxDevices) {
    set_err(err, err_len, "point_face_distance_noalloc: device %d out of range", device);
    return HEXOPT_ERR_ARG;
  }
  if (np < 0 || nv <= 0 || nf <= 0 || !V_dev || !F_dev || (np > 0 && (!P_dev || !dist_dev))) {
    set_err(err, err_len, "point_face_distance_noalloc: bad arguments (np %lld, nv %lld, nf %lld)", (long long)np,
            (long long)nv, (long long)nf);
    return HEXOPT_ERR_ARG;
  }
  if (nf > kMaxFaces || nv > INT32_MAX) {
    set_err(err, err_len,
            "point_face_distance_noalloc: %lld faces exceed the static scratch (%zu MiB, up to %lld faces); "
            "use hexopt_point_face_distance",
            (long long)nf, kScratchBytes >> 20, (long long)kMaxFaces);
    return HEXOPT_ERR_UNSUPPORTED;
  }
  int rc = HEXOPT_OK, prev = -1, st_host = 0;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char *base = nullptr;
  size_t sort_bytes = 0;
  Layout L{};
  BvhDev b{};
  double box6[6];
  NA_CK(cudaGetDevice(&prev), "cudaGetDevice");
  NA_CK(cudaSetDevice(device), "cudaSetDevice");
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[device]) {
      void *p = nullptr;
      NA_CK(cudaGetSymbolAddress(&p, g_scratch), "cudaGetSymbolAddress (scratch set-up)");
      if (!p || ((uintptr_t)p & 255u)) {
        set_err(err, err_len, "point_face_distance_noalloc: scratch address %p is not 256-byte aligned", p);
        rc = HEXOPT_ERR_CUDA;
        goto done;
      }
      g_base[device] = p;
    }
    base = (unsigned char *)g_base[device];
  }
  // radix-sort workspace size for nf keys (a size query: no allocation)
  NA_CK(cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, (unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                       (int)nf, 0, 64, st),
        "radix-sort workspace query");
  L = layout(nf, sort_bytes);
  if (L.end > kScratchBytes) {
    set_err(err, err_len,
            "point_face_distance_noalloc: %lld faces need %zu bytes of scratch, the static scratch holds %zu",
            (long long)nf, L.end, kScratchBytes);
    rc = HEXOPT_ERR_UNSUPPORTED;
    goto done;
  }
  b.n = (int32_t)nf;
  b.tri = (const double *)(base + L.tri);
  b.child = (const int32_t *)(base + L.child);
  b.box = (const float *)(base + L.box);
  b.leaf_face = (const int32_t *)(base + L.leaf_face);
  b.node = (const float4 *)(base + L.node);
  b.leafd = (const float4 *)(base + L.leafd);
  NA_CK(cudaMemsetAsync(base + L.status, 0, sizeof(int), st), "clear status");
  NA_CK(cudaMemsetAsync(base + L.counters, 0, sizeof(unsigned) * std::max<int64_t>(nf - 1, 1), st), "clear counters");
  k_gather_tris<<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(V_dev, nv, F_dev, nf, (double *)(base + L.tri),
                                                             (int *)(base + L.status));
  k_centroid_box<<<1, 1024, 0, st>>>((const double *)(base + L.tri), nf, (double *)(base + L.box6));
  NA_CK(cudaGetLastError(), "gather launch");
  NA_CK(cudaMemcpyAsync(box6, base + L.box6, sizeof box6, cudaMemcpyDeviceToHost, st), "read centroid box");
  NA_CK(cudaStreamSynchronize(st), "centroid box");
  bvh_morton(b, box6, box6 + 3, (unsigned long long *)(base + L.keys), st);
  NA_CK(cub::DeviceRadixSort::SortKeys(base + L.sort, sort_bytes, (unsigned long long *)(base + L.keys),
                                       (unsigned long long *)(base + L.keys2), (int)nf, 0, 64, st),
        "radix sort");
  bvh_karras((int)nf, (const unsigned long long *)(base + L.keys2), (int32_t *)(base + L.child),
             (int32_t *)(base + L.parent), (int32_t *)(base + L.leaf_face), st);
  bvh_refit(b, (float *)(base + L.box), (const int32_t *)(base + L.parent), (unsigned *)(base + L.counters),
            (float4 *)(base + L.node), (float4 *)(base + L.leafd), st);
  if (np > 0) launch_ep_points(b, P_dev, nullptr, np, INFINITY, dist_dev, (int *)(base + L.status), st);
  NA_CK(cudaGetLastError(), "build / query launch");
  NA_CK(cudaMemcpyAsync(&st_host, base + L.status, sizeof(int), cudaMemcpyDeviceToHost, st), "read status");
  NA_CK(cudaStreamSynchronize(st), "query");
  if (st_host & 1) {
    set_err(err, err_len, "point_face_distance_noalloc: face vertex id out of range [0, %lld)", (long long)nv);
    rc = HEXOPT_ERR_ARG;
  } else if (st_host & 8) {
    set_err(err, err_len, "point_face_distance_noalloc: BVH traversal stack overflow");
    rc = HEXOPT_ERR_NUMERIC;
  }
done:
  if (prev >= 0) cudaSetDevice(prev);
  return rc;
}
