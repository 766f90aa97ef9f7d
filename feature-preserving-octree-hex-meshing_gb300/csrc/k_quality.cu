// k_quality.cu -- per-hex scaled Jacobian (scaled_jacobian, global_functions.cpp:2309-2356 with
// a_jacobian :2422-2442), the feature-weight schedule and HBM layout conversions.
//
// The scaled Jacobian is evaluated in FP64 with explicitly rounded products and sums in the
// reference's evaluation order, so corner values and inversion flags are bit-identical to the
// FP64 oracle on the same positions.
#include "hexopt_common.cuh"
#include "hexopt_kernels.h"
#include "hexopt_elem.cuh"

namespace hexopt {

__device__ __forceinline__ double norm3_rn(double a, double b, double c) {
  return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c)));
}

template <int K>
__device__ __forceinline__ double corner_sj(const double *X, const uint32_t hv[8]) {
  const double *p0 = X + 4 * (int64_t)hv[tet_v(K, 0)];
  double J[3][3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const double *q = X + 4 * (int64_t)hv[tet_v(K, j + 1)];
#pragma unroll
    for (int r = 0; r < 3; r++) J[r][j] = __dmul_rn(__dsub_rn(q[r], p0[r]), 0.5);
  }
  const double n1 = norm3_rn(J[0][0], J[1][0], J[2][0]);
  const double n2 = norm3_rn(J[0][1], J[1][1], J[2][1]);
  const double n3 = norm3_rn(J[0][2], J[1][2], J[2][2]);
  const double d = det3_rn(J);
  if (fabs(n1) < 1.e-7 || fabs(n2) < 1.e-7 || fabs(n3) < 1.e-7) return d;  // Precision (global_types.h:23)
  return __ddiv_rn(d, __dmul_rn(__dmul_rn(n1, n2), n3));
}

__global__ void __launch_bounds__(128) k_sj(KArgs a, double *V_Js, double *H_Js) {
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  double mn[1] = {1.0}, acc[2] = {0, 0};
  if (h < sg.end) {
    uint32_t hv[8];
#pragma unroll
    for (int c = 0; c < 8; c++) hv[c] = __ldg(a.hexv + hex_idx(h, c));
    double v[8];
    v[0] = corner_sj<0>(a.X, hv); v[1] = corner_sj<1>(a.X, hv); v[2] = corner_sj<2>(a.X, hv);
    v[3] = corner_sj<3>(a.X, hv); v[4] = corner_sj<4>(a.X, hv); v[5] = corner_sj<5>(a.X, hv);
    v[6] = corner_sj<6>(a.X, hv); v[7] = corner_sj<7>(a.X, hv);
    double hm = 1.0;
#pragma unroll
    for (int k = 0; k < 8; k++) if (hm > v[k]) hm = v[k];
    if (V_Js) {
#pragma unroll
      for (int k = 0; k < 8; k++) V_Js[8 * h + k] = v[k];
    }
    H_Js[h] = hm;
    mn[0] = hm;
    acc[0] = hm;
    acc[1] = hm < 0 ? 1.0 : 0.0;
  }
  __shared__ double smem[2][32];
  block_min<1>(mn, smem);
  double m0 = mn[0];
  block_sum<2>(acc, smem);
  double out[3] = {m0, acc[0], acc[1]};
  if (publish_partials<3>(out, a.partials, blockIdx.x, a.counters + sg.mesh, md.nhblk)) {
    double m = gather_partials_min(a.partials, md.hblk0, md.nhblk, 3, 0, smem);
    double g[2];  // components 1 and 2 of 3
    gather_partials_sums<2>(a.partials + 1, md.hblk0, md.nhblk, 3, g, smem);
    const double s = g[0], c = g[1];
    if (threadIdx.x == 0) {
      MeshScalars &S = a.sc[sg.mesh];
      S.sj_min = fmin(m, 1.0);
      S.sj_sum = s;
      S.n_inv = (int64_t)c;
      a.counters[sg.mesh] = 0;
    }
  }
}

// deviation_Jacobian = mean((H_Js - ave)^2), second pass as in the reference
__global__ void __launch_bounds__(128) k_sj_dev(KArgs a, const double *H_Js) {
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  MeshScalars &S = a.sc[sg.mesh];
  const double ave = S.sj_sum / (double)md.nh;
  double acc[1] = {0};
  if (h < sg.end) {
    const double d = H_Js[h] - ave;
    acc[0] = d * d;
  }
  __shared__ double smem[1][32];
  block_sum<1>(acc, smem);
  if (publish_partials<1>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nhblk)) {
    double s = gather_partials_sum(a.partials, md.hblk0, md.nhblk, 1, 0, smem);
    if (threadIdx.x == 0) {
      S.sj_dev = s / (double)md.nh;
      a.counters[sg.mesh] = 0;
    }
  }
}

// In-loop quality check of the mixed mode: corner scaled Jacobians in FP32 from the FP32 hi/lo edge
// frame; a corner whose FP32 value is within 1e-4 of zero (its sign, i.e. the inversion flag, is
// in doubt) or whose edges are near the Precision guard is re-evaluated bit-exactly in FP64.
// Per mesh: min, sum and inverted count (the deviation pass is not part of the check).
// The FP32 minimum (fast corners) and the FP64 minimum (re-evaluated corners) are kept apart so
// the per-corner minimum stays on the FP32 pipes; a corner re-evaluated in FP64 is rare.
template <int K>
__device__ __forceinline__ void corner_sj_fast(const float E12[12][3], const double *X, const uint32_t hv[8],
                                               float &m32, double &m64) {
  float E[3][3];
  tet_E12<K>(E12, E);
  const float n1 = sqrtf(E[0][0] * E[0][0] + E[1][0] * E[1][0] + E[2][0] * E[2][0]);
  const float n2 = sqrtf(E[0][1] * E[0][1] + E[1][1] * E[1][1] + E[2][1] * E[2][1]);
  const float n3 = sqrtf(E[0][2] * E[0][2] + E[1][2] * E[1][2] + E[2][2] * E[2][2]);
  const float sj = det3(E) / (n1 * n2 * n3);
  if (fabsf(sj) < 1e-4f || fminf(n1, fminf(n2, n3)) < 1e-5f || !(fabsf(sj) <= 2.f)) m64 = fmin(m64, corner_sj<K>(X, hv));
  else m32 = fminf(m32, sj);
}

__global__ void __launch_bounds__(128) k_sj_fast(KArgs a) {
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  double mn[1] = {1.0}, acc[2] = {0, 0};
  if (h < sg.end) {
    uint32_t hv[8];
#pragma unroll
    for (int c = 0; c < 8; c++) hv[c] = __ldg(a.hexv + hex_idx(h, c));
    float E12[12][3];
    hex_edges_split(a.X32, hv, E12);
    float m32 = 1.f;
    double m64 = 1.0;
    corner_sj_fast<0>(E12, a.X, hv, m32, m64); corner_sj_fast<1>(E12, a.X, hv, m32, m64);
    corner_sj_fast<2>(E12, a.X, hv, m32, m64); corner_sj_fast<3>(E12, a.X, hv, m32, m64);
    corner_sj_fast<4>(E12, a.X, hv, m32, m64); corner_sj_fast<5>(E12, a.X, hv, m32, m64);
    corner_sj_fast<6>(E12, a.X, hv, m32, m64); corner_sj_fast<7>(E12, a.X, hv, m32, m64);
    const double hm = fmin(double(m32), m64);
    mn[0] = hm;
    acc[0] = hm;
    acc[1] = hm < 0 ? 1.0 : 0.0;
  }
  __shared__ double smem[2][32];
  block_min<1>(mn, smem);
  double m0 = mn[0];
  block_sum<2>(acc, smem);
  // plain store of the block's partials: the per-mesh reduction is a separate launch, which
  // spares each of the many short blocks a fence and an atomic
  if (threadIdx.x == 0) {
    a.partials[3 * (int64_t)blockIdx.x] = m0;
    a.partials[3 * (int64_t)blockIdx.x + 1] = acc[0];
    a.partials[3 * (int64_t)blockIdx.x + 2] = acc[1];
  }
}

// One block of 512 per mesh: fixed-order reduction of the mesh's k_sj_fast partials.
__global__ void __launch_bounds__(512) k_sj_fast_finish(KArgs a) {
  const int m = blockIdx.x;
  const MeshDesc md = a.mesh[m];
  __shared__ double smem[2][32];
  const double mn = gather_partials_min(a.partials, md.hblk0, md.nhblk, 3, 0, smem);
  double g[2];  // components 1 and 2 of 3
  gather_partials_sums<2>(a.partials + 1, md.hblk0, md.nhblk, 3, g, smem);
  if (threadIdx.x == 0) {
    MeshScalars &S = a.sc[m];
    S.sj_min = fmin(mn, 1.0);
    S.sj_sum = g[0];
    S.n_inv = (int64_t)g[1];
  }
}

void launch_sj_check(const KArgs &a, int64_t hblk, cudaStream_t st) {
  k_sj_fast<<<(unsigned)hblk, a.hthreads, 0, st>>>(a);
  k_sj_fast_finish<<<(unsigned)a.n_meshes, 512, 0, st>>>(a);
}

void launch_scaled_jacobian(const KArgs &a, int64_t hblk, double *V_Js, double *H_Js, cudaStream_t st) {
  k_sj<<<(unsigned)hblk, a.hthreads, 0, st>>>(a, V_Js, H_Js);
  k_sj_dev<<<(unsigned)hblk, a.hthreads, 0, st>>>(a, H_Js);
}

// fc.lamda_T = fc.lamda_L = fc.lamda_C = min(LAMDA * max(Eq / Es * lamda_C, 1), BOUND)
// (grid_hex_meshing.cpp:3865-3869)
__global__ void k_fa_schedule(MeshScalars *sc, int n, double lamda0, double bound) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  MeshScalars &S = sc[m];
  if (!S.max_sat) {
    const double l = fmin(lamda0 * fmax(S.eq / S.es * S.lamda_C, 1.0), bound);
    S.lamda_C = S.lamda_T = S.lamda_L = l;
  }
  S.fa_iter += 1;
}
void launch_fa_schedule(MeshScalars *sc, int n_meshes, double lamda0, double bound, cudaStream_t st) {
  k_fa_schedule<<<(n_meshes + 127) / 128, 128, 0, st>>>(sc, n_meshes, lamda0, bound);
}

// ---------------------------------------------------------------------------- layout
__global__ void k_rows_to_aos4(const double *src, double *dst, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[4 * i] = src[3 * i]; dst[4 * i + 1] = src[3 * i + 1]; dst[4 * i + 2] = src[3 * i + 2]; dst[4 * i + 3] = 0;
}
__global__ void k_aos4_to_rows(const double *src, double *dst, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[3 * i] = src[4 * i]; dst[3 * i + 1] = src[4 * i + 1]; dst[3 * i + 2] = src[4 * i + 2];
}
// src: hexes of one mesh, mesh-local ids; writes global ids into the AoSoA array
__global__ void k_hex_to_aosoa(const uint32_t *src, int64_t h0, int64_t nh, uint32_t voff, uint32_t *dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nh) return;
  const int64_t h = h0 + i;
#pragma unroll
  for (int c = 0; c < 8; c++) dst[hex_idx(h, c)] = src[8 * i + c] + voff;
}

void launch_rows_to_aos4(const double *src, double *dst, int64_t n, cudaStream_t st) {
  if (n > 0) k_rows_to_aos4<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n);
}
__global__ void k_split_pos(const double *X, float *X32, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  store_split(X32, i, X[4 * i], X[4 * i + 1], X[4 * i + 2]);
}
void launch_split_pos(const double *X, float *X32, int64_t n, cudaStream_t st) {
  if (n > 0) k_split_pos<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(X, X32, n);
}
void launch_aos4_to_rows(const double *src, double *dst, int64_t n, cudaStream_t st) {
  if (n > 0) k_aos4_to_rows<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, dst, n);
}
void launch_hex_to_aosoa_mesh(const uint32_t *src, int64_t h0, int64_t nh, uint32_t voff, uint32_t *dst,
                              cudaStream_t st) {
  if (nh > 0) k_hex_to_aosoa<<<(unsigned)((nh + 255) / 256), 256, 0, st>>>(src, h0, nh, voff, dst);
}

}  // namespace hexopt
