// hexopt_elem.cuh -- per-hex element helpers shared by the SLIM and adjoint kernels: vertex
// gathers (AoS4), corner-tet edge matrices, the cube-corner signed permutation J = E R_k^T / s and
// its transpose for scattering forces, and the general (own-shape) J = E B.
#pragma once
#include "hexopt_common.cuh"
#include "hexopt_kernels.h"

namespace hexopt {

// ------------------------------------------------------------------------------- helpers
__device__ __forceinline__ void load_pos(const double *X, uint32_t v, double p[3]) {
  const double2 a = __ldg(reinterpret_cast<const double2 *>(X + 4 * (int64_t)v));
  const double b = __ldg(X + 4 * (int64_t)v + 2);
  p[0] = a.x; p[1] = a.y; p[2] = b;
}
template <typename T>
__device__ __forceinline__ void load_vec(const T *Y, uint32_t v, T p[3]) {
  p[0] = Y[4 * (int64_t)v]; p[1] = Y[4 * (int64_t)v + 1]; p[2] = Y[4 * (int64_t)v + 2];
}
__device__ __forceinline__ void load_vec(const float *Y, uint32_t v, float p[3]) {
  const float4 a = *reinterpret_cast<const float4 *>(Y + 4 * (int64_t)v);
  p[0] = a.x; p[1] = a.y; p[2] = a.z;
}
__device__ __forceinline__ void atomic_add3(double *Y, uint32_t v, double a, double b, double c) {
  atomicAdd(Y + 4 * (int64_t)v, a); atomicAdd(Y + 4 * (int64_t)v + 1, b); atomicAdd(Y + 4 * (int64_t)v + 2, c);
}
__device__ __forceinline__ void atomic_add3(float *Y, uint32_t v, float a, float b, float c) {
  atomicAdd(reinterpret_cast<float4 *>(Y + 4 * (int64_t)v), make_float4(a, b, c, 0.f));
}

// Edge matrix of corner tet k as columns (E[:, j] = P[tet_v(k,j+1)] - P[tet_v(k,0)]), from the
// hex corner gather hv[].  Positions are FP64; the subtraction happens in FP64 before any cast.
template <int K>
__device__ __forceinline__ void tet_edges(const double *X, const uint32_t hv[8], double E[3][3]) {
  double p0[3];
  load_pos(X, hv[tet_v(K, 0)], p0);
#pragma unroll
  for (int j = 0; j < 3; j++) {
    double q[3];
    load_pos(X, hv[tet_v(K, j + 1)], q);
    E[0][j] = q[0] - p0[0]; E[1][j] = q[1] - p0[1]; E[2][j] = q[2] - p0[2];
  }
}
template <int K, typename T>
__device__ __forceinline__ void tet_edges_vec(const T *Y, const uint32_t hv[8], T E[3][3]) {
  T p0[3];
  load_vec(Y, hv[tet_v(K, 0)], p0);
#pragma unroll
  for (int j = 0; j < 3; j++) {
    T q[3];
    load_vec(Y, hv[tet_v(K, j + 1)], q);
    E[0][j] = q[0] - p0[0]; E[1][j] = q[1] - p0[1]; E[2][j] = q[2] - p0[2];
  }
}

// J = E R_k^T (cube-corner tet k): J[:, edge_axis(k,j)] = edge_sign(k,j) * E[:, j]
template <int K, typename T, typename S>
__device__ __forceinline__ void cube_J(const S E[3][3], T scale, T J[3][3]) {
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int a = edge_axis(K, j);
    const T sg = T(edge_sign(K, j)) * scale;
#pragma unroll
    for (int r = 0; r < 3; r++) J[r][a] = T(E[r][j]) * sg;
  }
}
// Forces of a cube tet from the stress Q (3x3): f_{j+1} = sign * Q[:, axis_j], f_0 = -sum.
template <int K, typename T, typename A>
__device__ __forceinline__ void cube_scatter(const T Q[3][3], T scale, A F[8][3]) {
  A f0[3] = {0, 0, 0};
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int a = edge_axis(K, j);
    const T sg = T(edge_sign(K, j)) * scale;
    const int c = tet_v(K, j + 1);
#pragma unroll
    for (int r = 0; r < 3; r++) {
      A v = A(Q[r][a] * sg);
      F[c][r] += v;
      f0[r] += v;
    }
  }
#pragma unroll
  for (int r = 0; r < 3; r++) F[tet_v(K, 0)][r] -= f0[r];
}
// General (own-shape) tet: J = E B, forces G = Q B^T (columns are f_1..f_3).
template <int K, typename T, typename S>
__device__ __forceinline__ void gen_J(const S E[3][3], const double *B, T J[3][3]) {
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) J[r][c] = T(E[r][0]) * T(B[0 * 3 + c]) + T(E[r][1]) * T(B[1 * 3 + c]) + T(E[r][2]) * T(B[2 * 3 + c]);
}
template <int K, typename T, typename A>
__device__ __forceinline__ void gen_scatter(const T Q[3][3], const double *B, A F[8][3]) {
  A f0[3] = {0, 0, 0};
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int c = tet_v(K, j + 1);
#pragma unroll
    for (int r = 0; r < 3; r++) {
      A v = A(Q[r][0] * T(B[j * 3 + 0]) + Q[r][1] * T(B[j * 3 + 1]) + Q[r][2] * T(B[j * 3 + 2]));
      F[c][r] += v;
      f0[r] += v;
    }
  }
#pragma unroll
  for (int r = 0; r < 3; r++) F[tet_v(K, 0)][r] -= f0[r];
}

// symmetric 3x3 stored as (xx, yy, zz, xy, xz, yz) times a 3x3
template <typename T>
__device__ __forceinline__ void sym_mul(const T c[6], const T J[3][3], T Q[3][3]) {
#pragma unroll
  for (int col = 0; col < 3; col++) {
    Q[0][col] = c[0] * J[0][col] + c[3] * J[1][col] + c[4] * J[2][col];
    Q[1][col] = c[3] * J[0][col] + c[1] * J[1][col] + c[5] * J[2][col];
    Q[2][col] = c[4] * J[0][col] + c[5] * J[1][col] + c[2] * J[2][col];
  }
}

__device__ __forceinline__ void load_hex(const uint32_t *hexv, int64_t h, uint32_t hv[8]) {
#pragma unroll
  for (int c = 0; c < 8; c++) hv[c] = __ldg(hexv + hex_idx(h, c));
}

// ---------------------------------------------------------------- 12-edge hex frame
// The 24 tet edges of the 8 corner tets are the 12 hex edges, each used twice.  Edge e joins
// corners (lo, hi) with lo < hi and is stored as P[hi] - P[lo]; the edge (c0 -> cj) of a corner
// tet is +E[e] when cj > c0, else -E[e].  Everything below folds at compile time.
__host__ __device__ __forceinline__ constexpr int hex_edge_ord(int lo, int hi) {
  return (lo == 0 && hi == 1) ? 0 : (lo == 1 && hi == 2) ? 1 : (lo == 2 && hi == 3) ? 2 : (lo == 0 && hi == 3) ? 3
       : (lo == 4 && hi == 5) ? 4 : (lo == 5 && hi == 6) ? 5 : (lo == 6 && hi == 7) ? 6 : (lo == 4 && hi == 7) ? 7
       : (lo == 0 && hi == 4) ? 8 : (lo == 1 && hi == 5) ? 9 : (lo == 2 && hi == 6) ? 10 : 11;
}
__host__ __device__ __forceinline__ constexpr int hex_edge_id(int a, int b) {
  return hex_edge_ord(a < b ? a : b, a < b ? b : a);
}
__host__ __device__ __forceinline__ constexpr int hex_edge_lo(int e) {
  return e == 0 ? 0 : e == 1 ? 1 : e == 2 ? 2 : e == 3 ? 0 : e == 4 ? 4 : e == 5 ? 5 : e == 6 ? 6 : e == 7 ? 4
       : e == 8 ? 0 : e == 9 ? 1 : e == 10 ? 2 : 3;
}
__host__ __device__ __forceinline__ constexpr int hex_edge_hi(int e) {
  return e == 0 ? 1 : e == 1 ? 2 : e == 2 ? 3 : e == 3 ? 3 : e == 4 ? 5 : e == 5 ? 6 : e == 6 ? 7 : e == 7 ? 7
       : e == 8 ? 4 : e == 9 ? 5 : e == 10 ? 6 : 7;
}

// Gather the 8 corner positions (FP64) and form the 12 edges in FP64, stored as T.
template <typename T>
__device__ __forceinline__ void hex_edges_pos(const double *X, const uint32_t hv[8], T E12[12][3]) {
  double P[8][3];
#pragma unroll
  for (int c = 0; c < 8; c++) load_pos(X, hv[c], P[c]);
#pragma unroll
  for (int e = 0; e < 12; e++)
#pragma unroll
    for (int r = 0; r < 3; r++) E12[e][r] = T(P[hex_edge_hi(e)][r] - P[hex_edge_lo(e)][r]);
}
// FP32 hi/lo split of one position: hi = fl32(x), lo = fl32(x - hi), so hi + lo carries x to
// about 48 bits.  Layout per vertex: hi.x hi.y hi.z 0 lo.x lo.y lo.z 0 (two float4).
__device__ __forceinline__ void store_split(float *X32, int64_t v, double x, double y, double z) {
  const float hx = float(x), hy = float(y), hz = float(z);
  reinterpret_cast<float4 *>(X32)[2 * v] = make_float4(hx, hy, hz, 0.f);
  reinterpret_cast<float4 *>(X32)[2 * v + 1] =
      make_float4(float(x - double(hx)), float(y - double(hy)), float(z - double(hz)), 0.f);
}
// Hex edges from the split positions, all in FP32: e = (hi_b - hi_a) + (lo_b - lo_a).  The
// hi difference is exact for nearby points (Sterbenz) and otherwise rounds once, so each edge is
// within ~1.5 FP32 ulps of the FP64 edge, with no FP64 instruction (GB300's FP64 pipe is a small
// fraction of its FP32 rate).
__device__ __forceinline__ void hex_edges_split(const float *X32, const uint32_t hv[8], float E12[12][3]) {
  float H[8][3], L[8][3];
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const float4 h = __ldg(reinterpret_cast<const float4 *>(X32) + 2 * (int64_t)hv[c]);
    const float4 l = __ldg(reinterpret_cast<const float4 *>(X32) + 2 * (int64_t)hv[c] + 1);
    H[c][0] = h.x; H[c][1] = h.y; H[c][2] = h.z;
    L[c][0] = l.x; L[c][1] = l.y; L[c][2] = l.z;
  }
#pragma unroll
  for (int e = 0; e < 12; e++)
#pragma unroll
    for (int r = 0; r < 3; r++)
      E12[e][r] = __fadd_rn(__fsub_rn(H[hex_edge_hi(e)][r], H[hex_edge_lo(e)][r]),
                            __fsub_rn(L[hex_edge_hi(e)][r], L[hex_edge_lo(e)][r]));
}
// Edge frame in the arithmetic type of the mode: FP32 from the split, FP64 from X.
template <typename ET>
__device__ __forceinline__ void hex_edges_mode(const KArgs &a, const uint32_t hv[8], ET E12[12][3]) {
  if constexpr (sizeof(ET) == 4) hex_edges_split(a.X32, hv, E12);
  else hex_edges_pos(a.X, hv, E12);
}
template <typename T>
__device__ __forceinline__ void hex_edges_vec(const T *Y, const uint32_t hv[8], T E12[12][3]) {
  T P[8][3];
#pragma unroll
  for (int c = 0; c < 8; c++) load_vec(Y, hv[c], P[c]);
#pragma unroll
  for (int e = 0; e < 12; e++)
#pragma unroll
    for (int r = 0; r < 3; r++) E12[e][r] = P[hex_edge_hi(e)][r] - P[hex_edge_lo(e)][r];
}
// Edge matrix (columns) of corner tet K from the 12-edge frame.
template <int K, typename T>
__device__ __forceinline__ void tet_E12(const T E12[12][3], T E[3][3]) {
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int c0 = tet_v(K, 0), cj = tet_v(K, j + 1);
    const int e = hex_edge_id(c0, cj);
    const T sg = cj > c0 ? T(1) : T(-1);
#pragma unroll
    for (int r = 0; r < 3; r++) E[r][j] = sg * E12[e][r];
  }
}
// Accumulate 3x3 "edge forces" G (columns for edges c0->cj) into corner forces.
template <int K, typename T, typename A>
__device__ __forceinline__ void scatter_cols(const T G[3][3], A F[8][3]) {
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int c0 = tet_v(K, 0), cj = tet_v(K, j + 1);
#pragma unroll
    for (int r = 0; r < 3; r++) {
      F[cj][r] += A(G[r][j]);
      F[c0][r] -= A(G[r][j]);
    }
  }
}
// J = E B and the transpose action G = Q B^T for a cube-target tet (B = signed permutation
// scaled by s) or an own-shape tet (B stored, 9 doubles).
template <int K, typename T>
__device__ __forceinline__ void apply_B(const T E[3][3], int32_t gs, const double *B, T s, T J[3][3]) {
  if (gs < 0) cube_J<K>(E, s, J);
  else gen_J<K>(E, B, J);
}
template <int K, typename T>
__device__ __forceinline__ void apply_BT(const T Q[3][3], int32_t gs, const double *B, T s, T G[3][3]) {
  if (gs < 0) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int a = edge_axis(K, j);
      const T sg = T(edge_sign(K, j)) * s;
#pragma unroll
      for (int r = 0; r < 3; r++) G[r][j] = Q[r][a] * sg;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int r = 0; r < 3; r++) G[r][j] = Q[r][0] * T(B[j * 3 + 0]) + Q[r][1] * T(B[j * 3 + 1]) + Q[r][2] * T(B[j * 3 + 2]);
  }
}

// Runtime-K forms of the corner-tet maps, for loops over the 8 tets that are not unrolled (one
// copy of the per-tet code): the cube-corner permutation becomes select chains, never a dynamic
// index into a register array, and every value equals the compile-time form's bit for bit.
template <typename T>
__device__ __forceinline__ void apply_B_rt(int K, const T E[3][3], int32_t gs, const double *B, T s, T J[3][3]) {
  if (gs < 0) {
    const int a0 = edge_axis(K, 0), a1 = edge_axis(K, 1);
    const T s0 = T(edge_sign(K, 0)) * s, s1 = T(edge_sign(K, 1)) * s, s2 = T(edge_sign(K, 2)) * s;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const T v0 = E[r][0] * s0, v1 = E[r][1] * s1, v2 = E[r][2] * s2;
      J[r][0] = a0 == 0 ? v0 : a1 == 0 ? v1 : v2;
      J[r][1] = a0 == 1 ? v0 : a1 == 1 ? v1 : v2;
      J[r][2] = a0 == 2 ? v0 : a1 == 2 ? v1 : v2;
    }
  } else {
    gen_J<0>(E, B, J);
  }
}
template <typename T>
__device__ __forceinline__ void apply_BT_rt(int K, const T Q[3][3], int32_t gs, const double *B, T s, T G[3][3]) {
  if (gs < 0) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int a = edge_axis(K, j);
      const T sg = T(edge_sign(K, j)) * s;
#pragma unroll
      for (int r = 0; r < 3; r++) G[r][j] = (a == 0 ? Q[r][0] : a == 1 ? Q[r][1] : Q[r][2]) * sg;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int r = 0; r < 3; r++) G[r][j] = Q[r][0] * T(B[j * 3 + 0]) + Q[r][1] * T(B[j * 3 + 1]) + Q[r][2] * T(B[j * 3 + 2]);
  }
}
// Edge matrix of corner tet K from a thread's column of 12-edge frames (entry e * 3 + r at
// col[(e * 3 + r) * stride]).
template <typename T>
__device__ __forceinline__ void tet_E_rt(int K, const T *col, int stride, T E[3][3]) {
  const int c0 = tet_v(K, 0);
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int cj = tet_v(K, j + 1);
    const int e = hex_edge_id(c0, cj);
    const T sg = cj > c0 ? T(1) : T(-1);
#pragma unroll
    for (int r = 0; r < 3; r++) E[r][j] = sg * col[(e * 3 + r) * stride];
  }
}

// ---------------------------------------------------------------- constraint items
// The constraint items of a mesh, in order: corners, tangent planes, feature lines, projection
// points (Tetralize_Set::b / bc), glue groups; e indexes the kind's global arrays.
enum ConsKind { CK_CORNER = 0, CK_TANGENT = 1, CK_LINE = 2, CK_PROJ = 3, CK_GROUP = 4 };
struct ConsItem {
  int kind;
  int64_t e;
};
__device__ __forceinline__ ConsItem cons_item(const MeshDesc &md, int64_t i) {
  int64_t li = i - md.kitem0[K_CONS];
  if (li < md.nc) return {CK_CORNER, md.c_off + li};
  li -= md.nc;
  if (li < md.nt) return {CK_TANGENT, md.t_off + li};
  li -= md.nt;
  if (li < md.nl) return {CK_LINE, md.l_off + li};
  li -= md.nl;
  if (li < md.nb) return {CK_PROJ, md.b_off + li};
  return {CK_GROUP, md.grp_off + (li - md.nb)};
}
// Glue group g: members m0..m1-1 of g_vs; coefficient (n / (n-1))^2 of the reference's rows
// x_j - sum_{k != j} x_k / (n-1) (slim_m.cpp:611-646); 0 for a single member.
__device__ __forceinline__ double glue_coef(int64_t n) {
  return n < 2 ? 0.0 : double(n) * double(n) / (double(n - 1) * double(n - 1));
}

}  // namespace hexopt
