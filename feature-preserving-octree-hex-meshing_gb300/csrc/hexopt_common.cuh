// hexopt_common.cuh -- device-side building blocks shared by the hexopt kernels (sm_103a).
//
//  * compile-time hex tables (hex_tetra_table, global_types.h:163-173) and the cube-corner edge
//    permutation each corner tet applies (J_t = E_t R_k^-1 / cbrt(6 vol_t), R_k a signed
//    permutation of the unit axes, so J is a signed column permutation of the edge matrix);
//  * 3x3 algebra, a one-sided Jacobi SVD and igl::polar_svd semantics;
//  * SLIM weights / energies (slim_m.cpp:108-381, 792-916);
//  * block-segmented deterministic reductions (per-mesh partials, last block finalises).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include "hexopt_dev.h"

namespace hexopt {

// ------------------------------------------------------------------------------- tables
// Row k of hex_tetra_table packed as 4 nibbles (corner j at bits 4j..4j+3).
__host__ __device__ __forceinline__ constexpr unsigned tet_row(int k) {
  return k == 0 ? 0x1430u : k == 1 ? 0x2501u : k == 2 ? 0x3612u : k == 3 ? 0x0723u
       : k == 4 ? 0x0574u : k == 5 ? 0x1645u : k == 6 ? 0x2756u : 0x3467u;
}
__host__ __device__ __forceinline__ constexpr int tet_v(int k, int j) { return (int)((tet_row(k) >> (4 * j)) & 0xFu); }
// Cube-corner tet k: edge j (to tet vertex j+1) runs along axis edge_axis(k,j) with sign edge_sign(k,j).
__host__ __device__ __forceinline__ constexpr int edge_axis(int k, int j) {
  return (int)(((k == 0 || k == 2) ? 0x021u : (k == 1 || k == 3) ? 0x120u : (k == 4 || k == 6) ? 0x201u : 0x210u) >> (4 * j)) & 0xF;
}
__host__ __device__ __forceinline__ constexpr int edge_sign(int k, int j) {
  // bit j set = negative
  return ((((k == 0) ? 0u : (k == 1) ? 1u : (k == 2) ? 5u : (k == 3) ? 4u : (k == 4) ? 4u : (k == 5) ? 5u : (k == 6) ? 7u : 6u) >> j) & 1u) ? -1 : 1;
}

// ------------------------------------------------------------------------------- enums
enum Energy { ARAP = 0, LOG_ARAP = 1, SYMMETRIC_DIRICHLET = 2, CONFORMAL = 3, EXP_CONFORMAL = 4,
              EXP_SYMMETRIC_DIRICHLET = 5 };

// ------------------------------------------------------------------------------- 3x3 helpers
template <typename T>
__device__ __forceinline__ T det3(const T m[3][3]) {
  // Eigen's 3x3 cofactor order (Eigen/src/LU/Determinant.h)
  return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[1][0] * (m[0][1] * m[2][2] - m[0][2] * m[2][1]) +
         m[2][0] * (m[0][1] * m[1][2] - m[0][2] * m[1][1]);
}

// Bit-reproducible FP64 determinant (no FMA contraction): sign parity with the oracle.
__device__ __forceinline__ double det3_rn(const double m[3][3]) {
  double a = __dsub_rn(__dmul_rn(m[1][1], m[2][2]), __dmul_rn(m[1][2], m[2][1]));
  double b = __dsub_rn(__dmul_rn(m[0][1], m[2][2]), __dmul_rn(m[0][2], m[2][1]));
  double c = __dsub_rn(__dmul_rn(m[0][1], m[1][2]), __dmul_rn(m[0][2], m[1][1]));
  return __dadd_rn(__dsub_rn(__dmul_rn(m[0][0], a), __dmul_rn(m[1][0], b)), __dmul_rn(m[2][0], c));
}

template <typename T>
__device__ __forceinline__ void adj3(const T m[3][3], T a[3][3]) {  // adjugate (transpose of cofactors)
  a[0][0] = m[1][1] * m[2][2] - m[1][2] * m[2][1];
  a[0][1] = m[0][2] * m[2][1] - m[0][1] * m[2][2];
  a[0][2] = m[0][1] * m[1][2] - m[0][2] * m[1][1];
  a[1][0] = m[1][2] * m[2][0] - m[1][0] * m[2][2];
  a[1][1] = m[0][0] * m[2][2] - m[0][2] * m[2][0];
  a[1][2] = m[0][2] * m[1][0] - m[0][0] * m[1][2];
  a[2][0] = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  a[2][1] = m[0][1] * m[2][0] - m[0][0] * m[2][1];
  a[2][2] = m[0][0] * m[1][1] - m[0][1] * m[1][0];
}

template <typename T> __device__ __forceinline__ T sq(T x) { return x * x; }
template <typename T> __device__ __forceinline__ T frob2(const T m[3][3]) {
  T s = 0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) s += m[i][j] * m[i][j];
  return s;
}

__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }

// ------------------------------------------------------------------------------- SVD
// One-sided (Hestenes) Jacobi SVD: A = U diag(s) V^T, s >= 0 descending, U, V orthogonal.
// W = U m U^T and the polar rotation do not depend on which valid SVD is returned, so this
// reproduces Eigen::JacobiSVD inside igl::polar_svd (polar_svd.cpp:36-64) up to rounding.
template <typename T>
__device__ void svd3(const T A[3][3], T U[3][3], T s[3], T Vm[3][3]) {
  T a[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) { a[i][j] = A[i][j]; Vm[i][j] = (i == j) ? T(1) : T(0); }
  const T tol = sizeof(T) == 8 ? T(1e-15) : T(1e-7);
  const int max_sweeps = sizeof(T) == 8 ? 12 : 6;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    bool rotated = false;
#pragma unroll
    for (int pq = 0; pq < 3; pq++) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      T al = a[0][p] * a[0][p] + a[1][p] * a[1][p] + a[2][p] * a[2][p];
      T be = a[0][q] * a[0][q] + a[1][q] * a[1][q] + a[2][q] * a[2][q];
      T ga = a[0][p] * a[0][q] + a[1][p] * a[1][q] + a[2][p] * a[2][q];
      if (ga == T(0) || fabs(ga) <= tol * sqrt(al * be)) continue;
      rotated = true;
      T zeta = (be - al) / (T(2) * ga);
      T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
      T c = rsqrt_t(T(1) + t * t), sn = c * t;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        T x = a[i][p], y = a[i][q];
        a[i][p] = c * x - sn * y;
        a[i][q] = sn * x + c * y;
        x = Vm[i][p]; y = Vm[i][q];
        Vm[i][p] = c * x - sn * y;
        Vm[i][q] = sn * x + c * y;
      }
    }
    if (!rotated) break;
  }
  T n0 = sqrt(a[0][0] * a[0][0] + a[1][0] * a[1][0] + a[2][0] * a[2][0]);
  T n1 = sqrt(a[0][1] * a[0][1] + a[1][1] * a[1][1] + a[2][1] * a[2][1]);
  T n2 = sqrt(a[0][2] * a[0][2] + a[1][2] * a[1][2] + a[2][2] * a[2][2]);
  // sort columns by norm, descending (branch-free swaps on registers)
#define HX_SWAPCOL(i, j, ni, nj)                                                    \
  if (nj > ni) {                                                                    \
    T tt = ni; ni = nj; nj = tt;                                                    \
    _Pragma("unroll") for (int r = 0; r < 3; r++) {                                 \
      tt = a[r][i]; a[r][i] = a[r][j]; a[r][j] = tt;                                \
      tt = Vm[r][i]; Vm[r][i] = Vm[r][j]; Vm[r][j] = tt;                            \
    }                                                                               \
  }
  HX_SWAPCOL(0, 1, n0, n1)
  HX_SWAPCOL(0, 2, n0, n2)
  HX_SWAPCOL(1, 2, n1, n2)
#undef HX_SWAPCOL
  s[0] = n0; s[1] = n1; s[2] = n2;
  T u0[3], u1[3], u2[3];
  if (n0 > T(0)) { T inv = T(1) / n0; u0[0] = a[0][0] * inv; u0[1] = a[1][0] * inv; u0[2] = a[2][0] * inv; }
  else { u0[0] = 1; u0[1] = 0; u0[2] = 0; }
  u1[0] = a[0][1]; u1[1] = a[1][1]; u1[2] = a[2][1];
  T pr = u1[0] * u0[0] + u1[1] * u0[1] + u1[2] * u0[2];
  u1[0] -= pr * u0[0]; u1[1] -= pr * u0[1]; u1[2] -= pr * u0[2];
  T l1 = sqrt(u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]);
  if (l1 > T(1e-30) && n1 > T(0)) {
    T inv = T(1) / l1; u1[0] *= inv; u1[1] *= inv; u1[2] *= inv;
  } else {
    T e[3] = {0, 0, 0};
    int m = (fabs(u0[0]) <= fabs(u0[1]) && fabs(u0[0]) <= fabs(u0[2])) ? 0 : (fabs(u0[1]) <= fabs(u0[2]) ? 1 : 2);
    e[m] = 1;
    T pe = e[0] * u0[0] + e[1] * u0[1] + e[2] * u0[2];
    u1[0] = e[0] - pe * u0[0]; u1[1] = e[1] - pe * u0[1]; u1[2] = e[2] - pe * u0[2];
    T inv = rsqrt_t(u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]);
    u1[0] *= inv; u1[1] *= inv; u1[2] *= inv;
  }
  u2[0] = u0[1] * u1[2] - u0[2] * u1[1];
  u2[1] = u0[2] * u1[0] - u0[0] * u1[2];
  u2[2] = u0[0] * u1[1] - u0[1] * u1[0];
  if (a[0][2] * u2[0] + a[1][2] * u2[1] + a[2][2] * u2[2] < T(0)) { u2[0] = -u2[0]; u2[1] = -u2[1]; u2[2] = -u2[2]; }
#pragma unroll
  for (int i = 0; i < 3; i++) { U[i][0] = u0[i]; U[i][1] = u1[i]; U[i][2] = u2[i]; }
}

// igl::polar_svd: R = U V^T with a reflection moved onto the smallest singular direction.
template <typename T>
__device__ void polar_svd3(const T J[3][3], T R[3][3], T U[3][3], T s[3], T Vm[3][3]) {
  svd3(J, U, s, Vm);
  T dU = det3(U), dV = det3(Vm);
  if (dU * dV < T(0)) {
#pragma unroll
    for (int i = 0; i < 3; i++) Vm[i][2] = -Vm[i][2];
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) R[i][j] = U[i][0] * Vm[j][0] + U[i][1] * Vm[j][1] + U[i][2] * Vm[j][2];
}

// ------------------------------------------------------------------------------- SLIM weights
// update_weights_and_closest_rotations, 3-D branch (slim_m.cpp:230-351).  Returns the weight
// vector m and, for the conformal energies, rescales R to U diag(closest_s) V^T.
template <typename T>
__device__ void slim_weights(int energy, T exp_f, const T s[3], const T U[3][3], const T Vm[3][3], T m[3], T R[3][3]) {
  const T s1 = s[0], s2 = s[1], s3 = s[2];
  switch (energy) {
    case SYMMETRIC_DIRICHLET: {
      // sqrt((2(s - s^-3)) / (2(s - 1))) = sqrt((s+1)(s^2+1)/s^3): same value without the
      // cancellation of the reference's form near s = 1.
#pragma unroll
      for (int i = 0; i < 3; i++) {
        T si = s[i];
        m[i] = sqrt((si + T(1)) * (si * si + T(1)) / (si * si * si));
      }
      break;
    }
    case ARAP: m[0] = m[1] = m[2] = T(1); break;
    case LOG_ARAP: {
#pragma unroll
      for (int i = 0; i < 3; i++) m[i] = sqrt((T(2) * (log(s[i]) / s[i])) / (T(2) * (s[i] - T(1))));
      break;
    }
    case EXP_SYMMETRIC_DIRICHLET: {
      T in_exp = exp_f * (s1 * s1 + T(1) / (s1 * s1) + s2 * s2 + T(1) / (s2 * s2) + s3 * s3 + T(1) / (s3 * s3));
      T et = exp(in_exp);
#pragma unroll
      for (int i = 0; i < 3; i++) {
        T si = s[i];
        T g = T(2) * (si - T(1) / (si * si * si)) * et * exp_f;
        m[i] = sqrt(g / (T(2) * (si - T(1))));
      }
      break;
    }
    case CONFORMAL:
    case EXP_CONFORMAL: {
      T cd = T(9) * pow(s1 * s2 * s3, T(5.0 / 3.0));
      T g[3];
      g[0] = (T(-2) * s2 * s3 * (s2 * s2 + s3 * s3 - T(2) * s1 * s1)) / cd;
      g[1] = (T(-2) * s1 * s3 * (s1 * s1 + s3 * s3 - T(2) * s2 * s2)) / cd;
      g[2] = (T(-2) * s1 * s2 * (s1 * s1 + s2 * s2 - T(2) * s3 * s3)) / cd;
      T cs = sqrt(s1 * s1 + s3 * s3) / sqrt(T(2));
      if (energy == EXP_CONFORMAL) {
        T in_exp = exp_f * ((s1 * s1 + s2 * s2 + s3 * s3) / (T(3) * pow(s1 * s2 * s3, T(2.0 / 3.0))));
        T et = exp(in_exp);
        g[0] *= et * exp_f; g[1] *= et * exp_f; g[2] *= et * exp_f;
      }
#pragma unroll
      for (int i = 0; i < 3; i++) m[i] = sqrt(g[i] / (T(2) * (s[i] - cs)));
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) R[i][j] = cs * (U[i][0] * Vm[j][0] + U[i][1] * Vm[j][1] + U[i][2] * Vm[j][2]);
      break;
    }
    default: m[0] = m[1] = m[2] = T(1);
  }
  const T eps = T(1e-8);
#pragma unroll
  for (int i = 0; i < 3; i++)
    if (fabs(s[i] - T(1)) < eps) m[i] = T(1);
}

// Per-tet energy density (compute_energy_with_jacobians 3-D branch, slim_m.cpp:850-912).
// The SVD-based energies (ARAP, LOG_ARAP, CONFORMAL, EXP_CONFORMAL) are out of line: the optimiser
// runs symmetric Dirichlet, and inlining a 3x3 SVD into every corner tet of the energy kernels
// would size their register allocation for code that does not run.
template <typename T>
__device__ __noinline__ T tet_energy_density_svd(int energy, T J00, T J01, T J02, T J10, T J11, T J12, T J20,
                                                 T J21, T J22) {
  const T J[3][3] = {{J00, J01, J02}, {J10, J11, J12}, {J20, J21, J22}};
  T R[3][3], U[3][3], s[3], Vm[3][3];
  polar_svd3(J, R, U, s, Vm);
  const T s1 = s[0], s2 = s[1], s3 = s[2];
  switch (energy) {
    case ARAP: return sq(s1 - T(1)) + sq(s2 - T(1)) + sq(s3 - T(1));
    case LOG_ARAP: return sq(log(s1)) + sq(log(fabs(s2))) + sq(log(fabs(s3)));
    case CONFORMAL: return (s1 * s1 + s2 * s2 + s3 * s3) / (T(3) * pow(s1 * s2 * s3, T(2.0 / 3.0)));
    case EXP_CONFORMAL: return exp((s1 * s1 + s2 * s2 + s3 * s3) / (T(3) * pow(s1 * s2 * s3, T(2.0 / 3.0))));
  }
  return T(NAN);
}
// Symmetric Dirichlet needs no SVD: sum s^2 = |J|_F^2 and sum s^-2 = |adj J|_F^2 / det^2.
template <typename T>
__device__ __forceinline__ T tet_energy_density(int energy, T exp_f, const T J[3][3]) {
  if (energy == SYMMETRIC_DIRICHLET || energy == EXP_SYMMETRIC_DIRICHLET) {
    T A[3][3];
    adj3(J, A);
    T d = det3(J);
    T e = frob2(J) + frob2(A) / (d * d);
    return energy == SYMMETRIC_DIRICHLET ? e : exp(exp_f * e);
  }
  return tet_energy_density_svd<T>(energy, J[0][0], J[0][1], J[0][2], J[1][0], J[1][1], J[1][2], J[2][0], J[2][1],
                                   J[2][2]);
}

// ------------------------------------------------------------------------------- reductions
// Per-thread accumulators.  SumAcc<double> is a plain FP64 sum.  SumAcc<float> is a compensated
// FP32 sum (Ogita, Rump & Oishi 2005, "Accurate sum and dot product": TwoSum and the FMA-based
// TwoProduct error-free transformations), carrying about twice FP32's precision on the FP32
// pipes -- GB300's FP64 rate is a small fraction of its FP32 rate, so per-item FP64 adds would
// bound the vector kernels.  value() hands the thread's total to the FP64 block reduction.
template <typename T> struct SumAcc;
template <> struct SumAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ void add_prod(double a, double b) { s += a * b; }
  __device__ __forceinline__ double value() const { return s; }
};
template <> struct SumAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = __fadd_rn(s, x);
    const float z = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(x, z)));
    s = t;
  }
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    add(p);
    c = __fadd_rn(c, e);
  }
  // fold in another accumulator's (sum, carry): TwoSum of the sums, carries added
  __device__ __forceinline__ void merge(float s2, float c2) {
    add(s2);
    c = __fadd_rn(c, c2);
  }
  __device__ __forceinline__ double value() const { return double(s) + double(c); }
};

// Exclusive prefix sum of v over the 32 lanes of a warp (all lanes must call it); total = sum.
__device__ __forceinline__ int warp_exclusive_sum(int v, int &total) {
  const int lane = threadIdx.x & 31;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

// Block-level sum of NV doubles (all threads get nothing back; thread 0 gets the total).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (*smem)[32]) {
#pragma unroll
  for (int k = 0; k < NV; k++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) smem[k][wid] = v[k];
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double x = lane < nw ? smem[k][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      v[k] = x;
    }
  }
}

template <int NV>
__device__ __forceinline__ void block_min(double (&v)[NV], double (*smem)[32]) {
#pragma unroll
  for (int k = 0; k < NV; k++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] = fmin(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) smem[k][wid] = v[k];
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double x = lane < nw ? smem[k][lane] : INFINITY;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_down_sync(0xffffffffu, x, o));
      v[k] = x;
    }
  }
}

// Writes this block's NV partials; returns true in thread 0 of the block that finished last
// among its mesh's blocks (after a fence, so all partials of the mesh are visible to it).
template <int NV>
__device__ __forceinline__ bool publish_partials(const double (&v)[NV], double *partials, int64_t blk_global,
                                                 unsigned *counter, unsigned nblk_mesh) {
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) partials[blk_global * NV + k] = v[k];
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    am_last = (prev == nblk_mesh - 1);
  }
  __syncthreads();
  return am_last;
}

// Block sum of compensated FP32 accumulators: the (sum, carry) pairs are reduced through the
// warps and the block with FP32 TwoSum merges, and only thread 0 converts the block total to
// FP64 (out[k] is valid in thread 0).  Vertex kernels do a few FP32 operations per item, so
// per-thread FP64 shuffles and conversions would keep GB300's slow FP64 pipe busy.
template <int NV>
__device__ __forceinline__ void block_sum_acc(SumAcc<float> (&v)[NV], double (&out)[NV], float (*smem)[2][32]) {
#pragma unroll
  for (int k = 0; k < NV; k++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float s2 = __shfl_down_sync(0xffffffffu, v[k].s, o), c2 = __shfl_down_sync(0xffffffffu, v[k].c, o);
      v[k].merge(s2, c2);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) { smem[k][0][wid] = v[k].s; smem[k][1][wid] = v[k].c; }
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
      SumAcc<float> x;
      x.s = lane < nw ? smem[k][0][lane] : 0.f;
      x.c = lane < nw ? smem[k][1][lane] : 0.f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_down_sync(0xffffffffu, x.s, o), c2 = __shfl_down_sync(0xffffffffu, x.c, o);
        x.merge(s2, c2);
      }
      out[k] = x.value();
    }
  }
}

// Fixed-order sum (by the last block) of a mesh's partials, k-th component.
__device__ __forceinline__ double gather_partials_sum(const double *partials, int64_t first_blk, int nblk, int NV,
                                                      int k, double (*smem)[32]) {
  double x = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) x += __ldcg(&partials[(first_blk + b) * NV + k]);
  double v[1] = {x};
  block_sum<1>(v, smem);
  return v[0];
}
// The same fixed-order sums for components 0..NV-1 at once.  Each thread adds its blocks
// b = tid, tid + blockDim, ... in that order, exactly as above, but with the loads of U blocks in
// flight together, so the last block's tail costs a few L2 round trips instead of one per block.
template <int NV>
__device__ __forceinline__ void gather_partials_sums(const double *partials, int64_t first_blk, int nblk, int stride,
                                                     double (&out)[NV], double (*smem)[32]) {
  constexpr int U = NV == 1 ? 16 : NV == 2 ? 8 : NV <= 4 ? 4 : 2;
  double x[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) x[k] = 0;
  const double *base = partials + first_blk * stride;
  const int bd = blockDim.x;
  int b = threadIdx.x;
  for (; b + (U - 1) * bd < nblk; b += U * bd) {
    double t[U][NV];
#pragma unroll
    for (int u = 0; u < U; u++)
#pragma unroll
      for (int k = 0; k < NV; k++) t[u][k] = __ldcg(base + (int64_t)(b + u * bd) * stride + k);
#pragma unroll
    for (int u = 0; u < U; u++)
#pragma unroll
      for (int k = 0; k < NV; k++) x[k] += t[u][k];
  }
  for (; b < nblk; b += bd)
#pragma unroll
    for (int k = 0; k < NV; k++) x[k] += __ldcg(base + (int64_t)b * stride + k);
  block_sum<NV>(x, smem);
#pragma unroll
  for (int k = 0; k < NV; k++) out[k] = x[k];
}
__device__ __forceinline__ double gather_partials_min(const double *partials, int64_t first_blk, int nblk, int NV,
                                                      int k, double (*smem)[32]) {
  // 16 loads in flight per thread (the minimum does not depend on the order)
  constexpr int U = 16;
  double x = INFINITY;
  const double *base = partials + first_blk * NV + k;
  const int bd = blockDim.x;
  int b = threadIdx.x;
  for (; b + (U - 1) * bd < nblk; b += U * bd) {
    double t[U];
#pragma unroll
    for (int u = 0; u < U; u++) t[u] = __ldcg(base + (int64_t)(b + u * bd) * NV);
#pragma unroll
    for (int u = 0; u < U; u++) x = fmin(x, t[u]);
  }
  for (; b < nblk; b += bd) x = fmin(x, __ldcg(base + (int64_t)b * NV));
  double v[1] = {x};
  block_min<1>(v, smem);
  return v[0];
}

}  // namespace hexopt
