// k_slim.cuh -- SLIM local/global iteration kernels on sm_103a, one thread per hex (8 corner tets).
//
// Stages (slim_m.cpp:1269-1288, one iteration of slim_solve2's fixed-N branch):
//   k_precompute     slim_precompute: per-tet inverse rest scale 1/cbrt(6 vol) (cube targets) or
//                    rest-edge inverse (own-shape targets)      grad.cpp:372-478 closed form
//   k_local          update_weights_and_closest_rotations + buildRhs: per-tet SVD, SD weights,
//                    stores C_t = M W^T W (6 values) and scatters A^T M f   slim_m.cpp:108-381, 1044-1092
//   k_spmv           matrix-free  y += sum_t K_t x  with K_t = (D_t^T D_t) (x) C_t  (buildA + L = A^T M A,
//                    slim_m.cpp:568-595, 918-1042, never assembled)
//   k_soft_*         add_soft_constraints / compute_soft_const_energy   slim_m.cpp:597-714, 735-790
//   k_cg_*           Eigen ConjugateGradient<Lower|Upper> + Jacobi, solved for the update
//                    delta = x - x0 with an FP64 initial residual      ConjugateGradient.h:39-80
//   k_ls_*           flip_avoiding_line_search + igl::line_search      flip_avoiding_line_search.cpp,
//                                                                       line_search.cpp:10-53
// Precision: ET = element coefficient / arithmetic type, VT = CG vector type.  FP64 mode uses
// <double,double>.  MIXED uses <float,float>: edges are formed from FP64 positions in FP64 and
// rounded once; the PCG solves for the update delta from an initial residual formed per element
// as M W^T W (R - J) B^T (no cancellation against A x0); positions are updated in FP64; every
// reduction accumulates in FP64; the step bound's root solve is FP64.
#pragma once
#include "hexopt_common.cuh"
#include "hexopt_kernels.h"
#include "hexopt_elem.cuh"

namespace hexopt {

// ------------------------------------------------------------------------------- precompute
// slim_precompute alone (hexopt_slim_precompute): per-tet 1/cbrt(6 vol) of cube-target tets,
// rest-edge inverse of own-shape tets, the scaled operator of general reference shapes (Bref),
// from the FP64 positions.
template <typename ET>
__global__ void __launch_bounds__(128) k_precompute(KArgs a) {
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  if (h >= sg.end) return;
  uint32_t hv[8];
  load_hex(a.hexv, h, hv);
  const int32_t gs = a.gslot[h];
  ET *Sinv = reinterpret_cast<ET *>(a.Sinv);
  bool degenerate = false;
#define HX_PRE(K)                                                                              \
  {                                                                                            \
    double E[3][3];                                                                            \
    tet_edges<K>(a.X, hv, E);                                                                  \
    const double d = det3(E);                                                                  \
    degenerate |= (d == 0.0);                                                                  \
    if (gs < 0) {                                                                              \
      Sinv[tet_idx<1>(h, K, 0)] = ET(1.0 / cbrt(d));                                            \
    } else if (a.Bref) {                                                                       \
      const double *Rf = a.Bref + ((int64_t)gs * 8 + K) * 9;                                   \
      double *B = a.Bgen + ((int64_t)gs * 8 + K) * 9;                                          \
      const double cd = cbrt(d);                                                               \
      _Pragma("unroll") for (int i = 0; i < 9; i++) B[i] = Rf[i] / cd;                         \
      Sinv[tet_idx<1>(h, K, 0)] = ET(1);                                                       \
    } else {                                                                                   \
      double A[3][3];                                                                          \
      adj3(E, A);                                                                              \
      double *B = a.Bgen + ((int64_t)gs * 8 + K) * 9;                                          \
      _Pragma("unroll") for (int i = 0; i < 3; i++)                                            \
      _Pragma("unroll") for (int j = 0; j < 3; j++) B[i * 3 + j] = A[i][j] / d;                 \
      Sinv[tet_idx<1>(h, K, 0)] = ET(1);                                                       \
    }                                                                                          \
  }
  HX_PRE(0) HX_PRE(1) HX_PRE(2) HX_PRE(3) HX_PRE(4) HX_PRE(5) HX_PRE(6) HX_PRE(7)
#undef HX_PRE
  if (degenerate) atomicOr(&a.sc[sg.mesh].status, 2);
}

// ------------------------------------------------------------------------------- local step
// One corner tet of the fused local step: (optional) volume snapshot, J, SVD, SLIM weights, the
// stored coefficients C' and the tet's contributions to b = A^T M f and to diag(L).  FP64 mode
// also scatters the initial residual r0 = b - A x0 = sum_t M W^T W (R - J) B^T (formed per
// element, so it carries no cancellation); mixed mode stores R instead and forms r0 in k_ir_resid
// from the FP64 positions.
// K is a run-time index (the 8 tets run as a loop that is not unrolled, so the SVD and weight
// code exists once: unrolled, the kernel outgrew the instruction cache); the hex's 12-edge frame
// and corner ids come from the thread's columns of block-shared arrays (stride kLocalThreads).
constexpr int kLocalThreads = 128;
template <typename ET, bool PRE>
__device__ __forceinline__ void local_tet(const KArgs &a, int64_t h, int32_t gs, int K, const ET *e12col, ET M,
                                          ET exp_f, int energy, const uint32_t *hvcol, bool &degenerate) {
  ET *gb = reinterpret_cast<ET *>(a.b), *gr = reinterpret_cast<ET *>(a.r), *gd = reinterpret_cast<ET *>(a.diag);
  auto hvk = [&](int c) { return hvcol[c * kLocalThreads]; };
  ET E[3][3];
  tet_E_rt(K, e12col, kLocalThreads, E);
  ET *Sinv = reinterpret_cast<ET *>(a.Sinv);
  double *B = gs >= 0 ? a.Bgen + ((int64_t)gs * 8 + K) * 9 : nullptr;
  ET is;
  if (PRE) {
    const ET d = det3(E);
    degenerate |= (d == ET(0));
    if (gs < 0) {
      is = ET(1) / cbrt(d);
    } else if (a.Bref) {
      // fixed reference shape: B = adj(R) / |det R|^(2/3) / cbrt(det E) (k_shapes.cu)
      const double *Rf = a.Bref + ((int64_t)gs * 8 + K) * 9;
      const double cd = cbrt(double(d));
#pragma unroll
      for (int i = 0; i < 9; i++) B[i] = Rf[i] / cd;
      is = ET(1);
    } else {
      ET A[3][3];
      adj3(E, A);
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) B[i * 3 + j] = double(A[i][j] / d);
      is = ET(1);
    }
    Sinv[tet_idx<1>(h, K, 0)] = is;
  } else {
    is = Sinv[tet_idx<1>(h, K, 0)];
  }
  ET J[3][3];
  apply_B_rt(K, E, gs, B, is, J);
  ET R[3][3], U[3][3], s[3], Vm[3][3], m[3];
  polar_svd3(J, R, U, s, Vm);
  slim_weights(energy, exp_f, s, U, Vm, m, R);
  // W = U diag(m) U^T is symmetric, so M W^T W = M U diag(m^2) U^T
  ET c[6];
  const ET m0 = M * m[0] * m[0], m1 = M * m[1] * m[1], m2 = M * m[2] * m[2];
  c[0] = U[0][0] * U[0][0] * m0 + U[0][1] * U[0][1] * m1 + U[0][2] * U[0][2] * m2;
  c[1] = U[1][0] * U[1][0] * m0 + U[1][1] * U[1][1] * m1 + U[1][2] * U[1][2] * m2;
  c[2] = U[2][0] * U[2][0] * m0 + U[2][1] * U[2][1] * m1 + U[2][2] * U[2][2] * m2;
  c[3] = U[0][0] * U[1][0] * m0 + U[0][1] * U[1][1] * m1 + U[0][2] * U[1][2] * m2;
  c[4] = U[0][0] * U[2][0] * m0 + U[0][1] * U[2][1] * m1 + U[0][2] * U[2][2] * m2;
  c[5] = U[1][0] * U[2][0] * m0 + U[1][1] * U[2][1] * m1 + U[1][2] * U[2][2] * m2;
  ET Q[3][3], G[3][3];
  sym_mul(c, R, Q);
  apply_BT_rt(K, Q, gs, B, is, G);
  {
    ET s0 = 0, s1 = 0, s2 = 0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      atomic_add3(gb, hvk(tet_v(K, j + 1)), G[0][j], G[1][j], G[2][j]);
      s0 += G[0][j]; s1 += G[1][j]; s2 += G[2][j];
    }
    atomic_add3(gb, hvk(tet_v(K, 0)), -s0, -s1, -s2);
  }
  if constexpr (sizeof(ET) == 4) {
    // mixed mode: the rotation is kept for the residual evaluations of the refined PCG (k_ir_*),
    // which also form the initial residual, from the FP64 positions
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) a.Rrot[tet_idx<9>(h, K, i * 3 + j)] = R[i][j];
    (void)gr;
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) R[i][j] -= J[i][j];
    sym_mul(c, R, Q);
    apply_BT_rt(K, Q, gs, B, is, G);
    ET s0 = 0, s1 = 0, s2 = 0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      atomic_add3(gr, hvk(tet_v(K, j + 1)), G[0][j], G[1][j], G[2][j]);
      s0 += G[0][j]; s1 += G[1][j]; s2 += G[2][j];
    }
    atomic_add3(gr, hvk(tet_v(K, 0)), -s0, -s1, -s2);
  }
  ET *C = reinterpret_cast<ET *>(a.Ccoef);
  ET w[4];
  if (gs < 0) {
    const ET s2 = is * is;  // fold 1 / cbrt(6 vol)^2 into the stored coefficients
#pragma unroll
    for (int i = 0; i < 6; i++) C[tet_idx<6>(h, K, i)] = c[i] * s2;
    w[0] = ET(3) * s2; w[1] = w[2] = w[3] = s2;  // |g_j|^2 of the cube-corner gradient rows
  } else {
#pragma unroll
    for (int i = 0; i < 6; i++) C[tet_idx<6>(h, K, i)] = c[i];
#pragma unroll
    for (int j = 0; j < 3; j++) w[j + 1] = ET(B[j * 3] * B[j * 3] + B[j * 3 + 1] * B[j * 3 + 1] + B[j * 3 + 2] * B[j * 3 + 2]);
    ET g0[3];
#pragma unroll
    for (int r = 0; r < 3; r++) g0[r] = ET(B[r] + B[3 + r] + B[6 + r]);
    w[0] = g0[0] * g0[0] + g0[1] * g0[1] + g0[2] * g0[2];
  }
#pragma unroll
  for (int j = 0; j < 4; j++) atomic_add3(gd, hvk(tet_v(K, j)), w[j] * c[0], w[j] * c[1], w[j] * c[2]);
}

// Each corner tet scatters its right-hand-side, residual and diagonal contributions straight to
// the vertex vectors (float atomics): holding 8 corners x 3 vectors per hex in registers would
// halve the occupancy of this latency-bound kernel.  Mixed mode runs 9 blocks of 128 per SM
// (56 registers, 72 B of spills; the shared-memory columns allow no tenth block): with the tets
// as a run-time loop more warps hide the FP32 SVD's dependency chains, 1.19 ms at 5 blocks,
// 1.10 at 6, 1.05 at 7, 1.01 at 8, 0.98 at 9 for 2.1M hexes.
template <typename ET, bool PRE>
__global__ void __launch_bounds__(kLocalThreads, sizeof(ET) == 4 ? 9 : 1) k_local(KArgs a) {
  __shared__ ET e12s[36][kLocalThreads];
  __shared__ uint32_t hvs[8][kLocalThreads];
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  if (h >= sg.end) return;
  const MeshScalars &S = a.sc[sg.mesh];
  const ET M = ET(S.M), exp_f = ET(S.exp_f);
  {
    uint32_t hv[8];
    load_hex(a.hexv, h, hv);
    ET E12[12][3];
    hex_edges_mode<ET>(a, hv, E12);
#pragma unroll
    for (int c = 0; c < 8; c++) hvs[c][threadIdx.x] = hv[c];
#pragma unroll
    for (int e = 0; e < 12; e++)
#pragma unroll
      for (int r = 0; r < 3; r++) e12s[e * 3 + r][threadIdx.x] = E12[e][r];
  }
  const int32_t gs = a.gslot[h];
  bool degenerate = false;
#pragma unroll 1
  for (int K = 0; K < 8; K++)
    local_tet<ET, PRE>(a, h, gs, K, &e12s[0][threadIdx.x], M, exp_f, a.energy, &hvs[0][threadIdx.x], degenerate);
  if (PRE && degenerate) atomicOr(&a.sc[sg.mesh].status, 2);
}

// q += S p for the soft-constraint block of L: item i of a constraint segment
template <typename VT>
__device__ __forceinline__ void soft_mv_item(const KArgs &a, const Seg &sg, int64_t i) {
  const MeshDesc md = a.mesh[sg.mesh];
  const MeshScalars &S = a.sc[sg.mesh];
  const VT *in = reinterpret_cast<const VT *>(a.p), *in_a = reinterpret_cast<const VT *>(a.pa);
  VT *out = reinterpret_cast<VT *>(a.q), *out_a = reinterpret_cast<VT *>(a.qa);
  const ConsItem it = cons_item(md, i);
  const int64_t e = it.e;
  if (S.glue && it.kind <= CK_LINE) return;
  if (it.kind == CK_CORNER || it.kind == CK_PROJ) {
    const bool pj = it.kind == CK_PROJ;
    const uint32_t v = (uint32_t)(md.v_off + (pj ? a.b_ids[e] : a.c_ids[e]));
    const VT lc = VT(pj ? S.lamda_P : S.lamda_C);
    const VT *p = in + 4 * (int64_t)v;
    atomic_add3(out, v, lc * p[0], lc * p[1], lc * p[2]);
    return;
  }
  if (it.kind == CK_TANGENT) {
    const uint32_t v = (uint32_t)(md.v_off + a.t_ids[e]);
    const double n0 = a.t_nrm[3 * e], n1 = a.t_nrm[3 * e + 1], n2 = a.t_nrm[3 * e + 2];
    const VT *p = in + 4 * (int64_t)v;
    const double s = S.lamda_T * (n0 * double(p[0]) + n1 * double(p[1]) + n2 * double(p[2]));
    atomic_add3(out, v, VT(s * n0), VT(s * n1), VT(s * n2));
    return;
  }
  if (it.kind == CK_GROUP) {
    const int64_t m0 = a.g_ptr[e], m1 = a.g_ptr[e + 1];
    const double c = S.lamda_G * glue_coef(m1 - m0);
    if (c == 0.0) return;
    double mean[3] = {0, 0, 0};
    for (int64_t k = m0; k < m1; k++)
      for (int d = 0; d < 3; d++) mean[d] += double(in[4 * (int64_t)a.g_vs[k] + d]);
    for (int d = 0; d < 3; d++) mean[d] /= double(m1 - m0);
    for (int64_t k = m0; k < m1; k++) {
      const uint32_t v = (uint32_t)a.g_vs[k];
      const VT *p = in + 4 * (int64_t)v;
      atomic_add3(out, v, VT(c * (double(p[0]) - mean[0])), VT(c * (double(p[1]) - mean[1])),
                  VT(c * (double(p[2]) - mean[2])));
    }
    return;
  }
  {
    const uint32_t v = (uint32_t)(md.v_off + a.l_ids[e]);
    const double ll = S.lamda_L;
    const double x0 = a.l_axis[3 * e], x1 = a.l_axis[3 * e + 1], x2 = a.l_axis[3 * e + 2];
    const VT *p = in + 4 * (int64_t)v;
    const double pa = double(in_a[e]);
    atomic_add3(out, v, VT(ll * (double(p[0]) - x0 * pa)), VT(ll * (double(p[1]) - x1 * pa)),
                VT(ll * (double(p[2]) - x2 * pa)));
    out_a[e] += VT(ll * (-(x0 * double(p[0]) + x1 * double(p[1]) + x2 * double(p[2])) + (x0 * x0 + x1 * x1 + x2 * x2) * pa));
  }
}

// ------------------------------------------------------------------------------- SpMV
// q += K p over the element terms: J' = E(p) B', Q = C' J', forces G = Q B'^T (the cube scale
// is folded into C').  crow points at the hex's coefficient of row 0 (tet 0, component 0); the
// row (K, i) is crow[(K * 6 + i) * 32], in global memory or in the block's shared-memory copy.
template <typename ET, int K>
__device__ __forceinline__ void spmv_tet(const KArgs &a, int32_t gs, const ET E12[12][3], const ET *crow,
                                         ET F[8][3]) {
  ET E[3][3], J[3][3], Q[3][3], G[3][3];
  tet_E12<K>(E12, E);
  const double *B = gs >= 0 ? a.Bgen + ((int64_t)gs * 8 + K) * 9 : nullptr;
  apply_B<K>(E, gs, B, ET(1), J);
  ET c[6];
#pragma unroll
  for (int i = 0; i < 6; i++) c[i] = crow[(K * 6 + i) * 32];
  sym_mul(c, J, Q);
  apply_BT<K>(Q, gs, B, ET(1), G);
  scatter_cols<K>(G, F);
}

// 16-byte asynchronous global -> shared copy (cp.async, cached in L2 only); completion is awaited
// with cp.async.wait_all by the issuing thread, a hardware wait on its own copies.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Mixed mode: 64 registers (8 blocks of 128 per SM), more gathers in flight outweigh the few
// spills; FP64 mode: 128 registers (4 blocks), as its 64-register build spills 1.6 KB a thread.
// Mixed mode: a warp whose 32 hexes fill one AoSoA tile copies the tile's 8 x 6 FP32
// coefficients (6 KB, contiguous) into shared memory with cp.async before it gathers the corner
// ids and directions, so the coefficient stream (70% of the bytes) is in flight while the
// dependent gathers wait; other warps (a mesh tail, or a batch mesh not starting on a multiple
// of 32 hexes) read the coefficients from global memory.
// Blocks past a.hblk (launched by the PCG iteration) apply the soft terms of one constraint
// segment each: they run in the SpMV's tail instead of a launch of their own.
template <typename ET>
__global__ void __launch_bounds__(128, sizeof(ET) == 4 ? 8 : 4) k_spmv(KArgs a) {
  if (blockIdx.x >= a.hblk) {
    const Seg cs = a.cseg[blockIdx.x - a.hblk];
    if (a.sc[cs.mesh].cg_done) return;
    for (int64_t i = cs.begin + threadIdx.x; i < cs.end; i += blockDim.x) soft_mv_item<ET>(a, cs, i);
    return;
  }
  const Seg sg = a.hseg[blockIdx.x];
  if (a.sc[sg.mesh].cg_done) return;
  const int64_t h = sg.begin + threadIdx.x;
  const ET *C = reinterpret_cast<const ET *>(a.Ccoef);
  const ET *crow = C + tet_idx<6>(h, 0, 0);
  bool staged = false;  // every lane of a staged warp is active
  if constexpr (sizeof(ET) == 4) {
    __shared__ __align__(16) float cs[4][48 * 32];  // blockDim.x <= 128
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t hw = sg.begin + 32 * w;  // the warp's first hex
    if ((hw & 31) == 0 && hw + 32 <= sg.end && w < 4) {
      const float *src = C + tet_idx<6>(hw, 0, 0);  // 1536 floats, 16-byte aligned
#pragma unroll
      for (int i = 0; i < 12; i++) cp_async16(&cs[w][(i * 32 + lane) * 4], src + (i * 32 + lane) * 4);
      crow = &cs[w][lane];
      staged = true;
    }
  }
  if (h >= sg.end) return;
  uint32_t hv[8];
  load_hex(a.hexv, h, hv);
  const int32_t gs = a.gslot[h];
  ET E12[12][3];
  hex_edges_vec(reinterpret_cast<const ET *>(a.p), hv, E12);
  if (staged) {
    cp_async_wait_all();
    __syncwarp();
  }
  ET F[8][3];
#pragma unroll
  for (int c = 0; c < 8; c++) F[c][0] = F[c][1] = F[c][2] = ET(0);
  spmv_tet<ET, 0>(a, gs, E12, crow, F);
  spmv_tet<ET, 1>(a, gs, E12, crow, F);
  spmv_tet<ET, 2>(a, gs, E12, crow, F);
  spmv_tet<ET, 3>(a, gs, E12, crow, F);
  spmv_tet<ET, 4>(a, gs, E12, crow, F);
  spmv_tet<ET, 5>(a, gs, E12, crow, F);
  spmv_tet<ET, 6>(a, gs, E12, crow, F);
  spmv_tet<ET, 7>(a, gs, E12, crow, F);
  ET *q = reinterpret_cast<ET *>(a.q);
#pragma unroll
  for (int c = 0; c < 8; c++) atomic_add3(q, hv[c], F[c][0], F[c][1], F[c][2]);
}

// Mixed mode, persistent and software-pipelined form of k_spmv (same sums per hex).  A unit is
// the 32 hexes one warp of k_spmv takes (unit u: segment u / upseg, hexes 32 (u % upseg) on);
// each warp walks the units with a stride of every warp of the grid.  While it computes unit k,
// the coefficient tile of unit k+1 (cp.async into the warp's other shared-memory stage), unit
// k+1's corner ids and cg_done flag, and unit k+2's segment are in flight, so a unit waits only
// for its L2 direction gathers.  Units that do not fill an aligned tile read their coefficients
// from global memory.  Blocks from npipe on apply the soft terms of one constraint segment each.
constexpr int kPipeWarps = 4;
struct PipeUnit {
  int64_t hb, he;  // hex range (hb >= he: nothing to do)
  int32_t mesh;
};
__device__ __forceinline__ PipeUnit pipe_unit(const KArgs &a, int64_t u, int64_t nunits, int upseg) {
  PipeUnit r{0, 0, 0};
  if (u < nunits) {
    const Seg s = a.hseg[u / upseg];
    r.hb = s.begin + 32 * (u % upseg);
    r.he = min(s.end, r.hb + 32);
    r.mesh = s.mesh;
  }
  return r;
}
static __global__ void __launch_bounds__(kPipeWarps * 32, 4) k_spmv_pipe(KArgs a, int npipe, int upseg) {
  if ((int)blockIdx.x >= npipe) {
    const Seg cs = a.cseg[blockIdx.x - npipe];
    if (a.sc[cs.mesh].cg_done) return;
    for (int64_t i = cs.begin + threadIdx.x; i < cs.end; i += blockDim.x) soft_mv_item<float>(a, cs, i);
    return;
  }
  __shared__ __align__(16) float cs[kPipeWarps][2][48 * 32];  // 48 KB
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float *C = reinterpret_cast<const float *>(a.Ccoef);
  const float *p = reinterpret_cast<const float *>(a.p);
  float *q = reinterpret_cast<float *>(a.q);
  const int64_t nunits = a.hblk * upseg, stride = (int64_t)npipe * kPipeWarps;
  int64_t u = (int64_t)blockIdx.x * kPipeWarps + w;
  // stage the coefficient tile of unit t into cs[w][st]; false when it reads global memory
  auto stage = [&](const PipeUnit &t, int st) -> bool {
    if ((t.hb & 31) != 0 || t.he - t.hb != 32) return false;
    const float *src = C + tet_idx<6>(t.hb, 0, 0);  // 1536 floats, 16-byte aligned
#pragma unroll
    for (int i = 0; i < 12; i++) cp_async16(&cs[w][st][(i * 32 + lane) * 4], src + (i * 32 + lane) * 4);
    return true;
  };
  auto load_ids = [&](const PipeUnit &t, uint32_t hv[8]) -> int32_t {
    const int64_t h = t.hb + lane;
    if (h < t.he) {
      load_hex(a.hexv, h, hv);
      return a.gslot[h];
    }
#pragma unroll
    for (int c = 0; c < 8; c++) hv[c] = 0;
    return -1;
  };
  PipeUnit cur = pipe_unit(a, u, nunits, upseg), nxt = pipe_unit(a, u + stride, nunits, upseg);
  uint32_t hv[8];
  int32_t gs = load_ids(cur, hv);
  int done = cur.hb < cur.he ? a.sc[cur.mesh].cg_done : 1;
  bool staged = stage(cur, 0);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  for (int st = 0; u < nunits; u += stride, st ^= 1) {
    // in flight while this unit computes: unit k+2's segment, unit k+1's ids, flag and tile
    const PipeUnit nn = pipe_unit(a, u + 2 * stride, nunits, upseg);
    uint32_t hn[8];
    const int32_t gs_n = load_ids(nxt, hn);
    const int done_n = nxt.hb < nxt.he ? a.sc[nxt.mesh].cg_done : 1;
    const bool staged_n = stage(nxt, st ^ 1);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    const int64_t h = cur.hb + lane;
    const bool live = !done && h < cur.he;
    float E12[12][3];
    if (live) hex_edges_vec(p, hv, E12);
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    __syncwarp();
    if (live) {
      const float *crow = staged ? &cs[w][st][lane] : C + tet_idx<6>(h, 0, 0);
      float F[8][3];
#pragma unroll
      for (int c = 0; c < 8; c++) F[c][0] = F[c][1] = F[c][2] = 0.f;
      spmv_tet<float, 0>(a, gs, E12, crow, F);
      spmv_tet<float, 1>(a, gs, E12, crow, F);
      spmv_tet<float, 2>(a, gs, E12, crow, F);
      spmv_tet<float, 3>(a, gs, E12, crow, F);
      spmv_tet<float, 4>(a, gs, E12, crow, F);
      spmv_tet<float, 5>(a, gs, E12, crow, F);
      spmv_tet<float, 6>(a, gs, E12, crow, F);
      spmv_tet<float, 7>(a, gs, E12, crow, F);
#pragma unroll
      for (int c = 0; c < 8; c++) atomic_add3(q, hv[c], F[c][0], F[c][1], F[c][2]);
    }
    __syncwarp();  // every lane is done with stage st before the next iteration refills it
    cur = nxt;
    nxt = nn;
#pragma unroll
    for (int c = 0; c < 8; c++) hv[c] = hn[c];
    gs = gs_n;
    done = done_n;
    staged = staged_n;
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// ------------------------------------------------------------------------------- soft terms
// add_soft_constraints (slim_m.cpp:597-714) over the constraint items (cons_item): projection
// points lamda_P |x - bc|^2 (ts.projection, :600-610); glue groups lamda_G (n/(n-1))^2
// sum_j |x_j - mean|^2 (ts.glue, :611-646); and, unless the mesh is glued (:647), corners, tangent
// planes and feature lines with their curve unknowns.  This kernel adds the rhs, the diagonal and
// (FP64 mode; mixed mode forms it in k_ir_soft) the residual at x0 (curve unknowns start at 0).
template <typename VT>
__global__ void __launch_bounds__(256) k_soft_rhs(KArgs a) {
  const Seg sg = a.cseg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const MeshScalars &S = a.sc[sg.mesh];
  VT *b = reinterpret_cast<VT *>(a.b), *r = reinterpret_cast<VT *>(a.r), *dg = reinterpret_cast<VT *>(a.diag);
  const ConsItem it = cons_item(md, i);
  const int64_t e = it.e;
  if (S.glue && it.kind <= CK_LINE) return;
  if (it.kind == CK_CORNER || it.kind == CK_PROJ) {
    const bool pj = it.kind == CK_PROJ;
    const uint32_t v = (uint32_t)(md.v_off + (pj ? a.b_ids[e] : a.c_ids[e]));
    const double lc = pj ? S.lamda_P : S.lamda_C;
    const double *cp = pj ? a.b_pos + 3 * e : a.c_pos + 3 * e;
    const double *x = a.X + 4 * (int64_t)v;
    const double c0 = cp[0], c1 = cp[1], c2 = cp[2];
    atomic_add3(b, v, VT(lc * c0), VT(lc * c1), VT(lc * c2));
    if constexpr (sizeof(VT) == 8) atomic_add3(r, v, VT(lc * (c0 - x[0])), VT(lc * (c1 - x[1])), VT(lc * (c2 - x[2])));
    atomic_add3(dg, v, VT(lc), VT(lc), VT(lc));
    return;
  }
  if (it.kind == CK_TANGENT) {
    const uint32_t v = (uint32_t)(md.v_off + a.t_ids[e]);
    const double lt = S.lamda_T;
    const double n0 = a.t_nrm[3 * e], n1 = a.t_nrm[3 * e + 1], n2 = a.t_nrm[3 * e + 2], d = a.t_dis[e];
    const double *x = a.X + 4 * (int64_t)v;
    const double res = lt * (d - (n0 * x[0] + n1 * x[1] + n2 * x[2]));
    atomic_add3(b, v, VT(lt * n0 * d), VT(lt * n1 * d), VT(lt * n2 * d));
    if constexpr (sizeof(VT) == 8) atomic_add3(r, v, VT(res * n0), VT(res * n1), VT(res * n2));
    atomic_add3(dg, v, VT(lt * n0 * n0), VT(lt * n1 * n1), VT(lt * n2 * n2));
    return;
  }
  if (it.kind == CK_GROUP) {
    const int64_t m0 = a.g_ptr[e], m1 = a.g_ptr[e + 1];
    const double c = S.lamda_G * glue_coef(m1 - m0);
    if (c == 0.0) return;
    double mean[3] = {0, 0, 0};
    for (int64_t k = m0; k < m1; k++)
      for (int d = 0; d < 3; d++) mean[d] += a.X[4 * (int64_t)a.g_vs[k] + d];
    for (int d = 0; d < 3; d++) mean[d] /= double(m1 - m0);
    const double w = c * (1.0 - 1.0 / double(m1 - m0));
    for (int64_t k = m0; k < m1; k++) {
      const uint32_t v = (uint32_t)a.g_vs[k];
      const double *x = a.X + 4 * (int64_t)v;
      if constexpr (sizeof(VT) == 8)
        atomic_add3(r, v, VT(c * (mean[0] - x[0])), VT(c * (mean[1] - x[1])), VT(c * (mean[2] - x[2])));
      atomic_add3(dg, v, VT(w), VT(w), VT(w));
    }
    return;
  }
  {
    const uint32_t v = (uint32_t)(md.v_off + a.l_ids[e]);
    const double ll = S.lamda_L;
    const double x0 = a.l_axis[3 * e], x1 = a.l_axis[3 * e + 1], x2 = a.l_axis[3 * e + 2];
    const double o0 = a.l_orig[3 * e], o1 = a.l_orig[3 * e + 1], o2 = a.l_orig[3 * e + 2];
    const double *x = a.X + 4 * (int64_t)v;
    atomic_add3(b, v, VT(ll * o0), VT(ll * o1), VT(ll * o2));
    if constexpr (sizeof(VT) == 8) atomic_add3(r, v, VT(ll * (o0 - x[0])), VT(ll * (o1 - x[1])), VT(ll * (o2 - x[2])));
    atomic_add3(dg, v, VT(ll), VT(ll), VT(ll));
    VT *ba = reinterpret_cast<VT *>(a.ba), *ra = reinterpret_cast<VT *>(a.ra), *dga = reinterpret_cast<VT *>(a.diaga);
    ba[e] = VT(ll * (-x0 * o0 - x1 * o1 - x2 * o2));
    if constexpr (sizeof(VT) == 8) ra[e] = VT(ll * (x0 * (x[0] - o0) + x1 * (x[1] - o1) + x2 * (x[2] - o2)));
    dga[e] = VT(ll * (x0 * x0 + x1 * x1 + x2 * x2));
  }
}

// The soft terms alone (the element SpMV launch runs them in its trailing blocks).
template <typename VT>
__global__ void __launch_bounds__(256) k_soft_mv(KArgs a) {
  const Seg sg = a.cseg[blockIdx.x];
  if (a.sc[sg.mesh].cg_done) return;
  const int64_t i = sg.begin + threadIdx.x;
  if (i < sg.end) soft_mv_item<VT>(a, sg, i);
}

// ------------------------------------------------------------------------------- CG vectors
// Unknown items of a mesh: [0, nv) vertices (3 coordinates), [nv, nv + nl) curve unknowns.
struct ItemRef {
  bool curve;
  int64_t idx;  // global vertex id or global curve entry
};
__device__ __forceinline__ ItemRef item_ref(const MeshDesc &md, int64_t i) {
  const int64_t li = i - md.v_off - md.l_off;
  if (li < md.nv) return {false, md.v_off + li};
  return {true, md.l_off + (li - md.nv)};
}

template <typename T> struct V3 { T x, y, z; };
__device__ __forceinline__ V3<float> ld3(const float *Y, int64_t v) {
  const float4 t = *reinterpret_cast<const float4 *>(Y + 4 * v);
  return {t.x, t.y, t.z};
}
__device__ __forceinline__ V3<double> ld3(const double *Y, int64_t v) {
  const double2 t = *reinterpret_cast<const double2 *>(Y + 4 * v);
  return {t.x, t.y, Y[4 * v + 2]};
}
__device__ __forceinline__ void st3(float *Y, int64_t v, V3<float> a) {
  *reinterpret_cast<float4 *>(Y + 4 * v) = make_float4(a.x, a.y, a.z, 0.f);
}
__device__ __forceinline__ void st3(double *Y, int64_t v, V3<double> a) {
  *reinterpret_cast<double2 *>(Y + 4 * v) = make_double2(a.x, a.y);
  Y[4 * v + 2] = a.z;
  Y[4 * v + 3] = 0.0;
}

// r0 is already formed (local step + soft terms): p = invd r0, delta = 0, q = prox p, norms.
// Held vertices (known_value_post) drop out of the unknowns: zero residual, direction and
// preconditioner; the rhs norm is Eigen's over the free rows of b_i - L_ib x_b.
template <typename VT>
__global__ void __launch_bounds__(256) k_cg_start(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  const MeshDesc md = a.mesh[sg.mesh];
  MeshScalars &S = a.sc[sg.mesh];
  const double prox = S.prox;
  double acc[3] = {0, 0, 0};  // |b|^2, |r|^2, r.p
  VT *r = reinterpret_cast<VT *>(a.r), *p = reinterpret_cast<VT *>(a.p), *d = reinterpret_cast<VT *>(a.d);
  VT *q = reinterpret_cast<VT *>(a.q), *invd = reinterpret_cast<VT *>(a.invd);
  const VT *b = reinterpret_cast<const VT *>(a.b), *dg = reinterpret_cast<const VT *>(a.diag);
  SumAcc<VT> s_bb, s_rr, s_rp;  // mixed mode: FP32 arithmetic, compensated sums
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve && a.has_fixed && a.vfix[it.idx]) {
      // a held vertex (known value): not an unknown -- no residual, direction or preconditioner
      const int64_t v = it.idx;
      const V3<VT> z{VT(0), VT(0), VT(0)};
      st3(p, v, z); st3(d, v, z); st3(invd, v, z); st3(q, v, z); st3(r, v, z);
    } else if (!it.curve && sizeof(VT) == 4) {
      const int64_t v = it.idx;
      const V3<VT> bb = ld3(b, v), rr = ld3(r, v), gg = ld3(dg, v);
      const VT pr = VT(prox);
      const VT b0 = bb.x + pr * VT(a.X[4 * v]), b1 = bb.y + pr * VT(a.X[4 * v + 1]), b2 = bb.z + pr * VT(a.X[4 * v + 2]);
      const VT i0 = VT(1) / (gg.x + pr), i1 = VT(1) / (gg.y + pr), i2 = VT(1) / (gg.z + pr);
      const VT p0 = i0 * rr.x, p1 = i1 * rr.y, p2 = i2 * rr.z;
      st3(p, v, V3<VT>{p0, p1, p2});
      st3(d, v, V3<VT>{VT(0), VT(0), VT(0)});
      st3(invd, v, V3<VT>{i0, i1, i2});
      st3(q, v, V3<VT>{pr * p0, pr * p1, pr * p2});
      s_bb.add_prod(b0, b0); s_bb.add_prod(b1, b1); s_bb.add_prod(b2, b2);
      s_rr.add_prod(rr.x, rr.x); s_rr.add_prod(rr.y, rr.y); s_rr.add_prod(rr.z, rr.z);
      s_rp.add_prod(rr.x, p0); s_rp.add_prod(rr.y, p1); s_rp.add_prod(rr.z, p2);
    } else if (!it.curve) {
      const int64_t v = it.idx;
      const V3<VT> bb = ld3(b, v), rr = ld3(r, v), gg = ld3(dg, v);
      const double x0 = a.X[4 * v], x1 = a.X[4 * v + 1], x2 = a.X[4 * v + 2];
      double b0 = double(bb.x) + prox * x0, b1 = double(bb.y) + prox * x1, b2 = double(bb.z) + prox * x2;
      if (a.has_fixed) {  // Eigen's rhs with known values: b_i - L_ib x_b (q holds L x_b, k_fixed_pre)
        const V3<VT> kq = ld3(q, v);
        b0 -= double(kq.x); b1 -= double(kq.y); b2 -= double(kq.z);
      }
      const double i0 = 1.0 / (double(gg.x) + prox), i1 = 1.0 / (double(gg.y) + prox), i2 = 1.0 / (double(gg.z) + prox);
      const double p0 = i0 * double(rr.x), p1 = i1 * double(rr.y), p2 = i2 * double(rr.z);
      st3(p, v, V3<VT>{VT(p0), VT(p1), VT(p2)});
      st3(d, v, V3<VT>{VT(0), VT(0), VT(0)});
      st3(invd, v, V3<VT>{VT(i0), VT(i1), VT(i2)});
      st3(q, v, V3<VT>{VT(prox * p0), VT(prox * p1), VT(prox * p2)});
      acc[0] += b0 * b0 + b1 * b1 + b2 * b2;
      acc[1] += double(rr.x) * double(rr.x) + double(rr.y) * double(rr.y) + double(rr.z) * double(rr.z);
      acc[2] += double(rr.x) * p0 + double(rr.y) * p1 + double(rr.z) * p2;
    } else {
      const int64_t e = it.idx;
      VT *ra = reinterpret_cast<VT *>(a.ra), *pa = reinterpret_cast<VT *>(a.pa), *da = reinterpret_cast<VT *>(a.da);
      VT *qa = reinterpret_cast<VT *>(a.qa), *invda = reinterpret_cast<VT *>(a.invda);
      const double bb = double(reinterpret_cast<const VT *>(a.ba)[e]);
      const double rr = double(ra[e]);
      const double g = double(reinterpret_cast<const VT *>(a.diaga)[e]);
      const double id = g != 0.0 ? 1.0 / g : 0.0;  // DiagonalPreconditioner: 0 without a diagonal
      const double pp = id * rr;
      pa[e] = VT(pp); da[e] = VT(0); invda[e] = VT(id); qa[e] = VT(0);
      acc[0] += bb * bb; acc[1] += rr * rr; acc[2] += rr * pp;
    }
  }
  if (sizeof(VT) == 4) {
    acc[0] += s_bb.value();
    acc[1] += s_rr.value();
    acc[2] += s_rp.value();
  }
  __shared__ double smem[3][32];
  block_sum<3>(acc, smem);
  if (publish_partials<3>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nvblk)) {
    double v[3];
    gather_partials_sums<3>(a.partials, md.vblk0, md.nvblk, 3, v, smem);
    const double v0 = v[0], v1 = v[1], v2 = v[2];
    if (threadIdx.x == 0) {
      S.rhs_norm2 = v0;
      S.threshold = a.cg_tol * a.cg_tol * v0;
      S.rn2 = v1;
      S.abs_new = v2;
      S.cg_iters = 0;
      S.cg_done = 0;
      if (v0 == 0.0) { S.cg_done = 1; S.cg_error = 0; }
      else if (v1 < S.threshold) { S.cg_done = 1; S.cg_error = sqrt(v1 / v0); }
      else if (a.cg_max_iter <= 0) { S.cg_done = 1; S.cg_error = sqrt(v1 / v0); }
      a.counters[sg.mesh] = 0;
    }
  }
}

// Items whose loads a mixed-mode vector kernel issues together before using them: the plain loop
// waits for each item's loads in turn.
constexpr int kChunk = 2;

// alpha = abs_new / (p . q)
template <typename VT>
__global__ void __launch_bounds__(256) k_cg_alpha(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  MeshScalars &S = a.sc[sg.mesh];
  if (S.cg_done) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const VT *p = reinterpret_cast<const VT *>(a.p), *q = reinterpret_cast<const VT *>(a.q);
  double acc[1] = {0};
  SumAcc<VT> pq;  // mixed mode: compensated FP32 dot product
  if constexpr (sizeof(VT) == 4) {
    // kChunk items' loads issued together, then summed in the item order of the loop below (a
    // curve entry as a vertex with zero y, z: adding 0 * 0 leaves the compensated sum unchanged)
    const VT *pa = reinterpret_cast<const VT *>(a.pa), *qa = reinterpret_cast<const VT *>(a.qa);
    for (int64_t i0 = sg.begin + threadIdx.x; i0 < sg.end; i0 += kChunk * blockDim.x) {
      V3<VT> pp[kChunk], qq[kChunk];
#pragma unroll
      for (int k = 0; k < kChunk; k++) {
        const int64_t i = i0 + k * blockDim.x;
        pp[k] = qq[k] = V3<VT>{VT(0), VT(0), VT(0)};
        if (i < sg.end) {
          const ItemRef it = item_ref(md, i);
          if (!it.curve) { pp[k] = ld3(p, it.idx); qq[k] = ld3(q, it.idx); }
          else { pp[k].x = pa[it.idx]; qq[k].x = qa[it.idx]; }
        }
      }
#pragma unroll
      for (int k = 0; k < kChunk; k++) {
        pq.add_prod(pp[k].x, qq[k].x); pq.add_prod(pp[k].y, qq[k].y); pq.add_prod(pp[k].z, qq[k].z);
      }
    }
  } else
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      const V3<VT> pp = ld3(p, it.idx), qq = ld3(q, it.idx);
      if (sizeof(VT) == 4) {
        pq.add_prod(pp.x, qq.x); pq.add_prod(pp.y, qq.y); pq.add_prod(pp.z, qq.z);
      } else {
        acc[0] += double(pp.x) * double(qq.x) + double(pp.y) * double(qq.y) + double(pp.z) * double(qq.z);
      }
    } else {
      const VT *pa = reinterpret_cast<const VT *>(a.pa), *qa = reinterpret_cast<const VT *>(a.qa);
      if constexpr (sizeof(VT) == 4) pq.add_prod(pa[it.idx], qa[it.idx]);
      else acc[0] += double(pa[it.idx]) * double(qa[it.idx]);
    }
  }
  __shared__ double smem[1][32];
  if constexpr (sizeof(VT) == 4) {
    __shared__ float fsm[1][2][32];
    SumAcc<float> v[1] = {pq};
    block_sum_acc<1>(v, acc, fsm);
  } else {
    block_sum<1>(acc, smem);
  }
  if (publish_partials<1>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nvblk)) {
    double g[1];
    gather_partials_sums<1>(a.partials, md.vblk0, md.nvblk, 1, g, smem);
    const double pAp = g[0];
    if (threadIdx.x == 0) {
      S.alpha = S.abs_new / pAp;
      if (!(pAp > 0.0)) S.status |= 4;
      a.counters[sg.mesh] = 0;
    }
  }
}

// delta += alpha p; r -= alpha q; rn2 = r.r; rz = r.(invd r); convergence / beta
template <typename VT>
__global__ void __launch_bounds__(256) k_cg_update(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  MeshScalars &S = a.sc[sg.mesh];
  if (S.cg_done) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const VT alpha = VT(S.alpha);
  double acc[2] = {0, 0};
  SumAcc<VT> s_rr, s_rz;  // mixed mode: compensated FP32 dot products
  if constexpr (sizeof(VT) == 4) {
    // kChunk items' loads together, then the update and the sums in the loop's item order (a
    // curve entry in the x lane, y and z zero; its r.r and r.z gain only 0 * 0 terms)
    VT *r = reinterpret_cast<VT *>(a.r), *d = reinterpret_cast<VT *>(a.d);
    const VT *p = reinterpret_cast<const VT *>(a.p), *q = reinterpret_cast<const VT *>(a.q);
    const VT *invd = reinterpret_cast<const VT *>(a.invd);
    VT *ra = reinterpret_cast<VT *>(a.ra), *da = reinterpret_cast<VT *>(a.da);
    const VT *pa = reinterpret_cast<const VT *>(a.pa), *qa = reinterpret_cast<const VT *>(a.qa);
    const VT *invda = reinterpret_cast<const VT *>(a.invda);
    for (int64_t i0 = sg.begin + threadIdx.x; i0 < sg.end; i0 += kChunk * blockDim.x) {
      V3<VT> pp[kChunk], qq[kChunk], id[kChunk], dd[kChunk], rr[kChunk];
      int64_t ix[kChunk];
      int kind[kChunk];  // 0 none, 1 vertex, 2 curve entry
#pragma unroll
      for (int k = 0; k < kChunk; k++) {
        const int64_t i = i0 + k * blockDim.x;
        const V3<VT> z{VT(0), VT(0), VT(0)};
        pp[k] = qq[k] = id[k] = dd[k] = rr[k] = z;
        kind[k] = 0;
        ix[k] = 0;
        if (i < sg.end) {
          const ItemRef it = item_ref(md, i);
          ix[k] = it.idx;
          if (!it.curve) {
            kind[k] = 1;
            pp[k] = ld3(p, it.idx); qq[k] = ld3(q, it.idx); id[k] = ld3(invd, it.idx);
            dd[k] = ld3(d, it.idx); rr[k] = ld3(r, it.idx);
          } else {
            kind[k] = 2;
            pp[k].x = pa[it.idx]; qq[k].x = qa[it.idx]; id[k].x = invda[it.idx];
            dd[k].x = da[it.idx]; rr[k].x = ra[it.idx];
          }
        }
      }
#pragma unroll
      for (int k = 0; k < kChunk; k++) {
        if (kind[k] == 0) continue;
        V3<VT> de = dd[k], re = rr[k];
        de.x += alpha * pp[k].x; de.y += alpha * pp[k].y; de.z += alpha * pp[k].z;
        re.x -= alpha * qq[k].x; re.y -= alpha * qq[k].y; re.z -= alpha * qq[k].z;
        if (kind[k] == 1) {
          if (a.has_fixed && a.vfix[ix[k]]) re = V3<VT>{VT(0), VT(0), VT(0)};
          st3(d, ix[k], de);
          st3(r, ix[k], re);
        } else {
          da[ix[k]] = de.x;
          ra[ix[k]] = re.x;
          re.y = re.z = VT(0);
        }
        s_rr.add_prod(re.x, re.x); s_rr.add_prod(re.y, re.y); s_rr.add_prod(re.z, re.z);
        s_rz.add_prod(re.x, id[k].x * re.x); s_rz.add_prod(re.y, id[k].y * re.y); s_rz.add_prod(re.z, id[k].z * re.z);
      }
    }
  } else
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      VT *r = reinterpret_cast<VT *>(a.r), *d = reinterpret_cast<VT *>(a.d);
      const VT *p = reinterpret_cast<const VT *>(a.p), *q = reinterpret_cast<const VT *>(a.q);
      const VT *invd = reinterpret_cast<const VT *>(a.invd);
      const int64_t v = it.idx;
      const V3<VT> pp = ld3(p, v), qq = ld3(q, v), id = ld3(invd, v);
      V3<VT> dd = ld3(d, v), rr = ld3(r, v);
      dd.x += alpha * pp.x; dd.y += alpha * pp.y; dd.z += alpha * pp.z;
      rr.x -= alpha * qq.x; rr.y -= alpha * qq.y; rr.z -= alpha * qq.z;
      if (a.has_fixed && a.vfix[v]) rr = V3<VT>{VT(0), VT(0), VT(0)};
      st3(d, v, dd);
      st3(r, v, rr);
      if (sizeof(VT) == 4) {
        s_rr.add_prod(rr.x, rr.x); s_rr.add_prod(rr.y, rr.y); s_rr.add_prod(rr.z, rr.z);
        s_rz.add_prod(rr.x, id.x * rr.x); s_rz.add_prod(rr.y, id.y * rr.y); s_rz.add_prod(rr.z, id.z * rr.z);
      } else {
        acc[0] += double(rr.x) * double(rr.x) + double(rr.y) * double(rr.y) + double(rr.z) * double(rr.z);
        acc[1] += double(rr.x) * double(id.x * rr.x) + double(rr.y) * double(id.y * rr.y) + double(rr.z) * double(id.z * rr.z);
      }
    } else {
      VT *ra = reinterpret_cast<VT *>(a.ra), *da = reinterpret_cast<VT *>(a.da);
      const VT *pa = reinterpret_cast<const VT *>(a.pa), *qa = reinterpret_cast<const VT *>(a.qa);
      const VT *invda = reinterpret_cast<const VT *>(a.invda);
      const int64_t e = it.idx;
      da[e] += alpha * pa[e];
      const VT rr = ra[e] - alpha * qa[e];
      ra[e] = rr;
      if constexpr (sizeof(VT) == 4) {
        s_rr.add_prod(rr, rr);
        s_rz.add_prod(rr, invda[e] * rr);
      } else {
        acc[0] += double(rr) * double(rr);
        acc[1] += double(rr) * double(invda[e] * rr);
      }
    }
  }
  __shared__ double smem[2][32];
  if constexpr (sizeof(VT) == 4) {
    __shared__ float fsm[2][2][32];
    SumAcc<float> v[2] = {s_rr, s_rz};
    block_sum_acc<2>(v, acc, fsm);
  } else {
    block_sum<2>(acc, smem);
  }
  if (publish_partials<2>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nvblk)) {
    double g[2];
    gather_partials_sums<2>(a.partials, md.vblk0, md.nvblk, 2, g, smem);
    const double rn2 = g[0], rz = g[1];
    if (threadIdx.x == 0) {
      S.rn2 = rn2;
      S.cg_error = sqrt(rn2 / S.rhs_norm2);
      if (rn2 < S.threshold) {
        S.cg_done = 1;
      } else {
        S.beta = rz / S.abs_new;
        S.rz_prev = S.abs_new;
        S.abs_new = rz;
        S.cg_iters += 1;
        if (S.cg_iters >= a.cg_max_iter) S.cg_done = 1;
      }
      a.counters[sg.mesh] = 0;
    }
  }
}

// p = invd r + beta p; q = prox p (vertex) / 0 (curve), ready for the next SpMV
template <typename VT>
__global__ void __launch_bounds__(256) k_cg_dir(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  const MeshScalars &S = a.sc[sg.mesh];
  if (S.cg_done) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const VT beta = VT(S.beta), prox = VT(S.prox);
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
  const ItemRef it = item_ref(md, i);
  if (!it.curve) {
    const VT *r = reinterpret_cast<const VT *>(a.r), *invd = reinterpret_cast<const VT *>(a.invd);
    VT *p = reinterpret_cast<VT *>(a.p), *q = reinterpret_cast<VT *>(a.q);
    const int64_t v = it.idx;
    const V3<VT> rr = ld3(r, v), id = ld3(invd, v);
    V3<VT> pp = ld3(p, v);
    pp.x = id.x * rr.x + beta * pp.x;
    pp.y = id.y * rr.y + beta * pp.y;
    pp.z = id.z * rr.z + beta * pp.z;
    st3(p, v, pp);
    st3(q, v, V3<VT>{prox * pp.x, prox * pp.y, prox * pp.z});
  } else {
    const VT *ra = reinterpret_cast<const VT *>(a.ra), *invda = reinterpret_cast<const VT *>(a.invda);
    VT *pa = reinterpret_cast<VT *>(a.pa), *qa = reinterpret_cast<VT *>(a.qa);
    const int64_t e = it.idx;
    pa[e] = invda[e] * ra[e] + beta * pa[e];
    qa[e] = VT(0);
  }
  }
}

// ------------------------------------------------------------------------------- held vertices
// known_value_post (slim_m.cpp:403-477): p = x_b (the held vertices' positions, 0 on the free
// ones) and q = 0, so that the element SpMV that follows leaves q = L_ib x_b for k_cg_start.
template <typename VT>
__global__ void __launch_bounds__(256) k_fixed_pre(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  const MeshDesc md = a.mesh[sg.mesh];
  if (threadIdx.x == 0) a.sc[sg.mesh].cg_done = 0;
  VT *p = reinterpret_cast<VT *>(a.p), *q = reinterpret_cast<VT *>(a.q);
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      const int64_t v = it.idx;
      const bool fx = a.vfix[v] != 0;
      st3(p, v, V3<VT>{VT(fx ? a.X[4 * v] : 0.0), VT(fx ? a.X[4 * v + 1] : 0.0), VT(fx ? a.X[4 * v + 2] : 0.0)});
      st3(q, v, V3<VT>{VT(0), VT(0), VT(0)});
    }
  }
}

// ------------------------------------------------------------------------------- adaptive loop
// The result mesh slim_solve2's adaptive branch checks (slim_m.cpp:1237-1260): type 1 (gluing)
// every vertex of a glue group at the mean of its group; type 0 (projection) the projection
// points at their targets bc.  Xm starts as a copy of X.
static __global__ void __launch_bounds__(256) k_result_positions(KArgs a, double *Xm, int type) {
  const Seg sg = a.cseg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const ConsItem it = cons_item(md, i);
  if (type == 1 && it.kind == CK_GROUP) {
    const int64_t m0 = a.g_ptr[it.e], m1 = a.g_ptr[it.e + 1];
    double mean[3] = {0, 0, 0};
    for (int64_t k = m0; k < m1; k++)
      for (int d = 0; d < 3; d++) mean[d] += a.X[4 * (int64_t)a.g_vs[k] + d];
    for (int d = 0; d < 3; d++) mean[d] /= double(m1 - m0);
    for (int64_t k = m0; k < m1; k++)
      for (int d = 0; d < 3; d++) Xm[4 * (int64_t)a.g_vs[k] + d] = mean[d];
  } else if (type == 0 && it.kind == CK_PROJ) {
    const int64_t v = md.v_off + a.b_ids[it.e];
    for (int d = 0; d < 3; d++) Xm[4 * v + d] = a.b_pos[3 * it.e + d];
  }
}

// Glue weight schedules, one thread per mesh, frozen meshes untouched.  before = 1: slim_solve's
// doubling at the start of iteration `iter` (lamda_glue *= 2 once iter > 3, while below 1e8,
// slim_m.cpp:1311-1312); before = 0: slim_solve2's update after an iteration,
// lamda_glue = min(1e4 max(E_quality / E_soft lamda_glue, 1), 1e16) (slim_m.cpp:1258).
static __global__ void k_glue_schedule(MeshScalars *sc, int n, int before, int iter) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  MeshScalars &S = sc[m];
  if (S.frozen) return;
  if (before) {
    if (iter > 3 && S.lamda_G < 1e8) S.lamda_G *= 2;
  } else {
    S.lamda_G = fmin(1e4 * fmax(S.eq / S.es * S.lamda_G, 1.0), 1e16);
  }
}

// ------------------------------------------------------------------------------- FP64 refinement
// Mixed mode solves L delta = r0 with FP32 PCG iterations but keeps the solve anchored to the
// FP64 positions: every cg_refine iterations the FP32 update d moves into the FP64 accumulator
// dd, and the residual r = b - L (x0 + dd) is re-evaluated from the FP64 positions instead of
// being carried by the FP32 recurrence (a residual replacement; the search direction p is kept,
// and beta restarts from the new r.z, so the Krylov process goes on).  The element part of the
// residual is M W^T W (R - J(x0 + dd)) B^T with R the local step's stored rotation; R - J(x0) is
// formed in double-float arithmetic (TwoSum / FMA error terms, about 48 bits) from the FP64
// positions' hi/lo split, so its error is relative to the residual, not to J; the soft and
// proximal parts are formed in FP64.  The initial residual of every solve is formed the same way.

// The 12 hex edges of X in double-float from the split positions: E = Eh + El to about 2^-48
// relative (TwoSum of the hi parts, the lo parts and the error term added in FP32).
__device__ __forceinline__ void hex_edges_split_df(const float *X32, const uint32_t hv[8], float Eh[12][3],
                                                   float El[12][3]) {
  float H[8][3], L[8][3];
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const float4 hh = __ldg(reinterpret_cast<const float4 *>(X32) + 2 * (int64_t)hv[c]);
    const float4 ll = __ldg(reinterpret_cast<const float4 *>(X32) + 2 * (int64_t)hv[c] + 1);
    H[c][0] = hh.x; H[c][1] = hh.y; H[c][2] = hh.z;
    L[c][0] = ll.x; L[c][1] = ll.y; L[c][2] = ll.z;
  }
#pragma unroll
  for (int e = 0; e < 12; e++)
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const float x = H[hex_edge_hi(e)][r], y = -H[hex_edge_lo(e)][r];
      const float sum = __fadd_rn(x, y);
      const float z = __fsub_rn(sum, x);
      const float err = __fadd_rn(__fsub_rn(x, __fsub_rn(sum, z)), __fsub_rn(y, z));
      Eh[e][r] = sum;
      El[e][r] = __fadd_rn(__fsub_rn(L[hex_edge_hi(e)][r], L[hex_edge_lo(e)][r]), err);
    }
}

// Corner tet K's element residual force G (columns: forces on the tet's vertices 1..3; vertex 0
// gets minus their sum), accumulated into F.  Edges of x = X + dd are Eh + Elo: Eh the hi part of
// X's double-float edges, Elo their lo part plus the edges of dd (both small next to Eh).
template <int K>
__device__ __forceinline__ void ir_tet(const KArgs &a, int64_t h, int32_t gs, const float Eh12[12][3],
                                       const float El12[12][3], const float *rrow, float F[8][3]) {
  float Eh[3][3], El[3][3];
  tet_E12<K>(Eh12, Eh);
  tet_E12<K>(El12, El);
  const float *Sinv = reinterpret_cast<const float *>(a.Sinv);
  const float *Cc = reinterpret_cast<const float *>(a.Ccoef);
  float res[3][3];
  float G[3][3], Q[3][3], c[6];
  if (gs < 0) {
    // J = is E R_k^T: column edge_axis(K, j) is sg E[:, j] with sg = +-is; R - J with the hi
    // product's exact error (FMA) and the lo part subtracted after the (near-cancelling) hi part
    const float is = Sinv[tet_idx<1>(h, K, 0)];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int ax = edge_axis(K, j);
      const float sg = float(edge_sign(K, j)) * is;
#pragma unroll
      for (int r = 0; r < 3; r++) {
        const float jh = __fmul_rn(Eh[r][j], sg);
        const float jl = __fadd_rn(__fmaf_rn(Eh[r][j], sg, -jh), __fmul_rn(El[r][j], sg));
        res[r][ax] = __fsub_rn(__fsub_rn(rrow[(K * 9 + r * 3 + ax) * 32], jh), jl);
      }
    }
#pragma unroll
    for (int i = 0; i < 6; i++) c[i] = Cc[tet_idx<6>(h, K, i)];
    // C' holds c is^2 (the scale folded in), and the force is is (c res) R_k = (C' res) R_k / is
    sym_mul(c, res, Q);
    apply_BT<K>(Q, gs, nullptr, 1.0f / is, G);
  } else {
    const double *B = a.Bgen + ((int64_t)gs * 8 + K) * 9;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int cc = 0; cc < 3; cc++) {
        double jv = 0;
#pragma unroll
        for (int k = 0; k < 3; k++) jv += (double(Eh[r][k]) + double(El[r][k])) * B[k * 3 + cc];
        res[r][cc] = float(double(rrow[(K * 9 + r * 3 + cc) * 32]) - jv);
      }
#pragma unroll
    for (int i = 0; i < 6; i++) c[i] = Cc[tet_idx<6>(h, K, i)];
    sym_mul(c, res, Q);
    apply_BT<K>(Q, gs, B, 1.0f, G);
  }
  scatter_cols<K>(G, F);
}

// r += element residual at X + dd (r starts at -prox dd, or at 0 for the initial residual).
// A warp whose 32 hexes fill one AoSoA tile copies the tile's 8 x 9 rotations (9 KB, contiguous)
// into shared memory with cp.async before its dependent corner gathers, as k_spmv does with C'.
static __global__ void __launch_bounds__(128, 4) k_ir_resid(KArgs a, int replace) {
  const Seg sg = a.hseg[blockIdx.x];
  if (replace && a.sc[sg.mesh].cg_done) return;
  const int64_t h = sg.begin + threadIdx.x;
  const float *rrow = a.Rrot + tet_idx<9>(h, 0, 0);  // row (K, i) at rrow[(K * 9 + i) * 32]
  bool staged = false;  // every lane of a staged warp is active
  {
    __shared__ __align__(16) float rs[4][72 * 32];  // blockDim.x <= 128
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t hw = sg.begin + 32 * w;
    if ((hw & 31) == 0 && hw + 32 <= sg.end && w < 4) {
      const float *src = a.Rrot + tet_idx<9>(hw, 0, 0);  // 2304 floats, 16-byte aligned
#pragma unroll
      for (int i = 0; i < 18; i++) cp_async16(&rs[w][(i * 32 + lane) * 4], src + (i * 32 + lane) * 4);
      rrow = &rs[w][lane];
      staged = true;
    }
  }
  if (h >= sg.end) return;
  uint32_t hv[8];
  load_hex(a.hexv, h, hv);
  const int32_t gs = a.gslot[h];
  float Eh[12][3], El[12][3];
  hex_edges_split_df(a.X32, hv, Eh, El);
  if (replace) {  // the update dd at FP32 (zero for the initial residual)
    float P[8][3];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const float4 u = __ldg(reinterpret_cast<const float4 *>(a.ddf) + hv[c]);
      P[c][0] = u.x; P[c][1] = u.y; P[c][2] = u.z;
    }
#pragma unroll
    for (int e = 0; e < 12; e++)
#pragma unroll
      for (int r = 0; r < 3; r++) El[e][r] = __fadd_rn(El[e][r], P[hex_edge_hi(e)][r] - P[hex_edge_lo(e)][r]);
  }
  if (staged) {
    cp_async_wait_all();
    __syncwarp();
  }
  float F[8][3];
#pragma unroll
  for (int c = 0; c < 8; c++) F[c][0] = F[c][1] = F[c][2] = 0.f;
  ir_tet<0>(a, h, gs, Eh, El, rrow, F);
  ir_tet<1>(a, h, gs, Eh, El, rrow, F);
  ir_tet<2>(a, h, gs, Eh, El, rrow, F);
  ir_tet<3>(a, h, gs, Eh, El, rrow, F);
  ir_tet<4>(a, h, gs, Eh, El, rrow, F);
  ir_tet<5>(a, h, gs, Eh, El, rrow, F);
  ir_tet<6>(a, h, gs, Eh, El, rrow, F);
  ir_tet<7>(a, h, gs, Eh, El, rrow, F);
  float *r = reinterpret_cast<float *>(a.r);
#pragma unroll
  for (int c = 0; c < 8; c++) atomic_add3(r, hv[c], F[c][0], F[c][1], F[c][2]);
}

// Soft-constraint residual at x = X + dd (curve unknowns a = dda), in FP64: corners and
// projection points lamda (c - x), tangent planes lamda_T n (d - n.x), lines lamda_L (o + a t - x)
// on the vertex rows and lamda_L (t.(x - o) - |t|^2 a) on the curve row (add_soft_constraints'
// system).  Glue groups and held vertices are FP64-mode only.
static __global__ void __launch_bounds__(256) k_ir_soft(KArgs a, int replace) {
  const Seg sg = a.cseg[blockIdx.x];
  const MeshScalars &S = a.sc[sg.mesh];
  if (replace && S.cg_done) return;
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = a.mesh[sg.mesh];
  float *r = reinterpret_cast<float *>(a.r);
  const ConsItem it = cons_item(md, i);
  const int64_t e = it.e;
  if (it.kind == CK_GROUP || (S.glue && it.kind <= CK_LINE)) return;
  const int32_t lv = it.kind == CK_CORNER ? a.c_ids[e] : it.kind == CK_TANGENT ? a.t_ids[e]
                   : it.kind == CK_LINE ? a.l_ids[e] : a.b_ids[e];
  const int64_t v = md.v_off + lv;
  const double x0 = a.X[4 * v] + a.dd[4 * v], x1 = a.X[4 * v + 1] + a.dd[4 * v + 1], x2 = a.X[4 * v + 2] + a.dd[4 * v + 2];
  if (it.kind == CK_CORNER || it.kind == CK_PROJ) {
    const double lc = it.kind == CK_PROJ ? S.lamda_P : S.lamda_C;
    const double *cp = it.kind == CK_PROJ ? a.b_pos + 3 * e : a.c_pos + 3 * e;
    atomic_add3(r, (uint32_t)v, float(lc * (cp[0] - x0)), float(lc * (cp[1] - x1)), float(lc * (cp[2] - x2)));
  } else if (it.kind == CK_TANGENT) {
    const double n0 = a.t_nrm[3 * e], n1 = a.t_nrm[3 * e + 1], n2 = a.t_nrm[3 * e + 2];
    const double res = S.lamda_T * (a.t_dis[e] - (n0 * x0 + n1 * x1 + n2 * x2));
    atomic_add3(r, (uint32_t)v, float(res * n0), float(res * n1), float(res * n2));
  } else {
    const double ll = S.lamda_L, al = a.dda[e];
    const double t0 = a.l_axis[3 * e], t1 = a.l_axis[3 * e + 1], t2 = a.l_axis[3 * e + 2];
    const double o0 = a.l_orig[3 * e], o1 = a.l_orig[3 * e + 1], o2 = a.l_orig[3 * e + 2];
    atomic_add3(r, (uint32_t)v, float(ll * (o0 + al * t0 - x0)), float(ll * (o1 + al * t1 - x1)),
                float(ll * (o2 + al * t2 - x2)));
    reinterpret_cast<float *>(a.ra)[e] =
        float(ll * (t0 * (x0 - o0) + t1 * (x1 - o1) + t2 * (x2 - o2) - (t0 * t0 + t1 * t1 + t2 * t2) * al));
  }
}

// Replacement, first pass over the unknowns: dd += d, d = 0 (curve entries: dda += da, da = 0),
// and r = -prox dd (the proximal term's residual prox (x0 - x)); the element and soft passes add
// the rest.
static __global__ void __launch_bounds__(256) k_ir_acc(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  const MeshScalars &S = a.sc[sg.mesh];
  if (S.cg_done) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const double prox = S.prox;
  float *d = reinterpret_cast<float *>(a.d), *r = reinterpret_cast<float *>(a.r);
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      const int64_t v = it.idx;
      const V3<float> dv = ld3(d, v);
      double2 u = *reinterpret_cast<const double2 *>(a.dd + 4 * v);
      double w = a.dd[4 * v + 2];
      u.x += double(dv.x); u.y += double(dv.y); w += double(dv.z);
      *reinterpret_cast<double2 *>(a.dd + 4 * v) = u;
      a.dd[4 * v + 2] = w;
      st3(a.ddf, v, V3<float>{float(u.x), float(u.y), float(w)});
      st3(d, v, V3<float>{0.f, 0.f, 0.f});
      st3(r, v, V3<float>{float(-prox * u.x), float(-prox * u.y), float(-prox * w)});
    } else {
      float *da = reinterpret_cast<float *>(a.da);
      a.dda[it.idx] += double(da[it.idx]);
      da[it.idx] = 0.f;
    }
  }
}

// Replacement, last pass: |r|^2 and r.z of the re-evaluated residual (compensated FP32 sums); the
// Eigen stopping test on it, and beta = (r.z) / (r.z before the update) for the next direction.
static __global__ void __launch_bounds__(256) k_ir_norm(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  MeshScalars &S = a.sc[sg.mesh];
  if (S.cg_done) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const float *r = reinterpret_cast<const float *>(a.r), *invd = reinterpret_cast<const float *>(a.invd);
  SumAcc<float> s_rr, s_rz;
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      const V3<float> rr = ld3(r, it.idx), id = ld3(invd, it.idx);
      s_rr.add_prod(rr.x, rr.x); s_rr.add_prod(rr.y, rr.y); s_rr.add_prod(rr.z, rr.z);
      s_rz.add_prod(rr.x, id.x * rr.x); s_rz.add_prod(rr.y, id.y * rr.y); s_rz.add_prod(rr.z, id.z * rr.z);
    } else {
      const float rr = reinterpret_cast<const float *>(a.ra)[it.idx];
      const float id = reinterpret_cast<const float *>(a.invda)[it.idx];
      s_rr.add_prod(rr, rr);
      s_rz.add_prod(rr, id * rr);
    }
  }
  double acc[2];
  __shared__ double smem[2][32];
  __shared__ float fsm[2][2][32];
  SumAcc<float> v[2] = {s_rr, s_rz};
  block_sum_acc<2>(v, acc, fsm);
  if (publish_partials<2>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nvblk)) {
    double g[2];
    gather_partials_sums<2>(a.partials, md.vblk0, md.nvblk, 2, g, smem);
    if (threadIdx.x == 0) {
      S.rn2 = g[0];
      S.cg_error = sqrt(g[0] / S.rhs_norm2);
      if (g[0] < S.threshold) {
        S.cg_done = 1;
      } else {
        S.beta = g[1] / S.rz_prev;
        S.abs_new = g[1];
      }
      a.counters[sg.mesh] = 0;
    }
  }
}

// After the PCG: the search direction d = fl32(dd + d) and da = fl32(dda + da), every mesh.
static __global__ void __launch_bounds__(256) k_ir_final(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  const MeshDesc md = a.mesh[sg.mesh];
  float *d = reinterpret_cast<float *>(a.d);
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      const int64_t v = it.idx;
      const V3<float> dv = ld3(d, v);
      const double2 u = *reinterpret_cast<const double2 *>(a.dd + 4 * v);
      const double w = a.dd[4 * v + 2];
      st3(d, v, V3<float>{float(u.x + double(dv.x)), float(u.y + double(dv.y)), float(w + double(dv.z))});
    } else {
      float *da = reinterpret_cast<float *>(a.da);
      da[it.idx] = float(a.dda[it.idx] + double(da[it.idx]));
    }
  }
}

// ------------------------------------------------------------------------------- line search
// Smallest positive root of det(E + t D) = 0 (get_min_pos_root_3D, flip_avoiding_line_search.cpp:
// 177-271), FP64.  The cubic is solved by the trigonometric / Cardano method of SolveP3 (:24-61).
static __device__ double smallest_pos_quad_zero(double a, double b, double c) {
  double t1, t2;
  if (fabs(a) > 1.0e-10) {
    const double delta_in = b * b - 4 * a * c;
    if (delta_in <= 0) return INFINITY;
    const double delta = sqrt(delta_in);
    if (b >= 0) {
      const double bd = -b - delta;
      t1 = 2 * c / bd;
      t2 = bd / (2 * a);
    } else {
      const double bd = -b + delta;
      t1 = bd / (2 * a);
      t2 = (2 * c) / bd;
    }
    if (a < 0) { const double tt = t1; t1 = t2; t2 = tt; }
    if (t1 > 0) return t2 > 0 ? t2 : t1;
    return INFINITY;
  }
  if (b == 0) return INFINITY;
  t1 = -c / b;
  return t1 > 0 ? t1 : INFINITY;
}

static __device__ double min_pos_root(const double E[3][3], const double D[3][3]) {
  double M[3][3];
  const double c3 = det3(D), c0 = det3(E);
  double c1 = 0, c2 = 0;
#pragma unroll
  for (int col = 0; col < 3; col++) {
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int cc = 0; cc < 3; cc++) M[r][cc] = (cc == col) ? D[r][cc] : E[r][cc];
    c1 += det3(M);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int cc = 0; cc < 3; cc++) M[r][cc] = (cc == col) ? E[r][cc] : D[r][cc];
    c2 += det3(M);
  }
  double a = -c3, b = -c2, c = -c1, d = -c0;
  if (fabs(a) <= 1.e-10) return smallest_pos_quad_zero(b, c, d);
  b /= a; c /= a; d /= a;
  // cubic x^3 + b x^2 + c x + d
  const double a2 = b * b;
  double q = (a2 - 3 * c) / 9;
  const double r = (b * (2 * a2 - 9 * c) + 27 * d) / 54;
  const double r2 = r * r, q3 = q * q * q;
  double x0, x1, x2;
  int nr;
  if (r2 < q3) {
    double t = r / sqrt(q3);
    t = fmin(1.0, fmax(-1.0, t));
    t = acos(t);
    const double a3 = b / 3;
    q = -2 * sqrt(q);
    x0 = q * cos(t / 3) - a3;
    x1 = q * cos((t + (2 * M_PI)) / 3) - a3;
    x2 = q * cos((t - (2 * M_PI)) / 3) - a3;
    nr = 3;
  } else {
    double A = -pow(fabs(r) + sqrt(r2 - q3), 1. / 3);
    if (r < 0) A = -A;
    const double Bc = (A == 0) ? 0 : q / A;
    const double a3 = b / 3;
    x0 = (A + Bc) - a3;
    x1 = -0.5 * (A + Bc) - a3;
    x2 = 0.5 * sqrt(3.) * (A - Bc);
    nr = 1;
    if (fabs(x2) < 1e-14) { x2 = x1; nr = 2; }
  }
  if (nr == 1) return (x0 >= 0) ? x0 : INFINITY;
  if (nr == 2) {
    const double mx = fmax(x0, x1), mn = fmin(x0, x1);
    if (mn > 0) return mn;
    if (mx > 0) return mx;
    return INFINITY;
  }
  // sort three
  double lo = fmin(x0, fmin(x1, x2)), hi = fmax(x0, fmax(x1, x2));
  double mid = x0 + x1 + x2 - lo - hi;
  if (lo > 0) return lo;
  if (mid > 0) return mid;
  if (hi > 0) return hi;
  return INFINITY;
}

template <typename VT, int K>
__device__ __forceinline__ void tet_dir(const VT *d, const uint32_t hv[8], double Dd[3][3]) {
  VT p0[3];
  load_vec(d, hv[tet_v(K, 0)], p0);
#pragma unroll
  for (int j = 0; j < 3; j++) {
    VT q[3];
    load_vec(d, hv[tet_v(K, j + 1)], q);
    Dd[0][j] = double(q[0]) - double(p0[0]);
    Dd[1][j] = double(q[1]) - double(p0[1]);
    Dd[2][j] = double(q[2]) - double(p0[2]);
  }
}

// FP64 energy density of corner tet K (vertices v0..v3 in tet_v order) at X + alpha d.  Out of
// line: it runs only for near-degenerate tets, and one copy per corner tet keeps the candidate
// loops of the line-search kernels small.
template <typename VT, int K>
__device__ __noinline__ double tet_energy_exact(const double *X, const VT *d, uint32_t v0, uint32_t v1, uint32_t v2,
                                                uint32_t v3, int32_t gs, const double *B, double is, double alpha,
                                                int energy, double exp_f) {
  const uint32_t vj[3] = {v1, v2, v3};
  double p0[3];
  VT d0[3];
  load_pos(X, v0, p0);
  load_vec(d, v0, d0);
  double Ed[3][3], Jd[3][3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    double q[3];
    VT dq[3];
    load_pos(X, vj[j], q);
    load_vec(d, vj[j], dq);
#pragma unroll
    for (int r = 0; r < 3; r++) Ed[r][j] = (q[r] - p0[r]) + alpha * (double(dq[r]) - double(d0[r]));
  }
  apply_B<K>(Ed, gs, B, is, Jd);
  return tet_energy_density<double>(energy, exp_f, Jd);
}

// Energy density of corner tet K at edges E (ET); tets with |det J| below 1e-3 are re-evaluated
// in FP64 from the FP64 positions (mixed mode only).
template <typename ET, typename VT, int K>
__device__ __forceinline__ void tet_energy_acc(const KArgs &a, int64_t h, const uint32_t hv[8], int32_t gs,
                                               const ET E[3][3], double alpha, SumAcc<ET> &fast, double &slow) {
  const ET *Sinv = reinterpret_cast<const ET *>(a.Sinv);
  const double *B = gs >= 0 ? a.Bgen + ((int64_t)gs * 8 + K) * 9 : nullptr;
  const ET is = Sinv[tet_idx<1>(h, K, 0)];
  ET J[3][3];
  apply_B<K>(E, gs, B, is, J);
  const ET e = tet_energy_density<ET>(a.energy, ET(a.sc_exp_f), J);
  if (sizeof(ET) == 4) {
    const ET d = det3(J);
    if (!(fabs(d) > ET(1e-3))) {
      slow += tet_energy_exact<VT, K>(a.X, reinterpret_cast<const VT *>(a.d), hv[tet_v(K, 0)], hv[tet_v(K, 1)],
                                      hv[tet_v(K, 2)], hv[tet_v(K, 3)], gs, B, double(is), alpha, a.energy,
                                      a.sc_exp_f);
      return;
    }
  }
  fast.add(e);
}

// Flip-avoiding step bound of corner tet K.  Only a root of det(E + t D) in [0, 1.25] can lower
// max_step = min(1, 0.8 min_root).  The cubic's coefficients are formed in ET and converted to the
// Bernstein basis on [0, 1.25]; when all four Bernstein coefficients keep the sign of det E with a
// margin that covers the ET rounding (bounded through Hadamard's inequality), there is no root in
// the interval and the tet is skipped.  Otherwise the smallest positive root is solved in FP64
// exactly as the reference does.
template <typename ET, int K>
__device__ __forceinline__ bool tet_bound(const ET E[3][3], const ET D[3][3]) {
  ET ne[3], nd[3];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    ne[j] = sqrt(E[0][j] * E[0][j] + E[1][j] * E[1][j] + E[2][j] * E[2][j]);
    nd[j] = sqrt(D[0][j] * D[0][j] + D[1][j] * D[1][j] + D[2][j] * D[2][j]);
  }
  const ET T = ET(1.25);
  const ET M0 = ne[0] * ne[1] * ne[2];
  const ET M1 = nd[0] * ne[1] * ne[2] + ne[0] * nd[1] * ne[2] + ne[0] * ne[1] * nd[2];
  const ET M2 = nd[0] * nd[1] * ne[2] + nd[0] * ne[1] * nd[2] + ne[0] * nd[1] * nd[2];
  const ET M3 = nd[0] * nd[1] * nd[2];
  // det(E + tD) = c0 + c1 t + c2 t^2 + c3 t^3
  ET Mx[3][3];
  const ET c0 = det3(E), c3 = det3(D);
  ET c1 = 0, c2 = 0;
#pragma unroll
  for (int col = 0; col < 3; col++) {
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int cc = 0; cc < 3; cc++) Mx[r][cc] = (cc == col) ? D[r][cc] : E[r][cc];
    c1 += det3(Mx);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int cc = 0; cc < 3; cc++) Mx[r][cc] = (cc == col) ? E[r][cc] : D[r][cc];
    c2 += det3(Mx);
  }
  const ET a1 = c1 * T, a2 = c2 * T * T, a3 = c3 * T * T * T;
  const ET b0 = c0, b1 = c0 + a1 / ET(3), b2 = c0 + ET(2) * a1 / ET(3) + a2 / ET(3), b3 = c0 + a1 + a2 + a3;
  const ET rel = sizeof(ET) == 4 ? ET(2e-5) : ET(1e-13);
  const ET err = rel * (M0 + M1 * T + M2 * T * T + M3 * T * T * T);
  const bool pos = b0 > err && b1 > err && b2 > err && b3 > err;
  const bool neg = b0 < -err && b1 < -err && b2 < -err && b3 < -err;
  return !(pos || neg);
}

// Corner tet K of hex h (K at run time) -> its FP64 edges and direction edges.
template <typename VT>
__device__ __forceinline__ void tet_edges_dir(const KArgs &a, const uint32_t hv[8], int K, double E[3][3],
                                              double D[3][3]) {
  const VT *d = reinterpret_cast<const VT *>(a.d);
  switch (K) {
    case 0: tet_edges<0>(a.X, hv, E); tet_dir<VT, 0>(d, hv, D); break;
    case 1: tet_edges<1>(a.X, hv, E); tet_dir<VT, 1>(d, hv, D); break;
    case 2: tet_edges<2>(a.X, hv, E); tet_dir<VT, 2>(d, hv, D); break;
    case 3: tet_edges<3>(a.X, hv, E); tet_dir<VT, 3>(d, hv, D); break;
    case 4: tet_edges<4>(a.X, hv, E); tet_dir<VT, 4>(d, hv, D); break;
    case 5: tet_edges<5>(a.X, hv, E); tet_dir<VT, 5>(d, hv, D); break;
    case 6: tet_edges<6>(a.X, hv, E); tet_dir<VT, 6>(d, hv, D); break;
    default: tet_edges<7>(a.X, hv, E); tet_dir<VT, 7>(d, hv, D); break;
  }
}

// Dense exact pass over the recorded tets: the reference's smallest positive root in FP64, one
// tet per thread, reduced per mesh by atomicMin on the bits of the (non-negative) root.
template <typename VT>
// Each thread keeps the minimum of its entries per mesh (flushed when the mesh changes); at the
// end a warp whose lanes all hold the same mesh takes one atomic instead of 32, which keeps the
// single-mesh case off one contended word.  Roots are non-negative, so their bit patterns order
// like the doubles.
__global__ void __launch_bounds__(128) k_ls_roots(KArgs a) {
  const unsigned n = *a.root_count;
  int32_t mesh = -1;
  unsigned long long best = ~0ull;
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const uint32_t code = a.root_list[e];
    const int64_t h = code >> 3;
    uint32_t hv[8];
    load_hex(a.hexv, h, hv);
    double E[3][3], D[3][3];
    tet_edges_dir<VT>(a, hv, (int)(code & 7), E, D);
    const double r = min_pos_root(E, D);
    const int32_t m = a.root_mesh[e];
    if (m != mesh) {
      if (mesh >= 0) atomicMin(a.root_min + mesh, best);
      mesh = m;
      best = ~0ull;
    }
    const unsigned long long rb = (unsigned long long)__double_as_longlong(r);
    best = rb < best ? rb : best;
  }
  const int32_t m0 = __shfl_sync(0xffffffffu, mesh, 0);
  const bool same = __all_sync(0xffffffffu, mesh == m0 || mesh < 0);
  if (same && m0 >= 0) {
    unsigned long long w = best;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, w, o);
      w = y < w ? y : w;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(a.root_min + m0, w);
  } else if (!same && mesh >= 0) {
    atomicMin(a.root_min + mesh, best);
  }
}

// max_step = min(1, 0.8 min_root) per mesh; re-arms the minimum and the list for the next call.
// One block of 128 per mesh (after k_ls_roots): the mesh's energy at the current positions from
// k_ls_bound's partials (fixed order), the step bound from the minimum root, and the line-search
// state reset.
static __global__ void __launch_bounds__(128) k_ls_bound_finish(KArgs a, int n_meshes) {
  const int m = blockIdx.x;
  const MeshDesc md = a.mesh[m];
  __shared__ double smem[1][32];
  double g[1];
  gather_partials_sums<1>(a.partials, md.hblk0, md.nhblk, 1, g, smem);
  if (threadIdx.x == 0) {
    if (m == 0) { *a.root_count = 0; *a.ls_active = (unsigned)n_meshes; *a.ls_round = 0; }
    MeshScalars &S = a.sc[m];
    S.old_eq = g[0];
    S.ls_done = 0;
    const double r = __longlong_as_double((long long)a.root_min[m]);
    S.min_root = r;
    S.max_step = fmin(1.0, r * 0.8);
    a.root_min[m] = (unsigned long long)__double_as_longlong(INFINITY);
  }
}



// Pass 1: step bound over the tets and the quality energy at the current X.  Mixed mode runs 8
// blocks of 128 per SM (64 registers, ~500 B of spills to L1): the kernel waits on its corner
// gathers, and twice the warps of the 128-register build hide more of that than the spills cost.
template <typename ET, typename VT>
__global__ void __launch_bounds__(128, sizeof(ET) == 4 ? 8 : 1) k_ls_bound(KArgs a) {
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  MeshScalars &S = a.sc[sg.mesh];
  double eq[1] = {0};
  unsigned need = 0;  // bit K: corner tet K needs the exact root
  if (h < sg.end) {
    uint32_t hv[8];
    load_hex(a.hexv, h, hv);
    const int32_t gs = a.gslot[h];
    ET E12[12][3];
    hex_edges_mode<ET>(a, hv, E12);
    // the energy at the current positions first, then the direction frame and the root screens,
    // so the two sets of temporaries are never live together
    SumAcc<ET> efast;
    double eslow = 0;
#define HX_LS_E(K)                                                \
    {                                                             \
      ET E[3][3];                                                 \
      tet_E12<K>(E12, E);                                         \
      tet_energy_acc<ET, VT, K>(a, h, hv, gs, E, 0.0, efast, eslow); \
    }
    HX_LS_E(0) HX_LS_E(1) HX_LS_E(2) HX_LS_E(3) HX_LS_E(4) HX_LS_E(5) HX_LS_E(6) HX_LS_E(7)
#undef HX_LS_E
    ET D12[12][3];
    {
      VT Dv[12][3];
      hex_edges_vec(reinterpret_cast<const VT *>(a.d), hv, Dv);
#pragma unroll
      for (int e = 0; e < 12; e++)
#pragma unroll
        for (int r = 0; r < 3; r++) D12[e][r] = ET(Dv[e][r]);
    }
#define HX_LS_B(K)                                                \
    {                                                             \
      ET E[3][3], D[3][3];                                        \
      tet_E12<K>(E12, E);                                         \
      tet_E12<K>(D12, D);                                         \
      if (tet_bound<ET, K>(E, D)) need |= 1u << K;              \
    }
    HX_LS_B(0) HX_LS_B(1) HX_LS_B(2) HX_LS_B(3) HX_LS_B(4) HX_LS_B(5) HX_LS_B(6) HX_LS_B(7)
#undef HX_LS_B
    eq[0] = S.M * (efast.value() + eslow);
  }
  {
    // record the tets that need the exact root (one reservation per warp)
    const int k = __popc(need);
    int total;
    const int off = warp_exclusive_sum(k, total);
    unsigned base = 0;
    if ((threadIdx.x & 31) == 0 && total > 0) base = atomicAdd(a.root_count, (unsigned)total);
    base = __shfl_sync(0xffffffffu, base, 0);
    int w = 0;
    for (int K = 0; K < 8; K++)
      if ((need >> K) & 1u) {
        a.root_list[base + off + w] = (uint32_t)(h * 8 + K);
        a.root_mesh[base + off + w] = sg.mesh;
        w++;
      }
  }
  __shared__ double smem[1][32];
  block_sum<1>(eq, smem);
  // plain store of the block's partial; k_ls_bound_finish reduces them per mesh
  if (threadIdx.x == 0) a.partials[blockIdx.x] = eq[0];
}

__device__ __forceinline__ double cand_alpha(const MeshScalars &S, int j) {
  return j > kHalvings - 1 ? 0.0 : ldexp(S.max_step, -j);
}

// Quality energy at the NC candidates j = round*NC .. round*NC + NC - 1 (E = E0 + alpha D).
// Persistent launch: a fixed grid walks the hex segments, so the rounds after the line search
// has accepted a step cost one scalar read per segment.  The one-candidate mixed pass runs 8
// blocks of 128 per SM (64 registers, ~230 B of spills): 0.253 -> 0.205 ms at 2.1M hexes.
template <typename ET, typename VT, int NC>
__global__ void __launch_bounds__(128, (sizeof(ET) == 4 && NC == 1) ? 8 : 1) k_ls_energy(KArgs a, int round, int64_t nseg) {
  __shared__ double smem[NC][32];
  if (*a.ls_active == 0) return;  // every mesh has accepted its step
  if (round == kRoundFromDevice) round = (int)*a.ls_round;
  for (int64_t sb = blockIdx.x; sb < nseg; sb += gridDim.x) {
    const Seg sg = a.hseg[sb];
    MeshScalars &S = a.sc[sg.mesh];
    if (S.ls_done) continue;
    const int64_t h = sg.begin + threadIdx.x;
    const MeshDesc md = a.mesh[sg.mesh];
    double acc[NC];
#pragma unroll
    for (int j = 0; j < NC; j++) acc[j] = 0;
    if (h < sg.end) {
      uint32_t hv[8];
      load_hex(a.hexv, h, hv);
      const int32_t gs = a.gslot[h];
      double al[NC];
#pragma unroll
      for (int j = 0; j < NC; j++) al[j] = cand_alpha(S, round * NC + j);
      ET E12[12][3], D12[NC == 1 ? 1 : 12][3];
      hex_edges_mode<ET>(a, hv, E12);
      {
        VT Dv[12][3];
        hex_edges_vec(reinterpret_cast<const VT *>(a.d), hv, Dv);
        // One candidate: fold the step into the edge frame, E + a D per edge.  A corner tet's
        // edges are these with a sign, and sg (E + a D) rounds exactly like sg E + a (sg D).
        const ET a0 = ET(al[0]);
#pragma unroll
        for (int e = 0; e < 12; e++)
#pragma unroll
          for (int r = 0; r < 3; r++) {
            if constexpr (NC == 1) E12[e][r] = E12[e][r] + a0 * ET(Dv[e][r]);
            else D12[e][r] = ET(Dv[e][r]);
          }
      }
      SumAcc<ET> efast[NC];
      double eslow[NC];
#pragma unroll
      for (int j = 0; j < NC; j++) eslow[j] = 0;
#define HX_LE(K)                                                             \
      if constexpr (NC == 1) {                                               \
        ET E[3][3];                                                          \
        tet_E12<K>(E12, E);                                                  \
        tet_energy_acc<ET, VT, K>(a, h, hv, gs, E, al[0], efast[0], eslow[0]); \
      } else {                                                               \
        ET E0[3][3], D[3][3];                                                \
        tet_E12<K>(E12, E0);                                                 \
        tet_E12<K>(D12, D);                                                  \
        _Pragma("unroll") for (int j = 0; j < NC; j++) {                     \
          ET E[3][3];                                                        \
          const ET aj = ET(al[j]);                                           \
          _Pragma("unroll") for (int r = 0; r < 3; r++)                      \
          _Pragma("unroll") for (int c = 0; c < 3; c++) E[r][c] = E0[r][c] + aj * D[r][c]; \
          tet_energy_acc<ET, VT, K>(a, h, hv, gs, E, al[j], efast[j], eslow[j]); \
        }                                                                    \
      }
      HX_LE(0) HX_LE(1) HX_LE(2) HX_LE(3) HX_LE(4) HX_LE(5) HX_LE(6) HX_LE(7)
#undef HX_LE
#pragma unroll
      for (int j = 0; j < NC; j++) acc[j] = S.M * (efast[j].value() + eslow[j]);
    }
    block_sum<NC>(acc, smem);
    if (publish_partials<NC>(acc, a.partials, sb, a.counters + sg.mesh, md.nhblk)) {
      double g[NC];
      gather_partials_sums<NC>(a.partials, md.hblk0, md.nhblk, NC, g, smem);
      if (threadIdx.x == 0)
        for (int j = 0; j < NC; j++) S.cand_eq[j] = g[j];
      if (threadIdx.x == 0) a.counters[sg.mesh] = 0;
    }
    __syncthreads();
  }
}

// Soft energy at the current X (round < 0) or at the candidates of `round`; its last block
// takes the line-search decision for the round (accept the first finite E <= E_old,
// line_search.cpp:26-47).  Terms as compute_soft_const_energy (slim_m.cpp:735-790).
template <typename VT>
__global__ void __launch_bounds__(256) k_ls_soft(KArgs a, int round) {
  const Seg sg = a.cseg[blockIdx.x];
  if (round == kRoundFromDevice) round = (int)*a.ls_round;
  if (round >= 0 && *a.ls_active == 0) return;  // every mesh has accepted its step
  MeshScalars &S = a.sc[sg.mesh];
  if (round >= 0 && S.ls_done) return;
  const int nc = round < 0 ? 1 : a.ls_cand;
  const int64_t i = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  const VT *d = reinterpret_cast<const VT *>(a.d);
  const VT *da = reinterpret_cast<const VT *>(a.da);
  double acc[kMaxCand];
#pragma unroll
  for (int j = 0; j < kMaxCand; j++) acc[j] = 0;
  if (i < sg.end) {
    const ConsItem it = cons_item(md, i);
    const int64_t e = it.e;
    if (it.kind == CK_GROUP) {
      const int64_t m0 = a.g_ptr[e], m1 = a.g_ptr[e + 1];
      const double c = S.lamda_G * glue_coef(m1 - m0);
      if (c != 0.0) {
#pragma unroll
        for (int j = 0; j < kMaxCand; j++) {
          if (j >= nc) break;
          const double al = round < 0 ? 0.0 : cand_alpha(S, round * nc + j);
          double mean[3] = {0, 0, 0};
          for (int64_t k = m0; k < m1; k++) {
            const int64_t v = a.g_vs[k];
            for (int q = 0; q < 3; q++) mean[q] += a.X[4 * v + q] + al * double(d[4 * v + q]);
          }
          for (int q = 0; q < 3; q++) mean[q] /= double(m1 - m0);
          double en = 0;
          for (int64_t k = m0; k < m1; k++) {
            const int64_t v = a.g_vs[k];
            for (int q = 0; q < 3; q++) {
              const double r = a.X[4 * v + q] + al * double(d[4 * v + q]) - mean[q];
              en += r * r;
            }
          }
          acc[j] += c * en;
        }
      }
    } else if (!(S.glue && it.kind <= CK_LINE)) {
      const int32_t lv = it.kind == CK_CORNER ? a.c_ids[e] : it.kind == CK_TANGENT ? a.t_ids[e]
                       : it.kind == CK_LINE ? a.l_ids[e] : a.b_ids[e];
      const int64_t v = md.v_off + lv;
      const double x0 = a.X[4 * v], x1 = a.X[4 * v + 1], x2 = a.X[4 * v + 2];
      const double d0 = double(d[4 * v]), d1 = double(d[4 * v + 1]), d2 = double(d[4 * v + 2]);
#pragma unroll
      for (int j = 0; j < kMaxCand; j++) {
        if (j >= nc) break;
        const double al = round < 0 ? 0.0 : cand_alpha(S, round * nc + j);
        const double y0 = x0 + al * d0, y1 = x1 + al * d1, y2 = x2 + al * d2;
        double en;
        if (it.kind == CK_CORNER || it.kind == CK_PROJ) {
          const double *cp = it.kind == CK_PROJ ? a.b_pos + 3 * e : a.c_pos + 3 * e;
          const double e0 = cp[0] - y0, e1 = cp[1] - y1, e2 = cp[2] - y2;
          en = (it.kind == CK_PROJ ? S.lamda_P : S.lamda_C) * (e0 * e0 + e1 * e1 + e2 * e2);
        } else if (it.kind == CK_TANGENT) {
          const double ad = a.t_nrm[3 * e] * y0 + a.t_nrm[3 * e + 1] * y1 + a.t_nrm[3 * e + 2] * y2 - a.t_dis[e];
          en = S.lamda_T * ad * ad;
        } else {
          const double al_ = double(da[e]);  // a_L = CG solution (curve unknowns start at 0)
          const double r0 = y0 - al_ * a.l_axis[3 * e] - a.l_orig[3 * e];
          const double r1 = y1 - al_ * a.l_axis[3 * e + 1] - a.l_orig[3 * e + 1];
          const double r2 = y2 - al_ * a.l_axis[3 * e + 2] - a.l_orig[3 * e + 2];
          en = S.lamda_L * (r0 * r0 + r1 * r1 + r2 * r2);
        }
        acc[j] += en;
      }
    }
  }
  __shared__ double smem[kMaxCand][32];
  // reduce only the live candidates (FP64 shuffles are slow on GB300); the sums are the same
  if (nc == 1) {
    double a1[1] = {acc[0]};
    block_sum<1>(a1, smem);
    acc[0] = a1[0];
  } else {
    block_sum<kMaxCand>(acc, smem);
  }
  if (publish_partials<kMaxCand>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.ncblk)) {
    double es[kMaxCand];
    if (nc == 1) {
      double g[1];
      gather_partials_sums<1>(a.partials, md.cblk0, md.ncblk, kMaxCand, g, smem);
      es[0] = g[0];
    } else {
      gather_partials_sums<kMaxCand>(a.partials, md.cblk0, md.ncblk, kMaxCand, es, smem);
    }
    if (threadIdx.x == 0) {
      if (round < 0) {
        S.old_es = es[0];
        S.old_e = S.old_eq + es[0];
      } else {
        for (int j = 0; j < nc; j++) {
          const int jj = round * nc + j;
          if (jj > kHalvings) break;
          const double e = S.cand_eq[j] + es[j];
          const bool bad = isnan(e) || isinf(e) || e > S.old_e;
          if (!bad) {
            S.ls_done = 1;
            atomicSub(a.ls_active, 1u);
            S.step = cand_alpha(S, jj);
            S.energy = e;
            S.eq = S.cand_eq[j];
            S.es = es[j];
            S.halvings = jj;
            break;
          }
        }
        if (!S.ls_done && (round + 1) * nc > kHalvings) {  // only NaN/Inf energies, even at step 0
          S.ls_done = 1; S.step = 0; S.energy = S.old_e; S.eq = S.old_eq; S.es = S.old_es;
          atomicSub(a.ls_active, 1u);
          S.halvings = kHalvings; S.status |= 1;
        }
      }
      a.counters[sg.mesh] = 0;
    }
  }
}

// X += step d; a_L = delta_a (a mesh whose adaptive loop has finished stays in place)
template <typename VT>
__global__ void __launch_bounds__(256) k_ls_apply(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  const MeshDesc md = a.mesh[sg.mesh];
  const MeshScalars &S = a.sc[sg.mesh];
  if (S.frozen) return;
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
  const ItemRef it = item_ref(md, i);
  if (!it.curve) {
    const VT *d = reinterpret_cast<const VT *>(a.d);
    const int64_t o = 4 * it.idx;
    const double st = S.step;
    double x[3];
#pragma unroll
    for (int c = 0; c < 3; c++) { x[c] = a.X[o + c] + st * double(d[o + c]); a.X[o + c] = x[c]; }
    store_split(a.X32, it.idx, x[0], x[1], x[2]);
  } else {
    const VT *da = reinterpret_cast<const VT *>(a.da);
    a.aL[it.idx] = double(da[it.idx]);
  }
  }
}



// One line-search energy pass over NC candidate steps.  Each (ET, VT, NC) is instantiated in a
// k_ls_energy_*.cu unit of its own, so the unrolled candidate loops compile in parallel.
// The persistent grid is the number of blocks resident at once (from this kernel's registers and
// the device's SM count, looked up once per block size), never more than the segments.
template <typename ET, typename VT, int NC>
void launch_ls_energy_nc(const KArgs &a, int round, int64_t hblk, cudaStream_t st) {
  static int grid_threads = 0, grid = 0;
  if (grid_threads != a.hthreads) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ls_energy<ET, VT, NC>, a.hthreads, 0) != cudaSuccess ||
        sms <= 0 || per_sm <= 0) {
      sms = 152; per_sm = 6;
    }
    grid = sms * per_sm;
    grid_threads = a.hthreads;
  }
  const int64_t g = hblk < grid ? hblk : grid;
  k_ls_energy<ET, VT, NC><<<(unsigned)g, a.hthreads, 0, st>>>(a, round, hblk);
}
#define HX_LS_ENERGY_INST(ET, VT, NC) \
  template void launch_ls_energy_nc<ET, VT, NC>(const KArgs &, int, int64_t, cudaStream_t);

}  // namespace hexopt
