// k_slim.cu -- SLIM local/global iteration on sm_103a, one thread per hex (8 corner tets).
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
// <double,double>; MIXED uses <float,float> with FP64 positions, FP64 residual, FP64 accumulation
// of every reduction, and FP64 for the step bound.
#include "hexopt_common.cuh"
#include "hexopt_kernels.h"
#include "hexopt_elem.cuh"

namespace hexopt {

// ------------------------------------------------------------------------------- precompute
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
    if (gs < 0) {                                                                              \
      const double d = det3(E);                                                                \
      degenerate |= (d == 0.0);                                                                \
      Sinv[tet_idx<1>(h, K, 0)] = ET(1.0 / cbrt(d));                                            \
    } else {                                                                                   \
      double A[3][3];                                                                          \
      adj3(E, A);                                                                              \
      const double d = det3(E);                                                                \
      degenerate |= (d == 0.0);                                                                \
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
template <typename ET, int K>
__device__ __forceinline__ void local_tet(const KArgs &a, int64_t h, const uint32_t hv[8], int32_t gs, ET M,
                                          ET exp_f, int energy, double F[8][3]) {
  double E[3][3];
  tet_edges<K>(a.X, hv, E);
  const ET *Sinv = reinterpret_cast<const ET *>(a.Sinv);
  const ET is = Sinv[tet_idx<1>(h, K, 0)];
  ET J[3][3];
  const double *B = gs >= 0 ? a.Bgen + ((int64_t)gs * 8 + K) * 9 : nullptr;
  if (gs < 0) cube_J<K>(E, is, J); else gen_J<K>(E, B, J);
  ET R[3][3], U[3][3], s[3], Vm[3][3], m[3];
  polar_svd3(J, R, U, s, Vm);
  slim_weights(energy, exp_f, s, U, Vm, m, R);
  // W = U diag(m) U^T is symmetric, so W^T W = U diag(m^2) U^T.
  ET c[6];
  const ET m0 = m[0] * m[0], m1 = m[1] * m[1], m2 = m[2] * m[2];
  c[0] = U[0][0] * U[0][0] * m0 + U[0][1] * U[0][1] * m1 + U[0][2] * U[0][2] * m2;
  c[1] = U[1][0] * U[1][0] * m0 + U[1][1] * U[1][1] * m1 + U[1][2] * U[1][2] * m2;
  c[2] = U[2][0] * U[2][0] * m0 + U[2][1] * U[2][1] * m1 + U[2][2] * U[2][2] * m2;
  c[3] = U[0][0] * U[1][0] * m0 + U[0][1] * U[1][1] * m1 + U[0][2] * U[1][2] * m2;
  c[4] = U[0][0] * U[2][0] * m0 + U[0][1] * U[2][1] * m1 + U[0][2] * U[2][2] * m2;
  c[5] = U[1][0] * U[2][0] * m0 + U[1][1] * U[2][1] * m1 + U[1][2] * U[2][2] * m2;
  // rhs stress M W^T W R
  ET Q[3][3];
  sym_mul(c, R, Q);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Q[i][j] *= M;
  ET *C = reinterpret_cast<ET *>(a.Ccoef);
  if (gs < 0) {
    const ET s2 = M * is * is;  // fold M / cbrt(6 vol)^2 into the stored coefficients
#pragma unroll
    for (int i = 0; i < 6; i++) C[tet_idx<6>(h, K, i)] = c[i] * s2;
    cube_scatter<K>(Q, is, F);
  } else {
#pragma unroll
    for (int i = 0; i < 6; i++) C[tet_idx<6>(h, K, i)] = c[i] * M;
    gen_scatter<K>(Q, B, F);
  }
}

template <typename ET>
__global__ void __launch_bounds__(128) k_local(KArgs a) {
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  if (h >= sg.end) return;
  const MeshScalars &S = a.sc[sg.mesh];
  const ET M = ET(S.M), exp_f = ET(S.exp_f);
  uint32_t hv[8];
  load_hex(a.hexv, h, hv);
  const int32_t gs = a.gslot[h];
  double F[8][3];
#pragma unroll
  for (int c = 0; c < 8; c++) F[c][0] = F[c][1] = F[c][2] = 0;
  local_tet<ET, 0>(a, h, hv, gs, M, exp_f, a.energy, F);
  local_tet<ET, 1>(a, h, hv, gs, M, exp_f, a.energy, F);
  local_tet<ET, 2>(a, h, hv, gs, M, exp_f, a.energy, F);
  local_tet<ET, 3>(a, h, hv, gs, M, exp_f, a.energy, F);
  local_tet<ET, 4>(a, h, hv, gs, M, exp_f, a.energy, F);
  local_tet<ET, 5>(a, h, hv, gs, M, exp_f, a.energy, F);
  local_tet<ET, 6>(a, h, hv, gs, M, exp_f, a.energy, F);
  local_tet<ET, 7>(a, h, hv, gs, M, exp_f, a.energy, F);
#pragma unroll
  for (int c = 0; c < 8; c++) atomic_add3(a.b, hv[c], F[c][0], F[c][1], F[c][2]);
}

// ------------------------------------------------------------------------------- SpMV
// out += K in for all element terms.  FROM_POS: `in` is the FP64 position array (initial
// residual); DIAG: also accumulate diag(K) into a.diag.
template <typename ET, typename OT, int K, bool FROM_POS, bool DIAG>
__device__ __forceinline__ void spmv_tet(const KArgs &a, const void *in, int64_t h, const uint32_t hv[8], int32_t gs,
                                         OT F[8][3], double Dg[8][3]) {
  ET J[3][3];
  const double *B = gs >= 0 ? a.Bgen + ((int64_t)gs * 8 + K) * 9 : nullptr;
  if (FROM_POS) {
    double E[3][3];
    tet_edges<K>(reinterpret_cast<const double *>(in), hv, E);
    if (gs < 0) cube_J<K>(E, ET(1), J); else gen_J<K>(E, B, J);
  } else {
    ET E[3][3];
    tet_edges_vec<K>(reinterpret_cast<const ET *>(in), hv, E);
    if (gs < 0) cube_J<K>(E, ET(1), J); else gen_J<K>(E, B, J);
  }
  const ET *C = reinterpret_cast<const ET *>(a.Ccoef);
  ET c[6];
#pragma unroll
  for (int i = 0; i < 6; i++) c[i] = C[tet_idx<6>(h, K, i)];
  ET Q[3][3];
  sym_mul(c, J, Q);
  if (gs < 0) cube_scatter<K>(Q, ET(1), F); else gen_scatter<K>(Q, B, F);
  if (DIAG) {
    // diag(K_t) at corner j, coordinate b: C[b][b] * |g_j|^2
    double w[4];
    if (gs < 0) {
      w[0] = 3; w[1] = w[2] = w[3] = 1;
    } else {
#pragma unroll
      for (int j = 0; j < 3; j++) w[j + 1] = B[j * 3] * B[j * 3] + B[j * 3 + 1] * B[j * 3 + 1] + B[j * 3 + 2] * B[j * 3 + 2];
      double g0[3];
#pragma unroll
      for (int r = 0; r < 3; r++) g0[r] = B[r] + B[3 + r] + B[6 + r];
      w[0] = g0[0] * g0[0] + g0[1] * g0[1] + g0[2] * g0[2];
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int cc = tet_v(K, j);
      Dg[cc][0] += w[j] * double(c[0]); Dg[cc][1] += w[j] * double(c[1]); Dg[cc][2] += w[j] * double(c[2]);
    }
  }
}

template <typename ET, typename OT, bool FROM_POS, bool DIAG>
__global__ void __launch_bounds__(128) k_spmv(KArgs a, const void *in, OT *out) {
  const Seg sg = a.hseg[blockIdx.x];
  if (!FROM_POS && a.sc[sg.mesh].cg_done) return;
  const int64_t h = sg.begin + threadIdx.x;
  if (h >= sg.end) return;
  uint32_t hv[8];
  load_hex(a.hexv, h, hv);
  const int32_t gs = a.gslot[h];
  OT F[8][3];
  double Dg[DIAG ? 8 : 1][3];
#pragma unroll
  for (int c = 0; c < 8; c++) F[c][0] = F[c][1] = F[c][2] = 0;
  if (DIAG)
#pragma unroll
    for (int c = 0; c < (DIAG ? 8 : 1); c++) Dg[c][0] = Dg[c][1] = Dg[c][2] = 0;
  spmv_tet<ET, OT, 0, FROM_POS, DIAG>(a, in, h, hv, gs, F, (double(*)[3])Dg);
  spmv_tet<ET, OT, 1, FROM_POS, DIAG>(a, in, h, hv, gs, F, (double(*)[3])Dg);
  spmv_tet<ET, OT, 2, FROM_POS, DIAG>(a, in, h, hv, gs, F, (double(*)[3])Dg);
  spmv_tet<ET, OT, 3, FROM_POS, DIAG>(a, in, h, hv, gs, F, (double(*)[3])Dg);
  spmv_tet<ET, OT, 4, FROM_POS, DIAG>(a, in, h, hv, gs, F, (double(*)[3])Dg);
  spmv_tet<ET, OT, 5, FROM_POS, DIAG>(a, in, h, hv, gs, F, (double(*)[3])Dg);
  spmv_tet<ET, OT, 6, FROM_POS, DIAG>(a, in, h, hv, gs, F, (double(*)[3])Dg);
  spmv_tet<ET, OT, 7, FROM_POS, DIAG>(a, in, h, hv, gs, F, (double(*)[3])Dg);
#pragma unroll
  for (int c = 0; c < 8; c++) atomic_add3(out, hv[c], F[c][0], F[c][1], F[c][2]);
  if (DIAG)
#pragma unroll
    for (int c = 0; c < (DIAG ? 8 : 1); c++) atomic_add3(a.diag, hv[c], Dg[c][0], Dg[c][1], Dg[c][2]);
}

// ------------------------------------------------------------------------------- soft terms
// Constraint items of a mesh: [0, nc) corners, [nc, nc+nt) tangent planes, [nc+nt, +nl) lines.
// mode 0: rhs and diagonal (add_soft_constraints)
template <typename VT>
__global__ void __launch_bounds__(256) k_soft_rhs(KArgs a) {
  const Seg sg = a.cseg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const MeshScalars &S = a.sc[sg.mesh];
  int64_t li = i - md.c_off - md.t_off - md.l_off;  // items of a mesh start at c_off+t_off+l_off
  if (li < md.nc) {
    const int64_t e = md.c_off + li;
    const uint32_t v = (uint32_t)(md.v_off + a.c_ids[e]);
    const double lc = S.lamda_C;
    atomic_add3(a.b, v, lc * a.c_pos[3 * e], lc * a.c_pos[3 * e + 1], lc * a.c_pos[3 * e + 2]);
    atomic_add3(a.diag, v, lc, lc, lc);
    return;
  }
  li -= md.nc;
  if (li < md.nt) {
    const int64_t e = md.t_off + li;
    const uint32_t v = (uint32_t)(md.v_off + a.t_ids[e]);
    const double lt = S.lamda_T;
    const double n0 = a.t_nrm[3 * e], n1 = a.t_nrm[3 * e + 1], n2 = a.t_nrm[3 * e + 2], d = a.t_dis[e];
    atomic_add3(a.b, v, lt * n0 * d, lt * n1 * d, lt * n2 * d);
    atomic_add3(a.diag, v, lt * n0 * n0, lt * n1 * n1, lt * n2 * n2);
    return;
  }
  li -= md.nt;
  {
    const int64_t e = md.l_off + li;
    const uint32_t v = (uint32_t)(md.v_off + a.l_ids[e]);
    const double ll = S.lamda_L;
    const double x0 = a.l_axis[3 * e], x1 = a.l_axis[3 * e + 1], x2 = a.l_axis[3 * e + 2];
    const double o0 = a.l_orig[3 * e], o1 = a.l_orig[3 * e + 1], o2 = a.l_orig[3 * e + 2];
    atomic_add3(a.b, v, ll * o0, ll * o1, ll * o2);
    atomic_add3(a.diag, v, ll, ll, ll);
    a.ba[e] = ll * (-x0 * o0 - x1 * o1 - x2 * o2);
    a.diaga[e] = ll * (x0 * x0 + x1 * x1 + x2 * x2);
  }
}

// out += S in  for the soft-constraint block of L (FP64 accumulation when OT = double).
template <typename IT, typename OT, bool FROM_POS>
__global__ void __launch_bounds__(256) k_soft_mv(KArgs a, const IT *in, const IT *in_a, OT *out, OT *out_a) {
  const Seg sg = a.cseg[blockIdx.x];
  if (!FROM_POS && a.sc[sg.mesh].cg_done) return;
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const MeshScalars &S = a.sc[sg.mesh];
  int64_t li = i - md.c_off - md.t_off - md.l_off;
  if (li < md.nc) {
    const uint32_t v = (uint32_t)(md.v_off + a.c_ids[md.c_off + li]);
    const double lc = S.lamda_C;
    const IT *p = in + 4 * (int64_t)v;
    atomic_add3(out, v, OT(lc * p[0]), OT(lc * p[1]), OT(lc * p[2]));
    return;
  }
  li -= md.nc;
  if (li < md.nt) {
    const int64_t e = md.t_off + li;
    const uint32_t v = (uint32_t)(md.v_off + a.t_ids[e]);
    const double n0 = a.t_nrm[3 * e], n1 = a.t_nrm[3 * e + 1], n2 = a.t_nrm[3 * e + 2];
    const IT *p = in + 4 * (int64_t)v;
    const double s = S.lamda_T * (n0 * double(p[0]) + n1 * double(p[1]) + n2 * double(p[2]));
    atomic_add3(out, v, OT(s * n0), OT(s * n1), OT(s * n2));
    return;
  }
  li -= md.nt;
  {
    const int64_t e = md.l_off + li;
    const uint32_t v = (uint32_t)(md.v_off + a.l_ids[e]);
    const double ll = S.lamda_L;
    const double x0 = a.l_axis[3 * e], x1 = a.l_axis[3 * e + 1], x2 = a.l_axis[3 * e + 2];
    const IT *p = in + 4 * (int64_t)v;
    const double pa = FROM_POS ? 0.0 : double(in_a[e]);  // curve unknowns start at 0
    atomic_add3(out, v, OT(ll * (double(p[0]) - x0 * pa)), OT(ll * (double(p[1]) - x1 * pa)),
                OT(ll * (double(p[2]) - x2 * pa)));
    out_a[e] += OT(ll * (-(x0 * double(p[0]) + x1 * double(p[1]) + x2 * double(p[2])) + (x0 * x0 + x1 * x1 + x2 * x2) * pa));
  }
}

// ------------------------------------------------------------------------------- CG vectors
// Unknown items of a mesh: [0, nv) vertices (3 coordinates), [nv, nv + nl) curve unknowns.
struct ItemRef {
  bool curve;
  int64_t idx;  // global vertex id or global curve entry
};
__device__ __forceinline__ ItemRef item_ref(const MeshDesc &md, int64_t i) {
  // vertex-kind item ids: v_off + l_off + local, so each mesh's block covers nv + nl items
  const int64_t li = i - md.v_off - md.l_off;
  if (li < md.nv) return {false, md.v_off + li};
  return {true, md.l_off + (li - md.nv)};
}

// r = b - A x0 (the element and soft parts were accumulated into q64), p = invd r, delta = 0
template <typename VT>
__global__ void __launch_bounds__(256) k_cg_start(KArgs a, const double *q64, const double *q64a) {
  const Seg sg = a.vseg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  MeshScalars &S = a.sc[sg.mesh];
  const double prox = S.prox;
  double acc[3] = {0, 0, 0};  // rhs_norm2, rn2, r.p
  VT *r = reinterpret_cast<VT *>(a.r), *p = reinterpret_cast<VT *>(a.p), *d = reinterpret_cast<VT *>(a.d);
  VT *q = reinterpret_cast<VT *>(a.q), *invd = reinterpret_cast<VT *>(a.invd);
  VT *ra = reinterpret_cast<VT *>(a.ra), *pa = reinterpret_cast<VT *>(a.pa), *da = reinterpret_cast<VT *>(a.da);
  VT *qa = reinterpret_cast<VT *>(a.qa), *invda = reinterpret_cast<VT *>(a.invda);
  if (i < sg.end) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      const int64_t o = 4 * it.idx;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double x0 = a.X[o + c];
        const double bb = a.b[o + c];             // A^T M f + soft rhs (no proximal part)
        const double bfull = bb + prox * x0;      // rhs of the reference system
        const double rr = bb - q64[o + c];         // b - A x0 (proximal parts cancel)
        const double id = 1.0 / (a.diag[o + c] + prox);
        const double pp = id * rr;
        r[o + c] = VT(rr); p[o + c] = VT(pp); d[o + c] = VT(0); invd[o + c] = VT(id);
        q[o + c] = VT(prox * pp);                  // q = prox p: first SpMV accumulates on top
        acc[0] += bfull * bfull; acc[1] += rr * rr; acc[2] += rr * pp;
      }
    } else {
      const int64_t e = it.idx;
      const double bb = a.ba[e];
      const double rr = bb - q64a[e];
      const double dg = a.diaga[e];
      const double id = dg != 0.0 ? 1.0 / dg : 0.0;  // DiagonalPreconditioner: 0 if no diagonal
      const double pp = id * rr;
      ra[e] = VT(rr); pa[e] = VT(pp); da[e] = VT(0); invda[e] = VT(id); qa[e] = VT(0);
      acc[0] += bb * bb; acc[1] += rr * rr; acc[2] += rr * pp;
    }
  }
  __shared__ double smem[3][32];
  block_sum<3>(acc, smem);
  const MeshDesc &mdr = md;
  if (publish_partials<3>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, mdr.nvblk)) {
    double v0 = gather_partials_sum(a.partials, mdr.vblk0, mdr.nvblk, 3, 0, smem);
    double v1 = gather_partials_sum(a.partials, mdr.vblk0, mdr.nvblk, 3, 1, smem);
    double v2 = gather_partials_sum(a.partials, mdr.vblk0, mdr.nvblk, 3, 2, smem);
    if (threadIdx.x == 0) {
      S.rhs_norm2 = v0;
      S.threshold = a.cg_tol * a.cg_tol * v0;
      S.rn2 = v1;
      S.abs_new = v2;
      S.cg_iters = 0;
      S.cg_done = 0;
      if (v0 == 0.0) { S.cg_done = 1; S.cg_error = 0; }
      else if (v1 < S.threshold) { S.cg_done = 1; S.cg_error = sqrt(v1 / v0); }
      a.counters[sg.mesh] = 0;
    }
  }
}

// alpha = abs_new / (p . q)
template <typename VT>
__global__ void __launch_bounds__(256) k_cg_alpha(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  MeshScalars &S = a.sc[sg.mesh];
  if (S.cg_done) return;
  const int64_t i = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  const VT *p = reinterpret_cast<const VT *>(a.p), *q = reinterpret_cast<const VT *>(a.q);
  const VT *pa = reinterpret_cast<const VT *>(a.pa), *qa = reinterpret_cast<const VT *>(a.qa);
  double acc[1] = {0};
  if (i < sg.end) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      const int64_t o = 4 * it.idx;
      acc[0] = double(p[o]) * double(q[o]) + double(p[o + 1]) * double(q[o + 1]) + double(p[o + 2]) * double(q[o + 2]);
    } else {
      acc[0] = double(pa[it.idx]) * double(qa[it.idx]);
    }
  }
  __shared__ double smem[1][32];
  block_sum<1>(acc, smem);
  if (publish_partials<1>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nvblk)) {
    double pAp = gather_partials_sum(a.partials, md.vblk0, md.nvblk, 1, 0, smem);
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
  const int64_t i = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  const VT alpha = VT(S.alpha);
  VT *r = reinterpret_cast<VT *>(a.r), *d = reinterpret_cast<VT *>(a.d);
  const VT *p = reinterpret_cast<const VT *>(a.p), *q = reinterpret_cast<const VT *>(a.q);
  const VT *invd = reinterpret_cast<const VT *>(a.invd);
  VT *ra = reinterpret_cast<VT *>(a.ra), *da = reinterpret_cast<VT *>(a.da);
  const VT *pa = reinterpret_cast<const VT *>(a.pa), *qa = reinterpret_cast<const VT *>(a.qa);
  const VT *invda = reinterpret_cast<const VT *>(a.invda);
  double acc[2] = {0, 0};
  if (i < sg.end) {
    const ItemRef it = item_ref(md, i);
    if (!it.curve) {
      const int64_t o = 4 * it.idx;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        d[o + c] += alpha * p[o + c];
        const VT rr = r[o + c] - alpha * q[o + c];
        r[o + c] = rr;
        acc[0] += double(rr) * double(rr);
        acc[1] += double(rr) * double(invd[o + c] * rr);
      }
    } else {
      const int64_t e = it.idx;
      da[e] += alpha * pa[e];
      const VT rr = ra[e] - alpha * qa[e];
      ra[e] = rr;
      acc[0] += double(rr) * double(rr);
      acc[1] += double(rr) * double(invda[e] * rr);
    }
  }
  __shared__ double smem[2][32];
  block_sum<2>(acc, smem);
  if (publish_partials<2>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nvblk)) {
    double rn2 = gather_partials_sum(a.partials, md.vblk0, md.nvblk, 2, 0, smem);
    double rz = gather_partials_sum(a.partials, md.vblk0, md.nvblk, 2, 1, smem);
    if (threadIdx.x == 0) {
      S.rn2 = rn2;
      S.cg_error = sqrt(rn2 / S.rhs_norm2);
      if (rn2 < S.threshold) {
        S.cg_done = 1;
      } else {
        S.beta = rz / S.abs_new;
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
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const VT beta = VT(S.beta), prox = VT(S.prox);
  const VT *r = reinterpret_cast<const VT *>(a.r), *invd = reinterpret_cast<const VT *>(a.invd);
  VT *p = reinterpret_cast<VT *>(a.p), *q = reinterpret_cast<VT *>(a.q);
  const ItemRef it = item_ref(md, i);
  if (!it.curve) {
    const int64_t o = 4 * it.idx;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const VT pp = invd[o + c] * r[o + c] + beta * p[o + c];
      p[o + c] = pp;
      q[o + c] = prox * pp;
    }
  } else {
    const VT *ra = reinterpret_cast<const VT *>(a.ra), *invda = reinterpret_cast<const VT *>(a.invda);
    VT *pa = reinterpret_cast<VT *>(a.pa), *qa = reinterpret_cast<VT *>(a.qa);
    const int64_t e = it.idx;
    pa[e] = invda[e] * ra[e] + beta * pa[e];
    qa[e] = VT(0);
  }
}

// ------------------------------------------------------------------------------- line search
// Smallest positive root of det(E + t D) = 0 (get_min_pos_root_3D, flip_avoiding_line_search.cpp:
// 177-271), FP64.  The cubic is solved by the trigonometric / Cardano method of SolveP3 (:24-61).
__device__ double smallest_pos_quad_zero(double a, double b, double c) {
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

__device__ double min_pos_root(const double E[3][3], const double D[3][3]) {
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

// Energy density of corner tet K at positions X + alpha d.  The edges are formed in FP64 and the
// density evaluated in ET; tets with |det J| below a threshold are re-evaluated in FP64.
template <typename ET, typename VT, int K>
__device__ __forceinline__ double tet_energy_at(const KArgs &a, int64_t h, const uint32_t hv[8], int32_t gs,
                                                const double E0[3][3], const double Dd[3][3], double alpha) {
  const ET *Sinv = reinterpret_cast<const ET *>(a.Sinv);
  double E[3][3];
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) E[r][c] = E0[r][c] + alpha * Dd[r][c];
  const double *B = gs >= 0 ? a.Bgen + ((int64_t)gs * 8 + K) * 9 : nullptr;
  ET J[3][3];
  const ET is = Sinv[tet_idx<1>(h, K, 0)];
  if (gs < 0) cube_J<K>(E, is, J); else gen_J<K>(E, B, J);
  ET e = tet_energy_density<ET>(a.energy, ET(a.sc_exp_f), J);
  if (sizeof(ET) == 4) {
    const ET d = det3(J);
    if (!(fabs(d) > ET(1e-3))) {  // near-degenerate: FP64 re-evaluation
      double Jd[3][3];
      if (gs < 0) cube_J<K>(E, double(is), Jd); else gen_J<K>(E, B, Jd);
      return tet_energy_density<double>(a.energy, a.sc_exp_f, Jd);
    }
  }
  return double(e);
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

// Pass 1: min positive root over tets (step bound) and the quality energy at the current X.
template <typename ET, typename VT>
__global__ void __launch_bounds__(128) k_ls_bound(KArgs a) {
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  MeshScalars &S = a.sc[sg.mesh];
  double mn[1] = {INFINITY}, eq[1] = {0};
  if (h < sg.end) {
    uint32_t hv[8];
    load_hex(a.hexv, h, hv);
    const int32_t gs = a.gslot[h];
    const VT *d = reinterpret_cast<const VT *>(a.d);
    double esum = 0;
#define HX_LS(K)                                                   \
    {                                                              \
      double E[3][3], Dd[3][3];                                    \
      tet_edges<K>(a.X, hv, E);                                    \
      tet_dir<VT, K>(d, hv, Dd);                                   \
      mn[0] = fmin(mn[0], min_pos_root(E, Dd));                    \
      esum += tet_energy_at<ET, VT, K>(a, h, hv, gs, E, Dd, 0.0);  \
    }
    HX_LS(0) HX_LS(1) HX_LS(2) HX_LS(3) HX_LS(4) HX_LS(5) HX_LS(6) HX_LS(7)
#undef HX_LS
    eq[0] = S.M * esum;
  }
  __shared__ double smem[1][32];
  block_min<1>(mn, smem);
  double acc[2] = {0, 0};
  if (threadIdx.x == 0) acc[0] = mn[0];
  block_sum<1>(eq, smem);
  if (threadIdx.x == 0) acc[1] = eq[0];
  if (publish_partials<2>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nhblk)) {
    double m = gather_partials_min(a.partials, md.hblk0, md.nhblk, 2, 0, smem);
    double e = gather_partials_sum(a.partials, md.hblk0, md.nhblk, 2, 1, smem);
    if (threadIdx.x == 0) {
      S.min_root = m;
      S.max_step = fmin(1.0, m * 0.8);
      S.old_eq = e;
      S.ls_done = 0;
      a.counters[sg.mesh] = 0;
    }
  }
}

__device__ __forceinline__ double cand_alpha(const MeshScalars &S, int j) {
  return j > kHalvings - 1 ? 0.0 : ldexp(S.max_step, -j);
}

// Quality energy at the candidates j = round*nc .. round*nc + nc - 1.
template <typename ET, typename VT>
__global__ void __launch_bounds__(128) k_ls_energy(KArgs a, int round) {
  const Seg sg = a.hseg[blockIdx.x];
  MeshScalars &S = a.sc[sg.mesh];
  if (S.ls_done) return;
  const int nc = a.ls_cand;
  const int64_t h = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  double acc[kMaxCand];
#pragma unroll
  for (int j = 0; j < kMaxCand; j++) acc[j] = 0;
  if (h < sg.end) {
    uint32_t hv[8];
    load_hex(a.hexv, h, hv);
    const int32_t gs = a.gslot[h];
    const VT *d = reinterpret_cast<const VT *>(a.d);
#define HX_LE(K)                                                            \
    {                                                                       \
      double E[3][3], Dd[3][3];                                             \
      tet_edges<K>(a.X, hv, E);                                             \
      tet_dir<VT, K>(d, hv, Dd);                                            \
      for (int j = 0; j < nc; j++) {                                        \
        const double al = cand_alpha(S, round * nc + j);                    \
        acc[j] += tet_energy_at<ET, VT, K>(a, h, hv, gs, E, Dd, al);        \
      }                                                                     \
    }
    HX_LE(0) HX_LE(1) HX_LE(2) HX_LE(3) HX_LE(4) HX_LE(5) HX_LE(6) HX_LE(7)
#undef HX_LE
#pragma unroll
    for (int j = 0; j < kMaxCand; j++) acc[j] *= S.M;
  }
  __shared__ double smem[kMaxCand][32];
  block_sum<kMaxCand>(acc, smem);
  if (publish_partials<kMaxCand>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nhblk)) {
    for (int j = 0; j < nc; j++) {
      double e = gather_partials_sum(a.partials, md.hblk0, md.nhblk, kMaxCand, j, smem);
      if (threadIdx.x == 0) S.cand_eq[j] = e;
    }
    if (threadIdx.x == 0) a.counters[sg.mesh] = 0;
  }
}

// Soft energy at the current X (round < 0) or at the candidates of `round`; its last block
// takes the line-search decision for the round (accept the first finite E <= E_old).
template <typename VT>
__global__ void __launch_bounds__(256) k_ls_soft(KArgs a, int round) {
  const Seg sg = a.cseg[blockIdx.x];
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
    int64_t li = i - md.c_off - md.t_off - md.l_off;
    int kind = 0;
    int64_t e;
    if (li < md.nc) { e = md.c_off + li; }
    else if ((li -= md.nc) < md.nt) { kind = 1; e = md.t_off + li; }
    else { li -= md.nt; kind = 2; e = md.l_off + li; }
    const int32_t lv = kind == 0 ? a.c_ids[e] : kind == 1 ? a.t_ids[e] : a.l_ids[e];
    const int64_t v = md.v_off + lv;
    const double x0 = a.X[4 * v], x1 = a.X[4 * v + 1], x2 = a.X[4 * v + 2];
    const double d0 = double(d[4 * v]), d1 = double(d[4 * v + 1]), d2 = double(d[4 * v + 2]);
    for (int j = 0; j < nc; j++) {
      const double al = round < 0 ? 0.0 : cand_alpha(S, round * nc + j);
      const double y0 = x0 + al * d0, y1 = x1 + al * d1, y2 = x2 + al * d2;
      double en;
      if (kind == 0) {
        const double e0 = a.c_pos[3 * e] - y0, e1 = a.c_pos[3 * e + 1] - y1, e2 = a.c_pos[3 * e + 2] - y2;
        en = S.lamda_C * (e0 * e0 + e1 * e1 + e2 * e2);
      } else if (kind == 1) {
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
  __shared__ double smem[kMaxCand][32];
  block_sum<kMaxCand>(acc, smem);
  if (publish_partials<kMaxCand>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.ncblk)) {
    double es[kMaxCand];
    for (int j = 0; j < nc; j++) es[j] = gather_partials_sum(a.partials, md.cblk0, md.ncblk, kMaxCand, j, smem);
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
            S.step = cand_alpha(S, jj);
            S.energy = e;
            S.eq = S.cand_eq[j];
            S.es = es[j];
            S.halvings = jj;
            break;
          }
        }
        if (!S.ls_done && (round + 1) * nc > kHalvings) {  // unreachable: step 0 is always accepted
          S.ls_done = 1; S.step = 0; S.energy = S.old_e; S.eq = S.old_eq; S.es = S.old_es;
          S.halvings = kHalvings; S.status |= 1;
        }
      }
      a.counters[sg.mesh] = 0;
    }
  }
}

// X += step d; a_L = delta_a
template <typename VT>
__global__ void __launch_bounds__(256) k_ls_apply(KArgs a) {
  const Seg sg = a.vseg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = a.mesh[sg.mesh];
  const MeshScalars &S = a.sc[sg.mesh];
  const ItemRef it = item_ref(md, i);
  if (!it.curve) {
    const VT *d = reinterpret_cast<const VT *>(a.d);
    const int64_t o = 4 * it.idx;
    const double st = S.step;
#pragma unroll
    for (int c = 0; c < 3; c++) a.X[o + c] = a.X[o + c] + st * double(d[o + c]);
  } else {
    const VT *da = reinterpret_cast<const VT *>(a.da);
    a.aL[it.idx] = double(da[it.idx]);
  }
}

// ------------------------------------------------------------------------------- launchers
#define HX_GRID(n) dim3((unsigned)(n))

template <typename ET, typename VT>
void launch_precompute(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_precompute<ET><<<HX_GRID(nblk), a.hthreads, 0, st>>>(a);
}
template <typename ET, typename VT>
void launch_local(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_local<ET><<<HX_GRID(nblk), a.hthreads, 0, st>>>(a);
}
template <typename ET, typename VT>
void launch_residual_elems(const KArgs &a, int64_t nblk, double *q64, cudaStream_t st) {
  k_spmv<ET, double, true, true><<<HX_GRID(nblk), a.hthreads, 0, st>>>(a, a.X, q64);
}
template <typename ET, typename VT>
void launch_spmv_elems(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_spmv<ET, VT, false, false><<<HX_GRID(nblk), a.hthreads, 0, st>>>(a, a.p, reinterpret_cast<VT *>(a.q));
}
template <typename VT>
void launch_soft_rhs(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_soft_rhs<VT><<<HX_GRID(nblk), a.vthreads, 0, st>>>(a);
}
template <typename VT>
void launch_soft_residual(const KArgs &a, int64_t nblk, double *q64, double *q64a, cudaStream_t st) {
  k_soft_mv<double, double, true><<<HX_GRID(nblk), a.vthreads, 0, st>>>(a, a.X, nullptr, q64, q64a);
}
template <typename VT>
void launch_soft_spmv(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_soft_mv<VT, VT, false><<<HX_GRID(nblk), a.vthreads, 0, st>>>(a, reinterpret_cast<const VT *>(a.p),
                                                          reinterpret_cast<const VT *>(a.pa),
                                                          reinterpret_cast<VT *>(a.q), reinterpret_cast<VT *>(a.qa));
}
template <typename VT>
void launch_cg_start(const KArgs &a, int64_t nblk, const double *q64, const double *q64a, cudaStream_t st) {
  k_cg_start<VT><<<HX_GRID(nblk), a.vthreads, 0, st>>>(a, q64, q64a);
}
template <typename VT>
void launch_cg_iter(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, cudaStream_t st) {
  launch_spmv_elems<VT, VT>(a, hblk, st);
  launch_soft_spmv<VT>(a, cblk, st);
  k_cg_alpha<VT><<<HX_GRID(vblk), a.vthreads, 0, st>>>(a);
  k_cg_update<VT><<<HX_GRID(vblk), a.vthreads, 0, st>>>(a);
  k_cg_dir<VT><<<HX_GRID(vblk), a.vthreads, 0, st>>>(a);
}
template <typename ET, typename VT>
void launch_line_search(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, cudaStream_t st) {
  k_ls_bound<ET, VT><<<HX_GRID(hblk), a.hthreads, 0, st>>>(a);
  k_ls_soft<VT><<<HX_GRID(cblk), a.vthreads, 0, st>>>(a, -1);
  const int rounds = (kHalvings + 1 + a.ls_cand - 1) / a.ls_cand;
  for (int r = 0; r < rounds; r++) {
    k_ls_energy<ET, VT><<<HX_GRID(hblk), a.hthreads, 0, st>>>(a, r);
    k_ls_soft<VT><<<HX_GRID(cblk), a.vthreads, 0, st>>>(a, r);
  }
  k_ls_apply<VT><<<HX_GRID(vblk), a.vthreads, 0, st>>>(a);
}

// explicit instantiations for the two modes
#define HX_INST(ET, VT)                                                                          \
  template void launch_precompute<ET, VT>(const KArgs &, int64_t, cudaStream_t);                 \
  template void launch_local<ET, VT>(const KArgs &, int64_t, cudaStream_t);                      \
  template void launch_residual_elems<ET, VT>(const KArgs &, int64_t, double *, cudaStream_t);   \
  template void launch_spmv_elems<ET, VT>(const KArgs &, int64_t, cudaStream_t);                 \
  template void launch_soft_rhs<VT>(const KArgs &, int64_t, cudaStream_t);                       \
  template void launch_soft_residual<VT>(const KArgs &, int64_t, double *, double *, cudaStream_t); \
  template void launch_soft_spmv<VT>(const KArgs &, int64_t, cudaStream_t);                      \
  template void launch_cg_start<VT>(const KArgs &, int64_t, const double *, const double *, cudaStream_t); \
  template void launch_cg_iter<VT>(const KArgs &, int64_t, int64_t, int64_t, cudaStream_t);      \
  template void launch_line_search<ET, VT>(const KArgs &, int64_t, int64_t, int64_t, cudaStream_t);
HX_INST(double, double)
HX_INST(float, float)
#undef HX_INST

}  // namespace hexopt
