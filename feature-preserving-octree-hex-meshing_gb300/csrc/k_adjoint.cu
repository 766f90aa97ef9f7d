// k_adjoint.cu -- forward / backward pair of the total optimisation energy
//   E(X) = sum_t M (|J_t|_F^2 + |J_t^-1|_F^2) + soft(X)        (compute_energy_total,
//          slim_m.cpp:716-790, symmetric Dirichlet branch :885-888)
// with the operator frozen at the last precompute (J_t = E_t(X) B_t, as within a SLIM iteration).
// The backward pass recomputes every corner Jacobian from X instead of storing it:
//   dE/dJ = 2 M (J - J^-T J^-1 J^-T),   dE/dE_t = dE/dJ B_t^T,
// scattered to the four tet vertices (vertex 0 gets minus the sum of the edge columns).
// Soft terms: corners 2 lc (x - c), tangent planes 2 lt (n.x - d) n, lines 2 ll (x - a u - o).
#include "hexopt_elem.cuh"

namespace hexopt {

template <typename ET, int K, bool BWD>
__device__ __forceinline__ double adj_tet(const KArgs &a, int64_t h, const uint32_t hv[8], int32_t gs, ET M,
                                          double F[8][3]) {
  double E[3][3];
  tet_edges<K>(a.Xa, hv, E);
  const ET *Sinv = reinterpret_cast<const ET *>(a.Sinv);
  const ET is = Sinv[tet_idx<1>(h, K, 0)];
  const double *B = gs >= 0 ? a.Bgen + ((int64_t)gs * 8 + K) * 9 : nullptr;
  ET J[3][3];
  if (gs < 0) cube_J<K>(E, is, J); else gen_J<K>(E, B, J);
  ET A[3][3];
  adj3(J, A);
  const ET d = det3(J);
  const ET e = frob2(J) + frob2(A) / (d * d);
  if (BWD) {
    // J^-1 = A / d;  J^-T J^-1 J^-T = A^T A A^T / d^3
    ET T1[3][3], Q[3][3];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) T1[i][j] = A[0][i] * A[0][j] + A[1][i] * A[1][j] + A[2][i] * A[2][j];  // A^T A
    const ET id3 = ET(1) / (d * d * d);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const ET t = T1[i][0] * A[j][0] + T1[i][1] * A[j][1] + T1[i][2] * A[j][2];  // (A^T A A^T)[i][j]
        Q[i][j] = ET(2) * M * (J[i][j] - t * id3);
      }
    if (gs < 0) cube_scatter<K>(Q, is, F); else gen_scatter<K>(Q, B, F);
  }
  return double(M) * double(e);
}

template <typename ET, bool BWD>
__global__ void __launch_bounds__(128) k_adj_elems(KArgs a) {
  const Seg sg = a.hseg[blockIdx.x];
  const int64_t h = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  MeshScalars &S = a.sc[sg.mesh];
  double acc[1] = {0};
  if (h < sg.end) {
    uint32_t hv[8];
    load_hex(a.hexv, h, hv);
    const int32_t gs = a.gslot[h];
    const ET M = ET(S.M);
    double F[8][3];
#pragma unroll
    for (int c = 0; c < 8; c++) F[c][0] = F[c][1] = F[c][2] = 0;
    acc[0] += adj_tet<ET, 0, BWD>(a, h, hv, gs, M, F);
    acc[0] += adj_tet<ET, 1, BWD>(a, h, hv, gs, M, F);
    acc[0] += adj_tet<ET, 2, BWD>(a, h, hv, gs, M, F);
    acc[0] += adj_tet<ET, 3, BWD>(a, h, hv, gs, M, F);
    acc[0] += adj_tet<ET, 4, BWD>(a, h, hv, gs, M, F);
    acc[0] += adj_tet<ET, 5, BWD>(a, h, hv, gs, M, F);
    acc[0] += adj_tet<ET, 6, BWD>(a, h, hv, gs, M, F);
    acc[0] += adj_tet<ET, 7, BWD>(a, h, hv, gs, M, F);
    if (BWD)
#pragma unroll
      for (int c = 0; c < 8; c++) atomic_add3(a.grad, hv[c], F[c][0], F[c][1], F[c][2]);
  }
  if (BWD) return;
  __shared__ double smem[1][32];
  block_sum<1>(acc, smem);
  if (publish_partials<1>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.nhblk)) {
    double e = gather_partials_sum(a.partials, md.hblk0, md.nhblk, 1, 0, smem);
    if (threadIdx.x == 0) {
      S.adj_eq = e;
      a.counters[sg.mesh] = 0;
    }
  }
}

template <bool BWD>
__global__ void __launch_bounds__(256) k_adj_soft(KArgs a) {
  const Seg sg = a.cseg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  const MeshDesc md = a.mesh[sg.mesh];
  MeshScalars &S = a.sc[sg.mesh];
  double acc[1] = {0};
  if (i < sg.end) {
    const ConsItem it = cons_item(md, i);
    const int64_t e = it.e;
    if (it.kind == CK_GROUP) {
      // lamda_G (n/(n-1))^2 sum_j |x_j - mean|^2; its gradient 2 c (x_j - mean) (the mean's own
      // derivative sums to zero over the group)
      const int64_t m0 = a.g_ptr[e], m1 = a.g_ptr[e + 1];
      const double c = S.lamda_G * glue_coef(m1 - m0);
      if (c != 0.0) {
        double mean[3] = {0, 0, 0};
        for (int64_t k = m0; k < m1; k++)
          for (int d = 0; d < 3; d++) mean[d] += a.Xa[4 * (int64_t)a.g_vs[k] + d];
        for (int d = 0; d < 3; d++) mean[d] /= double(m1 - m0);
        for (int64_t k = m0; k < m1; k++) {
          const int64_t v = a.g_vs[k];
          const double r0 = a.Xa[4 * v] - mean[0], r1 = a.Xa[4 * v + 1] - mean[1], r2 = a.Xa[4 * v + 2] - mean[2];
          acc[0] += c * (r0 * r0 + r1 * r1 + r2 * r2);
          if (BWD) atomic_add3(a.grad, (uint32_t)v, 2 * c * r0, 2 * c * r1, 2 * c * r2);
        }
      }
    } else if (!(S.glue && it.kind <= CK_LINE)) {
      if (it.kind == CK_CORNER || it.kind == CK_PROJ) {
        const bool pj = it.kind == CK_PROJ;
        const int64_t v = md.v_off + (pj ? a.b_ids[e] : a.c_ids[e]);
        const double *cp = pj ? a.b_pos + 3 * e : a.c_pos + 3 * e;
        const double lc = pj ? S.lamda_P : S.lamda_C;
        const double r0 = a.Xa[4 * v] - cp[0], r1 = a.Xa[4 * v + 1] - cp[1], r2 = a.Xa[4 * v + 2] - cp[2];
        acc[0] = lc * (r0 * r0 + r1 * r1 + r2 * r2);
        if (BWD) atomic_add3(a.grad, (uint32_t)v, 2 * lc * r0, 2 * lc * r1, 2 * lc * r2);
      } else if (it.kind == CK_TANGENT) {
        const int64_t v = md.v_off + a.t_ids[e];
        const double n0 = a.t_nrm[3 * e], n1 = a.t_nrm[3 * e + 1], n2 = a.t_nrm[3 * e + 2];
        const double ad = n0 * a.Xa[4 * v] + n1 * a.Xa[4 * v + 1] + n2 * a.Xa[4 * v + 2] - a.t_dis[e];
        acc[0] = S.lamda_T * ad * ad;
        const double g = 2 * S.lamda_T * ad;
        if (BWD) atomic_add3(a.grad, (uint32_t)v, g * n0, g * n1, g * n2);
      } else {
        const int64_t v = md.v_off + a.l_ids[e];
        const double al = a.aL[e];
        const double r0 = a.Xa[4 * v] - al * a.l_axis[3 * e] - a.l_orig[3 * e];
        const double r1 = a.Xa[4 * v + 1] - al * a.l_axis[3 * e + 1] - a.l_orig[3 * e + 1];
        const double r2 = a.Xa[4 * v + 2] - al * a.l_axis[3 * e + 2] - a.l_orig[3 * e + 2];
        acc[0] = S.lamda_L * (r0 * r0 + r1 * r1 + r2 * r2);
        if (BWD) atomic_add3(a.grad, (uint32_t)v, 2 * S.lamda_L * r0, 2 * S.lamda_L * r1, 2 * S.lamda_L * r2);
      }
    }
  }
  if (BWD) return;
  __shared__ double smem[1][32];
  block_sum<1>(acc, smem);
  if (publish_partials<1>(acc, a.partials, blockIdx.x, a.counters + sg.mesh, md.ncblk)) {
    double e = gather_partials_sum(a.partials, md.cblk0, md.ncblk, 1, 0, smem);
    if (threadIdx.x == 0) {
      S.adj_es = e;
      a.counters[sg.mesh] = 0;
    }
  }
}

template <typename ET>
void launch_energy_fwd(const KArgs &a, int64_t hblk, int64_t cblk, cudaStream_t st) {
  k_adj_elems<ET, false><<<(unsigned)hblk, a.hthreads, 0, st>>>(a);
  k_adj_soft<false><<<(unsigned)cblk, a.vthreads, 0, st>>>(a);
}
template <typename ET>
void launch_energy_bwd(const KArgs &a, int64_t hblk, int64_t cblk, cudaStream_t st) {
  k_adj_elems<ET, true><<<(unsigned)hblk, a.hthreads, 0, st>>>(a);
  k_adj_soft<true><<<(unsigned)cblk, a.vthreads, 0, st>>>(a);
}
template void launch_energy_fwd<double>(const KArgs &, int64_t, int64_t, cudaStream_t);
template void launch_energy_fwd<float>(const KArgs &, int64_t, int64_t, cudaStream_t);
template void launch_energy_bwd<double>(const KArgs &, int64_t, int64_t, cudaStream_t);
template void launch_energy_bwd<float>(const KArgs &, int64_t, int64_t, cudaStream_t);

}  // namespace hexopt
