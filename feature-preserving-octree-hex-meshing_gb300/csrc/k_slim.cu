// k_slim.cu -- launchers of the SLIM local/global iteration (kernels in k_slim.cuh).
//
// Stages (slim_m.cpp:1269-1288, one iteration of slim_solve2's fixed-N branch): precompute, local
// step, matrix-free PCG, flip-avoiding line search.  The line-search energy passes are compiled in
// the k_ls_energy_*.cu units; this unit only declares them.
#include "k_slim.cuh"

namespace hexopt {

#define HX_LS_ENERGY_EXTERN(ET, VT)                                                                 \
  extern template void launch_ls_energy_nc<ET, VT, 1>(const KArgs &, int, int64_t, cudaStream_t);   \
  extern template void launch_ls_energy_nc<ET, VT, 2>(const KArgs &, int, int64_t, cudaStream_t);   \
  extern template void launch_ls_energy_nc<ET, VT, 3>(const KArgs &, int, int64_t, cudaStream_t);   \
  extern template void launch_ls_energy_nc<ET, VT, 4>(const KArgs &, int, int64_t, cudaStream_t);   \
  extern template void launch_ls_energy_nc<ET, VT, 5>(const KArgs &, int, int64_t, cudaStream_t);   \
  extern template void launch_ls_energy_nc<ET, VT, 6>(const KArgs &, int, int64_t, cudaStream_t);   \
  extern template void launch_ls_energy_nc<ET, VT, 7>(const KArgs &, int, int64_t, cudaStream_t);   \
  extern template void launch_ls_energy_nc<ET, VT, 8>(const KArgs &, int, int64_t, cudaStream_t);
HX_LS_ENERGY_EXTERN(double, double)
HX_LS_ENERGY_EXTERN(float, float)
#undef HX_LS_ENERGY_EXTERN
// One candidate-energy pass alone (timing): the pass of round 0.
template <typename ET, typename VT>
void launch_ls_energy_pass(const KArgs &a, int64_t hblk, cudaStream_t st) {
  switch (a.ls_cand) {
    case 1: launch_ls_energy_nc<ET, VT, 1>(a, 0, hblk, st); break;
    case 2: launch_ls_energy_nc<ET, VT, 2>(a, 0, hblk, st); break;
    case 3: launch_ls_energy_nc<ET, VT, 3>(a, 0, hblk, st); break;
    case 4: launch_ls_energy_nc<ET, VT, 4>(a, 0, hblk, st); break;
    case 5: launch_ls_energy_nc<ET, VT, 5>(a, 0, hblk, st); break;
    case 6: launch_ls_energy_nc<ET, VT, 6>(a, 0, hblk, st); break;
    case 7: launch_ls_energy_nc<ET, VT, 7>(a, 0, hblk, st); break;
    default: launch_ls_energy_nc<ET, VT, 8>(a, 0, hblk, st); break;
  }
}

// ------------------------------------------------------------------------------- launchers
template <typename ET, typename VT>
void launch_precompute(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_precompute<ET><<<(unsigned)nblk, a.hthreads, 0, st>>>(a);
}
template <typename ET, typename VT>
void launch_local(const KArgs &a, int64_t nblk, bool pre, cudaStream_t st) {
  if (pre) k_local<ET, true><<<(unsigned)nblk, a.hthreads, 0, st>>>(a);
  else k_local<ET, false><<<(unsigned)nblk, a.hthreads, 0, st>>>(a);
}
template <typename ET, typename VT>
void launch_spmv_elems(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_spmv<ET><<<(unsigned)nblk, a.hthreads, 0, st>>>(a);
}
template <typename VT>
void launch_soft_rhs(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_soft_rhs<VT><<<(unsigned)nblk, a.vthreads, 0, st>>>(a);
}
template <typename VT>
void launch_cg_start(const KArgs &a, int64_t nblk, cudaStream_t st) {
  k_cg_start<VT><<<(unsigned)nblk, a.vthreads, 0, st>>>(a);
}
template <typename VT>
void launch_cg_iter(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, cudaStream_t st, bool with_dir) {
  k_spmv<VT><<<(unsigned)(hblk + cblk), a.hthreads, 0, st>>>(a);  // element and soft terms
  k_cg_alpha<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
  k_cg_update<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
  if (with_dir) k_cg_dir<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
}
// The vector side of one PCG iteration without its element SpMV (timing).
template <typename VT>
void launch_cg_vec(const KArgs &a, int64_t vblk, int64_t cblk, cudaStream_t st) {
  k_soft_mv<VT><<<(unsigned)cblk, a.vthreads, 0, st>>>(a);
  k_cg_alpha<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
  k_cg_update<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
  k_cg_dir<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
}
template <typename VT>
void launch_cg_dir(const KArgs &a, int64_t vblk, cudaStream_t st) {
  k_cg_dir<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
}
void launch_ir_residual(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, bool replace, cudaStream_t st) {
  if (replace) k_ir_acc<<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
  k_ir_resid<<<(unsigned)hblk, a.hthreads, 0, st>>>(a, replace ? 1 : 0);
  k_ir_soft<<<(unsigned)cblk, a.vthreads, 0, st>>>(a, replace ? 1 : 0);
  if (replace) k_ir_norm<<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
}
template <typename VT>
void launch_fixed_pre(const KArgs &a, int64_t hblk, int64_t vblk, cudaStream_t st) {
  k_fixed_pre<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
  k_spmv<VT><<<(unsigned)hblk, a.hthreads, 0, st>>>(a);
}
void launch_result_positions(const KArgs &a, int64_t cblk, double *Xm, int type, cudaStream_t st) {
  k_result_positions<<<(unsigned)cblk, a.vthreads, 0, st>>>(a, Xm, type);
}
void launch_glue_schedule(MeshScalars *sc, int n, int before, int iter, cudaStream_t st) {
  k_glue_schedule<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(sc, n, before, iter);
}
void launch_ir_final(const KArgs &a, int64_t vblk, cudaStream_t st) {
  k_ir_final<<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
}
template <typename ET, typename VT>
void launch_line_search(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, cudaStream_t st) {
  k_ls_bound<ET, VT><<<(unsigned)hblk, a.hthreads, 0, st>>>(a);
  k_ls_roots<VT><<<152 * 4, 128, 0, st>>>(a);
  k_ls_bound_finish<<<(unsigned)a.n_meshes, 128, 0, st>>>(a, a.n_meshes);
  k_ls_soft<VT><<<(unsigned)cblk, a.vthreads, 0, st>>>(a, -1);
  const int rounds = (kHalvings + 1 + a.ls_cand - 1) / a.ls_cand;
  for (int r = 0; r < rounds; r++) {
    switch (a.ls_cand) {
      case 1: launch_ls_energy_nc<ET, VT, 1>(a, r, hblk, st); break;
      case 2: launch_ls_energy_nc<ET, VT, 2>(a, r, hblk, st); break;
      case 3: launch_ls_energy_nc<ET, VT, 3>(a, r, hblk, st); break;
      case 4: launch_ls_energy_nc<ET, VT, 4>(a, r, hblk, st); break;
      case 5: launch_ls_energy_nc<ET, VT, 5>(a, r, hblk, st); break;
      case 6: launch_ls_energy_nc<ET, VT, 6>(a, r, hblk, st); break;
      case 7: launch_ls_energy_nc<ET, VT, 7>(a, r, hblk, st); break;
      default: launch_ls_energy_nc<ET, VT, 8>(a, r, hblk, st); break;
    }
    k_ls_soft<VT><<<(unsigned)cblk, a.vthreads, 0, st>>>(a, r);
  }
  k_ls_apply<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
}

// explicit instantiations for the two modes
#define HX_INST(ET, VT)                                                                          \
  template void launch_precompute<ET, VT>(const KArgs &, int64_t, cudaStream_t);                 \
  template void launch_local<ET, VT>(const KArgs &, int64_t, bool, cudaStream_t);                \
  template void launch_spmv_elems<ET, VT>(const KArgs &, int64_t, cudaStream_t);                 \
  template void launch_soft_rhs<VT>(const KArgs &, int64_t, cudaStream_t);                       \
  template void launch_cg_start<VT>(const KArgs &, int64_t, cudaStream_t);                       \
  template void launch_cg_iter<VT>(const KArgs &, int64_t, int64_t, int64_t, cudaStream_t, bool); \
  template void launch_cg_dir<VT>(const KArgs &, int64_t, cudaStream_t);                         \
  template void launch_cg_vec<VT>(const KArgs &, int64_t, int64_t, cudaStream_t);                \
  template void launch_fixed_pre<VT>(const KArgs &, int64_t, int64_t, cudaStream_t);             \
  template void launch_line_search<ET, VT>(const KArgs &, int64_t, int64_t, int64_t, cudaStream_t); \
  template void launch_ls_energy_pass<ET, VT>(const KArgs &, int64_t, cudaStream_t);
HX_INST(double, double)
HX_INST(float, float)
#undef HX_INST

}  // namespace hexopt
