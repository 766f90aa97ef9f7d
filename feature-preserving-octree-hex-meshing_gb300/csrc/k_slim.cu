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
// Persistent blocks of k_spmv_pipe: the resident blocks of the whole device, at most one warp
// per 32-hex unit.
static int spmv_pipe_blocks(const KArgs &a) {
  static int resident = 0;
  if (resident == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmv_pipe, kPipeWarps * 32, 0);
    resident = std::max(1, sms * per_sm);
  }
  const int64_t units = a.hblk * (a.hthreads / 32);
  return (int)std::max<int64_t>(1, std::min<int64_t>(resident, (units + kPipeWarps - 1) / kPipeWarps));
}
static void launch_spmv_pipe(const KArgs &a, int64_t cblk, cudaStream_t st) {
  const int npipe = spmv_pipe_blocks(a);
  k_spmv_pipe<<<(unsigned)(npipe + cblk), kPipeWarps * 32, 0, st>>>(a, npipe, a.hthreads / 32);
}
template <typename ET, typename VT>
void launch_spmv_elems(const KArgs &a, int64_t nblk, cudaStream_t st) {
  if constexpr (sizeof(ET) == 4) launch_spmv_pipe(a, 0, st);
  else k_spmv<ET><<<(unsigned)nblk, a.hthreads, 0, st>>>(a);
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
  if constexpr (sizeof(VT) == 4) launch_spmv_pipe(a, cblk, st);  // element and soft terms
  else k_spmv<VT><<<(unsigned)(hblk + cblk), a.hthreads, 0, st>>>(a);
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
// One round of candidate passes: the elastic energies, then the soft energies whose last block
// takes the round's decision (round = kRoundFromDevice: the round counter on the device).
template <typename ET, typename VT>
static void launch_ls_round(const KArgs &a, int r, int64_t hblk, int64_t cblk, cudaStream_t st) {
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

// The end of a WHILE iteration: next round, and another iteration only while a mesh is still
// searching and rounds remain (at most `rounds` iterations however the flags stand).
static __global__ void k_ls_next(KArgs a, cudaGraphConditionalHandle h, int rounds) {
  const unsigned r = *a.ls_round + 1;
  *a.ls_round = r;
  cudaGraphSetConditional(h, (*a.ls_active > 0 && (int)r < rounds) ? 1u : 0u);
}

template <typename ET, typename VT>
cudaError_t launch_line_search(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, cudaStream_t st,
                               cudaStream_t body) {
  k_ls_bound<ET, VT><<<(unsigned)hblk, a.hthreads, 0, st>>>(a);
  k_ls_roots<VT><<<152 * 4, 128, 0, st>>>(a);
  k_ls_bound_finish<<<(unsigned)a.n_meshes, 128, 0, st>>>(a, a.n_meshes);  // also round = 0
  k_ls_soft<VT><<<(unsigned)cblk, a.vthreads, 0, st>>>(a, -1);
  const int rounds = (kHalvings + 1 + a.ls_cand - 1) / a.ls_cand;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  if (body && cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd) == cudaSuccess &&
      cs == cudaStreamCaptureStatusActive) {
    // a WHILE node whose body runs one round: the graph stops at the first round that leaves no
    // mesh searching, instead of launching rounds - 1 passes that only check a flag.  Any
    // failure from here on is returned, so that the caller discards the capture: a body without
    // its k_ls_next would never clear the condition.
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &np);
    if (e != cudaSuccess) return e;
    e = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return e;
    cudaGraph_t bg = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(body, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    launch_ls_round<ET, VT>(a, kRoundFromDevice, hblk, cblk, body);
    k_ls_next<<<1, 1, 0, body>>>(a, h, rounds);
    const cudaError_t le = cudaGetLastError();
    e = cudaStreamEndCapture(body, &bg);
    if (le != cudaSuccess) return le;
    if (e != cudaSuccess) return e;
    k_ls_apply<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
    return cudaGetLastError();
  }
  for (int r = 0; r < rounds; r++) launch_ls_round<ET, VT>(a, r, hblk, cblk, st);
  k_ls_apply<VT><<<(unsigned)vblk, a.vthreads, 0, st>>>(a);
  return cudaSuccess;
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
  template cudaError_t launch_line_search<ET, VT>(const KArgs &, int64_t, int64_t, int64_t, cudaStream_t, cudaStream_t); \
  template void launch_ls_energy_pass<ET, VT>(const KArgs &, int64_t, cudaStream_t);
HX_INST(double, double)
HX_INST(float, float)
#undef HX_INST

}  // namespace hexopt
