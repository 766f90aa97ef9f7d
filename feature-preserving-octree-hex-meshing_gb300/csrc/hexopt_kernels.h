// hexopt_kernels.h -- kernel argument block and launcher declarations (host + device).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "hexopt_dev.h"

namespace hexopt {

// Everything a kernel may touch, passed by value.  Vector pointers whose scalar type depends on
// the arithmetic mode are void*.
struct KArgs {
  // batch tables
  const MeshDesc *mesh;
  MeshScalars *sc;
  const Seg *hseg, *vseg, *cseg;
  int64_t hblk;  // hex blocks: an element-SpMV launch's blocks past them run the soft terms
  double *partials;
  unsigned *counters;
  // geometry
  const uint32_t *hexv;  // AoSoA corners
  const int32_t *gslot;  // per hex: -1 cube target, else own-shape slot
  double *X;             // positions AoS4 FP64
  float *X32;            // FP32 hi/lo split of X per vertex: hi.xyz, 0, lo.xyz, 0 (x = hi + lo to ~48 bits)
  double *aL;            // curve parameters (FP64)
  void *Sinv;            // per tet 1/cbrt(6 vol) (ET, AoSoA NC=1)
  void *Ccoef;           // per tet C_t (ET, AoSoA NC=6)
  double *Bgen;          // own-shape rest inverses, 9 per tet
  const double *Bref;    // general reference shapes (k_shapes.cu): adj(R) / |det R|^(2/3) per tet slot, or
                         // null; with it every hex has a slot and the precompute sets Bgen = Bref / cbrt(det E)
  // linear system right-hand side and diagonal (VT)
  void *b, *diag, *ba, *diaga;
  // CG vectors (VT)
  void *d, *r, *p, *q, *invd;
  void *da, *ra, *pa, *qa, *invda;
  // mixed mode's FP64 refinement: per-tet rotations R of the local step (FP32, AoSoA NC=9), and
  // the update accumulated in FP64 between residual replacements (vertices AoS4, curve entries)
  float *Rrot;
  double *dd, *dda;
  float *ddf;  // fl32(dd) per vertex (AoS4), written with dd: the residual pass's corner gathers
  // constraints
  const int32_t *c_ids; const double *c_pos;
  const int32_t *t_ids; double *t_nrm; double *t_dis;
  const int32_t *l_ids; double *l_axis; double *l_orig;
  const int32_t *b_ids; const double *b_pos;      // projection points and their targets bc
  const int64_t *g_ptr; const int32_t *g_vs;      // glue groups: member ranges, global vertex ids
  const uint8_t *vfix;                            // held (known-value) vertices, or null
  int has_fixed;
  // parameters
  int energy;
  int cg_max_iter;
  int ls_cand;
  int n_meshes;
  double cg_tol;
  double sc_exp_f;
  int cg_refine;  // mixed mode: inner FP32 iterations between residual replacements
  int hthreads;   // block size of hex-kind launches (<= 128)
  int vthreads;   // block size of vertex / constraint launches (<= 256)
  // adjoint
  double *Xa;     // evaluation point (AoS4 FP64)
  double *grad;   // dE/dX (AoS4 FP64)
  // flip-avoiding step bound: corner tets whose cubic may have a root in [0, 1.25] (8 h + K),
  // their meshes, the count, and the per-mesh minimum root (bits of a non-negative double)
  uint32_t *root_list;
  int32_t *root_mesh;
  unsigned *root_count;
  unsigned long long *root_min;
  // meshes whose line search has not accepted a step yet (later candidate passes exit when 0)
  unsigned *ls_active;
  // the line-search round of a graph's WHILE loop (passes launched with round kRoundFromDevice)
  unsigned *ls_round;
};
constexpr int kRoundFromDevice = -2;

template <typename ET, typename VT> void launch_precompute(const KArgs &a, int64_t nblk, cudaStream_t st);
// fused local step; pre = also take the volume snapshot (slim_precompute) at the current X
template <typename ET, typename VT> void launch_local(const KArgs &a, int64_t nblk, bool pre, cudaStream_t st);
template <typename ET, typename VT> void launch_spmv_elems(const KArgs &a, int64_t nblk, cudaStream_t st);
template <typename VT> void launch_soft_rhs(const KArgs &a, int64_t nblk, cudaStream_t st);
template <typename VT> void launch_cg_start(const KArgs &a, int64_t nblk, cudaStream_t st);
// one PCG iteration: SpMV, soft block, alpha, update and (with_dir) the next direction
template <typename VT>
void launch_cg_iter(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, cudaStream_t st, bool with_dir = true);
template <typename VT> void launch_cg_dir(const KArgs &a, int64_t vblk, cudaStream_t st);
template <typename VT> void launch_cg_vec(const KArgs &a, int64_t vblk, int64_t cblk, cudaStream_t st);
// Mixed mode's FP64 iterative refinement of the PCG (k_slim.cuh): the residual b - A x at
// x = X + dd re-evaluated from the FP64 positions (element terms in double-float, soft and
// proximal terms in FP64); `replace` = a replacement inside the CG (accumulate d into dd first,
// then take the new residual's norms), else the initial residual of the solve.
void launch_ir_residual(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, bool replace, cudaStream_t st);
// Held vertices: q = L_ib x_b (element part) for the rhs norm of the known-value solve.
template <typename VT> void launch_fixed_pre(const KArgs &a, int64_t hblk, int64_t vblk, cudaStream_t st);
// Result mesh of the adaptive branch: Xm (a copy of X) with glue groups at their means (type 1)
// or projection points at bc (type 0); glue weight schedules (k_slim.cuh).
void launch_result_positions(const KArgs &a, int64_t cblk, double *Xm, int type, cudaStream_t st);
void launch_glue_schedule(MeshScalars *sc, int n, int before, int iter, cudaStream_t st);
// After the last PCG iteration: the search direction d = fl32(dd + d) (curve entries likewise).
void launch_ir_final(const KArgs &a, int64_t vblk, cudaStream_t st);
template <typename ET, typename VT> void launch_ls_energy_pass(const KArgs &a, int64_t hblk, cudaStream_t st);
// body: with st capturing into a graph, a second stream that is not; the candidate rounds then
// become a WHILE node that stops once every mesh has accepted (otherwise fixed rounds that no-op)
template <typename ET, typename VT>
cudaError_t launch_line_search(const KArgs &a, int64_t hblk, int64_t vblk, int64_t cblk, cudaStream_t st,
                               cudaStream_t body = nullptr);

// Launches per call of the launchers above (for the launch count).
constexpr int kLaunchesCgIter = 4;  // element + soft SpMV, alpha, update, direction
constexpr int kLaunchesIrInitial = 2, kLaunchesIrReplace = 4, kLaunchesIrFinal = 1;

// ---- reference shapes (k_shapes.cu) ----
// Bref of every hex from its reference corners: P8 (nh x 8 x 3) when given, else the current
// positions X through the hexes; cube / h_flag as compute_referenceMesh.
void launch_ref_shapes(const double *P8, const uint32_t *hexv, const double *X, const uint8_t *hflag, int cube,
                       int64_t nh, double *Bref, cudaStream_t st);

// Bref from explicit reference tets (ntet x 4 x 3 corners, device order)
void launch_ref_from_tets(const double *RT, int64_t ntet, double *Bref, cudaStream_t st);
// rigidDeformCubes on an exploded mesh (every hex owns its 8 corners): hexes with no held corner
// become the unit cube fitted to their corners (Procrustes with scaling, no reflection).
void launch_rigid_cubes(const uint32_t *hexv, double *X, float *X32, const uint8_t *vfix, int64_t nh, cudaStream_t st);

// ---- adjoint (k_adjoint.cu) ----
template <typename ET> void launch_energy_fwd(const KArgs &a, int64_t hblk, int64_t cblk, cudaStream_t st);
template <typename ET> void launch_energy_bwd(const KArgs &a, int64_t hblk, int64_t cblk, cudaStream_t st);

// ---- quality (k_quality.cu) ----
void launch_scaled_jacobian(const KArgs &a, int64_t hblk, double *V_Js, double *H_Js, cudaStream_t st);
// FP32-screened minimum / inversion check used inside the mixed-mode optimiser iteration
void launch_sj_check(const KArgs &a, int64_t hblk, cudaStream_t st);
// weight schedule + report packing for the feature-alignment step
void launch_fa_schedule(MeshScalars *sc, int n_meshes, double lamda0, double bound, cudaStream_t st);

// ---- layout helpers (k_layout.cu) ----
void launch_rows_to_aos4(const double *src, double *dst, int64_t n, cudaStream_t st);
void launch_aos4_to_rows(const double *src, double *dst, int64_t n, cudaStream_t st);
// X32 <- hi/lo split of the FP64 positions (after every host-side write of X)
void launch_split_pos(const double *X, float *X32, int64_t n, cudaStream_t st);
void launch_hex_to_aosoa_mesh(const uint32_t *src, int64_t h0, int64_t nh, uint32_t voff, uint32_t *dst,
                              cudaStream_t st);

// ---- area-uniform surface samples (k_sample.cu) ----
// n samples of the triangles (V rows, F) drawn with SplitMix64 counters from `seed`, into P (n x 3).
cudaError_t sample_surface(const double *V, const int32_t *F, int64_t nf, int64_t n, uint64_t seed, double *P,
                           void *scratch, size_t scratch_bytes, cudaStream_t st);
size_t sample_scratch_bytes(int64_t nf);

// ---- Morton ordering of the batch (k_order.cu) ----
// Sorts the vertices (by position) and hexes (by centroid) of every mesh along a Morton curve of
// the mesh's bounding box (box_d: 6 doubles per mesh), meshes kept contiguous; writes both
// permutations each way.  rows: caller-order vertex rows (NV x 3), H: caller hexes (mesh-local
// ids); voff_d / hoff_d: n_meshes + 1 offsets; scratch: order_scratch_bytes(NV, NH) bytes.
cudaError_t order_batch(const double *rows, const uint32_t *H, int64_t NV, int64_t NH, const int64_t *voff_d,
                        const int64_t *hoff_d, int n_meshes, const double *box_d, int32_t *vnew2old, int32_t *vold2new,
                        int32_t *hnew2old, int32_t *hold2new, void *scratch, size_t scratch_bytes, cudaStream_t st);
size_t order_scratch_bytes(int64_t NV, int64_t NH);
void launch_hex_perm(const uint32_t *H, const int32_t *hnew2old, const int32_t *vold2new, int64_t nh, const int64_t *hoff,
                     const int64_t *voff, int n_meshes, uint32_t *hexv, cudaStream_t st);
// dst[i] = src[perm[i]] (rows of `width` doubles; perm null = copy)
void launch_gather_rows(const double *src, const int32_t *perm, int64_t n, int width, double *dst, cudaStream_t st);
// X[i] = rows[new2old[i]] / rows[i] = X[old2new[i]] (null = identity)
void launch_rows_to_aos4_perm(const double *rows, const int32_t *new2old, int64_t n, double *X, cudaStream_t st);
void launch_aos4_to_rows_perm(const double *X, const int32_t *old2new, int64_t n, double *rows, cudaStream_t st);

}  // namespace hexopt
