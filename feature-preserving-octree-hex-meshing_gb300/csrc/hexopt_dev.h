// hexopt_dev.h -- structures shared by the host runtime (hexopt_api.cu) and the kernels.
//
// HBM layout (one batch of meshes, concatenated):
//  * vertex vectors: AoS with stride 4 (x, y, z, pad) -- one 32 B (FP64) / 16 B (FP32) load per
//    vertex gather; positions are always FP64;
//  * hex corners and per-tet coefficients: AoSoA in tiles of 32 hexes, so that with one thread per
//    hex every load instruction of a warp reads 32 consecutive words:
//       hexv[(h/32)*256 + c*32 + h%32]                 (corner c of hex h, global vertex id)
//       tet[(h/32)*32*8*NC + (k*NC + comp)*32 + h%32]    (component comp of corner tet k)
//  * curve (feature-line) unknowns a_L: plain arrays, appended after each mesh's vertices in the
//    "unknown items" numbering used by the vector kernels.
#pragma once
#include <stdint.h>

namespace hexopt {

constexpr int kMaxCand = 8;   // line-search step sizes evaluated per pass (upper bound)
constexpr int kHalvings = 21; // igl::line_search: cur_iter > 20 -> step 0 (line_search.cpp:31-34)

__host__ __device__ __forceinline__ int64_t hex_idx(int64_t h, int c) { return (h >> 5) * 256 + c * 32 + (h & 31); }
template <int NC>
__host__ __device__ __forceinline__ int64_t tet_idx(int64_t h, int k, int comp) {
  return (h >> 5) * (32 * 8 * NC) + (k * NC + comp) * 32 + (h & 31);
}

struct Seg {
  int32_t mesh;
  int32_t blk_in_mesh;
  int64_t begin, end;  // item range (global item ids of the launch kind)
};

// Per-mesh description (device copy of host data).
struct MeshDesc {
  int64_t v_off, nv;  // vertices
  int64_t h_off, nh;  // hexes
  int64_t c_off, nc;  // corner constraints
  int64_t t_off, nt;  // tangent-plane constraints
  int64_t l_off, nl;  // feature-line constraints (and curve unknowns)
  int64_t b_off, nb;  // projection points (Tetralize_Set::b / bc)
  int64_t grp_off, ngrp;  // glue groups (vertex copies tied to their mean)
  int64_t g_off;      // first own-shape slot (hexes with a per-tet rest matrix)
  // block tables of the SLIM launch kinds: first block and block count
  int64_t hblk0, vblk0, cblk0;
  int32_t nhblk, nvblk, ncblk, pad0;
  // generic launch kinds (kinds K_*): first block, block count, first item
  int64_t kblk0[8];
  int64_t kitem0[8];
  int64_t kcount[8];
  int32_t knblk[8];
};

// Launch kinds with per-mesh segment tables.
enum Kind { K_HEX = 0, K_VERT = 1, K_CONS = 2, K_TGTV = 3, K_SURFV = 4, K_PROJ = 5, K_LINE = 6, K_SURFF = 7 };

// Per-mesh scalars of one optimiser iteration (FP64).
struct MeshScalars {
  double M, prox, exp_f;
  double lamda_C, lamda_T, lamda_L, lamda0;
  // CG (Eigen semantics)
  double rhs_norm2, threshold, abs_new, alpha, beta, rn2, cg_error;
  double rz_prev;  // r.z before the last update (a replaced residual restarts beta from it)
  int32_t cg_iters, cg_done;
  // line search
  double min_root, max_step, old_e, old_eq, old_es;
  double cand_e[kMaxCand], cand_eq[kMaxCand], cand_es[kMaxCand];
  double step, energy, eq, es;
  int32_t ls_done, halvings;
  // quality
  double sj_min, sj_sum, sj_dev;
  int64_t n_inv;
  int32_t status;  // bit flags, see HEXOPT_STATUS_* in hexopt_gpu.h
  // feature-alignment schedule state (grid_hex_meshing.cpp:3852-3882, 4148-4184)
  int32_t fa_iter;   // outer iterations done
  int32_t max_sat;   // Max_dis_satisified: freezes the weight schedule
  double HR;         // Hausdorff ratio threshold (args.Hausdorff_ratio_t)
  double haus_diag, haus_max, haus_ave;
  double adj_eq, adj_es;  // energy_fwd parts
  // untangling / glue path (add_soft_constraints projection and glue terms, slim_solve2's
  // adaptive branch)
  double lamda_P, lamda_G;  // Tetralize_Set::lamda_projection, lamda_glue
  int32_t glue;             // glue terms on: the feature terms are off (slim_m.cpp:611, 647)
  int32_t frozen;           // adaptive loop finished for this mesh: later steps leave it in place
};

}  // namespace hexopt
