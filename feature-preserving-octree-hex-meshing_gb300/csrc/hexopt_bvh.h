// hexopt_bvh.h -- LBVH / target / Hausdorff structures shared by the runtime and k_bvh.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "hexopt_dev.h"

namespace hexopt {

// A linear BVH over n triangles.  Internal nodes 0..n-2 (root 0), leaves in sorted order; a
// child id >= 0 is an internal node, < 0 is leaf ~id.  Boxes: (2n-1) x 6 floats, internal nodes
// first then leaves.  Static trees read triangles from `tri` (9 doubles per face id); dynamic
// trees gather them from the positions X through F (3 global vertex ids per face).
struct BvhDev {
  int32_t n;
  int32_t pad;
  const int32_t *child;
  const float *box;
  const int32_t *leaf_face;
  const double *tri;
  const int32_t *F;
  const double *X;
  // packed internal nodes, 64 B each: both children's boxes and ids in one record
  // (lo/hi of the left box, lo/hi of the right box, left id, right id)
  const float4 *node;
  // per leaf (sorted order), 48 B: first vertex and the two edges from it in FP32 -- the
  // screening data of the leaf's triangle
  const float4 *leafd;
  // static trees only (null otherwise): 128-byte internal node records with both children's
  // oriented boxes -- rows of an orthonormal frame and the extents along them -- and ids
  const float4 *onode;
};

// Per-mesh refit view of a dynamic (hex-boundary) surface tree: the tree and the buffers the
// refit writes.
struct RefitDev {
  BvhDev b;
  float *box;
  const int32_t *parent;
  unsigned *counters;
  float4 *node;
  float4 *leafd;
};

// Queries that exceed the per-thread traversal budget are finished by a warp-cooperative pass.
struct Overflow {
  int64_t *item;     // query item ids
  int32_t *mesh;     // their meshes
  unsigned *count;   // number of entries
  double *best;      // per query item: best (squared for closest point) distance found so far
  int32_t *face;     // per query item: face of that best (closest point)
  double *pt;        // per query item: closest point (3)
};

// Batched exact evaluation.  The traversals record, per query, the leaves that FP32 cannot
// rule out (in visiting order) into one flat list; a dense pass evaluates every entry in FP64
// (one entry per thread), and a per-query pass applies the sequential improvement rule in
// recorded order.  Queries whose candidates do not fit go to the exact per-thread fallback.
struct CandBuf {
  int32_t *leaf, *qi;     // [cap] leaf (sorted order) and query item of each entry
  double *x, *d;          // [cap] exact value (squared distance / PointDistanceEP) and plane distance
  unsigned *count;        // entries used
  int64_t cap;
  int32_t *q_off, *q_cnt; // per query item: first entry and entry count (-1: fallback)
  double *qpos;           // per query item: the query point (3)
  int32_t *q_mesh;        // per query item: its mesh
  unsigned *fb_count;     // fallback list: count, items, meshes
  int64_t *fb_item;
  int32_t *fb_mesh;
};

// A mesh's target triangle mesh (mf.tri / tri_tree): geometry, per-face normals of
// build_aabb_tree, and the feature curves as polylines over its vertices.
struct TargetDev {
  BvhDev bvh;
  const double *TV;       // target vertices, rows of 3
  const double *tri;      // 9 doubles per face
  const double *FN;       // face normals (3 per face)
  // per face, 16 doubles: PointDistanceEP's set-up of the face (edges scaled by the dominant
  // normal component, unit normal, plane offset, double area, dominant axis), formed once
  const double *EP;
  const double *VNc;      // angle-weighted vertex normal of each corner (9 per face)
  const double *ENc;      // uniform edge normal of the edge opposite each corner (9 per face)
  const int64_t *curve_ptr;
  const int32_t *curve_vs;
  const uint8_t *curve_closed;
};

struct ProjArgs {
  Overflow ovf;
  CandBuf cand;
  const Seg *seg;
  const MeshDesc *mesh;
  MeshScalars *sc;
  const TargetDev *tgt;
  const double *X;
  const int32_t *t_ids;
  double *t_nrm, *t_dis;
  const int32_t *l_ids, *l_curve;
  double *l_axis, *l_orig;
  // per projection item: the leaf that won its previous query (-1: none), whose FP32 upper
  // bound at the new position seeds the traversal's pruning bound
  int32_t *seed;
  int budget;  // per-thread traversal pops before the warp pass takes a query over (0: default)
};

struct HausMesh {
  double tgt_lo[3], tgt_hi[3];  // bbox of the target vertices (static)
  double diag;                  // inflated bbox diagonal of both surfaces
  double side_max[2], side_mean[2];
  double max_dist, ave_dist;
};

struct HausArgs {
  Overflow ovf;
  CandBuf cand;
  double *dist;             // per sample item of the side being processed
  const Seg *seg;
  const MeshDesc *mesh;
  MeshScalars *sc;
  const TargetDev *tgt;
  const BvhDev *surf;       // per mesh: dynamic BVH over the boundary triangles
  HausMesh *hm;
  const double *X;
  const int64_t *tgt_vs;    // K_TGTV items: referenced target vertices (target-local ids)
  const int64_t *surf_vs;   // K_SURFV items: referenced surface vertices (global ids)
  double *partials;
  unsigned *counters;
  int32_t *seed;            // per sample item of this side: the previous winning leaf (-1: none)
  int budget;               // per-thread traversal pops before the warp pass (0: default)
};

void bvh_morton(const BvhDev &b, const double lo[3], const double hi[3], unsigned long long *keys, cudaStream_t st);
// range (optional, 2 per internal node): the node's first and last leaf in sorted order
void bvh_karras(int n, const unsigned long long *keys, int32_t *child, int32_t *parent, int32_t *leaf_face,
                cudaStream_t st, int32_t *range = nullptr);
// oriented boxes of every node of a fitted static tree (obb: (2n - 1) x 64 B scratch) and the
// 128-byte oriented records built from them
void bvh_orient(const BvhDev &b, const int32_t *range, float4 *obb, float4 *onode, cudaStream_t st);
// refit boxes bottom-up and rewrite the packed node records
void bvh_refit(const BvhDev &b, float *box, const int32_t *parent, unsigned *counters, float4 *node, float4 *leafd,
               cudaStream_t st);
// every mesh's surface tree in one launch (segment table over the surface faces, kind K_SURFF);
// node records written as each internal node's box is finalised
void bvh_refit_batch(const RefitDev *R, const Seg *seg, const MeshDesc *md, int64_t nblk, int threads,
                     cudaStream_t st);
// both passes of the tangent-plane projection
void launch_project(const ProjArgs &p, int64_t nblk, cudaStream_t st);
void launch_curve_project(const ProjArgs &p, int64_t nblk, cudaStream_t st);
void launch_signed_distance(const TargetDev &t, int64_t np, const double *P, double *S, int32_t *I, double *C,
                            double *N, int *status, cudaStream_t st);
void launch_haus_bbox(const HausArgs &h, int64_t nblk, cudaStream_t st);
// both passes of one Hausdorff side (per-sample distances into h.dist) and its reduction
void launch_haus_side(const HausArgs &h, int side, int64_t nblk, cudaStream_t st);
// after both sides: each mesh's Hausdorff max and mean from the two sides' results
void launch_haus_combine(HausMesh *hm, int n, cudaStream_t st);
void launch_ep_points(const BvhDev &b, const double *P, const int64_t *ids, int64_t n, double upper, double *dist,
                      int *status, cudaStream_t st);
void launch_maxmean(const double *dist, int64_t n, double upper, double *out3, cudaStream_t st);
void launch_fa_haus_flag(MeshScalars *sc, const HausMesh *hm, int n, cudaStream_t st);
// PointDistanceEP's per-face set-up of a static triangle set (tri: 9 doubles per face)
void launch_ep_faces(const double *tri, int64_t nf, double *EP, cudaStream_t st);

}  // namespace hexopt
