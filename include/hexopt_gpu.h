/*
 * hexopt_gpu.h -- C ABI of libhexopt_gpu.so, the GB300 (sm_103a) implementation of the
 * octree hex mesher's geometric-optimisation hot path.
 *
 * Every entry point returns an int status (HEXOPT_OK == 0); hexopt_last_error() gives the
 * message of the last failure.  Arguments are plain pointers and sizes; unless a name says
 * "_device", pointers are host memory.  Array conventions: vertices are row-major n x 3
 * doubles (x, y, z per vertex); hexes are 8 uint32 corner ids per hex in the reference's
 * corner order (hex_ref_shape, global_types.h:208-218); ids inside per-mesh arrays are local
 * to their mesh.  A context holds one batch of meshes (n_meshes >= 1) resident in HBM and a
 * CUDA stream; calls on one context are not re-entrant.
 *
 * Correspondence with the reference interface this library stands in for (file:line inside the
 * reference project):
 *   hexopt_scaled_jacobian        <- bool scaled_jacobian(Mesh&, Mesh_Quality&)        global_functions.h:81
 *   hexopt_slim_precompute        <- slim_precompute(V, F, V_init, SLIMData&, SLIM_ENERGY, Tetralize_Set)
 *                                                                                      slim_m.h:102-108
 *   hexopt_slim_iterate           <- slim_solve2(SLIMData&, iter_num, type) fixed-N branch  slim_m.h:114
 *   hexopt_slim_m_opt             <- optimization::slim_m_opt(Tetralize_Set&, iter, type)   optimization.h:32
 *   hexopt_signed_distance        <- igl::signed_distance_pseudonormal (called by dirty_graph_projection,
 *                                    grid_hex_meshing.cpp:4031-4078) over build_aabb_tree  (:4231-4248)
 *   hexopt_project_features       <- dirty_graph_projection               grid_hex_meshing.cpp:3954-4082
 *   hexopt_hausdorff              <- void compute(const Mesh&, const Mesh&, double& diag, double& max,
 *                                    double& ave)                                       metro_hausdorff.h:37
 *   hexopt_feature_alignment_step <- one pass of the feature_alignment loop   grid_hex_meshing.cpp:3855-3882
 *   hexopt_aabb_*                 <- struct AABB / struct Ray                             aabb.h:5-115
 */
#ifndef HEXOPT_GPU_H
#define HEXOPT_GPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define HEXOPT_API __attribute__((visibility("default")))
#else
#define HEXOPT_API
#endif

/* ---- status codes ---- */
#define HEXOPT_OK 0
#define HEXOPT_ERR_ARG 1         /* invalid argument (sizes, ids out of range, NULL) */
#define HEXOPT_ERR_CUDA 2        /* a CUDA call failed */
#define HEXOPT_ERR_STATE 3       /* call order (e.g. iterate before precompute) */
#define HEXOPT_ERR_NUMERIC 4     /* NaN/Inf or degenerate element detected on the device */
#define HEXOPT_ERR_UNSUPPORTED 5 /* option outside what the library implements */
#define HEXOPT_ERR_NOMEM 6       /* device allocation failed */

/* ---- per-mesh device status bits (hexopt_slim_report.status) ---- */
#define HEXOPT_STATUS_NONFINITE_ENERGY 1  /* line search met only NaN/Inf energies */
#define HEXOPT_STATUS_DEGENERATE_TET 2    /* zero-volume tet at precompute (reference: Inf/NaN) */
#define HEXOPT_STATUS_CG_BREAKDOWN 4      /* p^T A p <= 0 in the PCG */
#define HEXOPT_STATUS_BVH_OVERFLOW 8      /* a BVH traversal stack overflowed */

/* ---- SLIM_ENERGY (global_types.h:58-66) ---- */
#define HEXOPT_ARAP 0
#define HEXOPT_LOG_ARAP 1
#define HEXOPT_SYMMETRIC_DIRICHLET 2
#define HEXOPT_CONFORMAL 3
#define HEXOPT_EXP_CONFORMAL 4
#define HEXOPT_EXP_SYMMETRIC_DIRICHLET 5

/* ---- arithmetic modes ---- */
#define HEXOPT_FP64 0  /* plain: every stage in FP64 */
#define HEXOPT_MIXED 1 /* FP32 local step / energy / SpMV, FP64 accumulation, FP64-refined PCG */

typedef struct hexopt_ctx hexopt_ctx;

/* Mesh_Quality subset (global_types.h:487-511). */
typedef struct hexopt_quality {
  double min_Jacobian;
  double ave_Jacobian;
  double deviation_Jacobian;
  int64_t n_inverted; /* hexes whose minimum corner scaled Jacobian is < 0 */
} hexopt_quality;

typedef struct hexopt_slim_params {
  int energy;          /* SLIM_ENERGY; the reference's feature alignment uses SYMMETRIC_DIRICHLET */
  int precision;       /* HEXOPT_FP64 or HEXOPT_MIXED */
  double weight_opt;   /* SLIMData::weight_opt: M per tet, proximal term 1e-5 * weight_opt */
  double exp_factor;   /* SLIMData::exp_factor of the exponential energies: slim_precompute resets it to
                          1.0 (slim_m.cpp:1125, 1181) after slim_m_opt set 5.0, so 1.0 reproduces
                          the reference */
  int cg_max_iter;     /* 20 (slim_m.cpp:495) */
  double cg_tol;       /* 1e-8 (slim_m.cpp:494) */
  int ls_candidates;   /* step sizes evaluated per line-search pass, 1..8: the same result either way;
                          more per pass means fewer passes but more work per pass (1 is fastest when
                          the first steps are usually accepted, as on the benchmark workloads) */
  int cube;            /* compute_referenceMesh 'cube' flag: 1 in feature alignment */
  int cg_refine;       /* HEXOPT_MIXED only: FP32 PCG iterations between residual replacements, where
                          the accumulated update moves to FP64 and the residual b - A x is
                          re-evaluated from the FP64 positions; <= 0 selects 10 (ignored in FP64) */
  int variant;         /* 0: the reference's slim_m SLIM (optimization::slim_m_opt); 1: its modified
                          igl::slim (optimization::slim_opt_igl, extern/libigl/include/igl/
                          slim.cpp:1190-1288), whose per-tet weight is weight_opt / 2 (:1243-1246) */
} hexopt_slim_params;

typedef struct hexopt_slim_report {
  double energy;         /* SLIMData::energy (total / mesh_area) */
  double energy_quality; /* SLIMData::engery_quality */
  double energy_soft;    /* SLIMData::engery_soft */
  double cg_error;       /* relative residual |b - A x| / |b| of the last CG (mixed mode: from the last
                            re-evaluated residual when it was the last update, else the recurrence) */
  double max_step;       /* flip-avoiding step bound of the last line search */
  double step;           /* accepted step */
  int32_t cg_iters;
  int32_t halvings;
  int32_t status;        /* HEXOPT_STATUS_* bits */
  int32_t pad;
} hexopt_slim_report;

typedef struct hexopt_fa_report {
  hexopt_slim_report slim;
  hexopt_quality quality;     /* scaled Jacobian after the step */
  double lamda;               /* feature weight after the schedule update */
  double hausdorff_diag, hausdorff_max, hausdorff_ave; /* when requested, else -1 */
} hexopt_fa_report;

/* ---- context ---- */
HEXOPT_API int hexopt_create(hexopt_ctx **ctx, int device);
HEXOPT_API void hexopt_destroy(hexopt_ctx *ctx);
HEXOPT_API const char *hexopt_last_error(const hexopt_ctx *ctx);
/* Synchronises the context's stream. */
HEXOPT_API int hexopt_sync(hexopt_ctx *ctx);

/* Device order of the meshes uploaded next.  mode 1 sorts every mesh's vertices by the Morton code
 * of their position and its hexes by that of their centroid, inside the mesh's bounding box, so
 * corner gathers and scatters of neighbouring hexes share cache lines whatever numbering the
 * caller uses; 0 keeps the caller's order; 2 (the default) sorts unless the caller's numbering is
 * already coherent (median corner-id span of a hex and median first-corner jump between
 * consecutive hexes within 4 nv^(2/3), as a structured grid's row order, which coalesces the
 * corner gathers better than a Morton curve).  The ABI speaks the caller's order either way:
 * every vertex id, per-vertex row and per-hex output is mapped at the boundary. */
HEXOPT_API int hexopt_set_ordering(hexopt_ctx *ctx, int mode);

/* ---- meshes ----
 * Uploads a batch: mesh m has nv[m] vertices and nh[m] hexes; V and H are the meshes' arrays
 * concatenated.  h_flag (may be NULL = all 1) marks hexes whose target is a cube of equal volume
 * (1) or their own shape at precompute time (0), as compute_referenceMesh's H_flag. */
HEXOPT_API int hexopt_upload_meshes(hexopt_ctx *ctx, int n_meshes, const int64_t *nv, const int64_t *nh, const double *V,
                         const uint32_t *H, const uint8_t *h_flag);
HEXOPT_API int hexopt_set_positions(hexopt_ctx *ctx, const double *V);
HEXOPT_API int hexopt_get_positions(hexopt_ctx *ctx, double *V);
/* Asynchronous forms for streaming positions through the optimiser: the host <-> device copies
 * run on the context's upload and download streams and overlap the computation queued on its
 * compute stream.
 * set_positions_async: V (nv x 3, caller order) is read after the call returns, so it must stay
 * valid and unchanged until hexopt_sync returns; the positions take effect for the work queued
 * after the call.
 * get_positions_async: the positions after the work queued so far, written into V (nv x 3,
 * caller order) once the copy completes (hexopt_sync, or hexopt_timer_stop, waits for it).
 * Page-locked host buffers let the copies overlap; pageable ones still give correct results. */
HEXOPT_API int hexopt_set_positions_async(hexopt_ctx *ctx, const double *V);
HEXOPT_API int hexopt_get_positions_async(hexopt_ctx *ctx, double *V);
HEXOPT_API int64_t hexopt_num_vertices(const hexopt_ctx *ctx);
HEXOPT_API int64_t hexopt_num_hexes(const hexopt_ctx *ctx);
HEXOPT_API int hexopt_num_meshes(const hexopt_ctx *ctx);

/* ---- quality: scaled_jacobian (global_functions.cpp:2309-2356) for every mesh ----
 * V_Js (8 per hex) and H_Js (1 per hex) may be NULL; q has n_meshes entries. */
HEXOPT_API int hexopt_scaled_jacobian(hexopt_ctx *ctx, double *V_Js, double *H_Js, hexopt_quality *q);

/* ---- soft constraints (Feature_Constraints, global_types.h:583-610) ----
 * Per-mesh counts, concatenated arrays, mesh-local vertex ids. */
HEXOPT_API int hexopt_set_corners(hexopt_ctx *ctx, const int64_t *nC, const int32_t *ids, const double *C);
HEXOPT_API int hexopt_set_tangents(hexopt_ctx *ctx, const int64_t *nT, const int32_t *ids, const double *normal,
                        const double *dis);
HEXOPT_API int hexopt_set_lines(hexopt_ctx *ctx, const int64_t *nL, const int32_t *ids, const double *axis,
                     const double *origin);
/* lamda_C / lamda_T / lamda_L per mesh (n_meshes each) */
HEXOPT_API int hexopt_set_weights(hexopt_ctx *ctx, const double *lamda_C, const double *lamda_T, const double *lamda_L);
HEXOPT_API int hexopt_get_tangents(hexopt_ctx *ctx, double *normal, double *dis);
HEXOPT_API int hexopt_get_lines(hexopt_ctx *ctx, double *axis, double *origin);

/* ---- reference shapes: compute_referenceMesh (global_functions.cpp:3735-3806) ----
 * By default the reference shape of each hex comes from its positions at the precompute, with
 * params.cube and the upload's h_flag: cube = 1 a cube of the hex's 24-tet volume, cube = 0 the
 * edge-averaged cuboid scaled to that volume, h_flag = 0 the hex's own corners.  P8 (n_hexes x 8
 * x 3, the batch's hexes in order, corners in hex order) makes those corners the source instead,
 * as the untangling path builds its shapes from another mesh's positions
 * (optimization.cpp:584); NULL restores the default.  Takes effect at the next precompute. */
HEXOPT_API int hexopt_set_reference_hexes(hexopt_ctx *ctx, const double *P8);
/* The reference tets themselves, as compute_referenceMesh writes them into Tetralize_Set::RT:
 * 4 x 3 corner rows per tet, 8 tets per hex in hex_tetra_table order (n_hexes x 8 x 4 x 3
 * doubles, the batch's hexes in order).  Any shapes -- cubes, cuboids, a hex's own corners --
 * are taken as given; the operator of each tet is then grad_tet_ref's (grad.cpp:372-478) at the
 * tet's positions at the next precompute.  NULL restores the default. */
HEXOPT_API int hexopt_set_reference_tets(hexopt_ctx *ctx, const double *RT);

/* ---- untangling path: Tetralize_Set's projection, glue and known-value terms ----
 * Projection points (ts.b / ts.bc, ts.projection): per mesh nB[m] vertex ids and targets (nB x
 * 3) with weight lamda_projection[m] (may be NULL: unchanged); soft term lamda |x - bc|^2
 * (add_soft_constraints, slim_m.cpp:600-610). */
HEXOPT_API int hexopt_set_projection(hexopt_ctx *ctx, const int64_t *nB, const int32_t *ids, const double *bc,
                                     const double *lamda_projection);
/* Glue groups (ts.glue, V_ranges): per mesh n_groups[m] groups of vertex copies, group_ptr with
 * n_groups[m] + 1 offsets per mesh into that mesh's part of group_vs (mesh-local vertex ids; a
 * vertex in at most one group), weight lamda_glue[m] (may be NULL).  Each copy is tied to the
 * others of its group: lamda (n/(n-1))^2 |x_j - mean|^2 (slim_m.cpp:611-646).  A glued mesh drops
 * its corner / tangent / line terms (:647); feature lines must be cleared first.  FP64 only. */
HEXOPT_API int hexopt_set_glue(hexopt_ctx *ctx, const int64_t *n_groups, const int64_t *group_ptr,
                               const int32_t *group_vs, const double *lamda_glue);
/* Held vertices (known_value_post, slim_m.cpp:403-477): per mesh nF[m] vertex ids held at their
 * current positions; the solve runs over the other vertices (and curve unknowns).  FP64 only. */
HEXOPT_API int hexopt_set_fixed(hexopt_ctx *ctx, const int64_t *nF, const int32_t *ids);

typedef struct hexopt_adaptive_report {
  int32_t iterations;   /* SLIM iterations this mesh ran */
  int32_t converged;    /* 1 when its result mesh's minimum scaled Jacobian became > 0 */
  double min_Jacobian, ave_Jacobian;  /* of the result mesh after its last iteration */
  double energy, energy_quality, energy_soft;
  double lamda_glue;    /* glue weight after its last iteration */
  int32_t status, pad;
} hexopt_adaptive_report;

/* The iter_num = -1 branch of slim_solve2 (schedule 2, slim_m.cpp:1191-1268) and of slim_solve
 * (schedule 1, :1293-1394), after slim_precompute: up to max_iter (50 in the reference) SLIM
 * iterations; after each, the result mesh -- glue groups at their means (type 1) or projection
 * points at their targets (type 0) -- is checked with scaled_jacobian and a mesh stops once its
 * minimum is > 0.  Schedule 2 starts lamda_glue at 1e4 and sets it to
 * min(1e4 max(E_quality / E_soft lamda_glue, 1), 1e16) after each gluing iteration; schedule 1
 * doubles it before iterations 5, 6, ... while it is below 1e8.  rep: n_meshes or NULL. */
HEXOPT_API int hexopt_slim_solve_adaptive(hexopt_ctx *ctx, int type, int schedule, int max_iter,
                                          hexopt_adaptive_report *rep);

typedef struct hexopt_untangle_report {
  int32_t success;      /* pipeline2's result: the glued mesh's minimum scaled Jacobian is >= 0 */
  int32_t iterations;   /* SLIM iterations of the gluing solve */
  double min_Jacobian, ave_Jacobian;  /* of the glued mesh */
  double energy, lamda_glue;
} hexopt_untangle_report;

/* optimization::pipeline2 for hex meshes (optimization.cpp:416-434, rigidDeformCubes :456-494,
 * glueInternalNodes :552-669): every hex gets its own copy of its corners -- the boundary-
 * flagged vertices' copies held, each other hex replaced by the unit cube Procrustes-fitted to
 * its corners -- and the copies are glued back by the adaptive gluing solve (schedule 2, at most
 * max_iter = 50 iterations) with edge-averaged cuboid reference shapes of the input mesh
 * (compute_referenceMesh(..., false)).  The context's positions (the boundary-projected BV) are
 * replaced by the glued ones.  params: energy (the reference's Tetralize_Set default is
 * CONFORMAL), weight_opt, FP64; boundary: one flag per vertex of the batch.  rep: n_meshes. */
HEXOPT_API int hexopt_untangle(hexopt_ctx *ctx, const hexopt_slim_params *params, const uint8_t *boundary,
                               int max_iter, hexopt_untangle_report *rep);

/* ---- SLIM ---- */
HEXOPT_API int hexopt_slim_precompute(hexopt_ctx *ctx, const hexopt_slim_params *params);
/* iters fixed-count SLIM iterations (slim_solve2, slim_m.cpp:1269-1288); rep: n_meshes or NULL */
HEXOPT_API int hexopt_slim_iterate(hexopt_ctx *ctx, int iters, hexopt_slim_report *rep);
/* slim_precompute + iterate, as optimization::slim_m_opt(ts, iters, -1) */
HEXOPT_API int hexopt_slim_m_opt(hexopt_ctx *ctx, const hexopt_slim_params *params, int iters, hexopt_slim_report *rep);
/* curve parameters a_L after the last solve (sum of nL) */
HEXOPT_API int hexopt_get_curve_params(hexopt_ctx *ctx, double *a_L);

/* The smoothing stage (grid_hex_meshing.cpp:2979-3056): `outer` rounds (3 in the reference) of
 * cube reference shapes at the current positions and `inner` (5) iterations of the modified
 * igl::slim (optimization::slim_opt_igl, optimization.cpp:970-1005; params.variant is taken as 1,
 * cube as 1) with whatever soft constraints are set (the stage itself sets none).  rep: the last
 * round's report per mesh, or NULL. */
HEXOPT_API int hexopt_smoothing(hexopt_ctx *ctx, const hexopt_slim_params *params, int outer, int inner,
                                hexopt_slim_report *rep);

/* ---- closest point on a target triangle mesh ----
 * Target of mesh m: triangles TF over TV (mesh-local ids), built into a GPU LBVH with the face,
 * angle-weighted vertex and uniform edge normals of build_aabb_tree. */
HEXOPT_API int hexopt_set_target(hexopt_ctx *ctx, int mesh, int64_t nv, const double *TV, int64_t nf, const int32_t *TF);
/* signed_distance_pseudonormal of np host points against mesh m's target. */
HEXOPT_API int hexopt_signed_distance(hexopt_ctx *ctx, int mesh, int64_t np, const double *P, double *S, int32_t *I, double *C,
                           double *N);

/* Feature projection sets (dirty_graph_projection): per mesh the regular boundary vertices that
 * get tangent planes (ids), the line vertices with their curve (line_ids, line_curve) and the
 * feature curves as polylines over the target's vertices (curve_ptr / curve_vs, closed flag). */
HEXOPT_API int hexopt_set_feature_sets(hexopt_ctx *ctx, const int64_t *n_regular, const int32_t *regular_ids,
                            const int64_t *n_line, const int32_t *line_ids, const int32_t *line_curve,
                            const int64_t *n_curves, const int64_t *curve_ptr, const int32_t *curve_vs,
                            const uint8_t *curve_closed);
/* Recomputes tangent planes and line targets from the current positions. */
HEXOPT_API int hexopt_project_features(hexopt_ctx *ctx);
/* Work counters of the last BVH query pass (projection, or a Hausdorff side): the queries that
 * went past the per-thread traversal budget to the group-cooperative pass, the candidate leaves
 * recorded for exact FP64 evaluation, and the queries finished by the exact per-thread search
 * after a frontier or candidate overflow. */
HEXOPT_API int hexopt_query_stats(hexopt_ctx *ctx, int64_t *warp_queries, int64_t *candidates, int64_t *fallbacks);
/* Per-thread traversal budget of the BVH queries: node pops a query may take alone before the
 * group-cooperative pass takes it over (0 = the defaults: 128 for the projection, 96 for the
 * Hausdorff sides).  Results do not depend on it. */
HEXOPT_API int hexopt_set_query_budget(hexopt_ctx *ctx, int pops);


/* ---- Hausdorff (metro_hausdorff.cpp:358-506): vertex-sampled, two-sided ---- */
HEXOPT_API int hexopt_hausdorff(hexopt_ctx *ctx, int64_t nv0, const double *V0, int64_t nf0, const int32_t *F0, int64_t nv1,
                     const double *V1, int64_t nf1, const int32_t *F1, double *diag, double *max_dist,
                     double *ave_dist);
/* The hex mesh's boundary surface of mesh m (extract_surface_conforming_mesh: boundary quads split
 * 0-1-2 / 2-3-0, global_functions.cpp:1021-1060) as nf triangles over the mesh's vertices. */
HEXOPT_API int hexopt_set_surface(hexopt_ctx *ctx, int mesh, int64_t nf, const int32_t *F);
/* Between each mesh's target and its boundary surface at the current positions (n_meshes each). */
HEXOPT_API int hexopt_hausdorff_meshes(hexopt_ctx *ctx, double *diag, double *max_dist, double *ave_dist);
/* One-sided distances of np host points to the triangles (V, F): min over faces of vcg's
 * PointDistanceEP (the sample distance of the uniform-area Hausdorff mode). */
HEXOPT_API int hexopt_point_face_distance(hexopt_ctx *ctx, int64_t np, const double *P, int64_t nv, const double *V, int64_t nf,
                               const int32_t *F, double *dist);

/* The same two-sided check over n_samples area-uniform random samples of each surface instead of
 * the vertices (the uniform-sample mode): samples drawn on the device from `seed` with SplitMix64
 * counters (surface 1 continuing after surface 0's 3 n_samples counters), face picked by
 * cumulative area, barycentric (1 - sqrt(u1), sqrt(u1)(1 - u2), sqrt(u1) u2); each sample's
 * distance is PointDistanceEP minimised over the other surface, with the vertex mode's rules --
 * upper bound = the inflated bbox diagonal, samples reaching it dropped, max over both sides,
 * ave = the larger mean.  samples0 / samples1 (n_samples x 3 each) receive the samples, or NULL. */
HEXOPT_API int hexopt_hausdorff_uniform(hexopt_ctx *ctx, int64_t nv0, const double *V0, int64_t nf0, const int32_t *F0,
                                        int64_t nv1, const double *V1, int64_t nf1, const int32_t *F1,
                                        int64_t n_samples, uint64_t seed, double *diag, double *max_dist,
                                        double *ave_dist, double *samples0, double *samples1);

/* ---- the optimiser iteration: one pass of feature_alignment's loop body ----
 * projection -> slim_precompute -> one SLIM iteration -> weight schedule -> scaled Jacobian
 * (-> Hausdorff when do_hausdorff).  lamda0 = feature_weight * MESHRATIO (0.05), upper bound 1e16. */
HEXOPT_API int hexopt_fa_begin(hexopt_ctx *ctx, const hexopt_slim_params *params, double lamda0, double hausdorff_ratio_t);
HEXOPT_API int hexopt_feature_alignment_step(hexopt_ctx *ctx, int do_hausdorff, hexopt_fa_report *rep);
/* The same step with the download of its result queued in the same call: V (nv x 3 float64, the
 * caller's vertex order, as hexopt_get_positions_async) receives the positions the step's line
 * search produced.  They are staged and copied on the download stream as soon as the line search
 * has applied its step, beside the step's scaled-Jacobian check and Hausdorff passes, instead of
 * after them; complete after hexopt_sync.  V must stay alive until then (page-locked memory lets
 * the copy overlap the computation). */
HEXOPT_API int hexopt_feature_alignment_step_get(hexopt_ctx *ctx, int do_hausdorff, hexopt_fa_report *rep, double *V);
/* Captures one step (without report download) in a CUDA graph and replays it.  on: 0 = off,
 * 1 = on (the line-search rounds become a conditional WHILE node), 2 = on with the rounds as
 * fixed launches (a graph whose kernel nodes a per-kernel profiler can capture). */
HEXOPT_API int hexopt_use_graph(hexopt_ctx *ctx, int on);

/* ---- adjoint of the total energy (symmetric Dirichlet over corner tets + soft terms) ----
 * With the operator frozen at the last precompute: E per mesh, and dE/dX (n x 3, all meshes). */
HEXOPT_API int hexopt_energy_fwd(hexopt_ctx *ctx, const double *X, double *E);
HEXOPT_API int hexopt_energy_bwd(hexopt_ctx *ctx, double *grad);

/* ---- launch tuning ---- */
/* kind 0: threads per hex block (32, 64, 128); 1: threads per vertex block (64, 128, 256);
 * 2: vertices per thread of the vertex kernels (1, 2, 4, 8, 16; default 8) */
HEXOPT_API int hexopt_set_block_size(hexopt_ctx *ctx, int kind, int threads);
/* Times one SLIM iteration per setting (hex block 64/128, vertex block 128/256, 4/8 vertices per
 * thread, 1/2/4 line-search candidates) on the live problem and keeps the fastest; positions and
 * solver state are restored.  Needs slim_precompute (or fa_begin) first. */
HEXOPT_API int hexopt_autotune(hexopt_ctx *ctx);
HEXOPT_API int hexopt_get_tuning(const hexopt_ctx *ctx, int *hex_block, int *vert_block, int *vert_items,
                                 int *ls_candidates);
/* CUDA-event timing on the context's stream: start records an event, stop records a second one,
 * synchronises and returns the elapsed milliseconds between them. */
HEXOPT_API int hexopt_timer_start(hexopt_ctx *ctx);
HEXOPT_API int hexopt_timer_stop(hexopt_ctx *ctx, double *ms);
/* Average device time of one launch of a stage, timed with CUDA events over `reps` back-to-back
 * launches on the current state (after slim_precompute / an iteration):
 *   0 element SpMV of the PCG   1 local step   2 line-search energy pass (ls_candidates steps)
 *   3 scaled-Jacobian check as the feature-alignment loop runs it (FP64 in plain mode; FP32
 *     screen with FP64 re-evaluation near the minimum in mixed mode)
 *   4 feature projection        5 one full SLIM iteration
 *   6 adjoint forward (energy at the last energy_fwd point)   7 adjoint backward (gradient)
 *   8 the vector side of one PCG iteration (soft-term product, step length, update, direction)
 *   9 one FP64 residual replacement of the mixed-mode PCG (no launch in plain mode)
 * Stages 0-2 and 8-9 leave the solver scratch in an unspecified state; positions are not
 * modified by 0-4 and 8-9 (stage 5 advances them like slim_iterate); 6-7 need one energy_fwd
 * and energy_bwd first. */
HEXOPT_API int hexopt_time_stage(hexopt_ctx *ctx, int stage, int reps, double *ms_per_launch);
/* Kernel launches issued by this context since creation (for the bench's launch count). */
HEXOPT_API int64_t hexopt_launch_count(const hexopt_ctx *ctx);

/* ---- no-allocation variant (no counterpart in the reference) ----
 * hexopt_point_face_distance on caller-owned DEVICE arrays -- P_dev (np x 3), V_dev (nv x 3),
 * F_dev (nf x 3 vertex ids), dist_dev (np) -- on CUDA device `device` and the caller's `stream`
 * (a cudaStream_t; NULL = the legacy default stream), with no device allocation: the triangle
 * soup, the LBVH, the sort workspace and the status word live in one static 80 MiB device array
 * per device.  For callers that must not allocate or free device memory: cudaFree synchronises
 * the whole device and stalls work on other streams, and a caller running under a fixed
 * device-memory budget (a pool that owns the rest of HBM) cannot have a library take memory.
 * No context is needed (creating one allocates).
 *   limit:     nf <= 262,144 faces; a larger surface returns HEXOPT_ERR_UNSUPPORTED with both
 *              sizes in the message (use hexopt_point_face_distance).  np is not limited.
 *   set-up:    the first call on a device resolves the static array's address, which loads it;
 *              when that happens lazily it must come before any stream capture on the device,
 *              so make one small call up front.  The call synchronises `stream` and is not
 *              itself meant to be captured.  Under CUDA_MODULE_LOADING=EAGER the 80 MiB are
 *              reserved on every device as soon as a context loads this library, called or not.
 *   races:     every call on a device shares that one array: calls overlapping in time (two
 *              streams, two host threads) race and give wrong results -- serialise them.
 *   zeroing:   the parts that must start at zero (BVH refit counters, status word) are cleared
 *              by the call itself on `stream`; nothing is assumed between calls.
 *   errors:    status as elsewhere; the message goes to err (err_len bytes, may be NULL). */
HEXOPT_API int hexopt_point_face_distance_noalloc(int device, void *stream, int64_t np, const double *P_dev, int64_t nv,
                                                  const double *V_dev, int64_t nf, const int32_t *F_dev,
                                                  double *dist_dev, char *err, size_t err_len);

/* ---- hex-mesh files in the reference's formats (host only, no device) ----
 * write: format 0 = MEDIT .mesh as h_io::write_hybrid_mesh_MESH (io.cpp:295-325), 1 = legacy
 * ASCII .vtk as h_io::write_hybrid_mesh_VTK (io.cpp:102-180) with the boundary flags (may be
 * NULL: all 0) as its "fixed" point data; numbers at iostream's default 6 significant digits.
 * read: the Vertices / Hexahedra blocks of a .mesh; call with V or H NULL (or *nv, *nh too small)
 * to get the sizes in *nv, *nh, then again with arrays of those sizes. */
HEXOPT_API int hexopt_write_hex_mesh(const char *path, int format, int64_t nv, const double *V, int64_t nh,
                                     const uint32_t *H, const uint8_t *boundary);
HEXOPT_API int hexopt_read_hex_mesh(const char *path, int64_t *nv, int64_t *nh, double *V, uint32_t *H);

/* ---- aabb.h value types (Ray / AABB, aabb.h:5-115) on the host ---- */
typedef struct hexopt_aabb { double min[3], max[3]; } hexopt_aabb;
typedef struct hexopt_ray { double o[3], d[3], dRcp[3]; double mint, maxt; } hexopt_ray;
HEXOPT_API void hexopt_aabb_merge(hexopt_aabb *a, const hexopt_aabb *b);
HEXOPT_API double hexopt_aabb_squared_distance(const hexopt_aabb *a, const double *p);
HEXOPT_API int hexopt_aabb_ray_intersect(const hexopt_aabb *a, const hexopt_ray *r, double *nearT, double *farT);
HEXOPT_API int hexopt_aabb_largest_axis(const hexopt_aabb *a);
HEXOPT_API double hexopt_aabb_surface_area(const hexopt_aabb *a);

#ifdef __cplusplus
}
#endif
#endif
