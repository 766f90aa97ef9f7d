/*
 * hexopt_oracle.h -- CPU restatement of the reference's FP64 geometric-optimisation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA path and the
 * timed CPU baseline ("port") of bench.py.  Nothing in the product links it, and the product
 * never falls back to it.  It is pinned against outputs of the reference's own code (built
 * from its sources into oracle/_ref by oracle/Makefile) through the fixtures in tests/golden.
 *
 * Every routine cites the reference function it restates (path inside the reference
 * project, file:line).  All arithmetic is IEEE double, compiled with -ffp-contract=off so
 * x86-64 and aarch64 hosts produce identical bits.
 *
 * Conventions: vertex arrays are row-major (n x 3, xyz interleaved); hexes are 8 uint32
 * corner ids in the reference's corner order; tets are the 8 corner tets of each hex taken
 * from hex_tetra_table (tet id = 8*hex + corner).
 */
#ifndef HEXOPT_ORACLE_H
#define HEXOPT_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* SLIM_ENERGY (global_types.h:58-66) */
enum { ORC_ARAP = 0, ORC_LOG_ARAP, ORC_SYMMETRIC_DIRICHLET, ORC_CONFORMAL, ORC_EXP_CONFORMAL,
       ORC_EXP_SYMMETRIC_DIRICHLET };

/* scaled_jacobian for hex meshes (global_functions.cpp:2309-2356, a_jacobian :2422-2442).
 * V_Js (8*nh) and H_Js (nh) may be NULL. */
void orc_scaled_jacobian(int64_t nv, const double *V, int64_t nh, const uint32_t *H,
                         double *V_Js, double *H_Js, double *min_J, double *ave_J,
                         double *dev_J, int64_t *n_inverted);

/* Per-tet reference shapes: compute_referenceMesh + hex2cuboid_ + hex2tet24
 * (global_functions.cpp:3735-3806, 3994-4022).  RT: (8*nh) x 4 x 3. h_flag NULL = all true. */
void orc_reference_mesh(const double *V, int64_t nh, const uint32_t *H, const uint8_t *h_flag,
                        int cube, double *RT);

/* grad_tet_ref (extern/libigl/include/igl/grad.cpp:372-478) for the 8 corner tets of each
 * hex: per tet, the gradient 3-vector of each of its 4 vertices' hat functions.
 * Dg: (8*nh) x 4 x 3. */
void orc_grad_ref(const double *V, int64_t nh, const uint32_t *H, const double *RT, double *Dg);

typedef struct orc_slim_problem {
  int64_t nv, nh;
  const double *V;          /* nv x 3 positions used for the reference shapes and grad_ref */
  const double *UV;         /* nv x 3 starting positions (V_o) */
  const uint32_t *H;        /* nh x 8 */
  const uint8_t *h_flag;    /* nh; NULL = every hex targets a cube */
  int cube;                 /* compute_referenceMesh 'cube' argument */
  int energy;               /* SLIM_ENERGY */
  double weight_opt;        /* SLIMData::weight_opt */
  double exp_factor;        /* SLIMData::exp_factor */
  /* Feature_Constraints (global_types.h:583-610) */
  int64_t nC; const int32_t *ids_C; const double *C; double lamda_C;
  int64_t nT; const int32_t *ids_T; const double *normal_T; const double *dis_T; double lamda_T;
  int64_t nL; const int32_t *ids_L; const double *Axa_L; const double *origin_L; double lamda_L;
  /* Tetralize_Set::projection branch */
  int projection; int64_t nB; const int32_t *b; const double *bc; double lamda_projection;
} orc_slim_problem;

typedef struct orc_slim_result {
  double energy;          /* SLIMData::energy (divided by mesh_area) */
  double energy_quality;  /* SLIMData::engery_quality of the last energy evaluation */
  double energy_soft;     /* SLIMData::engery_soft of the last energy evaluation */
  int cg_iters;           /* CG iterations of the last solve */
  double cg_error;        /* CG relative residual estimate of the last solve */
  double max_step;        /* flip-avoiding step bound of the last line search */
  double step;            /* accepted step of the last line search */
  int halvings;           /* line-search halvings of the last iteration */
} orc_slim_result;

/* optimization::slim_m_opt (optimization.cpp:883-900) with a fixed iteration count:
 * slim_precompute (slim_m.cpp:1095-1132) then slim_solve2's fixed-N branch
 * (slim_m.cpp:1269-1288).  V_o: nv x 3 out; a_L: nL out (may be NULL when nL == 0).
 * Returns 0 on success. */
int orc_slim_m_opt(const orc_slim_problem *p, int iters, double *V_o, double *a_L,
                   orc_slim_result *res);

/* Energy of positions X with curve parameters a_L (compute_energy_total, slim_m.cpp:716-733),
 * with the gradient operator frozen at p->V.  Per-tet energies (already multiplied by M) go to
 * E_tet when non-NULL.  Returns the undivided total; *eq / *es get the two parts. */
double orc_slim_energy(const orc_slim_problem *p, const double *X, const double *a_L,
                       double *E_tet, double *eq, double *es);

/* Gradient of orc_slim_energy w.r.t. X (nv x 3) with the operator frozen (adjoint oracle,
 * symmetric Dirichlet only). */
void orc_slim_energy_grad(const orc_slim_problem *p, const double *X, const double *a_L,
                          double *G);

/* flip_avoiding::compute_max_step_from_singularities over the corner tets
 * (extern/libigl/include/igl/flip_avoiding_line_search.cpp:273-298). */
double orc_max_step(int64_t nv, const double *X, const double *Dir, int64_t nh, const uint32_t *H);

/* --- closest point / pseudonormal projection (libigl signed_distance_pseudonormal) --- */
typedef struct orc_tree orc_tree;
/* build_aabb_tree (grid_hex_meshing.cpp:4231-4248): AABB + face/vertex/edge normals. */
orc_tree *orc_tree_build(int64_t nv, const double *TV, int64_t nf, const int32_t *TF);
void orc_tree_free(orc_tree *t);
/* signed_distance_pseudonormal (extern/libigl/include/igl/signed_distance.cpp:186-257):
 * S signed distance, I face id, C closest point, N pseudonormal. */
void orc_signed_distance(const orc_tree *t, int64_t np, const double *P, double *S, int32_t *I,
                         double *C, double *N);
/* point_line_projection (global_functions.cpp:3454-3465) */
void orc_point_line_projection(const double *v1, const double *v2, const double *v, double *pv,
                               double *t);

/* LINE branch of dirty_graph_projection (grid_hex_meshing.cpp:3963-4025): per line vertex
 * lines[i] of X (nv x 3), the closest point on its curve line_curve[i] (curves as chains of TV
 * vertices, curve_ptr / curve_vs, closed flags) -> origin (nl x 3) and the segment's unit
 * tangent -> axis (nl x 3). */
void orc_curve_targets(int64_t nl, const double *X, const int32_t *lines, const int32_t *line_curve,
                       const double *TV, const int64_t *curve_ptr, const int32_t *curve_vs,
                       const uint8_t *closed, double *origin, double *axis);

/* --- Hausdorff (metro_hausdorff.cpp:358-506, vcg sampling.h:224-289, 547-603) --- */
void orc_hausdorff(int64_t nv0, const double *V0, int64_t nf0, const int32_t *F0,
                   int64_t nv1, const double *V1, int64_t nf1, const int32_t *F1,
                   double *bbox_diag, double *max_dist, double *ave_dist);
/* One-sided sampled distance: for each sample point, min over faces of vcg's PointDistanceEP
 * (no upper bound).  dist: ns out. */
void orc_point_face_distance(int64_t ns, const double *P, int64_t nv, const double *V, int64_t nf,
                             const int32_t *F, double *dist);

#ifdef __cplusplus
}
#endif
#endif
