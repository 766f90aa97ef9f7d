// ref_harness.cpp -- C entry points over the reference's OWN code, used only to generate the
// golden fixtures that pin the oracle (tests/golden/make_golden.py).  Compiled together with
// the reference sources slim_m.cpp, optimization.cpp, global_functions.cpp, global_types.cpp
// and metro_hausdorff.cpp where they lie in the reference tree (oracle/Makefile); the output
// goes to oracle/_ref/, which is never committed.  TEST INFRASTRUCTURE ONLY.
#include "slim_m.h"
#include "optimization.h"
#include "global_functions.h"
#include "metro_hausdorff.h"
#include "igl/signed_distance.h"
#include "igl/per_face_normals.h"
#include "igl/per_vertex_normals.h"
#include "igl/per_edge_normals.h"
#include "igl/flip_avoiding_line_search.h"
#include "igl/grad.h"
#include <cstdint>
#include <vector>

// Internal to slim_m.cpp (non-static there): the per-tet energy sum.
double compute_energy_with_jacobians(SLIMData &s, const Eigen::MatrixXd &V, const Eigen::MatrixXi &F,
                                     const Eigen::MatrixXd &Ji, Eigen::MatrixXd &uv, Eigen::VectorXd &areas);
void compute_jacobians(SLIMData &s, const Eigen::MatrixXd &uv);

static Mesh make_hex_mesh(int64_t nv, const double *V, int64_t nh, const uint32_t *H) {
  Mesh m;
  m.type = Mesh_type::Hex;
  m.V.resize(3, nv);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) m.V(d, i) = V[3 * i + d];
  m.Hs.resize(nh);
  for (int64_t h = 0; h < nh; h++) {
    m.Hs[h].id = (uint32_t)h;
    m.Hs[h].vs.assign(H + 8 * h, H + 8 * h + 8);
  }
  return m;
}

static Mesh make_tri_mesh(int64_t nv, const double *V, int64_t nf, const int32_t *F) {
  Mesh m;
  m.type = Mesh_type::Tri;
  m.V.resize(3, nv);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) m.V(d, i) = V[3 * i + d];
  m.Fs.resize(nf);
  for (int64_t f = 0; f < nf; f++) {
    m.Fs[f].id = (uint32_t)f;
    m.Fs[f].vs = {(uint32_t)F[3 * f], (uint32_t)F[3 * f + 1], (uint32_t)F[3 * f + 2]};
  }
  return m;
}

extern "C" {

int ref_scaled_jacobian(int64_t nv, const double *V, int64_t nh, const uint32_t *H, double *V_Js, double *H_Js,
                        double *out4) {
  Mesh m = make_hex_mesh(nv, V, nh, H);
  Mesh_Quality mq;
  scaled_jacobian(m, mq);
  for (int64_t i = 0; i < 8 * nh; i++) V_Js[i] = mq.V_Js[i];
  for (int64_t i = 0; i < nh; i++) H_Js[i] = mq.H_Js[i];
  out4[0] = mq.min_Jacobian;
  out4[1] = mq.ave_Jacobian;
  out4[2] = mq.deviation_Jacobian;
  int64_t inv = 0;
  for (int64_t i = 0; i < nh; i++) inv += mq.H_Js[i] < 0;
  out4[3] = (double)inv;
  return 0;
}

// The reference shapes and the gradient operator of the 8 corner tets of each hex
// (compute_referenceMesh + igl::grad_ref), exported densely: Dg[t][j][c] = G(c*T + t, T(t,j)).
int ref_grad(int64_t nv, const double *V, int64_t nh, const uint32_t *H, const uint8_t *h_flag, int cube,
             double *RT_out, double *Dg) {
  Eigen::MatrixXd mV(nv, 3);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) mV(i, d) = V[3 * i + d];
  Mesh m = make_hex_mesh(nv, V, nh, H);
  std::vector<bool> hf(nh, true);
  if (h_flag)
    for (int64_t h = 0; h < nh; h++) hf[h] = h_flag[h] != 0;
  std::vector<uint32_t> Hids(nh);
  for (int64_t h = 0; h < nh; h++) Hids[h] = (uint32_t)h;
  std::vector<Eigen::MatrixXd> RT;
  compute_referenceMesh(mV, m.Hs, hf, Hids, RT, cube != 0);
  int64_t nt = 8 * nh;
  Eigen::MatrixXi T(nt, 4);
  for (int64_t h = 0; h < nh; h++)
    for (int k = 0; k < 8; k++)
      for (int j = 0; j < 4; j++) T(8 * h + k, j) = H[8 * h + hex_tetra_table[k][j]];
  Eigen::SparseMatrix<double> G;
  igl::grad_ref(mV, T, RT, G, true);
  Eigen::MatrixXd Gd = Eigen::MatrixXd(G);
  for (int64_t t = 0; t < nt; t++) {
    for (int j = 0; j < 4; j++)
      for (int d = 0; d < 3; d++) RT_out[(t * 4 + j) * 3 + d] = RT[t](j, d);
    for (int j = 0; j < 4; j++)
      for (int c = 0; c < 3; c++) Dg[(t * 4 + j) * 3 + c] = Gd(c * nt + t, T(t, j));
  }
  return 0;
}

// optimization::slim_m_opt(ts, iters, -1) on a Tetralize_Set built the way feature_alignment
// builds it (grid_hex_meshing.cpp:3783-3862).  out: energy, engery_quality, engery_soft.
int ref_slim_m_opt(int64_t nv, const double *V, int64_t nh, const uint32_t *H, const uint8_t *h_flag, int cube,
                   int energy_type, double weight_opt, int64_t nC, const int32_t *ids_C, const double *C,
                   double lamda_C, int64_t nT, const int32_t *ids_T, const double *normal_T, const double *dis_T,
                   double lamda_T, int64_t nL, const int32_t *ids_L, const double *Axa_L, const double *origin_L,
                   double lamda_L, int iters, double *V_o, double *out3) {
  Tetralize_Set ts;
  ts.V.resize(nv, 3);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) ts.V(i, d) = V[3 * i + d];
  ts.T.resize(8 * nh, 4);
  for (int64_t h = 0; h < nh; h++)
    for (int k = 0; k < 8; k++)
      for (int j = 0; j < 4; j++) ts.T(8 * h + k, j) = H[8 * h + hex_tetra_table[k][j]];
  Mesh m = make_hex_mesh(nv, V, nh, H);
  std::vector<bool> hf(nh, true);
  if (h_flag)
    for (int64_t h = 0; h < nh; h++) hf[h] = h_flag[h] != 0;
  std::vector<uint32_t> Hids(nh);
  for (int64_t h = 0; h < nh; h++) Hids[h] = (uint32_t)h;
  ts.b.resize(0);
  ts.bc.resize(0, 3);
  ts.regionb.resize(0);
  ts.regionbc.resize(0, 3);
  ts.energy_type = (SLIM_ENERGY)energy_type;
  ts.UV = ts.V;
  ts.projection = false;
  ts.global = true;
  ts.glue = false;
  ts.lamda_glue = 0;
  Feature_Constraints &fc = ts.fc;
  fc.ids_C.resize(nC);
  fc.C.resize(nC, 3);
  for (int64_t i = 0; i < nC; i++) {
    fc.ids_C[i] = ids_C[i];
    for (int d = 0; d < 3; d++) fc.C(i, d) = C[3 * i + d];
  }
  fc.ids_T.resize(nT);
  fc.normal_T.resize(nT, 3);
  fc.dis_T.resize(nT);
  for (int64_t i = 0; i < nT; i++) {
    fc.ids_T[i] = ids_T[i];
    fc.dis_T[i] = dis_T[i];
    for (int d = 0; d < 3; d++) fc.normal_T(i, d) = normal_T[3 * i + d];
  }
  fc.ids_L.resize(nL);
  fc.Axa_L.resize(nL, 3);
  fc.origin_L.resize(nL, 3);
  for (int64_t i = 0; i < nL; i++) {
    fc.ids_L[i] = ids_L[i];
    for (int d = 0; d < 3; d++) {
      fc.Axa_L(i, d) = Axa_L[3 * i + d];
      fc.origin_L(i, d) = origin_L[3 * i + d];
    }
  }
  fc.lamda_C = lamda_C;
  fc.lamda_T = lamda_T;
  fc.lamda_L = lamda_L;
  compute_referenceMesh(ts.UV, m.Hs, hf, Hids, ts.RT, cube != 0);
  optimization opt;
  opt.weight_opt = weight_opt;
  opt.slim_m_opt(ts, (uint32_t)iters, -1);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) V_o[3 * i + d] = ts.UV(i, d);
  out3[0] = opt.energy;
  out3[1] = opt.engery_quality;
  out3[2] = opt.engery_soft;
  return 0;
}

// optimization::pipeline2() for a hex mesh (optimization.cpp:416-434): rigidDeformCubes, then
// glueInternalNodes (per-hex vertex copies glued by the adaptive slim_solve2 branch with the
// boundary copies held at their positions, optimization.cpp:552-669).  The mesh's vertices carry
// their hex neighbourhoods and boundary flags as the mesher builds them.  V_out gets the glued
// positions (mean of each vertex's copies), out4 = {success, min_J, ave_J, opt.energy}.
int ref_pipeline2(int64_t nv, const double *V, int64_t nh, const uint32_t *H, const uint8_t *boundary,
                  double weight_opt, double *V_out, double *out4) {
  optimization opt;
  opt.weight_opt = weight_opt;
  Mesh &m = opt.mesh;
  m = make_hex_mesh(nv, V, nh, H);
  m.Vs.resize(nv);
  for (int64_t i = 0; i < nv; i++) {
    m.Vs[i].id = (uint32_t)i;
    m.Vs[i].v = {V[3 * i], V[3 * i + 1], V[3 * i + 2]};
    m.Vs[i].boundary = boundary[i] != 0;
  }
  for (int64_t h = 0; h < nh; h++)
    for (int c = 0; c < 8; c++) m.Vs[H[8 * h + c]].neighbor_hs.push_back((uint32_t)h);
  Eigen::MatrixXd BV(nv, 3);
  std::vector<Deform_V_Type> types(nv, Deform_V_Type::Free);
  for (int64_t i = 0; i < nv; i++) {
    for (int d = 0; d < 3; d++) BV(i, d) = V[3 * i + d];
    if (boundary[i]) types[i] = Deform_V_Type::Fixed;
  }
  opt.assign_constraints(BV, types);
  const bool ok = opt.pipeline2();
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) V_out[3 * i + d] = opt.mesh.V(d, i);
  out4[0] = ok ? 1.0 : 0.0;
  out4[1] = opt.mq.min_Jacobian;
  out4[2] = opt.mq.ave_Jacobian;
  out4[3] = opt.energy;
  return 0;
}

// optimization::slim_m_opt(ts, iters, -1) with the projection term on (ts.projection, ts.b /
// ts.bc, lamda_projection; add_soft_constraints slim_m.cpp:600-610) and no feature constraints.
int ref_slim_m_opt_proj(int64_t nv, const double *V, int64_t nh, const uint32_t *H, double weight_opt, int64_t nB,
                        const int32_t *b, const double *bc, double lamda_projection, int iters, double *V_o,
                        double *out3) {
  Tetralize_Set ts;
  ts.V.resize(nv, 3);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) ts.V(i, d) = V[3 * i + d];
  ts.T.resize(8 * nh, 4);
  for (int64_t h = 0; h < nh; h++)
    for (int k = 0; k < 8; k++)
      for (int j = 0; j < 4; j++) ts.T(8 * h + k, j) = H[8 * h + hex_tetra_table[k][j]];
  Mesh m = make_hex_mesh(nv, V, nh, H);
  std::vector<bool> hf(nh, true);
  std::vector<uint32_t> Hids(nh);
  for (int64_t h = 0; h < nh; h++) Hids[h] = (uint32_t)h;
  ts.b.resize(nB);
  ts.bc.resize(nB, 3);
  for (int64_t i = 0; i < nB; i++) {
    ts.b[i] = b[i];
    for (int d = 0; d < 3; d++) ts.bc(i, d) = bc[3 * i + d];
  }
  ts.regionb.resize(0);
  ts.regionbc.resize(0, 3);
  ts.energy_type = SYMMETRIC_DIRICHLET;
  ts.UV = ts.V;
  ts.projection = true;
  ts.lamda_projection = lamda_projection;
  ts.global = true;
  ts.glue = false;
  ts.lamda_glue = 0;
  ts.fc.lamda_C = ts.fc.lamda_T = ts.fc.lamda_L = 0;
  compute_referenceMesh(ts.UV, m.Hs, hf, Hids, ts.RT, true);
  optimization opt;
  opt.weight_opt = weight_opt;
  opt.slim_m_opt(ts, (uint32_t)iters, -1);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) V_o[3 * i + d] = ts.UV(i, d);
  out3[0] = opt.energy;
  out3[1] = opt.engery_quality;
  out3[2] = opt.engery_soft;
  return 0;
}

// The smoothing stage (grid_hex_meshing.cpp:2979-3056) on a hex mesh: `outer` rounds of
// compute_referenceMesh(ts.V, ..., cube = true) and optimization::slim_opt_igl(ts, inner)
// (optimization.cpp:970-1005, the modified igl::slim: M = weight_opt / 2), with the stage's empty
// feature constraints.  out3 = {igl energy / mesh_area of the last solve (printed), min_J, ave_J}.
int ref_smoothing(int64_t nv, const double *V, int64_t nh, const uint32_t *H, double weight_opt, int outer,
                  int inner, double *V_out, double *out3) {
  Mesh m = make_hex_mesh(nv, V, nh, H);
  Tetralize_Set ts;
  ts.V.resize(nv, 3);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) ts.V(i, d) = V[3 * i + d];
  ts.T.resize(8 * nh, 4);
  for (int64_t h = 0; h < nh; h++)
    for (int k = 0; k < 8; k++)
      for (int j = 0; j < 4; j++) ts.T(8 * h + k, j) = H[8 * h + hex_tetra_table[k][j]];
  Feature_Constraints fc;
  fc.lamda_C = fc.lamda_L = fc.lamda_T = 0;
  ts.energy_type = SYMMETRIC_DIRICHLET;
  ts.UV = ts.V;
  ts.fc = fc;
  ts.projection = false;
  ts.global = true;
  ts.glue = false;
  ts.lamda_glue = 0;
  ts.lamda_region = 0;
  ts.b.resize(0);
  ts.bc.resize(0, 3);
  ts.lamda_b = 0;
  optimization opt;
  opt.weight_opt = weight_opt;
  std::vector<bool> inout(nh, true);
  std::vector<uint32_t> Hids(nh);
  for (int64_t h = 0; h < nh; h++) Hids[h] = (uint32_t)h;
  for (int i = 0; i < outer; i++) {
    compute_referenceMesh(ts.V, m.Hs, inout, Hids, ts.RT, true);
    opt.slim_opt_igl(ts, (uint32_t)inner);
    m.V = ts.V.transpose();
  }
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) V_out[3 * i + d] = ts.V(i, d);
  Mesh_Quality mq;
  scaled_jacobian(m, mq);
  out3[0] = 0;
  out3[1] = mq.min_Jacobian;
  out3[2] = mq.ave_Jacobian;
  return 0;
}

// Per-tet energies at positions X with the operator of slim_precompute at V
// (compute_energy_with_jacobians), used to pin the per-element energy.
int ref_tet_energy(int64_t nv, const double *V, const double *X, int64_t nh, const uint32_t *H, int energy_type,
                   double weight_opt, double *E_tet) {
  Tetralize_Set ts;
  ts.V.resize(nv, 3);
  Eigen::MatrixXd mX(nv, 3);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) { ts.V(i, d) = V[3 * i + d]; mX(i, d) = X[3 * i + d]; }
  ts.T.resize(8 * nh, 4);
  for (int64_t h = 0; h < nh; h++)
    for (int k = 0; k < 8; k++)
      for (int j = 0; j < 4; j++) ts.T(8 * h + k, j) = H[8 * h + hex_tetra_table[k][j]];
  Mesh m = make_hex_mesh(nv, V, nh, H);
  std::vector<bool> hf(nh, true);
  std::vector<uint32_t> Hids(nh);
  for (int64_t h = 0; h < nh; h++) Hids[h] = (uint32_t)h;
  ts.UV = ts.V;
  ts.projection = false;
  ts.glue = false;
  ts.energy_type = (SLIM_ENERGY)energy_type;
  compute_referenceMesh(ts.UV, m.Hs, hf, Hids, ts.RT, true);
  SLIMData s;
  s.weight_opt = weight_opt;
  slim_precompute(ts.V, ts.T, ts.UV, s, ts.energy_type, ts);
  compute_jacobians(s, mX);
  Eigen::VectorXd one(1);
  SLIMData s1;  // only dim, f_n, slim_energy and exp_factor are read
  s1.dim = 3;
  s1.f_n = 1;
  s1.slim_energy = s.slim_energy;
  s1.exp_factor = s.exp_factor;
  for (int64_t t = 0; t < 8 * nh; t++) {
    Eigen::MatrixXd Ji = s.Ji.row(t);
    one(0) = s.M(t);
    E_tet[t] = compute_energy_with_jacobians(s1, s.V, s.F, Ji, mX, one);
  }
  return 0;
}

int ref_max_step(int64_t nv, const double *X, const double *Dir, int64_t nh, const uint32_t *H, double *out) {
  Eigen::MatrixXd mX(nv, 3), mD(nv, 3);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) { mX(i, d) = X[3 * i + d]; mD(i, d) = Dir[3 * i + d]; }
  Eigen::MatrixXi T(8 * nh, 4);
  for (int64_t h = 0; h < nh; h++)
    for (int k = 0; k < 8; k++)
      for (int j = 0; j < 4; j++) T(8 * h + k, j) = H[8 * h + hex_tetra_table[k][j]];
  *out = igl::flip_avoiding::compute_max_step_from_singularities(mX, T, mD);
  return 0;
}

// build_aabb_tree (grid_hex_meshing.cpp:4231-4248) + signed_distance_pseudonormal.
int ref_signed_distance(int64_t nv, const double *TV, int64_t nf, const int32_t *TF, int64_t np, const double *P,
                        double *S, int32_t *I, double *C, double *N) {
  Eigen::MatrixXd V(nv, 3), Pm(np, 3);
  Eigen::MatrixXi F(nf, 3);
  for (int64_t i = 0; i < nv; i++)
    for (int d = 0; d < 3; d++) V(i, d) = TV[3 * i + d];
  for (int64_t f = 0; f < nf; f++)
    for (int d = 0; d < 3; d++) F(f, d) = TF[3 * f + d];
  for (int64_t i = 0; i < np; i++)
    for (int d = 0; d < 3; d++) Pm(i, d) = P[3 * i + d];
  igl::AABB<Eigen::MatrixXd, 3> tree;
  tree.init(V, F);
  Eigen::MatrixXd FN, VN, EN;
  Eigen::MatrixXi E;
  Eigen::VectorXi EMAP;
  igl::per_face_normals(V, F, FN);
  igl::per_vertex_normals(V, F, igl::PER_VERTEX_NORMALS_WEIGHTING_TYPE_ANGLE, FN, VN);
  igl::per_edge_normals(V, F, igl::PER_EDGE_NORMALS_WEIGHTING_TYPE_UNIFORM, FN, EN, E, EMAP);
  Eigen::VectorXd Sv;
  Eigen::VectorXi Iv;
  Eigen::MatrixXd Cv, Nv;
  igl::signed_distance_pseudonormal(Pm, V, F, tree, FN, VN, EN, EMAP, Sv, Iv, Cv, Nv);
  for (int64_t i = 0; i < np; i++) {
    S[i] = Sv(i);
    I[i] = Iv(i);
    for (int d = 0; d < 3; d++) { C[3 * i + d] = Cv(i, d); N[3 * i + d] = Nv(i, d); }
  }
  return 0;
}

// compute(const Mesh&, const Mesh&, diag, max, ave) (metro_hausdorff.cpp:358-506)
int ref_hausdorff(int64_t nv0, const double *V0, int64_t nf0, const int32_t *F0, int64_t nv1, const double *V1,
                  int64_t nf1, const int32_t *F1, double *out3) {
  const Mesh m0 = make_tri_mesh(nv0, V0, nf0, F0);
  const Mesh m1 = make_tri_mesh(nv1, V1, nf1, F1);
  double diag, mx, ave;
  compute(m0, m1, diag, mx, ave);
  out3[0] = diag;
  out3[1] = mx;
  out3[2] = ave;
  return 0;
}

}  // extern "C"
