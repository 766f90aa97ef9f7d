// hexopt_reference_shim.cpp -- the reference's own hot-path entry points, with their exact C++
// signatures, implemented over libhexopt_gpu.so's C ABI.
//
// Built inside the reference's tree (its headers on the include path) in place of:
//   slim_m.cpp              slim_precompute (both overloads), slim_solve, slim_solve2   slim_m.h:89-114
//   metro_hausdorff.cpp     the three compute() overloads                             metro_hausdorff.h:35-37
//   global_functions.cpp    scaled_jacobian(Mesh&, Mesh_Quality&)                     global_functions.h:81
//                           (only that one definition; compiled in when HEXOPT_SHIM_SCALED_JACOBIAN
//                           is defined, after the CPU definition is removed from that file)
// so that optimization::slim_m_opt (optimization.cpp:883-900), feature_alignment
// (grid_hex_meshing.cpp:3783-3912), stop_criterior_satisfied and hausdorff_ratio_check
// (:4148-4327) compile and link unchanged and run their optimiser iterations on the GPU.
//
// Scope: every SLIM form the reference's callers use -- the six SLIM energies over the 8 corner
// tets of each hex (F holds 8 tets per hex in hex_tetra_table order), whatever reference tets
// ts.RT holds, corner / tangent-plane / feature-line soft constraints, the projection and glue
// terms, known_value_post, fixed iteration counts and the adaptive (iter_num = -1) branches of
// slim_solve2 and slim_solve; with HEXOPT_SHIM_SLIM_OPT_IGL, optimization::slim_opt_igl (the
// modified igl::slim of the smoothing stage).  The conversions themselves are in
// hexopt_shim_core.h.  Forms no reference caller reaches (region terms, the 2-D quad path, the
// modified igl::slim's glue groups) throw std::runtime_error naming the form: there is no CPU
// fallback behind this file.
//
// Environment: HEXOPT_DEVICE (CUDA device, default 0); HEXOPT_PRECISION=mixed selects the
// FP32/FP64 mixed mode (default: plain FP64, the reference's arithmetic).
#include "slim_m.h"
#include "metro_hausdorff.h"
#include "global_functions.h"

#include "hexopt_gpu.h"
#include "hexopt_shim_core.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

namespace hexopt_shim {

// One context for the SLIM state (the mesh of the last slim_precompute) and one for the
// stateless calls (quality, Hausdorff), so a quality check between precompute and solve does
// not evict the solver's mesh.
struct Contexts {
  hexopt_ctx *slim = nullptr, *aux = nullptr;
  const SLIMData *loaded = nullptr;  // SLIMData whose mesh the slim context holds
  ~Contexts() {
    if (slim) hexopt_destroy(slim);
    if (aux) hexopt_destroy(aux);
  }
};

static Contexts &contexts() {
  static Contexts c;
  return c;
}

static int device() {
  const char *d = std::getenv("HEXOPT_DEVICE");
  return d ? std::atoi(d) : 0;
}

static int precision() {
  const char *p = std::getenv("HEXOPT_PRECISION");
  return (p && std::strcmp(p, "mixed") == 0) ? HEXOPT_MIXED : HEXOPT_FP64;
}

static void ck(hexopt_ctx *c, int rc, const char *what) {
  if (rc == HEXOPT_OK) return;
  std::string msg = std::string("hexopt ") + what + " failed (status " + std::to_string(rc) + ")";
  if (c) msg += std::string(": ") + hexopt_last_error(c);
  throw std::runtime_error(msg);
}

static hexopt_ctx *get(hexopt_ctx *&slot) {
  if (!slot) ck(nullptr, hexopt_create(&slot, device()), "create");
  return slot;
}

[[noreturn]] static void unsupported(const std::string &what) {
  throw std::runtime_error("hexopt GPU path: " + what + " is outside the GPU hot path");
}

// Eigen matrices -> row-major host arrays of the C ABI.
static std::vector<double> rows3(const Eigen::MatrixXd &M) {
  std::vector<double> out(3 * (size_t)M.rows());
  for (int64_t i = 0; i < M.rows(); i++)
    for (int d = 0; d < 3; d++) out[3 * i + d] = M(i, d);
  return out;
}

static std::vector<int32_t> ids(const Eigen::VectorXi &v) {
  return std::vector<int32_t>(v.data(), v.data() + v.size());
}

static std::vector<int32_t> tets_rows(const Eigen::MatrixXi &F) {
  if (F.cols() != 4) unsupported("a tet list whose rows are not 4 vertices");
  std::vector<int32_t> T(4 * (size_t)F.rows());
  for (int64_t i = 0; i < F.rows(); i++)
    for (int k = 0; k < 4; k++) T[4 * i + k] = F(i, k);
  return T;
}

static std::vector<double> rt_rows(const std::vector<Eigen::MatrixXd> &RT, int64_t ntets) {
  std::vector<double> out;
  if (RT.empty()) return out;
  if ((int64_t)RT.size() != ntets) unsupported("reference tets whose count differs from the tets'");
  out.resize(12 * (size_t)ntets);
  for (int64_t t = 0; t < ntets; t++) {
    if (RT[t].rows() != 4 || RT[t].cols() != 3) unsupported("reference tets that are not 4 x 3");
    for (int j = 0; j < 4; j++)
      for (int d = 0; d < 3; d++) out[12 * t + 3 * j + d] = RT[t](j, d);
  }
  return out;
}

// Uploads data's mesh, constraints and weights into the SLIM context and runs the precompute
// (hexopt_shim_core::load_slim on the plain arrays of data and data.ts).
static void load(SLIMData &data) {
  Contexts &C = contexts();
  hexopt_ctx *c = get(C.slim);
  const Tetralize_Set &ts = data.ts;
  if (ts.regionb.size() > 0 && ts.lamda_region != 0) unsupported("region constraints");
  C.loaded = nullptr;
  const std::vector<int32_t> T = tets_rows(data.F);
  const std::vector<double> RT = rt_rows(ts.RT, data.F.rows());
  const std::vector<double> V = rows3(data.V);
  const std::vector<double> Vo = data.V_o.rows() == data.V.rows() ? rows3(data.V_o) : V;
  const Feature_Constraints &fc = ts.fc;
  const std::vector<int32_t> iC = ids(fc.ids_C), iT = ids(fc.ids_T), iL = ids(fc.ids_L), ib = ids(data.b);
  const std::vector<double> Cp = fc.ids_C.size() ? rows3(fc.C) : std::vector<double>();
  const std::vector<double> Tn = fc.ids_T.size() ? rows3(fc.normal_T) : std::vector<double>();
  const std::vector<double> Ta(fc.dis_T.data(), fc.dis_T.data() + fc.ids_T.size());
  const std::vector<double> La = fc.ids_L.size() ? rows3(fc.Axa_L) : std::vector<double>();
  const std::vector<double> Lo = fc.ids_L.size() ? rows3(fc.origin_L) : std::vector<double>();
  const std::vector<double> bc = data.b.size() ? rows3(data.bc) : std::vector<double>();
  std::vector<double> post;
  if (ts.known_value_post) post = rows3(ts.post_Variables);
  hexopt_shim_core::SlimSetup st;
  st.nv = data.V.rows();
  st.V = V.data();
  st.V_o = Vo.data();
  st.ntets = data.F.rows();
  st.T = T.data();
  st.RT = RT.empty() ? nullptr : RT.data();
  st.energy = (int)data.slim_energy;
  st.precision = precision();
  st.weight_opt = data.weight_opt;
  st.nC = (int64_t)iC.size(); st.ids_C = iC.data(); st.C = Cp.data(); st.lamda_C = fc.lamda_C;
  st.nT = (int64_t)iT.size(); st.ids_T = iT.data(); st.normal_T = Tn.data(); st.dis_T = Ta.data(); st.lamda_T = fc.lamda_T;
  st.nL = (int64_t)iL.size(); st.ids_L = iL.data(); st.Axa_L = La.data(); st.origin_L = Lo.data(); st.lamda_L = fc.lamda_L;
  st.projection = ts.projection;
  st.nB = (int64_t)ib.size(); st.b = ib.data(); st.bc = bc.data(); st.lamda_projection = ts.lamda_projection;
  st.glue = ts.glue;
  st.n_ranges = (int64_t)ts.V_ranges.size(); st.V_ranges = ts.V_ranges.data(); st.lamda_glue = ts.lamda_glue;
  st.known_value_post = ts.known_value_post;
  st.post_index = ts.post_index;
  st.post_Variables = post.empty() ? nullptr : post.data();
  std::string err;
  const int rc = hexopt_shim_core::load_slim(c, st, err);
  if (rc == HEXOPT_ERR_UNSUPPORTED) unsupported(err);
  if (rc != HEXOPT_OK) throw std::runtime_error("hexopt " + err);
  C.loaded = &data;
}

// The positions (and curve parameters) of the SLIM context back into data.V_o / data.a_L.
static void download(SLIMData &data) {
  hexopt_ctx *c = contexts().slim;
  std::vector<double> X(3 * (size_t)data.V_o.rows());
  ck(c, hexopt_get_positions(c, X.data()), "get_positions");
  for (int64_t i = 0; i < data.V_o.rows(); i++)
    for (int d = 0; d < 3; d++) data.V_o(i, d) = X[3 * i + d];
  if (data.a_L.size() > 0) ck(c, hexopt_get_curve_params(c, data.a_L.data()), "get_curve_params");
}

}  // namespace hexopt_shim

using namespace hexopt_shim;

// slim_m.cpp:1095-1132: the reference's bookkeeping, then the GPU precompute and the initial
// energy (compute_energy_total / mesh_area).
void slim_precompute(Eigen::MatrixXd &V, Eigen::MatrixXi &F, Eigen::MatrixXd &V_init, SLIMData &data,
                     SLIM_ENERGY slim_energy, Tetralize_Set ts) {
  data.V = V;
  data.F = F;
  data.V_o = V_init;
  data.v_num = V.rows();
  data.f_num = F.rows();
  data.slim_energy = slim_energy;
  data.ts = ts;
  data.b = ts.b;
  data.bc = ts.bc;
  data.a_L.resize(ts.fc.ids_L.rows());
  data.a_L.setZero();
  data.proximal_p = 0.00001 * data.weight_opt;
  data.M.resize(F.rows());
  data.M.setConstant(data.weight_opt);
  data.mesh_area = data.M.sum();
  data.mesh_improvement_3d = ts.global;
  data.exp_factor = 1.0;
  data.dim = 3;
  load(data);
  // data.energy: the start value of the first line search, which recomputes it anyway; the
  // library's energy_fwd evaluates the symmetric Dirichlet energy
  if (slim_energy == SYMMETRIC_DIRICHLET && !ts.glue && !ts.projection && !ts.known_value_post) {
    hexopt_ctx *c = contexts().slim;
    const std::vector<double> X = rows3(data.V_o);
    double E = 0;
    ck(c, hexopt_energy_fwd(c, X.data(), &E), "energy_fwd");
    data.energy = E / data.mesh_area;
  }
}

// The 18-argument overload (slim_m.h:89-100) feeds the projection / region path of slim_opt.
void slim_precompute(Eigen::MatrixXd &, Eigen::MatrixXi &, Eigen::MatrixXd &, SLIMData &, SLIM_ENERGY,
                     Eigen::VectorXi &, Eigen::MatrixXd &, Eigen::VectorXi &, Eigen::MatrixXd &, Eigen::VectorXi &,
                     Eigen::MatrixXd &, Eigen::MatrixXd &, Eigen::VectorXi &, Eigen::MatrixXd &, Eigen::VectorXd &,
                     Eigen::VectorXi &, Eigen::MatrixXd &, bool, bool) {
  unsupported("slim_precompute with explicit projection / region arguments");
}

// The iter_num = -1 branch of slim_solve2 (schedule 2) / slim_solve (schedule 1): SLIM iterations
// until the result mesh (glue groups at their means, or projection points at bc) has a positive
// minimum scaled Jacobian, at most 50, with the glue weight schedules, printing as the reference.
static Eigen::MatrixXd adaptive(SLIMData &data, int type, int schedule, bool verbose) {
  hexopt_ctx *c = contexts().slim;
  hexopt_adaptive_report rep;
  std::memset(&rep, 0, sizeof rep);
  ck(c, hexopt_slim_solve_adaptive(c, type, schedule, 50, &rep), "slim_solve_adaptive");
  data.energy = rep.energy;
  data.engery_quality = rep.energy_quality;
  data.engery_soft = rep.energy_soft;
  data.ts.lamda_glue = rep.lamda_glue;
  if (verbose) {
    if (!rep.converged) std::cout << "min J " << rep.min_Jacobian << "; ave J " << rep.ave_Jacobian << std::endl;
    std::cout << "iterations taken " << rep.iterations << std::endl;
  }
  download(data);
  return data.V_o;
}

// slim_m.cpp:1189-1291: the fixed-count branch (:1269-1288) prints the energy after each
// iteration as the reference does; iter_num = -1 runs the adaptive branch (:1191-1268).
Eigen::MatrixXd slim_solve2(SLIMData &data, int iter_num, int type, bool verbose) {
  Contexts &C = contexts();
  if (C.loaded != &data) load(data);
  if (iter_num < 0) return adaptive(data, type, 2, verbose);
  hexopt_ctx *c = C.slim;
  hexopt_slim_report rep;
  std::memset(&rep, 0, sizeof rep);
  for (int i = 0; i < iter_num; i++) {
    ck(c, hexopt_slim_iterate(c, 1, &rep), "slim_iterate");
    data.energy = rep.energy;
    std::cout << "energy at iter: " << i << " :" << data.energy << std::endl;
  }
  if (iter_num > 0) {
    data.engery_quality = rep.energy_quality;
    data.engery_soft = rep.energy_soft;
  }
  download(data);
  return data.V_o;
}

// slim_m.cpp:1293-1394: as slim_solve2, with slim_solve's glue weight doubling in the adaptive
// branch (:1311-1312).
Eigen::MatrixXd slim_solve(SLIMData &data, int iter_num, int type, bool verbose) {
  Contexts &C = contexts();
  if (C.loaded != &data) load(data);
  if (iter_num < 0) return adaptive(data, type, 1, verbose);
  return slim_solve2(data, iter_num, type, verbose);
}

// metro_hausdorff.cpp:358-506: vertex-sampled two-sided Hausdorff between two triangle meshes
// (Mesh::V is 3 x n column-major, i.e. row-major n x 3).
static void tri_faces(const Mesh &m, std::vector<int32_t> &F) {
  F.resize(3 * m.Fs.size());
  for (size_t i = 0; i < m.Fs.size(); i++)
    for (int k = 0; k < 3; k++) F[3 * i + k] = (int32_t)m.Fs[i].vs[k];
}

void compute(const Mesh &mesh0, const Mesh &mesh1, double &bbox_diagonal, double &max_hausdorff_dis,
             double &ave_hausdorff_dis) {
  hexopt_ctx *c = get(contexts().aux);
  std::vector<int32_t> F0, F1;
  tri_faces(mesh0, F0);
  tri_faces(mesh1, F1);
  ck(c, hexopt_hausdorff(c, mesh0.V.cols(), mesh0.V.data(), (int64_t)mesh0.Fs.size(), F0.data(), mesh1.V.cols(),
                         mesh1.V.data(), (int64_t)mesh1.Fs.size(), F1.data(), &bbox_diagonal, &max_hausdorff_dis,
                         &ave_hausdorff_dis),
     "hausdorff");
}

// metro_hausdorff.cpp:12-195: ratio = (float)max / inflated-bbox diagonal; 0 over the threshold.
int compute(Mesh &mesh0, Mesh &mesh1, double &hausdorff_ratio, double &hausdorff_ratio_threshold) {
  double diag = 0, mx = 0, ave = 0;
  compute(static_cast<const Mesh &>(mesh0), static_cast<const Mesh &>(mesh1), diag, mx, ave);
  hausdorff_ratio = (float)mx / diag;
  printf("%f  wrt bounding box diagonal\n", hausdorff_ratio);
  if (hausdorff_ratio > hausdorff_ratio_threshold) return false;
  return true;
}

// metro_hausdorff.cpp:196-357: as above, also the distance threshold and the mean ratio line.
int compute(Mesh &mesh0, Mesh &mesh1, double &hausdorff_ratio, double &hausdorff_ratio_threshold,
            double &hausdorff_dis_threshold) {
  double diag = 0, mx = 0, ave = 0;
  compute(static_cast<const Mesh &>(mesh0), static_cast<const Mesh &>(mesh1), diag, mx, ave);
  hausdorff_ratio = (float)mx / diag;
  hausdorff_dis_threshold = hausdorff_ratio_threshold * diag;
  printf("%f  wrt bounding box diagonal\n", hausdorff_ratio);
  printf("%f  average wrt bounding box diagonal\n", ave / diag);
  if (hausdorff_ratio > hausdorff_ratio_threshold) return false;
  return true;
}

#ifdef HEXOPT_SHIM_SCALED_JACOBIAN
// global_functions.cpp:2309-2356 (hex branch): per-corner scaled Jacobians V_Js, per-hex minima
// H_Js, mean, variance and minimum, and the flipped-element count line.
bool scaled_jacobian(Mesh &hmi, Mesh_Quality &mq) {
  if (hmi.type != Mesh_type::Hex) unsupported("scaled_jacobian of a non-hex mesh");
  hexopt_ctx *c = get(contexts().aux);
  const int64_t nv = hmi.V.cols(), nh = (int64_t)hmi.Hs.size();
  std::vector<uint32_t> H(8 * (size_t)nh);
  for (int64_t i = 0; i < nh; i++)
    for (int j = 0; j < 8; j++) H[8 * i + j] = hmi.Hs[i].vs[j];
  ck(c, hexopt_upload_meshes(c, 1, &nv, &nh, hmi.V.data(), H.data(), nullptr), "upload_meshes");
  mq.V_Js.resize(nh * 8);
  mq.H_Js.resize(nh);
  hexopt_quality q;
  ck(c, hexopt_scaled_jacobian(c, mq.V_Js.data(), mq.H_Js.data(), &q), "scaled_jacobian");
  mq.min_Jacobian = q.min_Jacobian;
  mq.ave_Jacobian = q.ave_Jacobian;
  mq.deviation_Jacobian = q.deviation_Jacobian;
  if (q.n_inverted > 0) std::cout << "flipped elements: " << q.n_inverted << std::endl;
  return true;
}
#endif

#ifdef HEXOPT_SHIM_SLIM_OPT_IGL
#include "optimization.h"
// optimization::slim_opt_igl (optimization.cpp:970-1005) -- the modified igl::slim of the
// smoothing stage (extern/libigl/include/igl/slim.cpp:1190-1288: M = weight_opt / 2, symmetric
// Dirichlet) -- compiled in when that definition is removed from optimization.cpp.  The stage's
// feature constraints are honoured; the igl variant's b / bc, region and Vgroups terms, which
// the smoothing stage leaves empty, are rejected.
void optimization::slim_opt_igl(Tetralize_Set &ts, const uint32_t iter) {
  if (ts.projection || ts.b.size() > 0 || (ts.regionb.size() > 0 && ts.lamda_region != 0) || !ts.Vgroups.empty())
    unsupported("the modified igl::slim's b / region / Vgroups terms");
  hexopt_ctx *c = get(contexts().slim);
  contexts().loaded = nullptr;
  const std::vector<int32_t> T = tets_rows(ts.T);
  const std::vector<double> RT = rt_rows(ts.RT, ts.T.rows());
  const std::vector<double> V = rows3(ts.V);
  const Feature_Constraints &fc = ts.fc;
  const std::vector<int32_t> iC = ids(fc.ids_C), iT = ids(fc.ids_T), iL = ids(fc.ids_L);
  const std::vector<double> Cp = fc.ids_C.size() ? rows3(fc.C) : std::vector<double>();
  const std::vector<double> Tn = fc.ids_T.size() ? rows3(fc.normal_T) : std::vector<double>();
  const std::vector<double> Ta(fc.dis_T.data(), fc.dis_T.data() + fc.ids_T.size());
  const std::vector<double> La = fc.ids_L.size() ? rows3(fc.Axa_L) : std::vector<double>();
  const std::vector<double> Lo = fc.ids_L.size() ? rows3(fc.origin_L) : std::vector<double>();
  hexopt_shim_core::SlimSetup st;
  st.nv = ts.V.rows();
  st.V = V.data();
  st.V_o = V.data();
  st.ntets = ts.T.rows();
  st.T = T.data();
  st.RT = RT.empty() ? nullptr : RT.data();
  st.energy = HEXOPT_SYMMETRIC_DIRICHLET;
  st.precision = precision();
  st.weight_opt = weight_opt;
  st.variant = 1;
  st.nC = (int64_t)iC.size(); st.ids_C = iC.data(); st.C = Cp.data(); st.lamda_C = fc.lamda_C;
  st.nT = (int64_t)iT.size(); st.ids_T = iT.data(); st.normal_T = Tn.data(); st.dis_T = Ta.data(); st.lamda_T = fc.lamda_T;
  st.nL = (int64_t)iL.size(); st.ids_L = iL.data(); st.Axa_L = La.data(); st.origin_L = Lo.data(); st.lamda_L = fc.lamda_L;
  std::string err;
  const int rc = hexopt_shim_core::load_slim(c, st, err);
  if (rc == HEXOPT_ERR_UNSUPPORTED) unsupported(err);
  if (rc != HEXOPT_OK) throw std::runtime_error("hexopt " + err);
  hexopt_slim_report rep;
  std::memset(&rep, 0, sizeof rep);
  for (uint32_t i = 0; i < iter; i++) {
    ck(c, hexopt_slim_iterate(c, 1, &rep), "slim_iterate");
    std::cout << "energy: " << rep.energy << std::endl;  // igl/slim.cpp:1281
  }
  std::vector<double> X(3 * (size_t)ts.V.rows());
  ck(c, hexopt_get_positions(c, X.data()), "get_positions");
  for (int64_t i = 0; i < ts.V.rows(); i++)
    for (int d = 0; d < 3; d++) ts.V(i, d) = X[3 * i + d];
}
#endif
