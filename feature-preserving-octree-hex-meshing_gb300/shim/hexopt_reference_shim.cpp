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
// Scope: the forms the feature-alignment loop uses -- symmetric Dirichlet energy over the 8
// corner tets of each hex (F holds 8 tets per hex in hex_tetra_table order), cube or own-shape
// reference tets, corner / tangent-plane / feature-line soft constraints, fixed iteration counts.
// Other forms (adaptive iteration count, glue, projection and region terms, other energies,
// scaffold post variables, 2-D quad quality) throw std::runtime_error naming the form: there is
// no CPU fallback behind this file.
//
// Environment: HEXOPT_DEVICE (CUDA device, default 0); HEXOPT_PRECISION=mixed selects the
// FP32/FP64 mixed mode (default: plain FP64, the reference's arithmetic).
#include "slim_m.h"
#include "metro_hausdorff.h"
#include "global_functions.h"

#include "hexopt_gpu.h"

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

// Hexes from the 8-tets-per-hex list: tet j of hex h starts at corner j (hex_tetra_table[j][0]
// == j, global_types.h:163-173), and the other three corners must follow the table.
static std::vector<uint32_t> hexes_from_tets(const Eigen::MatrixXi &F) {
  if (F.cols() != 4 || F.rows() % 8 != 0) unsupported("a tet list that is not 8 corner tets per hex");
  const int64_t nh = F.rows() / 8;
  std::vector<uint32_t> H(8 * (size_t)nh);
  for (int64_t h = 0; h < nh; h++) {
    for (int j = 0; j < 8; j++) H[8 * h + j] = (uint32_t)F(8 * h + j, 0);
    for (int j = 0; j < 8; j++)
      for (int k = 0; k < 4; k++)
        if ((uint32_t)F(8 * h + j, k) != H[8 * h + hex_tetra_table[j][k]])
          unsupported("a tet list that is not 8 corner tets per hex");
  }
  return H;
}

// compute_referenceMesh's per-hex choice (global_functions.cpp:3735-3806), read back from the
// reference tets: 1 = the corner tets of a cube, 0 = the hex's own corners at V.
static std::vector<uint8_t> hflags_from_rt(const std::vector<Eigen::MatrixXd> &RT, const Eigen::MatrixXi &F,
                                           const Eigen::MatrixXd &V) {
  const int64_t nh = F.rows() / 8;
  std::vector<uint8_t> flag(nh, 1);
  if (RT.empty()) return flag;
  if ((int64_t)RT.size() != F.rows()) unsupported("reference tets whose count differs from the tets'");
  for (int64_t h = 0; h < nh; h++) {
    bool cube = true, own = true;
    for (int j = 0; j < 8 && (cube || own); j++) {
      const Eigen::MatrixXd &R = RT[8 * h + j];
      if (R.rows() != 4 || R.cols() != 3) unsupported("reference tets that are not 4 x 3");
      double a = 0;
      for (int k = 1; k < 4; k++) a = std::max(a, (R.row(k) - R.row(0)).norm());
      for (int k = 1; k < 4 && cube; k++)
        for (int d = 0; d < 3; d++) {
          const double want = a * (hex_ref_shape[hex_tetra_table[j][k]][d] - hex_ref_shape[hex_tetra_table[j][0]][d]);
          if (std::fabs(R(k, d) - R(0, d) - want) > 1e-9 * a) { cube = false; break; }
        }
      for (int k = 0; k < 4 && own; k++)
        for (int d = 0; d < 3; d++)
          if (R(k, d) != V(F(8 * h + j, k), d)) { own = false; break; }
    }
    if (!cube && !own) unsupported("reference tets other than cubes or the hex's own shape");
    flag[h] = cube ? 1 : 0;
  }
  return flag;
}

// Uploads data's mesh, constraints and weights into the SLIM context and runs the precompute.
static void load(SLIMData &data) {
  Contexts &C = contexts();
  hexopt_ctx *c = get(C.slim);
  const Tetralize_Set &ts = data.ts;
  if (data.slim_energy != SYMMETRIC_DIRICHLET) unsupported("a SLIM energy other than SYMMETRIC_DIRICHLET");
  if (ts.projection || data.Projection) unsupported("the projection penalty (Tetralize_Set::projection)");
  if (ts.glue) unsupported("the glue penalty (Tetralize_Set::glue)");
  if (ts.known_value_post) unsupported("known_value_post elimination");
  if (ts.regionb.size() > 0 && ts.lamda_region != 0) unsupported("region constraints");
  const std::vector<uint32_t> H = hexes_from_tets(data.F);
  const std::vector<uint8_t> hf = hflags_from_rt(ts.RT, data.F, data.V);
  const int64_t nv = data.V.rows(), nh = (int64_t)H.size() / 8;
  const std::vector<double> V = rows3(data.V);
  C.loaded = nullptr;
  ck(c, hexopt_upload_meshes(c, 1, &nv, &nh, V.data(), H.data(), hf.data()), "upload_meshes");
  const Feature_Constraints &fc = ts.fc;
  const int64_t nC = fc.ids_C.size(), nT = fc.ids_T.size(), nL = fc.ids_L.size();
  const std::vector<int32_t> iC = ids(fc.ids_C), iT = ids(fc.ids_T), iL = ids(fc.ids_L);
  const std::vector<double> Cp = nC ? rows3(fc.C) : std::vector<double>(), Tn = nT ? rows3(fc.normal_T) : std::vector<double>();
  const std::vector<double> Ta(fc.dis_T.data(), fc.dis_T.data() + nT);
  const std::vector<double> La = nL ? rows3(fc.Axa_L) : std::vector<double>(), Lo = nL ? rows3(fc.origin_L) : std::vector<double>();
  ck(c, hexopt_set_corners(c, &nC, iC.data(), Cp.data()), "set_corners");
  ck(c, hexopt_set_tangents(c, &nT, iT.data(), Tn.data(), Ta.data()), "set_tangents");
  ck(c, hexopt_set_lines(c, &nL, iL.data(), La.data(), Lo.data()), "set_lines");
  ck(c, hexopt_set_weights(c, &fc.lamda_C, &fc.lamda_T, &fc.lamda_L), "set_weights");
  hexopt_slim_params p;
  std::memset(&p, 0, sizeof p);
  p.energy = HEXOPT_SYMMETRIC_DIRICHLET;
  p.precision = precision();
  p.weight_opt = data.weight_opt;
  p.exp_factor = data.exp_factor;
  p.cg_max_iter = 20;
  p.cg_tol = 1e-8;
  p.ls_candidates = 1;
  p.cube = 1;
  ck(c, hexopt_slim_precompute(c, &p), "slim_precompute");
  // iterations start from V_init (data.V_o); the precompute snapshot was taken at data.V
  if (data.V_o.rows() == data.V.rows() && data.V_o != data.V) {
    const std::vector<double> X = rows3(data.V_o);
    ck(c, hexopt_set_positions(c, X.data()), "set_positions");
  }
  C.loaded = &data;
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
  hexopt_ctx *c = contexts().slim;
  const std::vector<double> X = rows3(data.V_o);
  double E = 0;
  ck(c, hexopt_energy_fwd(c, X.data(), &E), "energy_fwd");
  data.energy = E / data.mesh_area;
}

// The 18-argument overload (slim_m.h:89-100) feeds the projection / region path of slim_opt.
void slim_precompute(Eigen::MatrixXd &, Eigen::MatrixXi &, Eigen::MatrixXd &, SLIMData &, SLIM_ENERGY,
                     Eigen::VectorXi &, Eigen::MatrixXd &, Eigen::VectorXi &, Eigen::MatrixXd &, Eigen::VectorXi &,
                     Eigen::MatrixXd &, Eigen::MatrixXd &, Eigen::VectorXi &, Eigen::MatrixXd &, Eigen::VectorXd &,
                     Eigen::VectorXi &, Eigen::MatrixXd &, bool, bool) {
  unsupported("slim_precompute with explicit projection / region arguments");
}

// slim_m.cpp:1189-1291, fixed-count branch (:1269-1288): iter_num SLIM iterations, the energy
// printed after each as the reference does.
Eigen::MatrixXd slim_solve2(SLIMData &data, int iter_num, int type, bool verbose) {
  (void)type;
  (void)verbose;
  if (iter_num < 0) unsupported("the adaptive iteration count (iter_num == -1)");
  Contexts &C = contexts();
  if (C.loaded != &data) load(data);
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
  std::vector<double> X(3 * (size_t)data.V_o.rows());
  ck(c, hexopt_get_positions(c, X.data()), "get_positions");
  for (int64_t i = 0; i < data.V_o.rows(); i++)
    for (int d = 0; d < 3; d++) data.V_o(i, d) = X[3 * i + d];
  if (data.a_L.size() > 0) ck(c, hexopt_get_curve_params(c, data.a_L.data()), "get_curve_params");
  return data.V_o;
}

// slim_m.cpp:1293-1394 (glue doubling after iteration 3) belongs to the untangling path.
Eigen::MatrixXd slim_solve(SLIMData &, int, int, bool) {
  unsupported("slim_solve (the untangling / glue driver)");
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
