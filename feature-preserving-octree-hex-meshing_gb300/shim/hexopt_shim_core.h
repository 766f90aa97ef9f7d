// hexopt_shim_core.h -- the conversions behind the drop-in shim (hexopt_reference_shim.cpp),
// free of the reference's headers: the shim turns SLIMData / Tetralize_Set into the plain arrays
// of SlimSetup, and everything from there on -- the hexes recovered from the tet list, the
// reference tets, the soft-constraint sets, the glue groups from V_ranges, the held vertices of
// known_value_post, the precompute at V and the start at V_o -- lives here, where a program
// without the reference tree can run it against the library.
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "hexopt_gpu.h"

namespace hexopt_shim_core {

// hex_tetra_table (global_types.h:163-173): corner tet k of a hex is corners (k, ...) -- the first
// corner of tet k is corner k.
static const int kHexTetra[8][4] = {{0, 3, 4, 1}, {1, 0, 5, 2}, {2, 1, 6, 3}, {3, 2, 7, 0},
                                    {4, 7, 5, 0}, {5, 4, 6, 1}, {6, 5, 7, 2}, {7, 6, 4, 3}};

// The hexes of a tet list of 8 corner tets per hex in hex_tetra_table order (as slim_m_opt's
// callers build ts.T); false with a message when the list is not of that form.
inline bool hexes_from_tets(const int32_t *T, int64_t ntets, std::vector<uint32_t> &H, std::string &err) {
  if (ntets % 8 != 0) { err = "a tet list that is not 8 corner tets per hex"; return false; }
  const int64_t nh = ntets / 8;
  H.assign(8 * (size_t)nh, 0);
  for (int64_t h = 0; h < nh; h++) {
    for (int j = 0; j < 8; j++) H[8 * h + j] = (uint32_t)T[4 * (8 * h + j)];
    for (int j = 0; j < 8; j++)
      for (int k = 0; k < 4; k++)
        if ((uint32_t)T[4 * (8 * h + j) + k] != H[8 * h + kHexTetra[j][k]]) {
          err = "a tet list that is not 8 corner tets per hex";
          return false;
        }
  }
  return true;
}

// Tetralize_Set::V_ranges -> glue groups: range i is [V_ranges[i-1] + 1, V_ranges[i]] (the first
// from 0), consecutive vertex ids (slim_m.cpp:611-646).
inline bool groups_from_ranges(const uint32_t *V_ranges, int64_t n, int64_t nv, std::vector<int64_t> &ptr,
                               std::vector<int32_t> &vs, std::string &err) {
  ptr.assign(1, 0);
  vs.clear();
  int64_t start = 0;
  for (int64_t i = 0; i < n; i++) {
    const int64_t end = V_ranges[i];
    if (end < start || end >= nv) { err = "V_ranges that are not increasing vertex ranges"; return false; }
    for (int64_t v = start; v <= end; v++) vs.push_back((int32_t)v);
    ptr.push_back((int64_t)vs.size());
    start = end + 1;
  }
  return true;
}

// What a slim_precompute call hands the optimiser, as plain arrays (row-major n x 3 vertices).
struct SlimSetup {
  int64_t nv = 0;
  const double *V = nullptr;    // slim_precompute's V: the tets' volumes for the operator
  const double *V_o = nullptr;  // its V_init: where the iterations start (may be V)
  int64_t ntets = 0;
  const int32_t *T = nullptr;   // ntets x 4
  const double *RT = nullptr;   // ntets x 4 x 3 reference tets (ts.RT), or null: cubes
  int energy = HEXOPT_SYMMETRIC_DIRICHLET, precision = HEXOPT_FP64, variant = 0;
  double weight_opt = 1.0;
  // Feature_Constraints
  int64_t nC = 0; const int32_t *ids_C = nullptr; const double *C = nullptr; double lamda_C = 0;
  int64_t nT = 0; const int32_t *ids_T = nullptr; const double *normal_T = nullptr; const double *dis_T = nullptr;
  double lamda_T = 0;
  int64_t nL = 0; const int32_t *ids_L = nullptr; const double *Axa_L = nullptr; const double *origin_L = nullptr;
  double lamda_L = 0;
  // Tetralize_Set::projection (b, bc, lamda_projection)
  bool projection = false; int64_t nB = 0; const int32_t *b = nullptr; const double *bc = nullptr;
  double lamda_projection = 0;
  // Tetralize_Set::glue (V_ranges, lamda_glue)
  bool glue = false; int64_t n_ranges = 0; const uint32_t *V_ranges = nullptr; double lamda_glue = 0;
  // known_value_post: vertices post_index.. held at post_Variables ((nv - post_index) x 3)
  bool known_value_post = false; int64_t post_index = 0; const double *post_Variables = nullptr;
};

inline int fail(std::string &err, int rc, const std::string &what) {
  err = what;
  return rc;
}

// Loads a SlimSetup into a context (one mesh) and runs the precompute: the shim's slim_precompute.
inline int load_slim(hexopt_ctx *c, const SlimSetup &s, std::string &err) {
  std::vector<uint32_t> H;
  if (!hexes_from_tets(s.T, s.ntets, H, err)) return HEXOPT_ERR_UNSUPPORTED;
  const int64_t nv = s.nv, nh = (int64_t)H.size() / 8;
  auto ck = [&](int rc, const char *what) {
    if (rc != HEXOPT_OK) err = std::string(what) + ": " + hexopt_last_error(c);
    return rc;
  };
  int rc;
  if ((rc = ck(hexopt_upload_meshes(c, 1, &nv, &nh, s.V, H.data(), nullptr), "upload_meshes"))) return rc;
  if (s.RT && (rc = ck(hexopt_set_reference_tets(c, s.RT), "set_reference_tets"))) return rc;
  // glue turns the feature terms off (slim_m.cpp:647): nothing of them is loaded then
  const int64_t zero = 0;
  const bool feat = !s.glue;
  if ((rc = ck(hexopt_set_corners(c, feat ? &s.nC : &zero, s.ids_C, s.C), "set_corners"))) return rc;
  if ((rc = ck(hexopt_set_tangents(c, feat ? &s.nT : &zero, s.ids_T, s.normal_T, s.dis_T), "set_tangents"))) return rc;
  if ((rc = ck(hexopt_set_lines(c, feat ? &s.nL : &zero, s.ids_L, s.Axa_L, s.origin_L), "set_lines"))) return rc;
  if ((rc = ck(hexopt_set_weights(c, &s.lamda_C, &s.lamda_T, &s.lamda_L), "set_weights"))) return rc;
  if (s.projection && (rc = ck(hexopt_set_projection(c, &s.nB, s.b, s.bc, &s.lamda_projection), "set_projection")))
    return rc;
  if (s.glue) {
    std::vector<int64_t> ptr;
    std::vector<int32_t> vs;
    if (!groups_from_ranges(s.V_ranges, s.n_ranges, nv, ptr, vs, err)) return HEXOPT_ERR_UNSUPPORTED;
    const int64_t ng = (int64_t)ptr.size() - 1;
    if ((rc = ck(hexopt_set_glue(c, &ng, ptr.data(), vs.data(), &s.lamda_glue), "set_glue"))) return rc;
  }
  if (s.known_value_post) {
    // the reference solves with the held rows at post_Variables but leaves V_o's rows where they
    // are; its callers set both alike, and only that case is one consistent problem
    const double *start = s.V_o ? s.V_o : s.V;
    for (int64_t i = s.post_index; i < nv; i++)
      for (int d = 0; d < 3; d++)
        if (s.post_Variables[3 * (i - s.post_index) + d] != start[3 * i + d])
          return fail(err, HEXOPT_ERR_UNSUPPORTED, "known_value_post with post_Variables other than the held rows of V_init");
    std::vector<int32_t> ids;
    for (int64_t i = s.post_index; i < nv; i++) ids.push_back((int32_t)i);
    const int64_t nf = (int64_t)ids.size();
    if (ids.empty()) ids.push_back(0);
    if ((rc = ck(hexopt_set_fixed(c, &nf, ids.data()), "set_fixed"))) return rc;
  }
  hexopt_slim_params p;
  std::memset(&p, 0, sizeof p);
  p.energy = s.energy;
  p.precision = s.precision;
  p.weight_opt = s.weight_opt;
  p.exp_factor = 1.0;  // slim_precompute's reset (slim_m.cpp:1125)
  p.cg_max_iter = 20;
  p.cg_tol = 1e-8;
  p.ls_candidates = 1;
  p.cube = 1;
  p.variant = s.variant;
  if ((rc = ck(hexopt_slim_precompute(c, &p), "slim_precompute"))) return rc;
  // the iterations start from V_init; the precompute took the operator at V
  if (s.V_o && s.V_o != s.V && std::memcmp(s.V_o, s.V, sizeof(double) * 3 * (size_t)nv) != 0)
    if ((rc = ck(hexopt_set_positions(c, s.V_o), "set_positions"))) return rc;
  return HEXOPT_OK;
}

}  // namespace hexopt_shim_core
