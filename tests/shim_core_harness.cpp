// shim_core_harness.cpp -- C entry points over hexopt_shim_core.h (the drop-in shim's conversions)
// for tests/test_gpu_shim_core.py, which compiles this file against libhexopt_gpu.so on the GPU
// machine and feeds it the plain arrays the shim would build from SLIMData / Tetralize_Set.
// TEST INFRASTRUCTURE ONLY.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hexopt_shim_core.h"

static int report(int rc, const std::string &msg, char *err, int err_len) {
  if (rc != HEXOPT_OK && err && err_len > 0) std::snprintf(err, (size_t)err_len, "%s", msg.c_str());
  return rc;
}

extern "C" {

// slim_precompute at V with the setup, start at V_o, `iters` fixed SLIM iterations (slim_solve2's
// fixed branch); out_V = positions, out3 = energy / mesh_area, energy_quality, energy_soft.
int harness_slim(int64_t nv, const double *V, const double *V_o, int64_t ntets, const int32_t *T, const double *RT,
                 int energy, double weight_opt, int variant, int64_t nC, const int32_t *ids_C, const double *C,
                 double lamda_C, int64_t nT, const int32_t *ids_T, const double *normal_T, const double *dis_T,
                 double lamda_T, int64_t nL, const int32_t *ids_L, const double *Axa_L, const double *origin_L,
                 double lamda_L, int iters, double *out_V, double *out3, char *err, int err_len) {
  hexopt_ctx *c = nullptr;
  int rc = hexopt_create(&c, 0);
  if (rc) return report(rc, "create", err, err_len);
  hexopt_shim_core::SlimSetup s;
  s.nv = nv; s.V = V; s.V_o = V_o; s.ntets = ntets; s.T = T; s.RT = RT;
  s.energy = energy; s.weight_opt = weight_opt; s.variant = variant;
  s.nC = nC; s.ids_C = ids_C; s.C = C; s.lamda_C = lamda_C;
  s.nT = nT; s.ids_T = ids_T; s.normal_T = normal_T; s.dis_T = dis_T; s.lamda_T = lamda_T;
  s.nL = nL; s.ids_L = ids_L; s.Axa_L = Axa_L; s.origin_L = origin_L; s.lamda_L = lamda_L;
  std::string msg;
  rc = hexopt_shim_core::load_slim(c, s, msg);
  hexopt_slim_report rep;
  std::memset(&rep, 0, sizeof rep);
  if (!rc) rc = hexopt_slim_iterate(c, iters, &rep);
  if (!rc) rc = hexopt_get_positions(c, out_V);
  if (rc && msg.empty()) msg = hexopt_last_error(c);
  out3[0] = rep.energy; out3[1] = rep.energy_quality; out3[2] = rep.energy_soft;
  hexopt_destroy(c);
  return report(rc, msg, err, err_len);
}

// The gluing solve as glueInternalNodes sets it up: copies glued by V_ranges, the copies from
// post_index on held (known_value_post), the adaptive slim_solve2 branch of type 1.
int harness_glue(int64_t nv, const double *V, int64_t ntets, const int32_t *T, const double *RT, int64_t n_ranges,
                 const uint32_t *V_ranges, int64_t post_index, const double *post, double lamda_glue, int energy,
                 double weight_opt, int max_iter, double *out_V, int32_t *iterations, double *min_J, char *err,
                 int err_len) {
  hexopt_ctx *c = nullptr;
  int rc = hexopt_create(&c, 0);
  if (rc) return report(rc, "create", err, err_len);
  hexopt_shim_core::SlimSetup s;
  s.nv = nv; s.V = V; s.V_o = V; s.ntets = ntets; s.T = T; s.RT = RT;
  s.energy = energy; s.weight_opt = weight_opt;
  s.glue = true; s.n_ranges = n_ranges; s.V_ranges = V_ranges; s.lamda_glue = lamda_glue;
  s.known_value_post = post_index < nv; s.post_index = post_index; s.post_Variables = post;
  std::string msg;
  rc = hexopt_shim_core::load_slim(c, s, msg);
  hexopt_adaptive_report rep;
  std::memset(&rep, 0, sizeof rep);
  if (!rc) rc = hexopt_slim_solve_adaptive(c, 1, 2, max_iter, &rep);
  if (!rc) rc = hexopt_get_positions(c, out_V);
  if (rc && msg.empty()) msg = hexopt_last_error(c);
  *iterations = rep.iterations;
  *min_J = rep.min_Jacobian;
  hexopt_destroy(c);
  return report(rc, msg, err, err_len);
}

int harness_hexes_from_tets(const int32_t *T, int64_t ntets, uint32_t *H) {
  std::vector<uint32_t> h;
  std::string msg;
  if (!hexopt_shim_core::hexes_from_tets(T, ntets, h, msg)) return HEXOPT_ERR_UNSUPPORTED;
  std::memcpy(H, h.data(), sizeof(uint32_t) * h.size());
  return HEXOPT_OK;
}

}  // extern "C"
