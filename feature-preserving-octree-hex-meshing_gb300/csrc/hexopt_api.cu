// hexopt_api.cu -- host runtime behind the C ABI of include/hexopt_gpu.h.
//
// One context = one compute stream (with two copy streams for the asynchronous transfers and the
// side streams of a step's parallel branches, all ordered against it by events) + one batch of
// meshes resident in HBM.  Every compute stage is a kernel launch over per-mesh segment tables
// (no block straddles two meshes).  The scalar
// reductions (energies, dot products, minima) are per mesh and summed in a fixed order; the
// per-vertex scatters (right-hand side, SpMV product, residual, gradient) use float atomics, so
// positions are not bit-reproducible from run to run (the order of the atomic adds varies).
// The host only uploads inputs, orders launches and downloads results; there is no CPU compute
// path.
#include <cuda_runtime.h>
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/hexopt_gpu.h"
#include "hexopt_bvh.h"
#include "hexopt_kernels.h"

using namespace hexopt;

namespace {

// Device allocations made by any context; a captured step graph holds raw buffer addresses, so a
// graph captured before the count changed is re-captured before its next replay.
std::atomic<uint64_t> g_device_allocs{0};

// ------------------------------------------------------------------ device buffer
struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t n) {
    if (n == 0) n = 16;
    if (n <= bytes) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    else p = nullptr;
    g_device_allocs.fetch_add(1, std::memory_order_relaxed);
    return e;
  }
  template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

struct KindTable {
  std::vector<Seg> segs;
  DBuf dev;
  int64_t nblk = 0;
};

// One set of BVH query buffers: the overflow list of the cooperative pass, per-sample distances,
// the batched exact evaluation's candidate lists and the fallback list.
struct QueryBufs {
  DBuf ovf_item, ovf_mesh, ovf_count, ovf_best, ovf_face, ovf_pt, hdist;
  DBuf cand_leaf, cand_qi, cand_x, cand_d, cand_count, q_off, q_cnt, qpos, q_mesh, fb_count, fb_item, fb_mesh;
  int64_t cand_cap = 0;
};

struct StaticBvh {  // device LBVH over a fixed triangle set
  DBuf child, parent, box, leaf_face, tri, counters, node, leafd, onode;
  int32_t n = 0;
  BvhDev dev() const {
    BvhDev b{};
    b.n = n;
    b.child = child.as<int32_t>();
    b.box = box.as<float>();
    b.leaf_face = leaf_face.as<int32_t>();
    b.tri = tri.as<double>();
    b.node = node.as<float4>();
    b.leafd = leafd.as<float4>();
    b.onode = onode.as<float4>();
    return b;
  }
};

struct TargetHost {
  bool set = false;
  int64_t nv = 0, nf = 0;
  std::vector<double> TV;
  StaticBvh bvh;
  DBuf TVd, FN, VNc, ENc, EP, curve_ptr, curve_vs, curve_closed;
  int64_t n_curves = 0;
  double lo[3], hi[3];
  std::vector<int64_t> ref_vs;  // vertices referenced by a face (target-local ids)
};

struct SurfaceHost {
  bool set = false;
  int64_t nf = 0;
  DBuf F, child, parent, box, leaf_face, counters, node, leafd;
  std::vector<int64_t> ref_vs;  // referenced vertices (global ids)
};

}  // namespace

struct hexopt_ctx {
  int device = 0;
  cudaStream_t st = nullptr;
  std::string err;
  int64_t launches = 0;
  // batch
  int n_meshes = 0;
  int64_t NV = 0, NH = 0, NC = 0, NT = 0, NL = 0, NG = 0;
  std::vector<MeshDesc> md;
  DBuf md_d, sc_d;
  std::vector<MeshScalars> sc;
  DBuf X, X32, hexv, gslot, Sinv, Ccoef, Bgen, aL;
  DBuf b, diag, ba, diaga;
  DBuf d, r, p, q, invd, da, ra, pa, qa, invda;
  DBuf Rrot, dd, dda, ddf;  // mixed mode's FP64 refinement: stored rotations, FP64 update (+ its FP32 copy)
  // general reference shapes (compute_referenceMesh with cube = 0, or reference corners set by the
  // caller): per-hex h_flag, optional reference corners, shapes, and the all-hex slot tables
  DBuf hflag_d, ref_p8, Bref, gslot_all, Bgen_all;
  bool has_ref_p8 = false, rest_fixed = false;
  bool has_ref_tets = false;  // explicit reference tets (ref_p8 then holds 96 doubles per hex)
  DBuf stage, stage2, HJs, VJs, Xa, grad, Xbak;
  DBuf root_list, root_mesh, root_count, root_min;  // flip-avoid bound: tets needing the exact root
  bool adj_ready = false;
  DBuf partials, counters;
  DBuf c_ids, c_pos, t_ids, t_nrm, t_dis, l_ids, l_axis, l_orig, l_curve;
  std::vector<int64_t> nC, nT, nL;
  std::vector<double> lamC, lamT, lamL;
  // untangling / glue path: projection points, glue groups, held vertices
  std::vector<int64_t> nB, nG;
  int64_t NB = 0, NGR = 0;
  DBuf b_ids, b_pos, g_ptr, g_vs, vfix, Xm;
  std::vector<uint8_t> fixed_h;  // host copy of the held-vertex flags (for argument checks)
  std::vector<uint32_t> H_h;     // host copy of the hexes (mesh-local corner ids), for untangling
  // device order of the batch (Morton-sorted vertices and hexes); the caller's order at the ABI
  int ordering = 2;  // 0 caller order, 1 Morton, 2 Morton unless the caller's numbering is coherent
  bool ordered = false;
  int query_budget = 0;  // per-thread BVH traversal pops before the warp pass (0: the defaults below)
  DBuf vnew2old, vold2new, hnew2old, hold2new;
  std::vector<int32_t> vold2new_h, hnew2old_h;
  bool has_fixed = false, has_glue = false;
  KindTable kind[8];
  // items per block: hex 128, unknowns 256 x ipt, constraints 256, queries 128
  int block[8] = {128, 256, 256, 128, 128, 128, 128, 128};  // K_CONS follows K_VERT's size
  int ipt[8] = {1, 8, 1, 1, 1, 1, 1, 1};                     // items per thread of each kind
  // SLIM
  hexopt_slim_params params{};
  bool precomputed = false;
  bool mixed = false;
  // targets / surfaces
  std::vector<TargetHost> tgt;
  std::vector<SurfaceHost> surf;
  DBuf tgt_d, surf_d, refit_d, hm_d, tgt_vs_d, surf_vs_d;
  int64_t n_surf_faces = 0;  // surface faces of the batch (items of K_SURFF)
  // BVH query buffers, two sets: set 0 serves the projection and Hausdorff side 1, set 1 Hausdorff
  // side 0, so that the two sides run at the same time
  QueryBufs qb[2];
  DBuf qseed;           // previous winning leaf per query: projection, Hausdorff side 0, side 1
  int64_t qseed_n = 0;  // items per region of qseed
  std::vector<int64_t> tgt_vs_cnt, surf_vs_cnt;
  bool haus_ready = false;
  // feature alignment
  double lamda0 = 0.05, HR = 0.005;
  bool fa_ready = false;
  bool use_graph = false;
  bool graph_conditionals = true;  // the line-search rounds as a WHILE node when captured
  cudaGraphExec_t graph_exec = nullptr;
  bool graph_hausdorff = false;
  int64_t graph_launches = 0;
  // what the captured graph baked in: launch tables, buffer addresses, parameters
  uint64_t tables_epoch = 0, graph_tables = 0, graph_allocs = 0;
  hexopt_slim_params graph_params{};
  double graph_lamda0 = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // asynchronous position transfers: one copy stream each way (an upload never queues behind a
  // download), staging buffers each way, and the events that order them against the compute
  // stream (input copied / consumed, output staged / copied)
  cudaStream_t ust = nullptr, dst = nullptr;
  cudaEvent_t in_ready = nullptr, in_free = nullptr, out_ready = nullptr, out_done = nullptr;
  // recorded by each feature-alignment step once its line search has applied the step (an event
  // record node in the step's graph): the positions are final from there on
  cudaEvent_t ev_xfinal = nullptr;
  DBuf in_stage, out_stage;
  // the end of a step forks three ways (Hausdorff side 1 on st, side 0 and the SJ check on their
  // own streams) and joins before the Hausdorff combine; each branch reduces into its own region
  // of the partials and counters (region 0: the step's kernels and the SJ check, 1: side 1 and
  // the bbox, 2: side 0)
  cudaStream_t hs0 = nullptr, hsj = nullptr;
  cudaStream_t lsb = nullptr;  // captures the body of the line search's WHILE node
  cudaEvent_t ev_fork = nullptr, ev_bbox = nullptr, ev_side0 = nullptr, ev_sj = nullptr;
  cudaEvent_t ev_pfork = nullptr, ev_proj = nullptr;  // the projection beside the local step
  int64_t part_region = 0;  // doubles per partials region
};

namespace {

int fail(hexopt_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? HEXOPT_ERR_NOMEM : HEXOPT_ERR_CUDA, \
                  "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);     \
  } while (0)

#define CKL()                                                                                 \
  do {                                                                                        \
    cudaError_t e_ = cudaGetLastError();                                                      \
    if (e_ != cudaSuccess)                                                                    \
      return fail(ctx, HEXOPT_ERR_CUDA, "launch: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

}  // namespace

// Whether the caller's numbering already keeps neighbouring hexes' corners close in memory: in
// every mesh, the median over hexes of the corner-id span (max - min) and the median jump of the
// first corner between consecutive hexes both stay within 4 nv^(2/3) -- a 3-D coherent numbering
// (a structured grid's rows, planes) spans about one plane, nv^(2/3); a random one about nv.
static bool numbering_coherent(const hexopt_ctx *c, int n_meshes, const int64_t *nv, const int64_t *nh, const uint32_t *H) {
  int64_t ho = 0;
  for (int m = 0; m < n_meshes; m++) {
    const double lim = 4.0 * std::cbrt((double)nv[m] * (double)nv[m]);
    std::vector<uint32_t> span(nh[m]), jump(nh[m] > 1 ? nh[m] - 1 : 1, 0);
    for (int64_t h = 0; h < nh[m]; h++) {
      const uint32_t *q = H + 8 * (ho + h);
      uint32_t lo = q[0], hi = q[0];
      for (int k = 1; k < 8; k++) { lo = std::min(lo, q[k]); hi = std::max(hi, q[k]); }
      span[h] = hi - lo;
      if (h > 0) {
        const uint32_t a = q[0], b = H[8 * (ho + h - 1)];
        jump[h - 1] = a > b ? a - b : b - a;
      }
    }
    std::nth_element(span.begin(), span.begin() + span.size() / 2, span.end());
    std::nth_element(jump.begin(), jump.begin() + jump.size() / 2, jump.end());
    if (span[span.size() / 2] > lim || jump[jump.size() / 2] > lim) return false;
    ho += nh[m];
  }
  (void)c;
  return true;
}

// device order <-> caller order
static const int32_t *vn2o(const hexopt_ctx *c) { return c->ordered ? c->vnew2old.as<int32_t>() : nullptr; }
static const int32_t *vo2n(const hexopt_ctx *c) { return c->ordered ? c->vold2new.as<int32_t>() : nullptr; }
static const int32_t *hn2o(const hexopt_ctx *c) { return c->ordered ? c->hnew2old.as<int32_t>() : nullptr; }
static const int32_t *ho2n(const hexopt_ctx *c) { return c->ordered ? c->hold2new.as<int32_t>() : nullptr; }
// a caller's mesh-local vertex id -> the device's mesh-local id
static int32_t local_vid(const hexopt_ctx *c, int m, int32_t v) {
  if (!c->ordered) return v;
  const int64_t o = c->md[m].v_off;
  return (int32_t)(c->vold2new_h[o + v] - o);
}

namespace {

template <typename T>
cudaError_t upload(DBuf &buf, const T *src, size_t n, cudaStream_t st) {
  cudaError_t e = buf.ensure(n * sizeof(T));
  if (e != cudaSuccess) return e;
  if (n && src) return cudaMemcpyAsync(buf.p, src, n * sizeof(T), cudaMemcpyHostToDevice, st);
  return cudaSuccess;
}

// Build the segment table of one launch kind: counts per mesh, items numbered from item0.
void build_kind(hexopt_ctx *c, int k, const std::vector<int64_t> &count, const std::vector<int64_t> &item0) {
  KindTable &t = c->kind[k];
  t.segs.clear();
  const int B = c->block[k] * c->ipt[k];
  for (int m = 0; m < c->n_meshes; m++) {
    const int64_t n = count[m];
    const int64_t nb = std::max<int64_t>(1, (n + B - 1) / B);
    c->md[m].kblk0[k] = (int64_t)t.segs.size();
    c->md[m].knblk[k] = (int32_t)nb;
    c->md[m].kitem0[k] = item0[m];
    c->md[m].kcount[k] = n;
    for (int64_t bk = 0; bk < nb; bk++) {
      Seg s;
      s.mesh = m;
      s.blk_in_mesh = (int32_t)bk;
      s.begin = item0[m] + bk * B;
      s.end = std::min(item0[m] + n, s.begin + B);
      if (s.begin > s.end) s.begin = s.end;
      t.segs.push_back(s);
    }
  }
  t.nblk = (int64_t)t.segs.size();
}

int ensure_query_buffers(hexopt_ctx *ctx);

int rebuild_tables(hexopt_ctx *ctx) {
  const int M = ctx->n_meshes;
  ctx->tables_epoch++;  // grid sizes of a captured graph are stale
  ctx->block[K_CONS] = ctx->block[K_VERT];  // constraint launches use the vertex block size
  std::vector<int64_t> cnt(M), it0(M);
  int64_t off_c = 0, off_t = 0, off_l = 0, off_b = 0, off_g = 0;
  for (int m = 0; m < M; m++) {
    MeshDesc &d = ctx->md[m];
    d.c_off = off_c; d.nc = ctx->nC[m];
    d.t_off = off_t; d.nt = ctx->nT[m];
    d.l_off = off_l; d.nl = ctx->nL[m];
    d.b_off = off_b; d.nb = ctx->nB[m];
    d.grp_off = off_g; d.ngrp = ctx->nG[m];
    off_c += d.nc; off_t += d.nt; off_l += d.nl; off_b += d.nb; off_g += d.ngrp;
  }
  ctx->NC = off_c; ctx->NT = off_t; ctx->NL = off_l;
  for (int m = 0; m < M; m++) { cnt[m] = ctx->md[m].nh; it0[m] = ctx->md[m].h_off; }
  build_kind(ctx, K_HEX, cnt, it0);
  for (int m = 0; m < M; m++) { cnt[m] = ctx->md[m].nv + ctx->md[m].nl; it0[m] = ctx->md[m].v_off + ctx->md[m].l_off; }
  build_kind(ctx, K_VERT, cnt, it0);
  for (int m = 0; m < M; m++) {
    const MeshDesc &d = ctx->md[m];
    cnt[m] = d.nc + d.nt + d.nl + d.nb + d.ngrp;
    it0[m] = d.c_off + d.t_off + d.l_off + d.b_off + d.grp_off;
  }
  build_kind(ctx, K_CONS, cnt, it0);
  for (int m = 0; m < M; m++) { cnt[m] = ctx->md[m].nt; it0[m] = ctx->md[m].t_off; }
  build_kind(ctx, K_PROJ, cnt, it0);
  for (int m = 0; m < M; m++) { cnt[m] = ctx->md[m].nl; it0[m] = ctx->md[m].l_off; }
  build_kind(ctx, K_LINE, cnt, it0);
  {
    int64_t o = 0;
    for (int m = 0; m < M; m++) { cnt[m] = m < (int)ctx->tgt_vs_cnt.size() ? ctx->tgt_vs_cnt[m] : 0; it0[m] = o; o += cnt[m]; }
    build_kind(ctx, K_TGTV, cnt, it0);
    o = 0;
    for (int m = 0; m < M; m++) { cnt[m] = m < (int)ctx->surf_vs_cnt.size() ? ctx->surf_vs_cnt[m] : 0; it0[m] = o; o += cnt[m]; }
    build_kind(ctx, K_SURFV, cnt, it0);
  }
  {
    int64_t o = 0;
    for (int m = 0; m < M; m++) {
      cnt[m] = (m < (int)ctx->surf.size() && ctx->surf[m].set) ? ctx->surf[m].nf : 0;
      it0[m] = o;
      o += cnt[m];
    }
    ctx->n_surf_faces = o;
    build_kind(ctx, K_SURFF, cnt, it0);
  }
  for (int m = 0; m < M; m++) {
    MeshDesc &d = ctx->md[m];
    d.hblk0 = d.kblk0[K_HEX]; d.nhblk = d.knblk[K_HEX];
    d.vblk0 = d.kblk0[K_VERT]; d.nvblk = d.knblk[K_VERT];
    d.cblk0 = d.kblk0[K_CONS]; d.ncblk = d.knblk[K_CONS];
  }
  int64_t maxblk = 0;
  for (int k = 0; k < 8; k++) {
    maxblk = std::max(maxblk, ctx->kind[k].nblk);
    CK(upload(ctx->kind[k].dev, ctx->kind[k].segs.data(), ctx->kind[k].segs.size(), ctx->st));
  }
  ctx->part_region = (maxblk + 1) * kMaxCand;
  CK(ctx->partials.ensure(sizeof(double) * (size_t)ctx->part_region * 3));
  CK(upload(ctx->md_d, ctx->md.data(), ctx->md.size(), ctx->st));
  return ensure_query_buffers(ctx);
}

KArgs make_args(hexopt_ctx *c) {
  KArgs a{};
  a.mesh = c->md_d.as<MeshDesc>();
  a.sc = c->sc_d.as<MeshScalars>();
  a.hseg = c->kind[K_HEX].dev.as<Seg>();
  a.vseg = c->kind[K_VERT].dev.as<Seg>();
  a.cseg = c->kind[K_CONS].dev.as<Seg>();
  a.hblk = c->kind[K_HEX].nblk;
  a.partials = c->partials.as<double>();
  a.counters = c->counters.as<unsigned>();
  a.hexv = c->hexv.as<uint32_t>();
  a.gslot = c->gslot.as<int32_t>();
  a.X = c->X.as<double>();
  a.X32 = c->X32.as<float>();
  a.aL = c->aL.as<double>();
  a.Sinv = c->Sinv.p;
  a.Ccoef = c->Ccoef.p;
  a.Bgen = c->Bgen.as<double>();
  a.Bref = nullptr;
  if (c->rest_fixed) {  // every hex has a slot (its own index) and a general reference shape
    a.gslot = c->gslot_all.as<int32_t>();
    a.Bgen = c->Bgen_all.as<double>();
    a.Bref = c->Bref.as<double>();
  }
  a.b = c->b.p; a.diag = c->diag.p; a.ba = c->ba.p; a.diaga = c->diaga.p;
  a.d = c->d.p; a.r = c->r.p; a.p = c->p.p; a.q = c->q.p; a.invd = c->invd.p;
  a.da = c->da.p; a.ra = c->ra.p; a.pa = c->pa.p; a.qa = c->qa.p; a.invda = c->invda.p;
  a.Rrot = c->Rrot.as<float>();
  a.dd = c->dd.as<double>();
  a.dda = c->dda.as<double>();
  a.ddf = c->ddf.as<float>();
  a.cg_refine = c->params.cg_refine > 0 ? c->params.cg_refine : 10;
  a.c_ids = c->c_ids.as<int32_t>(); a.c_pos = c->c_pos.as<double>();
  a.t_ids = c->t_ids.as<int32_t>(); a.t_nrm = c->t_nrm.as<double>(); a.t_dis = c->t_dis.as<double>();
  a.l_ids = c->l_ids.as<int32_t>(); a.l_axis = c->l_axis.as<double>(); a.l_orig = c->l_orig.as<double>();
  a.b_ids = c->b_ids.as<int32_t>(); a.b_pos = c->b_pos.as<double>();
  a.g_ptr = c->g_ptr.as<int64_t>(); a.g_vs = c->g_vs.as<int32_t>();
  a.vfix = c->vfix.as<uint8_t>();
  a.has_fixed = c->has_fixed ? 1 : 0;
  a.energy = c->params.energy;
  a.cg_max_iter = c->params.cg_max_iter;
  a.ls_cand = c->params.ls_candidates;
  a.cg_tol = c->params.cg_tol;
  a.sc_exp_f = c->params.exp_factor;
  a.hthreads = c->block[K_HEX];
  a.vthreads = c->block[K_VERT];
  a.Xa = c->Xa.as<double>();
  a.grad = c->grad.as<double>();
  a.root_list = c->root_list.as<uint32_t>();
  a.root_mesh = c->root_mesh.as<int32_t>();
  a.root_count = c->root_count.as<unsigned>();
  a.root_min = c->root_min.as<unsigned long long>();
  a.ls_active = c->root_count.as<unsigned>() + 1;
  a.ls_round = c->root_count.as<unsigned>() + 2;
  a.n_meshes = c->n_meshes;
  return a;
}

int alloc_vectors(hexopt_ctx *ctx) {
  const size_t nv4 = (size_t)std::max<int64_t>(ctx->NV, 1) * 4;
  const size_t nl = (size_t)std::max<int64_t>(ctx->NL, 1);
  const size_t vt = ctx->mixed ? sizeof(float) : sizeof(double);
  for (DBuf *bf : {&ctx->b, &ctx->diag, &ctx->d, &ctx->r, &ctx->p, &ctx->q, &ctx->invd}) CK(bf->ensure(nv4 * vt));
  CK(ctx->aL.ensure(nl * sizeof(double)));
  for (DBuf *bf : {&ctx->ba, &ctx->diaga, &ctx->da, &ctx->ra, &ctx->pa, &ctx->qa, &ctx->invda}) CK(bf->ensure(nl * vt));
  const size_t nt = (size_t)((ctx->NH + 31) / 32 * 32) * 8;
  CK(ctx->Sinv.ensure(nt * vt));
  CK(ctx->Ccoef.ensure(nt * 6 * vt));
  CK(ctx->Bgen.ensure((size_t)std::max<int64_t>(ctx->NG, 1) * 8 * 9 * sizeof(double)));
  if (ctx->mixed) {
    CK(ctx->Rrot.ensure(nt * 9 * sizeof(float)));
    CK(ctx->dd.ensure(nv4 * sizeof(double)));
    CK(ctx->dda.ensure(nl * sizeof(double)));
    CK(ctx->ddf.ensure(nv4 * sizeof(float)));
  }
  // every corner tet may need the exact root: the list holds all of them
  const size_t nroot = (size_t)ctx->NH * 8;
  CK(ctx->root_list.ensure(nroot * sizeof(uint32_t)));
  CK(ctx->root_mesh.ensure(nroot * sizeof(int32_t)));
  CK(ctx->root_count.ensure(3 * sizeof(unsigned)));  // [0] root-list length, [1] line searches open, [2] round
  CK(ctx->root_min.ensure(sizeof(unsigned long long) * ctx->n_meshes));
  {
    CK(cudaMemsetAsync(ctx->root_count.p, 0, 3 * sizeof(unsigned), ctx->st));
    std::vector<double> inf(ctx->n_meshes, INFINITY);
    CK(cudaMemcpyAsync(ctx->root_min.p, inf.data(), sizeof(double) * ctx->n_meshes, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  return HEXOPT_OK;
}

// compute_referenceMesh for the general shapes: every hex gets a slot (its index) and Bref from its
// reference corners (set_reference_hexes) or from the current positions.
int build_ref_shapes(hexopt_ctx *ctx) {
  const size_t nt = (size_t)ctx->NH * 8;
  CK(ctx->Bref.ensure(nt * 9 * sizeof(double)));
  CK(ctx->Bgen_all.ensure(nt * 9 * sizeof(double)));
  if (ctx->gslot_all.bytes < sizeof(int32_t) * (size_t)ctx->NH) {
    std::vector<int32_t> id(ctx->NH);
    for (int64_t h = 0; h < ctx->NH; h++) id[h] = (int32_t)h;
    CK(upload(ctx->gslot_all, id.data(), id.size(), ctx->st));
  }
  if (ctx->has_ref_tets)
    launch_ref_from_tets(ctx->ref_p8.as<double>(), ctx->NH * 8, ctx->Bref.as<double>(), ctx->st);
  else
    launch_ref_shapes(ctx->has_ref_p8 ? ctx->ref_p8.as<double>() : nullptr, ctx->hexv.as<uint32_t>(),
                      ctx->X.as<double>(), ctx->hflag_d.as<uint8_t>(), ctx->params.cube, ctx->NH,
                      ctx->Bref.as<double>(), ctx->st);
  ctx->launches++;
  CKL();
  return HEXOPT_OK;
}

int push_scalars(hexopt_ctx *ctx) {
  CK(upload(ctx->sc_d, ctx->sc.data(), ctx->sc.size(), ctx->st));
  return HEXOPT_OK;
}
int pull_scalars(hexopt_ctx *ctx) {
  CK(cudaMemcpyAsync(ctx->sc.data(), ctx->sc_d.p, sizeof(MeshScalars) * ctx->sc.size(), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

// ------------------------------------------------------------------ SLIM stages
template <typename ET, typename VT>
int run_precompute(hexopt_ctx *ctx) {
  KArgs a = make_args(ctx);
  launch_precompute<ET, VT>(a, ctx->kind[K_HEX].nblk, ctx->st);
  ctx->launches += 1;
  CKL();
  return HEXOPT_OK;
}

int run_projection(hexopt_ctx *ctx, cudaStream_t s = nullptr);
static cudaError_t ensure_side_streams(hexopt_ctx *ctx);

template <typename ET, typename VT>
int run_iteration(hexopt_ctx *ctx, bool pre, bool project) {
  KArgs a = make_args(ctx);
  cudaStream_t st = ctx->st;
  if (project) {
    // the feature projection (tangent planes and line targets for the soft terms) beside the
    // local step, which reads only positions and writes only the elastic terms; joined before
    // the soft terms are assembled
    CK(ensure_side_streams(ctx));
    CK(cudaEventRecord(ctx->ev_pfork, st));
    CK(cudaStreamWaitEvent(ctx->hs0, ctx->ev_pfork, 0));
    int rc = run_projection(ctx, ctx->hs0);
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev_proj, ctx->hs0));
  }
  const size_t nv4 = (size_t)ctx->NV * 4;
  CK(cudaMemsetAsync(ctx->b.p, 0, nv4 * sizeof(VT), st));
  CK(cudaMemsetAsync(ctx->diag.p, 0, nv4 * sizeof(VT), st));
  CK(cudaMemsetAsync(ctx->r.p, 0, nv4 * sizeof(VT), st));
  const int64_t hb = ctx->kind[K_HEX].nblk, vb = ctx->kind[K_VERT].nblk, cb = ctx->kind[K_CONS].nblk;
  launch_local<ET, VT>(a, hb, pre, st);
  if (project) CK(cudaStreamWaitEvent(st, ctx->ev_proj, 0));
  launch_soft_rhs<VT>(a, cb, st);
  ctx->launches += 2;
  if (ctx->has_fixed) {  // q = L_ib x_b for the known-value solve's rhs norm
    launch_fixed_pre<VT>(a, hb, vb, st);
    ctx->launches += 2;
  }
  const int iters = ctx->params.cg_max_iter;
  if (sizeof(VT) == 4) {
    // mixed: FP32 PCG on the update, anchored to the FP64 positions by residual replacements
    CK(cudaMemsetAsync(ctx->dd.p, 0, nv4 * sizeof(double), st));
    if (ctx->NL) CK(cudaMemsetAsync(ctx->dda.p, 0, (size_t)ctx->NL * sizeof(double), st));
    launch_ir_residual(a, hb, vb, cb, false, st);
    ctx->launches += kLaunchesIrInitial;
  }
  launch_cg_start<VT>(a, vb, st);
  ctx->launches += 1;
  for (int i = 0; i < iters; i++) {
    const bool replace = sizeof(VT) == 4 && (i + 1) % a.cg_refine == 0 && i + 1 < iters;
    launch_cg_iter<VT>(a, hb, vb, cb, st, !replace);
    ctx->launches += kLaunchesCgIter - (replace ? 1 : 0);
    if (replace) {
      launch_ir_residual(a, hb, vb, cb, true, st);
      launch_cg_dir<VT>(a, vb, st);
      ctx->launches += kLaunchesIrReplace + 1;
    }
  }
  if (sizeof(VT) == 4) {
    launch_ir_final(a, vb, st);
    ctx->launches += kLaunchesIrFinal;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(st, &cs));
  CK(ensure_side_streams(ctx));
  CK((launch_line_search<ET, VT>(a, hb, vb, cb, st, ctx->graph_conditionals ? ctx->lsb : nullptr)));
  const int rounds = (kHalvings + 1 + ctx->params.ls_candidates - 1) / ctx->params.ls_candidates;
  // captured: the rounds are a WHILE node, counted here as one iteration (3 kernels)
  ctx->launches += cs == cudaStreamCaptureStatusActive && ctx->graph_conditionals ? 5 + 3 : 5 + 2 * rounds;
  CKL();
  return HEXOPT_OK;
}

int dispatch_precompute(hexopt_ctx *ctx) {
  return ctx->mixed ? run_precompute<float, float>(ctx) : run_precompute<double, double>(ctx);
}
int dispatch_iteration(hexopt_ctx *ctx, bool pre = false, bool project = false) {
  return ctx->mixed ? run_iteration<float, float>(ctx, pre, project) : run_iteration<double, double>(ctx, pre, project);
}

// SLIMData::energy is the accepted total divided by mesh_area = sum of M over the tets
// (slim_m.cpp:1129-1130, 1284-1285).
void fill_report(const MeshScalars &S, int64_t nh, hexopt_slim_report &r) {
  r.energy = S.energy / (S.M * 8.0 * (double)nh);
  r.energy_quality = S.eq;
  r.energy_soft = S.es;
  r.cg_error = S.cg_error;
  r.max_step = S.max_step;
  r.step = S.step;
  r.cg_iters = S.cg_iters;
  r.halvings = S.halvings;
  r.status = S.status;
  r.pad = 0;
}

// ------------------------------------------------------------------ BVH builds
// oriented: also the oriented node records (trees that the target queries walk)
int build_static_bvh(hexopt_ctx *ctx, StaticBvh &B, const std::vector<double> &tri, int64_t nf, bool oriented) {
  B.n = (int32_t)nf;
  if (nf == 0) return HEXOPT_OK;
  CK(upload(B.tri, tri.data(), tri.size(), ctx->st));
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t f = 0; f < nf; f++)
    for (int c = 0; c < 3; c++) {
      const double *p = &tri[f * 9 + c * 3];
      double cen = (tri[f * 9 + c] + tri[f * 9 + 3 + c] + tri[f * 9 + 6 + c]) / 3;
      (void)p;
      lo[c] = std::min(lo[c], cen);
      hi[c] = std::max(hi[c], cen);
    }
  CK(B.child.ensure(sizeof(int32_t) * 2 * std::max<int64_t>(nf - 1, 1)));
  CK(B.parent.ensure(sizeof(int32_t) * (2 * nf - 1)));
  CK(B.box.ensure(sizeof(float) * 6 * (2 * nf - 1)));
  CK(B.leaf_face.ensure(sizeof(int32_t) * nf));
  CK(B.counters.ensure(sizeof(unsigned) * std::max<int64_t>(nf - 1, 1)));
  CK(cudaMemsetAsync(B.counters.p, 0, sizeof(unsigned) * std::max<int64_t>(nf - 1, 1), ctx->st));
  CK(B.node.ensure(sizeof(float4) * 4 * std::max<int64_t>(nf - 1, 1)));
  CK(B.leafd.ensure(sizeof(float4) * 3 * nf));
  DBuf keys, keys2, tmp, range, obb;
  if (oriented && nf > 1) {
    CK(range.ensure(sizeof(int32_t) * 2 * (nf - 1)));
    CK(obb.ensure(sizeof(float4) * 4 * (2 * nf - 1)));
    CK(B.onode.ensure(sizeof(float4) * 8 * (nf - 1)));
  }
  CK(keys.ensure(sizeof(unsigned long long) * nf));
  CK(keys2.ensure(sizeof(unsigned long long) * nf));
  BvhDev bd = B.dev();
  bvh_morton(bd, lo, hi, keys.as<unsigned long long>(), ctx->st);
  size_t tb = 0;
  CK(cub::DeviceRadixSort::SortKeys(nullptr, tb, keys.as<unsigned long long>(), keys2.as<unsigned long long>(), (int)nf, 0, 64, ctx->st));
  CK(tmp.ensure(tb));
  CK(cub::DeviceRadixSort::SortKeys(tmp.p, tb, keys.as<unsigned long long>(), keys2.as<unsigned long long>(), (int)nf, 0, 64, ctx->st));
  bvh_karras((int)nf, keys2.as<unsigned long long>(), B.child.as<int32_t>(), B.parent.as<int32_t>(), B.leaf_face.as<int32_t>(), ctx->st,
             range.as<int32_t>());
  bd = B.dev();
  bvh_refit(bd, B.box.as<float>(), B.parent.as<int32_t>(), B.counters.as<unsigned>(), B.node.as<float4>(),
            B.leafd.as<float4>(), ctx->st);
  ctx->launches += 5;
  if (oriented && nf > 1) {
    bvh_orient(bd, range.as<int32_t>(), obb.as<float4>(), B.onode.as<float4>(), ctx->st);
    ctx->launches += 3;
  }
  CKL();
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

int upload_targets_table(hexopt_ctx *ctx) {
  std::vector<TargetDev> td(ctx->n_meshes);
  for (int m = 0; m < ctx->n_meshes; m++) {
    TargetDev t{};
    TargetHost &h = ctx->tgt[m];
    if (h.set) {
      t.bvh = h.bvh.dev();
      t.TV = h.TVd.as<double>();
      t.tri = h.bvh.tri.as<double>();
      t.FN = h.FN.as<double>();
      t.EP = h.EP.as<double>();
      t.VNc = h.VNc.as<double>();
      t.ENc = h.ENc.as<double>();
      t.curve_ptr = h.curve_ptr.as<int64_t>();
      t.curve_vs = h.curve_vs.as<int32_t>();
      t.curve_closed = h.curve_closed.as<uint8_t>();
    }
    td[m] = t;
  }
  CK(upload(ctx->tgt_d, td.data(), td.size(), ctx->st));
  std::vector<BvhDev> sd(ctx->n_meshes);
  for (int m = 0; m < ctx->n_meshes; m++) {
    BvhDev b{};
    SurfaceHost &s = ctx->surf[m];
    if (s.set) {
      b.n = (int32_t)s.nf;
      b.child = s.child.as<int32_t>();
      b.box = s.box.as<float>();
      b.leaf_face = s.leaf_face.as<int32_t>();
      b.F = s.F.as<int32_t>();
      b.X = ctx->X.as<double>();
      b.node = s.node.as<float4>();
      b.leafd = s.leafd.as<float4>();
    }
    sd[m] = b;
  }
  CK(upload(ctx->surf_d, sd.data(), sd.size(), ctx->st));
  std::vector<RefitDev> rd(ctx->n_meshes);
  for (int m = 0; m < ctx->n_meshes; m++) {
    RefitDev r{};
    SurfaceHost &s = ctx->surf[m];
    r.b = sd[m];
    if (s.set) {
      r.box = s.box.as<float>();
      r.parent = s.parent.as<int32_t>();
      r.counters = s.counters.as<unsigned>();
      r.node = s.node.as<float4>();
      r.leafd = s.leafd.as<float4>();
    }
    rd[m] = r;
  }
  CK(upload(ctx->refit_d, rd.data(), rd.size(), ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

int ensure_query_buffers(hexopt_ctx *ctx) {
  int64_t n = 1;
  for (int k : {K_PROJ, K_TGTV, K_SURFV}) {
    int64_t tot = 0;
    for (int m = 0; m < ctx->n_meshes; m++) tot += ctx->md[m].kcount[k];
    n = std::max(n, tot);
  }
  CK(ctx->qseed.ensure(sizeof(int32_t) * 3 * n));
  CK(cudaMemsetAsync(ctx->qseed.p, 0xFF, sizeof(int32_t) * 3 * n, ctx->st));  // -1: no seed yet
  ctx->qseed_n = n;
  // up to kQueryCandidates recorded candidates per query on average (a query over its share goes
  // to the exact fallback)
  constexpr int64_t kQueryCandidates = 16;
  for (QueryBufs &q : ctx->qb) {
    CK(q.ovf_item.ensure(sizeof(int64_t) * n));
    CK(q.ovf_mesh.ensure(sizeof(int32_t) * n));
    CK(q.ovf_count.ensure(sizeof(unsigned)));
    CK(q.ovf_best.ensure(sizeof(double) * n));
    CK(q.ovf_face.ensure(sizeof(int32_t) * n));
    CK(q.ovf_pt.ensure(sizeof(double) * 3 * n));
    CK(q.hdist.ensure(sizeof(double) * n));
    q.cand_cap = kQueryCandidates * n;
    CK(q.cand_leaf.ensure(sizeof(int32_t) * q.cand_cap));
    CK(q.cand_qi.ensure(sizeof(int32_t) * q.cand_cap));
    CK(q.cand_x.ensure(sizeof(double) * q.cand_cap));
    CK(q.cand_d.ensure(sizeof(double) * q.cand_cap));
    CK(q.cand_count.ensure(sizeof(unsigned)));
    CK(q.q_off.ensure(sizeof(int32_t) * n));
    CK(q.q_cnt.ensure(sizeof(int32_t) * n));
    CK(q.qpos.ensure(sizeof(double) * 3 * n));
    CK(q.q_mesh.ensure(sizeof(int32_t) * n));
    CK(q.fb_count.ensure(sizeof(unsigned)));
    CK(q.fb_item.ensure(sizeof(int64_t) * n));
    CK(q.fb_mesh.ensure(sizeof(int32_t) * n));
  }
  return HEXOPT_OK;
}

CandBuf make_cand(const QueryBufs &q) {
  CandBuf b{};
  b.leaf = q.cand_leaf.as<int32_t>();
  b.qi = q.cand_qi.as<int32_t>();
  b.x = q.cand_x.as<double>();
  b.d = q.cand_d.as<double>();
  b.count = q.cand_count.as<unsigned>();
  b.cap = q.cand_cap;
  b.q_off = q.q_off.as<int32_t>();
  b.q_cnt = q.q_cnt.as<int32_t>();
  b.qpos = q.qpos.as<double>();
  b.q_mesh = q.q_mesh.as<int32_t>();
  b.fb_count = q.fb_count.as<unsigned>();
  b.fb_item = q.fb_item.as<int64_t>();
  b.fb_mesh = q.fb_mesh.as<int32_t>();
  return b;
}

Overflow make_ovf(const QueryBufs &q) {
  Overflow o{};
  o.item = q.ovf_item.as<int64_t>();
  o.mesh = q.ovf_mesh.as<int32_t>();
  o.count = q.ovf_count.as<unsigned>();
  o.best = q.ovf_best.as<double>();
  o.face = q.ovf_face.as<int32_t>();
  o.pt = q.ovf_pt.as<double>();
  return o;
}

ProjArgs make_proj(hexopt_ctx *c, int kind) {
  ProjArgs p{};
  p.ovf = make_ovf(c->qb[0]);
  p.cand = make_cand(c->qb[0]);
  p.seg = c->kind[kind].dev.as<Seg>();
  p.mesh = c->md_d.as<MeshDesc>();
  p.sc = c->sc_d.as<MeshScalars>();
  p.tgt = c->tgt_d.as<TargetDev>();
  p.X = c->X.as<double>();
  p.t_ids = c->t_ids.as<int32_t>(); p.t_nrm = c->t_nrm.as<double>(); p.t_dis = c->t_dis.as<double>();
  p.l_ids = c->l_ids.as<int32_t>(); p.l_curve = c->l_curve.as<int32_t>();
  p.l_axis = c->l_axis.as<double>(); p.l_orig = c->l_orig.as<double>();
  p.seed = c->qseed.as<int32_t>();
  p.budget = c->query_budget > 0 ? c->query_budget : 128;  // no benchmark projection query needs more
  return p;
}

HausArgs make_haus(hexopt_ctx *c, int kind) {
  HausArgs h{};
  const int set = kind == K_TGTV ? 1 : 0, region = kind == K_TGTV ? 2 : 1;  // side 0: set 1, region 2
  h.ovf = make_ovf(c->qb[set]);
  h.cand = make_cand(c->qb[set]);
  h.dist = c->qb[set].hdist.as<double>();
  h.seg = c->kind[kind].dev.as<Seg>();
  h.mesh = c->md_d.as<MeshDesc>();
  h.sc = c->sc_d.as<MeshScalars>();
  h.tgt = c->tgt_d.as<TargetDev>();
  h.surf = c->surf_d.as<BvhDev>();
  h.hm = c->hm_d.as<HausMesh>();
  h.X = c->X.as<double>();
  h.tgt_vs = c->tgt_vs_d.as<int64_t>();
  h.surf_vs = c->surf_vs_d.as<int64_t>();
  h.partials = c->partials.as<double>() + region * c->part_region;
  h.counters = c->counters.as<unsigned>() + region * c->n_meshes;
  h.seed = c->qseed.as<int32_t>() + (kind == K_SURFV ? 2 : 1) * c->qseed_n;
  h.budget = c->query_budget > 0 ? c->query_budget : 96;  // side 0's long queries do better cooperatively
  return h;
}

int run_projection(hexopt_ctx *ctx, cudaStream_t s) {
  if (!s) s = ctx->st;
  if (ctx->NT) {
    launch_project(make_proj(ctx, K_PROJ), ctx->kind[K_PROJ].nblk, s);
    ctx->launches += 5;
  }
  if (ctx->NL) {
    launch_curve_project(make_proj(ctx, K_LINE), ctx->kind[K_LINE].nblk, s);
    ctx->launches++;
  }
  CKL();
  return HEXOPT_OK;
}

static cudaError_t ensure_side_streams(hexopt_ctx *ctx) {
  if (ctx->hs0) return cudaSuccess;
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->hs0, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->hsj, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->lsb, cudaStreamNonBlocking);
  for (cudaEvent_t *ev : {&ctx->ev_fork, &ctx->ev_bbox, &ctx->ev_side0, &ctx->ev_sj, &ctx->ev_pfork, &ctx->ev_proj})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  return e;
}

// The scaled-Jacobian check of a step (fast FP32 screen in mixed mode, the bit-exact pass in FP64).
static void launch_step_sj(hexopt_ctx *ctx, cudaStream_t s) {
  KArgs a = make_args(ctx);
  if (ctx->mixed) launch_sj_check(a, ctx->kind[K_HEX].nblk, s);
  else launch_scaled_jacobian(a, ctx->kind[K_HEX].nblk, nullptr, ctx->HJs.as<double>(), s);
  ctx->launches += 3;
}

// Both Hausdorff sides at the current positions, side 0 (with the refit of the hex-boundary trees
// it searches) on a second stream, side 1 on the context's stream; with_sj also runs the step's
// SJ check on a third.  The branches share only the bbox diagonal (written before either side
// starts) and join before the two sides' results are combined.  Inside a capture the branches
// become parallel graph branches.
int run_hausdorff(hexopt_ctx *ctx, bool with_sj) {
  CK(ensure_side_streams(ctx));
  cudaStream_t st = ctx->st, s0 = ctx->hs0;
  CK(cudaEventRecord(ctx->ev_fork, st));
  if (with_sj) {
    CK(cudaStreamWaitEvent(ctx->hsj, ctx->ev_fork, 0));
    launch_step_sj(ctx, ctx->hsj);
    CK(cudaEventRecord(ctx->ev_sj, ctx->hsj));
  }
  CK(cudaStreamWaitEvent(s0, ctx->ev_fork, 0));
  // refit every mesh's surface tree at the current positions, one launch for the batch
  if (ctx->n_surf_faces > 0) {
    bvh_refit_batch(ctx->refit_d.as<RefitDev>(), ctx->kind[K_SURFF].dev.as<Seg>(), ctx->md_d.as<MeshDesc>(),
                    ctx->kind[K_SURFF].nblk, ctx->block[K_SURFF] * ctx->ipt[K_SURFF], s0);
    ctx->launches += 1;
  }
  launch_haus_bbox(make_haus(ctx, K_SURFV), ctx->kind[K_SURFV].nblk, st);
  CK(cudaEventRecord(ctx->ev_bbox, st));
  CK(cudaStreamWaitEvent(s0, ctx->ev_bbox, 0));
  launch_haus_side(make_haus(ctx, K_TGTV), 0, ctx->kind[K_TGTV].nblk, s0);
  CK(cudaEventRecord(ctx->ev_side0, s0));
  launch_haus_side(make_haus(ctx, K_SURFV), 1, ctx->kind[K_SURFV].nblk, st);
  CK(cudaStreamWaitEvent(st, ctx->ev_side0, 0));
  if (with_sj) CK(cudaStreamWaitEvent(st, ctx->ev_sj, 0));
  launch_haus_combine(ctx->hm_d.as<HausMesh>(), ctx->n_meshes, st);
  ctx->launches += 14;
  CKL();
  return HEXOPT_OK;
}

int check_ctx(hexopt_ctx *ctx) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (ctx->n_meshes <= 0) return fail(ctx, HEXOPT_ERR_STATE, "no meshes uploaded");
  return HEXOPT_OK;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

int hexopt_create(hexopt_ctx **out, int device) {
  if (!out) return HEXOPT_ERR_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return HEXOPT_ERR_CUDA;
  if (device < 0 || device >= n) return HEXOPT_ERR_ARG;
  hexopt_ctx *ctx = new hexopt_ctx();
  ctx->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete ctx;
    return HEXOPT_ERR_CUDA;
  }
  ctx->params.energy = HEXOPT_SYMMETRIC_DIRICHLET;
  ctx->params.precision = HEXOPT_FP64;
  ctx->params.weight_opt = 1.0;
  ctx->params.exp_factor = 1.0;  // slim_precompute leaves SLIMData::exp_factor at 1 (slim_m.cpp:1125)
  ctx->params.cg_max_iter = 20;
  ctx->params.cg_tol = 1e-8;
  ctx->params.ls_candidates = 1;
  ctx->params.cube = 1;
  *out = ctx;
  return HEXOPT_OK;
}

void hexopt_destroy(hexopt_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->ust) cudaStreamSynchronize(ctx->ust);
  if (ctx->dst) cudaStreamSynchronize(ctx->dst);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (cudaEvent_t e : {ctx->in_ready, ctx->in_free, ctx->out_ready, ctx->out_done, ctx->ev_xfinal})
    if (e) cudaEventDestroy(e);
  if (ctx->hs0) cudaStreamSynchronize(ctx->hs0);
  if (ctx->hsj) cudaStreamSynchronize(ctx->hsj);
  for (cudaEvent_t e : {ctx->ev_fork, ctx->ev_bbox, ctx->ev_side0, ctx->ev_sj, ctx->ev_pfork, ctx->ev_proj})
    if (e) cudaEventDestroy(e);
  if (ctx->hs0) cudaStreamDestroy(ctx->hs0);
  if (ctx->hsj) cudaStreamDestroy(ctx->hsj);
  if (ctx->lsb) cudaStreamDestroy(ctx->lsb);
  if (ctx->ust) cudaStreamDestroy(ctx->ust);
  if (ctx->dst) cudaStreamDestroy(ctx->dst);
  if (ctx->st) cudaStreamDestroy(ctx->st);
  delete ctx;
}

const char *hexopt_last_error(const hexopt_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int hexopt_sync(hexopt_ctx *ctx) {
  if (!ctx) return HEXOPT_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->st));
  if (ctx->ust) CK(cudaStreamSynchronize(ctx->ust));
  if (ctx->dst) CK(cudaStreamSynchronize(ctx->dst));
  if (ctx->hs0) CK(cudaStreamSynchronize(ctx->hs0));
  if (ctx->hsj) CK(cudaStreamSynchronize(ctx->hsj));
  return HEXOPT_OK;
}

int64_t hexopt_num_vertices(const hexopt_ctx *ctx) { return ctx ? ctx->NV : 0; }
int64_t hexopt_num_hexes(const hexopt_ctx *ctx) { return ctx ? ctx->NH : 0; }
int hexopt_num_meshes(const hexopt_ctx *ctx) { return ctx ? ctx->n_meshes : 0; }
int64_t hexopt_launch_count(const hexopt_ctx *ctx) { return ctx ? ctx->launches : 0; }

int hexopt_set_ordering(hexopt_ctx *ctx, int mode) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (mode < 0 || mode > 2) return fail(ctx, HEXOPT_ERR_ARG, "set_ordering: mode must be 0, 1 or 2");
  ctx->ordering = mode;
  return HEXOPT_OK;
}

int hexopt_upload_meshes(hexopt_ctx *ctx, int n_meshes, const int64_t *nv, const int64_t *nh, const double *V,
                         const uint32_t *H, const uint8_t *h_flag) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (n_meshes <= 0 || !nv || !nh || !V || !H) return fail(ctx, HEXOPT_ERR_ARG, "upload_meshes: bad arguments");
  CK(cudaSetDevice(ctx->device));
  int64_t NV = 0, NH = 0;
  for (int m = 0; m < n_meshes; m++) {
    if (nv[m] <= 0 || nh[m] <= 0) return fail(ctx, HEXOPT_ERR_ARG, "mesh %d: empty (nv=%lld nh=%lld)", m, (long long)nv[m], (long long)nh[m]);
    NV += nv[m];
    NH += nh[m];
  }
  if (NV >= (int64_t)UINT32_MAX) return fail(ctx, HEXOPT_ERR_ARG, "too many vertices in one batch");
  if (NH >= ((int64_t)1 << 29)) return fail(ctx, HEXOPT_ERR_ARG, "too many hexes in one batch (limit 2^29)");
  // validate hex ids (host, integer pass over the input)
  {
    int64_t ho = 0;
    for (int m = 0; m < n_meshes; m++) {
      for (int64_t i = 0; i < 8 * nh[m]; i++)
        if (H[8 * ho + i] >= (uint64_t)nv[m]) return fail(ctx, HEXOPT_ERR_ARG, "mesh %d: hex corner id out of range", m);
      ho += nh[m];
    }
  }
  ctx->n_meshes = n_meshes;
  ctx->NV = NV;
  ctx->NH = NH;
  ctx->md.assign(n_meshes, MeshDesc{});
  ctx->sc.assign(n_meshes, MeshScalars{});
  ctx->nC.assign(n_meshes, 0); ctx->nT.assign(n_meshes, 0); ctx->nL.assign(n_meshes, 0);
  ctx->nB.assign(n_meshes, 0); ctx->nG.assign(n_meshes, 0);
  ctx->NB = ctx->NGR = 0;
  ctx->fixed_h.assign(NV, 0);
  ctx->has_fixed = ctx->has_glue = false;
  ctx->lamC.assign(n_meshes, 0); ctx->lamT.assign(n_meshes, 0); ctx->lamL.assign(n_meshes, 0);
  ctx->tgt.clear(); ctx->tgt.resize(n_meshes);
  ctx->surf.clear(); ctx->surf.resize(n_meshes);
  ctx->tgt_vs_cnt.assign(n_meshes, 0);
  ctx->surf_vs_cnt.assign(n_meshes, 0);
  ctx->precomputed = false;
  ctx->fa_ready = false;
  ctx->haus_ready = false;
  if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
  int64_t vo = 0, ho = 0;
  for (int m = 0; m < n_meshes; m++) {
    ctx->md[m].v_off = vo; ctx->md[m].nv = nv[m];
    ctx->md[m].h_off = ho; ctx->md[m].nh = nh[m];
    vo += nv[m]; ho += nh[m];
  }
  CK(upload(ctx->stage, V, (size_t)NV * 3, ctx->st));
  ctx->H_h.assign(H, H + (size_t)NH * 8);
  CK(upload(ctx->stage2, H, (size_t)NH * 8, ctx->st));
  CK(ctx->X.ensure(sizeof(double) * 4 * NV));
  CK(ctx->X32.ensure(sizeof(float) * 8 * NV));
  const int64_t NHp = (NH + 31) / 32 * 32;
  CK(ctx->hexv.ensure(sizeof(uint32_t) * 8 * NHp));
  CK(cudaMemsetAsync(ctx->hexv.p, 0, sizeof(uint32_t) * 8 * NHp, ctx->st));
  ctx->ordered = ctx->ordering == 1 || (ctx->ordering == 2 && !numbering_coherent(ctx, n_meshes, nv, nh, H));
  ctx->vold2new_h.clear();
  ctx->hnew2old_h.clear();
  if (ctx->ordered) {
    // Morton order of every mesh's vertices and hexes inside its bounding box (device sort)
    std::vector<double> box(6 * n_meshes);
    std::vector<int64_t> voff(n_meshes + 1), hoff(n_meshes + 1);
    for (int m = 0; m < n_meshes; m++) {
      double *b = &box[6 * m];
      for (int d = 0; d < 3; d++) { b[d] = INFINITY; b[3 + d] = -INFINITY; }
      for (int64_t v = ctx->md[m].v_off; v < ctx->md[m].v_off + nv[m]; v++)
        for (int d = 0; d < 3; d++) { b[d] = std::min(b[d], V[3 * v + d]); b[3 + d] = std::max(b[3 + d], V[3 * v + d]); }
      voff[m] = ctx->md[m].v_off;
      hoff[m] = ctx->md[m].h_off;
    }
    voff[n_meshes] = NV;
    hoff[n_meshes] = NH;
    DBuf box_d, voff_d, hoff_d, scratch;
    CK(upload(box_d, box.data(), box.size(), ctx->st));
    CK(upload(voff_d, voff.data(), voff.size(), ctx->st));
    CK(upload(hoff_d, hoff.data(), hoff.size(), ctx->st));
    CK(ctx->vnew2old.ensure(sizeof(int32_t) * NV));
    CK(ctx->vold2new.ensure(sizeof(int32_t) * NV));
    CK(ctx->hnew2old.ensure(sizeof(int32_t) * NH));
    CK(ctx->hold2new.ensure(sizeof(int32_t) * NH));
    const size_t sb = order_scratch_bytes(NV, NH);
    CK(scratch.ensure(sb));
    CK(order_batch(ctx->stage.as<double>(), ctx->stage2.as<uint32_t>(), NV, NH, voff_d.as<int64_t>(), hoff_d.as<int64_t>(),
                   n_meshes, box_d.as<double>(), ctx->vnew2old.as<int32_t>(), ctx->vold2new.as<int32_t>(),
                   ctx->hnew2old.as<int32_t>(), ctx->hold2new.as<int32_t>(), scratch.p, sb, ctx->st));
    launch_rows_to_aos4_perm(ctx->stage.as<double>(), ctx->vnew2old.as<int32_t>(), NV, ctx->X.as<double>(), ctx->st);
    launch_hex_perm(ctx->stage2.as<uint32_t>(), ctx->hnew2old.as<int32_t>(), ctx->vold2new.as<int32_t>(), NH,
                    hoff_d.as<int64_t>(), voff_d.as<int64_t>(), n_meshes, ctx->hexv.as<uint32_t>(), ctx->st);
    ctx->vold2new_h.resize(NV);
    ctx->hnew2old_h.resize(NH);
    CK(cudaMemcpyAsync(ctx->vold2new_h.data(), ctx->vold2new.p, sizeof(int32_t) * NV, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(ctx->hnew2old_h.data(), ctx->hnew2old.p, sizeof(int32_t) * NH, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));  // the scratch buffers go out of scope
    ctx->launches += 8;
  } else {
    launch_rows_to_aos4(ctx->stage.as<double>(), ctx->X.as<double>(), NV, ctx->st);
    for (int m = 0; m < n_meshes; m++)
      launch_hex_to_aosoa_mesh(ctx->stage2.as<uint32_t>() + 8 * ctx->md[m].h_off, ctx->md[m].h_off, nh[m],
                               (uint32_t)ctx->md[m].v_off, ctx->hexv.as<uint32_t>(), ctx->st);
    ctx->launches += 1 + n_meshes;
  }
  launch_split_pos(ctx->X.as<double>(), ctx->X32.as<float>(), NV, ctx->st);
  ctx->launches += 1;
  // own-shape slots and h_flag, in the device's hex order
  std::vector<int32_t> gs(NH, -1);
  std::vector<uint8_t> hf(NH, 1);
  int64_t ng = 0;
  for (int64_t h = 0; h < NH; h++) {
    const int64_t o = ctx->ordered ? ctx->hnew2old_h[h] : h;
    if (h_flag && !h_flag[o]) { gs[h] = (int32_t)ng++; hf[h] = 0; }
  }
  ctx->NG = ng;
  CK(upload(ctx->gslot, gs.data(), gs.size(), ctx->st));
  CK(upload(ctx->hflag_d, hf.data(), hf.size(), ctx->st));
  ctx->has_ref_p8 = false;
  ctx->has_ref_tets = false;
  ctx->rest_fixed = false;
  CK(ctx->counters.ensure(sizeof(unsigned) * 3 * n_meshes));  // three regions (see part_region)
  CK(cudaMemsetAsync(ctx->counters.p, 0, sizeof(unsigned) * 3 * n_meshes, ctx->st));
  int rc = rebuild_tables(ctx);
  if (rc) return rc;
  CK(upload(ctx->sc_d, ctx->sc.data(), ctx->sc.size(), ctx->st));
  CK(ctx->HJs.ensure(sizeof(double) * NH));
  CK(cudaStreamSynchronize(ctx->st));
  CKL();
  return HEXOPT_OK;
}

int hexopt_set_positions(hexopt_ctx *ctx, const double *V) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!V) return fail(ctx, HEXOPT_ERR_ARG, "set_positions: NULL");
  CK(upload(ctx->stage, V, (size_t)ctx->NV * 3, ctx->st));
  launch_rows_to_aos4_perm(ctx->stage.as<double>(), vn2o(ctx), ctx->NV, ctx->X.as<double>(), ctx->st);
  launch_split_pos(ctx->X.as<double>(), ctx->X32.as<float>(), ctx->NV, ctx->st);
  ctx->launches += 2;
  CKL();
  return HEXOPT_OK;
}

static cudaError_t ensure_copy_streams(hexopt_ctx *ctx) {
  if (ctx->ust) return cudaSuccess;
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->ust, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->dst, cudaStreamNonBlocking);
  for (cudaEvent_t *ev : {&ctx->in_ready, &ctx->in_free, &ctx->out_ready, &ctx->out_done})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  return e;
}

int hexopt_set_positions_async(hexopt_ctx *ctx, const double *V) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!V) return fail(ctx, HEXOPT_ERR_ARG, "set_positions_async: NULL");
  CK(ensure_copy_streams(ctx));
  CK(ctx->in_stage.ensure(sizeof(double) * 3 * ctx->NV));
  // the copy waits until the previous input has been consumed, the compute stream until it lands
  CK(cudaStreamWaitEvent(ctx->ust, ctx->in_free, 0));
  CK(cudaMemcpyAsync(ctx->in_stage.p, V, sizeof(double) * 3 * ctx->NV, cudaMemcpyHostToDevice, ctx->ust));
  CK(cudaEventRecord(ctx->in_ready, ctx->ust));
  CK(cudaStreamWaitEvent(ctx->st, ctx->in_ready, 0));
  launch_rows_to_aos4_perm(ctx->in_stage.as<double>(), vn2o(ctx), ctx->NV, ctx->X.as<double>(), ctx->st);
  launch_split_pos(ctx->X.as<double>(), ctx->X32.as<float>(), ctx->NV, ctx->st);
  ctx->launches += 2;
  CKL();
  CK(cudaEventRecord(ctx->in_free, ctx->st));
  return HEXOPT_OK;
}

int hexopt_get_positions_async(hexopt_ctx *ctx, double *V) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!V) return fail(ctx, HEXOPT_ERR_ARG, "get_positions_async: NULL");
  CK(ensure_copy_streams(ctx));
  CK(ctx->out_stage.ensure(sizeof(double) * 3 * ctx->NV));
  // stage the positions after the work queued so far, once the previous copy has left the stage
  CK(cudaStreamWaitEvent(ctx->st, ctx->out_done, 0));
  launch_aos4_to_rows_perm(ctx->X.as<double>(), vo2n(ctx), ctx->NV, ctx->out_stage.as<double>(), ctx->st);
  ctx->launches++;
  CKL();
  CK(cudaEventRecord(ctx->out_ready, ctx->st));
  CK(cudaStreamWaitEvent(ctx->dst, ctx->out_ready, 0));
  CK(cudaMemcpyAsync(V, ctx->out_stage.p, sizeof(double) * 3 * ctx->NV, cudaMemcpyDeviceToHost, ctx->dst));
  CK(cudaEventRecord(ctx->out_done, ctx->dst));
  return HEXOPT_OK;
}

int hexopt_get_positions(hexopt_ctx *ctx, double *V) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!V) return fail(ctx, HEXOPT_ERR_ARG, "get_positions: NULL");
  CK(ctx->stage.ensure(sizeof(double) * 3 * ctx->NV));
  launch_aos4_to_rows_perm(ctx->X.as<double>(), vo2n(ctx), ctx->NV, ctx->stage.as<double>(), ctx->st);
  ctx->launches++;
  CK(cudaMemcpyAsync(V, ctx->stage.p, sizeof(double) * 3 * ctx->NV, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

int hexopt_scaled_jacobian(hexopt_ctx *ctx, double *V_Js, double *H_Js, hexopt_quality *q) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  KArgs a = make_args(ctx);
  double *vj = nullptr;
  if (V_Js) {
    CK(ctx->VJs.ensure(sizeof(double) * 8 * ctx->NH));
    vj = ctx->VJs.as<double>();
  }
  launch_scaled_jacobian(a, ctx->kind[K_HEX].nblk, vj, ctx->HJs.as<double>(), ctx->st);
  ctx->launches += 2;
  CKL();
  if (V_Js || H_Js) CK(ctx->stage.ensure(sizeof(double) * 8 * ctx->NH));
  if (V_Js) {  // the caller's hex order
    launch_gather_rows(vj, ho2n(ctx), ctx->NH, 8, ctx->stage.as<double>(), ctx->st);
    CK(cudaMemcpyAsync(V_Js, ctx->stage.p, sizeof(double) * 8 * ctx->NH, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  if (H_Js) {
    launch_gather_rows(ctx->HJs.as<double>(), ho2n(ctx), ctx->NH, 1, ctx->stage.as<double>(), ctx->st);
    CK(cudaMemcpyAsync(H_Js, ctx->stage.p, sizeof(double) * ctx->NH, cudaMemcpyDeviceToHost, ctx->st));
  }
  rc = pull_scalars(ctx);
  if (rc) return rc;
  if (q)
    for (int m = 0; m < ctx->n_meshes; m++) {
      const MeshScalars &S = ctx->sc[m];
      q[m].min_Jacobian = S.sj_min;
      q[m].ave_Jacobian = S.sj_sum / (double)ctx->md[m].nh;
      q[m].deviation_Jacobian = S.sj_dev;
      q[m].n_inverted = S.n_inv;
    }
  return HEXOPT_OK;
}

static int set_list(hexopt_ctx *ctx, const int64_t *counts, std::vector<int64_t> &dst, const int32_t *ids,
                    DBuf &ids_d, const char *what) {
  int64_t tot = 0;
  for (int m = 0; m < ctx->n_meshes; m++) {
    if (counts[m] < 0) return fail(ctx, HEXOPT_ERR_ARG, "%s: negative count", what);
    for (int64_t i = 0; i < counts[m]; i++)
      if (ids[tot + i] < 0 || ids[tot + i] >= ctx->md[m].nv) return fail(ctx, HEXOPT_ERR_ARG, "%s: vertex id out of range", what);
    tot += counts[m];
  }
  dst.assign(counts, counts + ctx->n_meshes);
  std::vector<int32_t> mapped(ids, ids + tot);
  if (ctx->ordered) {
    int64_t o = 0;
    for (int m = 0; m < ctx->n_meshes; m++)
      for (int64_t i = 0; i < counts[m]; i++, o++) mapped[o] = local_vid(ctx, m, mapped[o]);
  }
  CK(upload(ids_d, mapped.data(), (size_t)tot, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));  // the mapped copy goes out of scope
  return HEXOPT_OK;
}

int hexopt_set_corners(hexopt_ctx *ctx, const int64_t *nC, const int32_t *ids, const double *C) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = set_list(ctx, nC, ctx->nC, ids, ctx->c_ids, "set_corners");
  if (rc) return rc;
  int64_t tot = 0;
  for (int m = 0; m < ctx->n_meshes; m++) tot += nC[m];
  CK(upload(ctx->c_pos, C, (size_t)tot * 3, ctx->st));
  ctx->haus_ready = false;
  return rebuild_tables(ctx);
}

int hexopt_set_tangents(hexopt_ctx *ctx, const int64_t *nT, const int32_t *ids, const double *normal, const double *dis) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = set_list(ctx, nT, ctx->nT, ids, ctx->t_ids, "set_tangents");
  if (rc) return rc;
  int64_t tot = 0;
  for (int m = 0; m < ctx->n_meshes; m++) tot += nT[m];
  CK(upload(ctx->t_nrm, normal, (size_t)tot * 3, ctx->st));
  CK(upload(ctx->t_dis, dis, (size_t)tot, ctx->st));
  return rebuild_tables(ctx);
}

int hexopt_set_lines(hexopt_ctx *ctx, const int64_t *nL, const int32_t *ids, const double *axis, const double *origin) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = set_list(ctx, nL, ctx->nL, ids, ctx->l_ids, "set_lines");
  if (rc) return rc;
  int64_t tot = 0;
  for (int m = 0; m < ctx->n_meshes; m++) tot += nL[m];
  CK(upload(ctx->l_axis, axis, (size_t)tot * 3, ctx->st));
  CK(upload(ctx->l_orig, origin, (size_t)tot * 3, ctx->st));
  ctx->NL = tot;
  ctx->precomputed = false;  // unknown count changed
  return rebuild_tables(ctx);
}

int hexopt_set_projection(hexopt_ctx *ctx, const int64_t *nB, const int32_t *ids, const double *bc,
                          const double *lamda_projection) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!nB) return fail(ctx, HEXOPT_ERR_ARG, "set_projection: NULL counts");
  rc = set_list(ctx, nB, ctx->nB, ids, ctx->b_ids, "set_projection");
  if (rc) return rc;
  int64_t tot = 0;
  for (int m = 0; m < ctx->n_meshes; m++) tot += nB[m];
  CK(upload(ctx->b_pos, bc, (size_t)tot * 3, ctx->st));
  ctx->NB = tot;
  if (lamda_projection) {
    rc = pull_scalars(ctx);
    if (rc) return rc;
    for (int m = 0; m < ctx->n_meshes; m++) ctx->sc[m].lamda_P = lamda_projection[m];
    rc = push_scalars(ctx);
    if (rc) return rc;
  }
  return rebuild_tables(ctx);
}

int hexopt_set_glue(hexopt_ctx *ctx, const int64_t *n_groups, const int64_t *group_ptr, const int32_t *group_vs,
                    const double *lamda_glue) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!n_groups) return fail(ctx, HEXOPT_ERR_ARG, "set_glue: NULL counts");
  std::vector<int64_t> gp(1, 0);
  std::vector<int32_t> gv;
  int64_t po = 0, vo = 0;
  for (int m = 0; m < ctx->n_meshes; m++) {
    if (n_groups[m] < 0) return fail(ctx, HEXOPT_ERR_ARG, "set_glue: negative group count");
    if (n_groups[m] > 0 && ctx->nL[m] > 0)
      return fail(ctx, HEXOPT_ERR_UNSUPPORTED, "mesh %d: glue groups replace the feature terms; clear its feature lines first", m);
    if (n_groups[m] > 0 && (!group_ptr || !group_vs)) return fail(ctx, HEXOPT_ERR_ARG, "set_glue: NULL groups");
    const int64_t *pm = group_ptr + po + m;  // n_groups[m] + 1 entries per mesh
    std::vector<uint8_t> seen(ctx->md[m].nv, 0);
    for (int64_t g = 0; g < n_groups[m]; g++) {
      if (pm[g + 1] <= pm[g]) return fail(ctx, HEXOPT_ERR_ARG, "mesh %d: empty or unordered glue group %lld", m, (long long)g);
      for (int64_t k = pm[g]; k < pm[g + 1]; k++) {
        const int32_t v = group_vs[vo + (k - pm[0])];
        if (v < 0 || v >= ctx->md[m].nv) return fail(ctx, HEXOPT_ERR_ARG, "mesh %d: glue vertex id out of range", m);
        if (seen[v]++) return fail(ctx, HEXOPT_ERR_ARG, "mesh %d: vertex %d in two glue groups", m, v);
        gv.push_back((int32_t)(ctx->md[m].v_off + local_vid(ctx, m, v)));
      }
      gp.push_back((int64_t)gv.size());
    }
    po += n_groups[m];
    vo += n_groups[m] > 0 ? pm[n_groups[m]] - pm[0] : 0;
  }
  ctx->nG.assign(n_groups, n_groups + ctx->n_meshes);
  ctx->NGR = (int64_t)gp.size() - 1;
  ctx->has_glue = ctx->NGR > 0;
  CK(upload(ctx->g_ptr, gp.data(), gp.size(), ctx->st));
  if (gv.empty()) gv.push_back(0);
  CK(upload(ctx->g_vs, gv.data(), gv.size(), ctx->st));
  rc = pull_scalars(ctx);
  if (rc) return rc;
  for (int m = 0; m < ctx->n_meshes; m++) {
    ctx->sc[m].glue = n_groups[m] > 0 ? 1 : 0;
    if (lamda_glue) ctx->sc[m].lamda_G = lamda_glue[m];
  }
  rc = push_scalars(ctx);
  if (rc) return rc;
  ctx->precomputed = false;
  return rebuild_tables(ctx);
}

int hexopt_set_fixed(hexopt_ctx *ctx, const int64_t *nF, const int32_t *ids) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!nF) return fail(ctx, HEXOPT_ERR_ARG, "set_fixed: NULL counts");
  std::fill(ctx->fixed_h.begin(), ctx->fixed_h.end(), 0);
  int64_t tot = 0;
  for (int m = 0; m < ctx->n_meshes; m++) {
    if (nF[m] < 0) return fail(ctx, HEXOPT_ERR_ARG, "set_fixed: negative count");
    for (int64_t i = 0; i < nF[m]; i++) {
      const int32_t v = ids[tot + i];
      if (v < 0 || v >= ctx->md[m].nv) return fail(ctx, HEXOPT_ERR_ARG, "set_fixed: vertex id out of range");
      ctx->fixed_h[ctx->md[m].v_off + local_vid(ctx, m, v)] = 1;
    }
    tot += nF[m];
  }
  ctx->has_fixed = tot > 0;
  CK(upload(ctx->vfix, ctx->fixed_h.data(), ctx->fixed_h.size(), ctx->st));
  ctx->precomputed = false;
  ctx->tables_epoch++;
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

int hexopt_set_weights(hexopt_ctx *ctx, const double *lC, const double *lT, const double *lL) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  rc = pull_scalars(ctx);
  if (rc) return rc;
  for (int m = 0; m < ctx->n_meshes; m++) {
    if (lC) ctx->lamC[m] = ctx->sc[m].lamda_C = lC[m];
    if (lT) ctx->lamT[m] = ctx->sc[m].lamda_T = lT[m];
    if (lL) ctx->lamL[m] = ctx->sc[m].lamda_L = lL[m];
  }
  return push_scalars(ctx);
}

int hexopt_get_tangents(hexopt_ctx *ctx, double *normal, double *dis) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (ctx->NT) {
    if (normal) CK(cudaMemcpyAsync(normal, ctx->t_nrm.p, sizeof(double) * 3 * ctx->NT, cudaMemcpyDeviceToHost, ctx->st));
    if (dis) CK(cudaMemcpyAsync(dis, ctx->t_dis.p, sizeof(double) * ctx->NT, cudaMemcpyDeviceToHost, ctx->st));
  }
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

int hexopt_get_lines(hexopt_ctx *ctx, double *axis, double *origin) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (ctx->NL) {
    if (axis) CK(cudaMemcpyAsync(axis, ctx->l_axis.p, sizeof(double) * 3 * ctx->NL, cudaMemcpyDeviceToHost, ctx->st));
    if (origin) CK(cudaMemcpyAsync(origin, ctx->l_orig.p, sizeof(double) * 3 * ctx->NL, cudaMemcpyDeviceToHost, ctx->st));
  }
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

int hexopt_set_reference_hexes(hexopt_ctx *ctx, const double *P8) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (P8) {
    CK(upload(ctx->stage, P8, (size_t)ctx->NH * 24, ctx->st));
    CK(ctx->ref_p8.ensure(sizeof(double) * 24 * ctx->NH));
    launch_gather_rows(ctx->stage.as<double>(), hn2o(ctx), ctx->NH, 24, ctx->ref_p8.as<double>(), ctx->st);
    ctx->has_ref_p8 = true;
    ctx->has_ref_tets = false;
  } else {
    ctx->has_ref_p8 = false;
    ctx->has_ref_tets = false;
  }
  ctx->precomputed = false;
  ctx->tables_epoch++;
  return HEXOPT_OK;
}

int hexopt_set_reference_tets(hexopt_ctx *ctx, const double *RT) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!RT) return hexopt_set_reference_hexes(ctx, nullptr);
  CK(upload(ctx->stage, RT, (size_t)ctx->NH * 96, ctx->st));
  CK(ctx->ref_p8.ensure(sizeof(double) * 96 * ctx->NH));
  launch_gather_rows(ctx->stage.as<double>(), hn2o(ctx), ctx->NH, 96, ctx->ref_p8.as<double>(), ctx->st);
  ctx->has_ref_p8 = true;  // the shapes are fixed by the caller
  ctx->has_ref_tets = true;
  ctx->precomputed = false;
  ctx->tables_epoch++;
  CKL();
  return HEXOPT_OK;
}

int hexopt_slim_precompute(hexopt_ctx *ctx, const hexopt_slim_params *p) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!p) return fail(ctx, HEXOPT_ERR_ARG, "slim_precompute: NULL params");
  if (p->energy < 0 || p->energy > 5) return fail(ctx, HEXOPT_ERR_ARG, "unknown energy %d", p->energy);
  if (p->precision != HEXOPT_FP64 && p->precision != HEXOPT_MIXED) return fail(ctx, HEXOPT_ERR_ARG, "unknown precision");
  if (p->ls_candidates < 1 || p->ls_candidates > kMaxCand) return fail(ctx, HEXOPT_ERR_ARG, "ls_candidates must be 1..%d", kMaxCand);
  if (p->cg_max_iter < 0) return fail(ctx, HEXOPT_ERR_ARG, "cg_max_iter < 0");
  if (p->variant != 0 && p->variant != 1) return fail(ctx, HEXOPT_ERR_ARG, "unknown SLIM variant %d", p->variant);
  if (p->variant == 1 && (ctx->has_glue || ctx->NB > 0))
    return fail(ctx, HEXOPT_ERR_UNSUPPORTED,
                "the modified igl::slim's glue groups and b/bc terms (which no reference caller sets) are not built");
  if (p->precision == HEXOPT_MIXED && (ctx->has_glue || ctx->has_fixed))
    return fail(ctx, HEXOPT_ERR_UNSUPPORTED, "glue groups and held vertices run in HEXOPT_FP64 only");
  ctx->params = *p;
  ctx->mixed = p->precision == HEXOPT_MIXED;
  ctx->rest_fixed = !p->cube || ctx->has_ref_p8;
  rc = alloc_vectors(ctx);
  if (rc) return rc;
  if (ctx->rest_fixed) {
    rc = build_ref_shapes(ctx);
    if (rc) return rc;
  }
  rc = pull_scalars(ctx);
  if (rc) return rc;
  for (int m = 0; m < ctx->n_meshes; m++) {
    MeshScalars &S = ctx->sc[m];
    S.M = p->variant == 1 ? p->weight_opt / 2 : p->weight_opt;  // igl/slim.cpp:1243-1246 halves M
    S.prox = 0.00001 * p->weight_opt;  // slim_m.cpp:1118, igl/slim.cpp:1240
    S.exp_f = p->exp_factor;
    S.status = 0;
    S.frozen = 0;
  }
  rc = push_scalars(ctx);
  if (rc) return rc;
  // slim_precompute: data.a_L.setZero() (slim_m.cpp:1115)
  if (ctx->NL) CK(cudaMemsetAsync(ctx->aL.p, 0, sizeof(double) * ctx->NL, ctx->st));
  rc = dispatch_precompute(ctx);
  if (rc) return rc;
  ctx->precomputed = true;
  return HEXOPT_OK;
}

int hexopt_slim_iterate(hexopt_ctx *ctx, int iters, hexopt_slim_report *rep) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!ctx->precomputed) return fail(ctx, HEXOPT_ERR_STATE, "slim_iterate before slim_precompute");
  for (int i = 0; i < iters; i++) {
    rc = dispatch_iteration(ctx);
    if (rc) return rc;
  }
  if (rep) {
    rc = pull_scalars(ctx);
    if (rc) return rc;
    for (int m = 0; m < ctx->n_meshes; m++) fill_report(ctx->sc[m], ctx->md[m].nh, rep[m]);
  }
  return HEXOPT_OK;
}

int hexopt_slim_m_opt(hexopt_ctx *ctx, const hexopt_slim_params *p, int iters, hexopt_slim_report *rep) {
  int rc = hexopt_slim_precompute(ctx, p);
  if (rc) return rc;
  return hexopt_slim_iterate(ctx, iters, rep);
}

int hexopt_smoothing(hexopt_ctx *ctx, const hexopt_slim_params *params, int outer, int inner,
                     hexopt_slim_report *rep) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!params || outer < 0 || inner < 0) return fail(ctx, HEXOPT_ERR_ARG, "smoothing: bad arguments");
  hexopt_slim_params p = *params;
  p.variant = 1;
  p.cube = 1;
  for (int o = 0; o < outer; o++) {
    rc = hexopt_slim_precompute(ctx, &p);  // compute_referenceMesh(ts.V, ..., true) + slim_precompute
    if (rc) return rc;
    rc = hexopt_slim_iterate(ctx, inner, rep);
    if (rc) return rc;
  }
  return HEXOPT_OK;
}

int hexopt_get_curve_params(hexopt_ctx *ctx, double *a_L) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (ctx->NL && a_L) CK(cudaMemcpyAsync(a_L, ctx->aL.p, sizeof(double) * ctx->NL, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

// ---------------------------------------------------------------- targets / projection
int hexopt_set_target(hexopt_ctx *ctx, int mesh, int64_t nv, const double *TV, int64_t nf, const int32_t *TF) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (mesh < 0 || mesh >= ctx->n_meshes) return fail(ctx, HEXOPT_ERR_ARG, "set_target: bad mesh");
  if (nv <= 0 || nf <= 0 || !TV || !TF) return fail(ctx, HEXOPT_ERR_ARG, "set_target: empty target");
  for (int64_t i = 0; i < 3 * nf; i++)
    if (TF[i] < 0 || TF[i] >= nv) return fail(ctx, HEXOPT_ERR_ARG, "set_target: face id out of range");
  TargetHost &t = ctx->tgt[mesh];
  t.nv = nv;
  t.nf = nf;
  t.TV.assign(TV, TV + 3 * nv);
  // triangle soup and the normals of build_aabb_tree (per_face_normals, per_vertex_normals with
  // angle weights, per_edge_normals uniform -- left unnormalised as the reference leaves them).
  std::vector<double> tri(9 * nf), FN(3 * nf, 0.0), VN(3 * nv, 0.0), VNc(9 * nf), ENc(9 * nf);
  for (int64_t f = 0; f < nf; f++) {
    for (int c = 0; c < 3; c++)
      for (int d = 0; d < 3; d++) tri[9 * f + 3 * c + d] = TV[3 * (int64_t)TF[3 * f + c] + d];
    const double *p0 = &tri[9 * f], *p1 = &tri[9 * f + 3], *p2 = &tri[9 * f + 6];
    const double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]}, e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double r = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (r != 0)
      for (int d = 0; d < 3; d++) FN[3 * f + d] = n[d] / r;
  }
  for (int64_t f = 0; f < nf; f++) {
    double L[3];
    for (int c = 0; c < 3; c++) {
      const double *a = &tri[9 * f + 3 * ((c + 1) % 3)], *b = &tri[9 * f + 3 * ((c + 2) % 3)];
      L[c] = (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]);
    }
    for (int d = 0; d < 3; d++) {
      const double s1 = L[d], s2 = L[(d + 1) % 3], s3 = L[(d + 2) % 3];
      const double ang = std::acos((s3 + s2 - s1) / (2. * std::sqrt(s3 * s2)));
      for (int k = 0; k < 3; k++) VN[3 * (int64_t)TF[3 * f + d] + k] += ang * FN[3 * f + k];
    }
  }
  for (int64_t v = 0; v < nv; v++) {
    const double r = std::sqrt(VN[3 * v] * VN[3 * v] + VN[3 * v + 1] * VN[3 * v + 1] + VN[3 * v + 2] * VN[3 * v + 2]);
    if (r > 0)
      for (int d = 0; d < 3; d++) VN[3 * v + d] /= r;
  }
  // undirected edges: sort (min, max, face*3+corner)
  std::vector<std::pair<uint64_t, int64_t>> E(3 * nf);
  for (int64_t f = 0; f < nf; f++)
    for (int c = 0; c < 3; c++) {
      uint64_t a = (uint64_t)TF[3 * f + (c + 1) % 3], b = (uint64_t)TF[3 * f + (c + 2) % 3];
      if (a > b) std::swap(a, b);
      E[3 * f + c] = {a * (uint64_t)(nv + 1) + b, 3 * f + c};
    }
  std::sort(E.begin(), E.end());
  for (size_t i = 0; i < E.size();) {
    size_t j = i;
    double s[3] = {0, 0, 0};
    while (j < E.size() && E[j].first == E[i].first) {
      const int64_t f = E[j].second / 3;
      for (int d = 0; d < 3; d++) s[d] += FN[3 * f + d];
      j++;
    }
    for (size_t k = i; k < j; k++)
      for (int d = 0; d < 3; d++) ENc[9 * (E[k].second / 3) + 3 * (E[k].second % 3) + d] = s[d];
    i = j;
  }
  for (int64_t f = 0; f < nf; f++)
    for (int c = 0; c < 3; c++)
      for (int d = 0; d < 3; d++) VNc[9 * f + 3 * c + d] = VN[3 * (int64_t)TF[3 * f + c] + d];
  for (int d = 0; d < 3; d++) { t.lo[d] = INFINITY; t.hi[d] = -INFINITY; }
  std::vector<uint8_t> used(nv, 0);
  for (int64_t i = 0; i < 3 * nf; i++) used[TF[i]] = 1;
  for (int64_t v = 0; v < nv; v++)
    for (int d = 0; d < 3; d++) {
      t.lo[d] = std::min(t.lo[d], TV[3 * v + d]);
      t.hi[d] = std::max(t.hi[d], TV[3 * v + d]);
    }
  CK(upload(t.TVd, TV, (size_t)3 * nv, ctx->st));
  CK(upload(t.FN, FN.data(), FN.size(), ctx->st));
  CK(upload(t.VNc, VNc.data(), VNc.size(), ctx->st));
  CK(upload(t.ENc, ENc.data(), ENc.size(), ctx->st));
  rc = build_static_bvh(ctx, t.bvh, tri, nf, true);
  if (rc) return rc;
  CK(t.EP.ensure(sizeof(double) * 16 * nf));
  launch_ep_faces(t.bvh.tri.as<double>(), nf, t.EP.as<double>(), ctx->st);
  ctx->launches++;
  CKL();
  t.set = true;
  // referenced target vertices for the Hausdorff side 0 list
  t.ref_vs.clear();
  for (int64_t v = 0; v < nv; v++)
    if (used[v]) t.ref_vs.push_back(v);
  std::vector<int64_t> all;
  for (int m = 0; m < ctx->n_meshes; m++) {
    ctx->tgt_vs_cnt[m] = ctx->tgt[m].set ? (int64_t)ctx->tgt[m].ref_vs.size() : 0;
    if (ctx->tgt[m].set) all.insert(all.end(), ctx->tgt[m].ref_vs.begin(), ctx->tgt[m].ref_vs.end());
  }
  CK(upload(ctx->tgt_vs_d, all.data(), all.size(), ctx->st));
  rc = rebuild_tables(ctx);
  if (rc) return rc;
  return upload_targets_table(ctx);
}

int hexopt_signed_distance(hexopt_ctx *ctx, int mesh, int64_t np, const double *P, double *S, int32_t *I, double *C,
                           double *N) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (mesh < 0 || mesh >= ctx->n_meshes || !ctx->tgt[mesh].set) return fail(ctx, HEXOPT_ERR_STATE, "signed_distance: no target");
  if (np < 0 || (np > 0 && (!P || !S || !I || !C || !N))) return fail(ctx, HEXOPT_ERR_ARG, "signed_distance: bad arguments");
  if (np == 0) return HEXOPT_OK;
  DBuf Pd, Sd, Id, Cd, Nd, stat;
  CK(upload(Pd, P, (size_t)3 * np, ctx->st));
  CK(Sd.ensure(sizeof(double) * np)); CK(Id.ensure(sizeof(int32_t) * np));
  CK(Cd.ensure(sizeof(double) * 3 * np)); CK(Nd.ensure(sizeof(double) * 3 * np));
  CK(stat.ensure(sizeof(int)));
  CK(cudaMemsetAsync(stat.p, 0, sizeof(int), ctx->st));
  std::vector<TargetDev> td(ctx->n_meshes);
  CK(cudaMemcpyAsync(td.data(), ctx->tgt_d.p, sizeof(TargetDev) * ctx->n_meshes, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  launch_signed_distance(td[mesh], np, Pd.as<double>(), Sd.as<double>(), Id.as<int32_t>(), Cd.as<double>(), Nd.as<double>(),
                         stat.as<int>(), ctx->st);
  ctx->launches++;
  CKL();
  CK(cudaMemcpyAsync(S, Sd.p, sizeof(double) * np, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(I, Id.p, sizeof(int32_t) * np, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(C, Cd.p, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(N, Nd.p, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, ctx->st));
  int st = 0;
  CK(cudaMemcpyAsync(&st, stat.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (st) return fail(ctx, HEXOPT_ERR_NUMERIC, "signed_distance: BVH traversal stack overflow");
  return HEXOPT_OK;
}

int hexopt_set_feature_sets(hexopt_ctx *ctx, const int64_t *n_regular, const int32_t *regular_ids,
                            const int64_t *n_line, const int32_t *line_ids, const int32_t *line_curve,
                            const int64_t *n_curves, const int64_t *curve_ptr, const int32_t *curve_vs,
                            const uint8_t *curve_closed) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  int64_t nr = 0, nl = 0;
  for (int m = 0; m < ctx->n_meshes; m++) { nr += n_regular[m]; nl += n_line[m]; }
  std::vector<double> zn(3 * std::max<int64_t>(nr, 1), 0.0), zd(std::max<int64_t>(nr, 1), 0.0);
  rc = hexopt_set_tangents(ctx, n_regular, regular_ids, zn.data(), zd.data());
  if (rc) return rc;
  std::vector<double> zl(3 * std::max<int64_t>(nl, 1), 0.0);
  rc = hexopt_set_lines(ctx, n_line, line_ids, zl.data(), zl.data());
  if (rc) return rc;
  // per-mesh curves (concatenated per mesh; curve ids in line_curve are mesh-local)
  int64_t co = 0, vo = 0, lo = 0;
  std::vector<int32_t> lc(std::max<int64_t>(nl, 1));
  for (int m = 0; m < ctx->n_meshes; m++) {
    const int64_t ncv = n_curves ? n_curves[m] : 0;
    TargetHost &t = ctx->tgt[m];
    if (n_line[m] > 0 && !t.set) return fail(ctx, HEXOPT_ERR_STATE, "mesh %d: feature lines need a target", m);
    const int64_t *cp = curve_ptr + co + m;  // ncv + 1 entries per mesh
    std::vector<int64_t> ptr(ncv + 1);
    for (int64_t i = 0; i <= ncv; i++) ptr[i] = cp[i] - cp[0];
    const int64_t nvs = ptr[ncv];
    for (int64_t i = 0; i < nvs; i++)
      if (curve_vs[vo + i] < 0 || curve_vs[vo + i] >= t.nv) return fail(ctx, HEXOPT_ERR_ARG, "mesh %d: curve vertex out of range", m);
    for (int64_t i = 0; i < n_line[m]; i++) {
      if (line_curve[lo + i] < 0 || line_curve[lo + i] >= ncv) return fail(ctx, HEXOPT_ERR_ARG, "mesh %d: line curve id out of range", m);
      lc[lo + i] = line_curve[lo + i];
    }
    if (t.set) {
      CK(upload(t.curve_ptr, ptr.data(), ptr.size(), ctx->st));
      CK(upload(t.curve_vs, curve_vs + vo, (size_t)nvs, ctx->st));
      std::vector<uint8_t> cl(std::max<int64_t>(ncv, 1), 0);
      for (int64_t i = 0; i < ncv; i++) cl[i] = curve_closed[co + i];
      CK(upload(t.curve_closed, cl.data(), cl.size(), ctx->st));
      t.n_curves = ncv;
    }
    co += ncv;
    vo += nvs;
    lo += n_line[m];
  }
  CK(upload(ctx->l_curve, lc.data(), lc.size(), ctx->st));
  return upload_targets_table(ctx);
}

int hexopt_project_features(hexopt_ctx *ctx) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  return run_projection(ctx);
}

int hexopt_set_query_budget(hexopt_ctx *ctx, int pops) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (pops < 0 || pops > (1 << 20)) return fail(ctx, HEXOPT_ERR_ARG, "set_query_budget: pops must be 0..2^20");
  ctx->query_budget = pops;
  ctx->tables_epoch++;  // a captured step bakes the budget in
  return HEXOPT_OK;
}

int hexopt_query_stats(hexopt_ctx *ctx, int64_t *warp_queries, int64_t *candidates, int64_t *fallbacks) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  unsigned w = 0, c = 0, f = 0;
  const QueryBufs &q = ctx->qb[0];  // the projection, or Hausdorff side 1
  if (q.ovf_count.p) CK(cudaMemcpyAsync(&w, q.ovf_count.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
  if (q.cand_count.p) CK(cudaMemcpyAsync(&c, q.cand_count.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
  if (q.fb_count.p) CK(cudaMemcpyAsync(&f, q.fb_count.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (warp_queries) *warp_queries = w;
  if (candidates) *candidates = c;
  if (fallbacks) *fallbacks = f;
  return HEXOPT_OK;
}

// ---------------------------------------------------------------- Hausdorff
int hexopt_set_surface(hexopt_ctx *ctx, int mesh, int64_t nf, const int32_t *F) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (mesh < 0 || mesh >= ctx->n_meshes || nf <= 0 || !F) return fail(ctx, HEXOPT_ERR_ARG, "set_surface: bad arguments");
  const int64_t nv = ctx->md[mesh].nv, vo = ctx->md[mesh].v_off;
  std::vector<int32_t> G(3 * nf);
  std::vector<uint8_t> used(nv, 0);
  for (int64_t i = 0; i < 3 * nf; i++) {
    if (F[i] < 0 || F[i] >= nv) return fail(ctx, HEXOPT_ERR_ARG, "set_surface: vertex id out of range");
    const int32_t lv = local_vid(ctx, mesh, F[i]);
    G[i] = (int32_t)(lv + vo);
    used[lv] = 1;
  }
  SurfaceHost &s = ctx->surf[mesh];
  s.nf = nf;
  s.ref_vs.clear();
  for (int64_t v = 0; v < nv; v++)
    if (used[v]) s.ref_vs.push_back(vo + v);
  CK(upload(s.F, G.data(), G.size(), ctx->st));
  // topology from the current positions' centroids
  std::vector<double> tri(9 * nf);
  std::vector<double> Xh(3 * nv);
  CK(ctx->stage.ensure(sizeof(double) * 3 * ctx->NV));
  launch_aos4_to_rows(ctx->X.as<double>(), ctx->stage.as<double>(), ctx->NV, ctx->st);
  ctx->launches++;
  CK(cudaMemcpyAsync(Xh.data(), ctx->stage.as<double>() + 3 * vo, sizeof(double) * 3 * nv, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  for (int64_t f = 0; f < nf; f++)
    for (int c = 0; c < 3; c++)
      for (int d = 0; d < 3; d++) tri[9 * f + 3 * c + d] = Xh[3 * (int64_t)(G[3 * f + c] - vo) + d];
  StaticBvh tmp;
  rc = build_static_bvh(ctx, tmp, tri, nf, false);
  if (rc) return rc;
  // adopt the topology (child / parent / leaf order); boxes are refitted from X on use
  std::swap(s.child.p, tmp.child.p); std::swap(s.child.bytes, tmp.child.bytes);
  std::swap(s.parent.p, tmp.parent.p); std::swap(s.parent.bytes, tmp.parent.bytes);
  std::swap(s.box.p, tmp.box.p); std::swap(s.box.bytes, tmp.box.bytes);
  std::swap(s.leaf_face.p, tmp.leaf_face.p); std::swap(s.leaf_face.bytes, tmp.leaf_face.bytes);
  std::swap(s.counters.p, tmp.counters.p); std::swap(s.counters.bytes, tmp.counters.bytes);
  std::swap(s.node.p, tmp.node.p); std::swap(s.node.bytes, tmp.node.bytes);
  std::swap(s.leafd.p, tmp.leafd.p); std::swap(s.leafd.bytes, tmp.leafd.bytes);
  s.set = true;
  std::vector<int64_t> all;
  for (int m = 0; m < ctx->n_meshes; m++) {
    ctx->surf_vs_cnt[m] = ctx->surf[m].set ? (int64_t)ctx->surf[m].ref_vs.size() : 0;
    if (ctx->surf[m].set) all.insert(all.end(), ctx->surf[m].ref_vs.begin(), ctx->surf[m].ref_vs.end());
  }
  CK(upload(ctx->surf_vs_d, all.data(), all.size(), ctx->st));
  rc = rebuild_tables(ctx);
  if (rc) return rc;
  return upload_targets_table(ctx);
}

static int prepare_haus(hexopt_ctx *ctx) {
  for (int m = 0; m < ctx->n_meshes; m++)
    if (!ctx->tgt[m].set || !ctx->surf[m].set) return fail(ctx, HEXOPT_ERR_STATE, "mesh %d: Hausdorff needs set_target and set_surface", m);
  std::vector<HausMesh> hm(ctx->n_meshes);
  for (int m = 0; m < ctx->n_meshes; m++) {
    HausMesh h{};
    for (int d = 0; d < 3; d++) { h.tgt_lo[d] = ctx->tgt[m].lo[d]; h.tgt_hi[d] = ctx->tgt[m].hi[d]; }
    hm[m] = h;
  }
  CK(upload(ctx->hm_d, hm.data(), hm.size(), ctx->st));
  ctx->haus_ready = true;
  return HEXOPT_OK;
}

int hexopt_hausdorff_meshes(hexopt_ctx *ctx, double *diag, double *max_dist, double *ave_dist) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!ctx->haus_ready) {
    rc = prepare_haus(ctx);
    if (rc) return rc;
  }
  rc = run_hausdorff(ctx, false);
  if (rc) return rc;
  std::vector<HausMesh> hm(ctx->n_meshes);
  CK(cudaMemcpyAsync(hm.data(), ctx->hm_d.p, sizeof(HausMesh) * ctx->n_meshes, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  for (int m = 0; m < ctx->n_meshes; m++) {
    if (diag) diag[m] = hm[m].diag;
    if (max_dist) max_dist[m] = hm[m].max_dist;
    if (ave_dist) ave_dist[m] = hm[m].ave_dist;
  }
  return HEXOPT_OK;
}


// ---------------------------------------------------------------- standalone distances
static int ep_side(hexopt_ctx *ctx, const BvhDev &b, const double *P, const int64_t *ids, int64_t n, double upper,
                   double *out3, DBuf &dist, DBuf &stat) {
  CK(dist.ensure(sizeof(double) * std::max<int64_t>(n, 1)));
  launch_ep_points(b, P, ids, n, upper, dist.as<double>(), stat.as<int>(), ctx->st);
  launch_maxmean(dist.as<double>(), n, upper, out3, ctx->st);
  ctx->launches += 2;
  CKL();
  return HEXOPT_OK;
}

int hexopt_hausdorff(hexopt_ctx *ctx, int64_t nv0, const double *V0, int64_t nf0, const int32_t *F0, int64_t nv1,
                     const double *V1, int64_t nf1, const int32_t *F1, double *diag, double *max_dist,
                     double *ave_dist) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (nv0 <= 0 || nv1 <= 0 || nf0 <= 0 || nf1 <= 0 || !V0 || !V1 || !F0 || !F1)
    return fail(ctx, HEXOPT_ERR_ARG, "hausdorff: empty mesh");
  for (int64_t i = 0; i < 3 * nf0; i++) if (F0[i] < 0 || F0[i] >= nv0) return fail(ctx, HEXOPT_ERR_ARG, "hausdorff: F0 id out of range");
  for (int64_t i = 0; i < 3 * nf1; i++) if (F1[i] < 0 || F1[i] >= nv1) return fail(ctx, HEXOPT_ERR_ARG, "hausdorff: F1 id out of range");
  CK(cudaSetDevice(ctx->device));
  // union bbox of both vertex sets, inflated by 2% of its diagonal (metro_hausdorff.cpp:455-462)
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t v = 0; v < nv0; v++) for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], V0[3 * v + d]); hi[d] = std::max(hi[d], V0[3 * v + d]); }
  for (int64_t v = 0; v < nv1; v++) for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], V1[3 * v + d]); hi[d] = std::max(hi[d], V1[3 * v + d]); }
  const double e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
  const double off = std::sqrt(e0 * e0 + e1 * e1 + e2 * e2) * 0.02;
  const double f0 = e0 + 2 * off, f1 = e1 + 2 * off, f2 = e2 + 2 * off;
  const double D = std::sqrt(f0 * f0 + f1 * f1 + f2 * f2);
  std::vector<double> tri0(9 * nf0), tri1(9 * nf1);
  std::vector<uint8_t> u0(nv0, 0), u1(nv1, 0);
  for (int64_t f = 0; f < nf0; f++) for (int c = 0; c < 3; c++) { u0[F0[3 * f + c]] = 1; for (int d = 0; d < 3; d++) tri0[9 * f + 3 * c + d] = V0[3 * (int64_t)F0[3 * f + c] + d]; }
  for (int64_t f = 0; f < nf1; f++) for (int c = 0; c < 3; c++) { u1[F1[3 * f + c]] = 1; for (int d = 0; d < 3; d++) tri1[9 * f + 3 * c + d] = V1[3 * (int64_t)F1[3 * f + c] + d]; }
  std::vector<int64_t> r0, r1;
  for (int64_t v = 0; v < nv0; v++) if (u0[v]) r0.push_back(v);
  for (int64_t v = 0; v < nv1; v++) if (u1[v]) r1.push_back(v);
  StaticBvh B0, B1;
  int rc = build_static_bvh(ctx, B0, tri0, nf0, false);
  if (rc) return rc;
  rc = build_static_bvh(ctx, B1, tri1, nf1, false);
  if (rc) return rc;
  DBuf P0, P1, I0, I1, dist, stat, out;
  CK(upload(P0, V0, (size_t)3 * nv0, ctx->st));
  CK(upload(P1, V1, (size_t)3 * nv1, ctx->st));
  CK(upload(I0, r0.data(), r0.size(), ctx->st));
  CK(upload(I1, r1.data(), r1.size(), ctx->st));
  CK(stat.ensure(sizeof(int)));
  CK(cudaMemsetAsync(stat.p, 0, sizeof(int), ctx->st));
  CK(out.ensure(sizeof(double) * 6));
  rc = ep_side(ctx, B1.dev(), P0.as<double>(), I0.as<int64_t>(), (int64_t)r0.size(), D, out.as<double>(), dist, stat);
  if (rc) return rc;
  DBuf dist2;
  rc = ep_side(ctx, B0.dev(), P1.as<double>(), I1.as<int64_t>(), (int64_t)r1.size(), D, out.as<double>() + 3, dist2, stat);
  if (rc) return rc;
  double h[6];
  int st = 0;
  CK(cudaMemcpyAsync(h, out.p, sizeof h, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(&st, stat.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (st) return fail(ctx, HEXOPT_ERR_NUMERIC, "hausdorff: BVH traversal stack overflow");
  if (diag) *diag = D;
  if (max_dist) *max_dist = std::max(h[0], h[3]);
  if (ave_dist) *ave_dist = std::max(h[4] / h[5], h[1] / h[2]);
  return HEXOPT_OK;
}

// Both sides of the uniform-sample check: n samples of each surface against the other's BVH, max
// and sum / count of the distances below the upper bound D.
int hexopt_hausdorff_uniform(hexopt_ctx *ctx, int64_t nv0, const double *V0, int64_t nf0, const int32_t *F0, int64_t nv1,
                             const double *V1, int64_t nf1, const int32_t *F1, int64_t n_samples, uint64_t seed,
                             double *diag, double *max_dist, double *ave_dist, double *samples0, double *samples1) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (nv0 <= 0 || nv1 <= 0 || nf0 <= 0 || nf1 <= 0 || !V0 || !V1 || !F0 || !F1 || n_samples <= 0)
    return fail(ctx, HEXOPT_ERR_ARG, "hausdorff_uniform: empty mesh or no samples");
  for (int64_t i = 0; i < 3 * nf0; i++) if (F0[i] < 0 || F0[i] >= nv0) return fail(ctx, HEXOPT_ERR_ARG, "hausdorff_uniform: F0 id out of range");
  for (int64_t i = 0; i < 3 * nf1; i++) if (F1[i] < 0 || F1[i] >= nv1) return fail(ctx, HEXOPT_ERR_ARG, "hausdorff_uniform: F1 id out of range");
  CK(cudaSetDevice(ctx->device));
  // the upper bound: both vertex sets' bbox inflated by 2% of its diagonal (metro_hausdorff.cpp:455-462)
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t v = 0; v < nv0; v++) for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], V0[3 * v + d]); hi[d] = std::max(hi[d], V0[3 * v + d]); }
  for (int64_t v = 0; v < nv1; v++) for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], V1[3 * v + d]); hi[d] = std::max(hi[d], V1[3 * v + d]); }
  const double e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
  const double off = std::sqrt(e0 * e0 + e1 * e1 + e2 * e2) * 0.02;
  const double f0 = e0 + 2 * off, f1 = e1 + 2 * off, f2 = e2 + 2 * off;
  const double D = std::sqrt(f0 * f0 + f1 * f1 + f2 * f2);
  std::vector<double> tri0(9 * nf0), tri1(9 * nf1);
  for (int64_t f = 0; f < nf0; f++) for (int c = 0; c < 3; c++) for (int d = 0; d < 3; d++) tri0[9 * f + 3 * c + d] = V0[3 * (int64_t)F0[3 * f + c] + d];
  for (int64_t f = 0; f < nf1; f++) for (int c = 0; c < 3; c++) for (int d = 0; d < 3; d++) tri1[9 * f + 3 * c + d] = V1[3 * (int64_t)F1[3 * f + c] + d];
  StaticBvh B0, B1;
  int rc = build_static_bvh(ctx, B0, tri0, nf0, false);
  if (rc) return rc;
  rc = build_static_bvh(ctx, B1, tri1, nf1, false);
  if (rc) return rc;
  DBuf Vd0, Vd1, Fd0, Fd1, S0, S1, scratch, dist, stat, out;
  CK(upload(Vd0, V0, (size_t)3 * nv0, ctx->st));
  CK(upload(Vd1, V1, (size_t)3 * nv1, ctx->st));
  CK(upload(Fd0, F0, (size_t)3 * nf0, ctx->st));
  CK(upload(Fd1, F1, (size_t)3 * nf1, ctx->st));
  CK(S0.ensure(sizeof(double) * 3 * n_samples));
  CK(S1.ensure(sizeof(double) * 3 * n_samples));
  const size_t sb = std::max(sample_scratch_bytes(nf0), sample_scratch_bytes(nf1));
  CK(scratch.ensure(sb));
  // the two surfaces draw from disjoint counter ranges: surface 1 starts 3 n_samples after surface 0
  CK(sample_surface(Vd0.as<double>(), Fd0.as<int32_t>(), nf0, n_samples, seed, S0.as<double>(), scratch.p, sb, ctx->st));
  CK(sample_surface(Vd1.as<double>(), Fd1.as<int32_t>(), nf1, n_samples, seed + 3ull * (uint64_t)n_samples,
                    S1.as<double>(), scratch.p, sb, ctx->st));
  CK(stat.ensure(sizeof(int)));
  CK(cudaMemsetAsync(stat.p, 0, sizeof(int), ctx->st));
  CK(out.ensure(sizeof(double) * 6));
  rc = ep_side(ctx, B1.dev(), S0.as<double>(), nullptr, n_samples, D, out.as<double>(), dist, stat);
  if (rc) return rc;
  DBuf dist2;
  rc = ep_side(ctx, B0.dev(), S1.as<double>(), nullptr, n_samples, D, out.as<double>() + 3, dist2, stat);
  if (rc) return rc;
  ctx->launches += 6;
  double h[6];
  int st = 0;
  CK(cudaMemcpyAsync(h, out.p, sizeof h, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(&st, stat.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  if (samples0) CK(cudaMemcpyAsync(samples0, S0.p, sizeof(double) * 3 * n_samples, cudaMemcpyDeviceToHost, ctx->st));
  if (samples1) CK(cudaMemcpyAsync(samples1, S1.p, sizeof(double) * 3 * n_samples, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (st) return fail(ctx, HEXOPT_ERR_NUMERIC, "hausdorff_uniform: BVH traversal stack overflow");
  const double mx0 = h[2] > 0 ? h[0] : 0.0, mx1 = h[5] > 0 ? h[3] : 0.0;
  const double av0 = h[2] > 0 ? h[1] / h[2] : 0.0, av1 = h[5] > 0 ? h[4] / h[5] : 0.0;
  if (diag) *diag = D;
  if (max_dist) *max_dist = std::max(mx0, mx1);
  if (ave_dist) *ave_dist = std::max(av0, av1);
  return HEXOPT_OK;
}

int hexopt_point_face_distance(hexopt_ctx *ctx, int64_t np, const double *P, int64_t nv, const double *V, int64_t nf,
                               const int32_t *F, double *dist) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (np < 0 || nv <= 0 || nf <= 0 || !V || !F || (np > 0 && (!P || !dist))) return fail(ctx, HEXOPT_ERR_ARG, "point_face_distance: bad arguments");
  for (int64_t i = 0; i < 3 * nf; i++) if (F[i] < 0 || F[i] >= nv) return fail(ctx, HEXOPT_ERR_ARG, "point_face_distance: id out of range");
  if (np == 0) return HEXOPT_OK;
  CK(cudaSetDevice(ctx->device));
  std::vector<double> tri(9 * nf);
  for (int64_t f = 0; f < nf; f++) for (int c = 0; c < 3; c++) for (int d = 0; d < 3; d++) tri[9 * f + 3 * c + d] = V[3 * (int64_t)F[3 * f + c] + d];
  StaticBvh B;
  int rc = build_static_bvh(ctx, B, tri, nf, false);
  if (rc) return rc;
  DBuf Pd, Dd, stat;
  CK(upload(Pd, P, (size_t)3 * np, ctx->st));
  CK(Dd.ensure(sizeof(double) * np));
  CK(stat.ensure(sizeof(int)));
  CK(cudaMemsetAsync(stat.p, 0, sizeof(int), ctx->st));
  launch_ep_points(B.dev(), Pd.as<double>(), nullptr, np, INFINITY, Dd.as<double>(), stat.as<int>(), ctx->st);
  ctx->launches++;
  CKL();
  int st = 0;
  CK(cudaMemcpyAsync(dist, Dd.p, sizeof(double) * np, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaMemcpyAsync(&st, stat.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (st) return fail(ctx, HEXOPT_ERR_NUMERIC, "point_face_distance: BVH traversal stack overflow");
  return HEXOPT_OK;
}

// ---------------------------------------------------------------- feature alignment
int hexopt_fa_begin(hexopt_ctx *ctx, const hexopt_slim_params *p, double lamda0, double hausdorff_ratio_t) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!p) return fail(ctx, HEXOPT_ERR_ARG, "fa_begin: NULL params");
  ctx->lamda0 = lamda0;
  ctx->HR = hausdorff_ratio_t;
  // validate and allocate with a precompute at the current positions
  rc = hexopt_slim_precompute(ctx, p);
  if (rc) return rc;
  rc = pull_scalars(ctx);
  if (rc) return rc;
  for (int m = 0; m < ctx->n_meshes; m++) {
    MeshScalars &S = ctx->sc[m];
    S.lamda_C = S.lamda_T = S.lamda_L = lamda0;  // fc.lamda_C = fc.lamda_L = fc.lamda_T = LAMDA (:3811)
    S.lamda0 = lamda0;
    S.fa_iter = 0;
    S.max_sat = 0;
    S.HR = hausdorff_ratio_t;
  }
  rc = push_scalars(ctx);
  if (rc) return rc;
  ctx->fa_ready = true;  // a captured step stays valid while nothing it baked in has changed
  return HEXOPT_OK;
}

static bool same_params(const hexopt_slim_params &a, const hexopt_slim_params &b) {
  return a.energy == b.energy && a.precision == b.precision && a.weight_opt == b.weight_opt &&
         a.exp_factor == b.exp_factor && a.cg_max_iter == b.cg_max_iter && a.cg_tol == b.cg_tol &&
         a.ls_candidates == b.ls_candidates && a.cube == b.cube;
}

static int fa_enqueue(hexopt_ctx *ctx, int do_hausdorff) {
  int rc = 0;
  if (ctx->rest_fixed && !ctx->has_ref_p8) {  // compute_referenceMesh(ts.UV, ...) of this step
    rc = build_ref_shapes(ctx);
    if (rc) return rc;
  }
  // the projection runs beside the local step (slim_precompute fused into it)
  rc = dispatch_iteration(ctx, true, true);
  if (rc) return rc;
  if (!ctx->ev_xfinal) CK(cudaEventCreateWithFlags(&ctx->ev_xfinal, cudaEventDisableTiming));
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(ctx->st, &cs));
  if (cs == cudaStreamCaptureStatusActive) CK(cudaEventRecordWithFlags(ctx->ev_xfinal, ctx->st, cudaEventRecordExternal));
  else CK(cudaEventRecord(ctx->ev_xfinal, ctx->st));
  launch_fa_schedule(ctx->sc_d.as<MeshScalars>(), ctx->n_meshes, ctx->lamda0, 1e16, ctx->st);
  if (!do_hausdorff) launch_step_sj(ctx, ctx->st);
  if (do_hausdorff) {
    rc = run_hausdorff(ctx, true);  // the SJ check runs beside the two sides
    if (rc) return rc;
    launch_fa_haus_flag(ctx->sc_d.as<MeshScalars>(), ctx->hm_d.as<HausMesh>(), ctx->n_meshes, ctx->st);
    ctx->launches++;
  }
  CKL();
  return HEXOPT_OK;
}

static int fa_step(hexopt_ctx *ctx, int do_hausdorff, hexopt_fa_report *rep, double *V);

int hexopt_feature_alignment_step(hexopt_ctx *ctx, int do_hausdorff, hexopt_fa_report *rep) {
  return fa_step(ctx, do_hausdorff, rep, nullptr);
}

int hexopt_feature_alignment_step_get(hexopt_ctx *ctx, int do_hausdorff, hexopt_fa_report *rep, double *V) {
  if (ctx && !V) return fail(ctx, HEXOPT_ERR_ARG, "feature_alignment_step_get: NULL");
  return fa_step(ctx, do_hausdorff, rep, V);
}

// The step's download, queued right after the step: staged and copied on the download stream
// once the step's positions are final (ev_xfinal), beside the step's SJ check and Hausdorff
// passes; later work on the compute stream waits until the staging kernel has read X.
static int fa_queue_download(hexopt_ctx *ctx, double *V) {
  CK(ensure_copy_streams(ctx));
  CK(ctx->out_stage.ensure(sizeof(double) * 3 * ctx->NV));
  CK(cudaStreamWaitEvent(ctx->dst, ctx->ev_xfinal, 0));
  launch_aos4_to_rows_perm(ctx->X.as<double>(), vo2n(ctx), ctx->NV, ctx->out_stage.as<double>(), ctx->dst);
  ctx->launches++;
  CKL();
  CK(cudaEventRecord(ctx->out_ready, ctx->dst));
  CK(cudaStreamWaitEvent(ctx->st, ctx->out_ready, 0));
  CK(cudaMemcpyAsync(V, ctx->out_stage.p, sizeof(double) * 3 * ctx->NV, cudaMemcpyDeviceToHost, ctx->dst));
  CK(cudaEventRecord(ctx->out_done, ctx->dst));
  return HEXOPT_OK;
}

static int fa_step(hexopt_ctx *ctx, int do_hausdorff, hexopt_fa_report *rep, double *V) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!ctx->fa_ready) return fail(ctx, HEXOPT_ERR_STATE, "feature_alignment_step before fa_begin");
  if (do_hausdorff && !ctx->haus_ready) {
    rc = prepare_haus(ctx);
    if (rc) return rc;
  }
  if (ctx->use_graph) {
    if (ctx->graph_exec &&
        (ctx->graph_hausdorff != (do_hausdorff != 0) || ctx->graph_tables != ctx->tables_epoch ||
         ctx->graph_allocs != g_device_allocs.load(std::memory_order_relaxed) || ctx->graph_lamda0 != ctx->lamda0 ||
         !same_params(ctx->graph_params, ctx->params))) {
      cudaGraphExecDestroy(ctx->graph_exec);
      ctx->graph_exec = nullptr;
    }
    if (!ctx->graph_exec) {
      cudaGraph_t g;
      const int64_t l0 = ctx->launches;
      CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
      rc = fa_enqueue(ctx, do_hausdorff);
      cudaGraph_t gg = nullptr;
      cudaError_t e = cudaStreamEndCapture(ctx->st, &gg);
      if (rc) {  // a failed capture is discarded, never launched
        if (gg) cudaGraphDestroy(gg);
        return rc;
      }
      if (e != cudaSuccess) return fail(ctx, HEXOPT_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
      g = gg;
      CK(cudaGraphInstantiate(&ctx->graph_exec, g, 0));
      cudaGraphDestroy(g);
      ctx->graph_hausdorff = do_hausdorff != 0;
      ctx->graph_tables = ctx->tables_epoch;
      ctx->graph_allocs = g_device_allocs.load(std::memory_order_relaxed);
      ctx->graph_params = ctx->params;
      ctx->graph_lamda0 = ctx->lamda0;
      ctx->graph_launches = ctx->launches - l0;  // kernels in one replay
      ctx->launches = l0;                        // capture executed nothing
    }
    CK(cudaGraphLaunch(ctx->graph_exec, ctx->st));
    ctx->launches += ctx->graph_launches;
  } else {
    rc = fa_enqueue(ctx, do_hausdorff);
    if (rc) return rc;
  }
  if (V) {
    rc = fa_queue_download(ctx, V);
    if (rc) return rc;
  }
  if (rep) {
    rc = pull_scalars(ctx);
    if (rc) return rc;
    for (int m = 0; m < ctx->n_meshes; m++) {
      const MeshScalars &S = ctx->sc[m];
      fill_report(S, ctx->md[m].nh, rep[m].slim);
      rep[m].quality.min_Jacobian = S.sj_min;
      rep[m].quality.ave_Jacobian = S.sj_sum / (double)ctx->md[m].nh;
      rep[m].quality.deviation_Jacobian = -1;  // the step skips the deviation pass
      rep[m].quality.n_inverted = S.n_inv;
      rep[m].lamda = S.lamda_C;
      rep[m].hausdorff_diag = do_hausdorff ? S.haus_diag : -1;
      rep[m].hausdorff_max = do_hausdorff ? S.haus_max : -1;
      rep[m].hausdorff_ave = do_hausdorff ? S.haus_ave : -1;
    }
  }
  return HEXOPT_OK;
}

int hexopt_use_graph(hexopt_ctx *ctx, int on) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (on < 0 || on > 2) return fail(ctx, HEXOPT_ERR_ARG, "use_graph: on must be 0, 1 or 2");
  const bool cond = on == 1;
  if (ctx->graph_exec && cond != ctx->graph_conditionals) {  // the captured form changes
    cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
  }
  ctx->graph_conditionals = cond;
  ctx->use_graph = on != 0;
  if (!ctx->use_graph && ctx->graph_exec) {
    cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
  }
  return HEXOPT_OK;
}

// ---------------------------------------------------------------- adaptive loop / untangling
int hexopt_slim_solve_adaptive(hexopt_ctx *ctx, int type, int schedule, int max_iter, hexopt_adaptive_report *rep) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!ctx->precomputed) return fail(ctx, HEXOPT_ERR_STATE, "slim_solve_adaptive before slim_precompute");
  if (type != 0 && type != 1) return fail(ctx, HEXOPT_ERR_ARG, "slim_solve_adaptive: type must be 0 (projection) or 1 (gluing)");
  if (schedule != 1 && schedule != 2) return fail(ctx, HEXOPT_ERR_ARG, "slim_solve_adaptive: schedule must be 1 or 2");
  if (max_iter < 1) return fail(ctx, HEXOPT_ERR_ARG, "slim_solve_adaptive: max_iter < 1");
  const int M = ctx->n_meshes;
  rc = pull_scalars(ctx);
  if (rc) return rc;
  for (int m = 0; m < M; m++) {
    ctx->sc[m].frozen = 0;
    if (schedule == 2) ctx->sc[m].lamda_G = 1e4;  // LAMDA_GLUE_MIN_BOUND (slim_m.cpp:1197)
  }
  rc = push_scalars(ctx);
  if (rc) return rc;
  CK(ctx->Xm.ensure(sizeof(double) * 4 * ctx->NV));
  std::vector<hexopt_adaptive_report> out(M);
  std::vector<char> done(M, 0);
  for (int m = 0; m < M; m++) { std::memset(&out[m], 0, sizeof out[m]); }
  for (int it = 0; it < max_iter; it++) {
    if (schedule == 1) {
      launch_glue_schedule(ctx->sc_d.as<MeshScalars>(), M, 1, it, ctx->st);
      ctx->launches++;
    }
    rc = dispatch_iteration(ctx);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->Xm.p, ctx->X.p, sizeof(double) * 4 * ctx->NV, cudaMemcpyDeviceToDevice, ctx->st));
    KArgs a = make_args(ctx);
    launch_result_positions(a, ctx->kind[K_CONS].nblk, ctx->Xm.as<double>(), type, ctx->st);
    if (schedule == 2 && type == 1) launch_glue_schedule(ctx->sc_d.as<MeshScalars>(), M, 0, it, ctx->st);
    a.X = ctx->Xm.as<double>();  // scaled_jacobian of the result mesh (data.ts.m)
    launch_scaled_jacobian(a, ctx->kind[K_HEX].nblk, nullptr, ctx->HJs.as<double>(), ctx->st);
    ctx->launches += 4;
    CKL();
    rc = pull_scalars(ctx);
    if (rc) return rc;
    bool all = true, changed = false;
    for (int m = 0; m < M; m++) {
      if (done[m]) continue;
      const MeshScalars &S = ctx->sc[m];
      hexopt_adaptive_report &r = out[m];
      r.iterations = it + 1;
      r.min_Jacobian = S.sj_min;
      r.ave_Jacobian = S.sj_sum / (double)ctx->md[m].nh;
      r.energy = S.energy / (S.M * 8.0 * (double)ctx->md[m].nh);
      r.energy_quality = S.eq;
      r.energy_soft = S.es;
      r.lamda_glue = S.lamda_G;
      r.status = S.status;
      if (S.sj_min > 0) {  // the result mesh is untangled: this mesh stops here
        r.converged = 1;
        done[m] = 1;
        ctx->sc[m].frozen = 1;
        changed = true;
      } else {
        all = false;
      }
    }
    if (all) break;
    if (changed) {
      rc = push_scalars(ctx);
      if (rc) return rc;
    }
  }
  if (rep)
    for (int m = 0; m < M; m++) rep[m] = out[m];
  return HEXOPT_OK;
}

int hexopt_untangle(hexopt_ctx *ctx, const hexopt_slim_params *params, const uint8_t *boundary, int max_iter,
                    hexopt_untangle_report *rep) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!params || !boundary) return fail(ctx, HEXOPT_ERR_ARG, "untangle: NULL params or boundary flags");
  if (params->precision != HEXOPT_FP64) return fail(ctx, HEXOPT_ERR_UNSUPPORTED, "untangle runs in HEXOPT_FP64");
  if (max_iter < 1) return fail(ctx, HEXOPT_ERR_ARG, "untangle: max_iter < 1");
  const int M = ctx->n_meshes;
  // the mesh's positions are the boundary-projected positions BV (optimization::assign_constraints)
  std::vector<double> BV(3 * ctx->NV);
  rc = hexopt_get_positions(ctx, BV.data());
  if (rc) return rc;
  // exploded mesh: hex h owns copies 8h..8h+7 of its corners (mesh-local numbering); copies of one
  // vertex form its glue group (V_ranges, optimization.cpp:556-575); copies of boundary vertices
  // are held (known_value_post, :590-615)
  std::vector<int64_t> nv_e(M), nh_e(M), n_groups(M), nfix(M, 0);
  std::vector<double> Ve(3 * 8 * (size_t)ctx->NH);
  std::vector<uint32_t> He(8 * (size_t)ctx->NH);
  std::vector<int64_t> gptr;
  std::vector<int32_t> gvs, fix_ids;
  for (int m = 0; m < M; m++) {
    const int64_t h0 = ctx->md[m].h_off, nh = ctx->md[m].nh, v0 = ctx->md[m].v_off, nv = ctx->md[m].nv;
    nv_e[m] = 8 * nh;
    nh_e[m] = nh;
    std::vector<int64_t> cnt(nv + 1, 0);
    for (int64_t h = 0; h < nh; h++)
      for (int c = 0; c < 8; c++) {
        const uint32_t v = ctx->H_h[8 * (h0 + h) + c];
        He[8 * (h0 + h) + c] = (uint32_t)(8 * h + c);
        for (int d = 0; d < 3; d++) Ve[3 * (8 * (h0 + h) + c) + d] = BV[3 * (v0 + v) + d];
        cnt[v + 1]++;
        if (boundary[v0 + v]) { fix_ids.push_back((int32_t)(8 * h + c)); nfix[m]++; }
      }
    for (int64_t v = 0; v < nv; v++) cnt[v + 1] += cnt[v];
    std::vector<int32_t> slot(cnt.begin(), cnt.end() - 1);
    std::vector<int32_t> mem(8 * nh);
    for (int64_t h = 0; h < nh; h++)
      for (int c = 0; c < 8; c++) mem[slot[ctx->H_h[8 * (h0 + h) + c]]++] = (int32_t)(8 * h + c);
    int64_t groups = 0;
    for (int64_t v = 0; v < nv; v++) {
      if (cnt[v + 1] == cnt[v]) continue;  // a vertex no hex uses
      gptr.push_back((int64_t)gvs.size() - 0);
      for (int64_t k = cnt[v]; k < cnt[v + 1]; k++) gvs.push_back(mem[k]);
      groups++;
    }
    gptr.push_back((int64_t)gvs.size());
    n_groups[m] = groups;
  }
  // group_ptr per mesh: n_groups[m] + 1 entries, offsets into that mesh's group_vs segment
  std::vector<int64_t> gptr_local;
  {
    size_t k = 0;
    for (int m = 0; m < M; m++) {
      const int64_t base = gptr[k];
      for (int64_t g = 0; g <= n_groups[m]; g++) gptr_local.push_back(gptr[k + g] - base);
      k += n_groups[m] + 1;
    }
  }
  hexopt_ctx *c = nullptr;
  rc = hexopt_create(&c, ctx->device);
  if (rc) return fail(ctx, rc, "untangle: cannot create the exploded-mesh context");
  struct Guard { hexopt_ctx *c; ~Guard() { hexopt_destroy(c); } } guard{c};
  auto sub = [&](int code, const char *what) {
    return fail(ctx, code, "untangle: %s: %s", what, hexopt_last_error(c));
  };
  if ((rc = hexopt_upload_meshes(c, M, nv_e.data(), nh_e.data(), Ve.data(), He.data(), nullptr))) return sub(rc, "upload");
  if ((rc = hexopt_set_fixed(c, nfix.data(), fix_ids.data()))) return sub(rc, "set_fixed");
  std::vector<double> lg(M, 1e4);
  if ((rc = hexopt_set_glue(c, n_groups.data(), gptr_local.data(), gvs.data(), lg.data()))) return sub(rc, "set_glue");
  // reference shapes: compute_referenceMesh(BV, mesh.Hs, all true, Hids, ts.RT, false) (:584)
  if ((rc = hexopt_set_reference_hexes(c, Ve.data()))) return sub(rc, "set_reference_hexes");
  // rigidDeformCubes: the starting copies (ts.V = Cubes)
  launch_rigid_cubes(c->hexv.as<uint32_t>(), c->X.as<double>(), c->X32.as<float>(), c->vfix.as<uint8_t>(), c->NH, c->st);
  c->launches++;
  {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, HEXOPT_ERR_CUDA, "untangle: rigid cubes: %s", cudaGetErrorString(e));
  }
  hexopt_slim_params p = *params;
  p.cube = 0;
  if ((rc = hexopt_slim_precompute(c, &p))) return sub(rc, "slim_precompute");
  std::vector<hexopt_adaptive_report> ar(M);
  if ((rc = hexopt_slim_solve_adaptive(c, 1, 2, max_iter, ar.data()))) return sub(rc, "slim_solve_adaptive");
  // the glued positions: each vertex at the mean of its copies (:651-660)
  KArgs a = make_args(c);
  CK(cudaMemcpyAsync(c->Xm.p, c->X.p, sizeof(double) * 4 * c->NV, cudaMemcpyDeviceToDevice, c->st));
  launch_result_positions(a, c->kind[K_CONS].nblk, c->Xm.as<double>(), 1, c->st);
  CK(c->stage.ensure(sizeof(double) * 3 * c->NV));
  launch_aos4_to_rows_perm(c->Xm.as<double>(), vo2n(c), c->NV, c->stage.as<double>(), c->st);
  std::vector<double> Xe(3 * (size_t)c->NV);
  CK(cudaMemcpyAsync(Xe.data(), c->stage.p, sizeof(double) * 3 * c->NV, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int m = 0; m < M; m++) {
    const int64_t h0 = ctx->md[m].h_off, nh = ctx->md[m].nh, v0 = ctx->md[m].v_off;
    for (int64_t h = 0; h < nh; h++)
      for (int cc = 0; cc < 8; cc++) {
        const uint32_t v = ctx->H_h[8 * (h0 + h) + cc];
        for (int d = 0; d < 3; d++) BV[3 * (v0 + v) + d] = Xe[3 * (8 * (h0 + h) + cc) + d];
      }
  }
  rc = hexopt_set_positions(ctx, BV.data());
  if (rc) return rc;
  std::vector<hexopt_quality> q(M);
  rc = hexopt_scaled_jacobian(ctx, nullptr, nullptr, q.data());
  if (rc) return rc;
  if (rep)
    for (int m = 0; m < M; m++) {
      rep[m].success = q[m].min_Jacobian < 0 ? 0 : 1;
      rep[m].iterations = ar[m].iterations;
      rep[m].min_Jacobian = q[m].min_Jacobian;
      rep[m].ave_Jacobian = q[m].ave_Jacobian;
      rep[m].energy = ar[m].energy;
      rep[m].lamda_glue = ar[m].lamda_glue;
    }
  return HEXOPT_OK;
}

// ---------------------------------------------------------------- adjoint
int hexopt_energy_fwd(hexopt_ctx *ctx, const double *X, double *E) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!ctx->precomputed) return fail(ctx, HEXOPT_ERR_STATE, "energy_fwd before slim_precompute");
  if (ctx->params.energy != HEXOPT_SYMMETRIC_DIRICHLET) return fail(ctx, HEXOPT_ERR_UNSUPPORTED, "adjoint: symmetric Dirichlet only");
  CK(ctx->Xa.ensure(sizeof(double) * 4 * ctx->NV));
  if (X) {
    CK(upload(ctx->stage, X, (size_t)3 * ctx->NV, ctx->st));
    launch_rows_to_aos4_perm(ctx->stage.as<double>(), vn2o(ctx), ctx->NV, ctx->Xa.as<double>(), ctx->st);
  } else {
    CK(cudaMemcpyAsync(ctx->Xa.p, ctx->X.p, sizeof(double) * 4 * ctx->NV, cudaMemcpyDeviceToDevice, ctx->st));
  }
  KArgs a = make_args(ctx);
  if (ctx->mixed) launch_energy_fwd<float>(a, ctx->kind[K_HEX].nblk, ctx->kind[K_CONS].nblk, ctx->st);
  else launch_energy_fwd<double>(a, ctx->kind[K_HEX].nblk, ctx->kind[K_CONS].nblk, ctx->st);
  ctx->launches += 3;
  CKL();
  rc = pull_scalars(ctx);
  if (rc) return rc;
  if (E)
    for (int m = 0; m < ctx->n_meshes; m++) E[m] = ctx->sc[m].adj_eq + ctx->sc[m].adj_es;
  ctx->adj_ready = true;
  return HEXOPT_OK;
}

int hexopt_energy_bwd(hexopt_ctx *ctx, double *grad) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!ctx->adj_ready) return fail(ctx, HEXOPT_ERR_STATE, "energy_bwd before energy_fwd");
  CK(ctx->grad.ensure(sizeof(double) * 4 * ctx->NV));
  CK(cudaMemsetAsync(ctx->grad.p, 0, sizeof(double) * 4 * ctx->NV, ctx->st));
  KArgs a = make_args(ctx);
  if (ctx->mixed) launch_energy_bwd<float>(a, ctx->kind[K_HEX].nblk, ctx->kind[K_CONS].nblk, ctx->st);
  else launch_energy_bwd<double>(a, ctx->kind[K_HEX].nblk, ctx->kind[K_CONS].nblk, ctx->st);
  ctx->launches += 2;
  CKL();
  if (grad) {
    CK(ctx->stage.ensure(sizeof(double) * 3 * ctx->NV));
    launch_aos4_to_rows_perm(ctx->grad.as<double>(), vo2n(ctx), ctx->NV, ctx->stage.as<double>(), ctx->st);
    ctx->launches++;
    CK(cudaMemcpyAsync(grad, ctx->stage.p, sizeof(double) * 3 * ctx->NV, cudaMemcpyDeviceToHost, ctx->st));
  }
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

// ---------------------------------------------------------------- tuning
int hexopt_set_block_size(hexopt_ctx *ctx, int kind, int threads) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (kind == 0) {
    if (threads != 32 && threads != 64 && threads != 128) return fail(ctx, HEXOPT_ERR_ARG, "hex block size must be 32, 64 or 128");
    ctx->block[K_HEX] = threads;
  } else if (kind == 1) {
    if (threads != 64 && threads != 128 && threads != 256) return fail(ctx, HEXOPT_ERR_ARG, "vertex block size must be 64, 128 or 256");
    ctx->block[K_VERT] = threads;
  } else if (kind == 2) {
    if (threads != 1 && threads != 2 && threads != 4 && threads != 8 && threads != 16)
      return fail(ctx, HEXOPT_ERR_ARG, "vertex items per thread must be 1, 2, 4, 8 or 16");
    ctx->ipt[K_VERT] = threads;
  } else {
    return fail(ctx, HEXOPT_ERR_ARG, "unknown kind");
  }
  if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
  if (ctx->n_meshes > 0) return rebuild_tables(ctx);
  return HEXOPT_OK;
}

// Times one SLIM iteration for each (hex block, vertex block, vertices per thread, line-search
// candidates) setting on a copy of the positions, keeps the fastest, restores the positions and
// scalars.
int hexopt_autotune(hexopt_ctx *ctx) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!ctx->precomputed) return fail(ctx, HEXOPT_ERR_STATE, "autotune before slim_precompute");
  CK(ctx->Xbak.ensure(sizeof(double) * 4 * ctx->NV));
  CK(cudaMemcpyAsync(ctx->Xbak.p, ctx->X.p, sizeof(double) * 4 * ctx->NV, cudaMemcpyDeviceToDevice, ctx->st));
  rc = pull_scalars(ctx);
  if (rc) return rc;
  const std::vector<MeshScalars> sc0 = ctx->sc;
  const int hb[2] = {64, 128}, vb[2] = {128, 256}, vi[2] = {4, 8};
  // candidate counts whose energy-pass variants run without register spills in each mode
  const int lc[3] = {1, 2, ctx->mixed ? 4 : 2};
  float best = INFINITY;
  int bh = ctx->block[K_HEX], bv = ctx->block[K_VERT], bi = ctx->ipt[K_VERT], bl = ctx->params.ls_candidates;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 4; j++)
      for (int k = 0; k < 3; k++) {
        ctx->block[K_HEX] = hb[i];
        ctx->block[K_VERT] = vb[j & 1];
        ctx->ipt[K_VERT] = vi[j >> 1];
        ctx->params.ls_candidates = lc[k];
        rc = rebuild_tables(ctx);
        if (rc) return rc;
        float ms = 0;
        for (int rep = 0; rep < 2; rep++) {
          CK(cudaMemcpyAsync(ctx->X.p, ctx->Xbak.p, sizeof(double) * 4 * ctx->NV, cudaMemcpyDeviceToDevice, ctx->st)); launch_split_pos(ctx->X.as<double>(), ctx->X32.as<float>(), ctx->NV, ctx->st);
          ctx->sc = sc0;
          rc = push_scalars(ctx);
          if (rc) return rc;
          CK(cudaEventRecord(e0, ctx->st));
          rc = dispatch_iteration(ctx);
          if (rc) return rc;
          CK(cudaEventRecord(e1, ctx->st));
          CK(cudaEventSynchronize(e1));
          CK(cudaEventElapsedTime(&ms, e0, e1));
        }
        if (ms < best) { best = ms; bh = hb[i]; bv = vb[j & 1]; bi = vi[j >> 1]; bl = lc[k]; }
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->block[K_HEX] = bh;
  ctx->block[K_VERT] = bv;
  ctx->ipt[K_VERT] = bi;
  ctx->params.ls_candidates = bl;
  rc = rebuild_tables(ctx);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ctx->X.p, ctx->Xbak.p, sizeof(double) * 4 * ctx->NV, cudaMemcpyDeviceToDevice, ctx->st)); launch_split_pos(ctx->X.as<double>(), ctx->X32.as<float>(), ctx->NV, ctx->st);
  ctx->sc = sc0;
  rc = push_scalars(ctx);
  if (rc) return rc;
  if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
  CK(cudaStreamSynchronize(ctx->st));
  return HEXOPT_OK;
}

int hexopt_get_tuning(const hexopt_ctx *ctx, int *hex_block, int *vert_block, int *vert_items, int *ls_candidates) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (hex_block) *hex_block = ctx->block[K_HEX];
  if (vert_block) *vert_block = ctx->block[K_VERT];
  if (vert_items) *vert_items = ctx->ipt[K_VERT];
  if (ls_candidates) *ls_candidates = ctx->params.ls_candidates;
  return HEXOPT_OK;
}

// ---------------------------------------------------------------- aabb.h value types
void hexopt_aabb_merge(hexopt_aabb *a, const hexopt_aabb *b) {
  for (int d = 0; d < 3; d++) {
    a->min[d] = std::min(a->min[d], b->min[d]);
    a->max[d] = std::max(a->max[d], b->max[d]);
  }
}
double hexopt_aabb_squared_distance(const hexopt_aabb *a, const double *p) {
  double s = 0;
  for (int d = 0; d < 3; d++) {
    double e = 0;
    if (p[d] < a->min[d]) e = a->min[d] - p[d];
    else if (p[d] > a->max[d]) e = p[d] - a->max[d];
    s += e * e;
  }
  return s;
}
// slab test (AABB::rayIntersect, aabb.h:21-48): 1 on hit with the entry/exit parameters
int hexopt_aabb_ray_intersect(const hexopt_aabb *a, const hexopt_ray *r, double *nearT, double *farT) {
  double n = -INFINITY, f = INFINITY;
  for (int i = 0; i < 3; i++) {
    const double origin = r->o[i], minVal = a->min[i], maxVal = a->max[i];
    if (r->d[i] == 0) {
      if (origin < minVal || origin > maxVal) return 0;
    } else {
      double t1 = (minVal - origin) * r->dRcp[i], t2 = (maxVal - origin) * r->dRcp[i];
      if (t1 > t2) std::swap(t1, t2);
      n = std::max(t1, n);
      f = std::min(t2, f);
      if (!(n <= f)) return 0;
    }
  }
  if (nearT) *nearT = n;
  if (farT) *farT = f;
  return r->mint <= f && n <= r->maxt;
}
int hexopt_aabb_largest_axis(const hexopt_aabb *a) {
  const double e0 = a->max[0] - a->min[0], e1 = a->max[1] - a->min[1], e2 = a->max[2] - a->min[2];
  if (e0 >= e1 && e0 >= e2) return 0;
  if (e1 >= e2) return 1;
  return 2;
}
double hexopt_aabb_surface_area(const hexopt_aabb *a) {
  const double e0 = a->max[0] - a->min[0], e1 = a->max[1] - a->min[1], e2 = a->max[2] - a->min[2];
  return 2.0 * (e0 * e1 + e1 * e2 + e2 * e0);
}


// ---------------------------------------------------------------- timing
int hexopt_timer_start(hexopt_ctx *ctx) {
  if (!ctx) return HEXOPT_ERR_ARG;
  if (!ctx->ev0) CK(cudaEventCreate(&ctx->ev0));
  if (!ctx->ev1) CK(cudaEventCreate(&ctx->ev1));
  CK(cudaEventRecord(ctx->ev0, ctx->st));
  return HEXOPT_OK;
}

int hexopt_timer_stop(hexopt_ctx *ctx, double *ms) {
  if (!ctx || !ctx->ev0) return HEXOPT_ERR_ARG;
  if (ctx->dst) CK(cudaStreamWaitEvent(ctx->st, ctx->out_done, 0));  // asynchronous downloads included
  CK(cudaEventRecord(ctx->ev1, ctx->st));
  CK(cudaEventSynchronize(ctx->ev1));
  float f = 0;
  CK(cudaEventElapsedTime(&f, ctx->ev0, ctx->ev1));
  if (ms) *ms = f;
  return HEXOPT_OK;
}

}  // extern "C"

template <typename ET, typename VT>
static void stage_launch(hexopt_ctx *ctx, int stage) {
  KArgs a = make_args(ctx);
  const int64_t hb = ctx->kind[K_HEX].nblk;
  switch (stage) {
    case 0: launch_spmv_elems<ET, VT>(a, hb, ctx->st); break;
    case 1: launch_local<ET, VT>(a, hb, false, ctx->st); break;
    case 2: launch_ls_energy_pass<ET, VT>(a, hb, ctx->st); break;
    case 3:  // the per-iteration quality check as the loop runs it
      if (ctx->mixed) launch_sj_check(a, hb, ctx->st);
      else launch_scaled_jacobian(a, hb, nullptr, ctx->HJs.as<double>(), ctx->st);
      break;
    case 6: launch_energy_fwd<ET>(a, hb, ctx->kind[K_CONS].nblk, ctx->st); break;
    case 7:
      cudaMemsetAsync(ctx->grad.p, 0, sizeof(double) * 4 * ctx->NV, ctx->st);
      launch_energy_bwd<ET>(a, hb, ctx->kind[K_CONS].nblk, ctx->st);
      break;
    case 4: run_projection(ctx); break;
    case 8: launch_cg_vec<VT>(a, ctx->kind[K_VERT].nblk, ctx->kind[K_CONS].nblk, ctx->st); break;
    case 9:
      if (ctx->mixed) launch_ir_residual(a, hb, ctx->kind[K_VERT].nblk, ctx->kind[K_CONS].nblk, true, ctx->st);
      break;
    default: break;
  }
}

extern "C" {

int hexopt_time_stage(hexopt_ctx *ctx, int stage, int reps, double *ms_per_launch) {
  int rc = check_ctx(ctx);
  if (rc) return rc;
  if (!ctx->precomputed) return fail(ctx, HEXOPT_ERR_STATE, "time_stage before slim_precompute");
  if (stage < 0 || stage > 9 || reps <= 0) return fail(ctx, HEXOPT_ERR_ARG, "time_stage: bad stage or reps");
  if ((stage == 6 || stage == 7) && (!ctx->Xa.p || !ctx->grad.p))
    return fail(ctx, HEXOPT_ERR_STATE, "time_stage: energy stages need one energy_fwd and one energy_bwd first");
  if (stage <= 2 || stage >= 8) {
    // make the solver state well defined (one iteration), then reopen the per-mesh CG and
    // line-search flags so the timed launches do their full work
    rc = dispatch_iteration(ctx);
    if (rc) return rc;
    rc = pull_scalars(ctx);
    if (rc) return rc;
    for (auto &S : ctx->sc) {
      S.cg_done = 0;
      S.ls_done = 0;
      if (stage == 8) {  // keep the timed PCG updates from reaching the convergence test
        S.cg_iters = -(1 << 30);
        S.threshold = -1.0;
      }
    }
    rc = push_scalars(ctx);
    if (rc) return rc;
    const unsigned open = (unsigned)ctx->n_meshes;
    CK(cudaMemcpyAsync(ctx->root_count.as<unsigned>() + 1, &open, sizeof(unsigned), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  rc = hexopt_timer_start(ctx);
  if (rc) return rc;
  for (int i = 0; i < reps; i++) {
    if (stage == 5) {
      rc = dispatch_iteration(ctx);
      if (rc) return rc;
    } else if (ctx->mixed) {
      stage_launch<float, float>(ctx, stage);
    } else {
      stage_launch<double, double>(ctx, stage);
    }
  }
  CKL();
  double ms = 0;
  rc = hexopt_timer_stop(ctx, &ms);
  if (rc) return rc;
  if (ms_per_launch) *ms_per_launch = ms / reps;
  return HEXOPT_OK;
}

}  // extern "C"
