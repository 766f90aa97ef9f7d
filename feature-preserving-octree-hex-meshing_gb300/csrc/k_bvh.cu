// k_bvh.cu -- closest-point projection and Hausdorff distance on a GPU LBVH.
//
//  * LBVH build (Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees and
//    k-d trees"): 30-bit Morton codes of triangle centroids made unique with the face index,
//    radix-sorted (CUB), internal nodes from the longest common prefix, boxes fitted bottom-up
//    with per-node arrival counters.  Boxes are FP32, rounded outward, so every distance lower
//    bound stays conservative.  Dynamic surfaces (the hex mesh boundary) keep the topology and
//    are refitted from the current positions; static trees (the targets) also get an oriented
//    box per node (principal axes of its vertices), which the target queries prune with.
//  * closest point: Ericson's point-triangle test in FP64 (as igl::point_simplex_squared_distance)
//    under a depth-first traversal with nearest-child-first order and strict-improvement updates
//    (AABB::squared_distance, AABB.cpp:366-445); pseudonormal of the winning face restates
//    igl::pseudonormal_test (pseudonormal_test.cpp:14-120).
//  * Hausdorff: vcg's PointDistanceEP (vcg/simplex/face/distance.h:49-180) minimised over the
//    faces of the other surface, vertex-sampled both ways, bbox inflated by 2% of its diagonal
//    (metro_hausdorff.cpp:358-506, sampling.h:224-289).
// Traversal stacks are bounded (kStack entries); an overflow sets HEXOPT_STATUS_BVH_OVERFLOW and
// the query continues without the dropped subtrees -- no unbounded loop.
#include "hexopt_common.cuh"
#include "hexopt_bvh.h"

namespace hexopt {

constexpr int kStack = 96;

// ------------------------------------------------------------------------------- build
__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__device__ __forceinline__ void face_pts(const BvhDev &b, int32_t f, double p[3][3]) {
  if (b.tri) {  // static: triangles stored per face id
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int d = 0; d < 3; d++) p[c][d] = b.tri[(int64_t)f * 9 + c * 3 + d];
  } else {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const int64_t v = b.F[(int64_t)f * 3 + c];
#pragma unroll
      for (int d = 0; d < 3; d++) p[c][d] = b.X[4 * v + d];
    }
  }
}

__global__ void k_morton(BvhDev b, double lo0, double lo1, double lo2, double inv0, double inv1, double inv2,
                         unsigned long long *keys) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n) return;
  double p[3][3];
  face_pts(b, i, p);
  const double cx = (p[0][0] + p[1][0] + p[2][0]) / 3, cy = (p[0][1] + p[1][1] + p[2][1]) / 3,
               cz = (p[0][2] + p[1][2] + p[2][2]) / 3;
  const uint32_t x = (uint32_t)fmin(fmax((cx - lo0) * inv0 * 1024.0, 0.0), 1023.0);
  const uint32_t y = (uint32_t)fmin(fmax((cy - lo1) * inv1 * 1024.0, 0.0), 1023.0);
  const uint32_t z = (uint32_t)fmin(fmax((cz - lo2) * inv2 * 1024.0, 0.0), 1023.0);
  const uint32_t code = (expand_bits(x) << 2) | (expand_bits(y) << 1) | expand_bits(z);
  keys[i] = ((unsigned long long)code << 32) | (unsigned long long)(uint32_t)i;
}

__device__ __forceinline__ int lcp(const unsigned long long *k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  return __clzll(k[i] ^ k[j]);
}

__global__ void k_karras(int n, const unsigned long long *keys, int32_t *child, int32_t *parent, int32_t *leaf_face,
                         int32_t *range) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) leaf_face[i] = (int32_t)(keys[i] & 0xffffffffull);
  if (i >= n - 1) return;
  const int d = (lcp(keys, n, i, i + 1) - lcp(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = lcp(keys, n, i, i - d);
  int lmax = 2;
  while (lmax < 2 * n && lcp(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (lcp(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = lcp(keys, n, i, j);
  int s = 0;
  int div = 2;
  int t = (l + div - 1) / div;
  while (true) {
    if (lcp(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
    div *= 2;
    t = (l + div - 1) / div;
  }
  const int gamma = i + s * d + (d < 0 ? d : 0);
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  if (range) { range[2 * i] = lo; range[2 * i + 1] = hi; }  // the node's leaves, sorted order
  const int32_t left = (lo == gamma) ? ~gamma : gamma;
  const int32_t right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  child[2 * i] = left;
  child[2 * i + 1] = right;
  // parent of internal node c is c; of leaf k is (n - 1) + k in the parent table
  parent[left >= 0 ? left : (n - 1) + ~left] = i;
  parent[right >= 0 ? right : (n - 1) + ~right] = i;
  if (i == 0) parent[0] = -1;
}

__device__ __forceinline__ float down(double x) { float f = __double2float_rd(x); return f; }
__device__ __forceinline__ float up(double x) { float f = __double2float_ru(x); return f; }

// Leaf boxes, leaf screening frames and bottom-up union.  counters: n - 1 zeros on entry, zeros
// again on exit.
// Refit of leaf k: its screening frame and box, then the bottom-up walk; the second child to
// arrive at an internal node forms that node's box (and, when `node` is given, its packed
// record from the two now-final child boxes).
__device__ __forceinline__ void refit_leaf(const BvhDev &b, float *box, const int32_t *parent, unsigned *counters,
                                           float4 *leafd, float4 *node_rec, int32_t k) {
  const int n = b.n;
  double p[3][3];
  face_pts(b, b.leaf_face[k], p);
  {
    const float ax = float(p[0][0]), ay = float(p[0][1]), az = float(p[0][2]);
    const float bx = float(p[1][0] - p[0][0]), by = float(p[1][1] - p[0][1]), bz = float(p[1][2] - p[0][2]);
    const float cx = float(p[2][0] - p[0][0]), cy = float(p[2][1] - p[0][1]), cz = float(p[2][2] - p[0][2]);
    leafd[3 * (int64_t)k] = make_float4(ax, ay, az, bx);
    leafd[3 * (int64_t)k + 1] = make_float4(by, bz, cx, cy);
    // unit normal of (p1 - p0) x (p2 - p0), formed in FP64 and rounded once
    const double ux = p[1][0] - p[0][0], uy = p[1][1] - p[0][1], uz = p[1][2] - p[0][2];
    const double vx = p[2][0] - p[0][0], vy = p[2][1] - p[0][1], vz = p[2][2] - p[0][2];
    double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    const double nn = sqrt(nx * nx + ny * ny + nz * nz);
    if (nn > 0) { nx /= nn; ny /= nn; nz /= nn; }
    leafd[3 * (int64_t)k + 2] = make_float4(cz, float(nx), float(ny), float(nz));
  }
  float *lb = box + 6 * (int64_t)(n - 1 + k);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    lb[d] = down(fmin(p[0][d], fmin(p[1][d], p[2][d])));
    lb[3 + d] = up(fmax(p[0][d], fmax(p[1][d], p[2][d])));
  }
  if (n == 1) return;
  int32_t node = parent[n - 1 + k];
  __threadfence();
  for (int hops = 0; node >= 0 && node < n - 1 && hops < n; hops++) {  // bounded walk to the root
    if (atomicAdd(&counters[node], 1u) == 0) return;  // first child to arrive: the other finishes
    __threadfence();
    const int32_t l = b.child[2 * node], r = b.child[2 * node + 1];
    const float *bl = box + 6 * (int64_t)(l >= 0 ? l : n - 1 + ~l);
    const float *br = box + 6 * (int64_t)(r >= 0 ? r : n - 1 + ~r);
    float L[6], R[6];
#pragma unroll
    for (int d = 0; d < 6; d++) { L[d] = __ldcg(bl + d); R[d] = __ldcg(br + d); }
    float *bn = box + 6 * (int64_t)node;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      bn[d] = fminf(L[d], R[d]);
      bn[3 + d] = fmaxf(L[3 + d], R[3 + d]);
    }
    if (node_rec) {
      node_rec[4 * (int64_t)node] = make_float4(L[0], L[1], L[2], L[3]);
      node_rec[4 * (int64_t)node + 1] = make_float4(L[4], L[5], R[0], R[1]);
      node_rec[4 * (int64_t)node + 2] = make_float4(R[2], R[3], R[4], R[5]);
      node_rec[4 * (int64_t)node + 3] = make_float4(__int_as_float(l), __int_as_float(r), 0.f, 0.f);
    }
    counters[node] = 0;
    __threadfence();
    node = parent[node];
  }
}

// Leaf boxes, leaf screening frames and bottom-up union.  counters: n - 1 zeros on entry, zeros
// again on exit.
__global__ void k_refit(BvhDev b, float *box, const int32_t *parent, unsigned *counters, float4 *leafd) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.n) return;
  refit_leaf(b, box, parent, counters, leafd, nullptr, k);
}

// All meshes' surface trees at once: one thread per surface face of the batch.
__global__ void k_refit_batch(const RefitDev *R, const Seg *seg, const MeshDesc *md) {
  const Seg sg = seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const RefitDev &r = R[sg.mesh];
  const int32_t k = (int32_t)(i - md[sg.mesh].kitem0[K_SURFF]);
  if (k >= r.b.n) return;
  refit_leaf(r.b, r.box, r.parent, r.counters, r.leafd, r.node, k);
}

// ------------------------------------------------------------------------------- oriented boxes
// Static trees (the targets) also carry an oriented box per node: rows a0..a2 of an orthonormal
// frame rounded to FP32 and extents [lo_k, hi_k] of the node's vertices along them, formed in
// FP64 with the stored rows and rounded outward, so lo_k <= a_k . x <= hi_k for every point x of
// every triangle below the node.  A leaf takes its triangle's frame (first edge, in-plane normal
// to it, normal: zero thickness); an internal node of at most kObbLeaves leaves the principal axes
// of its vertices, and keeps them only where they enclose less volume than the axis-aligned box
// (which larger nodes always use).  Queries that start well away from a curved surface reach
// many more tilted axis-aligned boxes than oriented ones: on a 200k-triangle superellipsoid with
// queries on the faces of a cube around it, about a third of the internal nodes.
constexpr int kObbLeaves = 1024;

// Eigenvectors of a symmetric 3x3 matrix (cyclic Jacobi rotations, FP64), as the columns of v.
__device__ void sym3_eigvecs(double a[3][3], double v[3][3]) {
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) v[r][c] = r == c ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 16; sweep++) {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    const double dia = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (!(off > 1e-30 * dia)) break;
    for (int pq = 0; pq < 3; pq++) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const double apq = a[p][q];
      if (apq == 0.0) continue;
      const double th = (a[q][q] - a[p][p]) / (2.0 * apq);
      const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
      const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
      for (int k = 0; k < 3; k++) {  // columns p, q of a J
        const double akp = a[k][p], akq = a[k][q];
        a[k][p] = c * akp - sn * akq;
        a[k][q] = sn * akp + c * akq;
      }
      for (int k = 0; k < 3; k++) {  // rows p, q of J^T a
        const double apk = a[p][k], aqk = a[q][k];
        a[p][k] = c * apk - sn * aqk;
        a[q][k] = sn * apk + c * aqk;
      }
      for (int k = 0; k < 3; k++) {
        const double vkp = v[k][p], vkq = v[k][q];
        v[k][p] = c * vkp - sn * vkq;
        v[k][q] = sn * vkp + c * vkq;
      }
    }
  }
}

// Extents of points along the stored (FP32) rows, in FP64; rounded outward by obb_store.
struct ObbAcc {
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  double scale = 1.0;
  __device__ void add(const float a[3][3], const double p[3]) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double u = double(a[k][0]) * p[0] + double(a[k][1]) * p[1] + double(a[k][2]) * p[2];
      mn[k] = fmin(mn[k], u);
      mx[k] = fmax(mx[k], u);
    }
    scale = fmax(scale, 1.0 + fabs(p[0]) + fabs(p[1]) + fabs(p[2]));
  }
};

// 64-byte node box: (a0, a1.x), (a1.yz, a2.xy), (a2.z, lo), (hi, id -- set when packed)
__device__ void obb_store(float4 *o, const float a[3][3], const ObbAcc &acc) {
  float lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {  // the FP64 extents carry at most a few ulps of |p|_1
    lo[k] = __double2float_rd(acc.mn[k] - 1e-12 * acc.scale);
    hi[k] = __double2float_ru(acc.mx[k] + 1e-12 * acc.scale);
  }
  o[0] = make_float4(a[0][0], a[0][1], a[0][2], a[1][0]);
  o[1] = make_float4(a[1][1], a[1][2], a[2][0], a[2][1]);
  o[2] = make_float4(a[2][2], lo[0], lo[1], lo[2]);
  o[3] = make_float4(hi[0], hi[1], hi[2], 0.f);
}

__device__ __forceinline__ void unit_rows(float a[3][3]) {
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) a[r][c] = r == c ? 1.f : 0.f;
}

// leaves (sorted order): the triangle's own frame, or the coordinate axes if it is degenerate
__global__ void k_obb_leaf(BvhDev b, float4 *obb) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.n) return;
  double p[3][3];
  face_pts(b, b.leaf_face[k], p);
  const double e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
  const double e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
  const double nr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
  const double l1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
  const double l2 = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
  const double ln = sqrt(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
  float a[3][3];
  unit_rows(a);
  if (l1 > 0.0 && ln > 1e-9 * l1 * l2) {
    const double u[3] = {e1[0] / l1, e1[1] / l1, e1[2] / l1}, w[3] = {nr[0] / ln, nr[1] / ln, nr[2] / ln};
    const double v[3] = {w[1] * u[2] - w[2] * u[1], w[2] * u[0] - w[0] * u[2], w[0] * u[1] - w[1] * u[0]};
    for (int c = 0; c < 3; c++) { a[0][c] = float(u[c]); a[1][c] = float(v[c]); a[2][c] = float(w[c]); }
  }
  ObbAcc acc;
  for (int c = 0; c < 3; c++) acc.add(a, p[c]);
  obb_store(obb + 4 * (int64_t)(b.n - 1 + k), a, acc);
}

// internal nodes: principal axes of the vertices below (up to kObbLeaves leaves) where they
// enclose less volume than the axis-aligned box, else that box
__global__ void k_obb_node(BvhDev b, const int32_t *range, float4 *obb) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n - 1) return;
  const float *bx = b.box + 6 * (int64_t)i;
  float a[3][3];
  unit_rows(a);
  ObbAcc acc;
  for (int k = 0; k < 3; k++) { acc.mn[k] = bx[k]; acc.mx[k] = bx[3 + k]; }
  acc.scale = 0.0;  // the box's floats are kept as they are
  const int32_t lo = range[2 * i], hi = range[2 * i + 1];
  if (lo >= 0 && hi < b.n && hi - lo + 1 <= kObbLeaves) {
    double p[3][3];
    face_pts(b, b.leaf_face[lo], p);
    const double o[3] = {p[0][0], p[0][1], p[0][2]};
    double s1[3] = {0, 0, 0}, s2[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int32_t k = lo; k <= hi; k++) {
      face_pts(b, b.leaf_face[k], p);
      for (int c = 0; c < 3; c++) {
        const double d[3] = {p[c][0] - o[0], p[c][1] - o[1], p[c][2] - o[2]};
        for (int r = 0; r < 3; r++) {
          s1[r] += d[r];
          for (int t = 0; t < 3; t++) s2[r][t] += d[r] * d[t];
        }
      }
    }
    const double cnt = 3.0 * double(hi - lo + 1);
    double cv[3][3], v[3][3];
    for (int r = 0; r < 3; r++)
      for (int t = 0; t < 3; t++) cv[r][t] = s2[r][t] / cnt - (s1[r] / cnt) * (s1[t] / cnt);
    sym3_eigvecs(cv, v);
    float ar[3][3];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) ar[r][c] = float(v[c][r]);
    ObbAcc oa;
    for (int32_t k = lo; k <= hi; k++) {
      face_pts(b, b.leaf_face[k], p);
      for (int c = 0; c < 3; c++) oa.add(ar, p[c]);
    }
    // compare enclosed volumes (extents padded so that flat boxes still compare)
    const double pad = 1e-9 * oa.scale;
    double vo = 1.0, va = 1.0;
    for (int k = 0; k < 3; k++) {
      vo *= oa.mx[k] - oa.mn[k] + pad;
      va *= double(bx[3 + k]) - double(bx[k]) + pad;
    }
    if (vo < va) {
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) a[r][c] = ar[r][c];
      acc = oa;
    }
  }
  obb_store(obb + 4 * (int64_t)i, a, acc);
}

// 128-byte oriented node records: both children's boxes, each with the child's id in its last lane
__global__ void k_opack(int n, const int32_t *child, const float4 *obb, float4 *onode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  for (int s = 0; s < 2; s++) {
    const int32_t c = child[2 * i + s];
    float4 *o = onode + 8 * (int64_t)i + 4 * s;
    if (c >= 0 ? c >= n - 1 : ~c >= n) {  // malformed: an unbounded box, reported when visited
      o[0] = make_float4(1.f, 0.f, 0.f, 0.f);
      o[1] = make_float4(1.f, 0.f, 0.f, 0.f);
      o[2] = make_float4(1.f, -INFINITY, -INFINITY, -INFINITY);
      o[3] = make_float4(INFINITY, INFINITY, INFINITY, __int_as_float(c));
      continue;
    }
    const float4 *f = obb + 4 * (int64_t)(c >= 0 ? c : n - 1 + ~c);
    o[0] = f[0];
    o[1] = f[1];
    o[2] = f[2];
    float4 t = f[3];
    t.w = __int_as_float(c);
    o[3] = t;
  }
}

// ------------------------------------------------------------------------------- queries
__device__ __forceinline__ double box_d2(const float *bx, const double q[3]) {
  double s = 0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double lo = bx[d], hi = bx[3 + d];
    const double e = q[d] < lo ? lo - q[d] : (q[d] > hi ? q[d] - hi : 0.0);
    s += e * e;
  }
  return s;
}

// FP64 arithmetic with every product and sum rounded on its own (no fused multiply-add), in the
// operation order of the reference's CPU code, so the exact evaluations below give its bits.
__device__ __forceinline__ double nmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double nadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double nsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ndot(const double *a, const double *b) {
  return nadd(nadd(nmul(a[0], b[0]), nmul(a[1], b[1])), nmul(a[2], b[2]));
}
__device__ __forceinline__ void nsub3(const double *a, const double *b, double *o) {
  o[0] = nsub(a[0], b[0]); o[1] = nsub(a[1], b[1]); o[2] = nsub(a[2], b[2]);
}
__device__ __forceinline__ void ncross(const double *a, const double *b, double *o) {
  o[0] = nsub(nmul(a[1], b[2]), nmul(a[2], b[1]));
  o[1] = nsub(nmul(a[2], b[0]), nmul(a[0], b[2]));
  o[2] = nsub(nmul(a[0], b[1]), nmul(a[1], b[0]));
}

// Ericson's closest point on triangle (Real-Time Collision Detection 5.1.5), FP64, as
// igl::point_simplex_squared_distance (point_simplex_squared_distance.cpp:25-130).
__device__ void closest_pt_tri(const double p[3], const double a[3], const double b[3], const double c[3],
                               double out[3]) {
  double ab[3], ac[3], ap[3], bp[3], cp[3];
  nsub3(b, a, ab); nsub3(c, a, ac); nsub3(p, a, ap);
  const double d1 = ndot(ab, ap), d2 = ndot(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) { out[0] = a[0]; out[1] = a[1]; out[2] = a[2]; return; }
  nsub3(p, b, bp);
  const double d3 = ndot(ab, bp), d4 = ndot(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) { out[0] = b[0]; out[1] = b[1]; out[2] = b[2]; return; }
  const double vc = nsub(nmul(d1, d4), nmul(d3, d2));
  if (!(a[0] == b[0] && a[1] == b[1] && a[2] == b[2]) && vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
    const double v = d1 / nsub(d1, d3);
#pragma unroll
    for (int d = 0; d < 3; d++) out[d] = nadd(a[d], nmul(v, ab[d]));
    return;
  }
  nsub3(p, c, cp);
  const double d5 = ndot(ab, cp), d6 = ndot(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) { out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; return; }
  const double vb = nsub(nmul(d5, d2), nmul(d1, d6));
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    const double w = d2 / nsub(d2, d6);
#pragma unroll
    for (int d = 0; d < 3; d++) out[d] = nadd(a[d], nmul(w, ac[d]));
    return;
  }
  const double va = nsub(nmul(d3, d6), nmul(d5, d4));
  const double d43 = nsub(d4, d3), d56 = nsub(d5, d6);
  if (va <= 0.0 && d43 >= 0.0 && d56 >= 0.0) {
    const double w = d43 / nadd(d43, d56);
#pragma unroll
    for (int d = 0; d < 3; d++) out[d] = nadd(b[d], nmul(w, nsub(c[d], b[d])));
    return;
  }
  const double denom = 1.0 / nadd(nadd(va, vb), vc);
  const double v = nmul(vb, denom), w = nmul(vc, denom);
#pragma unroll
  for (int d = 0; d < 3; d++) out[d] = nadd(nadd(a[d], nmul(ab[d], v)), nmul(ac[d], w));
}

// ---- FP32 filtering with exact FP64 evaluation ----
// Traversal and leaf screening run in FP32 on coordinates taken relative to the leaf's first
// vertex (formed in FP64, rounded once); only the leaves that FP32 cannot rule out are evaluated
// in FP64, so the FP64 result is the one a pure FP64 search returns.  Boxes are stored rounded
// outward and the box margin covers the rounding of the query.
__device__ __forceinline__ float box_d2f(const float *bx, const float q[3]) {
  float s = 0.f;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const float e = fmaxf(fmaxf(bx[d] - q[d], q[d] - bx[3 + d]), 0.f);
    s = fmaf(e, e, s);
  }
  return s;
}

// FP32 segment distance |q - (v1 + t (v2 - v1))|, t clamped to [0, 1] (the ps_dist below).
__device__ __forceinline__ float seg_df(const float q[3], const float v1[3], const float v2[3]) {
  const float e[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
  const float w[3] = {q[0] - v1[0], q[1] - v1[1], q[2] - v1[2]};
  const float ee = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
  float t = ee > 0.f ? (w[0] * e[0] + w[1] * e[1] + w[2] * e[2]) / ee : 0.f;
  t = fminf(fmaxf(t, 0.f), 1.f);
  const float d0 = w[0] - e[0] * t, d1 = w[1] - e[1] * t, d2 = w[2] - e[2] * t;
  return sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
}

// ((v2 - v1) x (p - v1)) . n: the edge test of PointDistanceEP without its dominant-axis scaling
// (the projected 2-D cross product divided by n[axis] equals this for p in the plane).
__device__ __forceinline__ float edge_side(const float v1[3], const float v2[3], const float p[3], const float n[3]) {
  const float e[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
  const float w[3] = {p[0] - v1[0], p[1] - v1[1], p[2] - v1[2]};
  return (e[1] * w[2] - e[2] * w[1]) * n[0] + (e[2] * w[0] - e[0] * w[2]) * n[1] + (e[0] * w[1] - e[1] * w[0]) * n[2];
}

// FP32 bounds [lo, hi] of the exact FP64 distance from the query to leaf `leaf`'s triangle under
// the metric of MODE, from the leaf's FP32 screening frame (first vertex, the two edges from it,
// unit normal formed in FP64).  m = 1e-4 of the local scale plus 1e-6 of the absolute
// coordinates covers the FP32 evaluation; an edge test is decided only outside its error band
// (tb per unit edge length).
//   MODE 0 (Euclidean, the projection metric): the distance is the plane distance |d| when the
//     projection is inside, else the smallest of the three edge-segment distances, and it never
//     exceeds that smallest segment distance.  lo takes |d| when the projection may be inside,
//     hi only when it is inside for sure -- valid for any triangle shape.
//   MODE 1 (PointDistanceEP, the Hausdorff metric): follows the first failing edge test rather
//     than the nearest feature, so it can exceed the Euclidean distance; the FP64 branch is
//     replayed in FP32 and hi is INFINITY where a test falls inside its band (lo = |d| - m, as
//     the metric always measures to a point in the plane of the triangle).
// Triangles whose smallest angle is below ~1e-6 rad take `boxd` as lo and the largest vertex
// distance as hi (both metrics measure to a point of the triangle).
template <int MODE>
__device__ __forceinline__ void leaf_bounds(const float4 *leafd, int32_t leaf, const float qf[3], float boxd, float &lo,
                                            float &hi) {
  const float4 u = __ldg(leafd + 3 * (int64_t)leaf), v = __ldg(leafd + 3 * (int64_t)leaf + 1),
               w = __ldg(leafd + 3 * (int64_t)leaf + 2);
  const float qa[3] = {qf[0] - u.x, qf[1] - u.y, qf[2] - u.z};
  const float ab[3] = {u.w, v.x, v.y}, ac[3] = {v.z, v.w, w.x};
  const float cx = ab[1] * ac[2] - ab[2] * ac[1], cy = ab[2] * ac[0] - ab[0] * ac[2], cz = ab[0] * ac[1] - ab[1] * ac[0];
  const float lab = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2], lac = ac[0] * ac[0] + ac[1] * ac[1] + ac[2] * ac[2];
  const float c2 = cx * cx + cy * cy + cz * cz;
  const float L = fabsf(qa[0]) + fabsf(qa[1]) + fabsf(qa[2]) + sqrtf(lab) + sqrtf(lac);
  const float abs_scale = 1.f + fabsf(qf[0]) + fabsf(qf[1]) + fabsf(qf[2]);
  const float m = 1e-4f * L + 1e-6f * abs_scale;
  if (!(c2 >= 1e-12f * lab * lac)) {
    const float qb[3] = {qa[0] - ab[0], qa[1] - ab[1], qa[2] - ab[2]}, qc[3] = {qa[0] - ac[0], qa[1] - ac[1], qa[2] - ac[2]};
    const float da = qa[0] * qa[0] + qa[1] * qa[1] + qa[2] * qa[2], db = qb[0] * qb[0] + qb[1] * qb[1] + qb[2] * qb[2],
                dc = qc[0] * qc[0] + qc[1] * qc[1] + qc[2] * qc[2];
    lo = boxd;
    hi = sqrtf(fmaxf(fmaxf(da, db), dc)) + m;
    return;
  }
  const float n[3] = {w.y, w.z, w.w};
  const float d = n[0] * qa[0] + n[1] * qa[1] + n[2] * qa[2];
  const float ad = fabsf(d);
  const float p[3] = {qa[0] - n[0] * d, qa[1] - n[1] * d, qa[2] - n[2] * d};
  const float P0[3] = {0.f, 0.f, 0.f};
  const float tb = m + 3e-6f * abs_scale;
  const float lbc = sqrtf((ac[0] - ab[0]) * (ac[0] - ab[0]) + (ac[1] - ab[1]) * (ac[1] - ab[1]) + (ac[2] - ab[2]) * (ac[2] - ab[2]));
  const float t0 = tb * lbc, t1 = tb * sqrtf(lac), t2 = tb * sqrtf(lab);
  const float b0 = edge_side(ab, ac, p, n), b1 = edge_side(ac, P0, p, n), b2 = edge_side(P0, ab, p, n);
  if (MODE == 0) {
    const float smin = fminf(fminf(seg_df(qa, ab, ac), seg_df(qa, ac, P0)), seg_df(qa, P0, ab));
    const bool maybe_in = b0 > -t0 && b1 > -t1 && b2 > -t2;
    const bool surely_in = b0 > t0 && b1 > t1 && b2 > t2;
    lo = (maybe_in ? fminf(ad, smin) : smin) - m;
    hi = (surely_in ? fminf(ad, smin) : smin) + m;
    return;
  }
  lo = ad - m;
  hi = INFINITY;
  float val;
  if (fabsf(b0) <= t0) return;
  if (b0 < 0.f) { val = seg_df(qa, ab, ac); }
  else if (fabsf(b1) <= t1) return;
  else if (b1 < 0.f) { val = seg_df(qa, ac, P0); }
  else if (fabsf(b2) <= t2) return;
  else if (b2 < 0.f) { val = seg_df(qa, P0, ab); }
  else {
    // all three tests pass: interior unless the smallest is under 1e-6 of twice the area
    const float T = 1e-6f * sqrtf(c2);
    const float bm = fminf(fminf(b0, b1), b2);
    const float tm = fmaxf(fmaxf(t0, t1), t2) + 1e-4f * T;
    if (bm > T + tm) val = ad;
    else if (bm < T - tm) {
      // the smallest test picks the edge; a near tie between two of them is undecided
      const int k = (bm == b0) ? 0 : (bm == b1 ? 1 : 2);
      const float o1 = k == 0 ? b1 : b0, o2 = k == 2 ? b1 : b2;
      if (fminf(o1, o2) - bm <= 2.f * tm) return;
      val = k == 0 ? seg_df(qa, ab, ac) : (k == 1 ? seg_df(qa, ac, P0) : seg_df(qa, P0, ab));
    } else {
      return;
    }
  }
  lo = fmaxf(lo, val - m);
  hi = val + m;
}

struct EPFace {
  double p[3][3], edge[3][3], dir[3], off, darea;
  int axis;
};

__device__ void ep_setup(const double P[3][3], EPFace &e) {
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) e.p[c][d] = P[c][d];
  nsub3(P[1], P[0], e.edge[0]);
  nsub3(P[2], P[1], e.edge[1]);
  nsub3(P[0], P[2], e.edge[2]);
  ncross(e.edge[0], e.edge[1], e.dir);
  e.off = ndot(e.dir, P[0]);
  const double nn = sqrt(ndot(e.dir, e.dir));
  if (nn > 0) { e.dir[0] /= nn; e.dir[1] /= nn; e.dir[2] /= nn; e.off /= nn; }
  const double nx = fabs(e.dir[0]), ny = fabs(e.dir[1]), nz = fabs(e.dir[2]);
  double s;
  if (nx > ny && nx > nz) { e.axis = 0; s = 1 / e.dir[0]; }
  else if (ny > nz) { e.axis = 1; s = 1 / e.dir[1]; }
  else { e.axis = 2; s = 1 / e.dir[2]; }
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) e.edge[c][d] = nmul(e.edge[c][d], s);
  double a[3], b[3], x[3];
  nsub3(P[1], P[0], a);
  nsub3(P[2], P[0], b);
  ncross(a, b, x);
  e.darea = sqrt(ndot(x, x));
}

// The set-up above, stored per face (16 doubles) and read back: the same bits as forming it anew.
__device__ __forceinline__ void ep_store(const EPFace &e, double *o) {
  double2 *w = reinterpret_cast<double2 *>(o);
  w[0] = make_double2(e.edge[0][0], e.edge[0][1]);
  w[1] = make_double2(e.edge[0][2], e.edge[1][0]);
  w[2] = make_double2(e.edge[1][1], e.edge[1][2]);
  w[3] = make_double2(e.edge[2][0], e.edge[2][1]);
  w[4] = make_double2(e.edge[2][2], e.dir[0]);
  w[5] = make_double2(e.dir[1], e.dir[2]);
  w[6] = make_double2(e.off, e.darea);
  w[7] = make_double2(double(e.axis), 0.0);
}
__device__ __forceinline__ void ep_load(const double *o, const double P[3][3], EPFace &e) {
  const double2 *w = reinterpret_cast<const double2 *>(o);
  const double2 w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2), w3 = __ldg(w + 3), w4 = __ldg(w + 4),
                w5 = __ldg(w + 5), w6 = __ldg(w + 6), w7 = __ldg(w + 7);
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) e.p[c][d] = P[c][d];
  e.edge[0][0] = w0.x; e.edge[0][1] = w0.y; e.edge[0][2] = w1.x;
  e.edge[1][0] = w1.y; e.edge[1][1] = w2.x; e.edge[1][2] = w2.y;
  e.edge[2][0] = w3.x; e.edge[2][1] = w3.y; e.edge[2][2] = w4.x;
  e.dir[0] = w4.y; e.dir[1] = w5.x; e.dir[2] = w5.y;
  e.off = w6.x; e.darea = w6.y;
  e.axis = int(w7.x);
}

__global__ void k_ep_faces(const double *tri, int64_t nf, double *EP) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  double P[3][3];
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) P[c][d] = tri[f * 9 + c * 3 + d];
  EPFace e;
  ep_setup(P, e);
  ep_store(e, EP + 16 * f);
}

__device__ __forceinline__ double ps_dist(const double q[3], const double *v1, const double *v2) {
  double e[3], qv[3], pp[3];
  nsub3(v2, v1, e);
  nsub3(q, v1, qv);
  double t = ndot(qv, e) / ndot(e, e);
  t = t < 0 ? 0 : (t > 1 ? 1 : t);
#pragma unroll
  for (int d = 0; d < 3; d++) pp[d] = nsub(q[d], nadd(v1[d], nmul(e[d], t)));
  return sqrt(ndot(pp, pp));
}

__device__ void point_distance_ep(const EPFace &f, const double q[3], double &dist) {
  const double EPS = 0.000001;
  const double d = nsub(ndot(f.dir, q), f.off);
  if (d > dist || d < -dist) return;
  const double p[3] = {nsub(q[0], nmul(f.dir[0], d)), nsub(q[1], nmul(f.dir[1], d)), nsub(q[2], nmul(f.dir[2], d))};
  const int i1 = f.axis == 0 ? 1 : (f.axis == 1 ? 2 : 0), i2 = f.axis == 0 ? 2 : (f.axis == 1 ? 0 : 1);
  const double b0 = nsub(nmul(f.edge[1][i1], nsub(p[i2], f.p[1][i2])), nmul(f.edge[1][i2], nsub(p[i1], f.p[1][i1])));
  if (b0 <= 0) { const double x = ps_dist(q, f.p[1], f.p[2]); if (dist > x) dist = x; return; }
  const double b1 = nsub(nmul(f.edge[2][i1], nsub(p[i2], f.p[2][i2])), nmul(f.edge[2][i2], nsub(p[i1], f.p[2][i1])));
  if (b1 <= 0) { const double x = ps_dist(q, f.p[2], f.p[0]); if (dist > x) dist = x; return; }
  const double b2 = nsub(nmul(f.edge[0][i1], nsub(p[i2], f.p[0][i2])), nmul(f.edge[0][i2], nsub(p[i1], f.p[0][i1])));
  if (b2 <= 0) { const double x = ps_dist(q, f.p[0], f.p[1]); if (dist > x) dist = x; return; }
  double b = fmin(b0, b1);
  b = fmin(b, b2);
  if (b < nmul(EPS, f.darea)) {
    double bt;
    if (b == b0) bt = ps_dist(q, f.p[1], f.p[2]);
    else if (b == b1) bt = ps_dist(q, f.p[2], f.p[0]);
    else bt = ps_dist(q, f.p[0], f.p[1]);
    if (dist > bt) dist = bt;
    return;
  }
  dist = fabs(d);
}

// ---- traversal over packed nodes ----
// Each internal node is one 64-byte record with both children's boxes and ids, so a step is one
// dependent load.  Stack entries carry the box lower bound they were pushed with, so entries made
// obsolete by a later improvement are dropped when popped.
struct NodeRec { float lb[6], rb[6]; int32_t l, r; };
__device__ __forceinline__ NodeRec load_node(const float4 *node, int32_t i) {
  const float4 a = __ldg(node + 4 * (int64_t)i), b = __ldg(node + 4 * (int64_t)i + 1), c = __ldg(node + 4 * (int64_t)i + 2),
               d = __ldg(node + 4 * (int64_t)i + 3);
  NodeRec r;
  r.lb[0] = a.x; r.lb[1] = a.y; r.lb[2] = a.z; r.lb[3] = a.w; r.lb[4] = b.x; r.lb[5] = b.y;
  r.rb[0] = b.z; r.rb[1] = b.w; r.rb[2] = c.x; r.rb[3] = c.y; r.rb[4] = c.z; r.rb[5] = c.w;
  r.l = __float_as_int(d.x); r.r = __float_as_int(d.y);
  return r;
}

// Lower bound of the distance from qf to anything inside an oriented box (one half of a 128-byte
// record).  The rows are orthonormal to FP32 rounding (norm <= 1 + 2e-7), the projections carry
// a few ulps of |q|_1 and qf differs from the FP64 query by an ulp: mob = 2e-6 (1 + |qf|_1) and
// the relative factor cover all of it.
__device__ __forceinline__ float obb_dist(const float4 &f0, const float4 &f1, const float4 &f2, const float4 &f3,
                                          const float qf[3], float mob) {
  const float u0 = f0.x * qf[0] + f0.y * qf[1] + f0.z * qf[2];
  const float u1 = f0.w * qf[0] + f1.x * qf[1] + f1.y * qf[2];
  const float u2 = f1.z * qf[0] + f1.w * qf[1] + f2.x * qf[2];
  const float e0 = fmaxf(fmaxf(f2.y - u0, u0 - f3.x), 0.f);
  const float e1 = fmaxf(fmaxf(f2.z - u1, u1 - f3.y), 0.f);
  const float e2 = fmaxf(fmaxf(f2.w - u2, u2 - f3.z), 0.f);
  return sqrtf(e0 * e0 + e1 * e1 + e2 * e2) * (1.f - 1e-6f) - mob;
}

// Both children of internal node `node` with their lower bounds: oriented records (OB, static
// trees) or axis-aligned ones.  mbox = 1e-6 (1 + |qf|_1).
template <bool OB>
__device__ __forceinline__ void node_children(const BvhDev &b, int32_t node, const float qf[3], float mbox,
                                              int32_t &l, int32_t &r, float &dl, float &dr) {
  if constexpr (OB) {
    const float4 *o = b.onode + 8 * (int64_t)node;
    const float4 a0 = __ldg(o), a1 = __ldg(o + 1), a2 = __ldg(o + 2), a3 = __ldg(o + 3);
    const float4 b0 = __ldg(o + 4), b1 = __ldg(o + 5), b2 = __ldg(o + 6), b3 = __ldg(o + 7);
    dl = obb_dist(a0, a1, a2, a3, qf, 2.f * mbox);
    dr = obb_dist(b0, b1, b2, b3, qf, 2.f * mbox);
    l = __float_as_int(a3.w);
    r = __float_as_int(b3.w);
  } else {
    const NodeRec rec = load_node(b.node, node);
    dl = sqrtf(box_d2f(rec.lb, qf)) - mbox;
    dr = sqrtf(box_d2f(rec.rb, qf)) - mbox;
    l = rec.l;
    r = rec.r;
  }
}

// Exact FP64 evaluation of one leaf against the running best.  MODE 0: closest point (squared
// distance, strict improvement); MODE 1: PointDistanceEP from the current best as the upper bound.
template <int MODE>
__device__ __forceinline__ void eval_exact(const BvhDev &b, int32_t leaf, const double q[3], double &best, int32_t &bf,
                                           double bc[3]) {
  const int32_t f = b.leaf_face[leaf];
  double P[3][3];
  face_pts(b, f, P);
  if (MODE == 0) {
    double c[3];
    closest_pt_tri(q, P[0], P[1], P[2], c);
    double e[3];
    nsub3(q, c, e);
    const double cand = ndot(e, e);
    if (cand < best) { best = cand; bf = f; bc[0] = c[0]; bc[1] = c[1]; bc[2] = c[2]; }
  } else {
    EPFace fe;
    ep_setup(P, fe);
    point_distance_ep(fe, q, best);
  }
}

template <int MODE>
__device__ __forceinline__ float dist_bound(double x) {
  if (isinf(x)) return INFINITY;
  return MODE == 0 ? __double2float_ru(sqrt(x)) : __double2float_ru(x);
}

// Deferred exact evaluation.  The traversal keeps `ub`, an FP32 upper bound of the minimum
// (the smallest leaf `hi` seen, or the exact best rounded up), prunes on it, and records the
// leaves whose `lo` is within it in visiting order.  At the end only the recorded leaves whose
// `lo` is still within the final `ub` are evaluated in FP64, in the same order, with the same
// strict-improvement rule: every leaf left out has an exact distance above the minimum, so the
// result (distance, and face and point for MODE 0) is the one evaluating every visited leaf in
// FP64 gives.  A full list is first compacted, then evaluated and emptied.
constexpr int kCand = 8;

template <int MODE>
__device__ __forceinline__ void flush_cands(const BvhDev &b, const double q[3], int32_t *cl, float *cb, int &nc, float &ub,
                                            double &best, int32_t &bf, double bc[3]) {
  for (int k = 0; k < nc; k++)
    if (cb[k] <= ub) eval_exact<MODE>(b, cl[k], q, best, bf, bc);
  nc = 0;
  ub = fminf(ub, dist_bound<MODE>(best));
}

template <int MODE>
__device__ __forceinline__ void add_cand(const BvhDev &b, const double q[3], int32_t leaf, float lo, int32_t *cl, float *cb,
                                         int &nc, float &ub, double &best, int32_t &bf, double bc[3]) {
  if (nc == kCand) {
    int w = 0;
    for (int k = 0; k < nc; k++)
      if (cb[k] <= ub) { cl[w] = cl[k]; cb[w] = cb[k]; w++; }
    nc = w;
    if (nc == kCand) flush_cands<MODE>(b, q, cl, cb, nc, ub, best, bf, bc);
  }
  cl[nc] = leaf;
  cb[nc] = lo;
  nc++;
}

// Per-thread depth-first traversal with at most `budget` pops.  Returns 0 when done, 1 on stack
// overflow (result may be incomplete), 2 when the budget ran out (best is a valid upper bound).
template <int MODE, bool OB>
__device__ int thread_traverse(const BvhDev &b, const double q[3], double &best, int32_t &bf, double bc[3],
                               int budget) {
  const int n = b.n;
  const float qf[3] = {float(q[0]), float(q[1]), float(q[2])};
  const float mbox = 1e-6f * (1.f + fabsf(qf[0]) + fabsf(qf[1]) + fabsf(qf[2]));
  float ub = dist_bound<MODE>(best);
  if (n == 1) {
    eval_exact<MODE>(b, 0, q, best, bf, bc);
    return 0;
  }
  int32_t cl[kCand];
  float cb[kCand];
  int nc = 0;
  int32_t sn[kStack];
  float sd[kStack];
  int sp = 0, pops = 0;
  bool ok = true;
  sn[sp] = 0; sd[sp] = 0.f; sp++;
  while (sp > 0) {
    if (pops >= budget) {
      flush_cands<MODE>(b, q, cl, cb, nc, ub, best, bf, bc);
      return 2;
    }
    --sp;
    const int32_t node = sn[sp];
    const float d = sd[sp];
    pops++;
    if (d > ub) continue;
    if (node < 0) {
      const int32_t leaf = ~node;
      if (leaf >= n) { ok = false; continue; }
      float lo, hi;
      leaf_bounds<MODE>(b.leafd, leaf, qf, d, lo, hi);
      if (lo > ub) continue;
      ub = fminf(ub, hi);
      add_cand<MODE>(b, q, leaf, lo, cl, cb, nc, ub, best, bf, bc);
      continue;
    }
    if (node >= n - 1) { ok = false; continue; }
    int32_t cl_, cr_;
    float dl, dr;
    node_children<OB>(b, node, qf, mbox, cl_, cr_, dl, dr);
    if (cl_ >= n - 1 || cr_ >= n - 1 || ~cl_ >= n || ~cr_ >= n) { ok = false; continue; }
    const bool lnear = dl <= dr;
    const int32_t nearc = lnear ? cl_ : cr_, farc = lnear ? cr_ : cl_;
    const float dn = lnear ? dl : dr, df = lnear ? dr : dl;
    if (df <= ub) { if (sp < kStack) { sn[sp] = farc; sd[sp] = df; sp++; } else ok = false; }
    if (dn <= ub) { if (sp < kStack) { sn[sp] = nearc; sd[sp] = dn; sp++; } else ok = false; }
  }
  flush_cands<MODE>(b, q, cl, cb, nc, ub, best, bf, bc);
  return ok ? 0 : 1;
}

// ---- candidate collection (batched exact evaluation) ----
// The traversals below run in FP32 only: they prune on ub and record the leaves with lo <= ub
// in visiting order.  The exact FP64 values are computed afterwards by one dense pass over all
// queries' candidates (k_cand_eval) and reduced per query in recorded order (the *_finish
// kernels), which gives the sequential search's result: every leaf left out has an exact
// distance above the minimum.  A query with more candidates than it may record goes to the
// exact per-thread search above (the *_fallback kernels).
constexpr int kQCand = 16;     // candidates a per-thread query may hold
// The warp pass runs one query per group of kGroup lanes (two per warp): its frontiers are
// mostly narrower than a warp, so half-warp groups keep more lanes busy and twice the queries in
// flight per SM for the same shared memory.
constexpr int kGroup = 16;
constexpr int kGroupsPerBlock = 128 / kGroup;
constexpr int kWarpStack = 256;  // frontier entries a group may hold (overflow: exact fallback)
constexpr int kWarpCand = 64;  // candidates a warp-pass query may hold

__device__ __forceinline__ int warp_excl_scan(int v, int &total) {
  const int lane = threadIdx.x & 31;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

// Pruning bound from the leaf that won this query's previous search: its FP32 upper bound at q.
// Any leaf's upper bound bounds the minimum, so a seed never changes which leaves can attain the
// minimum nor their traversal order (hence not the winner); a stale seed only prunes less, and
// one outside the tree (an earlier target) is ignored.
template <int MODE>
__device__ __forceinline__ void seed_bound(const BvhDev &b, const int32_t *seed, int64_t i, const double q[3],
                                           float &ub) {
  if (!seed || b.n < 2) return;
  const int32_t s = seed[i];
  if (s < 0 || s >= b.n) return;
  const float qf[3] = {float(q[0]), float(q[1]), float(q[2])};
  float lo, hi;
  leaf_bounds<MODE>(b.leafd, s, qf, 0.f, lo, hi);
  ub = fminf(ub, hi);
}

// Per-thread collection with at most `budget` pops.  The stack is the thread's column of a
// block-shared array (entry k at sn[k * kBlockThreads]), kTStack entries deep: the per-pop pushes
// and pops stay in shared memory instead of local memory.  Returns 0 when done, 1 on stack
// overflow (candidates may miss subtrees), 2 when the budget ran out (ub stays a valid bound), 3
// when more than kQCand candidates remain after compaction; ub stays a valid bound in every case.
constexpr int kTStack = 32;
constexpr int kBlockThreads = 128;
template <int MODE, bool OB>
__device__ int thread_collect(const BvhDev &b, const double q[3], float &ub, int32_t *cl, float *cb, int &nc,
                              int budget, int32_t *sn, float *sd) {
  const int n = b.n;
  nc = 0;
  if (n == 1) {
    cl[0] = 0;
    cb[0] = -INFINITY;
    nc = 1;
    return 0;
  }
  const float qf[3] = {float(q[0]), float(q[1]), float(q[2])};
  const float mbox = 1e-6f * (1.f + fabsf(qf[0]) + fabsf(qf[1]) + fabsf(qf[2]));
  constexpr int S = kBlockThreads;
  int sp = 0, pops = 0;
  bool ok = true;
  sn[0] = 0; sd[0] = 0.f; sp++;
  while (sp > 0) {
    if (pops >= budget) return 2;
    --sp;
    const int32_t node = sn[sp * S];
    const float d = sd[sp * S];
    pops++;
    if (d > ub) continue;
    if (node < 0) {
      const int32_t leaf = ~node;
      if (leaf >= n) { ok = false; continue; }
      float lo, hi;
      leaf_bounds<MODE>(b.leafd, leaf, qf, d, lo, hi);
      if (lo > ub) continue;
      ub = fminf(ub, hi);
      if (nc == kQCand) {
        int w = 0;
        for (int k = 0; k < nc; k++)
          if (cb[k] <= ub) { cl[w] = cl[k]; cb[w] = cb[k]; w++; }
        nc = w;
        if (nc == kQCand) return 3;
      }
      cl[nc] = leaf;
      cb[nc] = lo;
      nc++;
      continue;
    }
    if (node >= n - 1) { ok = false; continue; }
    int32_t cl_, cr_;
    float dl, dr;
    node_children<OB>(b, node, qf, mbox, cl_, cr_, dl, dr);
    if (cl_ >= n - 1 || cr_ >= n - 1 || ~cl_ >= n || ~cr_ >= n) { ok = false; continue; }
    const bool lnear = dl <= dr;
    const int32_t nearc = lnear ? cl_ : cr_, farc = lnear ? cr_ : cl_;
    const float dn = lnear ? dl : dr, df = lnear ? dr : dl;
    if (df <= ub) { if (sp < kTStack) { sn[sp * S] = farc; sd[sp * S] = df; sp++; } else return 1; }
    if (dn <= ub) { if (sp < kTStack) { sn[sp * S] = nearc; sd[sp * S] = dn; sp++; } else return 1; }
  }
  return ok ? 0 : 1;
}

// Lanes of this thread's group: the mask, the lane within the group and the group's shift.
__device__ __forceinline__ unsigned group_shift() { return kGroup == 32 ? 0u : (threadIdx.x & 16u); }
__device__ __forceinline__ unsigned group_mask() {
  return kGroup == 32 ? 0xffffffffu : (0xffffu << group_shift());
}
__device__ __forceinline__ int group_lane() { return threadIdx.x & (kGroup - 1); }
__device__ __forceinline__ unsigned group_ballot(bool pred) {
  return (__ballot_sync(group_mask(), pred) & group_mask()) >> group_shift();
}
// Exclusive prefix sum over the group (all its lanes must call it); total = sum.
__device__ __forceinline__ int group_excl_scan(int v, int &total) {
  const unsigned gm = group_mask();
  const int gl = group_lane();
  int x = v;
#pragma unroll
  for (int o = 1; o < kGroup; o <<= 1) {
    const int y = __shfl_up_sync(gm, x, o, kGroup);
    if (gl >= o) x += y;
  }
  total = __shfl_sync(gm, x, kGroup - 1, kGroup);
  return x - v;
}

// In-order compaction of a group's shared candidate list to the entries with lo <= ub.
__device__ __forceinline__ int group_compact(int32_t *cl, float *cb, int nc, float ub) {
  const unsigned gm = group_mask();
  const int gl = group_lane();
  int w = 0;
  for (int k0 = 0; k0 < nc; k0 += kGroup) {
    const int k = k0 + gl;
    const bool keep = k < nc && cb[k] <= ub;
    const unsigned kb = group_ballot(keep);
    const int32_t lk = keep ? cl[k] : 0;
    const float bk = keep ? cb[k] : 0.f;
    __syncwarp(gm);
    if (keep) {
      const int pos = w + __popc(kb & ((1u << gl) - 1u));
      cl[pos] = lk;
      cb[pos] = bk;
    }
    w += __popc(kb);
    __syncwarp(gm);
  }
  return w;
}

// Group-cooperative collection for the queries left over by the per-thread pass: one query per
// group of kGroup lanes, up to kGroup frontier entries per step (one per lane), LIFO frontier
// and candidate list in shared memory, ub shared by the group.  Every collective names only
// the group's lanes, so the two groups of a warp may run different numbers of steps.  Returns
// 0 when done (cl/cb compacted to lo <= ub), 1 on frontier overflow or a malformed tree,
// 3 when more than kWarpCand candidates remain after compaction.
template <int MODE, bool OB>
__device__ int group_collect(const BvhDev &b, const double q[3], int32_t *sn, float *sd, int32_t *cl, float *cb,
                             float &ub, int &nc) {
  const unsigned gm = group_mask();
  const int gl = group_lane();
  const int n = b.n;
  const float qf[3] = {float(q[0]), float(q[1]), float(q[2])};
  const float mbox = 1e-6f * (1.f + fabsf(qf[0]) + fabsf(qf[1]) + fabsf(qf[2]));
  bool ok = true, full = false;
  int sz = 1;
  nc = 0;
  if (gl == 0) { sn[0] = n == 1 ? ~0 : 0; sd[0] = -INFINITY; }
  __syncwarp(gm);
  for (int guard = 0; sz > 0 && !full && guard < 4 * (2 * n + 64); guard++) {
    const int take = sz < kGroup ? sz : kGroup;
    const bool has = gl < take;
    const int32_t node = has ? sn[sz - take + gl] : 0;
    const float d = has ? sd[sz - take + gl] : INFINITY;
    __syncwarp(gm);
    sz -= take;
    int32_t push[2];
    float pd[2];
    int np = 0;
    bool cand = false;
    float lo = INFINITY, hi = INFINITY;
    if (has && d <= ub) {
      if (node < 0) {
        const int32_t leaf = ~node;
        if (leaf < n) {
          if (n == 1) { lo = -INFINITY; hi = INFINITY; }
          else leaf_bounds<MODE>(b.leafd, leaf, qf, d, lo, hi);
          cand = true;
        } else {
          ok = false;
        }
      } else if (node < n - 1) {
        int32_t cl_, cr_;
        float dl, dr;
        node_children<OB>(b, node, qf, mbox, cl_, cr_, dl, dr);
        if (cl_ >= n - 1 || cr_ >= n - 1 || ~cl_ >= n || ~cr_ >= n) {
          ok = false;
        } else {
          const bool lnear = dl <= dr;
          const float dn = lnear ? dl : dr, df = lnear ? dr : dl;
          if (df <= ub) { push[np] = lnear ? cr_ : cl_; pd[np] = df; np++; }
          if (dn <= ub) { push[np] = lnear ? cl_ : cr_; pd[np] = dn; np++; }
        }
      } else {
        ok = false;
      }
    }
    // tighten ub by this step's leaves, then record those still within it
    float hm = hi;
#pragma unroll
    for (int o = kGroup / 2; o > 0; o >>= 1) hm = fminf(hm, __shfl_xor_sync(gm, hm, o, kGroup));
    ub = fminf(ub, hm);
    const bool rec = cand && lo <= ub;
    const unsigned rb = group_ballot(rec);
    const int nrec = __popc(rb);
    if (nrec > 0) {
      if (nc + nrec > kWarpCand) {
        nc = group_compact(cl, cb, nc, ub);
        if (nc + nrec > kWarpCand) full = true;
      }
      if (!full) {
        if (rec) {
          const int pos = nc + __popc(rb & ((1u << gl) - 1u));
          cl[pos] = ~node;
          cb[pos] = lo;
        }
        nc += nrec;
      }
    }
    int total;
    const int off = group_excl_scan(np, total);
    const int room = kWarpStack - sz;
    for (int k = 0; k < np; k++)
      if (off + k < room) { sn[sz + off + k] = push[k]; sd[sz + off + k] = pd[k]; }
    if (total > room) ok = false;
    __syncwarp(gm);
    sz += total < room ? total : room;
  }
  __syncwarp(gm);
  if (full) return 3;
  if (sz > 0) ok = false;
  nc = group_compact(cl, cb, nc, ub);
  return group_ballot(!ok) ? 1 : 0;
}

constexpr int kThreadBudget = 96;  // pops per query before the warp pass when the caller gives none
__device__ __forceinline__ unsigned groups_total() { return gridDim.x * (blockDim.x / kGroup); }
__device__ __forceinline__ unsigned group_global() { return blockIdx.x * (blockDim.x / kGroup) + threadIdx.x / kGroup; }

__device__ __forceinline__ void push_overflow(const Overflow &o, int64_t item, int32_t mesh) {
  const unsigned k = atomicAdd(o.count, 1u);
  o.item[k] = item;
  o.mesh[k] = mesh;
}

__device__ __forceinline__ void push_fallback(const CandBuf &c, int64_t item, int32_t mesh) {
  const unsigned k = atomicAdd(c.fb_count, 1u);
  c.fb_item[k] = item;
  c.fb_mesh[k] = mesh;
  c.q_cnt[item] = -1;
}

__device__ __forceinline__ void store_query(const CandBuf &c, int64_t i, int32_t mesh, const double q[3], int64_t off,
                                            int cnt) {
  c.q_off[i] = (int32_t)off;
  c.q_cnt[i] = cnt;
  c.qpos[3 * i] = q[0]; c.qpos[3 * i + 1] = q[1]; c.qpos[3 * i + 2] = q[2];
  c.q_mesh[i] = mesh;
}

// Per-thread pass: every lane of the warp calls this (has = false for lanes without candidates
// to store); one atomic per warp reserves the warp's entries.  Returns false for a lane whose
// entries do not fit (the caller sends that query to the fallback).
__device__ bool store_cands_warp(const CandBuf &c, bool has, int64_t i, int32_t mesh, const double q[3],
                                 const int32_t *cl, const float *cb, int nc, float ub) {
  int k = 0;
  if (has)
    for (int j = 0; j < nc; j++) k += cb[j] <= ub;
  int total;
  const int off = warp_excl_scan(k, total);
  unsigned base = 0;
  if ((threadIdx.x & 31) == 0 && total > 0) base = atomicAdd(c.count, (unsigned)total);
  base = __shfl_sync(0xffffffffu, base, 0);
  if (!has) return true;
  const int64_t o = (int64_t)base + off;
  if (o + k > c.cap) return false;
  int w = 0;
  for (int j = 0; j < nc; j++)
    if (cb[j] <= ub) { c.leaf[o + w] = cl[j]; c.qi[o + w] = (int32_t)i; w++; }
  store_query(c, i, mesh, q, o, k);
  return true;
}

// Warp pass: one query per group, candidates already compacted in shared memory.
__device__ bool store_cands_query(const CandBuf &c, int64_t i, int32_t mesh, const double q[3], const int32_t *cl,
                                  int nc) {
  const int gl = group_lane();
  unsigned base = 0;
  if (gl == 0 && nc > 0) base = atomicAdd(c.count, (unsigned)nc);
  base = __shfl_sync(group_mask(), base, 0, kGroup);
  if ((int64_t)base + nc > c.cap) return false;
  for (int j = gl; j < nc; j += kGroup) { c.leaf[base + j] = cl[j]; c.qi[base + j] = (int32_t)i; }
  if (gl == 0) store_query(c, i, mesh, q, base, nc);
  return true;
}

// The dense exact pass: one candidate per thread.  MODE 0: squared point-triangle distance;
// MODE 1: PointDistanceEP without a bound, and the plane distance the bound test reads.
// SRC 0: the BVH of mesh m is tgt[m].bvh; SRC 1: surf[m].
template <int MODE, int SRC>
__global__ void __launch_bounds__(128) k_cand_eval(CandBuf c, const TargetDev *tgt, const BvhDev *surf) {
  const unsigned cnt = *c.count;
  const int64_t n = cnt < c.cap ? (int64_t)cnt : c.cap;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t qi = c.qi[e];
    const int32_t m = c.q_mesh[qi];
    const BvhDev &b = SRC == 0 ? tgt[m].bvh : surf[m];
    const double q[3] = {c.qpos[3 * (int64_t)qi], c.qpos[3 * (int64_t)qi + 1], c.qpos[3 * (int64_t)qi + 2]};
    double P[3][3];
    face_pts(b, b.leaf_face[c.leaf[e]], P);
    if (MODE == 0) {
      double cp[3], r[3];
      closest_pt_tri(q, P[0], P[1], P[2], cp);
      nsub3(q, cp, r);
      c.x[e] = ndot(r, r);
    } else {
      EPFace fe;
      if (SRC == 0 && tgt[m].EP) ep_load(tgt[m].EP + 16 * (int64_t)b.leaf_face[c.leaf[e]], P, fe);
      else ep_setup(P, fe);
      double x = INFINITY;
      point_distance_ep(fe, q, x);
      c.x[e] = x;
      c.d[e] = nsub(ndot(fe.dir, q), fe.off);
    }
  }
}

// pseudonormal_test: normal at the closest point c of face f (vertex / edge / face normal).
__device__ void pseudonormal(const TargetDev &t, int32_t f, const double c[3], double n[3]) {
  double A[3], B[3], C[3];
#pragma unroll
  for (int d = 0; d < 3; d++) { A[d] = t.tri[(int64_t)f * 9 + d]; B[d] = t.tri[(int64_t)f * 9 + 3 + d]; C[d] = t.tri[(int64_t)f * 9 + 6 + d]; }
  double e1[3], e2[3], x[3];
  nsub3(B, A, e1);
  nsub3(C, A, e2);
  ncross(e1, e2, x);
  const double area = sqrt(ndot(x, x));  // doublearea
  const double epsilon = 1e-12;
  int kind = 0, which = 0;  // 0 face, 1 vertex (which corner), 2 edge (opposite which corner)
  if (area > 1e-4) {
    double v2[3];
    nsub3(c, A, v2);
    const double d00 = ndot(e1, e1), d01 = ndot(e1, e2), d11 = ndot(e2, e2), d20 = ndot(v2, e1), d21 = ndot(v2, e2);
    const double den = nsub(nmul(d00, d11), nmul(d01, d01));
    double bb[3];
    bb[1] = nsub(nmul(d11, d20), nmul(d01, d21)) / den;
    bb[2] = nsub(nmul(d00, d21), nmul(d01, d20)) / den;
    bb[0] = nsub(1.0, nadd(bb[1], bb[2]));
    const int type = (bb[0] <= epsilon) + (bb[1] <= epsilon) + (bb[2] <= epsilon);
    if (type == 2) {
      kind = 1;
      which = bb[0] > epsilon ? 0 : (bb[1] > epsilon ? 1 : 2);
    } else if (type == 1) {
      kind = 2;
      which = bb[0] <= epsilon ? 0 : (bb[1] <= epsilon ? 1 : 2);
    }
  } else {
    const double *P[3] = {A, B, C};
    bool found = false;
    for (int v = 0; v < 3 && !found; v++) {
      double dv[3];
      nsub3(c, P[v], dv);
      if (sqrt(ndot(dv, dv)) < epsilon) { found = true; kind = 1; which = v; }
    }
    for (int e = 0; e < 3 && !found; e++) {
      const double *sp = P[(e + 1) % 3], *dp = P[(e + 2) % 3];
      double dms[3], smp[3];
      nsub3(dp, sp, dms);
      nsub3(sp, c, smp);
      const double vl = ndot(dms, dms);
      const double tt = -ndot(dms, smp) / vl;
      double z[3];
      if (tt < 0) {
        nsub3(c, sp, z);
      } else if (tt > 1) {
        nsub3(c, dp, z);
      } else {
        const double pr[3] = {nadd(nmul(nsub(1.0, tt), sp[0]), nmul(tt, dp[0])),
                              nadd(nmul(nsub(1.0, tt), sp[1]), nmul(tt, dp[1])),
                              nadd(nmul(nsub(1.0, tt), sp[2]), nmul(tt, dp[2]))};
        nsub3(c, pr, z);
      }
      if (sqrt(ndot(z, z)) < epsilon) { found = true; kind = 2; which = e; }
    }
  }
  const double *src = kind == 0 ? t.FN + 3 * (int64_t)f : kind == 1 ? t.VNc + 9 * (int64_t)f + 3 * which : t.ENc + 9 * (int64_t)f + 3 * which;
  n[0] = src[0]; n[1] = src[1]; n[2] = src[2];
}

// Tangent planes of the regular boundary vertices (dirty_graph_projection, :4031-4078):
// normal_T = pseudonormal, dis_T = normal_T . closest point.
__device__ __forceinline__ void write_tangent(const ProjArgs &p, const TargetDev &t, int64_t e, int32_t f,
                                              const double c[3]) {
  double n[3] = {0, 0, 0};
  if (f >= 0) pseudonormal(t, f, c, n);
  p.t_nrm[3 * e] = n[0]; p.t_nrm[3 * e + 1] = n[1]; p.t_nrm[3 * e + 2] = n[2];
  p.t_dis[e] = n[0] * c[0] + n[1] * c[1] + n[2] * c[2];
}

// The projection query of item i: tangent entry e and the vertex position.
__device__ __forceinline__ int64_t proj_entry(const ProjArgs &p, const MeshDesc &md, int64_t i, double q[3]) {
  const int64_t e = md.t_off + (i - md.kitem0[K_PROJ]);
  const int64_t v = md.v_off + p.t_ids[e];
  q[0] = p.X[4 * v]; q[1] = p.X[4 * v + 1]; q[2] = p.X[4 * v + 2];
  return e;
}

__global__ void __launch_bounds__(kBlockThreads) k_project(ProjArgs p) {
  __shared__ int32_t s_sn[kTStack][kBlockThreads];
  __shared__ float s_sd[kTStack][kBlockThreads];
  const Seg sg = p.seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  bool has = i < sg.end;
  double q[3] = {0, 0, 0};
  int32_t cl[kQCand];
  float cb[kQCand];
  int nc = 0;
  float ub = INFINITY;
  if (has) {
    const MeshDesc md = p.mesh[sg.mesh];
    const TargetDev &t = p.tgt[sg.mesh];
    proj_entry(p, md, i, q);
    int st = 0;
    seed_bound<0>(t.bvh, p.seed, i, q, ub);
    if (t.bvh.n > 0)
      st = thread_collect<0, true>(t.bvh, q, ub, cl, cb, nc, p.budget > 0 ? p.budget : kThreadBudget, &s_sn[0][threadIdx.x],
                             &s_sd[0][threadIdx.x]);
    if (st != 0) {
      // over budget, stack or candidate list: the cooperative pass restarts the query from the
      // root under the bound found so far (any leaf's upper bound bounds the minimum)
      p.ovf.best[i] = ub;
      push_overflow(p.ovf, i, sg.mesh);
      has = false;
    }
  }
  if (!store_cands_warp(p.cand, has, i, sg.mesh, q, cl, cb, nc, ub)) push_fallback(p.cand, i, sg.mesh);
}

__global__ void __launch_bounds__(128, 8) k_project_warp(ProjArgs p) {
  __shared__ int32_t sn[kGroupsPerBlock][kWarpStack];
  __shared__ float sd[kGroupsPerBlock][kWarpStack];
  __shared__ int32_t scl[kGroupsPerBlock][kWarpCand];
  __shared__ float scb[kGroupsPerBlock][kWarpCand];
  const int g = threadIdx.x / kGroup, gl = group_lane();
  const unsigned cnt = *p.ovf.count;
  for (unsigned k = group_global(); k < cnt; k += groups_total()) {
    const int64_t i = p.ovf.item[k];
    const int32_t m = p.ovf.mesh[k];
    const MeshDesc md = p.mesh[m];
    double q[3];
    proj_entry(p, md, i, q);
    float ub = (float)p.ovf.best[i];
    int nc = 0;
    const int st = group_collect<0, true>(p.tgt[m].bvh, q, sn[g], sd[g], scl[g], scb[g], ub, nc);
    if (st != 0) {  // frontier or candidate overflow: the exact per-thread search
      if (gl == 0) push_fallback(p.cand, i, m);
    } else if (!store_cands_query(p.cand, i, m, q, scl[g], nc) && gl == 0) {
      push_fallback(p.cand, i, m);
    }
    __syncwarp(group_mask());
  }
}

// Winner of each projection query in recorded order (strict improvement), its closest point and
// pseudonormal -> tangent plane.
__global__ void __launch_bounds__(128) k_project_finish(ProjArgs p) {
  const Seg sg = p.seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const int cnt = p.cand.q_cnt[i];
  if (cnt < 0) return;
  const MeshDesc md = p.mesh[sg.mesh];
  const TargetDev &t = p.tgt[sg.mesh];
  double q[3];
  const int64_t e = proj_entry(p, md, i, q);
  const int64_t o = p.cand.q_off[i];
  double best = INFINITY;
  int win = -1;
  for (int k = 0; k < cnt; k++) {
    const double x = p.cand.x[o + k];
    if (x < best) { best = x; win = k; }
  }
  int32_t f = -1;
  double c[3] = {0, 0, 0};
  if (win >= 0) {
    if (p.seed) p.seed[i] = p.cand.leaf[o + win];
    f = t.bvh.leaf_face[p.cand.leaf[o + win]];
    double P[3][3];
    face_pts(t.bvh, f, P);
    closest_pt_tri(q, P[0], P[1], P[2], c);
  }
  write_tangent(p, t, e, f, c);
}

// Queries whose candidates did not fit: the exact per-thread search (deferred in-thread
// evaluation), one thread per query.
__global__ void __launch_bounds__(128) k_project_fallback(ProjArgs p) {
  const unsigned cnt = *p.cand.fb_count;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
    const int64_t i = p.cand.fb_item[k];
    const int32_t m = p.cand.fb_mesh[k];
    const MeshDesc md = p.mesh[m];
    const TargetDev &t = p.tgt[m];
    double q[3];
    const int64_t e = proj_entry(p, md, i, q);
    double best = INFINITY, c[3] = {0, 0, 0};
    int32_t f = -1;
    if (t.bvh.n > 0 && thread_traverse<0, true>(t.bvh, q, best, f, c, 1 << 30) != 0) atomicOr(&p.sc[m].status, 8);
    write_tangent(p, t, e, f, c);
  }
}

// signed_distance_pseudonormal for arbitrary query points (rows) against mesh m's target
__global__ void __launch_bounds__(128) k_signed_distance(TargetDev t, int64_t np, const double *P, double *S,
                                                         int32_t *I, double *C, double *N, int *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double q[3] = {P[3 * i], P[3 * i + 1], P[3 * i + 2]};
  double best = INFINITY, c[3] = {0, 0, 0}, n[3] = {0, 0, 0};
  int32_t f = -1;
  if (t.bvh.n > 0 && thread_traverse<0, true>(t.bvh, q, best, f, c, 1 << 30) != 0) atomicOr(status, 8);
  double s = 1;
  if (f >= 0) {
    pseudonormal(t, f, c, n);
    double qc[3];
    nsub3(q, c, qc);
    s = ndot(qc, n) >= 0 ? 1. : -1.;
  }
  S[i] = s * sqrt(best);
  I[i] = f;
  C[3 * i] = c[0]; C[3 * i + 1] = c[1]; C[3 * i + 2] = c[2];
  N[3 * i] = n[0]; N[3 * i + 1] = n[1]; N[3 * i + 2] = n[2];
}

// Feature lines (dirty_graph_projection LINE branch, :3963-4025): nearest curve segment by
// point_line_projection (global_functions.cpp:3454-3465), ties to the lower segment index.
__global__ void __launch_bounds__(128) k_curve_project(ProjArgs p) {
  const Seg sg = p.seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = p.mesh[sg.mesh];
  const TargetDev &t = p.tgt[sg.mesh];
  const int64_t e = md.l_off + (i - md.kitem0[K_LINE]);
  const int64_t v = md.v_off + p.l_ids[e];
  const double q[3] = {p.X[4 * v], p.X[4 * v + 1], p.X[4 * v + 2]};
  const int32_t cu = p.l_curve[e];
  const int64_t c0 = t.curve_ptr[cu], c1 = t.curve_ptr[cu + 1];
  const int64_t size = c1 - c0;
  const int64_t len = t.curve_closed[cu] ? size : size - 1;
  double best = INFINITY, pv[3] = {0, 0, 0}, tg[3] = {1, 0, 0};
  for (int64_t j = 0; j < len; j++) {
    const double *a = t.TV + 3 * (int64_t)t.curve_vs[c0 + j];
    const double *b = t.TV + 3 * (int64_t)t.curve_vs[c0 + (j + 1) % size];
    const double vv1[3] = {q[0] - a[0], q[1] - a[1], q[2] - a[2]}, v21[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double n2 = v21[0] * v21[0] + v21[1] * v21[1] + v21[2] * v21[2];
    const double tt = n2 >= 1.e-7 ? (vv1[0] * v21[0] + vv1[1] * v21[1] + vv1[2] * v21[2]) / n2 : 0.0;
    double pp[3];
    if (tt >= 0.0 && tt <= 1.0) { pp[0] = a[0] + tt * v21[0]; pp[1] = a[1] + tt * v21[1]; pp[2] = a[2] + tt * v21[2]; }
    else if (tt < 0.0) { pp[0] = a[0]; pp[1] = a[1]; pp[2] = a[2]; }
    else { pp[0] = b[0]; pp[1] = b[1]; pp[2] = b[2]; }
    const double dx = q[0] - pp[0], dy = q[1] - pp[1], dz = q[2] - pp[2];
    const double dist = sqrt(dx * dx + dy * dy + dz * dz);
    if (dist < best) {
      best = dist;
      pv[0] = pp[0]; pv[1] = pp[1]; pv[2] = pp[2];
      const double ln = sqrt(n2);
      tg[0] = v21[0] / ln; tg[1] = v21[1] / ln; tg[2] = v21[2] / ln;
    }
  }
  if (len <= 0 && size > 0) {  // single-vertex curve: nearest curve vertex
    const double *a = t.TV + 3 * (int64_t)t.curve_vs[c0];
    pv[0] = a[0]; pv[1] = a[1]; pv[2] = a[2];
    tg[0] = 1; tg[1] = 0; tg[2] = 0;
  }
  p.l_orig[3 * e] = pv[0]; p.l_orig[3 * e + 1] = pv[1]; p.l_orig[3 * e + 2] = pv[2];
  p.l_axis[3 * e] = tg[0]; p.l_axis[3 * e + 1] = tg[1]; p.l_axis[3 * e + 2] = tg[2];
}

// ------------------------------------------------------------------------------- Hausdorff
// bbox of the referenced surface vertices at the current positions (per mesh), combined with the
// static target bbox -> inflated diagonal (the distance upper bound).
__global__ void __launch_bounds__(256) k_haus_bbox(HausArgs h) {
  const Seg sg = h.seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  const MeshDesc md = h.mesh[sg.mesh];
  double lo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {INFINITY, INFINITY, INFINITY};
  if (i < sg.end) {
    const int64_t v = h.surf_vs[i];
#pragma unroll
    for (int d = 0; d < 3; d++) { lo[d] = h.X[4 * v + d]; nhi[d] = -h.X[4 * v + d]; }
  }
  __shared__ double smem[6][32];
  double m[6] = {lo[0], lo[1], lo[2], nhi[0], nhi[1], nhi[2]};
  block_min<6>(m, smem);
  if (publish_partials<6>(m, h.partials, blockIdx.x, h.counters + sg.mesh, md.knblk[K_SURFV])) {
    double r[6];
    for (int k = 0; k < 6; k++) r[k] = gather_partials_min(h.partials, md.kblk0[K_SURFV], md.knblk[K_SURFV], 6, k, smem);
    if (threadIdx.x == 0) {
      HausMesh &hm = h.hm[sg.mesh];
      double L[3], Hh[3];
      for (int d = 0; d < 3; d++) {
        L[d] = fmin(r[d], hm.tgt_lo[d]);
        Hh[d] = fmax(-r[3 + d], hm.tgt_hi[d]);
      }
      const double e0 = Hh[0] - L[0], e1 = Hh[1] - L[1], e2 = Hh[2] - L[2];
      const double off = sqrt(e0 * e0 + e1 * e1 + e2 * e2) * 0.02;
      const double f0 = e0 + 2 * off, f1 = e1 + 2 * off, f2 = e2 + 2 * off;
      hm.diag = sqrt(f0 * f0 + f1 * f1 + f2 * f2);
      h.counters[sg.mesh] = 0;
    }
  }
}

// One side of the vertex-sampled Hausdorff: SIDE 0 = target vertices vs surface faces,
// SIDE 1 = surface vertices vs target faces.  Per-sample distance into h.dist (left at the upper
// bound when no face is closer), finished by the warp pass for samples over budget, then reduced.
template <int SIDE>
__device__ __forceinline__ void haus_query(const HausArgs &h, int64_t i, int32_t m, double q[3], const BvhDev *&b) {
  if (SIDE == 0) {
    const int64_t v = h.tgt_vs[i];
    const TargetDev &t = h.tgt[m];
    q[0] = t.TV[3 * v]; q[1] = t.TV[3 * v + 1]; q[2] = t.TV[3 * v + 2];
    b = &h.surf[m];
  } else {
    const int64_t v = h.surf_vs[i];
    q[0] = h.X[4 * v]; q[1] = h.X[4 * v + 1]; q[2] = h.X[4 * v + 2];
    b = &h.tgt[m].bvh;
  }
}

template <int SIDE>
__global__ void __launch_bounds__(kBlockThreads) k_haus_side(HausArgs h) {
  __shared__ int32_t s_sn[kTStack][kBlockThreads];
  __shared__ float s_sd[kTStack][kBlockThreads];
  const Seg sg = h.seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  bool has = i < sg.end;
  double q[3] = {0, 0, 0};
  int32_t cl[kQCand];
  float cb[kQCand];
  int nc = 0;
  float ub = INFINITY;
  if (has) {
    const BvhDev *b;
    haus_query<SIDE>(h, i, sg.mesh, q, b);
    ub = dist_bound<1>(h.hm[sg.mesh].diag);
    seed_bound<1>(*b, h.seed, i, q, ub);
    int st = 0;
    if (b->n > 0)
      st = thread_collect<1, SIDE == 1>(*b, q, ub, cl, cb, nc, h.budget > 0 ? h.budget : kThreadBudget, &s_sn[0][threadIdx.x],
                             &s_sd[0][threadIdx.x]);
    if (st != 0) {
      // over budget, stack or candidate list: the cooperative pass restarts the query from the
      // root under the bound found so far (any leaf's upper bound bounds the minimum)
      h.ovf.best[i] = ub;
      push_overflow(h.ovf, i, sg.mesh);
      has = false;
    }
  }
  if (!store_cands_warp(h.cand, has, i, sg.mesh, q, cl, cb, nc, ub)) push_fallback(h.cand, i, sg.mesh);
}

template <int SIDE>
__global__ void __launch_bounds__(128, 8) k_haus_warp(HausArgs h) {
  __shared__ int32_t sn[kGroupsPerBlock][kWarpStack];
  __shared__ float sd[kGroupsPerBlock][kWarpStack];
  __shared__ int32_t scl[kGroupsPerBlock][kWarpCand];
  __shared__ float scb[kGroupsPerBlock][kWarpCand];
  const int g = threadIdx.x / kGroup, gl = group_lane();
  const unsigned cnt = *h.ovf.count;
  for (unsigned k = group_global(); k < cnt; k += groups_total()) {
    const int64_t i = h.ovf.item[k];
    const int32_t m = h.ovf.mesh[k];
    double q[3];
    const BvhDev *b;
    haus_query<SIDE>(h, i, m, q, b);
    float ub = (float)h.ovf.best[i];
    int nc = 0;
    const int st = group_collect<1, SIDE == 1>(*b, q, sn[g], sd[g], scl[g], scb[g], ub, nc);
    if (st != 0) {  // frontier or candidate overflow: the exact per-thread search
      if (gl == 0) push_fallback(h.cand, i, m);
    } else if (!store_cands_query(h.cand, i, m, q, scl[g], nc) && gl == 0) {
      push_fallback(h.cand, i, m);
    }
    __syncwarp(group_mask());
  }
}

// Per-sample distance from the recorded candidates: PointDistanceEP's bound test against the
// running distance (from the inflated diagonal), then the minimum -- the sequential rule, replayed
// with the plane distance of each candidate.
template <int SIDE>
__global__ void __launch_bounds__(128) k_haus_finish(HausArgs h) {
  const Seg sg = h.seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const int cnt = h.cand.q_cnt[i];
  if (cnt < 0) return;
  const int64_t o = h.cand.q_off[i];
  double dist = h.hm[sg.mesh].diag;
  int wk = -1;
  for (int k = 0; k < cnt; k++) {
    const double d = h.cand.d[o + k];
    if (d > dist || d < -dist) continue;
    const double x = h.cand.x[o + k];
    if (dist > x) { dist = x; wk = k; }
  }
  h.dist[i] = dist;
  if (wk >= 0 && h.seed) h.seed[i] = h.cand.leaf[o + wk];
}

template <int SIDE>
__global__ void __launch_bounds__(128) k_haus_fallback(HausArgs h) {
  const unsigned cnt = *h.cand.fb_count;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
    const int64_t i = h.cand.fb_item[k];
    const int32_t m = h.cand.fb_mesh[k];
    double q[3];
    const BvhDev *b;
    haus_query<SIDE>(h, i, m, q, b);
    double dist = h.hm[m].diag;
    int32_t fd = -1;
    double cd[3];
    if (b->n > 0 && thread_traverse<1, SIDE == 1>(*b, q, dist, fd, cd, 1 << 30) != 0) atomicOr(&h.sc[m].status, 8);
    h.dist[i] = dist;
  }
}

// max / mean of one side (AddSample, sampling.h:224-256: samples at the upper bound are dropped)
template <int SIDE>
__global__ void __launch_bounds__(256) k_haus_reduce(HausArgs h) {
  const Seg sg = h.seg[blockIdx.x];
  const MeshDesc md = h.mesh[sg.mesh];
  HausMesh &hm = h.hm[sg.mesh];
  const double upper = hm.diag;
  double mx[1] = {INFINITY}, acc[2] = {0, 0};
  for (int64_t i = sg.begin + threadIdx.x; i < sg.end; i += blockDim.x) {
    const double d = h.dist[i];
    if (d != upper) { mx[0] = fmin(mx[0], -d); acc[0] += d; acc[1] += 1; }
  }
  __shared__ double smem[2][32];
  block_min<1>(mx, smem);
  const double bm = mx[0];
  block_sum<2>(acc, smem);
  double out[3] = {bm, acc[0], acc[1]};
  const int kind = SIDE == 0 ? K_TGTV : K_SURFV;
  if (publish_partials<3>(out, h.partials, blockIdx.x, h.counters + sg.mesh, md.knblk[kind])) {
    double m = gather_partials_min(h.partials, md.kblk0[kind], md.knblk[kind], 3, 0, smem);
    double g[2];  // components 1 and 2 of 3
    gather_partials_sums<2>(h.partials + 1, md.kblk0[kind], md.knblk[kind], 3, g, smem);
    const double s = g[0], c = g[1];
    if (threadIdx.x == 0) {
      hm.side_max[SIDE] = -m;
      hm.side_mean[SIDE] = s / c;
      h.counters[sg.mesh] = 0;
    }
  }
}

// Per-point minimum PointDistanceEP over a tree's faces, starting from `upper`.
__global__ void __launch_bounds__(128) k_ep_points(BvhDev b, const double *P, const int64_t *ids, int64_t n,
                                                   double upper, double *dist, int *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t v = ids ? ids[i] : i;
  const double q[3] = {P[3 * v], P[3 * v + 1], P[3 * v + 2]};
  double d = upper;
  int32_t fd = -1;
  double cd[3];
  if (b.n > 0 && thread_traverse<1, false>(b, q, d, fd, cd, 1 << 30) != 0) atomicOr(status, 8);
  dist[i] = d;
}

// max / mean over the samples whose distance went below `upper` (AddSample, sampling.h:224-256)
__global__ void __launch_bounds__(1024) k_maxmean(const double *dist, int64_t n, double upper, double *out3) {
  double mx[1] = {INFINITY}, acc[2] = {0, 0};
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = dist[i];
    if (d != upper) { mx[0] = fmin(mx[0], -d); acc[0] += d; acc[1] += 1; }
  }
  __shared__ double smem[2][32];
  block_min<1>(mx, smem);
  const double m = mx[0];
  block_sum<2>(acc, smem);
  if (threadIdx.x == 0) { out3[0] = -m; out3[1] = acc[0]; out3[2] = acc[1]; }
}

// Max_dis_satisified after a Hausdorff check (stop_criterior_satisfied, :4160-4176)
// Both sides reduced (they may run concurrently): the mesh's Hausdorff max and mean.
__global__ void k_haus_combine(HausMesh *hm, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  hm[m].max_dist = fmax(hm[m].side_max[0], hm[m].side_max[1]);
  hm[m].ave_dist = fmax(hm[m].side_mean[1], hm[m].side_mean[0]);
}

__global__ void k_fa_haus_flag(MeshScalars *sc, const HausMesh *hm, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  MeshScalars &S = sc[m];
  S.haus_diag = hm[m].diag;
  S.haus_max = hm[m].max_dist;
  S.haus_ave = hm[m].ave_dist;
  if (S.fa_iter - 1 >= 5) S.max_sat = (hm[m].max_dist / hm[m].diag) < 0.8 * S.HR;
}

// ------------------------------------------------------------------------------- launchers
// internal node records (64 B): both child boxes and child ids
__global__ void k_pack(int n, const int32_t *child, const float *box, float4 *node) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int32_t l = child[2 * i], r = child[2 * i + 1];
  const float *bl = box + 6 * (int64_t)(l >= 0 ? l : n - 1 + ~l);
  const float *br = box + 6 * (int64_t)(r >= 0 ? r : n - 1 + ~r);
  node[4 * (int64_t)i] = make_float4(bl[0], bl[1], bl[2], bl[3]);
  node[4 * (int64_t)i + 1] = make_float4(bl[4], bl[5], br[0], br[1]);
  node[4 * (int64_t)i + 2] = make_float4(br[2], br[3], br[4], br[5]);
  node[4 * (int64_t)i + 3] = make_float4(__int_as_float(l), __int_as_float(r), 0.f, 0.f);
}

void launch_ep_points(const BvhDev &b, const double *P, const int64_t *ids, int64_t n, double upper, double *dist,
                      int *status, cudaStream_t st) {
  if (n > 0) k_ep_points<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(b, P, ids, n, upper, dist, status);
}
void launch_maxmean(const double *dist, int64_t n, double upper, double *out3, cudaStream_t st) {
  k_maxmean<<<1, 1024, 0, st>>>(dist, n, upper, out3);
}
void launch_ep_faces(const double *tri, int64_t nf, double *EP, cudaStream_t st) {
  if (nf > 0) k_ep_faces<<<(unsigned)((nf + 127) / 128), 128, 0, st>>>(tri, nf, EP);
}
void launch_haus_combine(HausMesh *hm, int n, cudaStream_t st) {
  if (n > 0) k_haus_combine<<<(n + 127) / 128, 128, 0, st>>>(hm, n);
}
void launch_fa_haus_flag(MeshScalars *sc, const HausMesh *hm, int n, cudaStream_t st) {
  k_fa_haus_flag<<<(n + 127) / 128, 128, 0, st>>>(sc, hm, n);
}
void bvh_morton(const BvhDev &b, const double lo[3], const double hi[3], unsigned long long *keys, cudaStream_t st) {
  double inv[3];
  for (int d = 0; d < 3; d++) inv[d] = (hi[d] > lo[d]) ? 1.0 / (hi[d] - lo[d]) : 0.0;
  if (b.n > 0) k_morton<<<(b.n + 255) / 256, 256, 0, st>>>(b, lo[0], lo[1], lo[2], inv[0], inv[1], inv[2], keys);
}
void bvh_karras(int n, const unsigned long long *keys, int32_t *child, int32_t *parent, int32_t *leaf_face,
                cudaStream_t st, int32_t *range) {
  if (n > 0) k_karras<<<(n + 255) / 256, 256, 0, st>>>(n, keys, child, parent, leaf_face, range);
}
void bvh_orient(const BvhDev &b, const int32_t *range, float4 *obb, float4 *onode, cudaStream_t st) {
  if (b.n < 2) return;
  k_obb_leaf<<<(b.n + 127) / 128, 128, 0, st>>>(b, obb);
  k_obb_node<<<(b.n + 126) / 128, 128, 0, st>>>(b, range, obb);
  k_opack<<<(b.n + 126) / 128, 128, 0, st>>>(b.n, b.child, obb, onode);
}
void bvh_refit_batch(const RefitDev *R, const Seg *seg, const MeshDesc *md, int64_t nblk, int threads,
                     cudaStream_t st) {
  if (nblk > 0) k_refit_batch<<<(unsigned)nblk, threads, 0, st>>>(R, seg, md);
}
void bvh_refit(const BvhDev &b, float *box, const int32_t *parent, unsigned *counters, float4 *node, float4 *leafd,
               cudaStream_t st) {
  if (b.n <= 0) return;
  k_refit<<<(b.n + 127) / 128, 128, 0, st>>>(b, box, parent, counters, leafd);
  if (b.n > 1) k_pack<<<(b.n + 254) / 256, 256, 0, st>>>(b.n, b.child, box, node);
}
static const unsigned kWarpGrid = 1216;  // persistent warp-pass grid (152 SMs x 8 blocks of 4 warps)
static const unsigned kEvalGrid = 152 * 8;  // dense exact pass: grid-stride over the candidates
void launch_project(const ProjArgs &p, int64_t nblk, cudaStream_t st) {
  if (nblk <= 0) return;
  cudaMemsetAsync(p.ovf.count, 0, sizeof(unsigned), st);
  cudaMemsetAsync(p.cand.count, 0, sizeof(unsigned), st);
  cudaMemsetAsync(p.cand.fb_count, 0, sizeof(unsigned), st);
  k_project<<<(unsigned)nblk, 128, 0, st>>>(p);
  k_project_warp<<<kWarpGrid, 128, 0, st>>>(p);
  k_cand_eval<0, 0><<<kEvalGrid, 128, 0, st>>>(p.cand, p.tgt, nullptr);
  k_project_finish<<<(unsigned)nblk, 128, 0, st>>>(p);
  k_project_fallback<<<kWarpGrid, 128, 0, st>>>(p);
}
void launch_curve_project(const ProjArgs &p, int64_t nblk, cudaStream_t st) {
  if (nblk > 0) k_curve_project<<<(unsigned)nblk, 128, 0, st>>>(p);
}
void launch_signed_distance(const TargetDev &t, int64_t np, const double *P, double *S, int32_t *I, double *C,
                            double *N, int *status, cudaStream_t st) {
  if (np > 0) k_signed_distance<<<(unsigned)((np + 127) / 128), 128, 0, st>>>(t, np, P, S, I, C, N, status);
}
void launch_haus_bbox(const HausArgs &h, int64_t nblk, cudaStream_t st) {
  k_haus_bbox<<<(unsigned)nblk, 128, 0, st>>>(h);
}
void launch_haus_side(const HausArgs &h, int side, int64_t nblk, cudaStream_t st) {
  cudaMemsetAsync(h.ovf.count, 0, sizeof(unsigned), st);
  cudaMemsetAsync(h.cand.count, 0, sizeof(unsigned), st);
  cudaMemsetAsync(h.cand.fb_count, 0, sizeof(unsigned), st);
  if (side == 0) {  // target samples against the boundary surface
    k_haus_side<0><<<(unsigned)nblk, 128, 0, st>>>(h);
    k_haus_warp<0><<<kWarpGrid, 128, 0, st>>>(h);
    k_cand_eval<1, 1><<<kEvalGrid, 128, 0, st>>>(h.cand, h.tgt, h.surf);
    k_haus_finish<0><<<(unsigned)nblk, 128, 0, st>>>(h);
    k_haus_fallback<0><<<kWarpGrid, 128, 0, st>>>(h);
    k_haus_reduce<0><<<(unsigned)nblk, 128, 0, st>>>(h);
  } else {  // surface samples against the target
    k_haus_side<1><<<(unsigned)nblk, 128, 0, st>>>(h);
    k_haus_warp<1><<<kWarpGrid, 128, 0, st>>>(h);
    k_cand_eval<1, 0><<<kEvalGrid, 128, 0, st>>>(h.cand, h.tgt, h.surf);
    k_haus_finish<1><<<(unsigned)nblk, 128, 0, st>>>(h);
    k_haus_fallback<1><<<kWarpGrid, 128, 0, st>>>(h);
    k_haus_reduce<1><<<(unsigned)nblk, 128, 0, st>>>(h);
  }
}

}  // namespace hexopt
