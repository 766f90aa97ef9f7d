// k_bvh.cu -- closest-point projection and Hausdorff distance on a GPU LBVH.
//
//  * LBVH build (Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees and
//    k-d trees"): 30-bit Morton codes of triangle centroids made unique with the face index,
//    radix-sorted (CUB), internal nodes from the longest common prefix, boxes fitted bottom-up
//    with per-node arrival counters.  Boxes are FP32, rounded outward, so every distance lower
//    bound stays conservative.  Dynamic surfaces (the hex mesh boundary) keep the topology and
//    are refitted from the current positions.
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

__global__ void k_karras(int n, const unsigned long long *keys, int32_t *child, int32_t *parent, int32_t *leaf_face) {
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

// Leaf boxes and bottom-up union.  counters: n - 1 zeros on entry, zeros again on exit.
__global__ void k_refit(BvhDev b, float *box, const int32_t *parent, unsigned *counters) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.n) return;
  const int n = b.n;
  double p[3][3];
  face_pts(b, b.leaf_face[k], p);
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
    float *bn = box + 6 * (int64_t)node;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      bn[d] = fminf(__ldcg(bl + d), __ldcg(br + d));
      bn[3 + d] = fmaxf(__ldcg(bl + 3 + d), __ldcg(br + 3 + d));
    }
    counters[node] = 0;
    __threadfence();
    node = parent[node];
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

// Ericson's closest point on triangle (Real-Time Collision Detection 5.1.5), FP64.
__device__ void closest_pt_tri(const double p[3], const double a[3], const double b[3], const double c[3],
                               double out[3]) {
  double ab[3], ac[3], ap[3], bp[3], cp[3];
#pragma unroll
  for (int d = 0; d < 3; d++) { ab[d] = b[d] - a[d]; ac[d] = c[d] - a[d]; ap[d] = p[d] - a[d]; }
  const double d1 = ab[0] * ap[0] + ab[1] * ap[1] + ab[2] * ap[2], d2 = ac[0] * ap[0] + ac[1] * ap[1] + ac[2] * ap[2];
  if (d1 <= 0.0 && d2 <= 0.0) { out[0] = a[0]; out[1] = a[1]; out[2] = a[2]; return; }
#pragma unroll
  for (int d = 0; d < 3; d++) bp[d] = p[d] - b[d];
  const double d3 = ab[0] * bp[0] + ab[1] * bp[1] + ab[2] * bp[2], d4 = ac[0] * bp[0] + ac[1] * bp[1] + ac[2] * bp[2];
  if (d3 >= 0.0 && d4 <= d3) { out[0] = b[0]; out[1] = b[1]; out[2] = b[2]; return; }
  const double vc = d1 * d4 - d3 * d2;
  if (!(a[0] == b[0] && a[1] == b[1] && a[2] == b[2]) && vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
    const double v = d1 / (d1 - d3);
#pragma unroll
    for (int d = 0; d < 3; d++) out[d] = a[d] + v * ab[d];
    return;
  }
#pragma unroll
  for (int d = 0; d < 3; d++) cp[d] = p[d] - c[d];
  const double d5 = ab[0] * cp[0] + ab[1] * cp[1] + ab[2] * cp[2], d6 = ac[0] * cp[0] + ac[1] * cp[1] + ac[2] * cp[2];
  if (d6 >= 0.0 && d5 <= d6) { out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; return; }
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    const double w = d2 / (d2 - d6);
#pragma unroll
    for (int d = 0; d < 3; d++) out[d] = a[d] + w * ac[d];
    return;
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
#pragma unroll
    for (int d = 0; d < 3; d++) out[d] = b[d] + w * (c[d] - b[d]);
    return;
  }
  const double denom = 1.0 / (va + vb + vc);
  const double v = vb * denom, w = vc * denom;
#pragma unroll
  for (int d = 0; d < 3; d++) out[d] = a[d] + ab[d] * v + ac[d] * w;
}

// ---- FP32 filtering with exact FP64 evaluation ----
// Traversal and leaf screening run in FP32 on coordinates taken relative to the leaf's first
// vertex (formed in FP64, rounded once).  A face is evaluated in FP64 only when its FP32 lower
// bound is within a margin of the current best, so the FP64 result is the one a pure FP64
// search returns: boxes are stored rounded outward, the box margin covers the rounding of the
// query, and the leaf margin (1e-4 of the local scale) covers the FP32 point-triangle distance
// of triangles whose smallest angle is above ~0.6 degrees; thinner triangles fall back to their
// box distance as the lower bound.
__device__ __forceinline__ float box_d2f(const float *bx, const float q[3]) {
  float s = 0.f;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const float e = fmaxf(fmaxf(bx[d] - q[d], q[d] - bx[3 + d]), 0.f);
    s = fmaf(e, e, s);
  }
  return s;
}

// Squared distance from p to the triangle (0, b, c) in FP32 (Ericson's region tests).
__device__ __forceinline__ float tri_d2f(const float p[3], const float b[3], const float c[3]) {
  const float d1 = b[0] * p[0] + b[1] * p[1] + b[2] * p[2], d2 = c[0] * p[0] + c[1] * p[1] + c[2] * p[2];
  float x[3];
  if (d1 <= 0.f && d2 <= 0.f) { x[0] = 0.f; x[1] = 0.f; x[2] = 0.f; }
  else {
    const float bp[3] = {p[0] - b[0], p[1] - b[1], p[2] - b[2]};
    const float d3 = b[0] * bp[0] + b[1] * bp[1] + b[2] * bp[2], d4 = c[0] * bp[0] + c[1] * bp[1] + c[2] * bp[2];
    const float vc = d1 * d4 - d3 * d2;
    const float cp[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
    const float d5 = b[0] * cp[0] + b[1] * cp[1] + b[2] * cp[2], d6 = c[0] * cp[0] + c[1] * cp[1] + c[2] * cp[2];
    const float vb = d5 * d2 - d1 * d6;
    const float va = d3 * d6 - d5 * d4;
    if (d3 >= 0.f && d4 <= d3) { x[0] = b[0]; x[1] = b[1]; x[2] = b[2]; }
    else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
      const float v = d1 / (d1 - d3);
      x[0] = v * b[0]; x[1] = v * b[1]; x[2] = v * b[2];
    } else if (d6 >= 0.f && d5 <= d6) { x[0] = c[0]; x[1] = c[1]; x[2] = c[2]; }
    else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
      const float w = d2 / (d2 - d6);
      x[0] = w * c[0]; x[1] = w * c[1]; x[2] = w * c[2];
    } else if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
      const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
      x[0] = b[0] + w * (c[0] - b[0]); x[1] = b[1] + w * (c[1] - b[1]); x[2] = b[2] + w * (c[2] - b[2]);
    } else {
      const float den = 1.f / (va + vb + vc);
      const float v = vb * den, w = vc * den;
      x[0] = b[0] * v + c[0] * w; x[1] = b[1] * v + c[1] * w; x[2] = b[2] * v + c[2] * w;
    }
  }
  const float e0 = p[0] - x[0], e1 = p[1] - x[1], e2 = p[2] - x[2];
  return e0 * e0 + e1 * e1 + e2 * e2;
}

// Lower bound (FP32, with its margin applied) of the distance from q to face P.
__device__ __forceinline__ float leaf_lower_bound(const double q[3], const double P[3][3], const float *lbox,
                                                  const float qf[3]) {
  float qa[3], ab[3], ac[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    qa[d] = float(q[d] - P[0][d]);
    ab[d] = float(P[1][d] - P[0][d]);
    ac[d] = float(P[2][d] - P[0][d]);
  }
  const float cx = ab[1] * ac[2] - ab[2] * ac[1], cy = ab[2] * ac[0] - ab[0] * ac[2], cz = ab[0] * ac[1] - ab[1] * ac[0];
  const float lab = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2], lac = ac[0] * ac[0] + ac[1] * ac[1] + ac[2] * ac[2];
  const float L = fabsf(qa[0]) + fabsf(qa[1]) + fabsf(qa[2]) + sqrtf(lab) + sqrtf(lac);
  if (cx * cx + cy * cy + cz * cz >= 1e-4f * lab * lac)
    return sqrtf(tri_d2f(qa, ab, ac)) - 1e-4f * L;
  return sqrtf(box_d2f(lbox, qf)) - 1e-6f * (1.f + fabsf(qf[0]) + fabsf(qf[1]) + fabsf(qf[2]));
}

__device__ __forceinline__ const float *node_box(const BvhDev &b, int32_t c) {
  return b.box + 6 * (int64_t)(c >= 0 ? c : b.n - 1 + ~c);
}

// Nearest face (squared FP64 distance, face id, closest point).  Returns false on stack overflow.
__device__ bool bvh_closest(const BvhDev &b, const double q[3], double &best, int32_t &bf, double bc[3]) {
  int32_t stack[kStack];
  int sp = 0;
  bool ok = true;
  const int n = b.n;
  const float qf[3] = {float(q[0]), float(q[1]), float(q[2])};
  const float mbox = 1e-6f * (1.f + fabsf(qf[0]) + fabsf(qf[1]) + fabsf(qf[2]));
  float bestd = isinf(best) ? INFINITY : __double2float_ru(sqrt(best));
  stack[sp++] = n == 1 ? ~0 : 0;
  while (sp > 0) {
    const int32_t node = stack[--sp];
    if (node < 0) {
      const int32_t leaf = ~node;
      if (leaf >= n) { ok = false; continue; }
      const int32_t f = b.leaf_face[leaf];
      double p[3][3];
      face_pts(b, f, p);
      if (leaf_lower_bound(q, p, node_box(b, node), qf) > bestd) continue;
      double c[3];
      closest_pt_tri(q, p[0], p[1], p[2], c);
      const double e0 = q[0] - c[0], e1 = q[1] - c[1], e2 = q[2] - c[2];
      const double d2 = e0 * e0 + e1 * e1 + e2 * e2;
      if (d2 < best) {
        best = d2; bf = f; bc[0] = c[0]; bc[1] = c[1]; bc[2] = c[2];
        bestd = __double2float_ru(sqrt(best));
      }
      continue;
    }
    if (node >= n - 1) { ok = false; continue; }
    const int32_t l = b.child[2 * node], r = b.child[2 * node + 1];
    if (l >= n - 1 || r >= n - 1 || ~l >= n || ~r >= n) { ok = false; continue; }
    const float dl = sqrtf(box_d2f(node_box(b, l), qf)) - mbox;
    const float dr = sqrtf(box_d2f(node_box(b, r), qf)) - mbox;
    const int32_t nearc = dl <= dr ? l : r, farc = dl <= dr ? r : l;
    const float dn = fminf(dl, dr), df = fmaxf(dl, dr);
    if (df <= bestd) { if (sp < kStack) stack[sp++] = farc; else ok = false; }
    if (dn <= bestd) { if (sp < kStack) stack[sp++] = nearc; else ok = false; }
  }
  return ok;
}

// pseudonormal_test: normal at the closest point c of face f (vertex / edge / face normal).
__device__ void pseudonormal(const TargetDev &t, int32_t f, const double c[3], double n[3]) {
  double A[3], B[3], C[3];
#pragma unroll
  for (int d = 0; d < 3; d++) { A[d] = t.tri[(int64_t)f * 9 + d]; B[d] = t.tri[(int64_t)f * 9 + 3 + d]; C[d] = t.tri[(int64_t)f * 9 + 6 + d]; }
  const double e1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]}, e2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
  const double x0 = e1[1] * e2[2] - e1[2] * e2[1], x1 = e1[2] * e2[0] - e1[0] * e2[2], x2 = e1[0] * e2[1] - e1[1] * e2[0];
  const double area = sqrt(x0 * x0 + x1 * x1 + x2 * x2);  // doublearea
  const double epsilon = 1e-12;
  int kind = 0, which = 0;  // 0 face, 1 vertex (which corner), 2 edge (opposite which corner)
  if (area > 1e-4) {
    const double v2[3] = {c[0] - A[0], c[1] - A[1], c[2] - A[2]};
    const double d00 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2], d01 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
    const double d11 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
    const double d20 = v2[0] * e1[0] + v2[1] * e1[1] + v2[2] * e1[2], d21 = v2[0] * e2[0] + v2[1] * e2[1] + v2[2] * e2[2];
    const double den = d00 * d11 - d01 * d01;
    double bb[3];
    bb[1] = (d11 * d20 - d01 * d21) / den;
    bb[2] = (d00 * d21 - d01 * d20) / den;
    bb[0] = 1.0 - (bb[1] + bb[2]);
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
      const double dx = c[0] - P[v][0], dy = c[1] - P[v][1], dz = c[2] - P[v][2];
      if (sqrt(dx * dx + dy * dy + dz * dz) < epsilon) { found = true; kind = 1; which = v; }
    }
    for (int e = 0; e < 3 && !found; e++) {
      const double *s = P[(e + 1) % 3], *dd = P[(e + 2) % 3];
      const double dms[3] = {dd[0] - s[0], dd[1] - s[1], dd[2] - s[2]};
      const double smp[3] = {s[0] - c[0], s[1] - c[1], s[2] - c[2]};
      const double vl = dms[0] * dms[0] + dms[1] * dms[1] + dms[2] * dms[2];
      const double tt = -(dms[0] * smp[0] + dms[1] * smp[1] + dms[2] * smp[2]) / vl;
      double sq;
      if (tt < 0) {
        sq = smp[0] * smp[0] + smp[1] * smp[1] + smp[2] * smp[2];
      } else if (tt > 1) {
        const double z0 = c[0] - dd[0], z1 = c[1] - dd[1], z2 = c[2] - dd[2];
        sq = z0 * z0 + z1 * z1 + z2 * z2;
      } else {
        const double pr0 = (1.0 - tt) * s[0] + tt * dd[0], pr1 = (1.0 - tt) * s[1] + tt * dd[1], pr2 = (1.0 - tt) * s[2] + tt * dd[2];
        const double m0 = c[0] - pr0, m1 = c[1] - pr1, m2 = c[2] - pr2;
        sq = m0 * m0 + m1 * m1 + m2 * m2;
      }
      if (sqrt(sq) < epsilon) { found = true; kind = 2; which = e; }
    }
  }
  const double *src = kind == 0 ? t.FN + 3 * (int64_t)f : kind == 1 ? t.VNc + 9 * (int64_t)f + 3 * which : t.ENc + 9 * (int64_t)f + 3 * which;
  n[0] = src[0]; n[1] = src[1]; n[2] = src[2];
}

// Tangent planes of the regular boundary vertices (dirty_graph_projection, :4031-4078):
// normal_T = pseudonormal, dis_T = normal_T . closest point.
__global__ void __launch_bounds__(128) k_project(ProjArgs p) {
  const Seg sg = p.seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  if (i >= sg.end) return;
  const MeshDesc md = p.mesh[sg.mesh];
  const TargetDev &t = p.tgt[sg.mesh];
  const int64_t e = md.t_off + (i - md.kitem0[K_PROJ]);
  const int64_t v = md.v_off + p.t_ids[e];
  const double q[3] = {p.X[4 * v], p.X[4 * v + 1], p.X[4 * v + 2]};
  double best = INFINITY, c[3] = {0, 0, 0}, n[3] = {0, 0, 0};
  int32_t f = -1;
  if (t.bvh.n > 0 && !bvh_closest(t.bvh, q, best, f, c)) atomicOr(&p.sc[sg.mesh].status, 8);
  if (f >= 0) pseudonormal(t, f, c, n);
  p.t_nrm[3 * e] = n[0]; p.t_nrm[3 * e + 1] = n[1]; p.t_nrm[3 * e + 2] = n[2];
  p.t_dis[e] = n[0] * c[0] + n[1] * c[1] + n[2] * c[2];
}

// signed_distance_pseudonormal for arbitrary query points (rows) against mesh m's target
__global__ void __launch_bounds__(128) k_signed_distance(TargetDev t, int64_t np, const double *P, double *S,
                                                         int32_t *I, double *C, double *N, int *status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double q[3] = {P[3 * i], P[3 * i + 1], P[3 * i + 2]};
  double best = INFINITY, c[3] = {0, 0, 0}, n[3] = {0, 0, 0};
  int32_t f = -1;
  if (t.bvh.n > 0 && !bvh_closest(t.bvh, q, best, f, c)) atomicOr(status, 8);
  double s = 1;
  if (f >= 0) {
    pseudonormal(t, f, c, n);
    s = ((q[0] - c[0]) * n[0] + (q[1] - c[1]) * n[1] + (q[2] - c[2]) * n[2]) >= 0 ? 1. : -1.;
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
struct EPFace {
  double p[3][3], edge[3][3], dir[3], off, darea;
  int axis;
};

__device__ void ep_setup(const double P[3][3], EPFace &e) {
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) e.p[c][d] = P[c][d];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    e.edge[0][d] = P[1][d] - P[0][d];
    e.edge[1][d] = P[2][d] - P[1][d];
    e.edge[2][d] = P[0][d] - P[2][d];
  }
  e.dir[0] = e.edge[0][1] * e.edge[1][2] - e.edge[0][2] * e.edge[1][1];
  e.dir[1] = e.edge[0][2] * e.edge[1][0] - e.edge[0][0] * e.edge[1][2];
  e.dir[2] = e.edge[0][0] * e.edge[1][1] - e.edge[0][1] * e.edge[1][0];
  e.off = e.dir[0] * P[0][0] + e.dir[1] * P[0][1] + e.dir[2] * P[0][2];
  const double nn = sqrt(e.dir[0] * e.dir[0] + e.dir[1] * e.dir[1] + e.dir[2] * e.dir[2]);
  if (nn > 0) { e.dir[0] /= nn; e.dir[1] /= nn; e.dir[2] /= nn; e.off /= nn; }
  const double nx = fabs(e.dir[0]), ny = fabs(e.dir[1]), nz = fabs(e.dir[2]);
  double s;
  if (nx > ny && nx > nz) { e.axis = 0; s = 1 / e.dir[0]; }
  else if (ny > nz) { e.axis = 1; s = 1 / e.dir[1]; }
  else { e.axis = 2; s = 1 / e.dir[2]; }
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) e.edge[c][d] *= s;
  const double a0 = P[1][0] - P[0][0], a1 = P[1][1] - P[0][1], a2 = P[1][2] - P[0][2];
  const double b0 = P[2][0] - P[0][0], b1 = P[2][1] - P[0][1], b2 = P[2][2] - P[0][2];
  const double c0 = a1 * b2 - a2 * b1, c1 = a2 * b0 - a0 * b2, c2 = a0 * b1 - a1 * b0;
  e.darea = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
}

__device__ __forceinline__ double ps_dist(const double q[3], const double *v1, const double *v2) {
  const double e[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
  double t = ((q[0] - v1[0]) * e[0] + (q[1] - v1[1]) * e[1] + (q[2] - v1[2]) * e[2]) / (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
  t = t < 0 ? 0 : (t > 1 ? 1 : t);
  const double d0 = q[0] - (v1[0] + e[0] * t), d1 = q[1] - (v1[1] + e[1] * t), d2 = q[2] - (v1[2] + e[2] * t);
  return sqrt(d0 * d0 + d1 * d1 + d2 * d2);
}

__device__ void point_distance_ep(const EPFace &f, const double q[3], double &dist) {
  const double EPS = 0.000001;
  const double d = f.dir[0] * q[0] + f.dir[1] * q[1] + f.dir[2] * q[2] - f.off;
  if (d > dist || d < -dist) return;
  const double p[3] = {q[0] - f.dir[0] * d, q[1] - f.dir[1] * d, q[2] - f.dir[2] * d};
  const int i1 = f.axis == 0 ? 1 : (f.axis == 1 ? 2 : 0), i2 = f.axis == 0 ? 2 : (f.axis == 1 ? 0 : 1);
  const double b0 = f.edge[1][i1] * (p[i2] - f.p[1][i2]) - f.edge[1][i2] * (p[i1] - f.p[1][i1]);
  if (b0 <= 0) { const double x = ps_dist(q, f.p[1], f.p[2]); if (dist > x) dist = x; return; }
  const double b1 = f.edge[2][i1] * (p[i2] - f.p[2][i2]) - f.edge[2][i2] * (p[i1] - f.p[2][i1]);
  if (b1 <= 0) { const double x = ps_dist(q, f.p[2], f.p[0]); if (dist > x) dist = x; return; }
  const double b2 = f.edge[0][i1] * (p[i2] - f.p[0][i2]) - f.edge[0][i2] * (p[i1] - f.p[0][i1]);
  if (b2 <= 0) { const double x = ps_dist(q, f.p[0], f.p[1]); if (dist > x) dist = x; return; }
  double b = fmin(b0, b1);
  b = fmin(b, b2);
  if (b < EPS * f.darea) {
    double bt;
    if (b == b0) bt = ps_dist(q, f.p[1], f.p[2]);
    else if (b == b1) bt = ps_dist(q, f.p[2], f.p[0]);
    else bt = ps_dist(q, f.p[0], f.p[1]);
    if (dist > bt) dist = bt;
    return;
  }
  dist = fabs(d);
}

// min over faces of PointDistanceEP, starting from `dist` (the upper bound).  PointDistanceEP is
// never below the true point-triangle distance, so the FP32 lower bound screens faces the same
// way as in the closest-point search.
__device__ bool bvh_ep(const BvhDev &b, const double q[3], double &dist) {
  int32_t stack[kStack];
  int sp = 0;
  bool ok = true;
  const int n = b.n;
  const float qf[3] = {float(q[0]), float(q[1]), float(q[2])};
  const float mbox = 1e-6f * (1.f + fabsf(qf[0]) + fabsf(qf[1]) + fabsf(qf[2]));
  float bestd = __double2float_ru(dist);
  stack[sp++] = n == 1 ? ~0 : 0;
  while (sp > 0) {
    const int32_t node = stack[--sp];
    if (node < 0) {
      if (~node >= n) { ok = false; continue; }
      double P[3][3];
      face_pts(b, b.leaf_face[~node], P);
      if (leaf_lower_bound(q, P, node_box(b, node), qf) > bestd) continue;
      EPFace f;
      ep_setup(P, f);
      point_distance_ep(f, q, dist);
      bestd = __double2float_ru(dist);
      continue;
    }
    if (node >= n - 1) { ok = false; continue; }
    const int32_t l = b.child[2 * node], r = b.child[2 * node + 1];
    if (l >= n - 1 || r >= n - 1 || ~l >= n || ~r >= n) { ok = false; continue; }
    const float dl = sqrtf(box_d2f(node_box(b, l), qf)) - mbox;
    const float dr = sqrtf(box_d2f(node_box(b, r), qf)) - mbox;
    const int32_t nearc = dl <= dr ? l : r, farc = dl <= dr ? r : l;
    const float dn = fminf(dl, dr), df = fmaxf(dl, dr);
    if (df <= bestd) { if (sp < kStack) stack[sp++] = farc; else ok = false; }
    if (dn <= bestd) { if (sp < kStack) stack[sp++] = nearc; else ok = false; }
  }
  return ok;
}

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
// SIDE 1 = surface vertices vs target faces.
template <int SIDE>
__global__ void __launch_bounds__(128) k_haus_side(HausArgs h) {
  const Seg sg = h.seg[blockIdx.x];
  const int64_t i = sg.begin + threadIdx.x;
  const MeshDesc md = h.mesh[sg.mesh];
  HausMesh &hm = h.hm[sg.mesh];
  const double upper = hm.diag;
  double mx[1] = {-INFINITY}, acc[2] = {0, 0};
  if (i < sg.end) {
    double q[3];
    if (SIDE == 0) {
      const int64_t v = h.tgt_vs[i];
      const TargetDev &t = h.tgt[sg.mesh];
      q[0] = t.TV[3 * v]; q[1] = t.TV[3 * v + 1]; q[2] = t.TV[3 * v + 2];
    } else {
      const int64_t v = h.surf_vs[i];
      q[0] = h.X[4 * v]; q[1] = h.X[4 * v + 1]; q[2] = h.X[4 * v + 2];
    }
    double dist = upper;
    const BvhDev &b = SIDE == 0 ? h.surf[sg.mesh] : h.tgt[sg.mesh].bvh;
    if (b.n > 0 && !bvh_ep(b, q, dist)) atomicOr(&h.sc[sg.mesh].status, 8);
    if (dist != upper) { mx[0] = dist; acc[0] = dist; acc[1] = 1; }
  }
  __shared__ double smem[2][32];
  double nm[1] = {-mx[0]};
  block_min<1>(nm, smem);
  const double bm = -nm[0];
  block_sum<2>(acc, smem);
  double out[3] = {bm, acc[0], acc[1]};
  const int kind = SIDE == 0 ? K_TGTV : K_SURFV;
  if (publish_partials<3>(out, h.partials, blockIdx.x, h.counters + sg.mesh, md.knblk[kind])) {
    double m = -INFINITY;
    for (int b = threadIdx.x; b < md.knblk[kind]; b += blockDim.x)
      m = fmax(m, __ldcg(&h.partials[(md.kblk0[kind] + b) * 3]));
    double t[1] = {-m};
    block_min<1>(t, smem);
    double s = gather_partials_sum(h.partials, md.kblk0[kind], md.knblk[kind], 3, 1, smem);
    double c = gather_partials_sum(h.partials, md.kblk0[kind], md.knblk[kind], 3, 2, smem);
    if (threadIdx.x == 0) {
      hm.side_max[SIDE] = -t[0];
      hm.side_mean[SIDE] = s / c;
      if (SIDE == 1) {
        hm.max_dist = fmax(hm.side_max[0], hm.side_max[1]);
        hm.ave_dist = fmax(hm.side_mean[1], hm.side_mean[0]);
      }
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
  if (b.n > 0 && !bvh_ep(b, q, d)) atomicOr(status, 8);
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
void launch_ep_points(const BvhDev &b, const double *P, const int64_t *ids, int64_t n, double upper, double *dist,
                      int *status, cudaStream_t st) {
  if (n > 0) k_ep_points<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(b, P, ids, n, upper, dist, status);
}
void launch_maxmean(const double *dist, int64_t n, double upper, double *out3, cudaStream_t st) {
  k_maxmean<<<1, 1024, 0, st>>>(dist, n, upper, out3);
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
                cudaStream_t st) {
  if (n > 0) k_karras<<<(n + 255) / 256, 256, 0, st>>>(n, keys, child, parent, leaf_face);
}
void bvh_refit(const BvhDev &b, float *box, const int32_t *parent, unsigned *counters, cudaStream_t st) {
  if (b.n > 0) k_refit<<<(b.n + 127) / 128, 128, 0, st>>>(b, box, parent, counters);
}
void launch_project(const ProjArgs &p, int64_t nblk, cudaStream_t st) {
  if (nblk > 0) k_project<<<(unsigned)nblk, 128, 0, st>>>(p);
}
void launch_curve_project(const ProjArgs &p, int64_t nblk, cudaStream_t st) {
  if (nblk > 0) k_curve_project<<<(unsigned)nblk, 128, 0, st>>>(p);
}
void launch_signed_distance(const TargetDev &t, int64_t np, const double *P, double *S, int32_t *I, double *C,
                            double *N, int *status, cudaStream_t st) {
  if (np > 0) k_signed_distance<<<(unsigned)((np + 127) / 128), 128, 0, st>>>(t, np, P, S, I, C, N, status);
}
void launch_haus_bbox(const HausArgs &h, int64_t nblk, cudaStream_t st) {
  k_haus_bbox<<<(unsigned)nblk, 256, 0, st>>>(h);
}
void launch_haus_side(const HausArgs &h, int side, int64_t nblk, cudaStream_t st) {
  if (side == 0) k_haus_side<0><<<(unsigned)nblk, 128, 0, st>>>(h);
  else k_haus_side<1><<<(unsigned)nblk, 128, 0, st>>>(h);
}

}  // namespace hexopt
