/*
 * hexopt_oracle.c -- CPU restatement of the reference's FP64 optimisation path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker of the CUDA path and the timed CPU "port"
 * baseline.  Not linked by the product.  Pinned against the reference's own outputs through
 * tests/golden (generated from oracle/_ref, a build of the reference sources).
 *
 * Build: gcc -O2 -std=c99 -ffp-contract=off -fPIC -shared (see oracle/Makefile).
 */
#include "hexopt_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Topology tables that must equal the reference's (global_types.h:154-173, 208-218). */
static const int HEX_TET[8][4] = {
  {0, 3, 4, 1}, {1, 0, 5, 2}, {2, 1, 6, 3}, {3, 2, 7, 0},
  {4, 7, 5, 0}, {5, 4, 6, 1}, {6, 5, 7, 2}, {7, 6, 4, 3}};
static const int HEX_FACE[6][4] = {
  {0, 1, 2, 3}, {4, 7, 6, 5}, {0, 4, 5, 1}, {0, 3, 7, 4}, {3, 2, 6, 7}, {1, 5, 6, 2}};
static const double HEX_REF[8][3] = {
  {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
/* igl::grad_tet_ref face list and the vertex opposite each face (grad.cpp:406-411, 440-456) */
static const int TET_FACE[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
static const int TET_OPP[4] = {3, 1, 2, 0};

#define PRECISION 1.e-7 /* global_types.h:23 */

/* ------------------------------------------------------------------ small vector helpers */
static inline void sub3(const double *a, const double *b, double *o) {
  o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
static inline double dot3(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double norm3(const double *a) { return sqrt(dot3(a, a)); }
/* Eigen's fixed-size 3x3 determinant (Eigen/src/LU/Determinant.h, det3 cofactor order),
 * m[r][c]. */
static inline double det3m(double m[3][3]) {
  return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
         m[1][0] * (m[0][1] * m[2][2] - m[0][2] * m[2][1]) +
         m[2][0] * (m[0][1] * m[1][2] - m[0][2] * m[1][1]);
}

/* ------------------------------------------------------------------ scaled Jacobian */
/* a_jacobian (global_functions.cpp:2422-2442) */
static double a_jacobian(const double *c0, const double *c1, const double *c2, const double *c3) {
  double J[3][3];
  for (int r = 0; r < 3; r++) {
    J[r][0] = (c1[r] - c0[r]) * .5;
    J[r][1] = (c2[r] - c0[r]) * .5;
    J[r][2] = (c3[r] - c0[r]) * .5;
  }
  double n1 = sqrt(J[0][0] * J[0][0] + J[1][0] * J[1][0] + J[2][0] * J[2][0]);
  double n2 = sqrt(J[0][1] * J[0][1] + J[1][1] * J[1][1] + J[2][1] * J[2][1]);
  double n3 = sqrt(J[0][2] * J[0][2] + J[1][2] * J[1][2] + J[2][2] * J[2][2]);
  double sj = det3m(J);
  if (fabs(n1) < PRECISION || fabs(n2) < PRECISION || fabs(n3) < PRECISION) return sj;
  return sj / (n1 * n2 * n3);
}

void orc_scaled_jacobian(int64_t nv, const double *V, int64_t nh, const uint32_t *H,
                         double *V_Js, double *H_Js, double *min_J, double *ave_J,
                         double *dev_J, int64_t *n_inverted) {
  (void)nv;
  double ave = 0, mn = 1;
  int64_t inv = 0;
  double *hj = H_Js ? H_Js : (double *)malloc(sizeof(double) * (nh > 0 ? nh : 1));
  for (int64_t i = 0; i < nh; i++) {
    double hmin = 1;
    for (int j = 0; j < 8; j++) {
      const uint32_t *hv = H + 8 * i;
      double v = a_jacobian(V + 3 * (int64_t)hv[HEX_TET[j][0]], V + 3 * (int64_t)hv[HEX_TET[j][1]],
                            V + 3 * (int64_t)hv[HEX_TET[j][2]], V + 3 * (int64_t)hv[HEX_TET[j][3]]);
      if (hmin > v) hmin = v;
      if (V_Js) V_Js[8 * i + j] = v;
    }
    hj[i] = hmin;
    ave += hmin;
    if (mn > hmin) mn = hmin;
    if (hmin < 0) inv++;
  }
  ave /= (double)nh;
  double dev = 0;
  for (int64_t i = 0; i < nh; i++) dev += (hj[i] - ave) * (hj[i] - ave);
  dev /= (double)nh;
  if (!H_Js) free(hj);
  if (min_J) *min_J = mn;
  if (ave_J) *ave_J = ave;
  if (dev_J) *dev_J = dev;
  if (n_inverted) *n_inverted = inv;
}

/* ------------------------------------------------------------------ reference shapes */
/* hex2tet24 (global_functions.cpp:3994-4022): volume of the 24-tet split of a hex. */
static double hex2tet24(const double *V, const uint32_t *vs) {
  double fvs[6][3], hv[3] = {0, 0, 0};
  for (int i = 0; i < 6; i++) {
    fvs[i][0] = fvs[i][1] = fvs[i][2] = 0;
    for (int j = 0; j < 4; j++) {
      const double *p = V + 3 * (int64_t)vs[HEX_FACE[i][j]];
      fvs[i][0] += p[0]; fvs[i][1] += p[1]; fvs[i][2] += p[2];
    }
    fvs[i][0] /= 4; fvs[i][1] /= 4; fvs[i][2] /= 4;
  }
  for (int i = 0; i < 8; i++) {
    const double *p = V + 3 * (int64_t)vs[i];
    hv[0] += p[0]; hv[1] += p[1]; hv[2] += p[2];
  }
  hv[0] /= 8; hv[1] /= 8; hv[2] /= 8;
  double volume = 0;
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 4; j++) {
      const double *p0 = V + 3 * (int64_t)vs[HEX_FACE[i][j]];
      const double *p1 = V + 3 * (int64_t)vs[HEX_FACE[i][(j + 1) % 4]];
      double J[3][3];
      for (int r = 0; r < 3; r++) {
        J[r][0] = p0[r] - hv[r];
        J[r][1] = p1[r] - hv[r];
        J[r][2] = fvs[i][r] - hv[r];
      }
      volume += fabs(det3m(J) / 6);
    }
  return volume;
}

/* compute_referenceMesh / hex2cuboid_ (global_functions.cpp:3735-3806) */
void orc_reference_mesh(const double *V, int64_t nh, const uint32_t *H, const uint8_t *h_flag,
                        int cube, double *RT) {
  for (int64_t h = 0; h < nh; h++) {
    const uint32_t *vs = H + 8 * h;
    double v8[8][3];
    int flag = h_flag ? h_flag[h] : 1;
    if (!flag) {
      for (int i = 0; i < 8; i++)
        for (int d = 0; d < 3; d++) v8[i][d] = V[3 * (int64_t)vs[i] + d];
    } else {
      double e0 = 0, e1 = 0, e2 = 0;
      double volume = hex2tet24(V, vs);
      if (cube && fabs(volume) > 1e-20) {
        e0 = e1 = e2 = cbrt(volume);
      } else {
        double t[3];
#define EL(a, b) (sub3(V + 3 * (int64_t)vs[a], V + 3 * (int64_t)vs[b], t), norm3(t))
        e0 += EL(0, 1); e0 += EL(3, 2); e0 += EL(4, 5); e0 += EL(7, 6); e0 /= 4;
        e1 += EL(0, 3); e1 += EL(1, 2); e1 += EL(4, 7); e1 += EL(5, 6); e1 /= 4;
        e2 += EL(0, 4); e2 += EL(1, 5); e2 += EL(2, 6); e2 += EL(3, 7); e2 /= 4;
#undef EL
        double ratio = cbrt(volume / (e0 * e1 * e2));
        e0 *= ratio; e1 *= ratio; e2 *= ratio;
      }
      for (int i = 0; i < 8; i++) {
        v8[i][0] = HEX_REF[i][0] * e0;
        v8[i][1] = HEX_REF[i][1] * e1;
        v8[i][2] = HEX_REF[i][2] * e2;
      }
    }
    for (int k = 0; k < 8; k++)
      for (int j = 0; j < 4; j++)
        for (int d = 0; d < 3; d++) RT[((8 * h + k) * 4 + j) * 3 + d] = v8[HEX_TET[k][j]][d];
  }
}

/* igl::grad_tet_ref, uniform branch (extern/libigl/include/igl/grad.cpp:372-478), restated per
 * tet.  Volumes follow igl::volume (volume.cpp:15-31). */
void orc_grad_ref(const double *V, int64_t nh, const uint32_t *H, const double *RT, double *Dg) {
  int64_t nt = 8 * nh;
  for (int64_t t = 0; t < nt; t++) {
    const uint32_t *hv = H + 8 * (t / 8);
    int k = (int)(t % 8);
    const double *a = V + 3 * (int64_t)hv[HEX_TET[k][0]];
    const double *b = V + 3 * (int64_t)hv[HEX_TET[k][1]];
    const double *c = V + 3 * (int64_t)hv[HEX_TET[k][2]];
    const double *d = V + 3 * (int64_t)hv[HEX_TET[k][3]];
    double ad[3], bd[3], cd[3], x[3];
    sub3(a, d, ad); sub3(b, d, bd); sub3(c, d, cd);
    cross3(bd, cd, x);
    double vol = -dot3(ad, x) / 6.;
    const double *RF = RT + t * 12;
    double e01[3], e02[3], e03[3];
    sub3(RF + 0, RF + 3, e01); sub3(RF + 0, RF + 6, e02); sub3(RF + 0, RF + 9, e03);
    cross3(e01, e02, x);
    double volume_i = fabs(dot3(x, e03)) / 6;
    double scale_i = cbrt(vol / volume_i);
    for (int f = 0; f < 4; f++) {
      double e0[3], e1[3], n[3];
      const double *p0 = RF + 3 * TET_FACE[f][0];
      const double *p1 = RF + 3 * TET_FACE[f][1];
      const double *p2 = RF + 3 * TET_FACE[f][2];
      for (int r = 0; r < 3; r++) {
        e0[r] = (p0[r] - p1[r]) * scale_i;
        e1[r] = (p0[r] - p2[r]) * scale_i;
      }
      cross3(e0, e1, n);
      double area = norm3(n) / 2;
      double l0 = norm3(e0), l1 = norm3(e1);
      for (int r = 0; r < 3; r++) { e0[r] /= l0; e1[r] /= l1; }
      cross3(e0, e1, n);
      double ln = norm3(n);
      for (int r = 0; r < 3; r++) n[r] /= ln;
      double val = area / (3 * vol);
      int j = TET_OPP[f];
      for (int r = 0; r < 3; r++) Dg[(t * 4 + j) * 3 + r] = val * n[r];
    }
  }
}

/* ------------------------------------------------------------------ 3x3 SVD / polar */
/* One-sided (Hestenes) Jacobi SVD of a 3x3 matrix A = U diag(s) V^T, s sorted descending and
 * non-negative, U and V orthogonal.  Stands in for Eigen::JacobiSVD inside igl::polar_svd
 * (extern/libigl/include/igl/polar_svd.cpp:36-64).  W = U m U^T and the closest rotation do not
 * depend on which valid SVD is returned, so any accurate SVD reproduces the reference. */
static void svd3(double A[3][3], double U[3][3], double s[3], double Vm[3][3]) {
  double a[3][3];
  memcpy(a, A, sizeof a);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Vm[i][j] = (i == j);
  static const int P[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int sweep = 0; sweep < 40; sweep++) {
    int rotated = 0;
    for (int pq = 0; pq < 3; pq++) {
      int p = P[pq][0], q = P[pq][1];
      double al = 0, be = 0, ga = 0;
      for (int i = 0; i < 3; i++) {
        al += a[i][p] * a[i][p];
        be += a[i][q] * a[i][q];
        ga += a[i][p] * a[i][q];
      }
      if (ga == 0 || fabs(ga) <= 1e-15 * sqrt(al * be)) continue;
      rotated = 1;
      double zeta = (be - al) / (2 * ga);
      double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1 + zeta * zeta));
      double c = 1 / sqrt(1 + t * t), sn = c * t;
      for (int i = 0; i < 3; i++) {
        double x = a[i][p], y = a[i][q];
        a[i][p] = c * x - sn * y;
        a[i][q] = sn * x + c * y;
        x = Vm[i][p]; y = Vm[i][q];
        Vm[i][p] = c * x - sn * y;
        Vm[i][q] = sn * x + c * y;
      }
    }
    if (!rotated) break;
  }
  double nrm[3];
  for (int j = 0; j < 3; j++) nrm[j] = sqrt(a[0][j] * a[0][j] + a[1][j] * a[1][j] + a[2][j] * a[2][j]);
  int ord[3] = {0, 1, 2};
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (nrm[ord[j]] > nrm[ord[i]]) { int tmp = ord[i]; ord[i] = ord[j]; ord[j] = tmp; }
  double as[3][3], vs[3][3];
  for (int j = 0; j < 3; j++) {
    s[j] = nrm[ord[j]];
    for (int i = 0; i < 3; i++) { as[i][j] = a[i][ord[j]]; vs[i][j] = Vm[i][ord[j]]; }
  }
  memcpy(Vm, vs, sizeof vs);
  /* U columns: normalised, re-orthogonalised; missing directions completed. */
  double u0[3], u1[3], u2[3];
  if (s[0] > 0) { for (int i = 0; i < 3; i++) u0[i] = as[i][0] / s[0]; }
  else { u0[0] = 1; u0[1] = 0; u0[2] = 0; }
  for (int i = 0; i < 3; i++) u1[i] = as[i][1];
  double pr = dot3(u1, u0);
  for (int i = 0; i < 3; i++) u1[i] -= pr * u0[i];
  double l1 = norm3(u1);
  if (l1 > 1e-300 && s[1] > 0) {
    for (int i = 0; i < 3; i++) u1[i] /= l1;
  } else { /* any unit vector orthogonal to u0 */
    double e[3] = {0, 0, 0};
    int m = (fabs(u0[0]) <= fabs(u0[1]) && fabs(u0[0]) <= fabs(u0[2])) ? 0 : (fabs(u0[1]) <= fabs(u0[2]) ? 1 : 2);
    e[m] = 1;
    double pe = dot3(e, u0);
    for (int i = 0; i < 3; i++) u1[i] = e[i] - pe * u0[i];
    l1 = norm3(u1);
    for (int i = 0; i < 3; i++) u1[i] /= l1;
  }
  cross3(u0, u1, u2);
  double a2[3] = {as[0][2], as[1][2], as[2][2]};
  if (dot3(a2, u2) < 0) for (int i = 0; i < 3; i++) u2[i] = -u2[i];
  for (int i = 0; i < 3; i++) { U[i][0] = u0[i]; U[i][1] = u1[i]; U[i][2] = u2[i]; }
}

static void matmul3(double A[3][3], double B[3][3], double C[3][3]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}
static void matmul3T(double A[3][3], double B[3][3], double C[3][3]) { /* A * B^T */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) C[i][j] = A[i][0] * B[j][0] + A[i][1] * B[j][1] + A[i][2] * B[j][2];
}

/* igl::polar_svd: R = U V^T with the reflection moved to the smallest singular direction. */
static void polar_svd3(double J[3][3], double R[3][3], double U[3][3], double s[3], double Vm[3][3]) {
  svd3(J, U, s, Vm);
  matmul3T(U, Vm, R);
  if (det3m(R) < 0) {
    for (int i = 0; i < 3; i++) Vm[i][2] = -Vm[i][2];
    matmul3T(U, Vm, R);
  }
}

/* ------------------------------------------------------------------ SLIM state */
typedef struct slim_state {
  const orc_slim_problem *p;
  int64_t nv, nt, n;     /* vertices, tets, unknowns (3nv + nL) */
  double *Dg;            /* nt x 4 x 3 */
  double M, mesh_area, proximal_p;
  /* CSR pattern */
  int64_t *nbr_ptr; int32_t *nbr;   /* per-vertex sorted neighbour lists (includes itself) */
  int64_t *rowptr; int32_t *col; double *val;
  int64_t *curve_ptr; int32_t *curve_ids; /* per vertex: curve entries i with ids_L[i]==v */
  int32_t *tet_slot;     /* nt x 4 x 4: position of v_k in nbr(v_j) */
  double *W;             /* nt x 9 (row-major W) */
  double *R;             /* nt x 9 (row-major R) */
  double *rhs;
  double *a_L;
} slim_state;

static int cmp_i32(const void *x, const void *y) {
  int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
  return (a > b) - (a < b);
}

static int64_t find_pos(const int32_t *arr, int64_t n, int32_t key) {
  int64_t lo = 0, hi = n - 1;
  while (lo <= hi) {
    int64_t mid = (lo + hi) / 2;
    if (arr[mid] == key) return mid;
    if (arr[mid] < key) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

static void build_pattern(slim_state *S) {
  const orc_slim_problem *p = S->p;
  int64_t nv = S->nv, nh = p->nh;
  /* vertex -> hex incidence */
  int64_t *cnt = (int64_t *)calloc(nv + 1, sizeof(int64_t));
  for (int64_t h = 0; h < nh; h++)
    for (int c = 0; c < 8; c++) cnt[p->H[8 * h + c] + 1]++;
  for (int64_t v = 0; v < nv; v++) cnt[v + 1] += cnt[v];
  int32_t *inc = (int32_t *)malloc(sizeof(int32_t) * (cnt[nv] > 0 ? cnt[nv] : 1));
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (nv > 0 ? nv : 1));
  for (int64_t v = 0; v < nv; v++) fill[v] = cnt[v];
  for (int64_t h = 0; h < nh; h++)
    for (int c = 0; c < 8; c++) inc[fill[p->H[8 * h + c]]++] = (int32_t)h;
  /* neighbour lists */
  S->nbr_ptr = (int64_t *)calloc(nv + 1, sizeof(int64_t));
  int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * 8 * 64);
  int32_t **lists = (int32_t **)malloc(sizeof(int32_t *) * (nv > 0 ? nv : 1));
  int64_t total = 0;
  for (int64_t v = 0; v < nv; v++) {
    int64_t m = 0, nin = cnt[v + 1] - cnt[v];
    int32_t *buf = nin * 8 <= 512 ? tmp : (int32_t *)malloc(sizeof(int32_t) * nin * 8 + 8);
    buf[m++] = (int32_t)v;
    for (int64_t e = cnt[v]; e < cnt[v + 1]; e++)
      for (int c = 0; c < 8; c++) buf[m++] = (int32_t)p->H[8 * (int64_t)inc[e] + c];
    qsort(buf, m, sizeof(int32_t), cmp_i32);
    int64_t u = 0;
    for (int64_t i = 0; i < m; i++)
      if (u == 0 || buf[i] != buf[u - 1]) buf[u++] = buf[i];
    lists[v] = (int32_t *)malloc(sizeof(int32_t) * u);
    memcpy(lists[v], buf, sizeof(int32_t) * u);
    S->nbr_ptr[v + 1] = S->nbr_ptr[v] + u;
    total += u;
    if (buf != tmp) free(buf);
  }
  S->nbr = (int32_t *)malloc(sizeof(int32_t) * (total > 0 ? total : 1));
  for (int64_t v = 0; v < nv; v++) {
    memcpy(S->nbr + S->nbr_ptr[v], lists[v], sizeof(int32_t) * (S->nbr_ptr[v + 1] - S->nbr_ptr[v]));
    free(lists[v]);
  }
  free(lists); free(tmp); free(inc); free(fill); free(cnt);
  /* curve entries per vertex */
  int64_t nL = p->nL;
  S->curve_ptr = (int64_t *)calloc(nv + 1, sizeof(int64_t));
  for (int64_t i = 0; i < nL; i++) S->curve_ptr[p->ids_L[i] + 1]++;
  for (int64_t v = 0; v < nv; v++) S->curve_ptr[v + 1] += S->curve_ptr[v];
  S->curve_ids = (int32_t *)malloc(sizeof(int32_t) * (nL > 0 ? nL : 1));
  int64_t *cf = (int64_t *)malloc(sizeof(int64_t) * (nv > 0 ? nv : 1));
  for (int64_t v = 0; v < nv; v++) cf[v] = S->curve_ptr[v];
  for (int64_t i = 0; i < nL; i++) S->curve_ids[cf[p->ids_L[i]]++] = (int32_t)i;
  free(cf);
  /* rows */
  int64_t n = S->n;
  S->rowptr = (int64_t *)calloc(n + 1, sizeof(int64_t));
  for (int b = 0; b < 3; b++)
    for (int64_t v = 0; v < nv; v++) {
      int64_t deg = S->nbr_ptr[v + 1] - S->nbr_ptr[v];
      S->rowptr[b * nv + v + 1] = 3 * deg + (S->curve_ptr[v + 1] - S->curve_ptr[v]);
    }
  for (int64_t i = 0; i < nL; i++) S->rowptr[3 * nv + i + 1] = 4;
  for (int64_t r = 0; r < n; r++) S->rowptr[r + 1] += S->rowptr[r];
  S->col = (int32_t *)malloc(sizeof(int32_t) * (S->rowptr[n] > 0 ? S->rowptr[n] : 1));
  S->val = (double *)calloc(S->rowptr[n] > 0 ? S->rowptr[n] : 1, sizeof(double));
  for (int b = 0; b < 3; b++)
    for (int64_t v = 0; v < nv; v++) {
      int64_t r = b * nv + v, o = S->rowptr[r];
      int64_t deg = S->nbr_ptr[v + 1] - S->nbr_ptr[v];
      for (int bb = 0; bb < 3; bb++)
        for (int64_t e = 0; e < deg; e++) S->col[o++] = (int32_t)(bb * nv + S->nbr[S->nbr_ptr[v] + e]);
      for (int64_t e = S->curve_ptr[v]; e < S->curve_ptr[v + 1]; e++) S->col[o++] = (int32_t)(3 * nv + S->curve_ids[e]);
    }
  for (int64_t i = 0; i < nL; i++) {
    int64_t o = S->rowptr[3 * nv + i];
    int32_t v = p->ids_L[i];
    for (int b = 0; b < 3; b++) S->col[o++] = (int32_t)(b * nv + v);
    S->col[o++] = (int32_t)(3 * nv + i);
  }
  /* tet slots */
  S->tet_slot = (int32_t *)malloc(sizeof(int32_t) * 16 * (S->nt > 0 ? S->nt : 1));
  for (int64_t t = 0; t < S->nt; t++) {
    const uint32_t *hv = p->H + 8 * (t / 8);
    int k = (int)(t % 8);
    for (int j = 0; j < 4; j++) {
      int32_t vj = (int32_t)hv[HEX_TET[k][j]];
      const int32_t *lst = S->nbr + S->nbr_ptr[vj];
      int64_t deg = S->nbr_ptr[vj + 1] - S->nbr_ptr[vj];
      for (int kk = 0; kk < 4; kk++)
        S->tet_slot[t * 16 + j * 4 + kk] = (int32_t)find_pos(lst, deg, (int32_t)hv[HEX_TET[k][kk]]);
    }
  }
}

/* Adds v to L(row, col) where col must be present in the row pattern. */
static void L_add(slim_state *S, int64_t row, int64_t col, double v) {
  int64_t lo = S->rowptr[row], hi = S->rowptr[row + 1] - 1;
  while (lo <= hi) {
    int64_t mid = (lo + hi) / 2;
    if (S->col[mid] == col) { S->val[mid] += v; return; }
    if (S->col[mid] < col) lo = mid + 1; else hi = mid - 1;
  }
  abort(); /* pattern bug */
}

/* compute_jacobians (slim_m.cpp:84-106) for one tet: J[b][c] = D_c * u_b */
static void tet_jacobian(const slim_state *S, int64_t t, const double *X, double J[3][3]) {
  const uint32_t *hv = S->p->H + 8 * (t / 8);
  int k = (int)(t % 8);
  for (int b = 0; b < 3; b++)
    for (int c = 0; c < 3; c++) J[b][c] = 0;
  for (int j = 0; j < 4; j++) {
    const double *x = X + 3 * (int64_t)hv[HEX_TET[k][j]];
    const double *g = S->Dg + (t * 4 + j) * 3;
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 3; c++) J[b][c] += g[c] * x[b];
  }
}

/* per-tet energy value (compute_energy_with_jacobians 3-D branch, slim_m.cpp:850-912) */
static double tet_energy(int type, double expf_, double J[3][3]) {
  double R[3][3], U[3][3], s[3], Vm[3][3];
  polar_svd3(J, R, U, s, Vm);
  double s1 = s[0], s2 = s[1], s3 = s[2];
  switch (type) {
    case ORC_ARAP: return pow(s1 - 1, 2) + pow(s2 - 1, 2) + pow(s3 - 1, 2);
    case ORC_SYMMETRIC_DIRICHLET:
      return pow(s1, 2) + pow(s1, -2) + pow(s2, 2) + pow(s2, -2) + pow(s3, 2) + pow(s3, -2);
    case ORC_EXP_SYMMETRIC_DIRICHLET:
      return exp(expf_ * (pow(s1, 2) + pow(s1, -2) + pow(s2, 2) + pow(s2, -2) + pow(s3, 2) + pow(s3, -2)));
    case ORC_LOG_ARAP: return pow(log(s1), 2) + pow(log(fabs(s2)), 2) + pow(log(fabs(s3)), 2);
    case ORC_CONFORMAL:
      return (pow(s1, 2) + pow(s2, 2) + pow(s3, 2)) / (3 * pow(s1 * s2 * s3, 2. / 3.));
    case ORC_EXP_CONFORMAL:
      return exp((pow(s1, 2) + pow(s2, 2) + pow(s3, 2)) / (3 * pow(s1 * s2 * s3, 2. / 3.)));
  }
  return NAN;
}

/* compute_soft_const_energy (slim_m.cpp:735-790), feature and projection branches. */
static double soft_energy(const orc_slim_problem *p, const double *X, const double *a_L) {
  double e = 0;
  if (p->projection)
    for (int64_t i = 0; i < p->nB; i++) {
      const double *x = X + 3 * (int64_t)p->b[i];
      double d0 = p->bc[3 * i] - x[0], d1 = p->bc[3 * i + 1] - x[1], d2 = p->bc[3 * i + 2] - x[2];
      e += p->lamda_projection * (d0 * d0 + d1 * d1 + d2 * d2);
    }
  for (int64_t i = 0; i < p->nC; i++) {
    const double *x = X + 3 * (int64_t)p->ids_C[i];
    double d0 = p->C[3 * i] - x[0], d1 = p->C[3 * i + 1] - x[1], d2 = p->C[3 * i + 2] - x[2];
    e += p->lamda_C * (d0 * d0 + d1 * d1 + d2 * d2);
  }
  for (int64_t i = 0; i < p->nT; i++) {
    const double *x = X + 3 * (int64_t)p->ids_T[i];
    const double *nn = p->normal_T + 3 * i;
    double ad = nn[0] * x[0] + nn[1] * x[1] + nn[2] * x[2] - p->dis_T[i];
    e += p->lamda_T * ad * ad;
  }
  for (int64_t i = 0; i < p->nL; i++) {
    const double *x = X + 3 * (int64_t)p->ids_L[i];
    double q = 0;
    for (int d = 0; d < 3; d++) {
      double r = x[d] - a_L[i] * p->Axa_L[3 * i + d] - p->origin_L[3 * i + d];
      q += r * r;
    }
    e += p->lamda_L * q;
  }
  return e;
}

static double energy_total(const slim_state *S, const double *X, const double *a_L, double *E_tet,
                           double *eq, double *es) {
  double e = 0;
  for (int64_t t = 0; t < S->nt; t++) {
    double J[3][3];
    tet_jacobian(S, t, X, J);
    double et = S->M * tet_energy(S->p->energy, S->p->exp_factor, J);
    if (E_tet) E_tet[t] = et;
    e += et;
  }
  double s = soft_energy(S->p, X, a_L);
  if (eq) *eq = e;
  if (es) *es = s;
  return e + s;
}

/* update_weights_and_closest_rotations, 3-D branch (slim_m.cpp:230-378) */
static void local_step(slim_state *S, const double *X) {
  const double eps = 1e-8;
  const double sqrt_2 = sqrt(2);
  double exp_f = S->p->exp_factor;
  for (int64_t t = 0; t < S->nt; t++) {
    double J[3][3], R[3][3], U[3][3], s[3], Vm[3][3], m[3];
    tet_jacobian(S, t, X, J);
    polar_svd3(J, R, U, s, Vm);
    double s1 = s[0], s2 = s[1], s3 = s[2];
    switch (S->p->energy) {
      case ORC_ARAP: m[0] = m[1] = m[2] = 1; break;
      case ORC_LOG_ARAP: {
        double g1 = 2 * (log(s1) / s1), g2 = 2 * (log(s2) / s2), g3 = 2 * (log(s3) / s3);
        m[0] = sqrt(g1 / (2 * (s1 - 1))); m[1] = sqrt(g2 / (2 * (s2 - 1))); m[2] = sqrt(g3 / (2 * (s3 - 1)));
        break;
      }
      case ORC_SYMMETRIC_DIRICHLET: {
        double g1 = 2 * (s1 - pow(s1, -3)), g2 = 2 * (s2 - pow(s2, -3)), g3 = 2 * (s3 - pow(s3, -3));
        m[0] = sqrt(g1 / (2 * (s1 - 1))); m[1] = sqrt(g2 / (2 * (s2 - 1))); m[2] = sqrt(g3 / (2 * (s3 - 1)));
        break;
      }
      case ORC_EXP_SYMMETRIC_DIRICHLET: {
        double g1 = 2 * (s1 - pow(s1, -3)), g2 = 2 * (s2 - pow(s2, -3)), g3 = 2 * (s3 - pow(s3, -3));
        double in_exp = exp_f * (pow(s1, 2) + pow(s1, -2) + pow(s2, 2) + pow(s2, -2) + pow(s3, 2) + pow(s3, -2));
        double et = exp(in_exp);
        g1 *= et * exp_f; g2 *= et * exp_f; g3 *= et * exp_f;
        m[0] = sqrt(g1 / (2 * (s1 - 1))); m[1] = sqrt(g2 / (2 * (s2 - 1))); m[2] = sqrt(g3 / (2 * (s3 - 1)));
        break;
      }
      case ORC_CONFORMAL:
      case ORC_EXP_CONFORMAL: {
        double cd = 9 * (pow(s1 * s2 * s3, 5. / 3.));
        double g1 = (-2 * s2 * s3 * (pow(s2, 2) + pow(s3, 2) - 2 * pow(s1, 2))) / cd;
        double g2 = (-2 * s1 * s3 * (pow(s1, 2) + pow(s3, 2) - 2 * pow(s2, 2))) / cd;
        double g3 = (-2 * s1 * s2 * (pow(s1, 2) + pow(s2, 2) - 2 * pow(s3, 2))) / cd;
        double cs = sqrt(pow(s1, 2) + pow(s3, 2)) / sqrt_2;
        if (S->p->energy == ORC_EXP_CONFORMAL) {
          double in_exp = exp_f * ((pow(s1, 2) + pow(s2, 2) + pow(s3, 2)) / (3 * pow((s1 * s2 * s3), 2. / 3)));
          double et = exp(in_exp);
          g1 *= et * exp_f; g2 *= et * exp_f; g3 *= et * exp_f;
        }
        m[0] = sqrt(g1 / (2 * (s1 - cs))); m[1] = sqrt(g2 / (2 * (s2 - cs))); m[2] = sqrt(g3 / (2 * (s3 - cs)));
        double Ud[3][3];
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) Ud[i][j] = U[i][j] * cs;
        matmul3T(Ud, Vm, R);
        break;
      }
      default: m[0] = m[1] = m[2] = 1;
    }
    if (fabs(s1 - 1) < eps) m[0] = 1;
    if (fabs(s2 - 1) < eps) m[1] = 1;
    if (fabs(s3 - 1) < eps) m[2] = 1;
    double *W = S->W + 9 * t, *Rt = S->R + 9 * t;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        W[3 * i + j] = U[i][0] * m[0] * U[j][0] + U[i][1] * m[1] * U[j][1] + U[i][2] * m[2] * U[j][2];
        Rt[3 * i + j] = R[i][j];
      }
  }
}

/* build_linear_system + buildA + buildRhs + add_soft_constraints (slim_m.cpp:568-714,
 * 918-1092), assembled directly into the CSR pattern. */
static void build_system(slim_state *S, const double *Vo) {
  const orc_slim_problem *p = S->p;
  int64_t nv = S->nv, n3 = 3 * nv;
  memset(S->val, 0, sizeof(double) * S->rowptr[S->n]);
  memset(S->rhs, 0, sizeof(double) * S->n);
  for (int64_t t = 0; t < S->nt; t++) {
    const uint32_t *hv = p->H + 8 * (t / 8);
    int k = (int)(t % 8);
    const double *W = S->W + 9 * t, *R = S->R + 9 * t;
    double C[3][3], F[3][3], CR[3][3];
    for (int b = 0; b < 3; b++)
      for (int bb = 0; bb < 3; bb++)
        C[b][bb] = S->M * (W[0 * 3 + b] * W[0 * 3 + bb] + W[1 * 3 + b] * W[1 * 3 + bb] + W[2 * 3 + b] * W[2 * 3 + bb]);
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) F[a][c] = W[3 * a + 0] * R[0 * 3 + c] + W[3 * a + 1] * R[1 * 3 + c] + W[3 * a + 2] * R[2 * 3 + c];
    /* CR = M W^T F */
    for (int b = 0; b < 3; b++)
      for (int c = 0; c < 3; c++) CR[b][c] = S->M * (W[0 * 3 + b] * F[0][c] + W[1 * 3 + b] * F[1][c] + W[2 * 3 + b] * F[2][c]);
    const double *g = S->Dg + t * 12;
    for (int j = 0; j < 4; j++) {
      int32_t vj = (int32_t)hv[HEX_TET[k][j]];
      int64_t deg = S->nbr_ptr[vj + 1] - S->nbr_ptr[vj];
      for (int kk = 0; kk < 4; kk++) {
        double gjk = dot3(g + 3 * j, g + 3 * kk);
        int32_t pos = S->tet_slot[t * 16 + j * 4 + kk];
        for (int b = 0; b < 3; b++) {
          int64_t base = S->rowptr[b * nv + vj];
          for (int bb = 0; bb < 3; bb++) S->val[base + bb * deg + pos] += C[b][bb] * gjk;
        }
      }
      for (int b = 0; b < 3; b++) S->rhs[b * nv + vj] += dot3(g + 3 * j, CR[b]);
    }
  }
  /* proximal term */
  for (int b = 0; b < 3; b++)
    for (int64_t v = 0; v < nv; v++) {
      L_add(S, b * nv + v, b * nv + v, S->proximal_p);
      S->rhs[b * nv + v] += S->proximal_p * Vo[3 * v + b];
    }
  if (p->projection)
    for (int d = 0; d < 3; d++)
      for (int64_t i = 0; i < p->nB; i++) {
        int64_t r = d * nv + p->b[i];
        S->rhs[r] += p->lamda_projection * p->bc[3 * i + d];
        L_add(S, r, r, p->lamda_projection);
      }
  for (int d = 0; d < 3; d++)
    for (int64_t i = 0; i < p->nC; i++) {
      int64_t r = d * nv + p->ids_C[i];
      S->rhs[r] += p->lamda_C * p->C[3 * i + d];
      L_add(S, r, r, p->lamda_C);
    }
  for (int64_t i = 0; i < p->nT; i++) {
    int32_t v = p->ids_T[i];
    const double *nn = p->normal_T + 3 * i;
    for (int d = 0; d < 3; d++) {
      for (int dd = 0; dd < 3; dd++) L_add(S, d * nv + v, dd * nv + v, p->lamda_T * nn[d] * nn[dd]);
      S->rhs[d * nv + v] += p->lamda_T * nn[d] * p->dis_T[i];
    }
  }
  for (int64_t i = 0; i < p->nL; i++) {
    int32_t v = p->ids_L[i];
    const double *ax = p->Axa_L + 3 * i, *og = p->origin_L + 3 * i;
    double aa = 0, ao = 0;
    for (int d = 0; d < 3; d++) {
      L_add(S, d * nv + v, d * nv + v, p->lamda_L);
      L_add(S, d * nv + v, n3 + i, -p->lamda_L * ax[d]);
      L_add(S, n3 + i, d * nv + v, -p->lamda_L * ax[d]);
      S->rhs[d * nv + v] += p->lamda_L * og[d];
      aa += ax[d] * ax[d];
      ao += -ax[d] * og[d];
    }
    L_add(S, n3 + i, n3 + i, p->lamda_L * aa);
    S->rhs[n3 + i] += p->lamda_L * ao;
  }
}

static void spmv(const slim_state *S, const double *x, double *y) {
  for (int64_t r = 0; r < S->n; r++) {
    double acc = 0;
    for (int64_t e = S->rowptr[r]; e < S->rowptr[r + 1]; e++) acc += S->val[e] * x[S->col[e]];
    y[r] = acc;
  }
}
static double vdot(const double *a, const double *b, int64_t n) {
  double s = 0;
  for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* Eigen::ConjugateGradient<Lower|Upper> with the DiagonalPreconditioner
 * (extern/eigen/Eigen/src/IterativeLinearSolvers/ConjugateGradient.h:39-80,
 *  BasicPreconditioners.h:69-71), tol 1e-8, 20 iterations (slim_m.cpp:493-496). */
static int cg_solve(const slim_state *S, const double *b, double *x, double tol, int max_iter, double *err) {
  int64_t n = S->n;
  double *invd = (double *)malloc(sizeof(double) * n), *r = (double *)malloc(sizeof(double) * n);
  double *pp = (double *)malloc(sizeof(double) * n), *z = (double *)malloc(sizeof(double) * n);
  double *tmp = (double *)malloc(sizeof(double) * n);
  for (int64_t i = 0; i < n; i++) {
    invd[i] = 0;
    for (int64_t e = S->rowptr[i]; e < S->rowptr[i + 1]; e++)
      if (S->col[e] == i) { invd[i] = 1.0 / S->val[e]; break; }
  }
  int iters = 0;
  spmv(S, x, tmp);
  for (int64_t i = 0; i < n; i++) r[i] = b[i] - tmp[i];
  double rhsNorm2 = vdot(b, b, n);
  if (rhsNorm2 == 0) {
    memset(x, 0, sizeof(double) * n);
    *err = 0;
    goto done;
  }
  {
    double threshold = tol * tol * rhsNorm2;
    double rn2 = vdot(r, r, n);
    if (rn2 < threshold) { *err = sqrt(rn2 / rhsNorm2); goto done; }
    for (int64_t i = 0; i < n; i++) pp[i] = invd[i] * r[i];
    double absNew = vdot(r, pp, n);
    int i = 0;
    while (i < max_iter) {
      spmv(S, pp, tmp);
      double alpha = absNew / vdot(pp, tmp, n);
      for (int64_t j = 0; j < n; j++) x[j] += alpha * pp[j];
      for (int64_t j = 0; j < n; j++) r[j] -= alpha * tmp[j];
      rn2 = vdot(r, r, n);
      if (rn2 < threshold) break;
      for (int64_t j = 0; j < n; j++) z[j] = invd[j] * r[j];
      double absOld = absNew;
      absNew = vdot(r, z, n);
      double beta = absNew / absOld;
      for (int64_t j = 0; j < n; j++) pp[j] = z[j] + beta * pp[j];
      i++;
    }
    *err = sqrt(rn2 / rhsNorm2);
    iters = i;
  }
done:
  free(invd); free(r); free(pp); free(z); free(tmp);
  return iters;
}

/* ------------------------------------------------------------------ flip-avoiding line search */
/* Cubic x^3 + a x^2 + b x + c = 0 by the trigonometric / Cardano method as used by
 * flip_avoiding::SolveP3 (flip_avoiding_line_search.cpp:24-61); returns the number of real
 * roots in the same convention (1: x[0] real, x[1] +- i x[2]). */
static int solve_p3(double x[3], double a, double b, double c) {
  double a2 = a * a;
  double q = (a2 - 3 * b) / 9;
  double r = (a * (2 * a2 - 9 * b) + 27 * c) / 54;
  double r2 = r * r, q3 = q * q * q;
  if (r2 < q3) {
    double t = r / sqrt(q3);
    if (t < -1) t = -1;
    if (t > 1) t = 1;
    t = acos(t);
    a /= 3;
    q = -2 * sqrt(q);
    x[0] = q * cos(t / 3) - a;
    x[1] = q * cos((t + (2 * M_PI)) / 3) - a;
    x[2] = q * cos((t - (2 * M_PI)) / 3) - a;
    return 3;
  } else {
    double A = -pow(fabs(r) + sqrt(r2 - q3), 1. / 3);
    if (r < 0) A = -A;
    double B = (A == 0) ? 0 : q / A;
    a /= 3;
    x[0] = (A + B) - a;
    x[1] = -0.5 * (A + B) - a;
    x[2] = 0.5 * sqrt(3.) * (A - B);
    if (fabs(x[2]) < 1e-14) { x[2] = x[1]; return 2; }
    return 1;
  }
}

/* get_smallest_pos_quad_zero (flip_avoiding_line_search.cpp:63-109) */
static double smallest_pos_quad_zero(double a, double b, double c) {
  double t1, t2;
  if (fabs(a) > 1.0e-10) {
    double delta_in = b * b - 4 * a * c;
    if (delta_in <= 0) return INFINITY;
    double delta = sqrt(delta_in);
    if (b >= 0) {
      double bd = -b - delta;
      t1 = 2 * c / bd;
      t2 = bd / (2 * a);
    } else {
      double bd = -b + delta;
      t1 = bd / (2 * a);
      t2 = (2 * c) / bd;
    }
    if (a < 0) { double tt = t1; t1 = t2; t2 = tt; }
    if (t1 > 0) return t2 > 0 ? t2 : t1;
    return INFINITY;
  }
  if (b == 0) return INFINITY;
  t1 = -c / b;
  return t1 > 0 ? t1 : INFINITY;
}

/* get_min_pos_root_3D (flip_avoiding_line_search.cpp:177-271).  The coefficients of
 * det[[a+t da,1],[b+t db,1],[c+t dc,1],[d+t dd,1]] = -det(E + t D) with E the edge matrix
 * [b-a, c-a, d-a] and D the matching direction differences. */
static double min_pos_root_3d(const double *pa, const double *pb, const double *pc, const double *pd,
                              const double *da, const double *db, const double *dc, const double *dd) {
  double E[3][3], D[3][3];
  for (int r = 0; r < 3; r++) {
    E[r][0] = pb[r] - pa[r]; E[r][1] = pc[r] - pa[r]; E[r][2] = pd[r] - pa[r];
    D[r][0] = db[r] - da[r]; D[r][1] = dc[r] - da[r]; D[r][2] = dd[r] - da[r];
  }
  double M[3][3];
  /* c3 = det D, c0 = det E, c1 / c2 by column replacement */
  double c3 = det3m(D), c0 = det3m(E), c1 = 0, c2 = 0;
  for (int col = 0; col < 3; col++) {
    for (int r = 0; r < 3; r++)
      for (int cc = 0; cc < 3; cc++) M[r][cc] = (cc == col) ? D[r][cc] : E[r][cc];
    c1 += det3m(M);
    for (int r = 0; r < 3; r++)
      for (int cc = 0; cc < 3; cc++) M[r][cc] = (cc == col) ? E[r][cc] : D[r][cc];
    c2 += det3m(M);
  }
  double a = -c3, b = -c2, c = -c1, d = -c0;
  if (fabs(a) <= 1.e-10) return smallest_pos_quad_zero(b, c, d);
  b /= a; c /= a; d /= a;
  double res[3];
  int nr = solve_p3(res, b, c, d);
  switch (nr) {
    case 1: return (res[0] >= 0) ? res[0] : INFINITY;
    case 2: {
      double mx = res[0] > res[1] ? res[0] : res[1], mn = res[0] < res[1] ? res[0] : res[1];
      if (mn > 0) return mn;
      if (mx > 0) return mx;
      return INFINITY;
    }
    default: {
      for (int i = 0; i < 3; i++)
        for (int j = i + 1; j < 3; j++)
          if (res[j] < res[i]) { double tt = res[i]; res[i] = res[j]; res[j] = tt; }
      if (res[0] > 0) return res[0];
      if (res[1] > 0) return res[1];
      if (res[2] > 0) return res[2];
      return INFINITY;
    }
  }
}

double orc_max_step(int64_t nv, const double *X, const double *Dir, int64_t nh, const uint32_t *H) {
  (void)nv;
  double mx = INFINITY;
  for (int64_t t = 0; t < 8 * nh; t++) {
    const uint32_t *hv = H + 8 * (t / 8);
    int k = (int)(t % 8);
    int64_t i0 = hv[HEX_TET[k][0]], i1 = hv[HEX_TET[k][1]], i2 = hv[HEX_TET[k][2]], i3 = hv[HEX_TET[k][3]];
    double r = min_pos_root_3d(X + 3 * i0, X + 3 * i1, X + 3 * i2, X + 3 * i3, Dir + 3 * i0, Dir + 3 * i1,
                               Dir + 3 * i2, Dir + 3 * i3);
    if (r < mx) mx = r;
  }
  return mx;
}

/* ------------------------------------------------------------------ SLIM driver */
static int slim_init(slim_state *S, const orc_slim_problem *p) {
  memset(S, 0, sizeof *S);
  S->p = p;
  S->nv = p->nv;
  S->nt = 8 * p->nh;
  S->n = 3 * p->nv + p->nL;
  double *RT = (double *)malloc(sizeof(double) * 12 * (S->nt > 0 ? S->nt : 1));
  orc_reference_mesh(p->V, p->nh, p->H, p->h_flag, p->cube, RT);
  S->Dg = (double *)malloc(sizeof(double) * 12 * (S->nt > 0 ? S->nt : 1));
  orc_grad_ref(p->V, p->nh, p->H, RT, S->Dg);
  free(RT);
  /* slim_precompute (slim_m.cpp:1095-1132) */
  S->M = p->weight_opt;
  S->mesh_area = p->weight_opt * (double)S->nt;
  S->proximal_p = 0.00001 * p->weight_opt;
  S->W = (double *)malloc(sizeof(double) * 9 * (S->nt > 0 ? S->nt : 1));
  S->R = (double *)malloc(sizeof(double) * 9 * (S->nt > 0 ? S->nt : 1));
  S->rhs = (double *)malloc(sizeof(double) * (S->n > 0 ? S->n : 1));
  S->a_L = (double *)calloc(p->nL > 0 ? p->nL : 1, sizeof(double));
  build_pattern(S);
  return 0;
}

static void slim_free(slim_state *S) {
  free(S->Dg); free(S->nbr_ptr); free(S->nbr); free(S->rowptr); free(S->col); free(S->val);
  free(S->curve_ptr); free(S->curve_ids); free(S->tet_slot); free(S->W); free(S->R); free(S->rhs);
  free(S->a_L);
}

int orc_slim_m_opt(const orc_slim_problem *p, int iters, double *V_o, double *a_L, orc_slim_result *res) {
  slim_state S;
  slim_init(&S, p);
  int64_t nv = p->nv, n = S.n;
  memcpy(V_o, p->UV, sizeof(double) * 3 * nv);
  double eq = 0, es = 0;
  /* slim_precompute's initial energy (slim_m.cpp:1131); its value is overwritten below. */
  double energy = energy_total(&S, V_o, S.a_L, NULL, &eq, &es) / S.mesh_area;
  double *x = (double *)malloc(sizeof(double) * n), *dest = (double *)malloc(sizeof(double) * 3 * nv);
  double *dir = (double *)malloc(sizeof(double) * 3 * nv), *trial = (double *)malloc(sizeof(double) * 3 * nv);
  orc_slim_result r = {0};
  for (int it = 0; it < iters; it++) {
    /* local step */
    local_step(&S, V_o);
    /* global step */
    build_system(&S, V_o);
    for (int b = 0; b < 3; b++)
      for (int64_t v = 0; v < nv; v++) x[b * nv + v] = V_o[3 * v + b];
    for (int64_t i = 0; i < p->nL; i++) x[3 * nv + i] = 0;
    r.cg_iters = cg_solve(&S, S.rhs, x, 1e-8, 20, &r.cg_error);
    for (int b = 0; b < 3; b++)
      for (int64_t v = 0; v < nv; v++) dest[3 * v + b] = x[b * nv + v];
    for (int64_t i = 0; i < p->nL; i++) S.a_L[i] = x[3 * nv + i];
    /* flip_avoiding_line_search (flip_avoiding_line_search.cpp:302-317) */
    for (int64_t j = 0; j < 3 * nv; j++) dir[j] = dest[j] - V_o[j];
    double min_step = orc_max_step(nv, V_o, dir, p->nh, p->H);
    double step = min_step * 0.8 < 1. ? min_step * 0.8 : 1.;
    r.max_step = step;
    /* igl::line_search (line_search.cpp:10-53) */
    double old_e = energy_total(&S, V_o, S.a_L, NULL, &eq, &es);
    double new_e = old_e;
    int cur = 0, halv = 0;
    while (new_e >= old_e) {
      if (cur > 20) step = 0;
      for (int64_t j = 0; j < 3 * nv; j++) trial[j] = V_o[j] + step * dir[j];
      double ce = energy_total(&S, trial, S.a_L, NULL, &eq, &es);
      if (isnan(ce) || isinf(ce) || ce > old_e) {
        step /= 2;
        halv++;
      } else {
        memcpy(V_o, trial, sizeof(double) * 3 * nv);
        new_e = ce;
        break;
      }
      if (step == 0) break;
      cur++;
    }
    r.step = step;
    r.halvings = halv;
    energy = new_e / S.mesh_area;
  }
  r.energy = energy;
  r.energy_quality = eq;
  r.energy_soft = es;
  if (a_L)
    for (int64_t i = 0; i < p->nL; i++) a_L[i] = S.a_L[i];
  if (res) *res = r;
  free(x); free(dest); free(dir); free(trial);
  slim_free(&S);
  return 0;
}

double orc_slim_energy(const orc_slim_problem *p, const double *X, const double *a_L, double *E_tet,
                       double *eq, double *es) {
  slim_state S;
  memset(&S, 0, sizeof S);
  S.p = p; S.nv = p->nv; S.nt = 8 * p->nh; S.M = p->weight_opt;
  double *RT = (double *)malloc(sizeof(double) * 12 * (S.nt > 0 ? S.nt : 1));
  orc_reference_mesh(p->V, p->nh, p->H, p->h_flag, p->cube, RT);
  S.Dg = (double *)malloc(sizeof(double) * 12 * (S.nt > 0 ? S.nt : 1));
  orc_grad_ref(p->V, p->nh, p->H, RT, S.Dg);
  free(RT);
  double zero = 0;
  double e = energy_total(&S, X, a_L ? a_L : &zero, E_tet, eq, es);
  free(S.Dg);
  return e;
}

/* Analytic gradient of the symmetric Dirichlet energy + soft terms: per tet
 * dE/dJ = 2 M (J - J^{-T} J^{-1} J^{-T}), chained through the frozen operator D. */
void orc_slim_energy_grad(const orc_slim_problem *p, const double *X, const double *a_L, double *G) {
  slim_state S;
  memset(&S, 0, sizeof S);
  S.p = p; S.nv = p->nv; S.nt = 8 * p->nh; S.M = p->weight_opt;
  double *RT = (double *)malloc(sizeof(double) * 12 * (S.nt > 0 ? S.nt : 1));
  orc_reference_mesh(p->V, p->nh, p->H, p->h_flag, p->cube, RT);
  S.Dg = (double *)malloc(sizeof(double) * 12 * (S.nt > 0 ? S.nt : 1));
  orc_grad_ref(p->V, p->nh, p->H, RT, S.Dg);
  free(RT);
  memset(G, 0, sizeof(double) * 3 * p->nv);
  for (int64_t t = 0; t < S.nt; t++) {
    double J[3][3], Ji[3][3], Q[3][3], T1[3][3], T2[3][3];
    tet_jacobian(&S, t, X, J);
    double det = det3m(J);
    /* inverse via adjugate */
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    double JiT[3][3];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) JiT[i][j] = Ji[j][i];
    matmul3(JiT, Ji, T1);
    matmul3(T1, JiT, T2);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Q[i][j] = 2 * S.M * (J[i][j] - T2[i][j]);
    const uint32_t *hv = p->H + 8 * (t / 8);
    int k = (int)(t % 8);
    for (int j = 0; j < 4; j++) {
      const double *g = S.Dg + (t * 4 + j) * 3;
      double *gv = G + 3 * (int64_t)hv[HEX_TET[k][j]];
      for (int b = 0; b < 3; b++) gv[b] += Q[b][0] * g[0] + Q[b][1] * g[1] + Q[b][2] * g[2];
    }
  }
  for (int64_t i = 0; i < p->nC; i++) {
    const double *x = X + 3 * (int64_t)p->ids_C[i];
    double *gv = G + 3 * (int64_t)p->ids_C[i];
    for (int d = 0; d < 3; d++) gv[d] += 2 * p->lamda_C * (x[d] - p->C[3 * i + d]);
  }
  for (int64_t i = 0; i < p->nT; i++) {
    const double *x = X + 3 * (int64_t)p->ids_T[i];
    const double *nn = p->normal_T + 3 * i;
    double ad = nn[0] * x[0] + nn[1] * x[1] + nn[2] * x[2] - p->dis_T[i];
    double *gv = G + 3 * (int64_t)p->ids_T[i];
    for (int d = 0; d < 3; d++) gv[d] += 2 * p->lamda_T * ad * nn[d];
  }
  for (int64_t i = 0; i < p->nL; i++) {
    const double *x = X + 3 * (int64_t)p->ids_L[i];
    double *gv = G + 3 * (int64_t)p->ids_L[i];
    double al = a_L ? a_L[i] : 0;
    for (int d = 0; d < 3; d++) gv[d] += 2 * p->lamda_L * (x[d] - al * p->Axa_L[3 * i + d] - p->origin_L[3 * i + d]);
  }
  free(S.Dg);
}

/* ------------------------------------------------------------------ AABB + projection */
typedef struct tnode { double lo[3], hi[3]; int32_t left, right, prim; } tnode;
struct orc_tree {
  int64_t nv, nf;
  double *V; int32_t *F;
  double *FN, *VN, *EN;   /* face / vertex / edge normals */
  int32_t *EMAP;          /* 3*nf: edge opposite corner c of face f -> unique edge id (f + c*nf) */
  tnode *nodes; int64_t nn;
  int32_t *perm;
};

static double *g_cent; /* build-time centroid scratch */
static int g_axis;
static int cmp_cent(const void *x, const void *y) {
  double a = g_cent[3 * (*(const int32_t *)x) + g_axis], b = g_cent[3 * (*(const int32_t *)y) + g_axis];
  return (a > b) - (a < b);
}

static int32_t tree_build_rec(orc_tree *t, int32_t *ids, int64_t n) {
  int32_t me = (int32_t)t->nn++;
  tnode *nd = &t->nodes[me];
  for (int d = 0; d < 3; d++) { nd->lo[d] = INFINITY; nd->hi[d] = -INFINITY; }
  double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) {
      const double *v = t->V + 3 * (int64_t)t->F[3 * (int64_t)ids[i] + c];
      for (int d = 0; d < 3; d++) {
        if (v[d] < nd->lo[d]) nd->lo[d] = v[d];
        if (v[d] > nd->hi[d]) nd->hi[d] = v[d];
      }
    }
  if (n == 1) { nd->prim = ids[0]; nd->left = nd->right = -1; return me; }
  for (int64_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      double c = g_cent[3 * (int64_t)ids[i] + d];
      if (c < clo[d]) clo[d] = c;
      if (c > chi[d]) chi[d] = c;
    }
  int ax = 0;
  for (int d = 1; d < 3; d++)
    if (chi[d] - clo[d] > chi[ax] - clo[ax]) ax = d;
  g_axis = ax;
  qsort(ids, n, sizeof(int32_t), cmp_cent);
  int64_t h = n / 2;
  nd->prim = -1;
  int32_t l = tree_build_rec(t, ids, h);
  int32_t r = tree_build_rec(t, ids + h, n - h);
  t->nodes[me].left = l;
  t->nodes[me].right = r;
  return me;
}

static int cmp_edge(const void *x, const void *y) {
  const int64_t *a = (const int64_t *)x, *b = (const int64_t *)y;
  return (a[0] > b[0]) - (a[0] < b[0]);
}

orc_tree *orc_tree_build(int64_t nv, const double *TV, int64_t nf, const int32_t *TF) {
  orc_tree *t = (orc_tree *)calloc(1, sizeof(orc_tree));
  t->nv = nv; t->nf = nf;
  t->V = (double *)malloc(sizeof(double) * 3 * (nv > 0 ? nv : 1));
  memcpy(t->V, TV, sizeof(double) * 3 * nv);
  t->F = (int32_t *)malloc(sizeof(int32_t) * 3 * (nf > 0 ? nf : 1));
  memcpy(t->F, TF, sizeof(int32_t) * 3 * nf);
  /* per_face_normals (per_face_normals.cpp:15-40) */
  t->FN = (double *)calloc(3 * (nf > 0 ? nf : 1), sizeof(double));
  for (int64_t f = 0; f < nf; f++) {
    double e1[3], e2[3], n[3];
    const double *p0 = TV + 3 * (int64_t)TF[3 * f], *p1 = TV + 3 * (int64_t)TF[3 * f + 1], *p2 = TV + 3 * (int64_t)TF[3 * f + 2];
    sub3(p1, p0, e1); sub3(p2, p0, e2); cross3(e1, e2, n);
    double r = norm3(n);
    if (r != 0) for (int d = 0; d < 3; d++) t->FN[3 * f + d] = n[d] / r;
  }
  /* per_vertex_normals, angle weighting (per_vertex_normals.cpp, internal_angles.cpp) */
  t->VN = (double *)calloc(3 * (nv > 0 ? nv : 1), sizeof(double));
  for (int64_t f = 0; f < nf; f++) {
    double L[3];
    for (int c = 0; c < 3; c++) {
      double e[3];
      sub3(TV + 3 * (int64_t)TF[3 * f + (c + 1) % 3], TV + 3 * (int64_t)TF[3 * f + (c + 2) % 3], e);
      L[c] = dot3(e, e);
    }
    for (int d = 0; d < 3; d++) {
      double s1 = L[d], s2 = L[(d + 1) % 3], s3 = L[(d + 2) % 3];
      double ang = acos((s3 + s2 - s1) / (2. * sqrt(s3 * s2)));
      for (int k = 0; k < 3; k++) t->VN[3 * (int64_t)TF[3 * f + d] + k] += ang * t->FN[3 * f + k];
    }
  }
  for (int64_t v = 0; v < nv; v++) {
    double r = norm3(t->VN + 3 * v);
    if (r > 0) for (int d = 0; d < 3; d++) t->VN[3 * v + d] /= r;
  }
  /* per_edge_normals, uniform weighting (per_edge_normals.cpp:15-77) */
  int64_t ne3 = 3 * nf;
  int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * 2 * (ne3 > 0 ? ne3 : 1));
  for (int64_t c = 0; c < 3; c++)
    for (int64_t f = 0; f < nf; f++) {
      int64_t a = TF[3 * f + (c + 1) % 3], b = TF[3 * f + (c + 2) % 3];
      if (a > b) { int64_t tt = a; a = b; b = tt; }
      keys[2 * (f + c * nf)] = a * (nv + 1) + b;
      keys[2 * (f + c * nf) + 1] = f + c * nf;
    }
  qsort(keys, ne3, 2 * sizeof(int64_t), cmp_edge);
  t->EMAP = (int32_t *)malloc(sizeof(int32_t) * (ne3 > 0 ? ne3 : 1));
  int64_t ne = 0;
  for (int64_t i = 0; i < ne3; i++) {
    if (i > 0 && keys[2 * i] != keys[2 * (i - 1)]) ne++;
    t->EMAP[keys[2 * i + 1]] = (int32_t)ne;
  }
  if (ne3 > 0) ne++;
  free(keys);
  t->EN = (double *)calloc(3 * (ne > 0 ? ne : 1), sizeof(double));
  for (int64_t f = 0; f < nf; f++)
    for (int c = 0; c < 3; c++)
      for (int d = 0; d < 3; d++) t->EN[3 * (int64_t)t->EMAP[f + c * nf] + d] += t->FN[3 * f + d];
  /* The reference's per_edge_normals stops after the accumulation: edge normals stay
   * unnormalised (the sum of the adjacent face normals), and that length reaches normal_T. */
  /* AABB */
  t->nodes = (tnode *)malloc(sizeof(tnode) * (2 * nf + 1));
  g_cent = (double *)malloc(sizeof(double) * 3 * (nf > 0 ? nf : 1));
  for (int64_t f = 0; f < nf; f++)
    for (int d = 0; d < 3; d++)
      g_cent[3 * f + d] = (TV[3 * (int64_t)TF[3 * f] + d] + TV[3 * (int64_t)TF[3 * f + 1] + d] + TV[3 * (int64_t)TF[3 * f + 2] + d]) / 3;
  int32_t *ids = (int32_t *)malloc(sizeof(int32_t) * (nf > 0 ? nf : 1));
  for (int64_t f = 0; f < nf; f++) ids[f] = (int32_t)f;
  t->nn = 0;
  if (nf > 0) tree_build_rec(t, ids, nf);
  free(ids);
  free(g_cent);
  g_cent = NULL;
  return t;
}

void orc_tree_free(orc_tree *t) {
  if (!t) return;
  free(t->V); free(t->F); free(t->FN); free(t->VN); free(t->EN); free(t->EMAP); free(t->nodes);
  free(t);
}

/* point_simplex_squared_distance, triangle case (Ericson, Real-Time Collision Detection 5.1.5),
 * as used by igl (point_simplex_squared_distance.cpp:25-130). */
static void closest_pt_tri(const double *p, const double *a, const double *b, const double *c, double *out,
                           double *bary) {
  double ab[3], ac[3], ap[3], bp[3], cp[3];
  sub3(b, a, ab); sub3(c, a, ac); sub3(p, a, ap);
  double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) { bary[0] = 1; bary[1] = 0; bary[2] = 0; memcpy(out, a, 24); return; }
  sub3(p, b, bp);
  double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) { bary[0] = 0; bary[1] = 1; bary[2] = 0; memcpy(out, b, 24); return; }
  double vc = d1 * d4 - d3 * d2;
  if (!(a[0] == b[0] && a[1] == b[1] && a[2] == b[2])) {
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
      double v = d1 / (d1 - d3);
      bary[0] = 1 - v; bary[1] = v; bary[2] = 0;
      for (int d = 0; d < 3; d++) out[d] = a[d] + v * ab[d];
      return;
    }
  }
  sub3(p, c, cp);
  double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) { bary[0] = 0; bary[1] = 0; bary[2] = 1; memcpy(out, c, 24); return; }
  double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    double w = d2 / (d2 - d6);
    bary[0] = 1 - w; bary[1] = 0; bary[2] = w;
    for (int d = 0; d < 3; d++) out[d] = a[d] + w * ac[d];
    return;
  }
  double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
    double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    bary[0] = 0; bary[1] = 1 - w; bary[2] = w;
    for (int d = 0; d < 3; d++) out[d] = b[d] + w * (c[d] - b[d]);
    return;
  }
  double denom = 1.0 / (va + vb + vc);
  double v = vb * denom, w = vc * denom;
  bary[0] = 1.0 - v - w; bary[1] = v; bary[2] = w;
  for (int d = 0; d < 3; d++) out[d] = a[d] + ab[d] * v + ac[d] * w;
}

static double box_dist2(const tnode *nd, const double *p) {
  double s = 0;
  for (int d = 0; d < 3; d++) {
    double e = 0;
    if (p[d] < nd->lo[d]) e = nd->lo[d] - p[d];
    else if (p[d] > nd->hi[d]) e = p[d] - nd->hi[d];
    s += e * e;
  }
  return s;
}

static void tree_query(const orc_tree *t, int32_t node, const double *p, double *best, int32_t *bi, double *bc) {
  const tnode *nd = &t->nodes[node];
  if (nd->prim >= 0) {
    const int32_t *f = t->F + 3 * (int64_t)nd->prim;
    double c[3], bary[3], e[3];
    closest_pt_tri(p, t->V + 3 * (int64_t)f[0], t->V + 3 * (int64_t)f[1], t->V + 3 * (int64_t)f[2], c, bary);
    sub3(p, c, e);
    double d2 = dot3(e, e);
    if (d2 < *best) { *best = d2; *bi = nd->prim; memcpy(bc, c, 24); }
    return;
  }
  double dl = box_dist2(&t->nodes[nd->left], p), dr = box_dist2(&t->nodes[nd->right], p);
  if (dl <= dr) {
    if (dl < *best) tree_query(t, nd->left, p, best, bi, bc);
    if (dr < *best) tree_query(t, nd->right, p, best, bi, bc);
  } else {
    if (dr < *best) tree_query(t, nd->right, p, best, bi, bc);
    if (dl < *best) tree_query(t, nd->left, p, best, bi, bc);
  }
}

/* pseudonormal_test (extern/libigl/include/igl/pseudonormal_test.cpp:14-120) */
static void pseudonormal(const orc_tree *t, const double *q, int32_t f, const double *c, double *s, double *n) {
  const double *A = t->V + 3 * (int64_t)t->F[3 * (int64_t)f], *B = t->V + 3 * (int64_t)t->F[3 * (int64_t)f + 1];
  const double *C = t->V + 3 * (int64_t)t->F[3 * (int64_t)f + 2];
  double e1[3], e2[3], x[3];
  sub3(B, A, e1); sub3(C, A, e2); cross3(e1, e2, x);
  double area = norm3(x); /* doublearea */
  const double MIN_DOUBLE_AREA = 1e-4, epsilon = 1e-12;
  const double *nn = NULL;
  if (area > MIN_DOUBLE_AREA) {
    /* barycentric_coordinates (barycentric_coordinates.cpp:58-100) */
    double v0[3], v1[3], v2[3], b[3];
    sub3(B, A, v0); sub3(C, A, v1); sub3(c, A, v2);
    double d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1), d20 = dot3(v2, v0), d21 = dot3(v2, v1);
    double den = d00 * d11 - d01 * d01;
    b[1] = (d11 * d20 - d01 * d21) / den;
    b[2] = (d00 * d21 - d01 * d20) / den;
    b[0] = 1.0 - (b[1] + b[2]);
    int type = (b[0] <= epsilon) + (b[1] <= epsilon) + (b[2] <= epsilon);
    if (type == 2) {
      for (int k = 0; k < 3; k++)
        if (b[k] > epsilon) { nn = t->VN + 3 * (int64_t)t->F[3 * (int64_t)f + k]; break; }
    } else if (type == 1) {
      for (int k = 0; k < 3; k++)
        if (b[k] <= epsilon) { nn = t->EN + 3 * (int64_t)t->EMAP[t->nf * k + f]; break; }
    }
    if (!nn) nn = t->FN + 3 * (int64_t)f;
  } else {
    for (int v = 0; v < 3 && !nn; v++) {
      double d[3];
      sub3(c, t->V + 3 * (int64_t)t->F[3 * (int64_t)f + v], d);
      if (norm3(d) < epsilon) nn = t->VN + 3 * (int64_t)t->F[3 * (int64_t)f + v];
    }
    for (int e = 0; e < 3 && !nn; e++) {
      const double *sp = t->V + 3 * (int64_t)t->F[3 * (int64_t)f + (e + 1) % 3];
      const double *dp = t->V + 3 * (int64_t)t->F[3 * (int64_t)f + (e + 2) % 3];
      /* project_to_line_segment (project_to_line.cpp:57-97, project_to_line_segment.cpp) */
      double dms[3], smp[3];
      sub3(dp, sp, dms); sub3(sp, c, smp);
      double vl = dot3(dms, dms);
      double tt = -dot3(dms, smp) / vl, sq;
      double pr[3], pm[3];
      for (int k = 0; k < 3; k++) pr[k] = (1.0 - tt) * sp[k] + tt * dp[k];
      sub3(c, pr, pm);
      sq = dot3(pm, pm);
      if (tt < 0) { double z[3]; sub3(c, sp, z); sq = dot3(z, z); }
      else if (tt > 1) { double z[3]; sub3(c, dp, z); sq = dot3(z, z); }
      if (sqrt(sq) < epsilon) nn = t->EN + 3 * (int64_t)t->EMAP[t->nf * e + f];
    }
    if (!nn) nn = t->FN + 3 * (int64_t)f;
  }
  memcpy(n, nn, 24);
  double qc[3];
  sub3(q, c, qc);
  *s = (dot3(qc, n) >= 0 ? 1. : -1.);
}

void orc_signed_distance(const orc_tree *t, int64_t np, const double *P, double *S, int32_t *I, double *C,
                         double *N) {
  for (int64_t i = 0; i < np; i++) {
    double best = INFINITY, c[3] = {0, 0, 0}, s = 1, n[3] = {0, 0, 0};
    int32_t bi = -1;
    if (t->nf > 0) tree_query(t, 0, P + 3 * i, &best, &bi, c);
    if (bi >= 0) pseudonormal(t, P + 3 * i, bi, c, &s, n);
    if (S) S[i] = s * sqrt(best);
    if (I) I[i] = bi;
    if (C) memcpy(C + 3 * i, c, 24);
    if (N) memcpy(N + 3 * i, n, 24);
  }
}

void orc_point_line_projection(const double *v1, const double *v2, const double *v, double *pv, double *t) {
  double vv1[3], v21[3];
  sub3(v, v1, vv1); sub3(v2, v1, v21);
  double n2 = dot3(v21, v21);
  if (n2 >= PRECISION) *t = dot3(vv1, v21) / n2;
  else *t = 0;
  if (*t >= 0.0 && *t <= 1.0) for (int d = 0; d < 3; d++) pv[d] = v1[d] + *t * (v2[d] - v1[d]);
  else if (*t < 0.0) memcpy(pv, v1, 24);
  else if (*t > 1.0) memcpy(pv, v2, 24);
}

/* LINE branch of dirty_graph_projection (grid_hex_meshing.cpp:3963-4025): for each line vertex,
 * the closest point over the segments of its curve (a closed curve also has the segment from
 * its last vertex back to the first), the first such segment on ties, and that segment's unit
 * tangent.  A curve with no segment gives its single vertex and the tangent (1, 0, 0). */
void orc_curve_targets(int64_t nl, const double *X, const int32_t *lines, const int32_t *line_curve,
                       const double *TV, const int64_t *curve_ptr, const int32_t *curve_vs,
                       const uint8_t *closed, double *origin, double *axis) {
  for (int64_t i = 0; i < nl; i++) {
    const double *v = X + 3 * (int64_t)lines[i];
    const int32_t cu = line_curve[i];
    const int64_t c0 = curve_ptr[cu], size = curve_ptr[cu + 1] - c0;
    const int64_t len = closed[cu] ? size : size - 1;
    double best = INFINITY, pv[3] = {0, 0, 0}, tg[3] = {1, 0, 0};
    for (int64_t j = 0; j < len; j++) {
      const double *a = TV + 3 * (int64_t)curve_vs[c0 + j];
      const double *b = TV + 3 * (int64_t)curve_vs[c0 + (j + 1) % size];
      double pp[3], t, d[3];
      orc_point_line_projection(a, b, v, pp, &t);
      sub3(v, pp, d);
      const double dist = norm3(d);
      if (dist < best) {
        double e[3];
        sub3(b, a, e);
        const double ln = norm3(e);
        best = dist;
        memcpy(pv, pp, 24);
        for (int k = 0; k < 3; k++) tg[k] = e[k] / ln;
      }
    }
    if (len <= 0 && size > 0) memcpy(pv, TV + 3 * (int64_t)curve_vs[c0], 24);
    memcpy(origin + 3 * i, pv, 24);
    memcpy(axis + 3 * i, tg, 24);
  }
}

/* ------------------------------------------------------------------ Hausdorff */
/* vcg edge-plane face data (vcg/complex/algorithms/update/component_ep.h:45-75) */
typedef struct ep_face { double p[3][3]; double edge[3][3]; double dir[3]; double off; int axis; double darea; } ep_face;

static void ep_setup(const double *V, const int32_t *F, int64_t f, ep_face *e) {
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++) e->p[c][d] = V[3 * (int64_t)F[3 * f + c] + d];
  sub3(e->p[1], e->p[0], e->edge[0]);
  sub3(e->p[2], e->p[1], e->edge[1]);
  sub3(e->p[0], e->p[2], e->edge[2]);
  cross3(e->edge[0], e->edge[1], e->dir);
  e->off = dot3(e->dir, e->p[0]);
  double n = norm3(e->dir);
  if (n > 0) { for (int d = 0; d < 3; d++) e->dir[d] /= n; e->off /= n; }
  double nx = fabs(e->dir[0]), ny = fabs(e->dir[1]), nz = fabs(e->dir[2]), s;
  if (nx > ny && nx > nz) { e->axis = 0; s = 1 / e->dir[0]; }
  else if (ny > nz) { e->axis = 1; s = 1 / e->dir[1]; }
  else { e->axis = 2; s = 1 / e->dir[2]; }
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++) e->edge[c][d] *= s;
  double a[3], b[3], x[3];
  sub3(e->p[1], e->p[0], a); sub3(e->p[2], e->p[0], b); cross3(a, b, x);
  e->darea = norm3(x);
}

static double ps_dist(const double *q, const double *v1, const double *v2) {
  double e[3], qv[3], pp[3];
  sub3(v2, v1, e); sub3(q, v1, qv);
  double t = dot3(qv, e) / dot3(e, e);
  if (t < 0) t = 0; else if (t > 1) t = 1;
  for (int d = 0; d < 3; d++) pp[d] = q[d] - (v1[d] + e[d] * t);
  return norm3(pp);
}

/* vcg::face::PointDistanceEP (vcg/simplex/face/distance.h:49-180).  Updates *dist when the face
 * is closer; returns 1 when it did. */
static int point_distance_ep(const ep_face *f, const double *q, double *dist) {
  const double EPS = 0.000001;
  double d = dot3(f->dir, q) - f->off;
  if (d > *dist || d < -*dist) return 0;
  double p[3];
  for (int k = 0; k < 3; k++) p[k] = q[k] - f->dir[k] * d;
  int i1, i2; /* the two in-plane coordinates */
  if (f->axis == 0) { i1 = 1; i2 = 2; } else if (f->axis == 1) { i1 = 2; i2 = 0; } else { i1 = 0; i2 = 1; }
  double b0 = f->edge[1][i1] * (p[i2] - f->p[1][i2]) - f->edge[1][i2] * (p[i1] - f->p[1][i1]);
  if (b0 <= 0) {
    b0 = ps_dist(q, f->p[1], f->p[2]);
    if (*dist > b0) { *dist = b0; return 1; }
    return 0;
  }
  double b1 = f->edge[2][i1] * (p[i2] - f->p[2][i2]) - f->edge[2][i2] * (p[i1] - f->p[2][i1]);
  if (b1 <= 0) {
    b1 = ps_dist(q, f->p[2], f->p[0]);
    if (*dist > b1) { *dist = b1; return 1; }
    return 0;
  }
  double b2 = f->edge[0][i1] * (p[i2] - f->p[0][i2]) - f->edge[0][i2] * (p[i1] - f->p[0][i1]);
  if (b2 <= 0) {
    b2 = ps_dist(q, f->p[0], f->p[1]);
    if (*dist > b2) { *dist = b2; return 1; }
    return 0;
  }
  double b = b0 < b1 ? b0 : b1;
  if (b2 < b) b = b2;
  if (b < EPS * f->darea) {
    double bt;
    if (b == b0) bt = ps_dist(q, f->p[1], f->p[2]);
    else if (b == b1) bt = ps_dist(q, f->p[2], f->p[0]);
    else bt = ps_dist(q, f->p[0], f->p[1]);
    if (*dist > bt) { *dist = bt; return 1; }
    return 0;
  }
  *dist = fabs(d);
  return 1;
}

typedef struct ep_tree { ep_face *faces; tnode *nodes; int64_t nn; int64_t nf; } ep_tree;

static int32_t ep_build_rec(ep_tree *t, const double *V, const int32_t *F, int32_t *ids, int64_t n) {
  int32_t me = (int32_t)t->nn++;
  tnode *nd = &t->nodes[me];
  for (int d = 0; d < 3; d++) { nd->lo[d] = INFINITY; nd->hi[d] = -INFINITY; }
  double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) {
      const double *v = V + 3 * (int64_t)F[3 * (int64_t)ids[i] + c];
      for (int d = 0; d < 3; d++) {
        if (v[d] < nd->lo[d]) nd->lo[d] = v[d];
        if (v[d] > nd->hi[d]) nd->hi[d] = v[d];
      }
    }
  if (n == 1) { nd->prim = ids[0]; nd->left = nd->right = -1; return me; }
  for (int64_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      double c = g_cent[3 * (int64_t)ids[i] + d];
      if (c < clo[d]) clo[d] = c;
      if (c > chi[d]) chi[d] = c;
    }
  int ax = 0;
  for (int d = 1; d < 3; d++)
    if (chi[d] - clo[d] > chi[ax] - clo[ax]) ax = d;
  g_axis = ax;
  qsort(ids, n, sizeof(int32_t), cmp_cent);
  int64_t h = n / 2;
  nd->prim = -1;
  int32_t l = ep_build_rec(t, V, F, ids, h);
  int32_t r = ep_build_rec(t, V, F, ids + h, n - h);
  t->nodes[me].left = l;
  t->nodes[me].right = r;
  return me;
}

static void ep_tree_build(ep_tree *t, int64_t nv, const double *V, int64_t nf, const int32_t *F) {
  (void)nv;
  t->nf = nf;
  t->faces = (ep_face *)malloc(sizeof(ep_face) * (nf > 0 ? nf : 1));
  for (int64_t f = 0; f < nf; f++) ep_setup(V, F, f, &t->faces[f]);
  t->nodes = (tnode *)malloc(sizeof(tnode) * (2 * nf + 1));
  t->nn = 0;
  g_cent = (double *)malloc(sizeof(double) * 3 * (nf > 0 ? nf : 1));
  for (int64_t f = 0; f < nf; f++)
    for (int d = 0; d < 3; d++)
      g_cent[3 * f + d] = (V[3 * (int64_t)F[3 * f] + d] + V[3 * (int64_t)F[3 * f + 1] + d] + V[3 * (int64_t)F[3 * f + 2] + d]) / 3;
  int32_t *ids = (int32_t *)malloc(sizeof(int32_t) * (nf > 0 ? nf : 1));
  for (int64_t f = 0; f < nf; f++) ids[f] = (int32_t)f;
  if (nf > 0) ep_build_rec(t, V, F, ids, nf);
  free(ids); free(g_cent); g_cent = NULL;
}

static void ep_query(const ep_tree *t, int32_t node, const double *q, double *dist) {
  const tnode *nd = &t->nodes[node];
  if (nd->prim >= 0) { point_distance_ep(&t->faces[nd->prim], q, dist); return; }
  double dl = sqrt(box_dist2(&t->nodes[nd->left], q)), dr = sqrt(box_dist2(&t->nodes[nd->right], q));
  if (dl <= dr) {
    if (dl <= *dist) ep_query(t, nd->left, q, dist);
    if (dr <= *dist) ep_query(t, nd->right, q, dist);
  } else {
    if (dr <= *dist) ep_query(t, nd->right, q, dist);
    if (dl <= *dist) ep_query(t, nd->left, q, dist);
  }
}

void orc_point_face_distance(int64_t ns, const double *P, int64_t nv, const double *V, int64_t nf,
                             const int32_t *F, double *dist) {
  ep_tree t;
  ep_tree_build(&t, nv, V, nf, F);
  for (int64_t i = 0; i < ns; i++) {
    double d = INFINITY;
    if (nf > 0) ep_query(&t, 0, P + 3 * i, &d);
    dist[i] = d;
  }
  free(t.faces); free(t.nodes);
}

/* One direction of vcg::Sampling::Hausdorff in vertex-sampling mode (sampling.h:224-289,
 * 547-603): every face-referenced vertex of S1 against the faces of S2. */
static void hausdorff_one(int64_t nv1, const double *V1, int64_t nf1, const int32_t *F1, int64_t nv2,
                          const double *V2, int64_t nf2, const int32_t *F2, double upper, double *mx,
                          double *mean) {
  uint8_t *ref = (uint8_t *)calloc(nv1 > 0 ? nv1 : 1, 1);
  for (int64_t f = 0; f < nf1; f++)
    for (int c = 0; c < 3; c++) ref[F1[3 * f + c]] = 1;
  ep_tree t;
  ep_tree_build(&t, nv2, V2, nf2, F2);
  double m = -HUGE_VAL, s = 0;
  int64_t n = 0;
  for (int64_t v = 0; v < nv1; v++) {
    if (!ref[v]) continue;
    double d = upper;
    if (nf2 > 0) ep_query(&t, 0, V1 + 3 * v, &d);
    if (d == upper) continue;
    if (d > m) m = d;
    s += d;
    n++;
  }
  *mx = m;
  *mean = s / (double)n;
  free(ref); free(t.faces); free(t.nodes);
}

void orc_hausdorff(int64_t nv0, const double *V0, int64_t nf0, const int32_t *F0, int64_t nv1, const double *V1,
                   int64_t nf1, const int32_t *F1, double *bbox_diag, double *max_dist, double *ave_dist) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t v = 0; v < nv0; v++)
    for (int d = 0; d < 3; d++) {
      if (V0[3 * v + d] < lo[d]) lo[d] = V0[3 * v + d];
      if (V0[3 * v + d] > hi[d]) hi[d] = V0[3 * v + d];
    }
  for (int64_t v = 0; v < nv1; v++)
    for (int d = 0; d < 3; d++) {
      if (V1[3 * v + d] < lo[d]) lo[d] = V1[3 * v + d];
      if (V1[3 * v + d] > hi[d]) hi[d] = V1[3 * v + d];
    }
  double e[3];
  sub3(hi, lo, e);
  double diag = norm3(e), off = diag * 0.02;
  for (int d = 0; d < 3; d++) { lo[d] -= off; hi[d] += off; }
  sub3(hi, lo, e);
  double D = norm3(e);
  double m1, a1, m2, a2;
  hausdorff_one(nv0, V0, nf0, F0, nv1, V1, nf1, F1, D, &m1, &a1);
  hausdorff_one(nv1, V1, nf1, F1, nv0, V0, nf0, F0, D, &m2, &a2);
  *bbox_diag = D;
  *max_dist = m1 > m2 ? m1 : m2;
  *ave_dist = a2 > a1 ? a2 : a1;
}
