// k_shapes.cu -- per-tet reference shapes of compute_referenceMesh (global_functions.cpp:3735-3806,
// hex2tet24 :3994-4022) for the general case: the reference positions of each hex may be any
// positions (the current ones, or another mesh's, as the untangling path uses the boundary-
// projected original mesh), with cube = 1 (cube of the hex's 24-tet volume), cube = 0 (the
// edge-averaged cuboid scaled to that volume) or h_flag = 0 (the hex's own reference corners).
//
// Per corner tet t with reference edge matrix R (columns r1 - r0, r2 - r0, r3 - r0 of the tet's
// reference corners), grad_tet_ref (grad.cpp:372-478) scales the reference tet to the tet's
// signed volume at precompute and takes its hat-function gradients; with E the tet's edge
// matrix at precompute that operator is J = E B_t with
//       B_t = adj(R) / |det R|^(2/3) / cbrt(det E).
// This kernel stores Bref_t = adj(R) / |det R|^(2/3) (9 doubles per tet); the precompute divides
// it by cbrt(det E).  For the unit cube corner tets R_k this is R_k^-1 / cbrt(det E), the closed
// form the cube-target path uses.
#include "hexopt_common.cuh"
#include "hexopt_kernels.h"
#include "hexopt_elem.cuh"

namespace hexopt {

// hex_face_table (global_types.h:154-161)
__device__ __forceinline__ int hex_face(int f, int j) {
  constexpr unsigned T[6] = {0x3210u, 0x5674u, 0x1540u, 0x4730u, 0x7623u, 0x2651u};
  return (int)((T[f] >> (4 * j)) & 0xFu);
}

__global__ void __launch_bounds__(128) k_ref_shapes(const double *P8, const uint32_t *hexv, const double *X,
                                                    const uint8_t *hflag, int cube, int64_t nh, double *Bref) {
  const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nh) return;
  double P[8][3];
  if (P8) {
#pragma unroll
    for (int c = 0; c < 8; c++)
#pragma unroll
      for (int d = 0; d < 3; d++) P[c][d] = P8[(h * 8 + c) * 3 + d];
  } else {
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const uint32_t v = hexv[hex_idx(h, c)];
#pragma unroll
      for (int d = 0; d < 3; d++) P[c][d] = X[4 * (int64_t)v + d];
    }
  }
  double v8[8][3];
  if (hflag && !hflag[h]) {
#pragma unroll
    for (int c = 0; c < 8; c++)
#pragma unroll
      for (int d = 0; d < 3; d++) v8[c][d] = P[c][d];
  } else {
    // hex2tet24: 24 tets (hex center, face center, face edge), unsigned volumes summed
    double hc[3] = {0, 0, 0};
#pragma unroll
    for (int c = 0; c < 8; c++)
#pragma unroll
      for (int d = 0; d < 3; d++) hc[d] += P[c][d];
#pragma unroll
    for (int d = 0; d < 3; d++) hc[d] /= 8;
    double vol = 0;
#pragma unroll
    for (int f = 0; f < 6; f++) {
      double fc[3] = {0, 0, 0};
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int d = 0; d < 3; d++) fc[d] += P[hex_face(f, j)][d];
#pragma unroll
      for (int d = 0; d < 3; d++) fc[d] /= 4;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int a = hex_face(f, j), b = hex_face(f, (j + 1) & 3);
        double J[3][3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          J[d][0] = P[a][d] - hc[d];
          J[d][1] = P[b][d] - hc[d];
          J[d][2] = fc[d] - hc[d];
        }
        vol += fabs(det3(J) / 6);
      }
    }
    double e0, e1, e2;
    if (cube && fabs(vol) > 1e-20) {
      e0 = e1 = e2 = cbrt(vol);
    } else {
      auto len = [&](int a, int b) {
        const double x = P[a][0] - P[b][0], y = P[a][1] - P[b][1], z = P[a][2] - P[b][2];
        return sqrt(x * x + y * y + z * z);
      };
      e0 = (len(0, 1) + len(3, 2) + len(4, 5) + len(7, 6)) / 4;
      e1 = (len(0, 3) + len(1, 2) + len(4, 7) + len(5, 6)) / 4;
      e2 = (len(0, 4) + len(1, 5) + len(2, 6) + len(3, 7)) / 4;
      const double ratio = cbrt(vol / (e0 * e1 * e2));
      e0 *= ratio; e1 *= ratio; e2 *= ratio;
    }
    // hex_ref_shape corners scaled per axis
    constexpr unsigned bits[8] = {0u, 1u, 3u, 2u, 4u, 5u, 7u, 6u};  // (x, y, z) bits of corner c
#pragma unroll
    for (int c = 0; c < 8; c++) {
      v8[c][0] = (bits[c] & 1u) ? e0 : 0.0;
      v8[c][1] = (bits[c] & 2u) ? e1 : 0.0;
      v8[c][2] = (bits[c] & 4u) ? e2 : 0.0;
    }
  }
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double R[3][3], A[3][3];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int d = 0; d < 3; d++) R[d][j] = v8[tet_v(k, j + 1)][d] - v8[tet_v(k, 0)][d];
    adj3(R, A);
    const double dr = fabs(det3(R));
    const double s = 1.0 / cbrt(dr * dr);
    double *B = Bref + (h * 8 + k) * 9;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) B[i * 3 + j] = A[i][j] * s;
  }
}

// rigidDeformCubes (optimization.cpp:456-494) on the exploded mesh of the untangling path, where
// every hex owns its 8 corner vertices (starting at the original mesh's positions): a hex
// with no held corner is replaced by the unit cube fitted to its corners by igl::procrustes with
// scaling and without reflection (procrustes.cpp: centred point sets, scale = |Y_c| / |X_c|,
// R = polar rotation of X_c^T Y_c, t = mean(Y) - scale R^T mean(X)); a hex with a held corner
// keeps its corners.  X (AoS4) and its FP32 split are rewritten in place.
__global__ void __launch_bounds__(128) k_rigid_cubes(const uint32_t *hexv, double *X, float *X32, const uint8_t *vfix,
                                                     int64_t nh) {
  const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= nh) return;
  int64_t vc[8];
#pragma unroll
  for (int c = 0; c < 8; c++) vc[c] = hexv[hex_idx(h, c)];
  if (vfix)
    for (int c = 0; c < 8; c++)
      if (vfix[vc[c]]) return;
  constexpr unsigned bits[8] = {0u, 1u, 3u, 2u, 4u, 5u, 7u, 6u};  // hex_ref_shape (x, y, z) bits
  double Y[8][3], ym[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < 8; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) {
      Y[c][d] = X[4 * vc[c] + d];
      ym[d] += Y[c][d];
    }
#pragma unroll
  for (int d = 0; d < 3; d++) ym[d] /= 8;
  // centred cube corners are +-0.5 per axis: |X_c|_F = sqrt(8 * 3 * 0.25)
  double ny = 0;
#pragma unroll
  for (int c = 0; c < 8; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) ny += (Y[c][d] - ym[d]) * (Y[c][d] - ym[d]);
  const double scale = (sqrt(ny) / 8) / (sqrt(6.0) / 8);
  double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int c = 0; c < 8; c++) {
    double xc[3];
#pragma unroll
    for (int d = 0; d < 3; d++) xc[d] = (((bits[c] >> d) & 1u) ? 0.5 : -0.5) * scale;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) S[i][j] += xc[i] * (Y[c][j] - ym[j]);
  }
  double R[3][3], U[3][3], sv[3], Vm[3][3];
  polar_svd3(S, R, U, sv, Vm);
  // t = mean(Y) - scale R^T mean(X), mean(X) = (0.5, 0.5, 0.5); cube corner c -> scale R^T c + t
  double t[3];
#pragma unroll
  for (int d = 0; d < 3; d++) t[d] = ym[d] - scale * 0.5 * (R[0][d] + R[1][d] + R[2][d]);
#pragma unroll
  for (int c = 0; c < 8; c++) {
    double p[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double acc = 0;
#pragma unroll
      for (int i = 0; i < 3; i++) acc += (((bits[c] >> i) & 1u) ? 1.0 : 0.0) * R[i][d];
      p[d] = scale * acc + t[d];
      X[4 * vc[c] + d] = p[d];
    }
    store_split(X32, vc[c], p[0], p[1], p[2]);
  }
}

void launch_rigid_cubes(const uint32_t *hexv, double *X, float *X32, const uint8_t *vfix, int64_t nh, cudaStream_t st) {
  if (nh <= 0) return;
  k_rigid_cubes<<<(unsigned)((nh + 127) / 128), 128, 0, st>>>(hexv, X, X32, vfix, nh);
}

// Bref of every corner tet from explicit reference tets (compute_referenceMesh's output ts.RT:
// 4 x 3 corner rows per tet, tet 8h + k of hex h in hex_tetra_table order).
__global__ void __launch_bounds__(128) k_ref_from_tets(const double *RT, int64_t ntet, double *Bref) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntet) return;
  const double *r = RT + t * 12;
  double R[3][3], A[3][3];
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int d = 0; d < 3; d++) R[d][j] = r[3 * (j + 1) + d] - r[d];
  adj3(R, A);
  const double dr = fabs(det3(R));
  const double s = 1.0 / cbrt(dr * dr);
  double *B = Bref + t * 9;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) B[i * 3 + j] = A[i][j] * s;
}

void launch_ref_from_tets(const double *RT, int64_t ntet, double *Bref, cudaStream_t st) {
  if (ntet > 0) k_ref_from_tets<<<(unsigned)((ntet + 127) / 128), 128, 0, st>>>(RT, ntet, Bref);
}

void launch_ref_shapes(const double *P8, const uint32_t *hexv, const double *X, const uint8_t *hflag, int cube,
                       int64_t nh, double *Bref, cudaStream_t st) {
  if (nh <= 0) return;
  k_ref_shapes<<<(unsigned)((nh + 127) / 128), 128, 0, st>>>(P8, hexv, X, hflag, cube, nh, Bref);
}

}  // namespace hexopt
