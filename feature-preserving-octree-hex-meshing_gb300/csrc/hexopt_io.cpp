// hexopt_io.cpp -- hex-mesh files in the reference's formats (io.cpp), host code of the C ABI.
//
//   MEDIT .mesh  write_hybrid_mesh_MESH (io.cpp:295-325): "MeshVersionFormatted 1", "Dimension 3",
//                "Vertices n" with "x y z 0" rows, "Hexahedra" / count / eight 1-based ids and a
//                0 reference per row, "End"; read_hybrid_mesh_MESH's reading of the same blocks.
//   legacy .vtk  write_hybrid_mesh_VTK (io.cpp:102-180): ASCII UNSTRUCTURED_GRID, POINTS, CELLS of
//                "8 ids", CELL_TYPES 12 (VTK_HEXAHEDRON), POINT_DATA "SCALARS fixed int" = the
//                boundary flags.
// Numbers are written as an iostream writes a double by default (6 significant digits), as the
// reference's files are.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/hexopt_gpu.h"

extern "C" {

int hexopt_write_hex_mesh(const char *path, int format, int64_t nv, const double *V, int64_t nh, const uint32_t *H,
                          const uint8_t *boundary) {
  if (!path || nv < 0 || nh < 0 || (nv > 0 && !V) || (nh > 0 && !H)) return HEXOPT_ERR_ARG;
  if (format != 0 && format != 1) return HEXOPT_ERR_ARG;
  for (int64_t i = 0; i < 8 * nh; i++)
    if ((int64_t)H[i] >= nv) return HEXOPT_ERR_ARG;
  std::ofstream f(path);
  if (!f) return HEXOPT_ERR_ARG;
  if (format == 0) {
    f << "MeshVersionFormatted 1" << std::endl;
    f << "Dimension 3" << std::endl;
    f << "Vertices" << " " << nv << std::endl;
    for (int64_t i = 0; i < nv; i++) f << V[3 * i] << " " << V[3 * i + 1] << " " << V[3 * i + 2] << " " << 0 << std::endl;
    f << "Hexahedra" << std::endl;
    f << nh << std::endl;
    for (int64_t h = 0; h < nh; h++) {
      for (int c = 0; c < 8; c++) f << H[8 * h + c] + 1 << " ";
      f << 0 << std::endl;
    }
    f << "End";
  } else {
    f << "# vtk DataFile Version 2.0" << std::endl << "mesh vtk data - converted from .off" << std::endl;
    f << "ASCII" << std::endl;
    f << "DATASET UNSTRUCTURED_GRID" << std::endl;
    f << "POINTS " << nv << " double" << std::endl;
    for (int64_t i = 0; i < nv; i++) f << V[3 * i] << " " << V[3 * i + 1] << " " << V[3 * i + 2] << std::endl;
    f << "CELLS " << nh << " " << nh * 9 << std::endl;
    for (int64_t h = 0; h < nh; h++) {
      f << " " << 8 << " ";
      for (int c = 0; c < 8; c++) f << H[8 * h + c] << " ";
      f << std::endl;
    }
    f << "CELL_TYPES " << nh << std::endl;
    for (int64_t h = 0; h < nh; h++) f << 12 << std::endl;
    f << "POINT_DATA " << nv << std::endl;
    f << "SCALARS fixed int" << std::endl;
    f << "LOOKUP_TABLE default" << std::endl;
    for (int64_t i = 0; i < nv; i++) f << ((boundary && boundary[i]) ? "1" : "0") << std::endl;
  }
  return f.good() ? HEXOPT_OK : HEXOPT_ERR_ARG;
}

int hexopt_read_hex_mesh(const char *path, int64_t *nv, int64_t *nh, double *V, uint32_t *H) {
  if (!path || !nv || !nh) return HEXOPT_ERR_ARG;
  std::ifstream f(path);
  if (!f) return HEXOPT_ERR_ARG;
  std::string tok;
  std::vector<double> v;
  std::vector<uint32_t> h;
  int64_t n_v = -1, n_h = -1;
  while (f >> tok) {
    if (tok == "Vertices") {
      if (!(f >> n_v) || n_v < 0) return HEXOPT_ERR_ARG;
      v.resize(3 * (size_t)n_v);
      for (int64_t i = 0; i < n_v; i++) {
        double ref;
        if (!(f >> v[3 * i] >> v[3 * i + 1] >> v[3 * i + 2] >> ref)) return HEXOPT_ERR_ARG;
      }
    } else if (tok == "Hexahedra") {
      if (!(f >> n_h) || n_h < 0) return HEXOPT_ERR_ARG;
      h.resize(8 * (size_t)n_h);
      for (int64_t i = 0; i < n_h; i++) {
        int64_t id, ref;
        for (int c = 0; c < 8; c++) {
          if (!(f >> id) || id < 1) return HEXOPT_ERR_ARG;
          h[8 * i + c] = (uint32_t)(id - 1);
        }
        if (!(f >> ref)) return HEXOPT_ERR_ARG;
      }
    } else if (tok == "End") {
      break;
    }
  }
  if (n_v < 0 || n_h < 0) return HEXOPT_ERR_ARG;
  for (uint32_t id : h)
    if ((int64_t)id >= n_v) return HEXOPT_ERR_ARG;
  const bool fits = V && H && *nv >= n_v && *nh >= n_h;
  if (fits) {
    std::memcpy(V, v.data(), sizeof(double) * v.size());
    std::memcpy(H, h.data(), sizeof(uint32_t) * h.size());
  }
  *nv = n_v;
  *nh = n_h;
  return HEXOPT_OK;
}

}  // extern "C"
