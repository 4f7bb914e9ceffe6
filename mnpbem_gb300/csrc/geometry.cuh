// Device view of a composite particle and its refined Green-function elements.
#pragma once
#include <vector>
#include <algorithm>
#include "common.cuh"

namespace mnpbem {

constexpr int MAX_ORDER = 8;
constexpr double DBL_EPS = 2.220446049250313e-16;  // MATLAB eps

struct GeomDev {
  int n = 0;                    // faces
  int order = 5;
  // geometry [n][3] / [n]
  const double* verts = nullptr;
  const int* faces = nullptr;   // [n][4], -1 = triangle
  const int* faces2 = nullptr;  // [n][9] curved elements (corners, edge midpoints, quad centre), or null
  double *pos = nullptr, *nvec = nullptr, *tvec1 = nullptr, *tvec2 = nullptr, *area = nullptr,
         *rad = nullptr;
  // quadrature rules
  int ntri = 0, n3 = 0, n4 = 0;
  const double *xt = nullptr, *yt = nullptr, *wt = nullptr;
  const double *x3 = nullptr, *y3 = nullptr, *w3 = nullptr;
  const double *x4 = nullptr, *y4 = nullptr, *w4 = nullptr;
  // refined elements in column-major order
  int64_t nref = 0;
  int* ref_row = nullptr;
  int* ref_col = nullptr;
  int64_t* col_off = nullptr;   // [n+1] offsets of each column's refined rows
  double* ref_g = nullptr;      // [nref][order+1]
  double* ref_f = nullptr;      // [nref][3][order+1]
};

struct DevBufSet {
  DevBuf verts, faces, faces2, quad, geo, col_off, ref_idx, ref_coef, part;
};

// faces2: NULL for flat elements, else [nfaces][9] curved connectivity into
// verts (interp = 'curv'; faces then holds the corners, faces2[:, 0:4])
mnpbem_status geometry_build(GeomDev& g, DevBufSet& b, const double* verts, int64_t nverts,
                             const int64_t* faces, const int64_t* faces2, int64_t nfaces,
                             const int* closed_part_start,
                             const int* closed_part_end, int nclosed, const mnpbem_quad* quad,
                             double rel_cut, double abs_cut, cudaStream_t st);

}  // namespace mnpbem
