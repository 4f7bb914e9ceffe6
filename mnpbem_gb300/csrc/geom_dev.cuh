// Device helpers of the geometry kernels: vector arithmetic, curved-element
// shape functions and the Taylor coefficients of a refined (point, face) pair.
#pragma once
#include "geometry.cuh"

namespace mnpbem {

__device__ __forceinline__ double3 d3(double x, double y, double z) { return make_double3(x, y, z); }
__device__ __forceinline__ double3 sub3(double3 a, double3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 cross3(double3 a, double3 b) {
  return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double3 ld3(const double* p, int64_t i) { return d3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void st3(double* p, int64_t i, double3 v) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }

// ------------------------------------------------- curved element helpers
// 6-node triangle (Misc/+shape/@tri/eval.m:16-22, deriv.m:45-56): corners 1-3,
// midpoints of edges 12, 23, 31
__device__ __forceinline__ void shape6(double x, double y, double* s, double* sx, double* sy) {
  const double z = 1 - x - y;
  s[0] = x * (2 * x - 1); s[1] = y * (2 * y - 1); s[2] = z * (2 * z - 1);
  s[3] = 4 * x * y; s[4] = 4 * y * z; s[5] = 4 * z * x;
  sx[0] = 4 * x - 1; sx[1] = 0; sx[2] = 1 - 4 * z; sx[3] = 4 * y; sx[4] = -4 * y; sx[5] = 4 * (z - x);
  sy[0] = 0; sy[1] = 4 * y - 1; sy[2] = 1 - 4 * z; sy[3] = 4 * x; sy[4] = 4 * (z - y); sy[5] = -4 * x;
}
// 9-node quadrilateral (Misc/+shape/@quad/eval.m:19-27, deriv.m:47-66): corners
// 1-4, midpoints of edges 12, 23, 34, 41, centre
__device__ __forceinline__ void shape9(double x, double y, double* s, double* sx, double* sy) {
  const double a0 = 0.5 * x * (x - 1), a1 = 1 - x * x, a2 = 0.5 * x * (1 + x);
  const double b0 = 0.5 * y * (y - 1), b1 = 1 - y * y, b2 = 0.5 * y * (1 + y);
  const double da0 = x - 0.5, da1 = -2 * x, da2 = x + 0.5;
  const double db0 = y - 0.5, db1 = -2 * y, db2 = y + 0.5;
  s[0] = a0 * b0; s[1] = a2 * b0; s[2] = a2 * b2; s[3] = a0 * b2; s[4] = a1 * b0;
  s[5] = a2 * b1; s[6] = a1 * b2; s[7] = a0 * b1; s[8] = a1 * b1;
  sx[0] = da0 * b0; sx[1] = da2 * b0; sx[2] = da2 * b2; sx[3] = da0 * b2; sx[4] = da1 * b0;
  sx[5] = da2 * b1; sx[6] = da1 * b2; sx[7] = da0 * b1; sx[8] = da1 * b1;
  sy[0] = a0 * db0; sy[1] = a2 * db0; sy[2] = a2 * db2; sy[3] = a0 * db2; sy[4] = a1 * db0;
  sy[5] = a2 * db1; sy[6] = a1 * db2; sy[7] = a0 * db1; sy[8] = a1 * db1;
}
// 6-node triangles of a curved element (totriangles_curv.m:22-30): a triangle,
// or the halves (1,2,3,5,6,9) and (3,4,1,7,8,9) of a quadrilateral
__device__ __forceinline__ void curv_tri_nodes(const int* f2, int t, int* nd) {
  if (f2[3] < 0) { nd[0] = f2[0]; nd[1] = f2[1]; nd[2] = f2[2]; nd[3] = f2[4]; nd[4] = f2[5]; nd[5] = f2[6]; }
  else if (t == 0) { nd[0] = f2[0]; nd[1] = f2[1]; nd[2] = f2[2]; nd[3] = f2[4]; nd[4] = f2[5]; nd[5] = f2[8]; }
  else { nd[0] = f2[2]; nd[1] = f2[3]; nd[2] = f2[0]; nd[3] = f2[6]; nd[4] = f2[7]; nd[5] = f2[8]; }
}
// point and weight 0.5 w |dp/dx x dp/dy| of a 6-node triangle (quad_curv.m:39-54)
__device__ __forceinline__ void curv_tri_point(const double* verts, const int* nd, double x, double y, double w,
                                               double3& p, double& wt) {
  double s[6], sx[6], sy[6];
  shape6(x, y, s, sx, sy);
  double3 px = d3(0, 0, 0), py = d3(0, 0, 0);
  p = d3(0, 0, 0);
  for (int k = 0; k < 6; ++k) {
    const double3 v = ld3(verts, nd[k]);
    p.x += s[k] * v.x; p.y += s[k] * v.y; p.z += s[k] * v.z;
    px.x += sx[k] * v.x; px.y += sx[k] * v.y; px.z += sx[k] * v.z;
    py.x += sy[k] * v.x; py.y += sy[k] * v.y; py.z += sy[k] * v.z;
  }
  const double3 nv = cross3(px, py);
  wt = 0.5 * w * sqrt(dot3(nv, nv));
}


// Taylor coefficients g[o], f[:, o] (o = 0..order) of the Green function
// between the point pi and face j, refined by the boundary-element rule over
// face j (Greenfun/@greenret/private/init.m:98-177; quad_flat.m:77-113 or, for
// curved elements, quad_curv.m:39-54).  go [order+1], fo [3][order+1].
__device__ __forceinline__ void near_coefficients(const GeomDev& g, double3 pi, int j, double* go, double* fo) {
  const int O = g.order;
  double3 pj = ld3(g.pos, j);
  double3 v0 = sub3(pj, pi);
  double r0 = sqrt(dot3(v0, v0));
  double ag[MAX_ORDER + 1], ax[MAX_ORDER + 1], ay[MAX_ORDER + 1], az[MAX_ORDER + 1];
  for (int o = 0; o <= O; ++o) ag[o] = ax[o] = ay[o] = az[o] = 0.0;
  const int* f = g.faces + 4 * j;
  int ntri = f[3] < 0 ? 1 : 2;
  double invfact[MAX_ORDER + 2];
  invfact[0] = 1.0;
  for (int o = 1; o <= O; ++o) invfact[o] = invfact[o - 1] / o;
  for (int tr = 0; tr < ntri; ++tr) {
    int a = tr == 0 ? f[0] : f[2], b = tr == 0 ? f[1] : f[3], c = tr == 0 ? f[2] : f[0];
    double3 va = ld3(g.verts, a), vb = ld3(g.verts, b), vc = ld3(g.verts, c);
    double3 nv = cross3(sub3(vb, va), sub3(vc, va));
    double atri = 0.5 * sqrt(dot3(nv, nv));
    int nd[6];
    if (g.faces2) curv_tri_nodes(g.faces2 + 9 * j, tr, nd);
    for (int q = 0; q < g.ntri; ++q) {
      double x = g.xt[q], y = g.yt[q], z = 1 - x - y;
      double3 pt;
      double w;
      if (g.faces2) {
        // curved elements: quad_curv.m:39-54
        curv_tri_point(g.verts, nd, x, y, g.wt[q], pt, w);
      } else {
        pt = d3(x * va.x + y * vb.x + z * vc.x, x * va.y + y * vb.y + z * vc.y, x * va.z + y * vb.z + z * vc.z);
        w = g.wt[q] * atri;
      }
      double3 v = sub3(pi, pt);
      double r = sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
      double dr = r - r0;
      double ir = 1.0 / r, ir2 = ir * ir, ir3 = ir2 * ir;
      double drp = 1.0;   // dr^o
      double drm = 0.0;   // dr^(o-1)
      for (int o = 0; o <= O; ++o) {
        ag[o] += (drp * ir * invfact[o]) * w;
        double ff = (o == 0) ? -ir3 : (-drp * ir3 * invfact[o] + drm * ir2 * invfact[o - 1]);
        ax[o] += v.x * ff * w; ay[o] += v.y * ff * w; az[o] += v.z * ff * w;
        drm = drp; drp *= dr;
      }
    }
  }
  for (int o = 0; o <= O; ++o) {
    go[o] = ag[o];
    fo[0 * (O + 1) + o] = ax[o];
    fo[1 * (O + 1) + o] = ay[o];
    fo[2 * (O + 1) + o] = az[o];
  }
}

}  // namespace mnpbem
