// Geometry set-up of the retarded Green function, once per particle (FP64).
//
//  k_norm_flat      Particles/@particle/private/norm_flat.m:8-62 (+ Misc/+misc/bradius.m:11-32)
//  k_norm_curv      Particles/@particle/private/norm_curv.m:8-62, quad_curv.m:13-59 (curved elements)
//  k_ref_count /    Greenfun/+green/refinematrix.m:28-68 with Misc/+misc/pdist2.m:13-17
//  k_ref_fill       (pattern 2 = self element, 1 = near pair), in MATLAB find() order
//  k_ref_diag_*     Greenfun/@greenret/private/init.m:42-95   (polar integration, 'cart')
//  k_ref_offdiag    Greenfun/@greenret/private/init.m:98-177  (28-point rule, 'cart')
//  k_closed_sum     Greenfun/@compgreenret/private/initclosed.m:19-89 + @greenret/diag.m:10-30
#include "geometry.cuh"
#include "geom_dev.cuh"
#include "profile.cuh"

namespace mnpbem {

// ------------------------------------------------------------------ norm_flat
__global__ void k_norm_flat(int n, const double* __restrict__ verts, const int* __restrict__ faces,
                            double* pos, double* nvec, double* tvec1, double* tvec2, double* area,
                            double* rad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int* f = faces + 4 * i;
  double3 v1 = ld3(verts, f[0]), v2 = ld3(verts, f[1]), v3 = ld3(verts, f[2]);
  bool quad = f[3] >= 0;
  double3 p;
  if (!quad) {
    p = d3((v1.x + v2.x + v3.x) / 3, (v1.y + v2.y + v3.y) / 3, (v1.z + v2.z + v3.z) / 3);
  } else {
    double3 v4 = ld3(verts, f[3]);
    p = d3((v1.x + v2.x + v3.x + v4.x) / 4, (v1.y + v2.y + v3.y + v4.y) / 4,
           (v1.z + v2.z + v3.z + v4.z) / 4);
  }
  // first triangle (1,2,3): vec1 = v1 - v2, vec2 = v3 - v2
  double3 a1 = sub3(v1, v2), b1 = sub3(v3, v2);
  double3 n1 = cross3(a1, b1);
  double ar1 = tri_area_rn(v1, v2, v3);
  double3 t1 = a1, nn = n1;
  double ar = ar1;
  if (quad) {
    // second triangle (3,4,1)
    double3 v4 = ld3(verts, f[3]);
    double3 a2 = sub3(v3, v4), b2 = sub3(v1, v4);
    double3 n2 = cross3(a2, b2);
    double ar2 = tri_area_rn(v3, v4, v1);
    ar = ar1 + ar2;
    if (ar2 > ar1) { t1 = a2; nn = n2; }
  }
  double l1 = sqrt(dot3(t1, t1)), ln = sqrt(dot3(nn, nn));
  t1 = d3(t1.x / l1, t1.y / l1, t1.z / l1);
  nn = d3(nn.x / ln, nn.y / ln, nn.z / ln);
  double3 t2 = cross3(nn, t1);
  st3(pos, i, p); st3(nvec, i, nn); st3(tvec1, i, t1); st3(tvec2, i, t2);
  area[i] = ar;
  // bradius: max distance between centroid and vertices
  int nvx = quad ? 4 : 3;
  double r = 0.0;
  for (int k = 0; k < nvx; ++k) {
    double3 d = sub3(p, ld3(verts, f[k]));
    r = fmax(r, sqrt(d.x * d.x + d.y * d.y + d.z * d.z));
  }
  rad[i] = r;
}

// ------------------------------------------------------------------ norm_curv
// Curved elements: area = sum of the boundary-element weights of quad_curv.m
// over the element's 6-node triangles; centroid and tangent vectors from the
// shape functions at the centre (norm_curv.m:22-51); orthonormal basis as in
// norm_curv.m:54-59.  bradius uses the corner vertices.
__global__ void k_norm_curv(int n, const double* __restrict__ verts, const int* __restrict__ faces2,
                            const double* __restrict__ xt, const double* __restrict__ yt,
                            const double* __restrict__ wt, int ntri, double* pos, double* nvec, double* tvec1,
                            double* tvec2, double* area, double* rad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int* f2 = faces2 + 9 * i;
  const bool quad = f2[3] >= 0;
  double ar = 0.0;
  for (int t = 0; t < (quad ? 2 : 1); ++t) {
    int nd[6];
    curv_tri_nodes(f2, t, nd);
    for (int q = 0; q < ntri; ++q) {
      double3 p;
      double w;
      curv_tri_point(verts, nd, xt[q], yt[q], wt[q], p, w);
      ar += w;
    }
  }
  int nd[6];
  curv_tri_nodes(f2, 0, nd);
  double3 p = d3(0, 0, 0), a = d3(0, 0, 0), b = d3(0, 0, 0);
  if (!quad) {
    const double c[6] = {-1.0 / 9, -1.0 / 9, -1.0 / 9, 4.0 / 9, 4.0 / 9, 4.0 / 9};
    const double cx[6] = {1.0 / 3, 0.0, -1.0 / 3, 4.0 / 3, -4.0 / 3, 0.0};
    const double cy[6] = {0.0, 1.0 / 3, -1.0 / 3, 4.0 / 3, 0.0, -4.0 / 3};
    for (int k = 0; k < 6; ++k) {
      const double3 v = ld3(verts, nd[k]);
      p.x += c[k] * v.x; p.y += c[k] * v.y; p.z += c[k] * v.z;
      a.x += cy[k] * v.x; a.y += cy[k] * v.y; a.z += cy[k] * v.z;
      b.x += cx[k] * v.x; b.y += cx[k] * v.y; b.z += cx[k] * v.z;
    }
  } else {
    p = ld3(verts, nd[5]);   // quadrilateral centre
    const double cx[6] = {1.0, 0.0, -1.0, 0.0, 0.0, 0.0};
    const double cy[6] = {0.0, -1.0, -1.0, 2.0, 2.0, -2.0};
    for (int k = 0; k < 6; ++k) {
      const double3 v = ld3(verts, nd[k]);
      a.x += cy[k] * v.x; a.y += cy[k] * v.y; a.z += cy[k] * v.z;
      b.x += cx[k] * v.x; b.y += cx[k] * v.y; b.z += cx[k] * v.z;
    }
  }
  double3 nn = cross3(a, b);
  const double ln = sqrt(dot3(nn, nn)), la = sqrt(dot3(a, a));
  nn = d3(nn.x / ln, nn.y / ln, nn.z / ln);
  const double3 t1 = d3(a.x / la, a.y / la, a.z / la);
  st3(pos, i, p); st3(nvec, i, nn); st3(tvec1, i, t1); st3(tvec2, i, cross3(nn, t1));
  area[i] = ar;
  double r = 0.0;
  for (int k = 0; k < (quad ? 4 : 3); ++k) {
    const double3 d = sub3(p, ld3(verts, f2[k]));
    r = fmax(r, sqrt(dot3(d, d)));
  }
  rad[i] = r;
}

// ------------------------------------------------------------- refine pattern
// Entry (i, j): 2 where pdist2 gives d == 0, 1 where (d - rad_j < abs_cut) or
// ((d - rad_j) / rad_i < rel_cut), else 0.
__device__ __forceinline__ int ref_flag(const double* pos, const double* rad, int i, int j,
                                        double sqj, double3 pj, double radj, double rel_cut,
                                        double abs_cut) {
  double3 pi = ld3(pos, i);
  double sqi = pi.x * pi.x + pi.y * pi.y + pi.z * pi.z;
  double dd2 = (sqi + sqj) - 2.0 * (pi.x * pj.x + pi.y * pj.y + pi.z * pj.z);
  if (dd2 < 1e-10) dd2 = 0.0;
  double d = sqrt(dd2);
  if (d == 0.0) return 2;
  double d2 = d - radj;
  double id = d2 / rad[i];
  return (d2 < abs_cut || id < rel_cut) ? 1 : 0;
}

// one warp per column j; counts[j] = nonzeros in column j
__global__ void k_ref_count(int n, const double* __restrict__ pos, const double* __restrict__ rad,
                            double rel_cut, double abs_cut, int* counts) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= n) return;
  int j = warp;
  double3 pj = ld3(pos, j);
  double sqj = pj.x * pj.x + pj.y * pj.y + pj.z * pj.z;
  double radj = rad[j];
  int cnt = 0;
  for (int i0 = 0; i0 < n; i0 += 32) {
    int i = i0 + lane;
    int fl = (i < n) ? ref_flag(pos, rad, i, j, sqj, pj, radj, rel_cut, abs_cut) : 0;
    cnt += __popc(__ballot_sync(0xffffffffu, fl != 0));
  }
  if (lane == 0) counts[j] = cnt;
}

// fill rows in ascending order for each column (column-major find order)
__global__ void k_ref_fill(int n, const double* __restrict__ pos, const double* __restrict__ rad,
                           double rel_cut, double abs_cut, const int64_t* __restrict__ offs,
                           int* rows, int* cols, signed char* kind) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= n) return;
  int j = warp;
  double3 pj = ld3(pos, j);
  double sqj = pj.x * pj.x + pj.y * pj.y + pj.z * pj.z;
  double radj = rad[j];
  int64_t base = offs[j];
  for (int i0 = 0; i0 < n; i0 += 32) {
    int i = i0 + lane;
    int fl = (i < n) ? ref_flag(pos, rad, i, j, sqj, pj, radj, rel_cut, abs_cut) : 0;
    unsigned m = __ballot_sync(0xffffffffu, fl != 0);
    if (fl) {
      int64_t at = base + __popc(m & ((1u << lane) - 1u));
      rows[at] = i; cols[at] = j; kind[at] = (signed char)fl;
    }
    base += __popc(m);
  }
}

// ---------------------------------------------------- diagonal (polar) terms
// Polar integration points of face j (quadpol_flat.m:33-77)
struct PolPoint { double3 p; double w; };

__device__ __forceinline__ PolPoint polar_point(const GeomDev& g, int j, int q) {
  const int* f = g.faces + 4 * j;
  PolPoint r;
  if (g.faces2) {
    // curved elements (quadpol_curv.m:34-85)
    const int* f2 = g.faces2 + 9 * j;
    if (f2[3] < 0) {
      int nd[6];
      curv_tri_nodes(f2, 0, nd);
      curv_tri_point(g.verts, nd, g.x3[q], g.y3[q], g.w3[q], r.p, r.w);
    } else {
      double s[9], sx[9], sy[9];
      shape9(g.x4[q], g.y4[q], s, sx, sy);
      double3 p = d3(0, 0, 0), px = d3(0, 0, 0), py = d3(0, 0, 0);
      for (int k = 0; k < 9; ++k) {
        const double3 v = ld3(g.verts, f2[k]);
        p.x += s[k] * v.x; p.y += s[k] * v.y; p.z += s[k] * v.z;
        px.x += sx[k] * v.x; px.y += sx[k] * v.y; px.z += sx[k] * v.z;
        py.x += sy[k] * v.x; py.y += sy[k] * v.y; py.z += sy[k] * v.z;
      }
      const double3 nv = cross3(px, py);
      r.p = p;
      r.w = g.w4[q] * sqrt(dot3(nv, nv));
    }
    return r;
  }
  if (f[3] < 0) {
    double x = g.x3[q], y = g.y3[q];
    double3 v1 = ld3(g.verts, f[0]), v2 = ld3(g.verts, f[1]), v3 = ld3(g.verts, f[2]);
    double z = 1 - x - y;
    r.p = d3(x * v1.x + y * v2.x + z * v3.x, x * v1.y + y * v2.y + z * v3.y,
             x * v1.z + y * v2.z + z * v3.z);
    r.w = g.w3[q] * g.area[j];
  } else {
    double x = g.x4[q], y = g.y4[q];
    double s[4] = {0.25 * (1 - x) * (1 - y), 0.25 * (1 + x) * (1 - y), 0.25 * (1 + x) * (1 + y),
                   0.25 * (1 - x) * (1 + y)};
    double sx[4] = {-0.25 * (1 - y), 0.25 * (1 - y), 0.25 * (1 + y), -0.25 * (1 + y)};
    double sy[4] = {-0.25 * (1 - x), -0.25 * (1 + x), 0.25 * (1 + x), 0.25 * (1 - x)};
    double3 p = d3(0, 0, 0), px = d3(0, 0, 0), py = d3(0, 0, 0);
    for (int k = 0; k < 4; ++k) {
      double3 v = ld3(g.verts, f[k]);
      p.x += s[k] * v.x; p.y += s[k] * v.y; p.z += s[k] * v.z;
      px.x += sx[k] * v.x; px.y += sx[k] * v.y; px.z += sx[k] * v.z;
      py.x += sy[k] * v.x; py.y += sy[k] * v.y; py.z += sy[k] * v.z;
    }
    double3 nv = cross3(px, py);
    r.p = p;
    r.w = g.w4[q] * sqrt(dot3(nv, nv));
  }
  return r;
}

__device__ __forceinline__ int npolar(const GeomDev& g, int j) { return g.faces[4 * j + 3] < 0 ? g.n3 : g.n4; }

__device__ __forceinline__ void atomic_max_pos(double* addr, double v) {
  // valid for non-negative doubles: their bit patterns order like the values
  atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

// global max of r over all points of all self elements (rr clamp of init.m:77)
__global__ void k_ref_diag_rmax(GeomDev g, const int* __restrict__ diag_idx, int ndiag, double* rmax) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= ndiag) return;
  int e = diag_idx[warp];
  int i = g.ref_row[e], j = g.ref_col[e];
  double3 pi = ld3(g.pos, i);
  double m = 0.0;
  int np = npolar(g, j);
  for (int q = lane; q < np; q += 32) {
    PolPoint pp = polar_point(g, j, q);
    double3 v = sub3(pi, pp.p);
    m = fmax(m, sqrt(dot3(v, v)));
  }
  for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) atomic_max_pos(rmax, m);
}

__device__ __forceinline__ double ipow(double x, int k) {  // x^k, k may be negative
  double r = 1.0;
  if (k < 0) { x = 1.0 / x; k = -k; }
  for (int t = 0; t < k; ++t) r *= x;
  return r;
}

// one warp per self element: g[o] and Cartesian f[:, o]
__global__ void k_ref_diag(GeomDev g, const int* __restrict__ diag_idx, int ndiag,
                           const double* __restrict__ rmax_p) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= ndiag) return;
  const int O = g.order;
  int e = diag_idx[warp];
  int i = g.ref_row[e], j = g.ref_col[e];
  double3 pi = ld3(g.pos, i), ni = ld3(g.nvec, i), t1 = ld3(g.tvec1, i), t2 = ld3(g.tvec2, i);
  double rclamp = 1e-4 * (*rmax_p);
  double acc_g[MAX_ORDER + 1], acc_n[MAX_ORDER + 1], acc_1[MAX_ORDER + 1], acc_2[MAX_ORDER + 1];
  for (int o = 0; o <= O; ++o) acc_g[o] = acc_n[o] = acc_1[o] = acc_2[o] = 0.0;
  int np = npolar(g, j);
  for (int q = lane; q < np; q += 32) {
    PolPoint pp = polar_point(g, j, q);
    double3 v = sub3(pi, pp.p);
    double r = sqrt(dot3(v, v));
    double rr = fmax(r, rclamp);
    double in = dot3(v, ni), in1 = dot3(v, t1), in2 = dot3(v, t2);
    double rr3 = rr * rr * rr;
    for (int o = 0; o <= O; ++o) {
      acc_g[o] += pp.w * ipow(r, o - 1);
      acc_n[o] += pp.w * ((o - 1) * in * ipow(r, o - 3));
      double ro = ipow(r, o);
      acc_1[o] += pp.w * ((o - 1) * in1 * ro / rr3);
      acc_2[o] += pp.w * ((o - 1) * in2 * ro / rr3);
    }
  }
  double fact = 1.0;
  for (int o = 0; o <= O; ++o) {
    if (o > 0) fact *= o;
    double sg = acc_g[o], sn = acc_n[o], s1 = acc_1[o], s2 = acc_2[o];
    for (int s = 16; s; s >>= 1) {
      sg += __shfl_xor_sync(0xffffffffu, sg, s);
      sn += __shfl_xor_sync(0xffffffffu, sn, s);
      s1 += __shfl_xor_sync(0xffffffffu, s1, s);
      s2 += __shfl_xor_sync(0xffffffffu, s2, s);
    }
    if (lane == 0) {
      sg /= fact; sn /= fact; s1 /= fact; s2 /= fact;
      g.ref_g[(int64_t)e * (O + 1) + o] = sg;
      double* f = g.ref_f + (int64_t)e * 3 * (O + 1);
      f[0 * (O + 1) + o] = ni.x * sn + t1.x * s1 + t2.x * s2;
      f[1 * (O + 1) + o] = ni.y * sn + t1.y * s1 + t2.y * s2;
      f[2 * (O + 1) + o] = ni.z * sn + t1.z * s1 + t2.z * s2;
    }
  }
}

// ------------------------------------------------- off-diagonal near pairs
// one thread per near pair (i, j): boundary-element rule over face j
// (quad_flat.m:77-113 / quad_curv.m:39-54, coefficients of init.m:98-177)
__global__ void k_ref_offdiag(GeomDev g, const int* __restrict__ off_idx, int noff) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= noff) return;
  int e = off_idx[t];
  int i = g.ref_row[e], j = g.ref_col[e];
  near_coefficients(g, ld3(g.pos, i), j, g.ref_g + (int64_t)e * (g.order + 1),
                    g.ref_f + (int64_t)e * 3 * (g.order + 1));
}

// --------------------------------------------------- closed-surface sum rule
// One block per column j of closed particle [s, e): f_j = sum_i A_i F0_ij / A_j
// with F0 the k = 0 surface derivative (refined entries: nvec_i . f[:, 0]).
// Then f(self j, :, 0) += nvec_j * (-2 pi - f_j).
__global__ void k_closed_sum(GeomDev g, int s, int e, const int64_t* __restrict__ col_off) {
  int j = s + blockIdx.x;
  if (j >= e) return;
  const int O = g.order;
  double3 pj = ld3(g.pos, j);
  double aj = g.area[j];
  double invaj = 1.0 / aj;
  int64_t r0 = col_off[j], r1 = col_off[j + 1];
  double acc = 0.0;
  for (int i = s + threadIdx.x; i < e; i += blockDim.x) {
    // refined entry?  rows of column j are sorted ascending
    int64_t lo = r0, hi = r1;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (g.ref_row[mid] < i) lo = mid + 1; else hi = mid;
    }
    double3 ni = ld3(g.nvec, i);
    double F;
    if (lo < r1 && g.ref_row[lo] == i) {
      const double* f = g.ref_f + lo * 3 * (O + 1);
      F = ni.x * f[0] + ni.y * f[O + 1] + ni.z * f[2 * (O + 1)];
    } else {
      double3 pi = ld3(g.pos, i);
      double3 v = sub3(pi, pj);
      double d = fmax(sqrt(dot3(v, v)), DBL_EPS);
      double in = dot3(ni, v);
      F = in * (-1.0 / d) / (d * d) * aj;
    }
    acc += g.area[i] * (F * invaj);
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double fj = red[0];
    // self element of column j
    int64_t lo = r0, hi = r1;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (g.ref_row[mid] < j) lo = mid + 1; else hi = mid;
    }
    if (lo < r1 && g.ref_row[lo] == j) {
      double3 nj = ld3(g.nvec, j);
      double val = -2.0 * M_PI * 1.0 - fj;
      double* f = g.ref_f + lo * 3 * (O + 1);
      f[0] += nj.x * val; f[O + 1] += nj.y * val; f[2 * (O + 1)] += nj.z * val;
    }
  }
}

// ============================================================== host driver
mnpbem_status geometry_build(GeomDev& g, DevBufSet& b, const double* verts, int64_t nverts,
                             const int64_t* faces, const int64_t* faces2, int64_t nfaces,
                             const int* closed_part_start,
                             const int* closed_part_end, int nclosed, const mnpbem_quad* quad,
                             double rel_cut, double abs_cut, cudaStream_t st) {
  const int n = (int)nfaces;
  g.n = n;
  ProfScope ps(PH_GEOMETRY, st, 0.0, 0.0, 0);
  // ---- upload vertices, faces, quadrature rules
  MNP_TRY(b.verts.ensure(sizeof(double) * 3 * nverts));
  MNP_CUDA(cudaMemcpyAsync(b.verts.ptr, verts, sizeof(double) * 3 * nverts, cudaMemcpyHostToDevice, st));
  {
    std::vector<int> f32(4 * (size_t)n);
    for (int64_t k = 0; k < 4 * nfaces; ++k) f32[k] = (int)faces[k];
    MNP_TRY(b.faces.ensure(sizeof(int) * 4 * n));
    MNP_CUDA(cudaMemcpyAsync(b.faces.ptr, f32.data(), sizeof(int) * 4 * n, cudaMemcpyHostToDevice, st));
    MNP_CUDA(cudaStreamSynchronize(st));
  }
  g.faces2 = nullptr;
  if (faces2) {
    std::vector<int> f9(9 * (size_t)n);
    for (int64_t k = 0; k < 9 * nfaces; ++k) f9[k] = (int)faces2[k];
    MNP_TRY(b.faces2.ensure(sizeof(int) * 9 * n));
    MNP_CUDA(cudaMemcpyAsync(b.faces2.ptr, f9.data(), sizeof(int) * 9 * n, cudaMemcpyHostToDevice, st));
    MNP_CUDA(cudaStreamSynchronize(st));
    g.faces2 = b.faces2.as<int>();
  }
  {
    std::vector<double> q;
    auto app = [&](const double* a, int m) { for (int k = 0; k < m; ++k) q.push_back(a[k]); };
    app(quad->x, quad->n_tri); app(quad->y, quad->n_tri); app(quad->w, quad->n_tri);
    app(quad->x3, quad->n_pol3); app(quad->y3, quad->n_pol3); app(quad->w3, quad->n_pol3);
    app(quad->x4, quad->n_pol4); app(quad->y4, quad->n_pol4); app(quad->w4, quad->n_pol4);
    MNP_TRY(b.quad.ensure(sizeof(double) * q.size()));
    MNP_CUDA(cudaMemcpyAsync(b.quad.ptr, q.data(), sizeof(double) * q.size(), cudaMemcpyHostToDevice, st));
    MNP_CUDA(cudaStreamSynchronize(st));
    double* base = b.quad.as<double>();
    g.ntri = quad->n_tri; g.n3 = quad->n_pol3; g.n4 = quad->n_pol4;
    g.xt = base; g.yt = base + g.ntri; g.wt = base + 2 * g.ntri;
    base += 3 * g.ntri;
    g.x3 = base; g.y3 = base + g.n3; g.w3 = base + 2 * g.n3;
    base += 3 * g.n3;
    g.x4 = base; g.y4 = base + g.n4; g.w4 = base + 2 * g.n4;
  }
  g.verts = b.verts.as<double>();
  g.faces = b.faces.as<int>();
  // ---- norm_flat + bradius
  MNP_TRY(b.geo.ensure(sizeof(double) * 14 * (size_t)n));
  double* G = b.geo.as<double>();
  g.pos = G; g.nvec = G + 3 * n; g.tvec1 = G + 6 * n; g.tvec2 = G + 9 * n; g.area = G + 12 * n;
  g.rad = G + 13 * n;
  if (ps.p) ps.p->acc[PH_GEOMETRY].launches += 1;
  if (g.faces2)
    k_norm_curv<<<(n + 127) / 128, 128, 0, st>>>(n, g.verts, g.faces2, g.xt, g.yt, g.wt, g.ntri, g.pos, g.nvec,
                                                   g.tvec1, g.tvec2, g.area, g.rad);
  else
    k_norm_flat<<<(n + 127) / 128, 128, 0, st>>>(n, g.verts, g.faces, g.pos, g.nvec, g.tvec1, g.tvec2,
                                                   g.area, g.rad);
  MNP_CHECK_LAUNCH();
  // ---- refinement pattern
  DevBuf counts;
  MNP_TRY(counts.ensure(sizeof(int) * n));
  int warps_per_block = 8;
  int nblk = (n + warps_per_block - 1) / warps_per_block;
  k_ref_count<<<nblk, 32 * warps_per_block, 0, st>>>(n, g.pos, g.rad, rel_cut, abs_cut, counts.as<int>());
  MNP_CHECK_LAUNCH();
  std::vector<int> hcnt(n);
  MNP_CUDA(cudaMemcpyAsync(hcnt.data(), counts.ptr, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> offs(n + 1, 0);
  for (int j = 0; j < n; ++j) offs[j + 1] = offs[j] + hcnt[j];
  int64_t nref = offs[n];
  g.nref = nref;
  MNP_TRY(b.col_off.ensure(sizeof(int64_t) * (n + 1)));
  MNP_CUDA(cudaMemcpyAsync(b.col_off.ptr, offs.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st));
  MNP_TRY(b.ref_idx.ensure(sizeof(int) * 2 * (size_t)std::max<int64_t>(nref, 1) + std::max<int64_t>(nref, 1)));
  g.ref_row = b.ref_idx.as<int>();
  g.ref_col = g.ref_row + nref;
  signed char* kind = reinterpret_cast<signed char*>(g.ref_col + nref);
  g.col_off = b.col_off.as<int64_t>();
  k_ref_fill<<<nblk, 32 * warps_per_block, 0, st>>>(n, g.pos, g.rad, rel_cut, abs_cut, g.col_off,
                                                     g.ref_row, g.ref_col, kind);
  MNP_CHECK_LAUNCH();
  const int O = g.order;
  MNP_TRY(b.ref_coef.ensure(sizeof(double) * 4 * (O + 1) * (size_t)std::max<int64_t>(nref, 1)));
  g.ref_g = b.ref_coef.as<double>();
  g.ref_f = g.ref_g + nref * (O + 1);
  MNP_CUDA(cudaMemsetAsync(b.ref_coef.ptr, 0, sizeof(double) * 4 * (O + 1) * (size_t)std::max<int64_t>(nref, 1), st));
  // ---- split refined entries into self (2) and near (1) lists
  std::vector<signed char> hkind(nref);
  if (nref) {
    MNP_CUDA(cudaMemcpyAsync(hkind.data(), kind, nref, cudaMemcpyDeviceToHost, st));
    MNP_CUDA(cudaStreamSynchronize(st));
  }
  std::vector<int> dl, ol;
  for (int64_t e = 0; e < nref; ++e) (hkind[e] == 2 ? dl : ol).push_back((int)e);
  DevBuf lists;
  MNP_TRY(lists.ensure(sizeof(int) * (dl.size() + ol.size() + 1) + 64));
  int* d_dl = lists.as<int>();
  int* d_ol = d_dl + dl.size();
  if (!dl.empty()) MNP_CUDA(cudaMemcpyAsync(d_dl, dl.data(), sizeof(int) * dl.size(), cudaMemcpyHostToDevice, st));
  if (!ol.empty()) MNP_CUDA(cudaMemcpyAsync(d_ol, ol.data(), sizeof(int) * ol.size(), cudaMemcpyHostToDevice, st));
  if (O > 0 && nref > 0) {
    if (!dl.empty()) {
      DevBuf rmax;
      MNP_TRY(rmax.ensure(sizeof(double)));
      MNP_CUDA(cudaMemsetAsync(rmax.ptr, 0, sizeof(double), st));
      int nd = (int)dl.size();
      k_ref_diag_rmax<<<(nd + 7) / 8, 256, 0, st>>>(g, d_dl, nd, rmax.as<double>());
      MNP_CHECK_LAUNCH();
      k_ref_diag<<<(nd + 7) / 8, 256, 0, st>>>(g, d_dl, nd, rmax.as<double>());
      MNP_CHECK_LAUNCH();
      MNP_CUDA(cudaStreamSynchronize(st));
    }
    if (!ol.empty()) {
      int no = (int)ol.size();
      k_ref_offdiag<<<(no + 127) / 128, 128, 0, st>>>(g, d_ol, no);
      MNP_CHECK_LAUNCH();
    }
  }
  // ---- closed surfaces
  for (int c = 0; c < nclosed; ++c) {
    int s = closed_part_start[c], e = closed_part_end[c];
    if (e > s) {
      k_closed_sum<<<e - s, 256, 0, st>>>(g, s, e, g.col_off);
      MNP_CHECK_LAUNCH();
    }
  }
  MNP_CUDA(cudaStreamSynchronize(st));
  return MNPBEM_OK;
}

}  // namespace mnpbem
