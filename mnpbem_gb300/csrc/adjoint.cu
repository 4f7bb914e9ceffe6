// Adjoint gradient of the plane-wave extinction cross section with respect to
// the vertex coordinates and to the dielectric function inside the particle.
// The reference has no gradients; the forward path it differentiates is
//   A x = b (BEM/@bemretiter/private/afun.m:6-35, solved by mldivide.m),
//   J = ext = 4 pi / k Im(pol* . e(dir))  (@planewaveret/extinction.m:12-16,
//            @spectrumret/farfield.m:15-74),
// with the matrices of Greenfun/@greenret/private/eval1.m (far pairs),
// greenret/private/init.m (Taylor coefficients of near pairs and self
// elements) and compgreenret/private/initclosed.m (closed-surface diagonal).
//
//   A^T lam = w  (w = dJ/dx),  dJ = Re(lam^T (db - dA x)) + dJ/dtheta|_x
//
// lam^T dA x contracts dG1, dH1, dG2, dH2 with rank-4 weights
//   W_ij = U_i . X_j   (U from lam, eps and normals; X = (sig, h) of the side)
// evaluated on the fly: one O(n^2) pass over all pairs with the far-field
// derivative, one pass over the near pairs (quadrature points of the source
// face) that replaces the far derivative by the refined one, one pass over
// the self elements (polar points), and per-face passes for the excitation,
// the explicit normals / eps of the alpha and De rows, the far-field phase of
// J and the chain rule of norm_flat.m (centroids, normals, areas -> vertices).
// Every accumulation is FP64 (atomicAdd on per-face / per-vertex arrays).
#include "adjoint.cuh"
#include "profile.cuh"

namespace mnpbem {

namespace {

__device__ __forceinline__ double3 v3(double x, double y, double z) { return make_double3(x, y, z); }
__device__ __forceinline__ double3 vsub(double3 a, double3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double3 vadd(double3 a, double3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ double3 vscale(double3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double vdot(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 vcross(double3 a, double3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double3 vld(const double* p, int64_t i) { return v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void vatomic(double* p, int64_t i, double3 v) {
  atomicAdd(p + 3 * i, v.x);
  atomicAdd(p + 3 * i + 1, v.y);
  atomicAdd(p + 3 * i + 2, v.z);
}
__device__ __forceinline__ double2 cexpi(double2 k, double d) {   // exp(i k d)
  double s, c;
  sincos(k.x * d, &s, &c);
  const double e = exp(-k.y * d);
  return make_double2(e * c, e * s);
}
__device__ __forceinline__ double2 cx(double r, double i) { return make_double2(r, i); }
__device__ __forceinline__ double2 cscl(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 imul(double2 a) { return make_double2(-a.y, a.x); }   // i a
// Re(a * b)
__device__ __forceinline__ double remul(double2 a, double2 b) { return a.x * b.x - a.y * b.y; }

// W = U . X (4 complex)
__device__ __forceinline__ double2 wdot(const double2* U, const double2* X) {
  double2 s = make_double2(0, 0);
#pragma unroll
  for (int r = 0; r < 4; ++r) s = cadd(s, cmul(U[r], X[r]));
  return s;
}

struct FarGrad {
  double3 gri;   // dJ / d r_i
  double3 grj;   // dJ / d r_j
  double3 gni;   // dJ / d n_i
  double gaj;    // dJ / d A_j
  double2 gk;    // d(lam^T A x) / dk   (medium 1 only)
};

// far-pair contribution -Re(WG dG + WF dF) of one medium (eval1.m:24-40, 110-124)
__device__ __forceinline__ void far_grad(double2 k, double2 WG, double2 WF, double3 R, double d, double3 ni,
                                         double Aj, FarGrad& g, bool want_k) {
  const double inv = 1.0 / d;
  const double3 Rh = vscale(R, inv);
  const double nR = vdot(ni, R);
  const double2 E = cexpi(k, d);
  const double2 ikm = cx(-k.y - inv, k.x);                      // ik - 1/d
  const double2 G = cscl(E, Aj * inv);
  const double2 phi = cscl(cmul(ikm, E), inv * inv);            // (ik - 1/d) e / d^2
  const double2 ik = cx(-k.y, k.x);
  // dphi/dd = e [1/d^4 + (ik - 1/d)(ik/d^2 - 2/d^3)]
  const double2 t2 = cx(ik.x * inv * inv - 2.0 * inv * inv * inv, ik.y * inv * inv);
  const double2 dphi = cmul(E, cadd(cx(inv * inv * inv * inv, 0.0), cmul(ikm, t2)));
  const double2 cG = cmul(WG, cmul(G, ikm));
  const double2 cFd = cscl(cmul(WF, dphi), nR * Aj);
  const double2 cFn = cscl(cmul(WF, phi), Aj);
  const double2 cd = cadd(cG, cFd);
  const double3 gR = vadd(vscale(Rh, cd.x), vscale(ni, cFn.x));  // Re(...)
  g.gri = vsub(g.gri, gR);
  g.grj = vadd(g.grj, gR);
  g.gni = vsub(g.gni, vscale(R, cFn.x));
  g.gaj -= remul(WG, cscl(E, inv)) + remul(WF, cscl(phi, nR));
  if (want_k) {
    // dG/dk = i d G ; dF/dk = nR A (-k e / d)
    const double2 dGk = imul(cscl(G, d));
    const double2 dFk = cscl(cmul(cscl(k, -inv), E), nR * Aj);
    g.gk = cadd(g.gk, cadd(cmul(WG, dGk), cmul(WF, dFk)));
  }
}

// closed-surface term Re(c_b dT_ab), T_ab = -A_a (n_a . R) / d^3, R = r_a - r_b
__device__ __forceinline__ void closed_far_grad(double cb, double3 R, double d, double3 na, double Aa,
                                                double3& gra, double3& grb, double3& gna, double& gaa) {
  const double inv = 1.0 / d, inv3 = inv * inv * inv;
  const double nR = vdot(na, R);
  const double T = -Aa * nR * inv3;
  gaa += cb * T / Aa;
  gna = vadd(gna, vscale(R, -cb * Aa * inv3));
  const double3 gR = vscale(vsub(vscale(na, inv3), vscale(R, 3.0 * nR * inv3 * inv * inv)), -cb * Aa);
  gra = vadd(gra, gR);
  grb = vsub(grb, gR);
}

constexpr int PG_COLS = 128, PG_ROWS = 16;

// all pairs i != j: far-field derivatives of both media + closed-surface term
__global__ void __launch_bounds__(PG_COLS) k_adj_pairs(AdjParams p) {
  const int64_t j = (int64_t)blockIdx.x * PG_COLS + threadIdx.x;
  const int64_t i0 = (int64_t)blockIdx.y * PG_ROWS;
  const bool jok = j < p.n;
  const int64_t jj = jok ? j : 0;
  const double3 rj = vld(p.pos, jj);
  const double Aj = p.area[jj];
  double2 X1[4], X2[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) { X1[r] = p.X[jj * 8 + r]; X2[r] = p.X[jj * 8 + 4 + r]; }
  const double cb = p.cb[jj];
  double3 grj = v3(0, 0, 0);
  double gaj = 0.0;
  double2 gk = make_double2(0, 0);
  const int lane = threadIdx.x & 31;
  for (int r = 0; r < PG_ROWS; ++r) {
    const int64_t i = i0 + r;
    if (i >= p.n) break;
    const double3 ri = vld(p.pos, i), ni = vld(p.nvec, i);
    const double Ai = p.area[i];
    FarGrad g;
    g.gri = g.grj = g.gni = v3(0, 0, 0);
    g.gaj = 0.0;
    g.gk = make_double2(0, 0);
    double3 cgi = v3(0, 0, 0), cgn = v3(0, 0, 0), cgj = v3(0, 0, 0);
    double cga = 0.0;
    if (jok && i != j) {
      const double3 R = vsub(ri, rj);
      const double d = sqrt(vdot(R, R));
      const double2* U = p.U + i * 16;
      far_grad(p.k1, wdot(U, X1), wdot(U + 4, X1), R, d, ni, Aj, g, true);
      far_grad(p.k2, wdot(U + 8, X2), wdot(U + 12, X2), R, d, ni, Aj, g, false);
      closed_far_grad(cb, R, d, ni, Ai, cgi, cgj, cgn, cga);
    }
    grj = vadd(grj, vadd(g.grj, cgj));
    gaj += g.gaj;
    gk = cadd(gk, g.gk);
    // row quantities: warp reduction, one atomic per warp
    double3 gi = vadd(g.gri, cgi), gn = vadd(g.gni, cgn);
    double ga = cga;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      gi.x += __shfl_xor_sync(0xffffffffu, gi.x, o);
      gi.y += __shfl_xor_sync(0xffffffffu, gi.y, o);
      gi.z += __shfl_xor_sync(0xffffffffu, gi.z, o);
      gn.x += __shfl_xor_sync(0xffffffffu, gn.x, o);
      gn.y += __shfl_xor_sync(0xffffffffu, gn.y, o);
      gn.z += __shfl_xor_sync(0xffffffffu, gn.z, o);
      ga += __shfl_xor_sync(0xffffffffu, ga, o);
    }
    if (lane == 0) {
      vatomic(p.gpos, i, gi);
      vatomic(p.gnv, i, gn);
      atomicAdd(p.garea + i, ga);
    }
  }
  if (jok) {
    vatomic(p.gpos, j, grj);
    atomicAdd(p.garea + j, gaj);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    gk.x += __shfl_xor_sync(0xffffffffu, gk.x, o);
    gk.y += __shfl_xor_sync(0xffffffffu, gk.y, o);
  }
  if (lane == 0) {
    atomicAdd(p.gk1, gk.x);
    atomicAdd(p.gk1 + 1, gk.y);
  }
}

// triangle tr (0 or 1) of face f: vertex ids (totriangles: (1,2,3), (3,4,1))
__device__ __forceinline__ void tri_ids(const int* f, int tr, int& a, int& b, int& c) {
  a = tr == 0 ? f[0] : f[2];
  b = tr == 0 ? f[1] : f[3];
  c = tr == 0 ? f[2] : f[0];
}

// gradient of area = |(vb - va) x (vc - va)| / 2 times ga onto the three vertices
__device__ __forceinline__ void tri_area_grad(double* gv, int a, int b, int c, double3 va, double3 vb, double3 vc,
                                              double ga) {
  const double3 N = vcross(vsub(vb, va), vsub(vc, va));
  const double nn = sqrt(vdot(N, N));
  const double3 gN = vscale(N, 0.5 * ga / nn);
  const double3 ge1 = vcross(vsub(vc, va), gN);
  const double3 ge2 = vcross(gN, vsub(vb, va));
  vatomic(gv, a, vscale(vadd(ge1, ge2), -1.0));
  vatomic(gv, b, ge1);
  vatomic(gv, c, ge2);
}

// refined off-diagonal pairs: the near derivative replaces the far one
// (greenret/private/init.m:98-177 coefficients, eval1.m:36-39 / 119-123)
__global__ void k_adj_near(AdjParams p) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.noff) return;
  const int e = p.off_idx[t];
  const int i = p.ref_row[e], j = p.ref_col[e];
  const int O = p.order;
  const double3 ri = vld(p.pos, i), rj = vld(p.pos, j), ni = vld(p.nvec, i);
  const double Ai = p.area[i], Aj = p.area[j];
  const double3 R = vsub(ri, rj);
  const double d = sqrt(vdot(R, R));
  const double3 Rh = vscale(R, 1.0 / d);
  const double2* U = p.U + (int64_t)i * 16;
  double2 X1[4], X2[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) { X1[r] = p.X[(int64_t)j * 8 + r]; X2[r] = p.X[(int64_t)j * 8 + 4 + r]; }
  const double2 W[4] = {wdot(U, X1), wdot(U + 4, X1), wdot(U + 8, X2), wdot(U + 12, X2)};
  const double2 ks[2] = {p.k1, p.k2};
  // remove the far derivative that the pair pass applied
  FarGrad g;
  g.gri = g.grj = g.gni = v3(0, 0, 0);
  g.gaj = 0.0;
  g.gk = make_double2(0, 0);
  far_grad(p.k1, W[0], W[1], R, d, ni, Aj, g, true);
  far_grad(p.k2, W[2], W[3], R, d, ni, Aj, g, false);
  double3 gri = vscale(g.gri, -1.0), grj = vscale(g.grj, -1.0), gni = vscale(g.gni, -1.0);
  double gaj = -g.gaj;
  double2 gk = cscl(g.gk, -1.0);
  const double cb = p.cb[j];
  {
    double3 ca = v3(0, 0, 0), cbv = v3(0, 0, 0), cn = v3(0, 0, 0);
    double cga = 0.0;
    closed_far_grad(cb, R, d, ni, Ai, ca, cbv, cn, cga);
    gri = vsub(gri, ca);
    grj = vsub(grj, cbv);
    gni = vsub(gni, cn);
    atomicAdd(p.garea + i, -cga);
  }
  // near derivative, per medium and per quadrature point of face j
  double2 E[2], c[2][MAX_ORDER_ADJ + 1];
  for (int m = 0; m < 2; ++m) {
    E[m] = cexpi(ks[m], d);
    double2 ik = cx(-ks[m].y, ks[m].x), pw = cx(1.0, 0.0);
    double fo = 1.0;
    for (int o = 0; o <= O; ++o) {
      if (o) fo *= o;
      c[m][o] = cscl(pw, 1.0 / fo);      // (ik)^o / o!
      pw = cmul(pw, ik);
    }
  }
  double2 gam[2] = {cx(0, 0), cx(0, 0)}, phn[2] = {cx(0, 0), cx(0, 0)};
  double2 sGd[2] = {cx(0, 0), cx(0, 0)}, sPd[2] = {cx(0, 0), cx(0, 0)};
  double2 sGk = cx(0, 0), sPk = cx(0, 0);
  double3 grho_sum = v3(0, 0, 0);
  double3 gni_sum = v3(0, 0, 0);
  double ccl_area_a = 0.0, ccl_area_b = 0.0;   // closed-surface area terms
  double3 ccl_na = v3(0, 0, 0), ccl_ra = v3(0, 0, 0);
  const double fac = -Ai / Aj;
  const int* f = p.faces + 4 * j;
  const int ntri = f[3] < 0 ? 1 : 2;
  // first pass: sums over the points (gam, phn, d-derivatives) per medium
  // and the per-point gradients, which need gam-independent factors only
  for (int tr = 0; tr < ntri; ++tr) {
    int a, b, cc;
    tri_ids(f, tr, a, b, cc);
    const double3 va = vld(p.verts, a), vb = vld(p.verts, b), vc = vld(p.verts, cc);
    const double3 N = vcross(vsub(vb, va), vsub(vc, va));
    const double atri = 0.5 * sqrt(vdot(N, N));
    double3 gva = v3(0, 0, 0), gvb = v3(0, 0, 0), gvc = v3(0, 0, 0);
    double gatri = 0.0;
    for (int q = 0; q < p.ntri; ++q) {
      const double x = p.xt[q], y = p.yt[q], z = 1 - x - y;
      const double3 pt = v3(x * va.x + y * vb.x + z * vc.x, x * va.y + y * vb.y + z * vc.y,
                            x * va.z + y * vb.z + z * vc.z);
      const double qw = p.wt[q];
      const double ww = qw * atri;
      const double3 rho = vsub(ri, pt);
      const double r = sqrt(vdot(rho, rho));
      const double ir = 1.0 / r;
      const double3 rh = vscale(rho, ir);
      const double nrho = vdot(ni, rho);
      const double dr = r - d;
      double3 gpt = v3(0, 0, 0);   // dJ / d rho (this point)
      double gw = 0.0;             // dJ / d ww
      for (int m = 0; m < 2; ++m) {
        double2 Gam = cx(0, 0), Gr = cx(0, 0), Gd = cx(0, 0), Psi = cx(0, 0), Pr = cx(0, 0), Pd = cx(0, 0);
        double2 Gk = cx(0, 0), Pk = cx(0, 0);
        double drp = 1.0, drm = 0.0, drmm = 0.0;   // dr^o, dr^(o-1), dr^(o-2)
        double fo = 1.0, fo1 = 1.0;                // o!, (o-1)!
        const double2 ik = cx(-ks[m].y, ks[m].x);
        double2 ikm1 = cx(1.0, 0.0);               // (ik)^(o-1) for o >= 1
        for (int o = 0; o <= O; ++o) {
          if (o) { fo1 = fo; fo *= o; }
          const double2 co = cscl(c[m][o], fo);    // (ik)^o
          const double gam_o = drp * ir / fo;
          const double gr_o = ((o ? o * drm * ir : 0.0) - drp * ir * ir) / fo;
          const double gd_o = -(o ? o * drm * ir : 0.0) / fo;
          double ps, psr, psd;
          if (o == 0) {
            ps = -ir * ir * ir;
            psr = 3.0 * ir * ir * ir * ir;
            psd = 0.0;
          } else {
            ps = -drp * ir * ir * ir / fo + drm * ir * ir / fo1;
            psr = -(o * drm * ir * ir * ir - 3.0 * drp * ir * ir * ir * ir) / fo +
                  ((o > 1 ? (o - 1) * drmm : 0.0) * ir * ir - 2.0 * drm * ir * ir * ir) / fo1;
            psd = o * drm * ir * ir * ir / fo - (o > 1 ? (o - 1) * drmm : 0.0) * ir * ir / fo1;
          }
          Gam = cadd(Gam, cscl(co, gam_o));
          Gr = cadd(Gr, cscl(co, gr_o));
          Gd = cadd(Gd, cscl(co, gd_o));
          Psi = cadd(Psi, cscl(co, ps));
          Pr = cadd(Pr, cscl(co, psr));
          Pd = cadd(Pd, cscl(co, psd));
          if (o && m == 0) {
            // d/dk (ik)^o = o i (ik)^(o-1)
            const double2 dko = cscl(imul(ikm1), (double)o);
            Gk = cadd(Gk, cscl(dko, gam_o));
            Pk = cadd(Pk, cscl(dko, ps));
          }
          if (o) ikm1 = cmul(ikm1, ik);
          drmm = drm;
          drm = drp;
          drp *= dr;
        }
        const double2 WgE = cmul(W[2 * m], E[m]), WfE = cmul(W[2 * m + 1], E[m]);
        gam[m] = cadd(gam[m], cscl(Gam, ww));
        phn[m] = cadd(phn[m], cscl(Psi, ww * nrho));
        sGd[m] = cadd(sGd[m], cscl(Gd, ww));
        sPd[m] = cadd(sPd[m], cscl(Pd, ww * nrho));
        if (m == 0) {
          sGk = cadd(sGk, cscl(Gk, ww));
          sPk = cadd(sPk, cscl(Pk, ww * nrho));
        }
        // crho = WgE ww Gr rh + WfE ww (n Psi + nrho Pr rh); dJ/drho = -Re(crho)
        const double2 a1 = cscl(cmul(WgE, Gr), ww);
        const double2 a2 = cscl(cmul(WfE, Psi), ww);
        const double2 a3 = cscl(cmul(WfE, Pr), ww * nrho);
        gpt = vsub(gpt, vadd(vscale(rh, a1.x + a3.x), vscale(ni, a2.x)));
        gw -= remul(WgE, Gam) + remul(WfE, cscl(Psi, nrho));
        gni_sum = vsub(gni_sum, vscale(rho, remul(WfE, cscl(Psi, ww))));
      }
      // closed-surface near term T = fac sum_w ww nrho / r^3 (order 0, k = 0)
      {
        const double ir3 = ir * ir * ir;
        const double Tq = fac * ww * nrho * ir3;
        ccl_area_a += cb * Tq / Ai;
        ccl_area_b -= cb * Tq / Aj;
        ccl_na = vadd(ccl_na, vscale(rho, cb * fac * ww * ir3));
        const double3 gq = vscale(vsub(vscale(ni, ir3), vscale(rho, 3.0 * nrho * ir3 * ir * ir)), cb * fac * ww);
        gpt = vadd(gpt, gq);
        gw += cb * fac * nrho * ir3;
      }
      grho_sum = vadd(grho_sum, gpt);
      // rho = r_i - x_w, x_w = x va + y vb + z vc
      gva = vsub(gva, vscale(gpt, x));
      gvb = vsub(gvb, vscale(gpt, y));
      gvc = vsub(gvc, vscale(gpt, z));
      gatri += gw * qw;
    }
    vatomic(p.gv, a, gva);
    vatomic(p.gv, b, gvb);
    vatomic(p.gv, cc, gvc);
    tri_area_grad(p.gv, a, b, cc, va, vb, vc, gatri);
  }
  gri = vadd(gri, grho_sum);
  gni = vadd(gni, gni_sum);
  gni = vadd(gni, ccl_na);
  // explicit d-dependence (incl. the phase): -Re(W E (sum d-derivatives + (gam or phn) ik))
  for (int m = 0; m < 2; ++m) {
    const double2 ik = cx(-ks[m].y, ks[m].x);
    const double2 cd = cadd(cmul(cmul(W[2 * m], E[m]), cadd(sGd[m], cmul(gam[m], ik))),
                            cmul(cmul(W[2 * m + 1], E[m]), cadd(sPd[m], cmul(phn[m], ik))));
    gri = vsub(gri, vscale(Rh, cd.x));
    grj = vadd(grj, vscale(Rh, cd.x));
  }
  // d/dk1 of the refined entries: E (sum dk-terms + (gam or phn) i d)
  gk = cadd(gk, cadd(cmul(cmul(W[0], E[0]), cadd(sGk, imul(cscl(gam[0], d)))),
                     cmul(cmul(W[1], E[0]), cadd(sPk, imul(cscl(phn[0], d))))));
  vatomic(p.gpos, i, gri);
  vatomic(p.gpos, j, grj);
  vatomic(p.gnv, i, gni);
  atomicAdd(p.garea + j, gaj);
  atomicAdd(p.garea + i, ccl_area_a);
  atomicAdd(p.garea + j, ccl_area_b);
  atomicAdd(p.gk1, gk.x);
  atomicAdd(p.gk1 + 1, gk.y);
}

// self elements: G_ii = sum_w ww sum_o (ik)^o r^(o-1) / o! over the polar
// points of face i (greenret/private/init.m:42-95); weights ww = w3 A_i for
// triangles, w4 |dx/du x dx/dv| for quadrilaterals (quadpol_flat.m:33-77)
__global__ void k_adj_self(AdjParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int O = p.order;
  const int* f = p.faces + 4 * i;
  const bool quad = f[3] >= 0;
  const int nv = quad ? 4 : 3;
  double3 vv[4];
  for (int a = 0; a < nv; ++a) vv[a] = vld(p.verts, f[a]);
  double3 cen = v3(0, 0, 0);
  for (int a = 0; a < nv; ++a) cen = vadd(cen, vv[a]);
  cen = vscale(cen, 1.0 / nv);
  const double2* U = p.U + (int64_t)i * 16;
  double2 X1[4], X2[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) { X1[r] = p.X[(int64_t)i * 8 + r]; X2[r] = p.X[(int64_t)i * 8 + 4 + r]; }
  const double2 WG[2] = {wdot(U, X1), wdot(U + 8, X2)};
  const double2 ks[2] = {p.k1, p.k2};
  double3 gv[4] = {v3(0, 0, 0), v3(0, 0, 0), v3(0, 0, 0), v3(0, 0, 0)};
  double garea = 0.0;
  double2 gk = cx(0, 0);
  const int npts = quad ? p.n4 : p.n3;
  for (int q = 0; q < npts; ++q) {
    double s[4], sx[4], sy[4];
    double w0;
    if (!quad) {
      const double x = p.x3[q], y = p.y3[q];
      s[0] = x; s[1] = y; s[2] = 1 - x - y; s[3] = 0;
      w0 = p.w3[q];
    } else {
      const double x = p.x4[q], y = p.y4[q];
      s[0] = 0.25 * (1 - x) * (1 - y); s[1] = 0.25 * (1 + x) * (1 - y);
      s[2] = 0.25 * (1 + x) * (1 + y); s[3] = 0.25 * (1 - x) * (1 + y);
      sx[0] = -0.25 * (1 - y); sx[1] = 0.25 * (1 - y); sx[2] = 0.25 * (1 + y); sx[3] = -0.25 * (1 + y);
      sy[0] = -0.25 * (1 - x); sy[1] = -0.25 * (1 + x); sy[2] = 0.25 * (1 + x); sy[3] = 0.25 * (1 - x);
      w0 = p.w4[q];
    }
    double3 pt = v3(0, 0, 0);
    for (int a = 0; a < nv; ++a) pt = vadd(pt, vscale(vv[a], s[a]));
    const double3 rho = vsub(cen, pt);
    const double r = sqrt(vdot(rho, rho));
    const double3 rh = vscale(rho, 1.0 / r);
    double ww, jn = 0.0;
    double3 jac = v3(0, 0, 0), px = v3(0, 0, 0), py = v3(0, 0, 0);
    if (!quad) {
      ww = w0 * p.area[i];
    } else {
      for (int a = 0; a < 4; ++a) { px = vadd(px, vscale(vv[a], sx[a])); py = vadd(py, vscale(vv[a], sy[a])); }
      jac = vcross(px, py);
      jn = sqrt(vdot(jac, jac));
      ww = w0 * jn;
    }
    double3 grho = v3(0, 0, 0);
    double gw = 0.0;
    for (int m = 0; m < 2; ++m) {
      const double2 ik = cx(-ks[m].y, ks[m].x);
      double2 pw = cx(1.0, 0.0), ikm1 = cx(1.0, 0.0);
      double2 Gam = cx(0, 0), Gr = cx(0, 0), Gk = cx(0, 0);
      double fo = 1.0;
      for (int o = 0; o <= O; ++o) {
        if (o) fo *= o;
        const double ro1 = pow(r, (double)(o - 1));
        Gam = cadd(Gam, cscl(pw, ro1 / fo));
        Gr = cadd(Gr, cscl(pw, (o - 1) * pow(r, (double)(o - 2)) / fo));
        if (o && m == 0) {
          Gk = cadd(Gk, cscl(imul(ikm1), (double)o * ro1 / fo));
          ikm1 = cmul(ikm1, ik);
        }
        pw = cmul(pw, ik);
      }
      grho = vsub(grho, vscale(rh, remul(WG[m], cscl(Gr, ww))));
      gw -= remul(WG[m], Gam);
      if (m == 0) gk = cadd(gk, cmul(WG[0], cscl(Gk, ww)));
    }
    // rho = cen - pt = sum_a (1/nv - s_a) v_a
    for (int a = 0; a < nv; ++a) gv[a] = vadd(gv[a], vscale(grho, 1.0 / nv - s[a]));
    if (!quad) {
      garea += gw * w0;
    } else {
      const double3 gj = vscale(jac, gw * w0 / jn);
      const double3 gpx = vcross(py, gj), gpy = vcross(gj, px);
      for (int a = 0; a < 4; ++a) gv[a] = vadd(gv[a], vadd(vscale(gpx, sx[a]), vscale(gpy, sy[a])));
    }
  }
  for (int a = 0; a < nv; ++a) vatomic(p.gv, f[a], gv[a]);
  atomicAdd(p.garea + i, garea);
  atomicAdd(p.gk1, gk.x);
  atomicAdd(p.gk1 + 1, gk.y);
}

// per face: weights U, X and the closed-surface factor c_i = WH1_ii + WH2_ii
//   u1 = lphi - i k0 e1 (lal . n),  v1 = la - i k0 e1 lDe n       (G1 rows)
//   UH1 = (e1 lDe, lal),  UG2 = -(u2, v2),  UH2 = -(e2 lDe, lal)   (H1, G2, H2)
__global__ void k_adj_weights(AdjParams p, const double2* lphi, const double2* la, const double2* lDe,
                              const double2* lal, const double2* x1, const double2* x2, int P, int ip) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double3 n = vld(p.nvec, i);
  const double2 e1 = p.eps1[i], e2 = p.eps2[i];
  const double k0 = p.k0;
  const double2 lal3[3] = {lal[3 * i], lal[3 * i + 1], lal[3 * i + 2]};
  const double2 la3[3] = {la[3 * i], la[3 * i + 1], la[3 * i + 2]};
  const double2 ln = cadd(cadd(cscl(lal3[0], n.x), cscl(lal3[1], n.y)), cscl(lal3[2], n.z));
  const double nc[3] = {n.x, n.y, n.z};
  double2* U = p.U + i * 16;
  for (int side = 0; side < 2; ++side) {
    const double2 e = side == 0 ? e1 : e2;
    const double sg = side == 0 ? 1.0 : -1.0;
    const double2 ike = cscl(imul(e), -k0);          // -i k0 e
    const double2 u = cadd(lphi[i], cmul(ike, ln));
    U[8 * side + 0] = cscl(u, sg);
    const double2 ikel = cmul(ike, lDe[i]);
    for (int c = 0; c < 3; ++c) U[8 * side + 1 + c] = cscl(cadd(la3[c], cscl(ikel, nc[c])), sg);
    U[8 * side + 4] = cscl(cmul(e, lDe[i]), sg);
    for (int c = 0; c < 3; ++c) U[8 * side + 5 + c] = cscl(lal3[c], sg);
  }
  double2* X = p.X + i * 8;
  const int W = 4 * P;
  X[0] = x1[i * W + ip];
  for (int c = 0; c < 3; ++c) X[1 + c] = x1[i * W + P + c * P + ip];
  X[4] = x2[i * W + ip];
  for (int c = 0; c < 3; ++c) X[5 + c] = x2[i * W + P + c * P + ip];
  // c_i = WH1_ii + WH2_ii (real part enters the closed-surface term)
  const double2 c = cadd(wdot(U + 4, X), wdot(U + 12, X + 4));
  p.cb[i] = c.x;
}

// per face: J's far-field phase and area, the plane-wave excitation b, and
// the explicit normals / eps1 of the alpha and De rows of afun.m
// GX1 = G1 [sig1 h1] and GX2 = G2 [sig2 h2] as [n][4], HX1 = H1 sig1 [n]
__global__ void k_adj_faces(AdjParams p, int which, const double* pol, const double* dir, const double2* lphi,
                            const double2* la, const double2* lDe, const double2* lal, const double2* GX1,
                            const double2* GX2, const double2* HX1, double* geps) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double3 r = vld(p.pos, i), n = vld(p.nvec, i);
  const double A = p.area[i];
  const double3 pl = v3(pol[0], pol[1], pol[2]), dv = v3(dir[0], dir[1], dir[2]);
  const double2 kb = p.kb;
  const double k0 = p.k0;
  const double2* X = p.X + i * 8;   // sig2 = X[4], h2 = X[5..7]
  double3 gpos = v3(0, 0, 0), gnv = v3(0, 0, 0);
  double garea = 0.0;
  const double2 e1 = p.eps1[i], e2 = p.eps2[i];
  const double s = vdot(r, dv);
  if (p.exc_out[i]) {
    if (which == 0) {
      // ext: J = Re(ah . h2 + as sig2), Phi = exp(-i kb dir.r) A
      const double2 Phi = cscl(cexpi(cscl(kb, -1.0), s), A);
      const double2 kq = cdiv(cx(4.0 * M_PI * k0, 0.0), kb);
      const double2 ph2 = cadd(cadd(cscl(X[5], pl.x), cscl(X[6], pl.y)), cscl(X[7], pl.z));
      const double2 Jt = cadd(cmul(cmul(kq, Phi), ph2), cscl(cmul(Phi, X[4]), -4.0 * M_PI * vdot(pl, dv)));
      const double2 dJr = cmul(imul(kb), Jt);   // i kb Jt; dJ/dr = Re(-i kb Jt) dir
      gpos = vsub(gpos, vscale(dv, dJr.x));
      garea += Jt.x / A;
    }
    // excitation on the outside: a = e / (i k0) pol, De = -e2 (n.pol) e, alpha = (kb/k0)(n.dir) e pol
    const double2 ph = cexpi(kb, s);
    const double2 lap = cadd(cadd(cscl(la[3 * i], pl.x), cscl(la[3 * i + 1], pl.y)), cscl(la[3 * i + 2], pl.z));
    const double2 lalp = cadd(cadd(cscl(lal[3 * i], pl.x), cscl(lal[3 * i + 1], pl.y)), cscl(lal[3 * i + 2], pl.z));
    const double npl = vdot(n, pl), ndr = vdot(n, dv);
    const double2 kk0 = cscl(kb, 1.0 / k0);
    gpos = vadd(gpos, vscale(dv, cmul(cmul(lap, ph), kk0).x));
    const double2 t1 = cmul(cscl(e2, -1.0), cmul(lDe[i], ph));
    gnv = vadd(gnv, vscale(pl, t1.x));
    gpos = vadd(gpos, vscale(dv, cmul(t1, imul(cscl(kb, npl))).x));
    const double2 t2 = cmul(kk0, cmul(lalp, ph));
    gnv = vadd(gnv, vscale(dv, t2.x));
    gpos = vadd(gpos, vscale(dv, cmul(t2, imul(cscl(kb, ndr))).x));
  }
  // explicit n and eps1 in alpha / De (A x enters dJ with a minus sign)
  const double2 ik0 = cx(0.0, k0);
  const double2 a = csub(cmul(e1, GX1[4 * i]), cmul(e2, GX2[4 * i]));
  double2 gn_c[3];
  const double nc[3] = {n.x, n.y, n.z};
  double2 nGh1 = cx(0, 0);
  for (int c = 0; c < 3; ++c) {
    const double2 b = csub(cmul(e1, GX1[4 * i + 1 + c]), cmul(e2, GX2[4 * i + 1 + c]));
    gn_c[c] = cmul(cscl(ik0, -1.0), cadd(cmul(lal[3 * i + c], a), cmul(lDe[i], b)));
    nGh1 = cadd(nGh1, cscl(GX1[4 * i + 1 + c], nc[c]));
  }
  gnv = vsub(gnv, v3(gn_c[0].x, gn_c[1].x, gn_c[2].x));
  const double2 lalN = cadd(cadd(cscl(lal[3 * i], n.x), cscl(lal[3 * i + 1], n.y)), cscl(lal[3 * i + 2], n.z));
  const double2 de = cadd(cadd(cmul(cmul(cscl(ik0, -1.0), lalN), GX1[4 * i]), cmul(lDe[i], HX1[i])),
                          cmul(cmul(cscl(ik0, -1.0), lDe[i]), nGh1));
  vatomic(p.gpos, i, gpos);
  vatomic(p.gnv, i, gnv);
  atomicAdd(p.garea + i, garea);
  atomicAdd(geps, de.x);
  atomicAdd(geps + 1, de.y);
}

// chain rule of norm_flat.m: centroid (mean of the vertices), unit normal and
// area of the triangle(s) -> vertices; a quadrilateral's normal is that of its
// larger triangle and its area the sum of both
__global__ void k_adj_norm_flat(AdjParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const int* f = p.faces + 4 * i;
  const int nv = f[3] >= 0 ? 4 : 3;
  const double3 gp = vld(p.gpos, i), gn = vld(p.gnv, i);
  const double ga = p.garea[i];
  for (int a = 0; a < nv; ++a) vatomic(p.gv, f[a], vscale(gp, 1.0 / nv));
  const int ntri = nv == 4 ? 2 : 1;
  double ar[2] = {0, 0};
  for (int tr = 0; tr < ntri; ++tr) {
    int a, b, c;
    tri_ids(f, tr, a, b, c);
    ar[tr] = tri_area_rn(vld(p.verts, a), vld(p.verts, b), vld(p.verts, c));   // the choice of k_norm_flat
  }
  const int big = (ntri == 2 && ar[1] > ar[0]) ? 1 : 0;
  for (int tr = 0; tr < ntri; ++tr) {
    int a, b, c;
    tri_ids(f, tr, a, b, c);
    // norm_flat: vec1 = v1 - v2, vec2 = v3 - v2, N = vec1 x vec2
    const double3 e1 = vsub(vld(p.verts, a), vld(p.verts, b)), e2 = vsub(vld(p.verts, c), vld(p.verts, b));
    const double3 N = vcross(e1, e2);
    const double nN = sqrt(vdot(N, N));
    const double3 nh = vscale(N, 1.0 / nN);
    double3 gN = vscale(nh, 0.5 * ga);
    if (tr == big) gN = vadd(gN, vscale(vsub(gn, vscale(nh, vdot(nh, gn))), 1.0 / nN));
    const double3 ge1 = vcross(e2, gN), ge2 = vcross(gN, e1);
    vatomic(p.gv, a, ge1);
    vatomic(p.gv, c, ge2);
    vatomic(p.gv, b, vscale(vadd(ge1, ge2), -1.0));
  }
}

// --------------------------------------------- transposed chain helpers
// in-place transpose of an n x n complex128 matrix (leading dimension ld)
template <typename C>
__global__ void k_transpose_sq(C* A, int64_t n, int64_t ld) {
  __shared__ C t1[32][33], t2[32][33];
  const int bx = blockIdx.x, by = blockIdx.y;
  if (bx < by) return;
  const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
  const int64_t r1 = (int64_t)by * 32, c1 = (int64_t)bx * 32;
  for (int k = ty; k < 32; k += 8) {
    const int64_t r = r1 + k, c = c1 + tx;
    t1[k][tx] = (r < n && c < n) ? A[r * ld + c] : C{};
    const int64_t r2 = c1 + k, c2 = r1 + tx;
    t2[k][tx] = (r2 < n && c2 < n) ? A[r2 * ld + c2] : C{};
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int64_t r = r1 + k, c = c1 + tx;
    if (r < n && c < n) A[r * ld + c] = t2[tx][k];
    const int64_t r2 = c1 + k, c2 = r1 + tx;
    if (bx != by && r2 < n && c2 < n) A[r2 * ld + c2] = t1[tx][k];
  }
}

// right-hand side w = dJ/dx for sig2 (gs2 [n]) and h2 (gh2 [n][3]) on faces
// whose outside medium is the excitation medium
__global__ void k_adj_rhs(AdjParams p, const double* pol, const double* dir, double2* gs2, double2* gh2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double3 r = vld(p.pos, i);
  const double3 pl = v3(pol[0], pol[1], pol[2]), dv = v3(dir[0], dir[1], dir[2]);
  double2 s = cx(0, 0), h[3] = {cx(0, 0), cx(0, 0), cx(0, 0)};
  if (p.exc_out[i]) {
    const double2 Phi = cscl(cexpi(cscl(p.kb, -1.0), vdot(r, dv)), p.area[i]);
    const double2 kq = cmul(cdiv(cx(4.0 * M_PI * p.k0, 0.0), p.kb), Phi);
    h[0] = cscl(kq, pl.x);
    h[1] = cscl(kq, pl.y);
    h[2] = cscl(kq, pl.z);
    s = cscl(Phi, -4.0 * M_PI * vdot(pl, dv));
  }
  gs2[i] = s;
  for (int c = 0; c < 3; ++c) gh2[3 * i + c] = h[c];
}

// right-hand side w = dJ/dx of the scattering cross section (scattering.m:14-31,
// farfield.m:15-74) and its explicit dependence on the face positions and
// areas through Phi_di = exp(-i k n_d . r_i) A_i, from the far fields e_d, h_d
// of the forward solve on the sphere at infinity (directions n_d, weights
// area_d, c_d = area_d / nb):
//   g_h2_i  = sum_d c_d Phi_di [i k0 (h_d* x n_d) + i k ((n_d x e_d*) x n_d)]
//   g_sig2_i = -i k sum_d c_d Phi_di n_d . (h_d* x n_d)
__global__ void k_adj_rhs_sca(AdjParams p, const double2* fields, const double* inf_nvec, const double* inf_area,
                              int ninf, int P, int ip, double nb, const double2* x2, double2* gs2, double2* gh2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  double2 s = cx(0, 0), h[3] = {cx(0, 0), cx(0, 0), cx(0, 0)};
  double3 gpos = v3(0, 0, 0);
  double garea = 0.0;
  if (p.exc_out[i]) {
    const double3 r = vld(p.pos, i);
    const double A = p.area[i];
    const double2 k = p.kb;
    const double2 ik = imul(k), ik0 = cx(0.0, p.k0);
    // forward sig2 and h2 of face i (polarisation ip); X[4..7] as in the weights
    double2 X[8];
    X[4] = x2[i * 4 * P + ip];
    for (int c = 0; c < 3; ++c) X[5 + c] = x2[i * 4 * P + P + c * P + ip];
    for (int q = 0; q < ninf; ++q) {
      const int d = P + q;
      const double3 nd = vld(inf_nvec, q);
      const double c = inf_area[q] / nb;
      double2 e[3], hh[3];
      for (int cc = 0; cc < 3; ++cc) {
        e[cc] = fields[((int64_t)d * 6 + cc) * P + ip];
        hh[cc] = fields[((int64_t)d * 6 + 3 + cc) * P + ip];
        hh[cc].y = -hh[cc].y;   // conj(h)
        e[cc].y = -e[cc].y;     // conj(e)
      }
      const double nc[3] = {nd.x, nd.y, nd.z};
      // A1 = h* x n ; B = n x e* ; A2 = B x n
      double2 A1[3], B[3], A2[3];
      for (int a = 0; a < 3; ++a) {
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        A1[a] = csub(cscl(hh[b1], nc[b2]), cscl(hh[b2], nc[b1]));
        B[a] = csub(cscl(e[b2], nc[b1]), cscl(e[b1], nc[b2]));
      }
      for (int a = 0; a < 3; ++a) {
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        A2[a] = csub(cscl(B[b1], nc[b2]), cscl(B[b2], nc[b1]));
      }
      const double2 Phi = cscl(cexpi(cscl(k, -1.0), vdot(nd, r)), A);
      const double2 cP = cscl(Phi, c);
      double2 nA1 = cx(0, 0);
      for (int a = 0; a < 3; ++a) {
        h[a] = cadd(h[a], cmul(cP, cadd(cmul(ik0, A1[a]), cmul(ik, A2[a]))));
        nA1 = cadd(nA1, cscl(A1[a], nc[a]));
      }
      s = csub(s, cmul(ik, cmul(cP, nA1)));
      // explicit: T = Phi [A1 . (i k0 h2) - i k (n . A1) sig2 + B . (i k (n x h2))]
      double2 T = csub(cx(0, 0), cmul(cmul(ik, nA1), X[4]));
      for (int a = 0; a < 3; ++a) {
        const int b1 = (a + 1) % 3, b2 = (a + 2) % 3;
        const double2 nxh = csub(cscl(X[5 + b2], nc[b1]), cscl(X[5 + b1], nc[b2]));
        T = cadd(T, cadd(cmul(A1[a], cmul(ik0, X[5 + a])), cmul(B[a], cmul(ik, nxh))));
      }
      const double2 cT = cmul(cP, T);
      gpos = vadd(gpos, vscale(nd, cmul(cscl(ik, -1.0), cT).x));
      garea += cT.x / A;
    }
  }
  gs2[i] = s;
  for (int c = 0; c < 3; ++c) gh2[3 * i + c] = h[c];
  vatomic(p.gpos, i, gpos);
  atomicAdd(p.garea + i, garea);
}

// elementwise steps of the transposed chain (per face, P = 1):
//   mode 0: gS2 += i k (L1 - L2) (n . t3)                 (after t3 = Di^T gH2')
//   mode 1: v3 = i k (L1 - L2) n t                         (t = Si^T gS2)
//   mode 2: gphi = -L1 t1 + i k L1 (n . gal),  ga = i k L1 n gDe - t3
__global__ void k_adj_chain(AdjParams p, int mode, const double2* a_in, const double2* b_in, double2* out1,
                            double2* out2, const double2* c_in) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double3 n = vld(p.nvec, i);
  const double nc[3] = {n.x, n.y, n.z};
  const double2 L1 = p.eps1[i], L2 = p.eps2[i];
  const double2 ik = cx(0.0, p.k0);
  const double2 ikL = cmul(ik, csub(L1, L2));
  if (mode == 0) {
    double2 s = cx(0, 0);
    for (int c = 0; c < 3; ++c) s = cadd(s, cscl(a_in[3 * i + c], nc[c]));
    out1[i] = cadd(out1[i], cmul(ikL, s));
  } else if (mode == 1) {
    for (int c = 0; c < 3; ++c) out1[3 * i + c] = cscl(cmul(ikL, a_in[i]), nc[c]);
  } else {
    // a_in = S1^T gDe (t1), b_in = gal, c_in = gDe; out1 = gphi, out2 = ga (holds S1^T gal on entry)
    const double2 ikL1 = cmul(ik, L1);
    double2 ngal = cx(0, 0);
    for (int c = 0; c < 3; ++c) ngal = cadd(ngal, cscl(b_in[3 * i + c], nc[c]));
    out1[i] = cadd(cscl(cmul(L1, a_in[i]), -1.0), cmul(ikL1, ngal));
    for (int c = 0; c < 3; ++c) out2[3 * i + c] = csub(cscl(cmul(ikL1, c_in[i]), nc[c]), out2[3 * i + c]);
  }
}

// elementwise steps of the transposed chain for complex type C (per face):
//   mode 0: o1 += i k0 (L1 - L2) (n . a)               a [n][3], o1 [n]
//   mode 1: o1  = i k0 (L1 - L2) n a                    a [n],    o1 [n][3]
//   mode 2: o1 += -L1 a + i k0 L1 (n . b)               (gphi)
//           o2  = d + i k0 L1 n c - o2                  (ga; o2 holds Sigma1^T gal, d = G1i^T gh1 or 0)
template <typename C>
__global__ void k_chainT(AdjParams p, int mode, const C* a, const C* b, C* o1, C* o2, const C* c, const C* d) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const double3 n = vld(p.nvec, i);
  const double nc[3] = {n.x, n.y, n.z};
  const double2 L1 = p.eps1[i], L2 = p.eps2[i];
  const double2 ik = cx(0.0, p.k0);
  const double2 ikL = cmul(ik, csub(L1, L2)), ikL1 = cmul(ik, L1);
  if (mode == 0) {
    double2 sm = cx(0, 0);
    for (int q = 0; q < 3; ++q) sm = cadd(sm, cscl(to_d(a[3 * i + q]), nc[q]));
    o1[i] = from_d<C>(cadd(to_d(o1[i]), cmul(ikL, sm)));
  } else if (mode == 1) {
    const double2 t = cmul(ikL, to_d(a[i]));
    for (int q = 0; q < 3; ++q) o1[3 * i + q] = from_d<C>(cscl(t, nc[q]));
  } else {
    double2 nb = cx(0, 0);
    for (int q = 0; q < 3; ++q) nb = cadd(nb, cscl(to_d(b[3 * i + q]), nc[q]));
    o1[i] = from_d<C>(cadd(to_d(o1[i]), csub(cmul(ikL1, nb), cmul(L1, to_d(a[i])))));
    const double2 t = cmul(ikL1, to_d(c[i]));
    for (int q = 0; q < 3; ++q) {
      const double2 dv = d ? to_d(d[3 * i + q]) : cx(0, 0);
      o2[3 * i + q] = from_d<C>(csub(cadd(dv, cscl(t, nc[q])), to_d(o2[3 * i + q])));
    }
  }
}

// y[N cols] partial sums of (Ahi + Alo)^T V over row chunk blockIdx.y:
// thread = column j (coalesced row reads), double-single accumulation
// (error-free products, TwoSum), partial [chunks][n][N] in FP64
struct DSa { float hi, lo; };
__device__ __forceinline__ void dsa_acc(DSa& s, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  const float t = s.hi + p;
  const float bp = t - s.hi;
  const float err = (s.hi - (t - bp)) + (p - bp);
  s.hi = t;
  s.lo += err + e;
}
template <int N>
__global__ void __launch_bounds__(128) k_gemm_t_ds(int64_t n, int64_t rows_per_chunk, const float2* __restrict__ Ahi,
                                                   const float2* __restrict__ Alo, int64_t lda,
                                                   const float2* __restrict__ Vh, const float2* __restrict__ Vl,
                                                   double2* __restrict__ part) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per_chunk, r1 = min(n, r0 + rows_per_chunk);
  DSa re[N], im[N];
  for (int c = 0; c < N; ++c) re[c] = im[c] = DSa{0.f, 0.f};
  for (int64_t i = r0; i < r1; ++i) {
    const float2 ah = Ahi[i * lda + j], al = Alo[i * lda + j];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const float2 vh = Vh[i * N + c], vl = Vl[i * N + c];
      dsa_acc(re[c], ah.x, vh.x);
      dsa_acc(re[c], -ah.y, vh.y);
      dsa_acc(im[c], ah.x, vh.y);
      dsa_acc(im[c], ah.y, vh.x);
      re[c].lo += (ah.x * vl.x - ah.y * vl.y) + (al.x * vh.x - al.y * vh.y);
      im[c].lo += (ah.x * vl.y + ah.y * vl.x) + (al.x * vh.y + al.y * vh.x);
    }
  }
  for (int c = 0; c < N; ++c)
    part[((int64_t)blockIdx.y * n + j) * N + c] =
        make_double2((double)re[c].hi + (double)re[c].lo, (double)im[c].hi + (double)im[c].lo);
}

__global__ void k_parts_sum(const double2* part, int chunks, int64_t count, double2* y, int accumulate) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  double2 sm = accumulate ? y[i] : cx(0, 0);
  for (int q = 0; q < chunks; ++q) sm = cadd(sm, part[q * count + i]);
  y[i] = sm;
}

// hi / lo complex64 planes of a strided complex128 source: dst[i][c] = src[i * stride + off + c]
__global__ void k_split_strided(const double2* src, int64_t n, int stride, int off, int N, float2* hi, float2* lo) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * N) return;
  const int64_t i = t / N;
  const int c = (int)(t % N);
  const double2 v = src[i * stride + off + c];
  const float2 h = make_float2((float)v.x, (float)v.y);
  hi[t] = h;
  lo[t] = make_float2((float)(v.x - (double)h.x), (float)(v.y - (double)h.y));
}

// r = w - [y1 ; y2] in the unknown layout (sig1 [n], h1 [n][3], sig2 [n], h2 [n][3]);
// y1, y2 [n][4] = (sig, h); w has zero sig1 / h1; norms[0] += |r|^2
__global__ void k_adj_resid(int64_t n, const double2* y1, const double2* y2, const double2* ws2, const double2* wh2,
                            double2* rs1, double2* rh1, double2* rs2, double2* rh2, double* norms) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (i < n) {
    double2 v = cscl(y1[4 * i], -1.0);
    rs1[i] = v;
    acc += cabs2(v);
    v = csub(ws2[i], y2[4 * i]);
    rs2[i] = v;
    acc += cabs2(v);
    for (int c = 0; c < 3; ++c) {
      v = cscl(y1[4 * i + 1 + c], -1.0);
      rh1[3 * i + c] = v;
      acc += cabs2(v);
      v = csub(wh2[3 * i + c], y2[4 * i + 1 + c]);
      rh2[3 * i + c] = v;
      acc += cabs2(v);
    }
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(norms, acc);
}

}  // namespace

void adj_transpose(double2* A, int64_t n, int64_t ld, cudaStream_t st) {
  dim3 g((unsigned)cdiv_up(n, 32), (unsigned)cdiv_up(n, 32));
  k_transpose_sq<double2><<<g, dim3(32, 8), 0, st>>>(A, n, ld);
}
void adj_transpose(float2* A, int64_t n, int64_t ld, cudaStream_t st) {
  dim3 g((unsigned)cdiv_up(n, 32), (unsigned)cdiv_up(n, 32));
  k_transpose_sq<float2><<<g, dim3(32, 8), 0, st>>>(A, n, ld);
}

void adj_rhs(const AdjParams& p, const double* pol, const double* dir, double2* gs2, double2* gh2, cudaStream_t st) {
  k_adj_rhs<<<(unsigned)cdiv_up(p.n, 128), 128, 0, st>>>(p, pol, dir, gs2, gh2);
}

void adj_rhs_sca(const AdjParams& p, const double2* fields, const double* inf_nvec, const double* inf_area,
                 int ninf, int P, int ip, double nb, const double2* x2, double2* gs2, double2* gh2, cudaStream_t st) {
  k_adj_rhs_sca<<<(unsigned)cdiv_up(p.n, 64), 64, 0, st>>>(p, fields, inf_nvec, inf_area, ninf, P, ip, nb, x2, gs2,
                                                           gh2);
}

void adj_chain_step(const AdjParams& p, int mode, const double2* a, const double2* b, double2* o1, double2* o2,
                    const double2* c, cudaStream_t st) {
  k_adj_chain<<<(unsigned)cdiv_up(p.n, 128), 128, 0, st>>>(p, mode, a, b, o1, o2, c);
}

template <typename C>
void adj_chainT(const AdjParams& p, int mode, const C* a, const C* b, C* o1, C* o2, const C* c, const C* d,
                cudaStream_t st) {
  k_chainT<C><<<(unsigned)cdiv_up(p.n, 128), 128, 0, st>>>(p, mode, a, b, o1, o2, c, d);
}
template void adj_chainT<float2>(const AdjParams&, int, const float2*, const float2*, float2*, float2*,
                                 const float2*, const float2*, cudaStream_t);
template void adj_chainT<double2>(const AdjParams&, int, const double2*, const double2*, double2*, double2*,
                                  const double2*, const double2*, cudaStream_t);

void adj_gemm_t_ds(int64_t n, const float2* Ahi, const float2* Alo, int64_t lda, const double2* V, int stride,
                   int off, float2* vsplit, double2* part, int chunks, double2* y, cudaStream_t st, bool accumulate) {
  const int N = 4;
  float2* Vh = vsplit;
  float2* Vl = vsplit + n * N;
  k_split_strided<<<(unsigned)cdiv_up(n * N, 256), 256, 0, st>>>(V, n, stride, off, N, Vh, Vl);
  const int64_t rpc = cdiv_up(n, (int64_t)chunks);
  dim3 g((unsigned)cdiv_up(n, 128), (unsigned)chunks);
  k_gemm_t_ds<4><<<g, 128, 0, st>>>(n, rpc, Ahi, Alo, lda, Vh, Vl, part);
  k_parts_sum<<<(unsigned)cdiv_up(n * N, 256), 256, 0, st>>>(part, chunks, n * N, y, accumulate ? 1 : 0);
}

void adj_resid(int64_t n, const double2* y1, const double2* y2, const double2* ws2, const double2* wh2, double2* rs1,
               double2* rh1, double2* rs2, double2* rh2, double* norms, cudaStream_t st) {
  k_adj_resid<<<(unsigned)cdiv_up(n, 128), 128, 0, st>>>(n, y1, y2, ws2, wh2, rs1, rh1, rs2, rh2, norms);
}

void adj_weights(const AdjParams& p, const double2* lphi, const double2* la, const double2* lDe,
                 const double2* lal, const double2* x1, const double2* x2, int P, int ip, cudaStream_t st) {
  k_adj_weights<<<(unsigned)cdiv_up(p.n, 128), 128, 0, st>>>(p, lphi, la, lDe, lal, x1, x2, P, ip);
}

void adj_geometry(const AdjParams& p, int which, const double* pol, const double* dir, const double2* lphi,
                  const double2* la, const double2* lDe, const double2* lal, const double2* GX1,
                  const double2* GX2, const double2* HX1, double* geps, cudaStream_t st) {
  ProfScope ps(PH_ASSEMBLE, st, 0.0, 0.0, 5);
  dim3 g((unsigned)cdiv_up(p.n, PG_COLS), (unsigned)cdiv_up(p.n, PG_ROWS));
  k_adj_pairs<<<g, PG_COLS, 0, st>>>(p);
  if (p.noff > 0) k_adj_near<<<(unsigned)cdiv_up(p.noff, 64), 64, 0, st>>>(p);
  k_adj_self<<<(unsigned)cdiv_up(p.n, 64), 64, 0, st>>>(p);
  k_adj_faces<<<(unsigned)cdiv_up(p.n, 128), 128, 0, st>>>(p, which, pol, dir, lphi, la, lDe, lal, GX1, GX2, HX1,
                                                           geps);
  k_adj_norm_flat<<<(unsigned)cdiv_up(p.n, 128), 128, 0, st>>>(p);
}

}  // namespace mnpbem
