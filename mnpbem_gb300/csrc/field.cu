// Electric and magnetic fields at points off the particle boundary: the
// Green function between a set of points (Particles/@compoint) and the
// particle, and Greenfun/@compgreenret/field.m:17-38
//     E = i k0 (G1 h1 + G2 h2) - (Gp1 sig1 + Gp2 sig2),  H = Gp1 x h1 + Gp2 x h2,
// where side 1 (2) collects the faces whose inside (outside) medium is the
// point's medium and G, Gp = grad G use that medium's wavenumber.  Points
// closer than RelCutoff element radii to a face (refinematrix.m:27-67 with the
// face's radius) take the refined Taylor coefficients of the (point, face)
// pair (Greenfun/@greenret/private/init.m:98-177), as the face pairs do.
#include "field.cuh"
#include "geom_dev.cuh"
#include "profile.cuh"

namespace mnpbem {

constexpr int FLD_MAXPOL = 4;

__device__ __forceinline__ int pt_flag(double3 p, const GeomDev& g, int j, double rel_cut, double abs_cut) {
  const double3 v = sub3(p, ld3(g.pos, j));
  const double d2 = sqrt(dot3(v, v)) - g.rad[j];
  return (d2 < abs_cut || d2 / g.rad[j] < rel_cut) ? 1 : 0;
}

// one warp per point: number of refined faces
__global__ void k_pt_count(int64_t m, const double* __restrict__ pts, GeomDev g, double rel_cut, double abs_cut,
                           int* counts) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= m) return;
  const double3 p = ld3(pts, w);
  int cnt = 0;
  for (int j0 = 0; j0 < g.n; j0 += 32) {
    const int j = j0 + lane;
    const int fl = j < g.n ? pt_flag(p, g, j, rel_cut, abs_cut) : 0;
    cnt += __popc(__ballot_sync(0xffffffffu, fl != 0));
  }
  if (lane == 0) counts[w] = cnt;
}

// one warp per point: refined faces in ascending order (rows of the CSR lists)
__global__ void k_pt_fill(int64_t m, const double* __restrict__ pts, GeomDev g, double rel_cut, double abs_cut,
                          const int64_t* __restrict__ offs, int* prow, int* pcol) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= m) return;
  const double3 p = ld3(pts, w);
  int64_t base = offs[w];
  for (int j0 = 0; j0 < g.n; j0 += 32) {
    const int j = j0 + lane;
    const int fl = j < g.n ? pt_flag(p, g, j, rel_cut, abs_cut) : 0;
    const unsigned msk = __ballot_sync(0xffffffffu, fl != 0);
    if (fl) {
      const int64_t at = base + __popc(msk & ((1u << lane) - 1u));
      prow[at] = (int)w;
      pcol[at] = j;
    }
    base += __popc(msk);
  }
}

__global__ void k_pt_coef(int64_t npair, const double* __restrict__ pts, GeomDev g, const int* __restrict__ prow,
                          const int* __restrict__ pcol, double* cg, double* cf) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npair) return;
  const int O = g.order;
  near_coefficients(g, ld3(pts, prow[t]), pcol[t], cg + t * (O + 1), cf + t * 3 * (O + 1));
}

struct FieldArgs {
  GeomDev g;
  const int* face_med;   // [2][n]
  const double* pts;
  const int* pt_med;     // 0-based
  const double2* kmed;
  double k0;
  int npol;
  const double2 *sig1, *sig2, *h1, *h2;
  const int64_t* offs;
  const int* pcol;
  const double *cg, *cf;
  double2 *e, *h;
};

// one block per point
__global__ void __launch_bounds__(128) k_pt_field(FieldArgs a) {
  const int64_t i = blockIdx.x;
  const GeomDev& g = a.g;
  const int n = g.n, O = g.order, P = a.npol;
  const int med = a.pt_med[i];
  const double2 k = a.kmed[med];
  const double2 ik = make_double2(-k.y, k.x);
  const double3 p = ld3(a.pts, i);
  const int64_t r0 = a.offs[i], r1 = a.offs[i + 1];
  double2 E[3][FLD_MAXPOL], H[3][FLD_MAXPOL];
  for (int c = 0; c < 3; ++c)
    for (int q = 0; q < FLD_MAXPOL; ++q) E[c][q] = H[c][q] = make_double2(0, 0);
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const bool s1 = a.face_med[j] == med, s2 = a.face_med[n + j] == med;
    if (!s1 && !s2) continue;
    const double3 v = sub3(p, ld3(g.pos, j));
    const double d = fmax(sqrt(dot3(v, v)), DBL_EPS);
    double sn, cs;
    sincos(k.x * d, &sn, &cs);
    const double ee = exp(-k.y * d);
    const double2 ph = make_double2(ee * cs, ee * sn);
    // refined pair?  (faces of row i are sorted ascending)
    int64_t lo = r0, hi = r1;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (a.pcol[mid] < j) lo = mid + 1; else hi = mid;
    }
    double2 G, Gp[3];
    if (lo < r1 && a.pcol[lo] == j) {
      const double* cg = a.cg + lo * (O + 1);
      const double* cf = a.cf + lo * 3 * (O + 1);
      double2 pw = make_double2(1, 0), gs = make_double2(0, 0), fs[3] = {gs, gs, gs};
      for (int o = 0; o <= O; ++o) {
        gs.x += cg[o] * pw.x; gs.y += cg[o] * pw.y;
        for (int c = 0; c < 3; ++c) { fs[c].x += cf[c * (O + 1) + o] * pw.x; fs[c].y += cf[c * (O + 1) + o] * pw.y; }
        pw = cmul(pw, ik);
      }
      G = cmul(gs, ph);
      for (int c = 0; c < 3; ++c) Gp[c] = cmul(fs[c], ph);
    } else {
      const double A = g.area[j], inv = 1.0 / d;
      G = make_double2(A * inv * ph.x, A * inv * ph.y);
      // (ik - 1/d) / d^2 * A * (p - pos_j)
      const double2 t = cmul(make_double2(-k.y - inv, k.x), ph);
      const double s = A * inv * inv;
      const double vc[3] = {v.x, v.y, v.z};
      for (int c = 0; c < 3; ++c) Gp[c] = make_double2(t.x * s * vc[c], t.y * s * vc[c]);
    }
    const double2 ik0G = make_double2(-a.k0 * G.y, a.k0 * G.x);
    for (int side = 0; side < 2; ++side) {
      if (!(side == 0 ? s1 : s2)) continue;
      const double2* sg = side == 0 ? a.sig1 : a.sig2;
      const double2* hh = side == 0 ? a.h1 : a.h2;
      for (int q = 0; q < P; ++q) {
        const double2 sv = sg[(int64_t)j * P + q];
        double2 hv[3];
        for (int c = 0; c < 3; ++c) hv[c] = hh[((int64_t)j * 3 + c) * P + q];
        for (int c = 0; c < 3; ++c) E[c][q] = csub(cadd(E[c][q], cmul(ik0G, hv[c])), cmul(Gp[c], sv));
        H[0][q] = cadd(H[0][q], csub(cmul(Gp[1], hv[2]), cmul(Gp[2], hv[1])));
        H[1][q] = cadd(H[1][q], csub(cmul(Gp[2], hv[0]), cmul(Gp[0], hv[2])));
        H[2][q] = cadd(H[2][q], csub(cmul(Gp[0], hv[1]), cmul(Gp[1], hv[0])));
      }
    }
  }
  // block reduction (fixed order): warp shuffles, then the four warps in order
  __shared__ double2 red[4][6 * FLD_MAXPOL];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = 0; c < 6; ++c)
    for (int q = 0; q < P; ++q) {
      double2 v = c < 3 ? E[c][q] : H[c - 3][q];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[wid][c * FLD_MAXPOL + q] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < 6 * P; t += blockDim.x) {
    const int c = t / P, q = t % P;
    double2 s = make_double2(0, 0);
    for (int w = 0; w < 4; ++w) s = cadd(s, red[w][c * FLD_MAXPOL + q]);
    double2* out = c < 3 ? a.e : a.h;
    out[(i * 3 + (c % 3)) * P + q] = s;
  }
}

mnpbem_status point_fields(const GeomDev& g, const int* face_med, int64_t npts, const double* pts,
                           const int* pt_med, const double2* kmed, int nmed, double k0, int npol,
                           const double2* sig1, const double2* sig2, const double2* h1, const double2* h2,
                           double2* e, double2* h, double rel_cut, double abs_cut, cudaStream_t st) {
  if (npts <= 0) return MNPBEM_OK;
  if (npol < 1 || npol > FLD_MAXPOL) { set_error("fields: npol must be 1..%d", FLD_MAXPOL); return MNPBEM_ERR_UNSUPPORTED; }
  if (npts > (int64_t)1 << 30) { set_error("fields: too many points"); return MNPBEM_ERR_UNSUPPORTED; }
  ProfScope ps(PH_SPECTRA, st, 0.0, 0.0, 4);
  DevBuf d_pts, d_med, d_k, counts, offs, pairs, coef;
  MNP_TRY(d_pts.ensure(sizeof(double) * 3 * npts));
  MNP_TRY(d_med.ensure(sizeof(int) * npts));
  MNP_TRY(d_k.ensure(sizeof(double2) * nmed));
  MNP_TRY(counts.ensure(sizeof(int) * npts));
  std::vector<int> med0(npts);
  for (int64_t i = 0; i < npts; ++i) {
    if (pt_med[i] < 1 || pt_med[i] > nmed) { set_error("fields: point %lld has an invalid medium", (long long)i); return MNPBEM_ERR_INVALID_ARG; }
    med0[i] = pt_med[i] - 1;
  }
  MNP_CUDA(cudaMemcpyAsync(d_pts.ptr, pts, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(d_med.ptr, med0.data(), sizeof(int) * npts, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(d_k.ptr, kmed, sizeof(double2) * nmed, cudaMemcpyHostToDevice, st));
  const unsigned wblk = (unsigned)cdiv_up(npts, (int64_t)8);
  k_pt_count<<<wblk, 256, 0, st>>>(npts, d_pts.as<double>(), g, rel_cut, abs_cut, counts.as<int>());
  MNP_CHECK_LAUNCH();
  std::vector<int> hc(npts);
  MNP_CUDA(cudaMemcpyAsync(hc.data(), counts.ptr, sizeof(int) * npts, cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  std::vector<int64_t> ho(npts + 1, 0);
  for (int64_t i = 0; i < npts; ++i) ho[i + 1] = ho[i] + hc[i];
  const int64_t npair = ho[npts];
  const int O = g.order;
  MNP_TRY(offs.ensure(sizeof(int64_t) * (npts + 1)));
  MNP_TRY(pairs.ensure(sizeof(int) * 2 * std::max<int64_t>(npair, 1)));
  MNP_TRY(coef.ensure(sizeof(double) * 4 * (O + 1) * std::max<int64_t>(npair, 1)));
  MNP_CUDA(cudaMemcpyAsync(offs.ptr, ho.data(), sizeof(int64_t) * (npts + 1), cudaMemcpyHostToDevice, st));
  int* prow = pairs.as<int>();
  int* pcol = prow + std::max<int64_t>(npair, 1);
  double* cg = coef.as<double>();
  double* cf = cg + (O + 1) * std::max<int64_t>(npair, 1);
  if (npair > 0) {
    k_pt_fill<<<wblk, 256, 0, st>>>(npts, d_pts.as<double>(), g, rel_cut, abs_cut, offs.as<int64_t>(), prow, pcol);
    MNP_CHECK_LAUNCH();
    k_pt_coef<<<(unsigned)cdiv_up(npair, (int64_t)128), 128, 0, st>>>(npair, d_pts.as<double>(), g, prow, pcol, cg, cf);
    MNP_CHECK_LAUNCH();
  }
  FieldArgs a;
  a.g = g; a.face_med = face_med; a.pts = d_pts.as<double>(); a.pt_med = d_med.as<int>();
  a.kmed = d_k.as<double2>(); a.k0 = k0; a.npol = npol;
  a.sig1 = sig1; a.sig2 = sig2; a.h1 = h1; a.h2 = h2;
  a.offs = offs.as<int64_t>(); a.pcol = pcol; a.cg = cg; a.cf = cf; a.e = e; a.h = h;
  k_pt_field<<<(unsigned)npts, 128, 0, st>>>(a);
  MNP_CHECK_LAUNCH();
  MNP_CUDA(cudaStreamSynchronize(st));   // the temporary buffers are released on return
  return MNPBEM_OK;
}

// ------------------------------------------------------------------------
// Fields and potentials on the boundary itself (Greenfun/@compgreenret/
// field.m:14-38 and potential.m:16-48 with p1 = p2 = the particle): the
// observation point of row i is face i's centroid on side `side` (0 inside,
// 1 outside), its medium face_med[side][i].  Per pair (i, j)
//     Hp = Gp + s 2 pi n_i [d == 0]      (H1p, s = +1, inside; H2p, s = -1)
//     E  = i k0 (G h1 + G h2) - Hp sig1 - Hp sig2,   H = Hp x h1 + Hp x h2
//     phi = G sig,  phip = (n_i . Hp) sig,  a = G h,  ap = (n_i . Hp) h
// over the faces j whose side-1 (side-2) medium is the observation medium;
// n_i . Hp equals F +- 2 pi [d == 0], the H1 / H2 of eval1.m:140-143.  Refined
// pairs use the face-pair Taylor coefficients of the geometry (column j's rows
// are ascending: binary search), including the closed-surface diagonal.

struct SurfArgs {
  GeomDev g;
  const int* face_med;   // [2][n] 0-based
  const double2* kmed;
  double k0;
  int npol, side;
  const double2 *sig1, *sig2, *h1, *h2;
  double2 *e, *h;               // [n][3][npol]      (field pass)
  double2 *phi, *phip, *a, *ap; // [n][npol], [n][3][npol] (potential pass)
};

__device__ __forceinline__ void surf_pair(const SurfArgs& a, int i, int j, double3 p, double3 ni, double2 k,
                                          double2 ik, double2& G, double2* Hp) {
  const GeomDev& g = a.g;
  const int O = g.order;
  const double3 v = sub3(p, ld3(g.pos, j));
  const double dt = sqrt(dot3(v, v));
  const double d = fmax(dt, DBL_EPS);
  double sn, cs;
  sincos(k.x * d, &sn, &cs);
  const double ee = exp(-k.y * d);
  const double2 ph = make_double2(ee * cs, ee * sn);
  int64_t lo = g.col_off[j], hi = g.col_off[j + 1];
  const int64_t end = hi;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (g.ref_row[mid] < i) lo = mid + 1; else hi = mid;
  }
  if (lo < end && g.ref_row[lo] == i) {
    const double* cg = g.ref_g + lo * (O + 1);
    const double* cf = g.ref_f + lo * 3 * (O + 1);
    double2 pw = make_double2(1, 0), gs = make_double2(0, 0), fs[3] = {gs, gs, gs};
    for (int o = 0; o <= O; ++o) {
      gs.x += cg[o] * pw.x; gs.y += cg[o] * pw.y;
      for (int c = 0; c < 3; ++c) { fs[c].x += cf[c * (O + 1) + o] * pw.x; fs[c].y += cf[c * (O + 1) + o] * pw.y; }
      pw = cmul(pw, ik);
    }
    G = cmul(gs, ph);
    for (int c = 0; c < 3; ++c) Hp[c] = cmul(fs[c], ph);
  } else {
    const double A = g.area[j], inv = 1.0 / d;
    G = make_double2(A * inv * ph.x, A * inv * ph.y);
    const double2 t = cmul(make_double2(-k.y - inv, k.x), ph);
    const double s = A * inv * inv;
    const double vc[3] = {v.x, v.y, v.z};
    for (int c = 0; c < 3; ++c) Hp[c] = make_double2(t.x * s * vc[c], t.y * s * vc[c]);
  }
  if (dt <= DBL_EPS) {     // d == 0 after d = max(d, eps): the +-2 pi term
    const double tp = a.side == 0 ? 2 * M_PI : -2 * M_PI;
    Hp[0].x += tp * ni.x; Hp[1].x += tp * ni.y; Hp[2].x += tp * ni.z;
  }
}

// one block (4 warps) per observation face; POT selects the potential pass
template <bool POT>
__global__ void __launch_bounds__(128) k_surf(SurfArgs a) {
  constexpr int NC = POT ? 8 : 6;   // phi, phip, a(3), ap(3)  |  E(3), H(3)
  const int i = blockIdx.x;
  const GeomDev& g = a.g;
  const int n = g.n, P = a.npol;
  const int med = a.face_med[a.side * n + i];
  const double2 k = a.kmed[med];
  const double2 ik = make_double2(-k.y, k.x);
  const double3 p = ld3(g.pos, i), ni = ld3(g.nvec, i);
  double2 acc[NC][FLD_MAXPOL];
  for (int c = 0; c < NC; ++c)
    for (int q = 0; q < FLD_MAXPOL; ++q) acc[c][q] = make_double2(0, 0);
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const bool s1 = a.face_med[j] == med, s2 = a.face_med[n + j] == med;
    if (!s1 && !s2) continue;
    double2 G, Hp[3];
    surf_pair(a, i, j, p, ni, k, ik, G, Hp);
    const double2 Hn = cadd(cadd(make_double2(ni.x * Hp[0].x, ni.x * Hp[0].y),
                                 make_double2(ni.y * Hp[1].x, ni.y * Hp[1].y)),
                            make_double2(ni.z * Hp[2].x, ni.z * Hp[2].y));
    const double2 ik0G = make_double2(-a.k0 * G.y, a.k0 * G.x);
    for (int sd = 0; sd < 2; ++sd) {
      if (!(sd == 0 ? s1 : s2)) continue;
      const double2* sg = sd == 0 ? a.sig1 : a.sig2;
      const double2* hh = sd == 0 ? a.h1 : a.h2;
#pragma unroll
      for (int q = 0; q < FLD_MAXPOL; ++q) {
        if (q >= P) break;
        const double2 sv = sg[(int64_t)j * P + q];
        double2 hv[3];
        for (int c = 0; c < 3; ++c) hv[c] = hh[((int64_t)j * 3 + c) * P + q];
        if (POT) {
          acc[0][q] = cadd(acc[0][q], cmul(G, sv));
          acc[1][q] = cadd(acc[1][q], cmul(Hn, sv));
          for (int c = 0; c < 3; ++c) {
            acc[2 + c][q] = cadd(acc[2 + c][q], cmul(G, hv[c]));
            acc[5 + c][q] = cadd(acc[5 + c][q], cmul(Hn, hv[c]));
          }
        } else {
          for (int c = 0; c < 3; ++c) acc[c][q] = csub(cadd(acc[c][q], cmul(ik0G, hv[c])), cmul(Hp[c], sv));
          acc[3][q] = cadd(acc[3][q], csub(cmul(Hp[1], hv[2]), cmul(Hp[2], hv[1])));
          acc[4][q] = cadd(acc[4][q], csub(cmul(Hp[2], hv[0]), cmul(Hp[0], hv[2])));
          acc[5][q] = cadd(acc[5][q], csub(cmul(Hp[0], hv[1]), cmul(Hp[1], hv[0])));
        }
      }
    }
  }
  // fixed-order block reduction: warp shuffles, then the four warps in order
  __shared__ double2 red[4][NC * FLD_MAXPOL];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; ++c)
#pragma unroll
    for (int q = 0; q < FLD_MAXPOL; ++q) {
      double2 v = acc[c][q];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[wid][c * FLD_MAXPOL + q] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < NC * P; t += blockDim.x) {
    const int c = t / P, q = t % P;
    double2 s = make_double2(0, 0);
    for (int w = 0; w < 4; ++w) s = cadd(s, red[w][c * FLD_MAXPOL + q]);
    double2* out;
    int64_t at;
    if (POT) {
      if (c < 2) { out = c == 0 ? a.phi : a.phip; at = (int64_t)i * P + q; }
      else { out = c < 5 ? a.a : a.ap; at = ((int64_t)i * 3 + (c - 2) % 3) * P + q; }
    } else {
      out = c < 3 ? a.e : a.h;
      at = ((int64_t)i * 3 + c % 3) * P + q;
    }
    if (out) out[at] = s;
  }
}

mnpbem_status surface_fields(const GeomDev& g, const int* face_med, const double2* kmed, double k0, int npol,
                             int side, const double2* sig1, const double2* sig2, const double2* h1,
                             const double2* h2, double2* e, double2* h, double2* phi, double2* phip,
                             double2* av, double2* ap, cudaStream_t st) {
  if (g.n <= 0) return MNPBEM_OK;
  if (npol < 1 || npol > FLD_MAXPOL) { set_error("surface fields: npol must be 1..%d", FLD_MAXPOL); return MNPBEM_ERR_UNSUPPORTED; }
  if (side != 0 && side != 1) { set_error("surface fields: inout must be 1 or 2"); return MNPBEM_ERR_INVALID_ARG; }
  ProfScope ps(PH_SPECTRA, st, 0.0, 0.0, (e || h) && (phi || phip || av || ap) ? 2 : 1);
  SurfArgs a;
  a.g = g; a.face_med = face_med; a.kmed = kmed; a.k0 = k0; a.npol = npol; a.side = side;
  a.sig1 = sig1; a.sig2 = sig2; a.h1 = h1; a.h2 = h2;
  a.e = e; a.h = h; a.phi = phi; a.phip = phip; a.a = av; a.ap = ap;
  if (e || h) {
    k_surf<false><<<(unsigned)g.n, 128, 0, st>>>(a);
    MNP_CHECK_LAUNCH();
  }
  if (phi || phip || av || ap) {
    k_surf<true><<<(unsigned)g.n, 128, 0, st>>>(a);
    MNP_CHECK_LAUNCH();
  }
  return MNPBEM_OK;
}

// ------------------------------------------------------------------------
// Far fields of the surface charges and currents in given directions
// (Simulation/retarded/@spectrumret/farfield.m:15-74): with the phase
// ph_j = exp(-i k dir . r_j) A_j over the faces whose inside (outside) medium
// is the embedding medium, through sig1 / h1 (sig2 / h2),
//     e = i k0 sum ph h - i k dir sum ph sig,   h = i k dir x sum ph h.
struct FarArgs {
  GeomDev g;
  const int* face_med;   // [2][n] 0-based
  int med;               // 0-based embedding medium
  double2 k;             // its wavenumber
  double k0;
  int npol;
  const double* dirs;    // [ndir][3]
  const double2 *sig1, *sig2, *h1, *h2;
  double2 *e, *h;        // [ndir][3][npol]
};

// one block (4 warps) per direction
__global__ void __launch_bounds__(128) k_far_dirs(FarArgs a) {
  const int d = blockIdx.x;
  const GeomDev& g = a.g;
  const int n = g.n, P = a.npol;
  const double3 dv = ld3(a.dirs, d);
  double2 acc[4][FLD_MAXPOL];   // sum ph sig, sum ph h (3)
  for (int c = 0; c < 4; ++c)
    for (int q = 0; q < FLD_MAXPOL; ++q) acc[c][q] = make_double2(0, 0);
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const bool s1 = a.face_med[j] == a.med, s2 = a.face_med[n + j] == a.med;
    if (!s1 && !s2) continue;
    const double s = dot3(dv, ld3(g.pos, j));
    double sn, cs;
    sincos(a.k.x * s, &sn, &cs);
    const double ee = exp(a.k.y * s) * g.area[j];
    const double2 ph = make_double2(ee * cs, -ee * sn);
    for (int sd = 0; sd < 2; ++sd) {
      if (!(sd == 0 ? s1 : s2)) continue;
      const double2* sg = sd == 0 ? a.sig1 : a.sig2;
      const double2* hh = sd == 0 ? a.h1 : a.h2;
#pragma unroll
      for (int q = 0; q < FLD_MAXPOL; ++q) {
        if (q >= P) break;
        acc[0][q] = cadd(acc[0][q], cmul(ph, sg[(int64_t)j * P + q]));
        for (int c = 0; c < 3; ++c) acc[1 + c][q] = cadd(acc[1 + c][q], cmul(ph, hh[((int64_t)j * 3 + c) * P + q]));
      }
    }
  }
  __shared__ double2 red[4][4 * FLD_MAXPOL];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int q = 0; q < FLD_MAXPOL; ++q) {
      double2 v = acc[c][q];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[wid][c * FLD_MAXPOL + q] = v;
    }
  __syncthreads();
  if (threadIdx.x < P) {
    const int q = threadIdx.x;
    double2 S[4];
    for (int c = 0; c < 4; ++c) {
      S[c] = make_double2(0, 0);
      for (int w = 0; w < 4; ++w) S[c] = cadd(S[c], red[w][c * FLD_MAXPOL + q]);
    }
    const double2 ik = make_double2(-a.k.y, a.k.x), ik0 = make_double2(0, a.k0);
    const double dd[3] = {dv.x, dv.y, dv.z};
    if (a.e)
      for (int c = 0; c < 3; ++c)
        a.e[((int64_t)d * 3 + c) * P + q] = csub(cmul(ik0, S[1 + c]), cmul(ik, make_double2(dd[c] * S[0].x, dd[c] * S[0].y)));
    if (a.h) {
      // i k dir x Ph
      const double2 c0 = csub(make_double2(dd[1] * S[3].x, dd[1] * S[3].y), make_double2(dd[2] * S[2].x, dd[2] * S[2].y));
      const double2 c1 = csub(make_double2(dd[2] * S[1].x, dd[2] * S[1].y), make_double2(dd[0] * S[3].x, dd[0] * S[3].y));
      const double2 c2 = csub(make_double2(dd[0] * S[2].x, dd[0] * S[2].y), make_double2(dd[1] * S[1].x, dd[1] * S[1].y));
      a.h[((int64_t)d * 3 + 0) * P + q] = cmul(ik, c0);
      a.h[((int64_t)d * 3 + 1) * P + q] = cmul(ik, c1);
      a.h[((int64_t)d * 3 + 2) * P + q] = cmul(ik, c2);
    }
  }
}

mnpbem_status far_fields(const GeomDev& g, const int* face_med, int med, double2 k, double k0, int npol,
                         int ndir, const double* dirs, const double2* sig1, const double2* sig2,
                         const double2* h1, const double2* h2, double2* e, double2* h, cudaStream_t st) {
  if (ndir <= 0 || g.n <= 0) return MNPBEM_OK;
  if (npol < 1 || npol > FLD_MAXPOL) { set_error("far fields: npol must be 1..%d", FLD_MAXPOL); return MNPBEM_ERR_UNSUPPORTED; }
  ProfScope ps(PH_SPECTRA, st, 0.0, 0.0, 1);
  FarArgs a;
  a.g = g; a.face_med = face_med; a.med = med; a.k = k; a.k0 = k0; a.npol = npol; a.dirs = dirs;
  a.sig1 = sig1; a.sig2 = sig2; a.h1 = h1; a.h2 = h2; a.e = e; a.h = h;
  k_far_dirs<<<(unsigned)ndir, 128, 0, st>>>(a);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

}  // namespace mnpbem
