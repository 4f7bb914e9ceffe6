// Excitation, the bemret solution chain, the FP64 residual of the full BEM
// operator, and the far-field cross sections.
#include "bem.cuh"
#include "farfield.cuh"
#include "dense.cuh"
#include "profile.cuh"

namespace mnpbem {

constexpr int MAXPOL = 4;

template <typename R> __device__ __forceinline__ cplx<R> cvt(double2 v) { return from_d<cplx<R>>(v); }

// ------------------------------------------------------------- excitation
__global__ void k_excitation(FaceData f, int P, const double* __restrict__ pol,
                             const double* __restrict__ dir, const LamParams* __restrict__ lp,
                             double2* phi, double2* a, double2* alpha, double2* De) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n) return;
  const double2 k = lp->kexc;
  const double k0 = lp->k0;
  double px = f.pos[3 * i], py = f.pos[3 * i + 1], pz = f.pos[3 * i + 2];
  double nx = f.nvec[3 * i], ny = f.nvec[3 * i + 1], nz = f.nvec[3 * i + 2];
  bool in1 = f.exc_in[i] != 0, in2 = f.exc_out[i] != 0;
  double2 e1 = f.eps1[i], e2 = f.eps2[i];
  for (int p = 0; p < P; ++p) {
    const double* d = dir + 3 * p;
    const double* q = pol + 3 * p;
    double s = px * d[0] + py * d[1] + pz * d[2];
    double sn, cs;
    sincos(k.x * s, &sn, &cs);
    double ee = exp(-k.y * s);
    // exp(i k s) / (i k0)
    double2 ph = make_double2(ee * sn / k0, -ee * cs / k0);
    double nd = nx * d[0] + ny * d[1] + nz * d[2];
    double2 ikn = make_double2(-k.y * nd, k.x * nd);   // i k (n . dir)
    double2 php = cmul(ikn, ph);
    double2 na1 = make_double2(0, 0), na2 = make_double2(0, 0);
    for (int c = 0; c < 3; ++c) {
      double2 a1 = in1 ? cscale(ph, q[c]) : make_double2(0, 0);
      double2 a2 = in2 ? cscale(ph, q[c]) : make_double2(0, 0);
      double2 a1p = in1 ? cscale(php, q[c]) : make_double2(0, 0);
      double2 a2p = in2 ? cscale(php, q[c]) : make_double2(0, 0);
      a[(i * 3 + c) * P + p] = csub(a2, a1);
      alpha[(i * 3 + c) * P + p] = csub(a2p, a1p);
      double nc = c == 0 ? nx : (c == 1 ? ny : nz);
      na1 = cadd(na1, cscale(a1, nc));
      na2 = cadd(na2, cscale(a2, nc));
    }
    phi[i * P + p] = make_double2(0, 0);
    // De = -i k0 (eps2 n.a2 - eps1 n.a1)
    double2 t = csub(cmul(e2, na2), cmul(e1, na1));
    De[i * P + p] = make_double2(k0 * t.y, -k0 * t.x);
  }
}

void launch_excitation(const FaceData& f, int P, const double* pol, const double* dir,
                       const LamParams* lp, double2* phi, double2* a, double2* alpha,
                       double2* De, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  k_excitation<<<(unsigned)cdiv_up(f.n, 128), 128, 0, st>>>(f, P, pol, dir, lp, phi, a, alpha, De);
}

// External potentials (compstruct exc of any excitation, e.g. dipoleret)
// -> excitation variables (BEM/@bemret/private/excitation.m, Garcia de Abajo
// and Howie Eqs. 10, 11, 15, 18):
//   phi = phi2 - phi1,  a = a2 - a1,
//   alpha = a2p - a1p - i k0 (n eps2 phi2 - n eps1 phi1),
//   De = eps2 phi2p - eps1 phi1p - i k0 (n . eps2 a2 - n . eps1 a1).
// pot: phi1, phi1p, phi2, phi2p [n][P] then a1, a1p, a2, a2p [n][3][P].
__global__ void k_excitation_ext(FaceData f, int P, const double2* __restrict__ pot,
                                 const LamParams* __restrict__ lp, double2* phi, double2* a, double2* alpha,
                                 double2* De) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n) return;
  const int64_t n = f.n;
  const double k0 = lp->k0;
  const double2 e1 = f.eps1[i], e2 = f.eps2[i];
  const double nv[3] = {f.nvec[3 * i], f.nvec[3 * i + 1], f.nvec[3 * i + 2]};
  const double2 *p1 = pot, *p1p = pot + n * P, *p2 = pot + 2 * n * P, *p2p = pot + 3 * n * P;
  const double2 *a1 = pot + 4 * n * P, *a1p = a1 + 3 * n * P, *a2 = a1 + 6 * n * P, *a2p = a1 + 9 * n * P;
  for (int p = 0; p < P; ++p) {
    const int64_t s = i * P + p;
    phi[s] = csub(p2[s], p1[s]);
    const double2 ep2 = cmul(e2, p2[s]), ep1 = cmul(e1, p1[s]);
    double2 na1 = make_double2(0, 0), na2 = make_double2(0, 0);
    for (int c = 0; c < 3; ++c) {
      const int64_t v = (i * 3 + c) * P + p;
      a[v] = csub(a2[v], a1[v]);
      // - i k0 n_c (eps2 phi2 - eps1 phi1)
      const double2 t = cscale(csub(ep2, ep1), nv[c]);
      alpha[v] = cadd(csub(a2p[v], a1p[v]), make_double2(k0 * t.y, -k0 * t.x));
      na1 = cadd(na1, cscale(a1[v], nv[c]));
      na2 = cadd(na2, cscale(a2[v], nv[c]));
    }
    const double2 t = csub(cmul(e2, na2), cmul(e1, na1));
    De[s] = cadd(csub(cmul(e2, p2p[s]), cmul(e1, p1p[s])), make_double2(k0 * t.y, -k0 * t.x));
  }
}

void launch_excitation_ext(const FaceData& f, int P, const double2* pot, const LamParams* lp, double2* phi,
                           double2* a, double2* alpha, double2* De, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  k_excitation_ext<<<(unsigned)cdiv_up(f.n, 128), 128, 0, st>>>(f, P, pot, lp, phi, a, alpha, De);
}

__global__ void k_face_eps(int64_t n, const int* __restrict__ med_in, const int* __restrict__ med_out,
                           const LamParams* __restrict__ lp, const double* __restrict__ nvec, double2* eps1,
                           double2* eps2, float2* eps1f, float2* eps2f, float2* Lf, float* nvecf) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 a = lp->eps[med_in[i]], b = lp->eps[med_out[i]];
  eps1[i] = a;
  eps2[i] = b;
  eps1f[i] = to_f(a);
  eps2f[i] = to_f(b);
  Lf[i] = to_f(csub(a, b));
  for (int c = 0; c < 3; ++c) nvecf[3 * i + c] = (float)nvec[3 * i + c];
}

void launch_face_eps(int64_t n, const int* med_in, const int* med_out, const LamParams* lp,
                     const double* nvec, double2* eps1, double2* eps2, float2* eps1f, float2* eps2f,
                     float2* Lf, float* nvecf, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  k_face_eps<<<(unsigned)cdiv_up(n, 256), 256, 0, st>>>(n, med_in, med_out, lp, nvec, eps1, eps2, eps1f,
                                                         eps2f, Lf, nvecf);
}

// ------------------------------------------------------ mldivide chain steps
template <typename R>
__global__ void k_chain_pre(FaceData f, int P, const cplx<R>* phi, const cplx<R>* a, cplx<R>* X4) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n) return;
  cplx<R> L1 = cvt<R>(f.eps1[i]);
  const int W = 4 * P;
  for (int p = 0; p < P; ++p) X4[i * W + p] = cmul(L1, phi[i * P + p]);
  for (int c = 0; c < 3 * P; ++c) X4[i * W + P + c] = a[i * 3 * P + c];
}

// alpha' = alpha - Sigma1 a + ik n (x) (L1 phi);  De' = De - Sigma1 (L1 phi) + ik n . (L1 a)
template <typename R>
__global__ void k_chain_alpha_de(FaceData f, int P, const LamParams* lp, const cplx<R>* phi, const cplx<R>* a,
                                 const cplx<R>* alpha, const cplx<R>* De, const cplx<R>* T4,
                                 cplx<R>* al, cplx<R>* Dp) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n) return;
  cplx<R> L1 = cvt<R>(f.eps1[i]);
  R n[3] = {(R)f.nvec[3 * i], (R)f.nvec[3 * i + 1], (R)f.nvec[3 * i + 2]};
  const int W = 4 * P;
  cplx<R> ik = mk<R>(0, (R)lp->k0);
  for (int p = 0; p < P; ++p) {
    cplx<R> lphi = cmul(L1, phi[i * P + p]);
    cplx<R> na = mk<R>(0, 0);
    for (int c = 0; c < 3; ++c) {
      int64_t idx = (i * 3 + c) * P + p;
      cplx<R> v = csub(alpha[idx], T4[i * W + P + c * P + p]);
      v = cadd(v, cmul(ik, cscale(lphi, n[c])));
      al[idx] = v;
      na = cadd(na, cscale(a[idx], n[c]));
    }
    cplx<R> d = csub(De[i * P + p], T4[i * W + p]);
    Dp[i * P + p] = cadd(d, cmul(ik, cmul(L1, na)));
  }
}

// u = De' + ik n . ((L1 - L2) t)
template <typename R>
__global__ void k_chain_u(FaceData f, int P, const LamParams* lp, const cplx<R>* Dp, const cplx<R>* t3, cplx<R>* u) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n) return;
  cplx<R> L = csub(cvt<R>(f.eps1[i]), cvt<R>(f.eps2[i]));
  R n[3] = {(R)f.nvec[3 * i], (R)f.nvec[3 * i + 1], (R)f.nvec[3 * i + 2]};
  cplx<R> ik = mk<R>(0, (R)lp->k0);
  for (int p = 0; p < P; ++p) {
    cplx<R> nt = mk<R>(0, 0);
    for (int c = 0; c < 3; ++c) nt = cadd(nt, cscale(t3[(i * 3 + c) * P + p], n[c]));
    u[i * P + p] = cadd(Dp[i * P + p], cmul(ik, cmul(L, nt)));
  }
}

// v = ik n (x) ((L1 - L2) sig2) + alpha'
template <typename R>
__global__ void k_chain_v(FaceData f, int P, const LamParams* lp, const cplx<R>* s2, const cplx<R>* al, cplx<R>* v3) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.n) return;
  cplx<R> L = csub(cvt<R>(f.eps1[i]), cvt<R>(f.eps2[i]));
  R n[3] = {(R)f.nvec[3 * i], (R)f.nvec[3 * i + 1], (R)f.nvec[3 * i + 2]};
  cplx<R> ik = mk<R>(0, (R)lp->k0);
  for (int p = 0; p < P; ++p) {
    cplx<R> ls = cmul(ik, cmul(L, s2[i * P + p]));
    for (int c = 0; c < 3; ++c) {
      int64_t idx = (i * 3 + c) * P + p;
      v3[idx] = cadd(cscale(ls, n[c]), al[idx]);
    }
  }
}

// Y = [sig2 + phi | h2 + a],  Z = [sig2 | h2]
template <typename R>
__global__ void k_chain_y(int64_t n, int P, const cplx<R>* s2, const cplx<R>* h2, const cplx<R>* phi,
                          const cplx<R>* a, cplx<R>* Y4, cplx<R>* Z4) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int W = 4 * P;
  for (int p = 0; p < P; ++p) {
    Y4[i * W + p] = cadd(s2[i * P + p], phi[i * P + p]);
    Z4[i * W + p] = s2[i * P + p];
  }
  for (int c = 0; c < 3 * P; ++c) {
    Y4[i * W + P + c] = cadd(h2[i * 3 * P + c], a[i * 3 * P + c]);
    Z4[i * W + P + c] = h2[i * 3 * P + c];
  }
}

template <typename R>
mnpbem_status apply_mldivide(const FaceData& f, int P, const LamParams* lp, const ChainMats<R>& m,
                             const cplx<R>* phi, const cplx<R>* a, const cplx<R>* alpha,
                             const cplx<R>* De, cplx<R>* x1, cplx<R>* x2, cplx<R>* work,
                             ChainGemm<R> gemm, void* ctx, cudaStream_t st) {
  using Cx = cplx<R>;
  const int64_t n = f.n;
  Cx* X4 = work;
  Cx* T4 = X4 + n * 4 * P;
  Cx* al = T4 + n * 4 * P;
  Cx* Dp = al + n * 3 * P;
  Cx* t3 = Dp + n * P;
  Cx* u = t3 + n * 3 * P;
  Cx* s2 = u + n * P;
  Cx* v3 = s2 + n * P;
  Cx* h2 = v3 + n * 3 * P;
  (void)s2;
  const Cx one = mk<R>(1, 0), zero = mk<R>(0, 0);
  unsigned nb = (unsigned)cdiv_up(n, 128);
  if (Profiler* pr = current_profiler()) pr->acc[PH_ELEMWISE].launches += 5;
  k_chain_pre<R><<<nb, 128, 0, st>>>(f, P, phi, a, X4);
  MNP_CHECK_LAUNCH();
  // Sigma1 = H1 G1^-1 shares G1's diagonal blocks
  for (int q = 0; q < m.ng1; ++q) {
    const int64_t o = m.g1_off[q];
    MNP_TRY(gemm(m.g1_n[q], 4 * P, m.g1_n[q], one, m.Sigma1 + o * m.ld + o, m.ld, X4 + o * 4 * P, 4 * P, zero,
                 T4 + o * 4 * P, 4 * P, st, ctx));
  }
  k_chain_alpha_de<R><<<nb, 128, 0, st>>>(f, P, lp, phi, a, alpha, De, T4, al, Dp);
  MNP_CHECK_LAUNCH();
  MNP_TRY(gemm(n, 3 * P, n, one, m.Deltai, m.ld, al, 3 * P, zero, t3, 3 * P, st, ctx));
  k_chain_u<R><<<nb, 128, 0, st>>>(f, P, lp, Dp, t3, u);
  MNP_CHECK_LAUNCH();
  // sig2 = Sigma \ u (in place)
  MNP_TRY(ldu_solve<R>(m.Sigma, n, m.ld, m.b, u, P, P, nullptr, gemm, ctx, st, m.bar));
  s2 = u;
  k_chain_v<R><<<nb, 128, 0, st>>>(f, P, lp, s2, al, v3);
  MNP_CHECK_LAUNCH();
  MNP_TRY(gemm(n, 3 * P, n, one, m.Deltai, m.ld, v3, 3 * P, zero, h2, 3 * P, st, ctx));
  // x1 = G1 \ [sig2 + phi | h2 + a], x2 = G2 \ [sig2 | h2]
  k_chain_y<R><<<nb, 128, 0, st>>>(n, P, s2, h2, phi, a, x1, x2);
  MNP_CHECK_LAUNCH();
  for (int q = 0; q < m.ng1; ++q)
    MNP_TRY(ldu_solve<R>(m.G1 + m.g1_off[q] * m.ld + m.g1_off[q], m.g1_n[q], m.ld, m.b, x1 + m.g1_off[q] * 4 * P,
                         4 * P, 4 * P, nullptr, gemm, ctx, st, m.bar));
  MNP_TRY(ldu_solve<R>(m.G2, n, m.ld, m.b, x2, 4 * P, 4 * P, nullptr, gemm, ctx, st, m.bar));
  return MNPBEM_OK;
}
template mnpbem_status apply_mldivide<float>(const FaceData&, int, const LamParams*, const ChainMats<float>&,
                                             const float2*, const float2*, const float2*,
                                             const float2*, float2*, float2*, float2*,
                                             ChainGemm<float>, void*, cudaStream_t);
template mnpbem_status apply_mldivide<double>(const FaceData&, int, const LamParams*, const ChainMats<double>&,
                                              const double2*, const double2*, const double2*,
                                              const double2*, double2*, double2*, double2*,
                                              ChainGemm<double>, void*, cudaStream_t);

// ------------------------------------------------------------ FP64 residual
__device__ __forceinline__ void block_add2(double v0, double v1, double* norms) {
  for (int o = 16; o; o >>= 1) {
    v0 += __shfl_xor_sync(0xffffffffu, v0, o);
    v1 += __shfl_xor_sync(0xffffffffu, v1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(norms, v0);
    atomicAdd(norms + 1, v1);
  }
}

__global__ void k_residual(FaceData f, int P, const LamParams* lp, const double2* Y1, const double2* Y2,
                           const double2* Z1, const double2* Z2, const double2* phi,
                           const double2* a, const double2* alpha, const double2* De,
                           double2* rphi, double2* ra, double2* ralpha, double2* rDe,
                           double* norms) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double rr = 0.0, bb = 0.0;
  if (i < f.n) {
    const int W = 4 * P;
    double2 e1 = f.eps1[i], e2 = f.eps2[i];
    double n[3] = {f.nvec[3 * i], f.nvec[3 * i + 1], f.nvec[3 * i + 2]};
    double2 ik = make_double2(0, lp->k0);
    for (int p = 0; p < P; ++p) {
      double2 y1s = Y1[i * W + p], y2s = Y2[i * W + p];
      double2 z1s = Z1[i * W + p], z2s = Z2[i * W + p];
      double2 es = csub(cmul(e1, y1s), cmul(e2, y2s));
      double2 nh = make_double2(0, 0);
      for (int c = 0; c < 3; ++c) {
        int64_t col = P + c * P + p;
        double2 y1h = Y1[i * W + col], y2h = Y2[i * W + col];
        double2 z1h = Z1[i * W + col], z2h = Z2[i * W + col];
        int64_t idx = (i * 3 + c) * P + p;
        double2 av = csub(y1h, y2h);
        double2 alv = csub(csub(z1h, z2h), cmul(ik, cscale(es, n[c])));
        double2 r1 = csub(a[idx], av), r2 = csub(alpha[idx], alv);
        ra[idx] = r1; ralpha[idx] = r2;
        rr += cabs2(r1) + cabs2(r2);
        bb += cabs2(a[idx]) + cabs2(alpha[idx]);
        nh = cadd(nh, cscale(csub(cmul(e1, y1h), cmul(e2, y2h)), n[c]));
      }
      double2 pv = csub(y1s, y2s);
      double2 dv = csub(csub(cmul(e1, z1s), cmul(e2, z2s)), cmul(ik, nh));
      double2 r0 = csub(phi[i * P + p], pv), r3 = csub(De[i * P + p], dv);
      rphi[i * P + p] = r0; rDe[i * P + p] = r3;
      rr += cabs2(r0) + cabs2(r3);
      bb += cabs2(phi[i * P + p]) + cabs2(De[i * P + p]);
    }
  }
  block_add2(rr, bb, norms);
}

void launch_residual(const FaceData& f, int P, const LamParams* lp, const double2* Y1, const double2* Y2,
                     const double2* Z1, const double2* Z2, const double2* phi, const double2* a,
                     const double2* alpha, const double2* De, double2* rphi, double2* ra,
                     double2* ralpha, double2* rDe, double* norms, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  k_residual<<<(unsigned)cdiv_up(f.n, 128), 128, 0, st>>>(f, P, lp, Y1, Y2, Z1, Z2, phi, a, alpha,
                                                         De, rphi, ra, ralpha, rDe, norms);
}

// ------------------------------------------------------------ conversions
__global__ void k_d2f(const double2* in, float2* out, int64_t cnt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) out[i] = to_f(in[i]);
}
__global__ void k_f2d(const float2* in, double2* out, int64_t cnt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) out[i] = to_d(in[i]);
}
void launch_cvt_d2f(const double2* in, float2* out, int64_t count, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  if (count > 0) k_d2f<<<(unsigned)cdiv_up(count, 256), 256, 0, st>>>(in, out, count);
}
void launch_cvt_f2d(const float2* in, double2* out, int64_t count, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  if (count > 0) k_f2d<<<(unsigned)cdiv_up(count, 256), 256, 0, st>>>(in, out, count);
}

template <typename C>
__global__ void k_axpy_norm(double2* x, const C* dx, int64_t cnt, double* norms) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double a = 0.0, b = 0.0;
  if (i < cnt) {
    double2 d = to_d(dx[i]);
    double2 v = cadd(x[i], d);
    x[i] = v;
    a = cabs2(d); b = cabs2(v);
  }
  block_add2(a, b, norms);
}
void launch_axpy_norm(double2* x, const float2* dx, int64_t count, double* norms, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  if (count > 0) k_axpy_norm<float2><<<(unsigned)cdiv_up(count, 256), 256, 0, st>>>(x, dx, count, norms);
}
void launch_axpy_norm(double2* x, const double2* dx, int64_t count, double* norms, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  if (count > 0) k_axpy_norm<double2><<<(unsigned)cdiv_up(count, 256), 256, 0, st>>>(x, dx, count, norms);
}

// ------------------------------------------------------------ Sigma stage
// per-face values in the working precision of the kernel
template <typename R> struct FaceVals;
template <> struct FaceVals<float> {
  const float2 *e1, *e2, *L;
  const float* nv;
  __host__ explicit FaceVals(const FaceData& f) : e1(f.eps1f), e2(f.eps2f), L(f.Lf), nv(f.nvecf) {}
};
template <> struct FaceVals<double> {
  const double2 *e1, *e2;
  const double* nv;
  __host__ explicit FaceVals(const FaceData& f) : e1(f.eps1), e2(f.eps2), nv(f.nvec) {}
};
__device__ __forceinline__ float2 face_L(const FaceVals<float>& v, int64_t i) { return v.L[i]; }
__device__ __forceinline__ double2 face_L(const FaceVals<double>& v, int64_t i) { return csub(v.e1[i], v.e2[i]); }

template <typename R>
__global__ void k_delta_sigma(int64_t n, const cplx<R>* S1, cplx<R>* S2, cplx<R>* D, int64_t ld,
                              FaceVals<R> fv) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t i = blockIdx.y;
  if (j >= n) return;
  cplx<R> s1 = S1[i * ld + j], s2 = S2[i * ld + j];
  D[i * ld + j] = csub(s1, s2);
  S2[i * ld + j] = csub(cmul(s1, fv.e1[j]), cmul(s2, fv.e2[j]));
}
template <typename R>
void launch_delta_sigma(int64_t n, const cplx<R>* S1, cplx<R>* S2_to_S, cplx<R>* D, int64_t ld,
                        const FaceData& f, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  dim3 grid((unsigned)cdiv_up(n, 256), (unsigned)n);
  k_delta_sigma<R><<<grid, 256, 0, st>>>(n, S1, S2_to_S, D, ld, FaceVals<R>(f));
}
template void launch_delta_sigma<float>(int64_t, const float2*, float2*, float2*, int64_t, const FaceData&,
                                        cudaStream_t);
template void launch_delta_sigma<double>(int64_t, const double2*, double2*, double2*, int64_t,
                                         const FaceData&, cudaStream_t);

// S_ij += k0^2 L_i Deltai_ij (n_i . n_j) L_j
template <typename R>
__global__ void k_sigma_add(int64_t n, cplx<R>* S, const cplx<R>* Di, int64_t ld, FaceVals<R> fv,
                            const LamParams* lp) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t i = blockIdx.y;
  if (j >= n) return;
  const R k2 = (R)(lp->k0 * lp->k0);
  const cplx<R> Li = face_L(fv, i), Lj = face_L(fv, j);
  const R nn = fv.nv[3 * i] * fv.nv[3 * j] + fv.nv[3 * i + 1] * fv.nv[3 * j + 1] + fv.nv[3 * i + 2] * fv.nv[3 * j + 2];
  cplx<R> t = cmul(cmul(Li, Di[i * ld + j]), mk<R>(nn, 0));
  t = cmul(t, Lj);
  S[i * ld + j] = cadd(S[i * ld + j], cscale(t, k2));
}
template <typename R>
void launch_sigma_add(int64_t n, cplx<R>* S, const cplx<R>* Di, int64_t ld, const FaceData& f,
                      const LamParams* lp, cudaStream_t st) {
  ProfScope ps_(PH_ELEMWISE, st, 0.0, 0.0, 1);
  dim3 grid((unsigned)cdiv_up(n, 256), (unsigned)n);
  k_sigma_add<R><<<grid, 256, 0, st>>>(n, S, Di, ld, FaceVals<R>(f), lp);
}
template void launch_sigma_add<float>(int64_t, float2*, const float2*, int64_t, const FaceData&,
                                      const LamParams*, cudaStream_t);
template void launch_sigma_add<double>(int64_t, double2*, const double2*, int64_t, const FaceData&,
                                       const LamParams*, cudaStream_t);

// ------------------------------------------------------------- far fields
// charges and currents packed per face: [n][4P] of (sig | h) for each side
struct PackedSrc {
  const double2 *x1, *x2;
  int P;
  __device__ double2 sig(int side, int64_t j, int p) const { return (side ? x2 : x1)[j * 4 * P + p]; }
  __device__ double2 h(int side, int64_t j, int c, int p) const { return (side ? x2 : x1)[j * 4 * P + P + c * P + p]; }
};

__global__ void __launch_bounds__(256) k_farfield(FaceData f, int P, const double2* x1,
                                                  const double2* x2, const double* dirs,
                                                  const LamParams* lp, double2* fields) {
  const int d = blockIdx.x;
  farfield_dir<MAXPOL>(f.n, P, f.pos, f.area, f.exc_in, f.exc_out, PackedSrc{x1, x2, P}, dirs[3 * d],
                       dirs[3 * d + 1], dirs[3 * d + 2], lp->kexc, lp->k0, d, fields);
}

void launch_farfield(const FaceData& f, int P, const double2* x1, const double2* x2,
                     const double* dirs, int ndir, const LamParams* lp, double2* fields,
                     cudaStream_t st) {
  ProfScope ps_(PH_SPECTRA, st, 0.0, 0.0, 1);
  k_farfield<<<ndir, 256, 0, st>>>(f, P, x1, x2, dirs, lp, fields);
}

__device__ __forceinline__ void cross_sections_body(int P, const double* pol, const double* inf_nvec,
                                                    const double* inf_area, int ninf,
                                                    const double2* fields, double2 k, double2 nb1,
                                                    double* ext, double* sca) {
  __shared__ double red[256];
  for (int p = 0; p < P; ++p) {
    double acc = 0.0;
    for (int d = threadIdx.x; d < ninf; d += blockDim.x) {
      const double2* F = fields + (int64_t)(P + d) * 6 * P;
      double2 e[3], h[3];
      for (int c = 0; c < 3; ++c) { e[c] = F[c * P + p]; h[c] = F[(3 + c) * P + p]; h[c].y = -h[c].y; }
      // e x conj(h)
      double2 cr0 = csub(cmul(e[1], h[2]), cmul(e[2], h[1]));
      double2 cr1 = csub(cmul(e[2], h[0]), cmul(e[0], h[2]));
      double2 cr2 = csub(cmul(e[0], h[1]), cmul(e[1], h[0]));
      const double* nv = inf_nvec + 3 * d;
      double ds = 0.5 * (nv[0] * cr0.x + nv[1] * cr1.x + nv[2] * cr2.x);
      acc += inf_area[d] * ds;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      // sca / (0.5 nb), real part
      double2 den = make_double2(0.5 * nb1.x, 0.5 * nb1.y);
      sca[p] = cdiv(make_double2(red[0], 0), den).x;
      // ext = 4 pi / k * imag(pol . e(dir_p))
      const double2* F = fields + (int64_t)p * 6 * P;
      double im = 0.0;
      for (int c = 0; c < 3; ++c) im += pol[3 * p + c] * F[c * P + p].y;
      ext[p] = cdiv(make_double2(4.0 * M_PI * im, 0), k).x;
    }
    __syncthreads();
  }
}

__global__ void k_cross_sections(int P, const double* pol, const double* inf_nvec,
                                 const double* inf_area, int ninf, const double2* fields,
                                 double2 k, double2 nb1, double* ext, double* sca) {
  cross_sections_body(P, pol, inf_nvec, inf_area, ninf, fields, k, nb1, ext, sca);
}

__global__ void k_cross_sections_lp(int P, const double* pol, const double* inf_nvec,
                                    const double* inf_area, int ninf, const double2* fields,
                                    const LamParams* lp, double* ext, double* sca) {
  const int w = lp->w;
  cross_sections_body(P, pol, inf_nvec, inf_area, ninf, fields, lp->kexc, lp->nb1, ext + (int64_t)w * P,
                      sca + (int64_t)w * P);
}

void launch_cross_sections_lp(int P, const double* pol, const double* inf_nvec,
                              const double* inf_area, int ninf, const double2* fields,
                              const LamParams* lp, double* ext, double* sca, cudaStream_t st) {
  ProfScope ps_(PH_SPECTRA, st, 0.0, 0.0, 1);
  k_cross_sections_lp<<<1, 256, 0, st>>>(P, pol, inf_nvec, inf_area, ninf, fields, lp, ext, sca);
}

void launch_cross_sections(int P, const double* pol, const double* inf_nvec, const double* inf_area,
                           int ninf, const double2* fields, double2 k_med, double2 nb1,
                           double* ext, double* sca, cudaStream_t st) {
  ProfScope ps_(PH_SPECTRA, st, 0.0, 0.0, 1);
  k_cross_sections<<<1, 256, 0, st>>>(P, pol, inf_nvec, inf_area, ninf, fields, k_med, nb1, ext, sca);
}

}  // namespace mnpbem
