// Per-wavelength assembly of the bemret matrices (compgreenret eval, FP64 math).
//
//  k_asm_far   Greenfun/@greenret/private/eval1.m:24-40 (G) and :110-124 (F, 'cart'),
//              H1/H2 = F +- 2 pi [d == 0] (:141-143), combined per particle block as in
//              Greenfun/@compgreenret/private/eval1.m:16-34 and BEM/@bemret/private/initmat.m:27-31
//  k_asm_near  the refined elements: G = sum_o g_o (ik)^o, F = sum_o (n_i . f_o) (ik)^o,
//              both times exp(ik d) (eval1.m:36-39, 119-123)
//
// One pass writes G1, H1, G2, H2 as complex128 and/or complex64 (row-major, ld).
#include "assemble.cuh"
#include "profile.cuh"

namespace mnpbem {

struct PairVal { double2 G, F; };

// ------------------------------------------------------- exp(i k d), FP64
// Table-driven evaluation (Cody-Waite argument reduction + short Taylor
// polynomials), a few FP64 FMAs per call instead of a library sincos and exp:
//   phase  th = Re(k) d = j (2 pi / 256) + t,  |t| <= pi / 256:
//          cis(th) = cis(2 pi j / 256) * (cos t + i sin t), Taylor to t^8;
//   decay  x = Im(k) d = y (ln 2 / 64) + u,   |u| <= ln 2 / 128:
//          exp(-x) = 2^(-floor(y/64)) * 2^(-(y mod 64)/64) * exp(-u), Taylor to u^7.
// The reduction constants are split in a 32-bit head (exact products with
// |j| < 2^20) and a tail; the tables come from the device's sincospi / exp2
// once per device.  Accuracy: a few ulp of the FP64 result.
constexpr int CIS_N = 256;
constexpr double CIS_INV = 40.74366543152521;        // 256 / (2 pi)
constexpr double CIS_C1 = 0.024543692605220713;      // 2 pi / 256, head
constexpr double CIS_C2 = 9.495469541415925e-13;     // 2 pi / 256, tail
constexpr double EXP_INV = 92.33248261689366;        // 64 / ln 2
constexpr double EXP_L1 = 0.01083042469326756;       // ln 2 / 64, head
constexpr double EXP_L2 = 2.9815858269852933e-12;    // ln 2 / 64, tail

struct CisTable {
  double2 cs[CIS_N];   // (cos, sin)(2 pi j / 256)
  double e2[64];       // 2^(-m / 64)
};
__device__ CisTable g_cis;

__global__ void k_cis_init() {
  const int j = threadIdx.x;
  double s, c;
  sincospi(2.0 * j / CIS_N, &s, &c);
  g_cis.cs[j] = make_double2(c, s);
  if (j < 64) g_cis.e2[j] = exp2(-j / 64.0);
}

struct CisShared {
  double2 cs[CIS_N];
  double e2[64];
};

__device__ __forceinline__ void cis_load(CisShared& t) {
  for (int q = threadIdx.x; q < CIS_N; q += blockDim.x) t.cs[q] = g_cis.cs[q];
  for (int q = threadIdx.x; q < 64; q += blockDim.x) t.e2[q] = g_cis.e2[q];
  __syncthreads();
}

// exp(i k d) for complex k (Im k >= 0 for passive media; any sign works)
__device__ __forceinline__ double2 cis_exp(const CisShared& T, double2 k, double d) {
  const double th = k.x * d;
  const double jf = rint(th * CIS_INV);
  const double t = fma(-jf, CIS_C2, fma(-jf, CIS_C1, th));
  const double t2 = t * t;
  const double sn = t * fma(t2, fma(t2, fma(t2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), 1.0);
  const double cn = fma(t2, fma(t2, fma(t2, fma(t2, 1.0 / 40320.0, -1.0 / 720.0), 1.0 / 24.0), -0.5), 1.0);
  const double2 tb = T.cs[((long long)jf) & (CIS_N - 1)];
  double cr = tb.x * cn - tb.y * sn;
  double sr = fma(tb.y, cn, tb.x * sn);
  if (k.y != 0.0) {
    const double x = k.y * d;
    double e;
    if (x > 700.0) {
      e = 0.0;
    } else {
      const double yf = rint(x * EXP_INV);
      const double u = fma(-yf, EXP_L2, fma(-yf, EXP_L1, x));
      const double v = -u;
      const double ev = fma(v, fma(v, fma(v, fma(v, fma(v, fma(v, fma(v, 1.0 / 5040.0, 1.0 / 720.0), 1.0 / 120.0),
                                                          1.0 / 24.0), 1.0 / 6.0), 0.5), 1.0), 1.0);
      const long long yi = (long long)yf;
      const long long nn = yi >> 6;                 // floor(y / 64)
      const int m = (int)(yi - (nn << 6));
      const double scale = __longlong_as_double((unsigned long long)(1023 - nn) << 52);   // 2^(-nn)
      e = ev * T.e2[m] * scale;
    }
    cr *= e;
    sr *= e;
  }
  return make_double2(cr, sr);
}

static bool g_cis_ready[64];
static mnpbem_status ensure_cis(cudaStream_t st) {
  int dev = 0;
  MNP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_error("device index out of range"); return MNPBEM_ERR_INVALID_ARG; }
  if (!g_cis_ready[dev]) {
    k_cis_init<<<1, CIS_N, 0, st>>>();
    MNP_CHECK_LAUNCH();
    if (!capturing_now()) g_cis_ready[dev] = true;
  }
  return MNPBEM_OK;
}

// G and F of one pair for wavenumber k (far-field formula); inv = 1 / d
__device__ __forceinline__ PairVal far_pair(const CisShared& T, double2 k, double dd, double inv, double in,
                                            double area) {
  const double2 ph = cis_exp(T, k, dd);
  const double ga = area * inv;
  PairVal v;
  v.G = make_double2(ga * ph.x, ga * ph.y);
  // (ik - 1/d) / d^2 * (n . r) * area
  const double inv2 = inv * inv;
  const double fa = in * area;
  const double2 tf = make_double2((-k.y - inv) * inv2 * fa, k.x * inv2 * fa);
  v.F = cmul(tf, ph);
  return v;
}

__device__ __forceinline__ void store_split(float2* hi, float2* lo, int64_t o, double2 v) {
  const float2 h = to_f(v);
  hi[o] = h;
  lo[o] = make_float2((float)(v.x - (double)h.x), (float)(v.y - (double)h.y));
}

template <bool W64, bool W32>
__device__ __forceinline__ void store4(const AsmParams& p, int64_t i, int64_t j, double2 g1, double2 h1,
                                       double2 g2, double2 h2) {
  if (W64 && W32) {
    int64_t o = i * p.ld32 + j;
    const float2 a = to_f(g1), b = to_f(h1), c = to_f(g2), d = to_f(h2);
    p.g1[o] = a; p.h1[o] = b; p.g2[o] = c; p.h2[o] = d;
    store_split(p.G1hi, p.G1lo, o, g1);
    store_split(p.H1hi, p.H1lo, o, h1);
    store_split(p.G2hi, p.G2lo, o, g2);
    store_split(p.H2hi, p.H2lo, o, h2);
    return;
  }
  if (W64) {
    int64_t o = i * p.ld64 + j;
    if (p.G1) p.G1[o] = g1;
    if (p.H1) p.H1[o] = h1;
    if (p.G2) p.G2[o] = g2;
    if (p.H2) p.H2[o] = h2;
  }
  if (W32) {
    int64_t o = i * p.ld32 + j;
    if (p.g1) p.g1[o] = to_f(g1);
    if (p.h1) p.h1[o] = to_f(h1);
    if (p.g2) p.g2[o] = to_f(g2);
    if (p.h2) p.h2[o] = to_f(h2);
  }
}

constexpr int ASM_COLS = 128;
constexpr int ASM_ROWS = 4;

template <bool W64, bool W32>
__global__ void __launch_bounds__(ASM_COLS) k_asm_far(AsmParams p) {
  __shared__ CisShared T;
  cis_load(T);
  int64_t j = (int64_t)blockIdx.x * ASM_COLS + threadIdx.x;
  int64_t i0 = (int64_t)blockIdx.y * ASM_ROWS;
  if (j >= p.n) return;
  double4_32a sj = p.src[j];
  int pj = p.part[j];
  const double twopi = 2.0 * M_PI;
#pragma unroll
  for (int r = 0; r < ASM_ROWS; ++r) {
    int64_t i = i0 + r;
    if (i >= p.n) break;
    double4_32a si = p.src[i];
    double4_32a ni = p.nrm[i];
    double x = si.x - sj.x, y = si.y - sj.y, z = si.z - sj.z;
    double dist = sqrt(x * x + y * y + z * z);
    double dd = fmax(dist, DBL_EPS_ASM);
    double delta = (dd == DBL_EPS_ASM) ? twopi : 0.0;
    double inv = 1.0 / dd;
    double in = x * ni.x + y * ni.y + z * ni.z;
    int pi = p.part[i];
    int m11 = p.med[0][pi][pj], m21 = p.med[1][pi][pj], m22 = p.med[2][pi][pj], m12 = p.med[3][pi][pj];
    double2 g1 = make_double2(0, 0), h1 = g1, g2 = g1, h2 = g1;
    if (m11) { PairVal v = far_pair(T, p.lp->k[m11 - 1], dd, inv, in, sj.w); g1 = v.G; h1 = make_double2(v.F.x + delta, v.F.y); }
    if (m21) { PairVal v = far_pair(T, p.lp->k[m21 - 1], dd, inv, in, sj.w); g1 = csub(g1, v.G); h1 = csub(h1, make_double2(v.F.x + delta, v.F.y)); }
    if (m22) { PairVal v = far_pair(T, p.lp->k[m22 - 1], dd, inv, in, sj.w); g2 = v.G; h2 = make_double2(v.F.x - delta, v.F.y); }
    if (m12) { PairVal v = far_pair(T, p.lp->k[m12 - 1], dd, inv, in, sj.w); g2 = csub(g2, v.G); h2 = csub(h2, make_double2(v.F.x - delta, v.F.y)); }
    store4<W64, W32>(p, i, j, g1, h1, g2, h2);
  }
}

// refined value for wavenumber k
__device__ __forceinline__ PairVal near_pair(const AsmParams& p, int64_t e, double2 k, double dd,
                                             double3 ni) {
  const int O = p.order;
  const double* g = p.ref_g + e * (O + 1);
  const double* f = p.ref_f + e * 3 * (O + 1);
  double2 ik = make_double2(-k.y, k.x);
  double2 pw = make_double2(1.0, 0.0);
  double2 G = make_double2(0, 0), F = make_double2(0, 0);
  for (int o = 0; o <= O; ++o) {
    double fo = ni.x * f[o] + ni.y * f[(O + 1) + o] + ni.z * f[2 * (O + 1) + o];
    G.x += g[o] * pw.x; G.y += g[o] * pw.y;
    F.x += fo * pw.x; F.y += fo * pw.y;
    pw = cmul(pw, ik);
  }
  double s, c;
  sincos(k.x * dd, &s, &c);
  double ee = exp(-k.y * dd);
  double2 ph = make_double2(ee * c, ee * s);
  PairVal v;
  v.G = cmul(G, ph);
  v.F = cmul(F, ph);
  return v;
}

template <bool W64, bool W32>
__global__ void k_asm_near(AsmParams p) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.nref) return;
  int i = p.ref_row[e], j = p.ref_col[e];
  double4_32a si = p.src[i], sj = p.src[j];
  double4_32a nn = p.nrm[i];
  double3 ni = make_double3(nn.x, nn.y, nn.z);
  double x = si.x - sj.x, y = si.y - sj.y, z = si.z - sj.z;
  double dist = sqrt(x * x + y * y + z * z);
  double dd = fmax(dist, DBL_EPS_ASM);
  double delta = (dd == DBL_EPS_ASM) ? 2.0 * M_PI : 0.0;
  int pi = p.part[i], pj = p.part[j];
  int m11 = p.med[0][pi][pj], m21 = p.med[1][pi][pj], m22 = p.med[2][pi][pj], m12 = p.med[3][pi][pj];
  double2 g1 = make_double2(0, 0), h1 = g1, g2 = g1, h2 = g1;
  if (m11) { PairVal v = near_pair(p, e, p.lp->k[m11 - 1], dd, ni); g1 = v.G; h1 = make_double2(v.F.x + delta, v.F.y); }
  if (m21) { PairVal v = near_pair(p, e, p.lp->k[m21 - 1], dd, ni); g1 = csub(g1, v.G); h1 = csub(h1, make_double2(v.F.x + delta, v.F.y)); }
  if (m22) { PairVal v = near_pair(p, e, p.lp->k[m22 - 1], dd, ni); g2 = v.G; h2 = make_double2(v.F.x - delta, v.F.y); }
  if (m12) { PairVal v = near_pair(p, e, p.lp->k[m12 - 1], dd, ni); g2 = csub(g2, v.G); h2 = csub(h2, make_double2(v.F.x - delta, v.F.y)); }
  store4<W64, W32>(p, i, j, g1, h1, g2, h2);
}

__global__ void k_pack_src(int n, const double* pos, const double* area, const double* nvec,
                           double4_32a* src, double4_32a* nrm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  src[i] = make_double4_32a(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], area[i]);
  nrm[i] = make_double4_32a(nvec[3 * i], nvec[3 * i + 1], nvec[3 * i + 2], 0.0);
}

void pack_sources(int n, const double* pos, const double* area, const double* nvec, double4_32a* src,
                  double4_32a* nrm, cudaStream_t st) {
  k_pack_src<<<(n + 255) / 256, 256, 0, st>>>(n, pos, area, nvec, src, nrm);
}

mnpbem_status assemble_launch(const AsmParams& p, bool w64, bool w32, cudaStream_t st) {
  // algorithmic bytes: the four n x n outputs written once per precision
  MNP_TRY(ensure_cis(st));
  const double nn = (double)p.n * p.n;
  ProfScope ps(PH_ASSEMBLE, st, 0.0, nn * 4.0 * ((w64 ? 16.0 : 0.0) + (w32 ? 8.0 : 0.0)),
               p.nref > 0 ? 2 : 1);
  dim3 grid((unsigned)cdiv_up(p.n, ASM_COLS), (unsigned)cdiv_up(p.n, ASM_ROWS));
  if (w64 && w32) k_asm_far<true, true><<<grid, ASM_COLS, 0, st>>>(p);
  else if (w64) k_asm_far<true, false><<<grid, ASM_COLS, 0, st>>>(p);
  else k_asm_far<false, true><<<grid, ASM_COLS, 0, st>>>(p);
  MNP_CHECK_LAUNCH();
  if (p.nref > 0) {
    unsigned nb = (unsigned)cdiv_up(p.nref, 128);
    if (w64 && w32) k_asm_near<true, true><<<nb, 128, 0, st>>>(p);
    else if (w64) k_asm_near<true, false><<<nb, 128, 0, st>>>(p);
    else k_asm_near<false, true><<<nb, 128, 0, st>>>(p);
    MNP_CHECK_LAUNCH();
  }
  return MNPBEM_OK;
}

}  // namespace mnpbem
