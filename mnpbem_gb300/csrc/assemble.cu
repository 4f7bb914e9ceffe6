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
constexpr int ASM_DS_ROWS = 8;

struct Val4 { double2 g1, h1, g2, h2; };

// G1, H1, G2, H2 of the pair (i, j) by the far-field formula
__device__ __forceinline__ Val4 far4(const AsmParams& p, const CisShared& T, int64_t i, const double4_32a& sj,
                                     int pj) {
  const double4_32a si = p.src[i];
  const double4_32a ni = p.nrm[i];
  const double x = si.x - sj.x, y = si.y - sj.y, z = si.z - sj.z;
  const double dist = sqrt(x * x + y * y + z * z);
  const double dd = fmax(dist, DBL_EPS_ASM);
  const double delta = (dd == DBL_EPS_ASM) ? 2.0 * M_PI : 0.0;
  const double inv = 1.0 / dd;
  const double in = x * ni.x + y * ni.y + z * ni.z;
  const int pi = p.part[i];
  const int m11 = p.med[0][pi][pj], m21 = p.med[1][pi][pj], m22 = p.med[2][pi][pj], m12 = p.med[3][pi][pj];
  Val4 o;
  o.g1 = make_double2(0, 0); o.h1 = o.g1; o.g2 = o.g1; o.h2 = o.g1;
  if (m11) { PairVal v = far_pair(T, p.lp->k[m11 - 1], dd, inv, in, sj.w); o.g1 = v.G; o.h1 = make_double2(v.F.x + delta, v.F.y); }
  if (m21) { PairVal v = far_pair(T, p.lp->k[m21 - 1], dd, inv, in, sj.w); o.g1 = csub(o.g1, v.G); o.h1 = csub(o.h1, make_double2(v.F.x + delta, v.F.y)); }
  if (m22) { PairVal v = far_pair(T, p.lp->k[m22 - 1], dd, inv, in, sj.w); o.g2 = v.G; o.h2 = make_double2(v.F.x - delta, v.F.y); }
  if (m12) { PairVal v = far_pair(T, p.lp->k[m12 - 1], dd, inv, in, sj.w); o.g2 = csub(o.g2, v.G); o.h2 = csub(o.h2, make_double2(v.F.x - delta, v.F.y)); }
  return o;
}

template <bool W64, bool W32>
__global__ void __launch_bounds__(ASM_COLS) k_asm_far(AsmParams p) {
  __shared__ CisShared T;
  cis_load(T);
  int64_t j = (int64_t)blockIdx.x * ASM_COLS + threadIdx.x;
  int64_t i0 = (int64_t)blockIdx.y * ASM_ROWS;
  if (j >= p.n) return;
  double4_32a sj = p.src[j];
  int pj = p.part[j];
#pragma unroll
  for (int r = 0; r < ASM_ROWS; ++r) {
    int64_t i = i0 + r;
    if (i >= p.n) break;
    const Val4 v = far4(p, T, i, sj, pj);
    store4<W64, W32>(p, i, j, v.g1, v.h1, v.g2, v.h2);
  }
}

// full (near-field) blocks of the H-matrices: entries of the complete Green
// function on leaf pairs of the cluster tree, FP64, block b row-major at
// val[q] + foff[b] (Greenfun/@hmatrix/fillval.m with compgreenret's eval)
__global__ void __launch_bounds__(256) k_asm_leaf(AsmParams p, LeafAsm la) {
  __shared__ CisShared T;
  cis_load(T);
  const int b = blockIdx.x;
  const int4 blk = la.fblk[b];   // (r0, m, c0, nb)
  const int64_t cnt = (int64_t)blk.y * blk.w;
  const int64_t off = la.foff[b];
  for (int64_t e = threadIdx.x; e < cnt; e += blockDim.x) {
    const int r = (int)(e / blk.w), c = (int)(e - (int64_t)r * blk.w);
    const int i = la.perm[blk.x + r], j = la.perm[blk.z + c];
    const Val4 v = far4(p, T, i, p.src[j], p.part[j]);
    la.val[0][off + e] = v.g1; la.val[1][off + e] = v.h1;
    la.val[2][off + e] = v.g2; la.val[3][off + e] = v.h2;
  }
}

// ------------------------------------------------- double-single assembly
// Mixed precision needs G1, H1, G2, H2 twice: as complex64 working matrices
// and, for the refinement residual, to ~48 bits as hi / lo complex64 planes.
// On GB300 FP64 runs at 1/64 of the FP32 rate, so the FP64 pass above is
// FP64-pipe bound.  This pass computes every entry in double-single
// arithmetic (value = hi + lo, two floats; error-free transformations of
// Dekker and Knuth: TwoSum, TwoProduct by FMA) and writes hi / lo directly.
// exp(ikd) uses the same table-driven reduction as the FP64 pass, with the
// 2 pi / 256 and ln 2 / 64 constants split in three floats and Taylor series
// of the reduced arguments whose small tails are kept in float.
// Accuracy: ~1e-14 relative per entry (tests compare with the FP64 pass).
struct dsf { float hi, lo; };

__device__ __forceinline__ dsf ds_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dsf ds_quick(float a, float b) {   // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dsf ds_from(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}
__device__ __forceinline__ dsf ds_add(dsf a, dsf b) {
  dsf s = ds_two_sum(a.hi, b.hi);
  const dsf t = ds_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = ds_quick(s.hi, s.lo);
  s.lo += t.lo;
  return ds_quick(s.hi, s.lo);
}
__device__ __forceinline__ dsf ds_neg(dsf a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dsf ds_sub(dsf a, dsf b) { return ds_add(a, ds_neg(b)); }
__device__ __forceinline__ dsf ds_mul(dsf a, dsf b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return ds_quick(p, e);
}
__device__ __forceinline__ dsf ds_mulf(dsf a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return ds_quick(p, e);
}
__device__ __forceinline__ dsf ds_sqrt(dsf a) {            // a > 0
  const float q = sqrtf(a.hi);
  const float p = q * q;
  const float pe = fmaf(q, q, -p);
  const float r = ((a.hi - p) - pe) + a.lo;               // a - q^2 (a.hi - p is exact near q^2)
  return ds_quick(q, r / (2.0f * q));
}
__device__ __forceinline__ dsf ds_recip(dsf a) {           // 1 / a
  const float q1 = 1.0f / a.hi;
  const dsf r = ds_sub(dsf{1.0f, 0.0f}, ds_mulf(a, q1));
  return ds_quick(q1, r.hi * q1);
}
struct dsc { dsf re, im; };
__device__ __forceinline__ dsc dsc_mul(dsc a, dsc b) {
  return {ds_sub(ds_mul(a.re, b.re), ds_mul(a.im, b.im)), ds_add(ds_mul(a.re, b.im), ds_mul(a.im, b.re))};
}
__device__ __forceinline__ dsc dsc_scale(dsc a, dsf s) { return {ds_mul(a.re, s), ds_mul(a.im, s)}; }

// reduction constants: three-float splits (heads with trailing zero bits so
// that j * head is exact for |j| < 2^12)
constexpr float CIS_F1 = 0.0245361328125f;           // 2 pi / 256 = F1 + F2 + F3 (F1: 12 bits)
constexpr float CIS_F2 = 7.55979363e-06f;
constexpr float CIS_F3 = 4.00522511e-14f;
constexpr float EXP_F1 = 0.010829925537109375f;      // ln 2 / 64 = F1 + F2 + F3 (F1: 12 bits)
constexpr float EXP_F2 = 4.99159114e-07f;
constexpr float EXP_F3 = 2.57280464e-14f;

struct CisTableF {
  float c_hi[CIS_N], c_lo[CIS_N], s_hi[CIS_N], s_lo[CIS_N];
  float e_hi[64], e_lo[64];
};
__device__ CisTableF g_cisf;
__global__ void k_cisf_init() {
  const int j = threadIdx.x;
  double sn, cs;
  sincospi(2.0 * j / CIS_N, &sn, &cs);
  dsf c = ds_from(cs), s = ds_from(sn);
  g_cisf.c_hi[j] = c.hi; g_cisf.c_lo[j] = c.lo;
  g_cisf.s_hi[j] = s.hi; g_cisf.s_lo[j] = s.lo;
  if (j < 64) {
    dsf e = ds_from(exp2(-j / 64.0));
    g_cisf.e_hi[j] = e.hi; g_cisf.e_lo[j] = e.lo;
  }
}

// x - j * (c1 + c2 + c3) for x in double-single, |j| < 2^12 integral:
// j c1 is exact (c1 has 12 significant bits) and cancels exactly against x.hi,
// j c2 is taken exactly as a TwoProduct, j c3 is below the double-single ulp
__device__ __forceinline__ dsf ds_reduce(dsf x, float j, float c1, float c2, float c3) {
  const float a = fmaf(-j, c1, x.hi);
  dsf t = ds_two_sum(a, x.lo);
  const float p2 = j * c2;
  t = ds_sub(t, dsf{p2, fmaf(j, c2, -p2)});
  return ds_sub(t, dsf{j * c3, 0.0f});
}

// exp(i k d) in double-single; k = (kr, ki) as double-single
__device__ __forceinline__ dsc ds_cis_exp(const CisTableF& T, dsf kr, dsf ki, bool lossy, dsf d) {
  const dsf th = ds_mul(kr, d);
  const float jf = rintf(th.hi * (float)CIS_INV);
  const dsf t = ds_reduce(th, jf, CIS_F1, CIS_F2, CIS_F3);
  // sin t = t - t^3/6 + [t^5/120 (1 - t^2/42 + t^4/3024)]
  // cos t = 1 - t^2/2 + [t^4/24 (1 - t^2/30 + t^4/1680)]
  // (|t| <= pi/256: the bracketed tails, < 1e-9, are accurate enough in float;
  //  the leading terms are kept in double-single)
  const float tf = t.hi, t2f = tf * tf;
  const dsf t2 = ds_mul(t, t);
  const dsf sixth = {0.16666667163372040f, -4.96705388e-09f};   // 1/6 split
  const dsf t3_6 = ds_mul(ds_mul(t2, t), sixth);
  const float s5 = (t2f * t2f * tf) * (1.0f / 120.0f) * fmaf(t2f, fmaf(t2f, 1.0f / 3024.0f, -1.0f / 42.0f), 1.0f);
  const dsf sn = ds_add(ds_sub(t, t3_6), dsf{s5, 0.0f});
  const float c4 = (t2f * t2f) * (1.0f / 24.0f) * fmaf(t2f, fmaf(t2f, 1.0f / 1680.0f, -1.0f / 30.0f), 1.0f);
  const dsf cn = ds_add(ds_sub(dsf{1.0f, 0.0f}, dsf{t2.hi * 0.5f, t2.lo * 0.5f}), dsf{c4, 0.0f});
  const int jj = ((int)jf) & (CIS_N - 1);
  const dsf tc = {T.c_hi[jj], T.c_lo[jj]}, ts = {T.s_hi[jj], T.s_lo[jj]};
  dsc r = {ds_sub(ds_mul(tc, cn), ds_mul(ts, sn)), ds_add(ds_mul(ts, cn), ds_mul(tc, sn))};
  if (lossy) {
    const dsf x = ds_mul(ki, d);
    if (x.hi > 80.0f) return {dsf{0, 0}, dsf{0, 0}};
    const float yf = rintf(x.hi * (float)EXP_INV);
    const dsf u = ds_reduce(x, yf, EXP_F1, EXP_F2, EXP_F3);
    // exp(-u) = (1 - u) + u^2/2 - [u^3/6 (1 - u/4 + u^2/20 - u^3/120)],  |u| <= ln2/128
    const float uf = u.hi;
    const dsf q = ds_mul(u, u);
    const float c3 = (uf * uf * uf) * (1.0f / 6.0f) * fmaf(uf, fmaf(uf, fmaf(uf, -1.0f / 120.0f, 1.0f / 20.0f), -0.25f), 1.0f);
    const dsf ex = ds_sub(ds_add(ds_sub(dsf{1.0f, 0.0f}, u), dsf{q.hi * 0.5f, q.lo * 0.5f}), dsf{c3, 0.0f});
    const int yi = (int)yf;
    const int nn = yi >> 6, m = yi - (nn << 6);
    dsf e = ds_mul(ex, dsf{T.e_hi[m], T.e_lo[m]});
    const float sc = ldexpf(1.0f, -nn);
    e.hi *= sc;
    e.lo *= sc;
    r = dsc_scale(r, e);
  }
  return r;
}

struct DsPair { dsc G, F; };
__device__ __forceinline__ DsPair ds_far_pair(const CisTableF& T, dsf kr, dsf ki, bool lossy, dsf d, dsf inv,
                                              dsf in, dsf area) {
  const dsc ph = ds_cis_exp(T, kr, ki, lossy, d);
  DsPair v;
  v.G = dsc_scale(ph, ds_mul(area, inv));
  // (ik - 1/d) / d^2 (n . r) area = ((-ki - inv) + i kr) inv^2 in area
  const dsf s = ds_mul(ds_mul(inv, inv), ds_mul(in, area));
  const dsc tf = {ds_mul(ds_sub(ds_neg(ki), inv), s), ds_mul(kr, s)};
  v.F = dsc_mul(tf, ph);
  return v;
}

__device__ __forceinline__ void ds_store(float2* hi, float2* lo, float2* w, int64_t o, dsc v) {
  const float2 h = make_float2(v.re.hi, v.im.hi);
  w[o] = h;
  hi[o] = h;
  lo[o] = make_float2(v.re.lo, v.im.lo);
}

template <int ROWS>
__global__ void __launch_bounds__(ASM_COLS) k_asm_far_ds(AsmParams p) {
  __shared__ CisTableF T;
  for (int q = threadIdx.x; q < CIS_N; q += blockDim.x) {
    T.c_hi[q] = g_cisf.c_hi[q]; T.c_lo[q] = g_cisf.c_lo[q];
    T.s_hi[q] = g_cisf.s_hi[q]; T.s_lo[q] = g_cisf.s_lo[q];
  }
  for (int q = threadIdx.x; q < 64; q += blockDim.x) { T.e_hi[q] = g_cisf.e_hi[q]; T.e_lo[q] = g_cisf.e_lo[q]; }
  __syncthreads();
  const int64_t j = (int64_t)blockIdx.x * ASM_COLS + threadIdx.x;
  const int64_t i0 = (int64_t)blockIdx.y * ROWS;
  if (j >= p.n) return;
  const float4 sjh = p.srcf[2 * j], sjl = p.srcf[2 * j + 1];
  const dsf xj = {sjh.x, sjl.x}, yj = {sjh.y, sjl.y}, zj = {sjh.z, sjl.z}, aj = {sjh.w, sjl.w};
  const int pj = p.part[j];
  // wavenumbers of the media in double-single (once per thread)
  dsf kr[ASM_MAXMED], ki[ASM_MAXMED];
  bool lossy[ASM_MAXMED];
  const int nmed = p.nmed;
  for (int m = 0; m < nmed; ++m) {
    kr[m] = ds_from(p.lp->k[m].x);
    ki[m] = ds_from(p.lp->k[m].y);
    lossy[m] = p.lp->k[m].y != 0.0;
  }
  const dsc zero = {dsf{0, 0}, dsf{0, 0}};
  for (int r = 0; r < ROWS; ++r) {
    const int64_t i = i0 + r;
    if (i >= p.n) break;
    const int64_t o = i * p.ld32 + j;
    if (i == j) {
      // self element: refined (and given its +-2 pi) by the near pass
      const float2 z = make_float2(0.f, 0.f);
      p.g1[o] = p.h1[o] = p.g2[o] = p.h2[o] = z;
      p.G1hi[o] = p.G1lo[o] = p.H1hi[o] = p.H1lo[o] = z;
      p.G2hi[o] = p.G2lo[o] = p.H2hi[o] = p.H2lo[o] = z;
      continue;
    }
    const float4 sih = p.srcf[2 * i], sil = p.srcf[2 * i + 1];
    const float4 nih = p.nrmf[2 * i], nil = p.nrmf[2 * i + 1];
    const dsf x = ds_sub(dsf{sih.x, sil.x}, xj), y = ds_sub(dsf{sih.y, sil.y}, yj), z = ds_sub(dsf{sih.z, sil.z}, zj);
    const dsf d2 = ds_add(ds_add(ds_mul(x, x), ds_mul(y, y)), ds_mul(z, z));
    const dsf d = ds_sqrt(d2);
    const dsf inv = ds_recip(d);
    const dsf in = ds_add(ds_add(ds_mul(x, dsf{nih.x, nil.x}), ds_mul(y, dsf{nih.y, nil.y})), ds_mul(z, dsf{nih.z, nil.z}));
    const int pi = p.part[i];
    const int m11 = p.med[0][pi][pj], m21 = p.med[1][pi][pj], m22 = p.med[2][pi][pj], m12 = p.med[3][pi][pj];
    dsc g1 = zero, h1 = zero, g2 = zero, h2 = zero;
    if (m11) { DsPair v = ds_far_pair(T, kr[m11 - 1], ki[m11 - 1], lossy[m11 - 1], d, inv, in, aj); g1 = v.G; h1 = v.F; }
    if (m21) { DsPair v = ds_far_pair(T, kr[m21 - 1], ki[m21 - 1], lossy[m21 - 1], d, inv, in, aj);
               g1 = {ds_sub(g1.re, v.G.re), ds_sub(g1.im, v.G.im)}; h1 = {ds_sub(h1.re, v.F.re), ds_sub(h1.im, v.F.im)}; }
    if (m22) { DsPair v = ds_far_pair(T, kr[m22 - 1], ki[m22 - 1], lossy[m22 - 1], d, inv, in, aj); g2 = v.G; h2 = v.F; }
    if (m12) { DsPair v = ds_far_pair(T, kr[m12 - 1], ki[m12 - 1], lossy[m12 - 1], d, inv, in, aj);
               g2 = {ds_sub(g2.re, v.G.re), ds_sub(g2.im, v.G.im)}; h2 = {ds_sub(h2.re, v.F.re), ds_sub(h2.im, v.F.im)}; }
    ds_store(p.G1hi, p.G1lo, p.g1, o, g1);
    ds_store(p.H1hi, p.H1lo, p.h1, o, h1);
    ds_store(p.G2hi, p.G2lo, p.g2, o, g2);
    ds_store(p.H2hi, p.H2lo, p.h2, o, h2);
  }
}

static bool g_cisf_ready[64];

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

__device__ __forceinline__ Val4 near4(const AsmParams& p, int64_t e, int i, int j) {
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
  return Val4{g1, h1, g2, h2};
}

template <bool W64, bool W32>
__global__ void k_asm_near(AsmParams p) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.nref) return;
  const int i = p.ref_row[e], j = p.ref_col[e];
  const Val4 v = near4(p, e, i, j);
  store4<W64, W32>(p, i, j, v.g1, v.h1, v.g2, v.h2);
}

// refined entries that fall in full blocks of the H-matrices (refined pairs in
// low-rank blocks keep the far-field kernel, as ACA does)
__global__ void k_asm_leaf_near(AsmParams p, LeafAsm la) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p.nref) return;
  const int i = p.ref_row[e], j = p.ref_col[e];
  const int ci = la.iperm[i], cj = la.iperm[j];
  const int b = la.fidx[(int64_t)la.leaf_of[ci] * la.nleaf + la.leaf_of[cj]];
  if (b < 0) return;
  const int4 blk = la.fblk[b];
  const int64_t o = la.foff[b] + (int64_t)(ci - blk.x) * blk.w + (cj - blk.z);
  const Val4 v = near4(p, e, i, j);
  la.val[0][o] = v.g1; la.val[1][o] = v.h1; la.val[2][o] = v.g2; la.val[3][o] = v.h2;
}

mnpbem_status assemble_leaves(const AsmParams& p, const LeafAsm& la, cudaStream_t st) {
  MNP_TRY(ensure_cis(st));
  if (la.nfull > 0) {
    ProfScope ps(PH_HMAT_BUILD, st, 0.0, 64.0 * (double)la.nvals, p.nref > 0 ? 2 : 1);
    k_asm_leaf<<<la.nfull, 256, 0, st>>>(p, la);
    MNP_CHECK_LAUNCH();
    if (p.nref > 0) {
      k_asm_leaf_near<<<(unsigned)cdiv_up(p.nref, 128), 128, 0, st>>>(p, la);
      MNP_CHECK_LAUNCH();
    }
  }
  return MNPBEM_OK;
}

__global__ void k_pack_src(int n, const double* pos, const double* area, const double* nvec,
                           double4_32a* src, double4_32a* nrm, float4* srcf, float4* nrmf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  src[i] = make_double4_32a(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], area[i]);
  nrm[i] = make_double4_32a(nvec[3 * i], nvec[3 * i + 1], nvec[3 * i + 2], 0.0);
  if (srcf) {
    const dsf a = ds_from(pos[3 * i]), b = ds_from(pos[3 * i + 1]), c = ds_from(pos[3 * i + 2]), w = ds_from(area[i]);
    srcf[2 * i] = make_float4(a.hi, b.hi, c.hi, w.hi);
    srcf[2 * i + 1] = make_float4(a.lo, b.lo, c.lo, w.lo);
    const dsf u = ds_from(nvec[3 * i]), v = ds_from(nvec[3 * i + 1]), t = ds_from(nvec[3 * i + 2]);
    nrmf[2 * i] = make_float4(u.hi, v.hi, t.hi, 0.f);
    nrmf[2 * i + 1] = make_float4(u.lo, v.lo, t.lo, 0.f);
  }
}

void pack_sources(int n, const double* pos, const double* area, const double* nvec, double4_32a* src,
                  double4_32a* nrm, float4* srcf, float4* nrmf, cudaStream_t st) {
  k_pack_src<<<(n + 255) / 256, 256, 0, st>>>(n, pos, area, nvec, src, nrm, srcf, nrmf);
}

__global__ void k_hilo_c128(const float2* hi, const float2* lo, double2* out, int64_t count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  out[i] = make_double2((double)hi[i].x + (double)lo[i].x, (double)hi[i].y + (double)lo[i].y);
}

void hilo_to_c128(const float2* hi, const float2* lo, double2* out, int64_t count, cudaStream_t st) {
  if (count > 0) k_hilo_c128<<<(unsigned)cdiv_up(count, 256), 256, 0, st>>>(hi, lo, out, count);
}

mnpbem_status assemble_launch(const AsmParams& p, bool w64, bool w32, cudaStream_t st) {
  // algorithmic bytes: the four n x n outputs written once per precision
  MNP_TRY(ensure_cis(st));
  const double nn = (double)p.n * p.n;
  ProfScope ps(PH_ASSEMBLE, st, 0.0, nn * 4.0 * ((w64 ? 16.0 : 0.0) + (w32 ? 8.0 : 0.0)),
               p.nref > 0 ? 2 : 1);
  dim3 grid((unsigned)cdiv_up(p.n, ASM_COLS), (unsigned)cdiv_up(p.n, ASM_ROWS));
  if (w64 && w32 && p.ds) {
    int dev = 0;
    MNP_CUDA(cudaGetDevice(&dev));
    if (!g_cisf_ready[dev]) {
      k_cisf_init<<<1, CIS_N, 0, st>>>();
      MNP_CHECK_LAUNCH();
      if (!capturing_now()) g_cisf_ready[dev] = true;
    }
    dim3 g2((unsigned)cdiv_up(p.n, ASM_COLS), (unsigned)cdiv_up(p.n, ASM_DS_ROWS));
    k_asm_far_ds<ASM_DS_ROWS><<<g2, ASM_COLS, 0, st>>>(p);
  } else if (w64 && w32) k_asm_far<true, true><<<grid, ASM_COLS, 0, st>>>(p);
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
