// H-matrices of the retarded Green functions and the Krylov vector kernels.
//
//  k_aca      one CTA per (low-rank block, matrix): partial-pivot adaptive cross
//             approximation (mex/hlib/aca.cpp:150-218) of the far-field kernel
//             of mex/acagreen/acagreen.cpp:76-131, FP64
//  k_hmv_t    R^T x of every low-rank block (one warp per rank-one term)
//  k_hmv_leaf y = H x row by row: one CTA per (leaf cluster, matrix), one warp
//             per row, summing the full blocks of the leaf and the rows of the
//             low-rank blocks that cover it (no atomics: every row is written
//             once, in a fixed order)
// The products run in double-single arithmetic on (hi, lo) float splits of
// the values, factors and vectors: FP64 runs at a small fraction of the FP32
// rate on this GPU, and each complex entry feeds 4 N multiply-adds.
#include "hmat.cuh"
#include "ds_math.cuh"
#include "profile.cuh"

namespace mnpbem {

namespace {

constexpr int ACA_T = 256;
constexpr int ACA_W = ACA_T / 32;
constexpr double ACA_ROW_TOL = 1e-10;   // ACATOL of mex/hlib/aca.h

// exp(ikd) / d area (G) or (r . n_i)(ik - 1/d) exp(ikd) / d^2 area (F)
__device__ __forceinline__ double2 aca_term(double2 k, double d, double inv, double in, double area, bool F) {
  double s, c;
  sincos(k.x * d, &s, &c);
  const double e = exp(-k.y * d);
  const double2 ph = make_double2(e * c, e * s);
  if (!F) return make_double2(ph.x * inv * area, ph.y * inv * area);
  const double f = inv * inv * in * area;
  return cmul(make_double2((-k.y - inv) * f, k.x * f), ph);
}

// entry (i, j) (cluster positions) of matrix q: G1 = g{1,1} - g{2,1} (q = 0),
// H1 (1), G2 = g{2,2} - g{1,2} (2), H2 (3); far-field kernel only
__device__ __forceinline__ double2 aca_entry(const AsmParams& p, const int* perm, int q, int i, int j) {
  const int fi = perm[i], fj = perm[j];
  const double4_32a si = p.src[fi], sj = p.src[fj], ni = p.nrm[fi];
  const double x = si.x - sj.x, y = si.y - sj.y, z = si.z - sj.z;
  const double d = sqrt(x * x + y * y + z * z);
  const double inv = 1.0 / d;
  const double in = x * ni.x + y * ni.y + z * ni.z;
  const int pi = p.part[fi], pj = p.part[fj];
  const int mp = p.med[q < 2 ? 0 : 2][pi][pj], mm = p.med[q < 2 ? 1 : 3][pi][pj];
  const bool F = q & 1;
  double2 v = make_double2(0.0, 0.0);
  if (mp) v = aca_term(p.lp->k[mp - 1], d, inv, in, sj.w, F);
  if (mm) v = csub(v, aca_term(p.lp->k[mm - 1], d, inv, in, sj.w, F));
  return v;
}

struct Red {
  double s1, s2, best;
  int idx;
};

__device__ __forceinline__ void red_merge(Red& a, const Red& b) {
  a.s1 += b.s1;
  a.s2 += b.s2;
  if (b.best > a.best || (b.best == a.best && b.idx < a.idx)) {
    a.best = b.best;
    a.idx = b.idx;
  }
}

__device__ __forceinline__ Red warp_red(Red v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Red w;
    w.s1 = __shfl_down_sync(0xffffffffu, v.s1, o);
    w.s2 = __shfl_down_sync(0xffffffffu, v.s2, o);
    w.best = __shfl_down_sync(0xffffffffu, v.best, o);
    w.idx = __shfl_down_sync(0xffffffffu, v.idx, o);
    red_merge(v, w);
  }
  return v;
}

// two sums and an argmax (largest value, first index on ties) over the CTA
__device__ Red block_red(Red v, Red* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_red(v);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    Red t = lane < ACA_W ? sh[lane] : Red{0.0, 0.0, -1.0, INT_MAX};
    t = warp_red(t);
    if (lane == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

__global__ void __launch_bounds__(ACA_T) k_aca(AsmParams p, HmatDev h) {
  __shared__ double2 coef[ACA_KMAX];
  __shared__ Red sh[33];
  __shared__ int s_nused;
  const int b = blockIdx.x, q = blockIdx.y;
  const int4 blk = h.lblk[b];
  const int m = blk.y, nb = blk.w, kc = h.kcap[b];
  double2* A = h.A[q] + h.aoff[b];
  double2* B = h.B[q] + h.boff[b];
  unsigned char* used = h.used + (int64_t)q * h.usz + h.uoff[b];
  for (int i = threadIdx.x; i < m; i += ACA_T) used[i] = 0;
  if (threadIdx.x == 0) s_nused = 0;
  __syncthreads();
  int r = 0, rank = kc;
  double nsum = 0.0;
  for (int k = 0; k < kc; ++k) {
    // row r, minus the rank-k approximation: B_k -= sum_l B_l A_l[r]
    for (int l = threadIdx.x; l < k; l += ACA_T) coef[l] = A[(int64_t)l * m + r];
    __syncthreads();
    Red v0{0.0, 0.0, -1.0, INT_MAX};
    for (int c = threadIdx.x; c < nb; c += ACA_T) {
      double2 v = aca_entry(p, h.perm, q, blk.x + r, blk.z + c);
      v0.s1 += v.x * v.x + v.y * v.y;
      for (int l = 0; l < k; ++l) v = csub(v, cmul(B[(int64_t)l * nb + c], coef[l]));
      B[(int64_t)k * nb + c] = v;
      const double a1 = fabs(v.x) + fabs(v.y);
      if (a1 > v0.best) { v0.best = a1; v0.idx = c; }
    }
    const Red rr = block_red(v0, sh);
    if (sqrt(rr.s1) < ACA_ROW_TOL) {
      // the reference keeps this column with a zero left factor
      for (int i = threadIdx.x; i < m; i += ACA_T) A[(int64_t)k * m + i] = make_double2(0.0, 0.0);
      rank = k + 1;
      break;
    }
    const int cp = rr.idx;
    if (cp < 0 || cp >= nb) { rank = k; break; }     // no finite pivot
    const double2 piv = B[(int64_t)k * nb + cp];
    // every thread holds the pivot before its owner rescales that entry
    __syncthreads();
    if (piv.x == 0.0 && piv.y == 0.0) { rank = k; break; }
    const double2 sc = cdiv(make_double2(1.0, 0.0), piv);
    Red v1{0.0, 0.0, -1.0, INT_MAX};
    for (int c = threadIdx.x; c < nb; c += ACA_T) {
      const double2 v = cmul(B[(int64_t)k * nb + c], sc);
      B[(int64_t)k * nb + c] = v;
      v1.s2 += v.x * v.x + v.y * v.y;
    }
    for (int l = threadIdx.x; l < k; l += ACA_T) coef[l] = B[(int64_t)l * nb + cp];
    if (threadIdx.x == 0 && !used[r]) {
      used[r] = 1;
      ++s_nused;
    }
    __syncthreads();
    // column cp, minus the rank-k approximation: A_k -= sum_l A_l B_l[cp]
    for (int i = threadIdx.x; i < m; i += ACA_T) {
      double2 v = aca_entry(p, h.perm, q, blk.x + i, blk.z + cp);
      for (int l = 0; l < k; ++l) v = csub(v, cmul(A[(int64_t)l * m + i], coef[l]));
      A[(int64_t)k * m + i] = v;
      v1.s1 += v.x * v.x + v.y * v.y;
      const double a1 = used[i] ? 0.0 : fabs(v.x) + fabs(v.y);
      if (a1 > v1.best) { v1.best = a1; v1.idx = i; }
    }
    const Red rc = block_red(v1, sh);
    const double nk = sqrt(rc.s1) * sqrt(rc.s2);
    if (nk < h.tol * nsum || s_nused >= m) { rank = k + 1; break; }
    nsum = sqrt(nsum * nsum + nk * nk);
    r = (rc.idx >= 0 && rc.idx < m) ? rc.idx : 0;
  }
  if (threadIdx.x == 0) h.rank[q * h.nlow + b] = rank;
}

template <int N>
__device__ __forceinline__ void warp_sum_ds(DS (&re)[N], DS (&im)[N]) {
#pragma unroll
  for (int c = 0; c < N; ++c)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const DS a{__shfl_xor_sync(0xffffffffu, re[c].hi, o), __shfl_xor_sync(0xffffffffu, re[c].lo, o)};
      const DS b{__shfl_xor_sync(0xffffffffu, im[c].hi, o), __shfl_xor_sync(0xffffffffu, im[c].lo, o)};
      re[c] = ds_add(re[c], a);
      im[c] = ds_add(im[c], b);
    }
}

__device__ __forceinline__ float2 f4hi(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 f4lo(float4 v) { return make_float2(v.z, v.w); }

template <int N>
__global__ void __launch_bounds__(256) k_hmv_t(HmatDev h) {
  const int b = blockIdx.x, q = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int4 blk = h.lblk[b];
  const int rank = h.rank[q * h.nlow + b];
  const float4* B = reinterpret_cast<const float4*>(h.B[q] + h.boff[b]);
  const float4* x = h.xs + (q < 2 ? 0 : (int64_t)h.n * N);
  float4* T = h.T + (int64_t)q * h.tsz + h.toff[b];
  for (int kk = warp; kk < rank; kk += 8) {
    DS re[N], im[N];
#pragma unroll
    for (int c = 0; c < N; ++c) re[c] = im[c] = DS{0.f, 0.f};
    for (int j = lane; j < blk.w; j += 32) {
      const float4 bv = B[(int64_t)kk * blk.w + j];
      const float4* xr = x + (int64_t)h.perm[blk.z + j] * N;
#pragma unroll
      for (int c = 0; c < N; ++c) {
        const float4 xv = xr[c];
        ds_cfma(re[c], im[c], f4hi(bv), f4lo(bv), f4hi(xv), f4lo(xv));
      }
    }
    warp_sum_ds<N>(re, im);
    if (lane == 0)
#pragma unroll
      for (int c = 0; c < N; ++c) T[kk * N + c] = make_float4(re[c].hi, im[c].hi, re[c].lo, im[c].lo);
  }
}

struct YPtrs {
  double2* y[4];
};

// rs CTAs share the rows of a leaf (grid.x = nleaf * rs) so that small trees
// still fill the SMs; each warp takes R consecutive rows, which share the
// gathered vector entries and give R independent accumulation chains
template <int N, int R>
__global__ void __launch_bounds__(256) k_hmv_leaf(HmatDev h, YPtrs ys, int rs) {
  const int l = blockIdx.x / rs, part = blockIdx.x - l * rs, q = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int2 lf = h.leaf[l];
  const float4* x = h.xs + (q < 2 ? 0 : (int64_t)h.n * N);
  double2* y = ys.y[q];
  const int e0 = h.lptr[l], e1 = h.lptr[l + 1];
  for (int rr = (part * 8 + warp) * R; rr < lf.y; rr += 8 * rs * R) {
    int ii[R];
    bool ok[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      ok[r] = rr + r < lf.y;
      ii[r] = lf.x + (ok[r] ? rr + r : rr);
    }
    DS re[R][N], im[R][N];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int c = 0; c < N; ++c) re[r][c] = im[r][c] = DS{0.f, 0.f};
    for (int e = e0; e < e1; ++e) {
      const int ent = h.lent[e];
      if (ent >= 0) {
        const int4 fb = h.fblk[ent];
        const float4* V0 = reinterpret_cast<const float4*>(h.val[q] + h.foff[ent]);
        const float4* V[R];
#pragma unroll
        for (int r = 0; r < R; ++r) V[r] = V0 + (int64_t)(ii[r] - fb.x) * fb.w;
        for (int j = lane; j < fb.w; j += 32) {
          float4 v[R];
#pragma unroll
          for (int r = 0; r < R; ++r) v[r] = V[r][j];
          const float4* xr = x + (int64_t)h.perm[fb.z + j] * N;
#pragma unroll
          for (int c = 0; c < N; ++c) {
            const float4 xv = xr[c];
#pragma unroll
            for (int r = 0; r < R; ++r) ds_cfma(re[r][c], im[r][c], f4hi(v[r]), f4lo(v[r]), f4hi(xv), f4lo(xv));
          }
        }
      } else {
        const int b = ~ent;
        const int4 lb = h.lblk[b];
        const int rank = h.rank[q * h.nlow + b];
        const int kc = h.kcap[b];
        const float4* A0 = h.At[q] + h.aoff[b];
        const float4* T = h.T + (int64_t)q * h.tsz + h.toff[b];
        for (int kk = lane; kk < rank; kk += 32) {
          float4 a[R];
#pragma unroll
          for (int r = 0; r < R; ++r) a[r] = A0[(int64_t)(ii[r] - lb.x) * kc + kk];
#pragma unroll
          for (int c = 0; c < N; ++c) {
            const float4 tv = T[kk * N + c];
#pragma unroll
            for (int r = 0; r < R; ++r) ds_cfma(re[r][c], im[r][c], f4hi(a[r]), f4lo(a[r]), f4hi(tv), f4lo(tv));
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      warp_sum_ds<N>(re[r], im[r]);
      if (lane == 0 && ok[r]) {
        double2* yr = y + (int64_t)h.perm[ii[r]] * N;
#pragma unroll
        for (int c = 0; c < N; ++c)
          yr[c] = make_double2((double)re[r][c].hi + (double)re[r][c].lo, (double)im[r][c].hi + (double)im[r][c].lo);
      }
    }
  }
}

__global__ void k_hmat_full(HmatDev h, int q, double2* out) {
  const int b = blockIdx.x;
  const int64_t n = h.n;
  if (b < h.nfull) {
    const int4 fb = h.fblk[b];
    const float4* V = reinterpret_cast<const float4*>(h.val[q] + h.foff[b]);
    for (int64_t e = threadIdx.x; e < (int64_t)fb.y * fb.w; e += blockDim.x) {
      const int r = (int)(e / fb.w), c = (int)(e - (int64_t)r * fb.w);
      out[(int64_t)h.perm[fb.x + r] * n + h.perm[fb.z + c]] = join4(V[e]);
    }
    return;
  }
  const int lb = b - h.nfull;
  const int4 blk = h.lblk[lb];
  const int rank = h.rank[q * h.nlow + lb];
  const double2* A = h.A[q] + h.aoff[lb];
  const float4* B = reinterpret_cast<const float4*>(h.B[q] + h.boff[lb]);
  for (int64_t e = threadIdx.x; e < (int64_t)blk.y * blk.w; e += blockDim.x) {
    const int r = (int)(e / blk.w), c = (int)(e - (int64_t)r * blk.w);
    double2 s = make_double2(0.0, 0.0);
    for (int k = 0; k < rank; ++k) cfma(s, A[(int64_t)k * blk.y + r], join4(B[(int64_t)k * blk.w + c]));
    out[(int64_t)h.perm[blk.x + r] * n + h.perm[blk.z + c]] = s;
  }
}

// complex128 -> float4 (hi, lo) in place
__device__ __forceinline__ void split_in_place(double2* p, int64_t i) {
  const double2 v = p[i];
  reinterpret_cast<float4*>(p)[i] = split4(v);
}

__global__ void k_split_vals(double2* v0, double2* v1, double2* v2, double2* v3, int64_t count) {
  double2* v[4] = {v0, v1, v2, v3};
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 4 * count;
       e += (int64_t)gridDim.x * blockDim.x)
    split_in_place(v[e / count], e % count);
}

__global__ void k_split_factors(HmatDev h) {
  const int b = blockIdx.x, q = blockIdx.y;
  const int4 blk = h.lblk[b];
  const int rank = h.rank[q * h.nlow + b];
  const double2* A = h.A[q] + h.aoff[b];
  float4* At = h.At[q] + h.aoff[b];
  const int kc = h.kcap[b];
  double2* B = h.B[q] + h.boff[b];
  for (int64_t e = threadIdx.x; e < (int64_t)rank * blk.y; e += blockDim.x) {
    const int64_t k = e / blk.y, i = e - k * blk.y;
    At[i * kc + k] = split4(A[e]);
  }
  for (int64_t e = threadIdx.x; e < (int64_t)rank * blk.w; e += blockDim.x) split_in_place(B, e);
}

__global__ void k_split_x(const double2* __restrict__ x1, const double2* __restrict__ x2, int64_t count,
                          float4* xs) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
    xs[e] = split4(x1[e]);
    xs[count + e] = split4(x2[e]);
  }
}

// ------------------------------------------------------------- Krylov vectors
__global__ void k_kv_dots(const double2* __restrict__ V, int64_t len, const double2* __restrict__ w,
                          double2* partial) {
  __shared__ double2 sh[8];
  const int i = blockIdx.y;
  const double2* v = V + (int64_t)i * len;
  double2 s = make_double2(0.0, 0.0);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len; e += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = v[e], b = w[e];
    s.x += a.x * b.x + a.y * b.y;      // conj(a) b
    s.y += a.x * b.y - a.y * b.x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 t = sh[0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) t = cadd(t, sh[k]);
    partial[(int64_t)i * gridDim.x + blockIdx.x] = t;
  }
}

__global__ void k_kv_update(const double2* __restrict__ V, int nv, int64_t len, const double2* __restrict__ hc,
                            double2* w) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len; e += (int64_t)gridDim.x * blockDim.x) {
    double2 s = w[e];
    for (int i = 0; i < nv; ++i) s = csub(s, cmul(hc[i], V[(int64_t)i * len + e]));
    w[e] = s;
  }
}

__global__ void k_kv_norm2(const double2* __restrict__ w, int64_t len, double* partial) {
  __shared__ double sh[8];
  double s = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len; e += (int64_t)gridDim.x * blockDim.x)
    s += w[e].x * w[e].x + w[e].y * w[e].y;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = sh[0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    partial[blockIdx.x] = t;
  }
}

__global__ void k_kv_scale(const double2* w, int64_t len, double s, double2* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = make_double2(s * w[e].x, s * w[e].y);
}

__global__ void k_kv_lincomb(KvTerms t, int64_t len, double2* out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len; e += (int64_t)gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int i = 0; i < t.n; ++i) cfma(s, t.c[i], t.v[i][e]);
    out[e] = s;
  }
}

__global__ void k_kv_pack_bx(int64_t n, int P, const double2* phi, const double2* a, const double2* alpha,
                             const double2* De, double2* x) {
  const int64_t W = 4 * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * W; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / W;
    const int c = (int)(e - i * W);
    double2 u, v;
    if (c < P) {
      u = phi[i * P + c];
      v = De[i * P + c];
    } else {
      u = a[i * 3 * P + (c - P)];
      v = alpha[i * 3 * P + (c - P)];
    }
    x[e] = u;
    x[n * W + e] = v;
  }
}

}  // namespace

mnpbem_status hmat_aca(const AsmParams& p, const HmatDev& h, cudaStream_t st) {
  if (h.nlow <= 0) return MNPBEM_OK;
  ProfScope ps(PH_HMAT_BUILD, st, 0.0, 0.0, 1);
  k_aca<<<dim3((unsigned)h.nlow, 4), ACA_T, 0, st>>>(p, h);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

mnpbem_status hmat_split(const HmatDev& h, cudaStream_t st) {
  ProfScope ps(PH_HMAT_BUILD, st, 0.0, 0.0, h.nlow > 0 ? 2 : 1);
  if (h.nvals > 0)
    k_split_vals<<<(unsigned)std::min<int64_t>(cdiv_up(4 * h.nvals, 256), 8192), 256, 0, st>>>(
        h.val[0], h.val[1], h.val[2], h.val[3], h.nvals);
  if (h.nlow > 0) k_split_factors<<<dim3((unsigned)h.nlow, 4), 256, 0, st>>>(h);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

mnpbem_status hmat_mv(const HmatDev& h, int N, const double2* x1, const double2* x2, double2* const* y,
                      double bytes, cudaStream_t st) {
  if (N != 4 && N != 8 && N != 12 && N != 16) {
    set_error("hmat_mv: %d columns (4, 8, 12 or 16 supported)", N);
    return MNPBEM_ERR_INVALID_ARG;
  }
  YPtrs ys{{y[0], y[1], y[2], y[3]}};
  ProfScope ps(PH_HMAT_MV, st, 0.0, bytes, h.nlow > 0 ? 3 : 2);
  const int64_t cnt = (int64_t)h.n * N;
  // CTAs per leaf: at least two waves of CTAs over the SMs, at least 8 rows per CTA
  const int rs = (int)std::max<int64_t>(1, std::min<int64_t>(cdiv_up(2 * 152, 4 * (int64_t)h.nleaf), 4));
  k_split_x<<<(unsigned)std::min<int64_t>(cdiv_up(cnt, 256), 4096), 256, 0, st>>>(x1, x2, cnt, h.xs);
#define HMV_CASE(NN)                                                                  \
  case NN:                                                                            \
    if (h.nlow > 0) k_hmv_t<NN><<<dim3((unsigned)h.nlow, 4), 256, 0, st>>>(h);        \
    k_hmv_leaf<NN, (NN <= 8 ? 2 : 1)><<<dim3((unsigned)(h.nleaf * rs), 4), 256, 0, st>>>(h, ys, rs); \
    break;
  switch (N) {
    HMV_CASE(4) HMV_CASE(8) HMV_CASE(12) HMV_CASE(16)
  }
#undef HMV_CASE
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

mnpbem_status hmat_full(const HmatDev& h, int q, double2* out, cudaStream_t st) {
  if (q < 0 || q > 3) {
    set_error("hmat_full: matrix index %d", q);
    return MNPBEM_ERR_INVALID_ARG;
  }
  k_hmat_full<<<(unsigned)(h.nfull + h.nlow), 256, 0, st>>>(h, q, out);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

void kv_dots(const double2* V, int nv, int64_t len, const double2* w, double2* partial, cudaStream_t st) {
  if (nv > 0) k_kv_dots<<<dim3(KV_BLOCKS, (unsigned)nv), 256, 0, st>>>(V, len, w, partial);
}
void kv_update(const double2* V, int nv, int64_t len, const double2* h, double2* w, cudaStream_t st) {
  if (nv > 0) k_kv_update<<<KV_BLOCKS, 256, 0, st>>>(V, nv, len, h, w);
}
void kv_norm2(const double2* w, int64_t len, double* partial, cudaStream_t st) {
  k_kv_norm2<<<KV_BLOCKS, 256, 0, st>>>(w, len, partial);
}
void kv_scale(const double2* w, int64_t len, double s, double2* out, cudaStream_t st) {
  k_kv_scale<<<KV_BLOCKS, 256, 0, st>>>(w, len, s, out);
}
void kv_lincomb(const KvTerms& t, int64_t len, double2* out, cudaStream_t st) {
  k_kv_lincomb<<<KV_BLOCKS, 256, 0, st>>>(t, len, out);
}
void kv_pack_bx(int64_t n, int P, const double2* phi, const double2* a, const double2* alpha, const double2* De,
                double2* x, cudaStream_t st) {
  k_kv_pack_bx<<<KV_BLOCKS, 256, 0, st>>>(n, P, phi, a, alpha, De, x);
}

}  // namespace mnpbem
