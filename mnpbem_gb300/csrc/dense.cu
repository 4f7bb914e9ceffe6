// Dense complex kernels: SIMT GEMM, shared-memory block inversion and the
// blocked Gauss-Jordan inversion that replaces MATLAB's inv() in
// BEM/@bemret/private/initmat.m:27-28,50,72.
//
// Gauss-Jordan without row interchanges: the matrices inverted by bemret
// (G1, G2, Sigma1 - Sigma2, Sigma) are strongly diagonally dominant (the
// diagonal is the column maximum in practice), which is the same property the
// reference's own native dense LU relies on (mex/hlib/lu.cpp:79-105 factorises
// without pivoting).  Each block step costs one rank-nb update of the whole
// matrix, so all O(n^3) work is a GEMM.  A pivot guard reports singular blocks.
#include <cooperative_groups.h>

#include "dense.cuh"
#include "ds_math.cuh"
#include "mbarrier.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

namespace mnpbem {

// ----------------------------------------------------------------- SIMT GEMM
template <typename R, int BK>
__global__ void __launch_bounds__(256) k_gemm_nn(int64_t M, int64_t N, int64_t K, cplx<R> alpha,
                                                 const cplx<R>* __restrict__ A, int64_t lda,
                                                 const cplx<R>* __restrict__ B, int64_t ldb,
                                                 cplx<R> beta, cplx<R>* __restrict__ C,
                                                 int64_t ldc) {
  using Cx = cplx<R>;
  __shared__ Cx As[BK][64 + 1];
  __shared__ Cx Bs[BK][64];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * 64, n0 = (int64_t)blockIdx.x * 64;
  Cx acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = mk<R>(0, 0);
  for (int64_t k0 = 0; k0 < K; k0 += BK) {
    for (int l = t; l < 64 * BK; l += 256) {
      int r = l / BK, c = l % BK;
      int64_t gr = m0 + r, gc = k0 + c;
      As[c][r] = (gr < M && gc < K) ? A[gr * lda + gc] : mk<R>(0, 0);
    }
    for (int l = t; l < BK * 64; l += 256) {
      int r = l / 64, c = l % 64;
      int64_t gr = k0 + r, gc = n0 + c;
      Bs[r][c] = (gr < K && gc < N) ? B[gr * ldb + gc] : mk<R>(0, 0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      Cx a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) cfma(acc[r][c], a[r], b[c]);
    }
    __syncthreads();
  }
  const bool zero_beta = (beta.x == 0 && beta.y == 0);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int64_t gr = m0 + ty + 16 * r;
    if (gr >= M) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int64_t gc = n0 + tx + 16 * c;
      if (gc >= N) continue;
      Cx v = cmul(alpha, acc[r][c]);
      if (!zero_beta) v = cadd(v, cmul(beta, C[gr * ldc + gc]));
      C[gr * ldc + gc] = v;
    }
  }
}

// ------------------------------------------------------- thin GEMM (N <= 16)
// Matrix times a few vectors, memory-bound on A.  A block of 8 warps owns
// TR rows; warp w streams its own slice of K (no barriers in the main loop),
// lanes stride by 32 over consecutive k (coalesced rows of A), each B row is
// read once per lane through L1 and reused for the TR rows.  The 8 partial
// sums per entry are combined in shared memory at the end.
constexpr int THIN_NMAX = 16, THIN_WARPS = 8;

template <typename R, int N, int TR>
__global__ void __launch_bounds__(32 * THIN_WARPS) k_gemm_thin(int64_t M, int64_t K, cplx<R> alpha,
                                                             const cplx<R>* __restrict__ A, int64_t lda,
                                                             const cplx<R>* __restrict__ B, int64_t ldb,
                                                             cplx<R> beta, cplx<R>* __restrict__ C,
                                                             int64_t ldc) {
  using Cx = cplx<R>;
  __shared__ Cx red[THIN_WARPS][TR][N];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t row0 = (int64_t)blockIdx.x * TR;
  const int64_t kw = (K + THIN_WARPS - 1) / THIN_WARPS;
  const int64_t kbeg = warp * kw, kend = min(K, kbeg + kw);
  const Cx* arow[TR];
#pragma unroll
  for (int r = 0; r < TR; ++r) arow[r] = A + min(row0 + r, M - 1) * lda;
  Cx acc[TR][N];
#pragma unroll
  for (int r = 0; r < TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) acc[r][c] = mk<R>(0, 0);
#pragma unroll 2
  for (int64_t k = kbeg + lane; k < kend; k += 32) {
    Cx bv[N];
#pragma unroll
    for (int c = 0; c < N; ++c) bv[c] = __ldg(B + k * ldb + c);
#pragma unroll
    for (int r = 0; r < TR; ++r) {
      const Cx av = __ldg(arow[r] + k);
#pragma unroll
      for (int c = 0; c < N; ++c) cfma(acc[r][c], av, bv[c]);
    }
  }
#pragma unroll
  for (int r = 0; r < TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) {
      Cx v = acc[r][c];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[warp][r][c] = v;
    }
  __syncthreads();
  const bool zero_beta = (beta.x == 0 && beta.y == 0);
  for (int t = threadIdx.x; t < TR * N; t += blockDim.x) {
    const int r = t / N, c = t % N;
    const int64_t row = row0 + r;
    if (row >= M) continue;
    Cx v = mk<R>(0, 0);
#pragma unroll
    for (int w = 0; w < THIN_WARPS; ++w) v = cadd(v, red[w][r][c]);
    Cx out = cmul(alpha, v);
    if (!zero_beta) out = cadd(out, cmul(beta, C[row * ldc + c]));
    C[row * ldc + c] = out;
  }
}

// complex64 variant with 16-byte loads: each lane takes two consecutive k
// (one float4 of A per row, two rows of B), halving the load instructions of
// the matrix stream.  Needs lda even and A 16-byte aligned; an odd K leaves
// one k that warp 0 adds at the end.
template <int N, int TR>
__global__ void __launch_bounds__(32 * THIN_WARPS) k_gemm_thin_c64(int64_t M, int64_t K, float2 alpha,
                                                                 const float2* __restrict__ A, int64_t lda,
                                                                 const float2* __restrict__ B, int64_t ldb,
                                                                 float2 beta, float2* __restrict__ C,
                                                                 int64_t ldc) {
  __shared__ float2 red[THIN_WARPS][TR][N];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t row0 = (int64_t)blockIdx.x * TR;
  const int64_t KP = K >> 1;   // pairs
  const int64_t kw = (KP + THIN_WARPS - 1) / THIN_WARPS;
  const int64_t pbeg = warp * kw, pend = min(KP, pbeg + kw);
  const float2* arow[TR];
#pragma unroll
  for (int r = 0; r < TR; ++r) arow[r] = A + min(row0 + r, M - 1) * lda;
  float2 acc[TR][N];
#pragma unroll
  for (int r = 0; r < TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) acc[r][c] = make_float2(0.f, 0.f);
#pragma unroll 2
  for (int64_t kp = pbeg + lane; kp < pend; kp += 32) {
    const int64_t k = 2 * kp;
    float2 b0[N], b1[N];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      b0[c] = __ldg(B + k * ldb + c);
      b1[c] = __ldg(B + (k + 1) * ldb + c);
    }
#pragma unroll
    for (int r = 0; r < TR; ++r) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(arow[r] + k));
      const float2 a0 = make_float2(a.x, a.y), a1 = make_float2(a.z, a.w);
#pragma unroll
      for (int c = 0; c < N; ++c) {
        cfma(acc[r][c], a0, b0[c]);
        cfma(acc[r][c], a1, b1[c]);
      }
    }
  }
  if ((K & 1) && warp == 0 && lane == 0) {
    const int64_t k = K - 1;
#pragma unroll
    for (int r = 0; r < TR; ++r)
#pragma unroll
      for (int c = 0; c < N; ++c) cfma(acc[r][c], arow[r][k], B[k * ldb + c]);
  }
#pragma unroll
  for (int r = 0; r < TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) {
      float2 v = acc[r][c];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[warp][r][c] = v;
    }
  __syncthreads();
  const bool zero_beta = (beta.x == 0 && beta.y == 0);
  for (int t = threadIdx.x; t < TR * N; t += blockDim.x) {
    const int r = t / N, c = t % N;
    const int64_t row = row0 + r;
    if (row >= M) continue;
    float2 v = make_float2(0.f, 0.f);
#pragma unroll
    for (int w = 0; w < THIN_WARPS; ++w) v = cadd(v, red[w][r][c]);
    float2 out = cmul(alpha, v);
    if (!zero_beta) out = cadd(out, cmul(beta, C[row * ldc + c]));
    C[row * ldc + c] = out;
  }
}

// ------------------------------------------- double-single thin GEMM (N <= 16)
constexpr int DS_WARPS = 8, DS_TR = 4;

// B (complex128) -> hi / lo complex64 planes
__global__ void k_split_hi_lo(const double2* __restrict__ B, int64_t count, float2* hi, float2* lo) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const double2 b = B[i];
  const float2 h = make_float2((float)b.x, (float)b.y);
  hi[i] = h;
  lo[i] = make_float2((float)(b.x - (double)h.x), (float)(b.y - (double)h.y));
}

template <int N, int TR, int UNR>
__global__ void __launch_bounds__(32 * DS_WARPS) k_gemm_thin_ds(int64_t M, int64_t K, const float2* __restrict__ Ahi,
                                                              const float2* __restrict__ Alo, int64_t lda,
                                                              const float2* __restrict__ Bh,
                                                              const float2* __restrict__ Bl, int64_t ldb,
                                                              double2* __restrict__ C, int64_t ldc) {
  __shared__ DS red[DS_WARPS][TR][N][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t row0 = (int64_t)blockIdx.x * TR;
  const int64_t kw = (K + DS_WARPS - 1) / DS_WARPS;
  const int64_t kbeg = warp * kw, kend = min(K, kbeg + kw);
  int64_t roff[TR];
#pragma unroll
  for (int r = 0; r < TR; ++r) roff[r] = min(row0 + r, M - 1) * lda;
  DS re[TR][N], im[TR][N];
#pragma unroll
  for (int r = 0; r < TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) re[r][c] = im[r][c] = DS{0.f, 0.f};
#pragma unroll UNR
  for (int64_t k = kbeg + lane; k < kend; k += 32) {
    float2 xh[N], xl[N];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      xh[c] = __ldg(Bh + k * ldb + c);
      xl[c] = __ldg(Bl + k * ldb + c);
    }
#pragma unroll
    for (int r = 0; r < TR; ++r) {
      const float2 ah = __ldg(Ahi + roff[r] + k), al = __ldg(Alo + roff[r] + k);
#pragma unroll
      for (int c = 0; c < N; ++c) {
        ds_acc_prod(re[r][c], ah.x, xh[c].x);
        ds_acc_prod(re[r][c], -ah.y, xh[c].y);
        ds_acc_prod(im[r][c], ah.x, xh[c].y);
        ds_acc_prod(im[r][c], ah.y, xh[c].x);
        // first-order corrections from the low parts (relative size 2^-24)
        re[r][c].lo += (ah.x * xl[c].x - ah.y * xl[c].y) + (al.x * xh[c].x - al.y * xh[c].y);
        im[r][c].lo += (ah.x * xl[c].y + ah.y * xl[c].x) + (al.x * xh[c].y + al.y * xh[c].x);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) {
      DS a = re[r][c], b = im[r][c];
      for (int o = 16; o; o >>= 1) {
        DS oa{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
        DS ob{__shfl_xor_sync(0xffffffffu, b.hi, o), __shfl_xor_sync(0xffffffffu, b.lo, o)};
        a = ds_add(a, oa);
        b = ds_add(b, ob);
      }
      if (lane == 0) { red[warp][r][c][0] = a; red[warp][r][c][1] = b; }
    }
  __syncthreads();
  for (int t = threadIdx.x; t < TR * N; t += blockDim.x) {
    const int r = t / N, c = t % N;
    const int64_t row = row0 + r;
    if (row >= M) continue;
    DS a{0.f, 0.f}, b{0.f, 0.f};
#pragma unroll
    for (int w = 0; w < DS_WARPS; ++w) {
      a = ds_add(a, red[w][r][c][0]);
      b = ds_add(b, red[w][r][c][1]);
    }
    C[row * ldc + c] = make_double2((double)a.hi + (double)a.lo, (double)b.hi + (double)b.lo);
  }
}

// FP32 variant of the same product from the hi planes only (plain FMA
// accumulation): for refinement steps whose residual is still large.
template <int N>
__global__ void __launch_bounds__(32 * DS_WARPS) k_gemm_thin_hi(int64_t M, int64_t K, const float2* __restrict__ Ahi,
                                                              int64_t lda, const float2* __restrict__ Bh, int64_t ldb,
                                                              double2* __restrict__ C, int64_t ldc) {
  __shared__ float2 red[DS_WARPS][DS_TR][N];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t row0 = (int64_t)blockIdx.x * DS_TR;
  const int64_t kw = (K + DS_WARPS - 1) / DS_WARPS;
  const int64_t kbeg = warp * kw, kend = min(K, kbeg + kw);
  int64_t roff[DS_TR];
#pragma unroll
  for (int r = 0; r < DS_TR; ++r) roff[r] = min(row0 + r, M - 1) * lda;
  float2 acc[DS_TR][N];
#pragma unroll
  for (int r = 0; r < DS_TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) acc[r][c] = make_float2(0.f, 0.f);
#pragma unroll 2
  for (int64_t k = kbeg + lane; k < kend; k += 32) {
    float2 xh[N];
#pragma unroll
    for (int c = 0; c < N; ++c) xh[c] = __ldg(Bh + k * ldb + c);
#pragma unroll
    for (int r = 0; r < DS_TR; ++r) {
      const float2 ah = __ldg(Ahi + roff[r] + k);
#pragma unroll
      for (int c = 0; c < N; ++c) cfma(acc[r][c], ah, xh[c]);
    }
  }
#pragma unroll
  for (int r = 0; r < DS_TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) {
      float2 v = acc[r][c];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[warp][r][c] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < DS_TR * N; t += blockDim.x) {
    const int r = t / N, c = t % N;
    const int64_t row = row0 + r;
    if (row >= M) continue;
    float2 v = make_float2(0.f, 0.f);
#pragma unroll
    for (int w = 0; w < DS_WARPS; ++w) v = cadd(v, red[w][r][c]);
    C[row * ldc + c] = make_double2(v.x, v.y);
  }
}

// the same product with 16-byte loads of A (two k per lane and load): even K
// and lda, 16-byte aligned A; the FP32 residual products of the refinement at
// large n, where the 8-byte loads above leave HBM half used
template <int N>
__global__ void __launch_bounds__(32 * DS_WARPS) k_gemm_thin_hi4(int64_t M, int64_t K, const float2* __restrict__ Ahi,
                                                               int64_t lda, const float2* __restrict__ Bh, int64_t ldb,
                                                               double2* __restrict__ C, int64_t ldc) {
  __shared__ float2 red[DS_WARPS][DS_TR][N];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t row0 = (int64_t)blockIdx.x * DS_TR;
  const int64_t KP = K >> 1;
  const int64_t kw = (KP + DS_WARPS - 1) / DS_WARPS;
  const int64_t pbeg = warp * kw, pend = min(KP, pbeg + kw);
  const float4* arow[DS_TR];
#pragma unroll
  for (int r = 0; r < DS_TR; ++r) arow[r] = reinterpret_cast<const float4*>(Ahi + min(row0 + r, M - 1) * lda);
  float2 acc[DS_TR][N];
#pragma unroll
  for (int r = 0; r < DS_TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) acc[r][c] = make_float2(0.f, 0.f);
#pragma unroll 2
  for (int64_t kp = pbeg + lane; kp < pend; kp += 32) {
    const int64_t k = 2 * kp;
    float2 x0[N], x1[N];
#pragma unroll
    for (int c = 0; c < N; ++c) {
      x0[c] = __ldg(Bh + k * ldb + c);
      x1[c] = __ldg(Bh + (k + 1) * ldb + c);
    }
    float4 a[DS_TR];
#pragma unroll
    for (int r = 0; r < DS_TR; ++r) a[r] = __ldg(arow[r] + kp);
#pragma unroll
    for (int r = 0; r < DS_TR; ++r) {
      const float2 a0 = make_float2(a[r].x, a[r].y), a1 = make_float2(a[r].z, a[r].w);
#pragma unroll
      for (int c = 0; c < N; ++c) {
        cfma(acc[r][c], a0, x0[c]);
        cfma(acc[r][c], a1, x1[c]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < DS_TR; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) {
      float2 v = acc[r][c];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[warp][r][c] = v;
    }
  __syncthreads();
  for (int t = threadIdx.x; t < DS_TR * N; t += blockDim.x) {
    const int r = t / N, c = t % N;
    const int64_t row = row0 + r;
    if (row >= M) continue;
    float2 v = make_float2(0.f, 0.f);
#pragma unroll
    for (int w = 0; w < DS_WARPS; ++w) v = cadd(v, red[w][r][c]);
    C[row * ldc + c] = make_double2(v.x, v.y);
  }
}

// ------------------------------------------- streamed thin GEMM (bulk copies)
// C[M x N] = A[M x K] * B[K x N], N <= 4, for a complex64 A far larger than
// L2 (the chain products and FP32 residuals of the refinement read a whole
// n x n matrix for a few right-hand sides: pure HBM streaming).  One CTA per
// SM owns a contiguous, balanced share of the rows.  A producer warp streams
// row segments of TS_KC complex values with bulk copies (cp.async.bulk: long
// sequential requests, TS_ST stages in flight) into shared memory; eight
// consumer warps take the chunk's k range in parallel (lane = k), read B
// through L1 and accumulate TS_TR rows x N in registers; at the end of a row
// block the warps' partial sums are added in a fixed order (deterministic).
// Sixteen consumer warps: TS_KG k groups x TS_RG row groups (TS_RPW rows each),
// so that each warp keeps few accumulators and each scheduler has four warps
// to hide the L1 / shared-memory latencies (eight warps with all rows each
// were latency bound: 29 % issue, 32 % of HBM).
// Waits are bounded; after a timeout every role skips the remaining waits
// (the result is then garbage and the error word is set) so that no barrier
// is left waiting.
constexpr int TS_TR = 8, TS_KC = 512, TS_ST = 4, TS_RG = 2, TS_KG = 8, TS_CW = TS_RG * TS_KG, TS_RPW = TS_TR / TS_RG;
constexpr int TS_THREADS = 32 * (TS_CW + 1);
constexpr int TS_STAGE = TS_TR * TS_KC * 8;               // 32 KB
constexpr int TS_SMEM = TS_ST * TS_STAGE;
__device__ int g_thin_stream_err;

__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void consumer_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(32 * TS_CW) : "memory");
}

// MODE 0: C (complex64) = alpha A B + beta C;  MODE 1: C (complex128) = A B
template <int N, int MODE>
__global__ void __launch_bounds__(TS_THREADS, 1)
    k_gemm_thin_stream(int64_t M, int64_t K, const float2* __restrict__ A, int64_t lda, const float2* __restrict__ B,
                       int64_t ldb, float2 alpha, float2 beta, void* __restrict__ Cv, int64_t ldc) {
  extern __shared__ __align__(128) unsigned char ts_smem[];
  __shared__ __align__(8) unsigned long long bars[2 * TS_ST];
  __shared__ float2 red[TS_KG][TS_TR][N];
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t rb = M * blockIdx.x / gridDim.x, re = M * (blockIdx.x + 1) / gridDim.x;
  const int64_t nchunk = (K + TS_KC - 1) / TS_KC;
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[TS_ST]);
  const uint32_t sbase = smem_u32(ts_smem);
  int* err = &g_thin_stream_err;
  volatile int* abort_v = &abort_flag;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TS_ST; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, TS_CW);
    }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (warp == TS_CW) {
    // ---------------- producer: row segments of the CTA's rows, block by block
    if (lane == 0) {
      int it = 0;
      for (int64_t r0 = rb; r0 < re && !*abort_v; r0 += TS_TR) {
        const int nr = (int)min((int64_t)TS_TR, re - r0);
        for (int64_t ch = 0; ch < nchunk; ++ch, ++it) {
          const int s = it % TS_ST;
          if (it >= TS_ST && !*abort_v && !mbar_wait(empty0 + 8 * s, ((it / TS_ST) - 1) & 1, err, 1)) *abort_v = 1;
          if (*abort_v) break;
          const int64_t k0 = ch * TS_KC;
          const uint32_t bytes = (uint32_t)min((int64_t)TS_KC, K - k0) * 8u;
          mbar_expect_tx(full0 + 8 * s, bytes * (uint32_t)nr);
          for (int r = 0; r < nr; ++r)
            bulk_copy_g2s(sbase + (uint32_t)(s * TS_STAGE + r * TS_KC * 8), A + (r0 + r) * lda + k0, bytes,
                          full0 + 8 * s);
        }
      }
      if (*abort_v) {
        // copies may still be landing: give them time before the CTA exits
        const unsigned long long t0 = gtimer();
        while (gtimer() - t0 < 200000ull) {
        }
      }
    }
  } else {
    // ---------------- consumers
    const float2* As = reinterpret_cast<const float2*>(ts_smem);
    const int rg = warp / TS_KG, kg = warp % TS_KG;
    int it = 0;
    for (int64_t r0 = rb; r0 < re; r0 += TS_TR) {
      const int nr = (int)min((int64_t)TS_TR, re - r0);
      const int nrw = max(0, min(TS_RPW, nr - rg * TS_RPW));   // this warp's rows in the block
      float2 acc[TS_RPW][N];
#pragma unroll
      for (int r = 0; r < TS_RPW; ++r)
#pragma unroll
        for (int c = 0; c < N; ++c) acc[r][c] = make_float2(0.f, 0.f);
      for (int64_t ch = 0; ch < nchunk; ++ch, ++it) {
        const int s = it % TS_ST;
        if (!*abort_v && !mbar_wait(full0 + 8 * s, (it / TS_ST) & 1, err, 2)) *abort_v = 1;
        const int64_t k0 = ch * TS_KC;
        const int kl = (int)min((int64_t)TS_KC, K - k0);
        const float2* Ast = As + s * (TS_TR * TS_KC) + rg * TS_RPW * TS_KC;
#pragma unroll
        for (int j = 0; j < TS_KC / (32 * TS_KG); ++j) {
          const int kk = kg * (TS_KC / TS_KG) + 32 * j + lane;
          if (kk < kl) {
            float2 b[N];
#pragma unroll
            for (int c = 0; c < N; ++c) b[c] = __ldg(B + (k0 + kk) * ldb + c);
#pragma unroll
            for (int r = 0; r < TS_RPW; ++r) {
              if (r < nrw) {
                const float2 a = Ast[r * TS_KC + kk];
#pragma unroll
                for (int c = 0; c < N; ++c) cfma(acc[r][c], a, b[c]);
              }
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty0 + 8 * s);
      }
#pragma unroll
      for (int r = 0; r < TS_RPW; ++r)
#pragma unroll
        for (int c = 0; c < N; ++c) {
          float2 v = acc[r][c];
#pragma unroll
          for (int o = 16; o; o >>= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
          }
          if (lane == 0) red[kg][rg * TS_RPW + r][c] = v;
        }
      consumer_sync();
      for (int t = threadIdx.x; t < nr * N; t += 32 * TS_CW) {
        const int r = t / N, c = t % N;
        float2 v = make_float2(0.f, 0.f);
#pragma unroll
        for (int w = 0; w < TS_KG; ++w) v = cadd(v, red[w][r][c]);
        const int64_t row = r0 + r;
        if (MODE == 0) {
          float2* C = reinterpret_cast<float2*>(Cv);
          float2 out = cmul(alpha, v);
          if (beta.x != 0.f || beta.y != 0.f) out = cadd(out, cmul(beta, C[row * ldc + c]));
          C[row * ldc + c] = out;
        } else {
          reinterpret_cast<double2*>(Cv)[row * ldc + c] = make_double2(v.x, v.y);
        }
      }
      consumer_sync();
    }
  }
  __syncthreads();
}

static int stream_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
      cudaGetLastError();
      sms = 148;
    }
  }
  return sms;
}

// the streamed kernel applies: N <= 4, even K and lda (16-byte row segments),
// a 16-byte aligned A, and a matrix of at least 2^22 entries.  Measured on
// GB300 (standalone, complex64): equal to the register-tiled kernel for N = 1,
// faster for N = 3 at n = 4000 (44 against 61 us), slower for N = 4 at
// n = 12000 (417 against 305 us); inside the multi-lane sweep at n = 4000 it
// shortens the thin-product phase by 15 %.  N = 4 uses it up to 2^26 entries.
static bool thin_stream_ok(int64_t M, int64_t N, int64_t K, const void* A, int64_t lda) {
  static int enabled = -1;
  if (enabled < 0) {
    const char* e = getenv("MNPBEM_THIN_STREAM");
    enabled = (e && e[0] == '0') ? 0 : 1;
  }
  const int64_t mk = M * K;
  return enabled && N >= 1 && N <= 4 && !(K & 1) && !(lda & 1) && !(reinterpret_cast<uintptr_t>(A) & 15) &&
         mk >= (int64_t(1) << 22) && (N <= 3 || mk <= (int64_t(1) << 26));
}

template <int MODE>
static mnpbem_status launch_thin_stream(int64_t M, int64_t N, int64_t K, const float2* A, int64_t lda,
                                        const float2* B, int64_t ldb, float2 alpha, float2 beta, void* C,
                                        int64_t ldc, cudaStream_t st) {
  static bool attr[2][5] = {};
  const unsigned grid = (unsigned)std::min<int64_t>(M, stream_sms());
#define TS_CASE(NN)                                                                                       \
  case NN:                                                                                                \
    if (!attr[MODE][NN]) {                                                                                \
      MNP_CUDA(cudaFuncSetAttribute(k_gemm_thin_stream<NN, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                    TS_SMEM));                                                            \
      attr[MODE][NN] = true;                                                                              \
    }                                                                                                     \
    k_gemm_thin_stream<NN, MODE><<<grid, TS_THREADS, TS_SMEM, st>>>(M, K, A, lda, B, ldb, alpha, beta, C, ldc); \
    break;
  switch (N) {
    TS_CASE(1) TS_CASE(2) TS_CASE(3) TS_CASE(4)
    default:
      set_error("thin stream GEMM: N must be 1..4");
      return MNPBEM_ERR_INVALID_ARG;
  }
#undef TS_CASE
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

mnpbem_status thin_stream_check(cudaStream_t st) {
  int* p = nullptr;
  MNP_CUDA(cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_thin_stream_err));
  int h = 0;
  MNP_CUDA(cudaMemcpyAsync(&h, p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  if (h) {
    MNP_CUDA(cudaMemsetAsync(p, 0, sizeof(int), st));
    set_error("streamed thin GEMM: a bounded pipeline wait expired (code %d)", h);
    return MNPBEM_ERR_TIMEOUT;
  }
  return MNPBEM_OK;
}

// B[:, 0:N] (row stride ldb) -> packed hi / lo planes [K][N]
__global__ void k_split_hi_lo_cols(const double2* __restrict__ B, int64_t ldb, int64_t K, int N, float2* hi,
                                   float2* lo) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K * N) return;
  const int64_t k = i / N;
  const double2 b = B[k * ldb + (i - k * N)];
  const float2 h = make_float2((float)b.x, (float)b.y);
  hi[i] = h;
  lo[i] = make_float2((float)(b.x - (double)h.x), (float)(b.y - (double)h.y));
}

static mnpbem_status gemm_thin_ds_block(int64_t M, int64_t N, int64_t K, const float2* Ahi, const float2* Alo,
                                        int64_t lda, const double2* B, int64_t ldb, double2* C, int64_t ldc,
                                        float2* bsplit, cudaStream_t st) {
  float2* Bh = bsplit;
  float2* Bl = bsplit + K * N;
  {
    ProfScope ps(PH_ELEMWISE, st, 0.0, 0.0, 1);
    if (ldb == N)
      k_split_hi_lo<<<(unsigned)cdiv_up(K * N, 256), 256, 0, st>>>(B, K * N, Bh, Bl);
    else
      k_split_hi_lo_cols<<<(unsigned)cdiv_up(K * N, 256), 256, 0, st>>>(B, ldb, K, (int)N, Bh, Bl);
    MNP_CHECK_LAUNCH();
  }
  const unsigned nblk = (unsigned)cdiv_up(M, (int64_t)DS_TR);
  if (!Alo) {
    ProfScope ps(PH_GEMM_SMALL, st, 8.0 * M * N * K, 8.0 * M * K + 8.0 * K * N + 16.0 * M * N);
    if (thin_stream_ok(M, N, K, Ahi, lda))
      return launch_thin_stream<1>(M, N, K, Ahi, lda, Bh, N, make_float2(1.f, 0.f), make_float2(0.f, 0.f), C, ldc, st);
    const bool v4 = !(K & 1) && !(lda & 1) && !(reinterpret_cast<uintptr_t>(Ahi) & 15);
#define HI_CASE(NN)                                                                                \
  case NN:                                                                                         \
    if (v4) k_gemm_thin_hi4<NN><<<nblk, 32 * DS_WARPS, 0, st>>>(M, K, Ahi, lda, Bh, N, C, ldc);    \
    else k_gemm_thin_hi<NN><<<nblk, 32 * DS_WARPS, 0, st>>>(M, K, Ahi, lda, Bh, N, C, ldc);        \
    break;
    switch (N) {
      HI_CASE(1) HI_CASE(2) HI_CASE(3) HI_CASE(4) HI_CASE(5) HI_CASE(6) HI_CASE(7) HI_CASE(8)
    }
#undef HI_CASE
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  ProfScope ps(PH_GEMM_SMALL, st, 8.0 * M * N * K, 16.0 * M * K + 16.0 * K * N + 16.0 * M * N);
  // two rows per block (80 registers, 3 blocks per SM) measured faster than
  // four rows (128 registers) or an unrolled k loop
  constexpr int TR = 2;
  const unsigned nb2 = (unsigned)cdiv_up(M, (int64_t)TR);
#define DS_CASE(NN)                                                                                        \
  case NN:                                                                                                 \
    k_gemm_thin_ds<NN, TR, 1><<<nb2, 32 * DS_WARPS, 0, st>>>(M, K, Ahi, Alo, lda, Bh, Bl, N, C, ldc);       \
    break;
  switch (N) {
    DS_CASE(1) DS_CASE(2) DS_CASE(3) DS_CASE(4) DS_CASE(5) DS_CASE(6) DS_CASE(7) DS_CASE(8)
  }
#undef DS_CASE
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

// columns in blocks of at most 8 (the kernels' register-tiled widths)
mnpbem_status gemm_thin_ds(int64_t M, int64_t N, int64_t K, const float2* Ahi, const float2* Alo,
                           int64_t lda, const double2* B, int64_t ldb, double2* C, int64_t ldc,
                           float2* bsplit, cudaStream_t st) {
  if (M <= 0 || N <= 0) return MNPBEM_OK;
  if (K <= 0 || ldb < N) { set_error("gemm_thin_ds: invalid sizes"); return MNPBEM_ERR_INVALID_ARG; }
  for (int64_t c0 = 0; c0 < N; c0 += 8) {
    const int64_t w = std::min<int64_t>(8, N - c0);
    MNP_TRY(gemm_thin_ds_block(M, w, K, Ahi, Alo, lda, B + c0, ldb, C + c0, ldc, bsplit, st));
  }
  return MNPBEM_OK;
}

template <typename R>
mnpbem_status gemm_simt(int64_t M, int64_t N, int64_t K, cplx<R> alpha, const cplx<R>* A,
                        int64_t lda, const cplx<R>* B, int64_t ldb, cplx<R> beta, cplx<R>* C,
                        int64_t ldc, cudaStream_t st) {
  if (M <= 0 || N <= 0) return MNPBEM_OK;
  if (sizeof(R) == 4 && N <= 8 && K > 1 && !(lda & 1) && !(reinterpret_cast<uintptr_t>(A) & 15)) {
    ProfScope ps(PH_GEMM_SMALL, st, 8.0 * M * N * K,
                 (double)sizeof(cplx<R>) * ((double)M * K + (double)K * N + 2.0 * M * N));
    const float2* Af = reinterpret_cast<const float2*>(A);
    const float2* Bf = reinterpret_cast<const float2*>(B);
    float2* Cf = reinterpret_cast<float2*>(C);
    const float2 al = make_float2((float)alpha.x, (float)alpha.y), be = make_float2((float)beta.x, (float)beta.y);
    if (N <= 4 && thin_stream_ok(M, N, K, Af, lda))
      return launch_thin_stream<0>(M, N, K, Af, lda, Bf, ldb, al, be, Cf, ldc, st);
#define C64_CASE(NN)                                                                                    \
  case NN:                                                                                              \
    k_gemm_thin_c64<NN, 4><<<(unsigned)cdiv_up(M, 4), 32 * THIN_WARPS, 0, st>>>(M, K, al, Af, lda, Bf, ldb, be, Cf, ldc); \
    break;
    switch (N) {
      C64_CASE(1) C64_CASE(2) C64_CASE(3) C64_CASE(4) C64_CASE(5) C64_CASE(6) C64_CASE(7) C64_CASE(8)
    }
#undef C64_CASE
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  if (N <= THIN_NMAX && K > 0) {
    ProfScope ps(PH_GEMM_SMALL, st, 8.0 * M * N * K,
                 (double)sizeof(cplx<R>) * ((double)M * K + (double)K * N + 2.0 * M * N));
    // rows per block: fewer for wide B so that the accumulators stay in registers
#define THIN_CASE(NN)                                                                              \
  case NN: {                                                                                       \
    constexpr int TR = NN <= 8 ? 4 : (sizeof(R) == 8 ? 1 : 2);                                     \
    k_gemm_thin<R, NN, TR><<<(unsigned)cdiv_up(M, TR), 32 * THIN_WARPS, 0, st>>>(M, K, alpha, A, lda, B, ldb, beta, C, ldc); \
    break;                                                                                         \
  }
    switch (N) {
      THIN_CASE(1) THIN_CASE(2) THIN_CASE(3) THIN_CASE(4) THIN_CASE(5) THIN_CASE(6) THIN_CASE(7)
      THIN_CASE(8) THIN_CASE(9) THIN_CASE(10) THIN_CASE(11) THIN_CASE(12) THIN_CASE(13) THIN_CASE(14)
      THIN_CASE(15) THIN_CASE(16)
    }
#undef THIN_CASE
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  dim3 grid((unsigned)cdiv_up(N, 64), (unsigned)cdiv_up(M, 64));
  if (grid.y > 65535) { set_error("gemm_simt: M too large"); return MNPBEM_ERR_INVALID_ARG; }
  constexpr int BK = sizeof(R) == 4 ? 16 : 8;
  const bool big = M >= 128 && N >= 128;
  ProfScope ps(big ? PH_GEMM_BIG : PH_GEMM_SMALL, st, 8.0 * M * N * K,
               (double)sizeof(cplx<R>) * ((double)M * K + (double)K * N + 2.0 * M * N));
  k_gemm_nn<R, BK><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}
template mnpbem_status gemm_simt<float>(int64_t, int64_t, int64_t, float2, const float2*, int64_t,
                                        const float2*, int64_t, float2, float2*, int64_t, cudaStream_t);
template mnpbem_status gemm_simt<double>(int64_t, int64_t, int64_t, double2, const double2*, int64_t,
                                         const double2*, int64_t, double2, double2*, int64_t,
                                         cudaStream_t);

// --------------------------------------------------- block inversion
// Largest per-block condition proxy max|A_kk| * max|inv(A_kk)|, kept as the
// bits of a non-negative float in status[1] (integer order = float order).
__device__ __forceinline__ void record_cond(int* status, double amax, double xmax) {
  double c = amax * xmax;
  if (!(c == c) || c > 3.0e38) c = 3.0e38;
  atomicMax(status + 1, __float_as_int((float)c));
}

// In-place Gauss-Jordan of one w x w block (w <= 64) with partial pivoting
// inside the block.  256 threads as a 16 x 16 grid; thread (ty, tx) keeps the
// 16 entries (ty + 16 i, tx + 16 j) in registers.  Pivoting is implicit: step p
// takes as pivot row r_p the row, among those not yet used, with the largest
// |a_rp| in column p, and eliminates with (r_p, p) in place of (p, p).  The
// matrix M this leaves satisfies inv(A)[q][r_k] = M[r_q][k], so the block is
// written out through the permutation.  Two __syncthreads per step: after the
// pivot column is published, and after the pivot row is.
template <typename R>
__global__ void __launch_bounds__(256) k_block_inv(const cplx<R>* __restrict__ A, int64_t lda, int w,
                                                   cplx<R>* __restrict__ X, int64_t ldx, int* status) {
  using Cx = cplx<R>;
  __shared__ Cx prow[2][64], pcol[2][64];
  __shared__ int prow_of[64], pos_of[64];
  __shared__ unsigned char used[64];
  __shared__ double red[8];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  Cx a[4][4];
  double amax = 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = ty + 16 * i, c = tx + 16 * j;
      a[i][j] = (r < w && c < w) ? A[r * lda + c] : mk<R>(r == c ? 1 : 0, 0);
      if (r < w && c < w) amax = fmax(amax, sqrt(cabs2(a[i][j])));
    }
  if (t < 64) used[t] = 0;
  for (int p = 0; p < w; ++p) {
    const int buf = p & 1;
    // 1. publish column p
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (tx + 16 * j == p) pcol[buf][ty + 16 * i] = a[i][j];
    __syncthreads();
    // 2. pivot row: largest modulus among the unused rows (first one on ties)
    int rp = -1;
    R best = -1;
    for (int r = 0; r < w; ++r) {
      if (used[r]) continue;
      const Cx v = pcol[buf][r];
      const R m2 = v.x * v.x + v.y * v.y;
      if (rp < 0 || m2 > best) { best = m2; rp = r; }
    }
    // 3. publish the pivot row
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (ty + 16 * i == rp) prow[buf][tx + 16 * j] = a[i][j];
    __syncthreads();
    if (t == 0) {
      used[rp] = 1;
      prow_of[p] = rp;
      pos_of[rp] = p;
    }
    const Cx piv = prow[buf][p];
    const R n2 = piv.x * piv.x + piv.y * piv.y;
    if (t == 0 && !(n2 > (R)1e-30 && n2 < (R)1e30)) atomicOr(status, 1);
    const R rn2 = (R)1 / n2;
    const Cx inv = mk<R>(piv.x * rn2, -piv.y * rn2);
    // One update a - pc_r pr_c serves every entry when the pivot column of pr
    // holds 1 + 1/a_pp and the pivot row of pc holds a_pp - 1:
    //   pivot row:    a_rc - (a_pp - 1) a_rc / a_pp = a_rc / a_pp
    //   column p:     a_ip - a_ip (1 + 1/a_pp)      = -a_ip / a_pp
    // (the pivot itself is set to 1/a_pp directly).
    Cx pr[4], pc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = tx + 16 * j;
      pr[j] = (c == p) ? mk<R>(1 + inv.x, inv.y) : cmul(prow[buf][c], inv);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = ty + 16 * i;
      pc[i] = (r == rp) ? mk<R>(piv.x - 1, piv.y) : pcol[buf][r];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const Cx v = csub(a[i][j], cmul(pc[i], pr[j]));
        a[i][j] = (ty + 16 * i == rp && tx + 16 * j == p) ? inv : v;
      }
  }
  __syncthreads();
  double xmax = 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = ty + 16 * i, c = tx + 16 * j;
      if (r < w && c < w) {
        X[(int64_t)pos_of[r] * ldx + prow_of[c]] = a[i][j];
        xmax = fmax(xmax, sqrt(cabs2(a[i][j])));
      }
    }
  // block maxima of |A| and |X| for the condition proxy
  for (int o = 16; o; o >>= 1) {
    amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    xmax = fmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
  }
  if ((t & 31) == 0) red[t >> 5] = amax;
  __syncthreads();
  if (t == 0) {
    double am = 0.0;
    for (int k = 0; k < 8; ++k) am = fmax(am, red[k]);
    red[0] = am;
  }
  __syncthreads();
  amax = red[0];
  __syncthreads();
  if ((t & 31) == 0) red[t >> 5] = xmax;
  __syncthreads();
  if (t == 0) {
    double xm = 0.0;
    for (int k = 0; k < 8; ++k) xm = fmax(xm, red[k]);
    record_cond(status, amax, xm);
  }
}

// ------------------------------------- 256-wide pivot block on a CTA cluster
// In-place Gauss-Jordan of one w x w complex64 block (w <= 256) by a cluster
// of PB_CL CTAs.  CTA r keeps rows [r*PB_RPC, (r+1)*PB_RPC) in registers:
// PB_TPR threads per row, thread (row l, phase ph) holding the columns
// ph + PB_TPR * j.  The pivots are taken in panels of 16:
//   1. the CTA owning the panel rows stages them in shared memory, inverts
//      the 16 x 16 pivot block X (Gauss-Jordan, one entry per thread) and
//      forms the new panel rows R = X * P (pivot columns replaced by X);
//   2. every CTA stages its own 16 panel-column entries C; cluster barrier;
//      the other CTAs copy R out of the owner's shared memory (distributed
//      shared memory reads, spread over the cluster);
//   3. every row i outside the panel: a_ij <- [j not a pivot column] a_ij
//      - sum_k C_ik R_kj; the panel rows take R.
// One cluster barrier per panel (R is double-buffered: a CTA may still be
// copying panel p's R when the owner of panel p + 1 writes the other buffer),
// 16 panels for w = 256.
// Rows and columns beyond w are identity and stay identity.
constexpr int PB_W = 256, PB_CL = 8, PB_RPC = PB_W / PB_CL, PB_THREADS = 512;
constexpr int PB_TPR = PB_THREADS / PB_RPC, PB_CPT = PB_W / PB_TPR, PB_PAN = 16;
constexpr int PB_SMEM = (3 * PB_PAN * PB_W + 2 * PB_RPC * PB_PAN + 2 * PB_PAN * PB_PAN) * (int)sizeof(float2);
static_assert(PB_PAN % PB_TPR == 0 || PB_TPR % PB_PAN == 0, "panel / thread layout");
static_assert(PB_RPC % PB_PAN == 0, "a panel lies inside one CTA");

__global__ void __cluster_dims__(PB_CL, 1, 1) __launch_bounds__(PB_THREADS, 1)
    k_block_inv_cluster(const float2* A, int64_t lda, int w, float2* X, int64_t ldx, int* status,
                        float2* __restrict__ Xr) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ float2 pb_smem[];
  float2* Rb = pb_smem;                              // [2][PAN][W]  new panel rows
  float2* P = Rb + 2 * PB_PAN * PB_W;                // [PAN][W]     owner: raw panel rows
  float2* Cb = P + PB_PAN * PB_W;                    // [2][RPC][PAN] own panel-column entries
  float2* Xs = Cb + 2 * PB_RPC * PB_PAN;             // [2][PAN][PAN] pivot block, two copies (owner)
  const int rank = (int)cluster.block_rank();
  const int t = threadIdx.x, lr = t / PB_TPR, ph = t % PB_TPR;
  const int grow = rank * PB_RPC + lr;
  __shared__ float cond_red[PB_THREADS / 32], cond_loc[2];
  float2 a[PB_CPT];
  float amax = 0.f;
#pragma unroll
  for (int j = 0; j < PB_CPT; ++j) {
    const int c = ph + PB_TPR * j;
    a[j] = (grow < w && c < w) ? A[(int64_t)grow * lda + c] : make_float2(grow == c ? 1.f : 0.f, 0.f);
    if (grow < w && c < w) amax = fmaxf(amax, sqrtf(a[j].x * a[j].x + a[j].y * a[j].y));
  }
  // CTA maximum of a per-thread value into cond_loc[slot]
  const auto cta_max = [&](float v, int slot) {
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((t & 31) == 0) cond_red[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
      float mx = 0.f;
      for (int k = 0; k < PB_THREADS / 32; ++k) mx = fmaxf(mx, cond_red[k]);
      cond_loc[slot] = mx;
    }
    __syncthreads();
  };
  cta_max(amax, 0);
  const int npan = (w + PB_PAN - 1) / PB_PAN;
  for (int pp = 0; pp < npan; ++pp) {
    const int p0 = pp * PB_PAN, owner = p0 / PB_RPC, lp0 = p0 % PB_RPC, buf = pp & 1;
    float2* R = Rb + buf * PB_PAN * PB_W;
    float2* C = Cb + buf * PB_RPC * PB_PAN;
    __syncthreads();                                  // the previous panel's reads of P / C are done
    // own panel-column entries (every CTA)
#pragma unroll
    for (int j = 0; j < PB_CPT; ++j) {
      const int c = ph + PB_TPR * j;
      if (c >= p0 && c < p0 + PB_PAN) C[lr * PB_PAN + (c - p0)] = a[j];
    }
    if (rank == owner) {
      if (lr >= lp0 && lr < lp0 + PB_PAN) {
#pragma unroll
        for (int j = 0; j < PB_CPT; ++j) P[(lr - lp0) * PB_W + ph + PB_TPR * j] = a[j];
      }
      __syncthreads();
      // 16 x 16 Gauss-Jordan of the pivot block, one entry per thread; the
      // pivot steps alternate between two copies of the block, so that one
      // block barrier per step suffices
      const int bi = t / PB_PAN, bj = t % PB_PAN;
      const bool act = t < PB_PAN * PB_PAN;
      if (act) Xs[bi * PB_PAN + bj] = P[bi * PB_W + p0 + bj];
      __syncthreads();
      for (int k = 0; k < PB_PAN; ++k) {
        const float2* Xc = Xs + (k & 1) * PB_PAN * PB_PAN;
        float2* Xn = Xs + ((k & 1) ^ 1) * PB_PAN * PB_PAN;
        if (act) {
          const float2 piv = Xc[k * PB_PAN + k];
          const float n2 = piv.x * piv.x + piv.y * piv.y;
          if (t == 0 && !(n2 > 1e-30f && n2 < 1e30f)) atomicOr(status, 1);
          const float rn = 1.f / n2;
          const float2 inv = make_float2(piv.x * rn, -piv.y * rn);
          const float2 aik = Xc[bi * PB_PAN + k], akj = Xc[k * PB_PAN + bj], aij = Xc[bi * PB_PAN + bj];
          float2 v;
          if (bi == k && bj == k) v = inv;
          else if (bi == k) v = cmul(akj, inv);
          else if (bj == k) v = make_float2(-(aik.x * inv.x - aik.y * inv.y), -(aik.x * inv.y + aik.y * inv.x));
          else v = csub(aij, cmul(aik, cmul(akj, inv)));
          Xn[bi * PB_PAN + bj] = v;
        }
        __syncthreads();
      }
      // PB_PAN is even: the result is back in the first copy
      static_assert(PB_PAN % 2 == 0, "the pivot block's Gauss-Jordan ends in its first copy");
      // R = X * P with the pivot columns replaced by X
      for (int e = t; e < PB_PAN * PB_W; e += PB_THREADS) {
        const int i = e / PB_W, c = e % PB_W;
        float2 r;
        if (c >= p0 && c < p0 + PB_PAN) {
          r = Xs[i * PB_PAN + (c - p0)];
        } else {
          r = make_float2(0.f, 0.f);
#pragma unroll
          for (int k = 0; k < PB_PAN; ++k) cfma(r, Xs[i * PB_PAN + k], P[k * PB_W + c]);
        }
        R[e] = r;
      }
    }
    cluster.sync();
    if (rank != owner) {
      const float4* src = reinterpret_cast<const float4*>(cluster.map_shared_rank(R, owner));
      float4* dst = reinterpret_cast<float4*>(R);
#pragma unroll 4
      for (int e = t; e < PB_PAN * PB_W / 2; e += PB_THREADS) dst[e] = src[e];
      __syncthreads();
    }
    // update of this CTA's rows
    const bool prow = (rank == owner) && lr >= lp0 && lr < lp0 + PB_PAN;
    if (prow) {
#pragma unroll
      for (int j = 0; j < PB_CPT; ++j) a[j] = R[(lr - lp0) * PB_W + ph + PB_TPR * j];
    } else {
      float2 cr[PB_PAN];
#pragma unroll
      for (int k = 0; k < PB_PAN; ++k) cr[k] = C[lr * PB_PAN + k];
#pragma unroll
      for (int j = 0; j < PB_CPT; ++j) {
        const int c = ph + PB_TPR * j;
        float2 acc = (c >= p0 && c < p0 + PB_PAN) ? make_float2(0.f, 0.f) : a[j];
#pragma unroll
        for (int k = 0; k < PB_PAN; ++k) {
          const float2 rv = R[k * PB_W + c];
          acc.x = fmaf(-cr[k].x, rv.x, acc.x);
          acc.x = fmaf(cr[k].y, rv.y, acc.x);
          acc.y = fmaf(-cr[k].x, rv.y, acc.y);
          acc.y = fmaf(-cr[k].y, rv.x, acc.y);
        }
        a[j] = acc;
      }
    }
  }
  float xmax = 0.f;
  if (grow < w) {
#pragma unroll
    for (int j = 0; j < PB_CPT; ++j) {
      const int c = ph + PB_TPR * j;
      if (c < w) xmax = fmaxf(xmax, sqrtf(a[j].x * a[j].x + a[j].y * a[j].y));
    }
  }
  cta_max(xmax, 1);
  // no CTA may exit while another can still write into (or read) its shared memory
  cluster.sync();
  if (rank == 0 && t == 0) {
    float am = 0.f, xm = 0.f;
    for (int r = 0; r < PB_CL; ++r) {
      const float* cl = cluster.map_shared_rank(cond_loc, r);
      am = fmaxf(am, cl[0]);
      xm = fmaxf(xm, cl[1]);
    }
    record_cond(status, am, xm);
  }
  // X may be the input block itself: every CTA read its rows at the start
  if (grow < w) {
#pragma unroll
    for (int j = 0; j < PB_CPT; ++j) {
      const int c = ph + PB_TPR * j;
      if (c < w) {
        X[(int64_t)grow * ldx + c] = a[j];
        if (Xr) {   // copy rounded to TF32 (nearest): the A operand of tensor-core products
          uint32_t x, y;
          asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(x) : "f"(a[j].x));
          asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(y) : "f"(a[j].y));
          Xr[(int64_t)grow * w + c] = make_float2(__uint_as_float(x), __uint_as_float(y));
        }
      }
    }
  }
  cluster.sync();
}

static mnpbem_status launch_block_inv_cluster(const float2* A, int64_t lda, int w, float2* X, int64_t ldx,
                                              int* status, cudaStream_t st, float2* Xr = nullptr) {
  static bool attr_set = false;
  if (!attr_set) {
    MNP_CUDA(cudaFuncSetAttribute(k_block_inv_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, PB_SMEM));
    attr_set = true;
  }
  ProfScope ps(PH_BLOCKINV, st, 8.0 * w * w * w, 0.0);
  k_block_inv_cluster<<<PB_CL, PB_THREADS, PB_SMEM, st>>>(A, lda, w, X, ldx, status, Xr);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

// ------------------------------------------------ TF32 rounding in place
// The tensor cores read an FP32 operand as TF32 by dropping its 13 low
// mantissa bits (truncation, biased towards zero); operands rounded to nearest
// beforehand (cvt.rna.tf32) carry half the error and no bias.  The B operand
// is rounded when it is expanded; this rounds an A operand.
__global__ void k_round_tf32(float* x, int64_t count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x[i]));
  x[i] = __uint_as_float(r);
}

void round_tf32(float* x, int64_t count, cudaStream_t st) {
  if (count <= 0) return;
  ProfScope ps(PH_ELEMWISE, st, 0.0, 8.0 * count, 1);
  k_round_tf32<<<(unsigned)cdiv_up(count, 256), 256, 0, st>>>(x, count);
}

// Ccol[n][bw] <- A[:, k0 .. k0 + bw) with the rows k0 .. k0 + bw zeroed and,
// if rna, rounded to TF32 (nearest): the A operand of the column-panel product
// and of the rank update of one fused Gauss-Jordan step.
__global__ void k_gj_take_col(const float2* __restrict__ A, int64_t lda, int64_t n, int64_t k0, int bw,
                              float2* __restrict__ Ccol, int rna) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * bw) return;
  const int64_t i = idx / bw;
  const int c = (int)(idx - i * bw);
  float2 v = make_float2(0.f, 0.f);
  if (i < k0 || i >= k0 + bw) {
    v = A[i * lda + k0 + c];
    if (rna) {
      uint32_t x, y;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(x) : "f"(v.x));
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(y) : "f"(v.y));
      v = make_float2(__uint_as_float(x), __uint_as_float(y));
    }
  }
  Ccol[idx] = v;
}

// --------------------------------------------------- blocked Gauss-Jordan
template <typename R>
mnpbem_status gj_status_copy(GJWork<R>& w, int* host2, cudaStream_t st) {
  host2[0] = host2[1] = 0;
  if (w.status.ptr) MNP_CUDA(cudaMemcpyAsync(host2, w.status.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (w.inner && w.inner->status.ptr)
    MNP_CUDA(cudaMemcpyAsync(host2 + 1, w.inner->status.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  return MNPBEM_OK;
}
template mnpbem_status gj_status_copy<float>(GJWork<float>&, int*, cudaStream_t);
template mnpbem_status gj_status_copy<double>(GJWork<double>&, int*, cudaStream_t);

template <typename R>
mnpbem_status gj_invert(cplx<R>* A, int64_t n, int64_t lda, GJWork<R>& w, GemmFn<R> big_gemm,
                        void* ctx, cudaStream_t st, bool read_status) {
  using Cx = cplx<R>;
  const int nb = w.nb;
  const size_t cs = sizeof(Cx);
  MNP_TRY(w.ccol.ensure(cs * n * nb));
  MNP_TRY(w.rrow.ensure(cs * n * nb));
  MNP_TRY(w.ncol.ensure(cs * n * nb));
  MNP_TRY(w.xblk.ensure(cs * nb * nb));
  MNP_TRY(w.status.ensure(2 * sizeof(int)));
  if (!w.nested) MNP_CUDA(cudaMemsetAsync(w.status.ptr, 0, 2 * sizeof(int), st));
  if (!w.nested && nb > 64 && (sizeof(R) == 8 || nb > PB_W)) {
    // pivot blocks wider than 64 are inverted by an inner Gauss-Jordan whose
    // pivot status this (outer) level clears now and reads at the end
    if (!w.inner) w.inner.reset(new GJWork<R>());
    // complex64 with pivot blocks wider than 256: 256-wide inner steps whose
    // own pivot blocks go to the cluster kernel; otherwise 64-wide steps
    w.inner->nb = (sizeof(R) == 4 && nb > PB_W) ? PB_W : 64;
    w.inner->nested = true;
    MNP_TRY(w.inner->status.ensure(2 * sizeof(int)));
    MNP_CUDA(cudaMemsetAsync(w.inner->status.ptr, 0, 2 * sizeof(int), st));
  }
  Cx* Ccol = w.ccol.template as<Cx>();   // [n][nb]
  Cx* Rrow = w.rrow.template as<Cx>();   // [nb][n]
  Cx* Ncol = w.ncol.template as<Cx>();   // [n][nb]
  Cx* X = w.xblk.template as<Cx>();      // [nb][nb]
  const Cx one = mk<R>(1, 0), zero = mk<R>(0, 0), mone = mk<R>(-1, 0);
  for (int64_t k0 = 0; k0 < n; k0 += nb) {
    const int bw = (int)std::min<int64_t>(nb, n - k0);
    if constexpr (sizeof(R) == 4) {
      // Fused step on the tensor-core path (all three products eligible):
      //   X <- inv(A_kk) read in place; Ccol <- TF32(A[:, k]) with rows k zeroed;
      //   A[k, :] <- X A[k, :] in place (the product copies its B operand before it
      //   runs); A[:, k] <- -Ccol X (rows k become 0); A <- A - Ccol A[k, :] with the
      //   k columns of the B operand read as zero (rows and columns k unchanged);
      //   A_kk <- X.  The same products as the general step below, without its
      //   panel copies and write-backs.
      TcGemmCtx* tc = reinterpret_cast<TcGemmCtx*>(ctx);
      const float2 b0 = make_float2(0.f, 0.f), b1 = make_float2(1.f, 0.f);
      float2* Af = reinterpret_cast<float2*>(A);
      float2* Cf = reinterpret_cast<float2*>(Ccol);
      float2* Xf = reinterpret_cast<float2*>(X);
      if (tc && w.fused && (bw <= PB_W || w.inner) && tc_gemm_eligible(*tc, bw, n, bw, Xf, bw, Af + k0 * lda, lda, b0) &&
          tc_gemm_eligible(*tc, n, bw, bw, Cf, bw, Af + k0, lda, b0) &&
          tc_gemm_eligible(*tc, n, n, bw, Cf, bw, Af, lda, b1)) {
        if (bw <= 64) {
          ProfScope ps(PH_BLOCKINV, st, 8.0 * bw * bw * bw, 0.0);
          k_block_inv<R><<<1, 256, 0, st>>>(A + k0 * lda + k0, lda, bw, X, bw, w.status.template as<int>());
          MNP_CHECK_LAUNCH();
        } else if (bw <= PB_W) {
          MNP_TRY(launch_block_inv_cluster(Af + k0 * lda + k0, lda, bw, Xf, bw, w.status.template as<int>(), st));
        } else {
          // wider pivot blocks: inner Gauss-Jordan (256-wide steps) on a copy
          MNP_CUDA(cudaMemcpy2DAsync(X, cs * bw, A + k0 * lda + k0, cs * lda, cs * bw, bw, cudaMemcpyDeviceToDevice,
                                     st));
          MNP_TRY(gj_invert<R>(X, bw, bw, *w.inner, big_gemm, ctx, st));
        }
        {
          ProfScope ps(PH_ELEMWISE, st, 0.0, 16.0 * n * bw, 1);
          k_gj_take_col<<<(unsigned)cdiv_up(n * bw, (int64_t)256), 256, 0, st>>>(Af, lda, n, k0, bw, Cf,
                                                                                 w.round_a ? 1 : 0);
          MNP_CHECK_LAUNCH();
        }
        MNP_TRY(tc_gemm_c64(*tc, bw, n, bw, b1, Xf, bw, Af + k0 * lda, lda, b0, Af + k0 * lda, lda, st));
        MNP_TRY(tc_gemm_c64(*tc, n, bw, bw, make_float2(-1.f, 0.f), Cf, bw, Xf, bw, b0, Af + k0, lda, st));
        MNP_TRY(tc_gemm_c64(*tc, n, n, bw, make_float2(-1.f, 0.f), Cf, bw, Af + k0 * lda, lda, b1, Af, lda, st,
                            k0, k0 + bw));
        MNP_CUDA(cudaMemcpy2DAsync(A + k0 * lda + k0, cs * lda, X, cs * bw, cs * bw, bw, cudaMemcpyDeviceToDevice, st));
        continue;
      }
    }
    // 1. Ccol <- A[:, k-block]
    MNP_CUDA(cudaMemcpy2DAsync(Ccol, cs * bw, A + k0, cs * lda, cs * bw, n, cudaMemcpyDeviceToDevice, st));
    // 2. X <- inv(A_kk): one shared-memory kernel for blocks up to 64, else
    //    an inner Gauss-Jordan with 64-wide steps on a copy of the block
    if (bw <= 64) {
      ProfScope ps(PH_BLOCKINV, st, 8.0 * bw * bw * bw, 0.0);
      k_block_inv<R><<<1, 256, 0, st>>>(Ccol + k0 * bw, bw, bw, X, bw, w.status.template as<int>());
      MNP_CHECK_LAUNCH();
    } else if (sizeof(R) == 4 && bw <= PB_W) {
      MNP_TRY(launch_block_inv_cluster(reinterpret_cast<const float2*>(Ccol + k0 * bw), bw, bw,
                                       reinterpret_cast<float2*>(X), bw, w.status.template as<int>(), st));
    } else {
      MNP_CUDA(cudaMemcpyAsync(X, Ccol + k0 * bw, cs * bw * bw, cudaMemcpyDeviceToDevice, st));
      MNP_TRY(gj_invert<R>(X, bw, bw, *w.inner, big_gemm, ctx, st));
    }
    // 3. R <- X * A[k-block, :], then zero its k-block columns
    MNP_TRY(big_gemm(bw, n, bw, one, X, bw, A + k0 * lda, lda, zero, Rrow, n, st, ctx));
    MNP_CUDA(cudaMemset2DAsync(Rrow + k0, cs * n, 0, cs * bw, bw, st));
    // 4. new column block <- -Ccol * X, then zero Ccol's k-block rows
    //    (on the tensor-core path Ccol, the A operand of this product and of
    //    the rank update, is first rounded to TF32; the pivot block it holds
    //    has already been inverted in full FP32)
    if (sizeof(R) == 4 && ctx && w.round_a) round_tf32(reinterpret_cast<float*>(Ccol), 2 * n * bw, st);
    MNP_TRY(big_gemm(n, bw, bw, mone, Ccol, bw, X, bw, zero, Ncol, bw, st, ctx));
    MNP_CUDA(cudaMemsetAsync(Ccol + k0 * bw, 0, cs * bw * bw, st));
    // 5. A <- A - Ccol * R  (rank-bw update of the whole matrix)
    MNP_TRY(big_gemm(n, n, bw, mone, Ccol, bw, Rrow, n, one, A, lda, st, ctx));
    // 6. write back row block, column block and the inverted pivot block
    MNP_CUDA(cudaMemcpy2DAsync(A + k0 * lda, cs * lda, Rrow, cs * n, cs * n, bw, cudaMemcpyDeviceToDevice, st));
    MNP_CUDA(cudaMemcpy2DAsync(A + k0, cs * lda, Ncol, cs * bw, cs * bw, n, cudaMemcpyDeviceToDevice, st));
    MNP_CUDA(cudaMemcpy2DAsync(A + k0 * lda + k0, cs * lda, X, cs * bw, cs * bw, bw, cudaMemcpyDeviceToDevice, st));
  }
  if (w.nested || !read_status) return MNPBEM_OK;
  int hs = 0;
  MNP_CUDA(cudaMemcpyAsync(&hs, w.status.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  if (w.inner) {
    int hi = 0;
    MNP_CUDA(cudaMemcpyAsync(&hi, w.inner->status.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    MNP_CUDA(cudaStreamSynchronize(st));
    hs |= hi;
  }
  if (hs) {
    set_error("block Gauss-Jordan inversion: zero or non-finite pivot");
    return MNPBEM_ERR_SINGULAR;
  }
  return MNPBEM_OK;
}

template mnpbem_status gj_invert<float>(float2*, int64_t, int64_t, GJWork<float>&, GemmFn<float>,
                                        void*, cudaStream_t, bool);
template mnpbem_status gj_invert<double>(double2*, int64_t, int64_t, GJWork<double>&,
                                         GemmFn<double>, void*, cudaStream_t, bool);

// ------------------------------------------------------ block LDU factors
// dst[rows][cols] (row stride ldd) <- src[rows][cols] (row stride lds),
// rounded to TF32 (nearest) when rna: the A operand of a tensor-core product
template <typename R>
__global__ void k_copy_panel(const cplx<R>* __restrict__ src, int64_t lds, int64_t rows, int cols,
                             cplx<R>* __restrict__ dst, int64_t ldd, int rna) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= rows * cols) return;
  const int64_t i = idx / cols;
  const int c = (int)(idx - i * cols);
  cplx<R> v = src[i * lds + c];
  if constexpr (sizeof(R) == 4) {
    if (rna) {
      uint32_t x, y;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(x) : "f"(v.x));
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(y) : "f"(v.y));
      v = mk<R>(__uint_as_float(x), __uint_as_float(y));
    }
  }
  dst[i * ldd + c] = v;
}

template <typename R>
static void copy_panel(const cplx<R>* src, int64_t lds, int64_t rows, int cols, cplx<R>* dst, int64_t ldd, bool rna,
                       cudaStream_t st) {
  if (rows <= 0 || cols <= 0) return;
  ProfScope ps(PH_ELEMWISE, st, 0.0, 2.0 * sizeof(cplx<R>) * rows * cols, 1);
  const int64_t cnt = rows * cols;
  k_copy_panel<R><<<(unsigned)cdiv_up(cnt, (int64_t)256), 256, 0, st>>>(src, lds, rows, cols, dst, ldd, rna ? 1 : 0);
}

// A_kk <- inv(A_kk) in place, with a copy in X (ld bw): 64-wide blocks with
// partial pivoting on one CTA, 256-wide complex64 blocks on a CTA cluster,
// whose copy in X is rounded to TF32 (nearest) for the tensor-core products
// (the tensor cores would otherwise truncate it)
template <typename R>
static mnpbem_status block_inverse(cplx<R>* Akk, int64_t lda, int bw, cplx<R>* X, int* status, cudaStream_t st) {
  if (bw <= 64) {
    ProfScope ps(PH_BLOCKINV, st, 8.0 * bw * bw * bw, 0.0);
    k_block_inv<R><<<1, 256, 0, st>>>(Akk, lda, bw, X, bw, status);
    MNP_CHECK_LAUNCH();
    MNP_CUDA(cudaMemcpy2DAsync(Akk, sizeof(cplx<R>) * lda, X, sizeof(cplx<R>) * bw, sizeof(cplx<R>) * bw, bw,
                               cudaMemcpyDeviceToDevice, st));
    return MNPBEM_OK;
  }
  if (sizeof(R) == 4 && bw <= PB_W)
    return launch_block_inv_cluster(reinterpret_cast<const float2*>(Akk), lda, bw, reinterpret_cast<float2*>(Akk), lda,
                                    status, st, reinterpret_cast<float2*>(X));
  set_error("block LDU: diagonal blocks of %d rows are not supported in this precision", bw);
  return MNPBEM_ERR_UNSUPPORTED;
}

template <typename R>
mnpbem_status ldu_factor(cplx<R>* A, int64_t n, int64_t lda, LDUWork<R>& w, int* status, GemmFn<R> gemm,
                         void* ctx, cudaStream_t st) {
  using Cx = cplx<R>;
  const int b = w.b, B = w.b * std::max(1, w.m);
  if (n <= 0) return MNPBEM_OK;
  const size_t cs = sizeof(Cx);
  MNP_TRY(w.ccol.ensure(cs * n * B));
  MNP_TRY(w.xblk.ensure(cs * b * b));
  const bool tc = sizeof(R) == 4 && ctx != nullptr;
  MNP_TRY(w.rrow.ensure(cs * n * b));
  const bool rna = tc && w.round_a;
  Cx* Cc = w.ccol.template as<Cx>();     // [n][B]: row i holds row k0 + i of the outer step's column panel
  Cx* X = w.xblk.template as<Cx>();
  const Cx one = mk<R>(1, 0), zero = mk<R>(0, 0), mone = mk<R>(-1, 0);
  for (int64_t k0 = 0; k0 < n; k0 += B) {
    const int64_t Bw = std::min<int64_t>(B, n - k0), e = k0 + Bw;
    for (int64_t s = 0; s < Bw; s += b) {
      const int64_t ks = k0 + s;
      const int bs = (int)std::min<int64_t>(b, e - ks);
      const int64_t kb = ks + bs, below = n - kb;
      MNP_TRY(block_inverse<R>(A + ks * lda + ks, lda, bs, X, status, st));
      if (below > 0) {
        Cx* Cs = Cc + (kb - k0) * B + s;
        // unscaled column panel (the A operand of every update of this step)
        copy_panel<R>(A + kb * lda + ks, lda, below, bs, Cs, B, rna, st);
        MNP_CHECK_LAUNCH();
        // L panel: A[kb:, ks:kb] = C X
        MNP_TRY(gemm(below, bs, bs, one, Cs, B, X, bs, zero, A + kb * lda + ks, lda, st, ctx));
        // U row: A[ks:kb, kb:] = X A[ks:kb, kb:] (the tensor-core product copies its
        // B operand before it runs, so it may write in place; the CUDA-core
        // products may not)
        bool inplace = false;
        if constexpr (sizeof(R) == 4) {
          if (tc)
            inplace = tc_gemm_eligible(*reinterpret_cast<TcGemmCtx*>(ctx), bs, below, bs, X, bs, A + ks * lda + kb,
                                       lda, make_float2(0.f, 0.f));
        }
        if (inplace) {
          MNP_TRY(gemm(bs, below, bs, one, X, bs, A + ks * lda + kb, lda, zero, A + ks * lda + kb, lda, st, ctx));
        } else {
          Cx* Rr = w.rrow.template as<Cx>();
          MNP_CUDA(cudaMemcpy2DAsync(Rr, cs * below, A + ks * lda + kb, cs * lda, cs * below, bs,
                                     cudaMemcpyDeviceToDevice, st));
          MNP_TRY(gemm(bs, below, bs, one, X, bs, Rr, below, zero, A + ks * lda + kb, lda, st, ctx));
        }
        if (kb < e) {
          // the later column panels of this outer step (all rows below) ...
          MNP_TRY(gemm(below, e - kb, bs, mone, Cs, B, A + ks * lda + kb, lda, one, A + kb * lda + kb, lda, st, ctx));
          // ... and the later rows of this outer step over the trailing columns
          if (e < n)
            MNP_TRY(gemm(e - kb, n - e, bs, mone, Cs, B, A + ks * lda + e, lda, one, A + kb * lda + e, lda, st, ctx));
        }
      }
    }
    // trailing update of rank Bw
    if (e < n) MNP_TRY(gemm(n - e, n - e, Bw, mone, Cc + (e - k0) * B, B, A + k0 * lda + e, lda, one, A + e * lda + e,
                            lda, st, ctx));
  }
  return MNPBEM_OK;
}

template <typename R>
mnpbem_status ldu_rsolve(cplx<R>* H, int64_t n, int64_t ldh, const cplx<R>* F, int64_t ldf, LDUWork<R>& w,
                         GemmFn<R> gemm, void* ctx, cudaStream_t st) {
  using Cx = cplx<R>;
  const int b = w.b, B = w.b * std::max(1, w.m);
  if (n <= 0) return MNPBEM_OK;
  MNP_TRY(w.ccol.ensure(sizeof(Cx) * n * B));
  const bool rna = sizeof(R) == 4 && ctx != nullptr && w.round_a;
  Cx* Cc = w.ccol.template as<Cx>();     // [n][B]: columns of the outer step
  const Cx one = mk<R>(1, 0), zero = mk<R>(0, 0), mone = mk<R>(-1, 0);
  // 1. W U = H (U unit upper), columns in increasing order; then V = W D^-1
  //    (D^-1 = the stored X_k) on each outer step's columns once they are final
  for (int64_t k0 = 0; k0 < n; k0 += B) {
    const int64_t Bw = std::min<int64_t>(B, n - k0), e = k0 + Bw;
    for (int64_t s = 0; s < Bw; s += b) {
      const int64_t ks = k0 + s;
      const int bs = (int)std::min<int64_t>(b, e - ks);
      copy_panel<R>(H + ks, ldh, n, bs, Cc + s, B, rna, st);
      MNP_CHECK_LAUNCH();
      if (ks + bs < e)
        MNP_TRY(gemm(n, e - ks - bs, bs, mone, Cc + s, B, F + ks * ldf + ks + bs, ldf, one, H + ks + bs, ldh, st, ctx));
    }
    if (e < n) MNP_TRY(gemm(n, n - e, Bw, mone, Cc, B, F + k0 * ldf + e, ldf, one, H + e, ldh, st, ctx));
    for (int64_t s = 0; s < Bw; s += b) {
      const int64_t ks = k0 + s;
      const int bs = (int)std::min<int64_t>(b, e - ks);
      MNP_TRY(gemm(n, bs, bs, one, Cc + s, B, F + ks * ldf + ks, ldf, zero, H + ks, ldh, st, ctx));
    }
  }
  // 2. S L = V (L unit lower), columns in decreasing order
  const int64_t nout = cdiv_up(n, (int64_t)B);
  for (int64_t q = nout - 1; q >= 0; --q) {
    const int64_t k0 = q * B, Bw = std::min<int64_t>(B, n - k0), e = k0 + Bw;
    const int64_t nin = cdiv_up(Bw, (int64_t)b);
    for (int64_t t = nin - 1; t >= 0; --t) {
      const int64_t ks = k0 + t * b;
      const int bs = (int)std::min<int64_t>(b, e - ks);
      copy_panel<R>(H + ks, ldh, n, bs, Cc + t * b, B, rna, st);
      MNP_CHECK_LAUNCH();
      if (ks > k0) MNP_TRY(gemm(n, ks - k0, bs, mone, Cc + t * b, B, F + ks * ldf + k0, ldf, one, H + k0, ldh, st, ctx));
    }
    if (k0 > 0) MNP_TRY(gemm(n, k0, Bw, mone, Cc, B, F + k0 * ldf, ldf, one, H, ldh, st, ctx));
  }
  return MNPBEM_OK;
}

// X[blk] <- X_k X[blk] for every diagonal block k (one CTA per block; a warp
// per row, lanes over the block's columns, N <= 16 right-hand sides)
template <typename R, int NB>
__global__ void __launch_bounds__(256) k_ldu_diag(const cplx<R>* __restrict__ F, int64_t ldf, int64_t n, int b,
                                                  cplx<R>* __restrict__ X, int64_t ldx, int N) {
  using Cx = cplx<R>;
  extern __shared__ unsigned char ldu_smem[];
  Cx* xs = reinterpret_cast<Cx*>(ldu_smem);   // [b][NB], columns N .. NB - 1 zero
  const int64_t k0 = (int64_t)blockIdx.x * b;
  const int bs = (int)min((int64_t)b, n - k0);
  for (int e = threadIdx.x; e < bs * NB; e += blockDim.x) {
    const int r = e / NB, c = e % NB;
    xs[e] = c < N ? X[(k0 + r) * ldx + c] : mk<R>(0, 0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int r = warp; r < bs; r += 8) {
    const Cx* frow = F + (k0 + r) * ldf + k0;
    Cx acc[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) acc[c] = mk<R>(0, 0);
    for (int l = lane; l < bs; l += 32) {
      const Cx f = frow[l];
#pragma unroll
      for (int c = 0; c < NB; ++c) cfma(acc[c], f, xs[l * NB + c]);
    }
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      Cx v = acc[c];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0 && c < N) X[(k0 + r) * ldx + c] = v;
    }
  }
}

// ------------------------------------------- triangular sweeps, one launch
// The forward (unit lower L) and backward (unit upper U) sweeps of the LDU
// solve for a few right-hand sides as one cooperative launch each.  Step s
// takes block k (k = s forward, nblk - 1 - s backward): every CTA stages x_k
// (b x N) in shared memory and subtracts F[i, k block] x_k from its rows i of
// the trailing (forward) or leading (backward) part; then the CTAs meet at a
// grid barrier before the next block is read.  One CTA of 16 warps per SM;
// rows go to the CTAs in groups (16 warps x 2 rows, by absolute index: group g
// to CTA g mod G); a warp takes two rows at a time (lanes along the rows,
// coalesced, both rows' loads in flight together) and reduces with shuffles.
// X is read with ld.global.cg (L2), since other CTAs updated it.  The grid
// barrier is a monotonic arrival counter (zeroed before the launch) with a
// bounded wait; on expiry the error word of the streamed thin products is
// set, an abort flag releases the other CTAs and every CTA returns.
constexpr int TRSV_THREADS = 512, TRSV_WARPS = TRSV_THREADS / 32;

__device__ __forceinline__ bool coop_barrier(unsigned* ctr, unsigned target, int* abortf) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    atomicAdd(ctr, 1u);
    const unsigned long long t0 = gtimer();
    while (*(volatile unsigned*)ctr < target) {
      if (*(volatile int*)abortf) { ok = 0; break; }
      if (gtimer() - t0 > MBAR_WAIT_NS) {
        atomicOr(&g_thin_stream_err, 64);
        atomicExch(abortf, 1);
        ok = 0;
        break;
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// one warp subtracts F[i, k block] x_k from RW rows i0, i0 + 1, ... at once
// (independent accumulators keep the RW rows' loads in flight together)
template <typename R, int NB, int RW>
__device__ __forceinline__ void trsv_rows(const cplx<R>* __restrict__ F, int64_t ldf, int64_t k0, int bs,
                                          const cplx<R>* xs, cplx<R>* X, int64_t ldx, int N, int64_t i0,
                                          int64_t r0, int64_t r1, int lane) {
  using Cx = cplx<R>;
  Cx acc[RW][NB];
#pragma unroll
  for (int q = 0; q < RW; ++q)
#pragma unroll
    for (int c = 0; c < NB; ++c) acc[q][c] = mk<R>(0, 0);
  const Cx* frow[RW];
  bool act[RW];
#pragma unroll
  for (int q = 0; q < RW; ++q) {
    act[q] = i0 + q >= r0 && i0 + q < r1;
    frow[q] = F + (act[q] ? i0 + q : r0) * ldf + k0;
  }
  // two of a lane's entries per row in flight at a time: the full unroll (a
  // row's entries all loaded first) raises the register count to 96-104 and
  // keeps these CTAs from sharing SMs with the other lanes' kernels
#pragma unroll 2
  for (int l = lane; l < bs; l += 32) {
    Cx f[RW];
#pragma unroll
    for (int q = 0; q < RW; ++q) f[q] = __ldg(frow[q] + l);
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      const Cx xv = xs[l * NB + c];
#pragma unroll
      for (int q = 0; q < RW; ++q) cfma(acc[q][c], f[q], xv);
    }
  }
#pragma unroll
  for (int q = 0; q < RW; ++q)
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      Cx v = acc[q][c];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (act[q] && lane == c && c < N) {
        Cx* xp = X + (i0 + q) * ldx + c;
        *xp = csub(__ldcg(xp), v);
      }
    }
}

template <typename R, int NB, bool LOWER>
__global__ void __launch_bounds__(TRSV_THREADS) k_trsv_unit(const cplx<R>* __restrict__ F, int64_t ldf, int64_t n,
                                                            int b, cplx<R>* X, int64_t ldx, int N, unsigned* bar) {
  using Cx = cplx<R>;
  constexpr int RW = NB <= 8 ? 2 : 1;          // rows per warp at a time
  constexpr int GRP = TRSV_WARPS * RW;         // rows per group: one pass of the CTA's warps
  extern __shared__ unsigned char trsv_smem[];
  Cx* xs = reinterpret_cast<Cx*>(trsv_smem);   // [b][NB], columns N .. NB - 1 zero
  const int nblk = (int)((n + b - 1) / b);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t G = gridDim.x;
  int* abortf = reinterpret_cast<int*>(bar + 1);
  for (int s = 0; s + 1 < nblk; ++s) {
    const int k = LOWER ? s : nblk - 1 - s;
    const int64_t k0 = (int64_t)k * b;
    const int bs = (int)min((int64_t)b, n - k0);
    for (int e = threadIdx.x; e < bs * NB; e += TRSV_THREADS) {
      const int r = e / NB, c = e % NB;
      xs[e] = c < N ? __ldcg(X + (k0 + r) * ldx + c) : mk<R>(0, 0);
    }
    __syncthreads();
    const int64_t r0 = LOWER ? k0 + bs : 0, r1 = LOWER ? n : k0;
    // groups of GRP rows by absolute index, group g to CTA g mod G
    int64_t g = r0 / GRP;
    g += (blockIdx.x - g % G + G) % G;
    for (; g * GRP < r1; g += G)
      trsv_rows<R, NB, RW>(F, ldf, k0, bs, xs, X, ldx, N, g * GRP + warp * RW, r0, r1, lane);
    if (!coop_barrier(bar, (unsigned)((s + 1) * G), abortf)) return;
  }
}

static int trsv_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
      cudaGetLastError();
      sms = 148;
    }
  }
  return sms;
}

template <typename R, int NB, bool LOWER>
static mnpbem_status launch_trsv(const cplx<R>* F, int64_t n, int64_t ldf, int b, cplx<R>* X, int64_t ldx, int N,
                                 unsigned* bar, cudaStream_t st) {
  using Cx = cplx<R>;
  const size_t smem = sizeof(Cx) * b * NB;
  static int per_sm = -1;
  if (per_sm < 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_unit<R, NB, LOWER>, TRSV_THREADS,
                                                      sizeof(Cx) * 256 * NB) != cudaSuccess) {
      cudaGetLastError();
      per_sm = 1;
    }
    per_sm = std::max(1, std::min(per_sm, 1));
  }
  const unsigned grid = (unsigned)(per_sm * trsv_sms());
  MNP_CUDA(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));
  ProfScope ps(PH_GEMM_SMALL, st, 4.0 * n * n * N, (double)sizeof(Cx) * 0.5 * n * n);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(TRSV_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MNP_CUDA(cudaLaunchKernelEx(&cfg, k_trsv_unit<R, NB, LOWER>, F, ldf, n, b, X, ldx, N, bar));
  return MNPBEM_OK;
}

template <typename R, bool LOWER>
static mnpbem_status trsv_sweep(const cplx<R>* F, int64_t n, int64_t ldf, int b, cplx<R>* X, int64_t ldx, int N,
                                unsigned* bar, cudaStream_t st) {
  if (N <= 4) return launch_trsv<R, 4, LOWER>(F, n, ldf, b, X, ldx, N, bar, st);
  if (N <= 8) return launch_trsv<R, 8, LOWER>(F, n, ldf, b, X, ldx, N, bar, st);
  return launch_trsv<R, 16, LOWER>(F, n, ldf, b, X, ldx, N, bar, st);
}

template <typename R>
mnpbem_status ldu_solve(const cplx<R>* F, int64_t n, int64_t ldf, int b, cplx<R>* X, int64_t ldx, int64_t N,
                        cplx<R>* tmp, GemmFn<R> gemm, void* ctx, cudaStream_t st, unsigned* bar) {
  using Cx = cplx<R>;
  if (n <= 0 || N <= 0) return MNPBEM_OK;
  const Cx one = mk<R>(1, 0), zero = mk<R>(0, 0), mone = mk<R>(-1, 0);
  const int64_t nblk = cdiv_up(n, (int64_t)b);
  const bool sweep = bar && N <= 16 && b <= 256;
  // forward: L unit lower
  if (sweep) {
    if (nblk > 1) MNP_TRY((trsv_sweep<R, true>(F, n, ldf, b, X, ldx, (int)N, bar, st)));
  } else {
    for (int64_t k = 0; k + 1 < nblk; ++k) {
      const int64_t k0 = k * b, kb = k0 + b;
      MNP_TRY(gemm(n - kb, N, b, mone, F + kb * ldf + k0, ldf, X + k0 * ldx, ldx, one, X + kb * ldx, ldx, st, ctx));
    }
  }
  // block diagonal
  if (N <= 16) {
    const size_t smem = sizeof(Cx) * b * (N <= 4 ? 4 : N <= 8 ? 8 : 16);
    ProfScope ps(PH_GEMM_SMALL, st, 8.0 * n * b * N, (double)sizeof(Cx) * ((double)n * b + 2.0 * n * N));
    const int Ni = (int)N;
    if (N <= 4) k_ldu_diag<R, 4><<<(unsigned)nblk, 256, smem, st>>>(F, ldf, n, b, X, ldx, Ni);
    else if (N <= 8) k_ldu_diag<R, 8><<<(unsigned)nblk, 256, smem, st>>>(F, ldf, n, b, X, ldx, Ni);
    else k_ldu_diag<R, 16><<<(unsigned)nblk, 256, smem, st>>>(F, ldf, n, b, X, ldx, Ni);
    MNP_CHECK_LAUNCH();
  } else {
    if (!tmp) { set_error("ldu_solve: workspace required for more than 16 right-hand sides"); return MNPBEM_ERR_INVALID_ARG; }
    for (int64_t k = 0; k < nblk; ++k) {
      const int64_t k0 = k * b;
      const int bs = (int)std::min<int64_t>(b, n - k0);
      MNP_CUDA(cudaMemcpy2DAsync(tmp, sizeof(Cx) * N, X + k0 * ldx, sizeof(Cx) * ldx, sizeof(Cx) * N, bs,
                                 cudaMemcpyDeviceToDevice, st));
      MNP_TRY(gemm(bs, N, bs, one, F + k0 * ldf + k0, ldf, tmp, N, zero, X + k0 * ldx, ldx, st, ctx));
    }
  }
  // backward: U unit upper
  if (sweep) {
    if (nblk > 1) MNP_TRY((trsv_sweep<R, false>(F, n, ldf, b, X, ldx, (int)N, bar, st)));
    return MNPBEM_OK;
  }
  for (int64_t k = nblk - 1; k >= 1; --k) {
    const int64_t k0 = k * b;
    const int bs = (int)std::min<int64_t>(b, n - k0);
    MNP_TRY(gemm(k0, N, bs, mone, F + k0, ldf, X + k0 * ldx, ldx, one, X, ldx, st, ctx));
  }
  return MNPBEM_OK;
}

template mnpbem_status ldu_factor<float>(float2*, int64_t, int64_t, LDUWork<float>&, int*, GemmFn<float>, void*,
                                         cudaStream_t);
template mnpbem_status ldu_factor<double>(double2*, int64_t, int64_t, LDUWork<double>&, int*, GemmFn<double>, void*,
                                          cudaStream_t);
template mnpbem_status ldu_rsolve<float>(float2*, int64_t, int64_t, const float2*, int64_t, LDUWork<float>&,
                                         GemmFn<float>, void*, cudaStream_t);
template mnpbem_status ldu_rsolve<double>(double2*, int64_t, int64_t, const double2*, int64_t, LDUWork<double>&,
                                          GemmFn<double>, void*, cudaStream_t);
template mnpbem_status ldu_solve<float>(const float2*, int64_t, int64_t, int, float2*, int64_t, int64_t, float2*,
                                        GemmFn<float>, void*, cudaStream_t, unsigned*);
template mnpbem_status ldu_solve<double>(const double2*, int64_t, int64_t, int, double2*, int64_t, int64_t, double2*,
                                         GemmFn<double>, void*, cudaStream_t, unsigned*);

}  // namespace mnpbem
