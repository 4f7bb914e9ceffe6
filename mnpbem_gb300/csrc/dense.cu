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
#include "dense.cuh"
#include "profile.cuh"

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

template <typename R>
mnpbem_status gemm_simt(int64_t M, int64_t N, int64_t K, cplx<R> alpha, const cplx<R>* A,
                        int64_t lda, const cplx<R>* B, int64_t ldb, cplx<R> beta, cplx<R>* C,
                        int64_t ldc, cudaStream_t st) {
  if (M <= 0 || N <= 0) return MNPBEM_OK;
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

// --------------------------------------------------- block inversion (smem)
// In-place Gauss-Jordan of one w x w block (w <= 64) held in shared memory.
template <typename R>
__global__ void __launch_bounds__(256) k_block_inv(const cplx<R>* __restrict__ A, int64_t lda, int w,
                                                   cplx<R>* __restrict__ X, int64_t ldx, int* status) {
  using Cx = cplx<R>;
  extern __shared__ unsigned char smem_raw[];
  Cx* S = reinterpret_cast<Cx*>(smem_raw);      // [w][w+1]
  Cx* prow = S + w * (w + 1);
  Cx* pcol = prow + w;
  const int ws = w + 1;
  const int t = threadIdx.x;
  for (int l = t; l < w * w; l += blockDim.x) {
    int r = l / w, c = l % w;
    S[r * ws + c] = A[r * lda + c];
  }
  __syncthreads();
  for (int p = 0; p < w; ++p) {
    if (t < w) { prow[t] = S[p * ws + t]; pcol[t] = S[t * ws + p]; }
    __syncthreads();
    Cx piv = prow[p];
    double a2 = cabs2(piv);
    if (t == 0 && !(a2 > 1e-280 && a2 < 1e280)) atomicOr(status, 1);
    Cx inv = cdiv(mk<R>(1, 0), piv);
    for (int l = t; l < w * w; l += blockDim.x) {
      int r = l / w, c = l % w;
      Cx v;
      if (r == p && c == p) v = inv;
      else if (r == p) v = cmul(prow[c], inv);
      else if (c == p) { v = cmul(pcol[r], inv); v.x = -v.x; v.y = -v.y; }
      else v = csub(S[r * ws + c], cmul(pcol[r], cmul(prow[c], inv)));
      S[r * ws + c] = v;
    }
    __syncthreads();
  }
  for (int l = t; l < w * w; l += blockDim.x) {
    int r = l / w, c = l % w;
    X[r * ldx + c] = S[r * ws + c];
  }
}

// --------------------------------------------------- blocked Gauss-Jordan
template <typename R>
mnpbem_status gj_invert(cplx<R>* A, int64_t n, int64_t lda, GJWork<R>& w, GemmFn<R> big_gemm,
                        void* ctx, cudaStream_t st) {
  using Cx = cplx<R>;
  const int nb = w.nb;
  const size_t cs = sizeof(Cx);
  MNP_TRY(w.ccol.ensure(cs * n * nb));
  MNP_TRY(w.rrow.ensure(cs * n * nb));
  MNP_TRY(w.ncol.ensure(cs * n * nb));
  MNP_TRY(w.xblk.ensure(cs * nb * nb));
  MNP_TRY(w.status.ensure(sizeof(int)));
  MNP_CUDA(cudaMemsetAsync(w.status.ptr, 0, sizeof(int), st));
  Cx* Ccol = w.ccol.template as<Cx>();   // [n][nb]
  Cx* Rrow = w.rrow.template as<Cx>();   // [nb][n]
  Cx* Ncol = w.ncol.template as<Cx>();   // [n][nb]
  Cx* X = w.xblk.template as<Cx>();      // [nb][nb]
  const size_t smem = cs * ((size_t)nb * (nb + 1) + 2 * nb);
  static bool attr_set[2] = {false, false};
  if (!attr_set[sizeof(R) == 8]) {
    MNP_CUDA(cudaFuncSetAttribute(k_block_inv<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(cs * (64 * 65 + 128))));
    attr_set[sizeof(R) == 8] = true;
  }
  const Cx one = mk<R>(1, 0), zero = mk<R>(0, 0), mone = mk<R>(-1, 0);
  for (int64_t k0 = 0; k0 < n; k0 += nb) {
    const int bw = (int)std::min<int64_t>(nb, n - k0);
    // 1. Ccol <- A[:, k-block]
    MNP_CUDA(cudaMemcpy2DAsync(Ccol, cs * bw, A + k0, cs * lda, cs * bw, n, cudaMemcpyDeviceToDevice, st));
    // 2. X <- inv(A_kk)
    ProfScope ps(PH_BLOCKINV, st, 8.0 * bw * bw * bw, 0.0);
    k_block_inv<R><<<1, 256, smem, st>>>(Ccol + k0 * bw, bw, bw, X, bw, w.status.template as<int>());
    MNP_CHECK_LAUNCH();
    // 3. R <- X * A[k-block, :], then zero its k-block columns
    MNP_TRY(gemm_simt<R>(bw, n, bw, one, X, bw, A + k0 * lda, lda, zero, Rrow, n, st));
    MNP_CUDA(cudaMemset2DAsync(Rrow + k0, cs * n, 0, cs * bw, bw, st));
    // 4. new column block <- -Ccol * X, then zero Ccol's k-block rows
    MNP_TRY(gemm_simt<R>(n, bw, bw, mone, Ccol, bw, X, bw, zero, Ncol, bw, st));
    MNP_CUDA(cudaMemsetAsync(Ccol + k0 * bw, 0, cs * bw * bw, st));
    // 5. A <- A - Ccol * R  (rank-bw update of the whole matrix)
    MNP_TRY(big_gemm(n, n, bw, mone, Ccol, bw, Rrow, n, one, A, lda, st, ctx));
    // 6. write back row block, column block and the inverted pivot block
    MNP_CUDA(cudaMemcpy2DAsync(A + k0 * lda, cs * lda, Rrow, cs * n, cs * n, bw, cudaMemcpyDeviceToDevice, st));
    MNP_CUDA(cudaMemcpy2DAsync(A + k0, cs * lda, Ncol, cs * bw, cs * bw, n, cudaMemcpyDeviceToDevice, st));
    MNP_CUDA(cudaMemcpy2DAsync(A + k0 * lda + k0, cs * lda, X, cs * bw, cs * bw, bw, cudaMemcpyDeviceToDevice, st));
  }
  int hs = 0;
  MNP_CUDA(cudaMemcpyAsync(&hs, w.status.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  if (hs) {
    set_error("block Gauss-Jordan inversion: zero or non-finite pivot");
    return MNPBEM_ERR_SINGULAR;
  }
  return MNPBEM_OK;
}

template mnpbem_status gj_invert<float>(float2*, int64_t, int64_t, GJWork<float>&, GemmFn<float>,
                                        void*, cudaStream_t);
template mnpbem_status gj_invert<double>(double2*, int64_t, int64_t, GJWork<double>&,
                                         GemmFn<double>, void*, cudaStream_t);

}  // namespace mnpbem
