// Dense complex linear algebra on the device (row-major, interleaved complex).
#pragma once
#include <memory>
#include "common.cuh"

namespace mnpbem {

// C = alpha * A[M x K] * B[K x N] + beta * C      (SIMT CUDA-core kernel)
template <typename R>
mnpbem_status gemm_simt(int64_t M, int64_t N, int64_t K, cplx<R> alpha, const cplx<R>* A,
                        int64_t lda, const cplx<R>* B, int64_t ldb, cplx<R> beta, cplx<R>* C,
                        int64_t ldc, cudaStream_t st);

// C[M x N] = (A_hi + A_lo)[M x K] * B[K x N] (columns in blocks of 8) with the product
// evaluated in double-single FP32 arithmetic (error-free products and
// TwoSum accumulation, ~48-bit accuracy): A_hi = fl32(A), A_lo = fl32(A - A_hi)
// are complex64 planes, B (row stride ldb) and C are complex128.
// bsplit: workspace of 2 K min(N, 8) complex64 (hi / lo planes of a block of B).
// Alo == NULL: FP32 product of the hi planes (FMA accumulation, ~24 bits).
mnpbem_status gemm_thin_ds(int64_t M, int64_t N, int64_t K, const float2* Ahi, const float2* Alo,
                           int64_t lda, const double2* B, int64_t ldb, double2* C, int64_t ldc,
                           float2* bsplit, cudaStream_t st);

// MNPBEM_ERR_TIMEOUT (and the word cleared) if a bounded wait of the streamed
// thin GEMM expired since the last check; synchronises st
mnpbem_status thin_stream_check(cudaStream_t st);

// x <- TF32(x) rounded to nearest, in place (count floats)
void round_tf32(float* x, int64_t count, cudaStream_t st);

// Workspace for in-place inversion of an n x n matrix by blocked Gauss-Jordan
// elimination without row interchanges.
template <typename R>
struct GJWork {
  DevBuf ccol, rrow, ncol, xblk, status;
  int nb = 64;
  bool round_a = true;               // round the A operand of the tensor-core updates to TF32 (nearest)
  bool fused = true;                 // tensor-core path: products written in place (no panel copies)
  bool nested = false;               // inner level: the outer level reads the pivot status
  std::unique_ptr<GJWork<R>> inner;  // Gauss-Jordan of pivot blocks wider than 64
};

// A <- inv(A) in place.  Returns MNPBEM_ERR_SINGULAR if a pivot guard trips.
// gemm_fn performs the rank-nb trailing updates (SIMT or tensor-core).
template <typename R>
using GemmFn = mnpbem_status (*)(int64_t M, int64_t N, int64_t K, cplx<R> alpha, const cplx<R>* A,
                                 int64_t lda, const cplx<R>* B, int64_t ldb, cplx<R> beta,
                                 cplx<R>* C, int64_t ldc, cudaStream_t st, void* ctx);
// read_status = false: nothing synchronises (usable inside a graph capture);
// the caller reads the pivot status later with gj_status_copy.
template <typename R>
mnpbem_status gj_invert(cplx<R>* A, int64_t n, int64_t lda, GJWork<R>& w, GemmFn<R> big_gemm,
                        void* ctx, cudaStream_t st, bool read_status = true);
// enqueue copies of the pivot status words (outer, inner) into host memory
template <typename R>
mnpbem_status gj_status_copy(GJWork<R>& w, int* host2, cudaStream_t st);

// ------------------------------------------------------ block LDU factors
// A = L D U in place: L unit block-lower (stored below the diagonal blocks),
// D block-diagonal with the inverses X_k of its blocks stored in the diagonal
// blocks, U unit block-upper (stored above them: U_kj = X_k A_kj after the
// updates of the steps before k).  Blocks of w.b rows; the trailing updates
// of w.m consecutive steps are gathered into one product of rank w.b * w.m.
// Each diagonal block is inverted with partial pivoting inside the block
// (CUDA-core path, 64-wide blocks) or by the 256-wide cluster kernel.
// Status words (device, cleared by ldu_status_clear): [0] != 0 when a block
// inverse met a zero or non-finite pivot; [1] the largest per-block condition
// proxy max|A_kk| * max|X_k| as the bits of a non-negative float.
template <typename R>
struct LDUWork {
  DevBuf ccol, rrow, xblk, tmp;
  int b = 64;
  int m = 1;
  bool round_a = true;   // tensor-core path: A operands rounded to nearest TF32
};
// status: int[2] in device memory (see above)
template <typename R>
mnpbem_status ldu_factor(cplx<R>* A, int64_t n, int64_t lda, LDUWork<R>& w, int* status, GemmFn<R> gemm,
                         void* ctx, cudaStream_t st);
// H [n x n] <- H F^-1 with F the block LDU factors of an n x n matrix (same b)
template <typename R>
mnpbem_status ldu_rsolve(cplx<R>* H, int64_t n, int64_t ldh, const cplx<R>* F, int64_t ldf, LDUWork<R>& w,
                         GemmFn<R> gemm, void* ctx, cudaStream_t st);
// X [n x N] <- F^-1 X in place (F block LDU factors with blocks of b rows).
// The transposed solve F^-T X is the same call on the in-place transpose of F.
// tmp: workspace of b * N values, used only for N > 16 (may be null otherwise).
// bar: two device words for the grid barrier of the one-launch triangular
// sweeps (N <= 16; one pair per stream); null: one product per block instead.
template <typename R>
mnpbem_status ldu_solve(const cplx<R>* F, int64_t n, int64_t ldf, int b, cplx<R>* X, int64_t ldx, int64_t N,
                        cplx<R>* tmp, GemmFn<R> gemm, void* ctx, cudaStream_t st, unsigned* bar = nullptr);

}  // namespace mnpbem
