// H-matrices of the retarded Green functions (cluster tree blocks, adaptive
// cross approximation of the far blocks) and the vector kernels of the
// preconditioned GMRES of the iterative solver.
#pragma once
#include "common.cuh"
#include "assemble.cuh"

namespace mnpbem {

constexpr int ACA_KMAX = 512;     // largest rank of a low-rank block
constexpr int HMV_NMAX = 16;      // columns of an H-matrix product (4 npol)

// Device view of the H-matrices of G1, H1, G2, H2 (q = 0..3) on one cluster
// tree.  Blocks are (first row, rows, first column, columns) in cluster order.
struct HmatDev {
  int n = 0, nfull = 0, nlow = 0, nleaf = 0;
  double tol = 1e-6;                 // ACA tolerance (htol)
  const int* perm = nullptr;         // [n] face at each cluster position
  const int4* fblk = nullptr;        // [nfull] full blocks
  const int64_t* foff = nullptr;     // [nfull] value offsets (row-major blocks)
  const int4* lblk = nullptr;        // [nlow] low-rank blocks
  const int* kcap = nullptr;         // [nlow] rank capacity min(kmax, rows, cols)
  const int64_t* aoff = nullptr;     // [nlow] offsets of the left factors [kcap][rows]
  const int64_t* boff = nullptr;     // [nlow] offsets of the right factors [kcap][cols]
  const int64_t* uoff = nullptr;     // [nlow] offsets of the ACA row flags
  const int64_t* toff = nullptr;     // [nlow] offsets of the products R^T x [kcap][HMV_NMAX]
  int64_t usz = 0, tsz = 0;          // per-matrix sizes of the row flags and products
  int64_t nvals = 0;                 // entries of the full blocks (per matrix)
  int* rank = nullptr;               // [4][nlow] ranks found by ACA
  // values and factors: complex128 while assembled / compressed, then split
  // in place into (hi, lo) float pairs, float4 (hi.re, hi.im, lo.re, lo.im),
  // for the double-single products
  double2* val[4] = {};              // full block values
  double2* A[4] = {};                // left factors, column k of block b at A + aoff + k rows (FP64)
  double2* B[4] = {};                // right factors (split in place)
  float4* At[4] = {};                // left factors split, row-major [rows][kcap] at At + aoff
  unsigned char* used = nullptr;     // [4][usz] ACA row flags
  const int2* leaf = nullptr;        // [nleaf] (first row, rows) of the leaf clusters
  const int* lptr = nullptr;         // [nleaf + 1] CSR of the blocks that cover each leaf's rows
  const int* lent = nullptr;         // b >= 0: full block b; ~b: low-rank block b
  float4* T = nullptr;               // [4][tsz] products R^T x of the low-rank blocks (hi / lo)
  float4* xs = nullptr;              // [2][n * HMV_NMAX] hi / lo split of the product's x1, x2
};

// low-rank blocks of the four matrices by ACA (mex/hlib/aca.cpp restated,
// kernel of mex/acagreen/acagreen.cpp greenret::getrow / getcol)
mnpbem_status hmat_aca(const AsmParams& p, const HmatDev& h, cudaStream_t st);
// values and right factors -> (hi, lo) float4 in place, left factors -> At
// (row-major, split) (after hmat_aca)
mnpbem_status hmat_split(const HmatDev& h, cudaStream_t st);
// y[q] = H_q x (x = x1 for q = 0, 1; x2 for q = 2, 3); x, y [n][N] in face order, N <= 16;
// double-single arithmetic on the split values (FP32 pipe, ~1e-14 relative)
// bytes: algorithmic bytes of the product (for the profiler)
mnpbem_status hmat_mv(const HmatDev& h, int N, const double2* x1, const double2* x2, double2* const* y,
                      double bytes, cudaStream_t st);
// H_q expanded to out [n][n] (face order, row-major; @hmatrix/full.m)
mnpbem_status hmat_full(const HmatDev& h, int q, double2* out, cudaStream_t st);

// ---- vectors of the Krylov solver (complex128, length len)
constexpr int KV_BLOCKS = 256;
// partial[i * KV_BLOCKS + blk] = partial sums of conj(V_i) . w  (V_i = V + i * len)
void kv_dots(const double2* V, int nv, int64_t len, const double2* w, double2* partial, cudaStream_t st);
// w -= sum_i h[i] V_i  (h on the device)
void kv_update(const double2* V, int nv, int64_t len, const double2* h, double2* w, cudaStream_t st);
// partial[blk] = partial sums of |w|^2
void kv_norm2(const double2* w, int64_t len, double* partial, cudaStream_t st);
// out = s w (s real; out may be w)
void kv_scale(const double2* w, int64_t len, double s, double2* out, cudaStream_t st);
// out = sum_i c[i] v[i] over up to 4 terms (out may be one of the v[i])
struct KvTerms {
  int n = 0;
  double2 c[4];
  const double2* v[4];
};
void kv_lincomb(const KvTerms& t, int64_t len, double2* out, cudaStream_t st);
// b-space (phi [n][P], a [n][3][P], alpha [n][3][P], De [n][P]) -> x-space
// ([n][4P] of (phi | a), then [n][4P] of (De | alpha)): the identification of
// bemretiter's pack.m / unpack.m
void kv_pack_bx(int64_t n, int P, const double2* phi, const double2* a, const double2* alpha,
                const double2* De, double2* x, cudaStream_t st);

}  // namespace mnpbem
