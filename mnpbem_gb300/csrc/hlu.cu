// H-matrix arithmetic on the GPU (LU, triangular solves, inversion, addition
// with ACA truncation) and the 'hmat' preconditioner of the iterative solver.
//
// The recursion follows mex/hlib/lu.h:30-223 (lu, lsolve, rsolve, solve),
// hmatrix.h:150-345 (add, subtract, add_mul, add_mul2, inv) and
// submatrix.h:50-263 (conversion, truncation, masks, products, cat) step for
// step, so that every low-rank block is truncated at the same points as the
// reference and with the same ACA (aca.cpp:150-218: partial pivoting by
// |re| + |im|, first maximum, rank cap min(max_rank, kmax)).  The host walks
// the cluster tree; each numeric step is a kernel on the device's H stream:
//   k_zgemm       C = alpha op(A) op(B) + beta C (column-major, 32 x 32 tiles)
//   k_lu_leaf     LU of a full leaf without row interchanges (lu.cpp:82-106:
//                 L lower with its diagonal, U unit upper), one CTA
//   k_trsm        op(T) X = B for T the L or the U of a leaf, one CTA per 32
//                 right-hand sides
//   k_inv_leaf    inverse of a full leaf, Gauss-Jordan with partial pivoting
//                 (the reference calls LAPACK getrf / getri), one CTA
//   k_aca         ACA of a full block or of a low-rank product, one CTA
// The rank an ACA finds is read back (the host needs it for the next shapes).
// Matrices are immutable once built and shared between blocks; they come from
// a stream-ordered pool and are freed on the H stream when the last block
// holding them goes away.  Arithmetic is FP64: the oracle restates the same
// recursion in NumPy and the two agree to rounding.
#include "hlu.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace mnpbem {
namespace hl {

constexpr double ACA_STOP = 1e-10;   // aca.h ACATOL

// ------------------------------------------------------------------ kernels
namespace {

__device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }

// C tile (TILE x TILE) of alpha op(A) op(B) (+ beta C) over K range
// [k0, k1), 256 threads (16 x 16, each TILE / 16 x TILE / 16 outputs).  With
// W != NULL the raw sums go to W + z M N (column-major M x N, z = blockIdx.z)
// for the ordered reduction of k_zgemm_reduce instead of C.
template <int TILE>
__global__ void __launch_bounds__(256) k_zgemm(int M, int N, int K, int kc, double2 alpha,
                                               const double2* __restrict__ A, int lda, int ta,
                                               const double2* __restrict__ B, int ldb, int tb, double2 beta,
                                               double2* __restrict__ C, int ldc, double2* __restrict__ W) {
  constexpr int R = TILE / 16;
  __shared__ double2 As[16][TILE + 1];   // [l][i]
  __shared__ double2 Bs[16][TILE + 1];   // [l][j]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.x * TILE, j0 = blockIdx.y * TILE;
  const int k0 = blockIdx.z * kc, k1 = min(K, k0 + kc);
  double2 acc[R][R];
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) acc[a][b] = make_double2(0.0, 0.0);
  for (int l0 = k0; l0 < k1; l0 += 16) {
    for (int e = threadIdx.x; e < 16 * TILE; e += 256) {
      // A tile: TILE rows (i) x 16 (l); B tile: 16 (l) x TILE columns (j)
      const int ii = ta ? e >> 4 : e % TILE, ll = ta ? e & 15 : e / TILE;
      const int i = i0 + ii, l = l0 + ll;
      double2 v = make_double2(0.0, 0.0);
      if (i < M && l < k1) v = ta ? A[l + (int64_t)i * lda] : A[i + (int64_t)l * lda];
      As[ll][ii] = v;
      const int jj = tb ? e % TILE : e >> 4, lb = tb ? e / TILE : e & 15;
      const int j = j0 + jj, l2 = l0 + lb;
      double2 w = make_double2(0.0, 0.0);
      if (j < N && l2 < k1) w = tb ? B[j + (int64_t)l2 * ldb] : B[l2 + (int64_t)j * ldb];
      Bs[lb][jj] = w;
    }
    __syncthreads();
#pragma unroll 4
    for (int l = 0; l < 16; ++l) {
      double2 av[R], bv[R];
#pragma unroll
      for (int a = 0; a < R; ++a) av[a] = As[l][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < R; ++b) bv[b] = Bs[l][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) cfma(acc[a][b], av[a], bv[b]);
    }
    __syncthreads();
  }
  const bool b0 = beta.x == 0.0 && beta.y == 0.0;
#pragma unroll
  for (int a = 0; a < R; ++a)
#pragma unroll
    for (int b = 0; b < R; ++b) {
      const int i = i0 + tx + 16 * a, j = j0 + ty + 16 * b;
      if (i < M && j < N) {
        if (W) {
          W[(int64_t)blockIdx.z * M * N + i + (int64_t)j * M] = acc[a][b];
        } else {
          double2* cp = C + i + (int64_t)j * ldc;
          double2 v = cmul(alpha, acc[a][b]);
          if (!b0) v = cadd(v, cmul(beta, *cp));
          *cp = v;
        }
      }
    }
}

// C = alpha sum_z W[z] + beta C, the parts summed in order z = 0, 1, ...
__global__ void k_zgemm_reduce(int M, int N, int nz, const double2* __restrict__ W, double2 alpha, double2 beta,
                               double2* __restrict__ C, int ldc) {
  const int64_t cnt = (int64_t)M * N;
  const bool b0 = beta.x == 0.0 && beta.y == 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    double2 s = W[e];
    for (int z = 1; z < nz; ++z) s = cadd(s, W[(int64_t)z * cnt + e]);
    const int i = (int)(e % M), j = (int)(e / M);
    double2* cp = C + i + (int64_t)j * ldc;
    double2 v = cmul(alpha, s);
    if (!b0) v = cadd(v, cmul(beta, *cp));
    *cp = v;
  }
}

// A = L U in place (n x n, ld lda): column j of L, then row j of U divided by
// L(j, j), then the trailing update (right-looking order of the same factors)
__global__ void __launch_bounds__(1024) k_lu_leaf(double2* A, int lda, int n, int* err) {
  for (int j = 0; j < n; ++j) {
    const double2 d = A[j + (int64_t)j * lda];
    if (d.x == 0.0 && d.y == 0.0) {
      if (threadIdx.x == 0) atomicOr(err, HL_ERR_PIVOT);
      return;
    }
    for (int c = j + 1 + threadIdx.x; c < n; c += blockDim.x) {
      double2* p = A + j + (int64_t)c * lda;
      *p = cdiv(*p, d);
    }
    __syncthreads();
    const int r = n - j - 1;
    for (int e = threadIdx.x; e < r * r; e += blockDim.x) {
      const int ri = j + 1 + e % r, ci = j + 1 + e / r;
      double2* p = A + ri + (int64_t)ci * lda;
      *p = csub(*p, cmul(A[ri + (int64_t)j * lda], A[j + (int64_t)ci * lda]));
    }
    __syncthreads();
  }
}

// op(T) X = X in place for the n x nrhs block X (ld ldx); T(i, j) = A(i, j)
// (trans 0) or A(j, i); lower: T lower triangular; unit: unit diagonal.
// One CTA of 32 x 32 threads per 32 right-hand sides.
__global__ void __launch_bounds__(1024) k_trsm(const double2* __restrict__ A, int lda, int n, int lower, int unit,
                                               int trans, double2* X, int ldx, int nrhs) {
  const int rl = threadIdx.x, col = blockIdx.x * 32 + threadIdx.y;
  const bool act = col < nrhs;
  double2* x = X + (int64_t)(act ? col : 0) * ldx;
  auto T = [&](int i, int j) { return trans ? A[j + (int64_t)i * lda] : A[i + (int64_t)j * lda]; };
  for (int s = 0; s < n; ++s) {
    const int j = lower ? s : n - 1 - s;
    if (!unit) {
      if (act && rl == 0) x[j] = cdiv(x[j], T(j, j));
      __syncthreads();
    }
    const double2 xj = act ? x[j] : make_double2(0.0, 0.0);
    if (lower) {
      for (int i = j + 1 + rl; i < n; i += 32)
        if (act) x[i] = csub(x[i], cmul(T(i, j), xj));
    } else {
      for (int i = rl; i < j; i += 32)
        if (act) x[i] = csub(x[i], cmul(T(i, j), xj));
    }
    __syncthreads();
  }
}

// inverse in place by Gauss-Jordan with partial pivoting (|re| + |im|, first
// maximum, as izamax); column swaps undone at the end
__global__ void __launch_bounds__(1024) k_inv_leaf(double2* A, int lda, int n, int* piv, int* err) {
  __shared__ double2 colj[HL_LEAF_MAX];
  __shared__ double bv[32];
  __shared__ int bi[32];
  __shared__ int p_s;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  for (int j = 0; j < n; ++j) {
    double v = -1.0;
    int vi = n;
    for (int i = j + tid; i < n; i += blockDim.x) {
      const double a = cabs1(A[i + (int64_t)j * lda]);
      if (a > v) { v = a; vi = i; }
    }
    for (int o = 16; o; o >>= 1) {
      const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, vi, o);
      if (v2 > v || (v2 == v && i2 < vi)) { v = v2; vi = i2; }
    }
    if (lane == 0) { bv[wid] = v; bi[wid] = vi; }
    __syncthreads();
    if (tid == 0) {
      double bvv = bv[0];
      int bii = bi[0];
      for (int w = 1; w < nw; ++w)
        if (bv[w] > bvv || (bv[w] == bvv && bi[w] < bii)) { bvv = bv[w]; bii = bi[w]; }
      p_s = bii;
      piv[j] = bii;
    }
    __syncthreads();
    const int p = p_s;
    if (p != j)
      for (int c = tid; c < n; c += blockDim.x) {
        double2* a = A + j + (int64_t)c * lda;
        double2* b = A + p + (int64_t)c * lda;
        const double2 t = *a;
        *a = *b;
        *b = t;
      }
    __syncthreads();
    const double2 d = A[j + (int64_t)j * lda];
    if (d.x == 0.0 && d.y == 0.0) {
      if (tid == 0) atomicOr(err, HL_ERR_PIVOT);
      return;
    }
    const double2 dinv = cdiv(make_double2(1.0, 0.0), d);
    for (int c = tid; c < n; c += blockDim.x) {
      double2* a = A + j + (int64_t)c * lda;
      *a = c == j ? dinv : cmul(*a, dinv);
    }
    for (int i = tid; i < n; i += blockDim.x) colj[i] = A[i + (int64_t)j * lda];
    __syncthreads();
    for (int e = tid; e < n * n; e += blockDim.x) {
      const int i = e % n, c = e / n;
      if (i == j) continue;
      const double2 f = colj[i];
      double2* a = A + i + (int64_t)c * lda;
      if (c == j) *a = cmul(make_double2(-f.x, -f.y), dinv);
      else *a = csub(*a, cmul(f, A[j + (int64_t)c * lda]));
    }
    __syncthreads();
  }
  for (int j = n - 1; j >= 0; --j) {
    const int p = piv[j];
    if (p != j)
      for (int i = tid; i < n; i += blockDim.x) {
        double2* a = A + i + (int64_t)j * lda;
        double2* b = A + i + (int64_t)p * lda;
        const double2 t = *a;
        *a = *b;
        *b = t;
      }
    __syncthreads();
  }
}

constexpr int ACA_THREADS = 256;

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < ACA_THREADS / 32; ++i) s += red[i];
  return s;
}
__device__ int block_argmax(double v, int vi, double* red, int* redi) {
  for (int o = 16; o; o >>= 1) {
    const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, vi, o);
    if (v2 > v || (v2 == v && i2 < vi)) { v = v2; vi = i2; }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) { red[w] = v; redi[w] = vi; }
  __syncthreads();
  double b = red[0];
  int bi = redi[0];
  for (int i = 1; i < ACA_THREADS / 32; ++i)
    if (red[i] > b || (red[i] == b && redi[i] < bi)) { b = red[i]; bi = redi[i]; }
  return bi;
}

// ACA of an m x n block given as a full matrix M (ld ldm, K = 0) or as the
// product Lk Rk^T (Lk m x K, Rk n x K, column-major): L [m][kcap] (ld m),
// R [n][kcap] (ld n), the rank in out[0]
__global__ void __launch_bounds__(ACA_THREADS) k_aca(int m, int n, int kcap, double tol, const double2* __restrict__ M,
                                                     int ldm, const double2* __restrict__ Lk,
                                                     const double2* __restrict__ Rk, int K, double2* L, double2* R,
                                                     unsigned char* used, int* out) {
  __shared__ double red[ACA_THREADS / 32];
  __shared__ int redi[ACA_THREADS / 32];
  const int tid = threadIdx.x;
  int r = 0, k = 0, nused = 0, rank = -1;
  double nsum = 0.0;
  for (int i = tid; i < m; i += ACA_THREADS) used[i] = 0;
  __syncthreads();
  while (k < kcap) {
    double2* bk = R + (int64_t)k * n;
    double2* ak = L + (int64_t)k * m;
    double s2 = 0.0;
    for (int j = tid; j < n; j += ACA_THREADS) {
      double2 v = make_double2(0.0, 0.0);
      if (K == 0) v = M[r + (int64_t)j * ldm];
      else
        for (int l = 0; l < K; ++l) cfma(v, Lk[r + (int64_t)l * m], Rk[j + (int64_t)l * n]);
      bk[j] = v;
      s2 += v.x * v.x + v.y * v.y;
    }
    if (sqrt(block_sum(s2, red)) < ACA_STOP) {
      for (int i = tid; i < m; i += ACA_THREADS) ak[i] = make_double2(0.0, 0.0);
      break;
    }
    double bv = -1.0;
    int bi = n;
    for (int j = tid; j < n; j += ACA_THREADS) {
      double2 v = bk[j];
      for (int l = 0; l < k; ++l) v = csub(v, cmul(R[j + (int64_t)l * n], L[r + (int64_t)l * m]));
      bk[j] = v;
      const double a = cabs1(v);
      if (a > bv) { bv = a; bi = j; }
    }
    const int c = block_argmax(bv, bi, red, redi);
    const double2 piv = bk[c];
    __syncthreads();
    if (piv.x == 0.0 && piv.y == 0.0) { rank = k; break; }
    const double2 sc = cdiv(make_double2(1.0, 0.0), piv);
    for (int j = tid; j < n; j += ACA_THREADS) bk[j] = cmul(bk[j], sc);
    __syncthreads();
    for (int i = tid; i < m; i += ACA_THREADS) {
      double2 v = make_double2(0.0, 0.0);
      if (K == 0) v = M[i + (int64_t)c * ldm];
      else
        for (int l = 0; l < K; ++l) cfma(v, Lk[i + (int64_t)l * m], Rk[c + (int64_t)l * n]);
      for (int l = 0; l < k; ++l) v = csub(v, cmul(L[i + (int64_t)l * m], R[c + (int64_t)l * n]));
      ak[i] = v;
    }
    if (tid == 0) used[r] = 1;
    ++nused;
    __syncthreads();
    double av = -1.0;
    int ai = m;
    double sa = 0.0, sb = 0.0;
    for (int i = tid; i < m; i += ACA_THREADS) {
      const double2 v = ak[i];
      sa += v.x * v.x + v.y * v.y;
      const double a = used[i] ? 0.0 : cabs1(v);
      if (a > av) { av = a; ai = i; }
    }
    for (int j = tid; j < n; j += ACA_THREADS) {
      const double2 v = bk[j];
      sb += v.x * v.x + v.y * v.y;
    }
    r = block_argmax(av, ai, red, redi);
    const double na = sqrt(block_sum(sa, red));
    const double nb = sqrt(block_sum(sb, red));
    const double nk = na * nb;
    if (nk < tol * nsum || nused >= m) break;
    nsum = sqrt(nsum * nsum + nk * nk);
    ++k;
  }
  if (tid == 0) out[0] = rank >= 0 ? rank : min(k + 1, kcap);
}

__global__ void k_add2(const double2* a, const double2* b, double2* out, int64_t cnt, double sb) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const double2 y = b[e];
    out[e] = make_double2(a[e].x + sb * y.x, a[e].y + sb * y.y);
  }
}
__global__ void k_eye(double2* out, int n) {
  const int64_t cnt = (int64_t)n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = make_double2(e % n == e / n ? 1.0 : 0.0, 0.0);
}
__global__ void k_negate(const double2* a, double2* out, int64_t cnt) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = make_double2(-a[e].x, -a[e].y);
}
// out[i + j m] = a[i + j m] * d[rows ? i : j]
__global__ void k_scale_rc(const double2* a, double2* out, int m, int n, const double2* d, int rows) {
  const int64_t cnt = (int64_t)m * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % m), j = (int)(e / m);
    out[e] = cmul(a[e], d[rows ? i : j]);
  }
}
// B (n x m, ld n) = A^T (A m x n, ld lda)
__global__ void k_transpose(const double2* A, int lda, int m, int n, double2* B) {
  __shared__ double2 t[32][33];
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int e = threadIdx.x; e < 1024; e += blockDim.x) {
    const int ii = e & 31, jj = e >> 5;
    if (i0 + ii < m && j0 + jj < n) t[jj][ii] = A[i0 + ii + (int64_t)(j0 + jj) * lda];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 1024; e += blockDim.x) {
    const int jj = e & 31, ii = e >> 5;
    if (i0 + ii < m && j0 + jj < n) B[j0 + jj + (int64_t)(i0 + ii) * n] = t[jj][ii];
  }
}
unsigned eblocks(int64_t cnt) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv_up(cnt, 256), 4096)); }

// ------------------------------------------------------ device resources
struct DevRes {
  cudaStream_t st = nullptr;
  cudaMemPool_t pool = nullptr;
};
std::mutex g_res_mu;
DevRes g_res[64];

mnpbem_status dev_res(int device, DevRes*& out) {
  if (device < 0 || device >= 64) {
    set_error("H-matrix arithmetic: device %d out of range", device);
    return MNPBEM_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lk(g_res_mu);
  DevRes& r = g_res[device];
  if (!r.st) {
    int cur = 0;
    MNP_CUDA(cudaGetDevice(&cur));
    MNP_CUDA(cudaSetDevice(device));
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaError_t e = cudaMemPoolCreate(&r.pool, &props);
    if (e == cudaSuccess) {
      uint64_t keep = ~0ull;   // keep freed blocks for reuse
      e = cudaMemPoolSetAttribute(r.pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&r.st, cudaStreamNonBlocking);
    cudaSetDevice(cur);
    if (e != cudaSuccess) {
      set_error("H-matrix arithmetic: stream / pool creation failed: %s", cudaGetErrorString(e));
      r.st = nullptr;
      return MNPBEM_ERR_CUDA;
    }
  }
  out = &r;
  return MNPBEM_OK;
}

}  // namespace

// ------------------------------------------------------------ tree, context
void Tree::pairs(int r, int c, std::vector<Key>& out) const {
  if (admiss(r, c)) {
    out.emplace_back(r, c);
    return;
  }
  int a[2], b[2];
  const int na = begin(r, a), nb = begin(c, b);
  for (int x = 0; x < na; ++x)
    for (int y = 0; y < nb; ++y) pairs(a[x], b[y], out);
}

Ctx::~Ctx() {
  if (host) cudaFreeHost(host);
  if (dev) cudaFreeAsync(dev, st);
}

mnpbem_status hl_stream(int device, cudaStream_t& st) {
  DevRes* r = nullptr;
  MNP_TRY(dev_res(device, r));
  st = r->st;
  return MNPBEM_OK;
}

mnpbem_status ctx_make(int device, std::shared_ptr<const Tree> t, double tol, int kmax, std::shared_ptr<Ctx>& out) {
  DevRes* r = nullptr;
  MNP_TRY(dev_res(device, r));
  auto c = std::make_shared<Ctx>();
  c->t = std::move(t);
  c->tol = tol;
  c->kmax = kmax;
  c->st = r->st;
  c->device = device;
  MNP_CUDA(cudaMallocHost(&c->host, 2 * sizeof(int)));
  MNP_CUDA(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&c->dev), 2 * sizeof(int), r->pool, r->st));
  MNP_CUDA(cudaMemsetAsync(c->dev, 0, 2 * sizeof(int), r->st));
  out = std::move(c);
  return MNPBEM_OK;
}

// hand the pool's free blocks beyond a small reserve back to the device (the
// pool keeps freed blocks for reuse inside one operation; between operations
// they would only be missing from the solver's own allocations)
static void pool_trim(int device) {
  DevRes* r = nullptr;
  if (dev_res(device, r) == MNPBEM_OK && r->pool) cudaMemPoolTrimTo(r->pool, (size_t)256 << 20);
}

mnpbem_status check_flags(Ctx& c) {
  MNP_CUDA(cudaMemcpyAsync(c.host, c.dev, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.st));
  MNP_CUDA(cudaStreamSynchronize(c.st));
  pool_trim(c.device);
  if (c.host[1] & HL_ERR_PIVOT) {
    MNP_CUDA(cudaMemsetAsync(c.dev + 1, 0, sizeof(int), c.st));
    set_error("H-matrix arithmetic: zero pivot in the LU or the inverse of a leaf block");
    return MNPBEM_ERR_SINGULAR;
  }
  return MNPBEM_OK;
}

mnpbem_status alloc(Ctx& c, int m, int n, DMat& out) {
  DevRes* r = nullptr;
  MNP_TRY(dev_res(c.device, r));
  const size_t bytes = sizeof(double2) * std::max<int64_t>(1, (int64_t)m * n);
  double2* p = nullptr;
  MNP_CUDA(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p), bytes, r->pool, c.st));
  cudaStream_t st = c.st;
  out.p = std::shared_ptr<double2>(p, [st](double2* q) { cudaFreeAsync(q, st); });
  out.m = m;
  out.n = n;
  return MNPBEM_OK;
}

mnpbem_status alloc_raw(Ctx& c, size_t bytes, std::shared_ptr<void>& out) {
  DevRes* r = nullptr;
  MNP_TRY(dev_res(c.device, r));
  void* p = nullptr;
  MNP_CUDA(cudaMallocFromPoolAsync(&p, std::max<size_t>(bytes, 16), r->pool, c.st));
  cudaStream_t st = c.st;
  out = std::shared_ptr<void>(p, [st](void* q) { cudaFreeAsync(q, st); });
  return MNPBEM_OK;
}

mnpbem_status upload(Ctx& c, const double2* host, int m, int n, DMat& out) {
  MNP_TRY(alloc(c, m, n, out));
  if ((int64_t)m * n > 0)
    MNP_CUDA(cudaMemcpyAsync(out.ptr(), host, sizeof(double2) * m * n, cudaMemcpyHostToDevice, c.st));
  return MNPBEM_OK;
}

// ------------------------------------------------------ dense primitives
namespace {

// a column-major sub-block view
struct View {
  const double2* p = nullptr;
  int ld = 0, m = 0, n = 0;
};
View whole(const DMat& a) { return View{a.ptr(), std::max(1, a.m), a.m, a.n}; }
View rows_of(const DMat& a, int r0, int nr) { return View{a.ptr() + r0, std::max(1, a.m), nr, a.n}; }
View block_of(const DMat& a, int r0, int nr, int c0, int nc) {
  return View{a.ptr() + r0 + (int64_t)c0 * std::max(1, a.m), std::max(1, a.m), nr, nc};
}

// FP64 runs at a small fraction of the FP32 rate on this GPU, so every product
// is spread over the SMs: 32 x 32 tiles when they alone give a full wave, else
// 16 x 16 tiles, and when those are still too few the K range is split
// across CTAs whose partial sums are added in a fixed order (deterministic).
constexpr int HL_WAVE = 148;
mnpbem_status gemm(Ctx& c, int M, int N, int K, double2 alpha, View A, int ta, View B, int tb, double2 beta,
                   double2* C, int ldc) {
  if (M <= 0 || N <= 0) return MNPBEM_OK;
  const int64_t t32 = cdiv_up(M, 32) * cdiv_up(N, 32);
  if (t32 >= HL_WAVE) {
    dim3 grid((unsigned)cdiv_up(M, 32), (unsigned)cdiv_up(N, 32), 1);
    k_zgemm<32><<<grid, 256, 0, c.st>>>(M, N, K, std::max(K, 1), alpha, A.p, A.ld, ta, B.p, B.ld, tb, beta, C, ldc,
                                        nullptr);
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  const int64_t t16 = cdiv_up(M, 16) * cdiv_up(N, 16);
  int nz = 1;
  if (t16 < HL_WAVE && K > 64) nz = (int)std::min<int64_t>(cdiv_up(HL_WAVE, t16), cdiv_up(K, 64));
  const int kc = (int)round_up(cdiv_up(std::max(K, 1), nz), 16);
  nz = (int)cdiv_up(std::max(K, 1), kc);
  dim3 grid((unsigned)cdiv_up(M, 16), (unsigned)cdiv_up(N, 16), (unsigned)nz);
  if (nz == 1) {
    k_zgemm<16><<<grid, 256, 0, c.st>>>(M, N, K, kc, alpha, A.p, A.ld, ta, B.p, B.ld, tb, beta, C, ldc, nullptr);
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  std::shared_ptr<void> W;
  MNP_TRY(alloc_raw(c, sizeof(double2) * (size_t)nz * M * N, W));
  double2* w = static_cast<double2*>(W.get());
  k_zgemm<16><<<grid, 256, 0, c.st>>>(M, N, K, kc, alpha, A.p, A.ld, ta, B.p, B.ld, tb, beta, C, ldc, w);
  MNP_CHECK_LAUNCH();
  k_zgemm_reduce<<<eblocks((int64_t)M * N), 256, 0, c.st>>>(M, N, nz, w, alpha, beta, C, ldc);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

const double2 ONE = {1.0, 0.0}, ZERO = {0.0, 0.0}, MONE = {-1.0, 0.0};

// new matrix = op(A) op(B)
mnpbem_status mul(Ctx& c, View A, int ta, View B, int tb, DMat& out) {
  const int M = ta ? A.n : A.m, K = ta ? A.m : A.n, N = tb ? B.m : B.n;
  MNP_TRY(alloc(c, M, N, out));
  return gemm(c, M, N, K, ONE, A, ta, B, tb, ZERO, out.ptr(), std::max(1, M));
}

mnpbem_status copy_view(Ctx& c, View a, DMat& out) {
  MNP_TRY(alloc(c, a.m, a.n, out));
  if (a.m > 0 && a.n > 0)
    MNP_CUDA(cudaMemcpy2DAsync(out.ptr(), sizeof(double2) * a.m, a.p, sizeof(double2) * a.ld, sizeof(double2) * a.m,
                               a.n, cudaMemcpyDeviceToDevice, c.st));
  return MNPBEM_OK;
}

mnpbem_status transpose(Ctx& c, View a, DMat& out) {
  MNP_TRY(alloc(c, a.n, a.m, out));
  if (a.m > 0 && a.n > 0) {
    dim3 grid((unsigned)cdiv_up(a.m, 32), (unsigned)cdiv_up(a.n, 32));
    k_transpose<<<grid, 256, 0, c.st>>>(a.p, a.ld, a.m, a.n, out.ptr());
    MNP_CHECK_LAUNCH();
  }
  return MNPBEM_OK;
}

// [A B] (same rows)
mnpbem_status hcat(Ctx& c, const DMat& a, const DMat& b, DMat& out) {
  MNP_TRY(alloc(c, a.m, a.n + b.n, out));
  const size_t sa = sizeof(double2) * a.m * a.n, sb = sizeof(double2) * b.m * b.n;
  if (sa) MNP_CUDA(cudaMemcpyAsync(out.ptr(), a.ptr(), sa, cudaMemcpyDeviceToDevice, c.st));
  if (sb) MNP_CUDA(cudaMemcpyAsync(out.ptr() + (int64_t)a.m * a.n, b.ptr(), sb, cudaMemcpyDeviceToDevice, c.st));
  return MNPBEM_OK;
}

// place a at (r0, c0) of out (ld out.m)
mnpbem_status place(Ctx& c, const DMat& a, DMat& out, int r0, int c0) {
  if (a.m > 0 && a.n > 0)
    MNP_CUDA(cudaMemcpy2DAsync(out.ptr() + r0 + (int64_t)c0 * out.m, sizeof(double2) * out.m, a.ptr(),
                               sizeof(double2) * a.m, sizeof(double2) * a.m, a.n, cudaMemcpyDeviceToDevice, c.st));
  return MNPBEM_OK;
}

mnpbem_status zeros(Ctx& c, int m, int n, DMat& out) {
  MNP_TRY(alloc(c, m, n, out));
  if ((int64_t)m * n > 0) MNP_CUDA(cudaMemsetAsync(out.ptr(), 0, sizeof(double2) * m * n, c.st));
  return MNPBEM_OK;
}

mnpbem_status add2(Ctx& c, const DMat& a, const DMat& b, double sb, DMat& out) {
  MNP_TRY(alloc(c, a.m, a.n, out));
  const int64_t cnt = (int64_t)a.m * a.n;
  if (cnt) {
    k_add2<<<eblocks(cnt), 256, 0, c.st>>>(a.ptr(), b.ptr(), out.ptr(), cnt, sb);
    MNP_CHECK_LAUNCH();
  }
  return MNPBEM_OK;
}

mnpbem_status negate(Ctx& c, const DMat& a, DMat& out) {
  MNP_TRY(alloc(c, a.m, a.n, out));
  const int64_t cnt = (int64_t)a.m * a.n;
  if (cnt) {
    k_negate<<<eblocks(cnt), 256, 0, c.st>>>(a.ptr(), out.ptr(), cnt);
    MNP_CHECK_LAUNCH();
  }
  return MNPBEM_OK;
}

// op(T) X = X in place on the view (ld, n rows, nrhs columns); T the L
// ('L', with its diagonal) or the U ('U', unit diagonal) of the leaf LU A
mnpbem_status trsm_left(Ctx& c, const DMat& A, char uplo, char trans, double2* X, int ldx, int nrhs) {
  const int n = A.m;
  if (n <= 0 || nrhs <= 0) return MNPBEM_OK;
  const int tr = trans == 'T';
  const int lower = (uplo == 'L') != (tr != 0);
  k_trsm<<<(unsigned)cdiv_up(nrhs, 32), dim3(32, 32), 0, c.st>>>(A.ptr(), A.m, n, lower, uplo == 'U' ? 1 : 0, tr, X,
                                                                   ldx, nrhs);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

// lu.cpp:110-124 solve(side, B, transB, A, uplo) as a new matrix, A the
// diagonal leaf of an LU: products with the inverses of its triangles (formed
// once per leaf) when it has them, else substitution
mnpbem_status trsm(Ctx& c, char side, View B, char trans, const Sub& A, char uplo, DMat& out) {
  const DMat& Ti = uplo == 'L' ? A.linv : A.uinv;
  const int tr = trans == 'T';
  if (Ti.p) {
    if (side == 'L') return mul(c, whole(Ti), tr, B, 0, out);
    return mul(c, B, 0, whole(Ti), tr, out);
  }
  if (side == 'L') {
    MNP_TRY(copy_view(c, B, out));
    return trsm_left(c, A.mat, uplo, trans, out.ptr(), std::max(1, out.m), out.n);
  }
  // X op(A) = B  <=>  op(A)^T X^T = B^T
  DMat Y;
  MNP_TRY(transpose(c, B, Y));
  MNP_TRY(trsm_left(c, A.mat, uplo, tr ? 'N' : 'T', Y.ptr(), std::max(1, Y.m), Y.n));
  return transpose(c, whole(Y), out);
}

// LU of a full leaf and the inverses of its triangles
mnpbem_status lu_dense(Ctx& c, const DMat& a, int i, Sub& out) {
  if (a.m > HL_LEAF_MAX || a.m != a.n) {
    set_error("H-matrix LU: leaf blocks of %d x %d are not supported (square, at most %d)", a.m, a.n, HL_LEAF_MAX);
    return MNPBEM_ERR_UNSUPPORTED;
  }
  const int n = a.m;
  out = Sub();
  out.row = out.col = i;
  out.flag = FLAG_FULL;
  MNP_TRY(copy_view(c, whole(a), out.mat));
  if (n == 0) return MNPBEM_OK;
  k_lu_leaf<<<1, 1024, 0, c.st>>>(out.mat.ptr(), n, n, c.dev + 1);
  MNP_CHECK_LAUNCH();
  for (int q = 0; q < 2; ++q) {
    DMat& X = q == 0 ? out.linv : out.uinv;
    MNP_TRY(alloc(c, n, n, X));
    k_eye<<<eblocks((int64_t)n * n), 256, 0, c.st>>>(X.ptr(), n);
    MNP_CHECK_LAUNCH();
    MNP_TRY(trsm_left(c, out.mat, q == 0 ? 'L' : 'U', 'N', X.ptr(), n, n));
  }
  return MNPBEM_OK;
}

mnpbem_status inv_dense(Ctx& c, const DMat& a, DMat& out) {
  if (a.m > HL_LEAF_MAX || a.m != a.n) {
    set_error("H-matrix inverse: leaf blocks of %d x %d are not supported (square, at most %d)", a.m, a.n,
              HL_LEAF_MAX);
    return MNPBEM_ERR_UNSUPPORTED;
  }
  MNP_TRY(copy_view(c, whole(a), out));
  if (a.m > 0) {
    std::shared_ptr<void> piv;
    MNP_TRY(alloc_raw(c, sizeof(int) * a.m, piv));
    k_inv_leaf<<<1, 1024, 0, c.st>>>(out.ptr(), a.m, a.m, static_cast<int*>(piv.get()), c.dev + 1);
    MNP_CHECK_LAUNCH();
  }
  return MNPBEM_OK;
}

// ACA of a full block (K = 0) or of Lk Rk^T; L, R get the rank's columns
mnpbem_status aca_run(Ctx& c, int m, int n, int kcap, View M, const DMat* Lk, const DMat* Rk, DMat& L, DMat& R) {
  MNP_TRY(alloc(c, m, std::max(kcap, 1), L));
  MNP_TRY(alloc(c, n, std::max(kcap, 1), R));
  int rank = 0;
  if (kcap > 0 && m > 0 && n > 0) {
    std::shared_ptr<void> used;
    MNP_TRY(alloc_raw(c, (size_t)m, used));
    k_aca<<<1, ACA_THREADS, 0, c.st>>>(m, n, kcap, c.tol, M.p, M.ld, Lk ? Lk->ptr() : nullptr,
                                        Rk ? Rk->ptr() : nullptr, Lk ? Lk->n : 0, L.ptr(), R.ptr(),
                                        static_cast<unsigned char*>(used.get()), c.dev);
    MNP_CHECK_LAUNCH();
    MNP_CUDA(cudaMemcpyAsync(c.host, c.dev, sizeof(int), cudaMemcpyDeviceToHost, c.st));
    MNP_CUDA(cudaStreamSynchronize(c.st));
    rank = c.host[0];
  }
  L.n = rank;
  R.n = rank;
  return MNPBEM_OK;
}

// ------------------------------------------------------ sub-matrices
const Tree& T(Ctx& c) { return *c.t; }
int rel(Ctx& c, int i, int parent) { return T(c).lo[i] - T(c).lo[parent]; }

Sub make_full(int r, int col, DMat m) {
  Sub s;
  s.row = r; s.col = col; s.flag = FLAG_FULL; s.mat = std::move(m);
  return s;
}
Sub make_rk(int r, int col, DMat l, DMat rr) {
  Sub s;
  s.row = r; s.col = col; s.flag = FLAG_RK; s.lhs = std::move(l); s.rhs = std::move(rr);
  return s;
}

// views of a block restricted to sub-clusters
View mat_view(Ctx& c, const Sub& A, int i, int j) {
  return block_of(A.mat, rel(c, i, A.row), T(c).size(i), rel(c, j, A.col), T(c).size(j));
}
View lhs_view(Ctx& c, const Sub& A, int i) { return rows_of(A.lhs, rel(c, i, A.row), T(c).size(i)); }
View rhs_view(Ctx& c, const Sub& A, int j) { return rows_of(A.rhs, rel(c, j, A.col), T(c).size(j)); }

// a sub-block as a matrix of its own: the matrix itself (shared: blocks are
// never modified once built) when the sub-block is all of it, else a copy
mnpbem_status take_block(Ctx& c, const DMat& a, int r0, int nr, int c0, int nc, DMat& out) {
  if (r0 == 0 && c0 == 0 && nr == a.m && nc == a.n) {
    out = a;
    return MNPBEM_OK;
  }
  return copy_view(c, block_of(a, r0, nr, c0, nc), out);
}
mnpbem_status take_rows(Ctx& c, const DMat& a, int r0, int nr, DMat& out) {
  return take_block(c, a, r0, nr, 0, a.n, out);
}
mnpbem_status lhs_take(Ctx& c, const Sub& A, int i, DMat& out) {
  return take_rows(c, A.lhs, rel(c, i, A.row), T(c).size(i), out);
}
mnpbem_status rhs_take(Ctx& c, const Sub& A, int j, DMat& out) {
  return take_rows(c, A.rhs, rel(c, j, A.col), T(c).size(j), out);
}

mnpbem_status truncate(Ctx& c, Sub& A) {
  if (A.flag != FLAG_RK) return MNPBEM_OK;
  DMat L, R;
  const int kcap = std::min(A.lhs.n, c.kmax);
  MNP_TRY(aca_run(c, A.lhs.m, A.rhs.m, kcap, View{}, &A.lhs, &A.rhs, L, R));
  A.lhs = std::move(L);
  A.rhs = std::move(R);
  return MNPBEM_OK;
}

mnpbem_status convert(Ctx& c, Sub& A, int flag) {
  if (A.flag == flag) return MNPBEM_OK;
  if (A.flag == FLAG_RK) {
    DMat m;
    MNP_TRY(mul(c, whole(A.lhs), 0, whole(A.rhs), 1, m));
    A = make_full(A.row, A.col, std::move(m));
    return MNPBEM_OK;
  }
  DMat L, R;
  const int m = A.mat.m, n = A.mat.n;
  MNP_TRY(aca_run(c, m, n, std::min(std::min(m, n), c.kmax), whole(A.mat), nullptr, nullptr, L, R));
  A = make_rk(A.row, A.col, std::move(L), std::move(R));
  return MNPBEM_OK;
}

mnpbem_status mask(Ctx& c, const Sub& A, int r, int col, Sub& out) {
  if (A.flag == FLAG_FULL) {
    DMat m;
    MNP_TRY(take_block(c, A.mat, rel(c, r, A.row), T(c).size(r), rel(c, col, A.col), T(c).size(col), m));
    out = make_full(r, col, std::move(m));
  } else {
    DMat l, rr;
    MNP_TRY(lhs_take(c, A, r, l));
    MNP_TRY(rhs_take(c, A, col, rr));
    out = make_rk(r, col, std::move(l), std::move(rr));
  }
  return MNPBEM_OK;
}

// acc += B (submatrix.h operator+=); acc.flag == 0: acc = B
mnpbem_status iadd(Ctx& c, Sub& acc, const Sub& B) {
  if (acc.flag == 0) {
    acc = B;
    return MNPBEM_OK;
  }
  if (acc.flag == FLAG_FULL) {
    DMat m;
    MNP_TRY(add2(c, acc.mat, B.mat, 1.0, m));
    acc.mat = std::move(m);
    return MNPBEM_OK;
  }
  DMat l, r;
  MNP_TRY(hcat(c, acc.lhs, B.lhs, l));
  MNP_TRY(hcat(c, acc.rhs, B.rhs, r));
  acc.lhs = std::move(l);
  acc.rhs = std::move(r);
  return truncate(c, acc);
}

mnpbem_status neg(Ctx& c, const Sub& A, Sub& out) {
  if (A.flag == FLAG_FULL) {
    DMat m;
    MNP_TRY(negate(c, A.mat, m));
    out = make_full(A.row, A.col, std::move(m));
  } else {
    DMat l;
    MNP_TRY(negate(c, A.lhs, l));
    out = make_rk(A.row, A.col, std::move(l), A.rhs);
  }
  return MNPBEM_OK;
}

// A - B as A += (-B)
mnpbem_status sub_minus(Ctx& c, const Sub& A, const Sub& B, Sub& out) {
  Sub nb;
  MNP_TRY(neg(c, B, nb));
  out = A;
  return iadd(c, out, nb);
}

// C(i, j) = A(i, k) B(k, j) (submatrix.h:196-219)
mnpbem_status mul_sub(Ctx& c, const Sub& A, const Sub& B, int i, int j, int k, Sub& out) {
  if (A.flag == FLAG_FULL && B.flag == FLAG_FULL) {
    DMat m;
    MNP_TRY(mul(c, mat_view(c, A, i, k), 0, mat_view(c, B, k, j), 0, m));
    out = make_full(i, j, std::move(m));
  } else if (A.flag == FLAG_FULL) {
    DMat l, r;
    MNP_TRY(mul(c, mat_view(c, A, i, k), 0, lhs_view(c, B, k), 0, l));
    MNP_TRY(rhs_take(c, B, j, r));
    out = make_rk(i, j, std::move(l), std::move(r));
  } else if (B.flag == FLAG_FULL) {
    DMat l, r;
    MNP_TRY(lhs_take(c, A, i, l));
    MNP_TRY(mul(c, mat_view(c, B, k, j), 1, rhs_view(c, A, k), 0, r));
    out = make_rk(i, j, std::move(l), std::move(r));
  } else {
    DMat S;
    MNP_TRY(mul(c, rhs_view(c, A, k), 1, lhs_view(c, B, k), 0, S));
    DMat l, r;
    if (S.m > S.n) {
      MNP_TRY(mul(c, lhs_view(c, A, i), 0, whole(S), 0, l));
      MNP_TRY(rhs_take(c, B, j, r));
    } else {
      MNP_TRY(lhs_take(c, A, i, l));
      MNP_TRY(mul(c, rhs_view(c, B, j), 0, whole(S), 1, r));
    }
    out = make_rk(i, j, std::move(l), std::move(r));
  }
  return MNPBEM_OK;
}

// submatrix.h:222-261: C[a][b] (na x nb sub-matrices) -> one block
mnpbem_status cat(Ctx& c, Sub C[2][2], int na, int nb, int row, int col, Sub& out) {
  if (C[0][0].flag == FLAG_FULL) {
    if (na == 1 && nb == 1) { out = make_full(row, col, C[0][0].mat); return MNPBEM_OK; }
    const int m = T(c).size(row), n = T(c).size(col);
    DMat M;
    MNP_TRY(alloc(c, m, n, M));
    int r0 = 0;
    for (int a = 0; a < na; ++a) {
      int c0 = 0;
      for (int b = 0; b < nb; ++b) {
        MNP_TRY(place(c, C[a][b].mat, M, r0, c0));
        c0 += C[a][b].mat.n;
      }
      r0 += C[a][0].mat.m;
    }
    out = make_full(row, col, std::move(M));
    return MNPBEM_OK;
  }
  if (na == 1 && nb == 1) { out = make_rk(row, col, C[0][0].lhs, C[0][0].rhs); return MNPBEM_OK; }
  const int m = T(c).size(row), n = T(c).size(col);
  DMat L, R;
  if (na == 2 && nb == 1) {
    // lhs [L0 0; 0 L1], rhs [R0 R1]
    const DMat &L0 = C[0][0].lhs, &L1 = C[1][0].lhs;
    MNP_TRY(zeros(c, m, L0.n + L1.n, L));
    MNP_TRY(place(c, L0, L, 0, 0));
    MNP_TRY(place(c, L1, L, L0.m, L0.n));
    MNP_TRY(hcat(c, C[0][0].rhs, C[1][0].rhs, R));
  } else if (na == 1 && nb == 2) {
    // lhs [L0 L1], rhs [R0 0; 0 R1]
    const DMat &R0 = C[0][0].rhs, &R1 = C[0][1].rhs;
    MNP_TRY(hcat(c, C[0][0].lhs, C[0][1].lhs, L));
    MNP_TRY(zeros(c, n, R0.n + R1.n, R));
    MNP_TRY(place(c, R0, R, 0, 0));
    MNP_TRY(place(c, R1, R, R0.m, R0.n));
  } else {
    // columns (0,0), (1,1), (1,0), (0,1): lhs [L00 0 0 L01; 0 L11 L10 0],
    // rhs [R00 0 R10 0; 0 R11 0 R01]
    const Sub *s00 = &C[0][0], *s11 = &C[1][1], *s10 = &C[1][0], *s01 = &C[0][1];
    const int k00 = s00->rank(), k11 = s11->rank(), k10 = s10->rank(), k01 = s01->rank();
    const int m0 = s00->lhs.m, n0 = s00->rhs.m;
    MNP_TRY(zeros(c, m, k00 + k11 + k10 + k01, L));
    MNP_TRY(zeros(c, n, k00 + k11 + k10 + k01, R));
    MNP_TRY(place(c, s00->lhs, L, 0, 0));
    MNP_TRY(place(c, s11->lhs, L, m0, k00));
    MNP_TRY(place(c, s10->lhs, L, m0, k00 + k11));
    MNP_TRY(place(c, s01->lhs, L, 0, k00 + k11 + k10));
    MNP_TRY(place(c, s00->rhs, R, 0, 0));
    MNP_TRY(place(c, s11->rhs, R, n0, k00));
    MNP_TRY(place(c, s10->rhs, R, 0, k00 + k11));
    MNP_TRY(place(c, s01->rhs, R, n0, k00 + k11 + k10));
  }
  out = make_rk(row, col, std::move(L), std::move(R));
  return MNPBEM_OK;
}

// ------------------------------------------------------ H-matrices
// operand of the recursive products: an H-matrix or one sub-matrix (whose
// find returns itself, submatrix.h find)
struct Op {
  const HM* h = nullptr;
  const Sub* s = nullptr;
  const Sub* find(int i, int j) const {
    if (s) return s;
    auto it = h->find(Key(i, j));
    return it == h->end() ? nullptr : &it->second;
  }
};
Op opH(const HM& h) { Op o; o.h = &h; return o; }
Op opS(const Sub& s) { Op o; o.s = &s; return o; }

mnpbem_status add_mul2(Ctx& c, Op A, Op B, int i, int j, int k, int flag, Sub& out) {
  const Sub *pA = A.find(i, k), *pB = B.find(k, j);
  if (pA && pB) {
    MNP_TRY(mul_sub(c, *pA, *pB, i, j, k, out));
    return convert(c, out, flag);
  }
  int bi[2], bj[2], bk[2];
  const int ni = T(c).begin(i, bi), nj = T(c).begin(j, bj), nk = T(c).begin(k, bk);
  Sub C[2][2];
  for (int a = 0; a < ni; ++a)
    for (int b = 0; b < nj; ++b)
      for (int q = 0; q < nk; ++q) {
        Sub s;
        if (pA) MNP_TRY(add_mul2(c, opS(*pA), B, bi[a], bj[b], bk[q], flag, s));
        else if (pB) MNP_TRY(add_mul2(c, A, opS(*pB), bi[a], bj[b], bk[q], flag, s));
        else MNP_TRY(add_mul2(c, A, B, bi[a], bj[b], bk[q], flag, s));
        MNP_TRY(iadd(c, C[a][b], s));
      }
  return cat(c, C, ni, nj, i, j, out);
}

mnpbem_status add_mul(Ctx& c, Op A, Op B, HM& C, int i, int j, int k) {
  const Sub *pA = A.find(i, k), *pB = B.find(k, j);
  const int adC = T(c).admiss(i, j);
  if (adC == 0) {
    int bi[2], bj[2], bk[2];
    const int ni = T(c).begin(i, bi), nj = T(c).begin(j, bj), nk = T(c).begin(k, bk);
    for (int a = 0; a < ni; ++a)
      for (int b = 0; b < nj; ++b)
        for (int q = 0; q < nk; ++q)
          MNP_TRY(add_mul(c, pA ? opS(*pA) : A, pB ? opS(*pB) : B, C, bi[a], bj[b], bk[q]));
    return MNPBEM_OK;
  }
  Sub s;
  if (pA && pB) {
    MNP_TRY(mul_sub(c, *pA, *pB, i, j, k, s));
    MNP_TRY(convert(c, s, adC));
  } else {
    MNP_TRY(add_mul2(c, A, B, i, j, k, adC, s));
  }
  return iadd(c, C[Key(i, j)], s);
}

mnpbem_status hmul(Ctx& c, Op A, Op B, int i, int j, int k, HM& C) {
  C.clear();
  return add_mul(c, A, B, C, i, j, k);
}

const Sub& at(const HM& A, Key p) {
  static const Sub empty;
  auto it = A.find(p);
  return it == A.end() ? empty : it->second;
}

// C(H) = A - B over the leaf pairs below (i, j)
mnpbem_status subtract(Ctx& c, const HM& A, const HM& B, int i, int j, HM& C) {
  std::vector<Key> ps;
  T(c).pairs(i, j, ps);
  C.clear();
  for (const Key& p : ps) {
    const Sub &a = at(A, p), &b = at(B, p);
    if (!a.flag || !b.flag) {
      set_error("H-matrix arithmetic: block (%d, %d) missing", p.first, p.second);
      return MNPBEM_ERR_INVALID_ARG;
    }
    MNP_TRY(sub_minus(c, a, b, C[p]));
  }
  return MNPBEM_OK;
}

mnpbem_status uminus(Ctx& c, const HM& A, int i, int j, HM& C) {
  std::vector<Key> ps;
  T(c).pairs(i, j, ps);
  C.clear();
  for (const Key& p : ps) MNP_TRY(neg(c, at(A, p), C[p]));
  return MNPBEM_OK;
}

// C[p] += A[p] + B[p] over the pairs below (i, j) (hmatrix.h add)
mnpbem_status add_into(Ctx& c, const HM& A, const HM& B, int i, int j, HM& C) {
  std::vector<Key> ps;
  T(c).pairs(i, j, ps);
  for (const Key& p : ps) {
    Sub s = at(A, p);
    if (!s.flag || !at(B, p).flag) {
      set_error("H-matrix arithmetic: block (%d, %d) missing", p.first, p.second);
      return MNPBEM_ERR_INVALID_ARG;
    }
    MNP_TRY(iadd(c, s, at(B, p)));
    MNP_TRY(iadd(c, C[p], s));
  }
  return MNPBEM_OK;
}

// ---- inversion (hmatrix.h:310-345)
mnpbem_status inv_rec(Ctx& c, const HM& A, int i, HM& C) {
  C.clear();
  if (T(c).leaf(i)) {
    DMat m;
    MNP_TRY(inv_dense(c, at(A, Key(i, i)).mat, m));
    C[Key(i, i)] = make_full(i, i, std::move(m));
    return MNPBEM_OK;
  }
  const int i0 = T(c).sons(i, 0), i1 = T(c).sons(i, 1);
  HM Y, t1, t2, S;
  MNP_TRY(inv_rec(c, A, i0, Y));
  MNP_TRY(hmul(c, opH(Y), opH(A), i0, i1, i0, t1));       // Y A01
  MNP_TRY(hmul(c, opH(A), opH(t1), i1, i1, i0, t2));      // A10 Y A01
  MNP_TRY(subtract(c, A, t2, i1, i1, S));
  MNP_TRY(inv_rec(c, S, i1, C));                          // C11 = inv(S)
  HM u1, u2, u3, t;
  MNP_TRY(hmul(c, opH(A), opH(Y), i1, i0, i0, u1));       // A10 Y
  MNP_TRY(hmul(c, opH(C), opH(u1), i1, i0, i1, u2));      // C11 A10 Y
  MNP_TRY(hmul(c, opH(A), opH(u2), i0, i0, i1, u3));      // A01 C11 A10 Y
  MNP_TRY(hmul(c, opH(Y), opH(u3), i0, i0, i0, t));       // Y A01 C11 A10 Y
  MNP_TRY(add_into(c, Y, t, i0, i0, C));                  // C00 = Y + t
  HM nY, w;
  MNP_TRY(uminus(c, Y, i0, i0, nY));
  MNP_TRY(hmul(c, opH(A), opH(C), i0, i1, i1, w));        // A01 C11
  MNP_TRY(add_mul(c, opH(nY), opH(w), C, i0, i1, i0));    // C01 = -Y A01 C11
  HM w2;
  MNP_TRY(hmul(c, opH(A), opH(nY), i1, i0, i0, w2));      // -A10 Y
  return add_mul(c, opH(C), opH(w2), C, i1, i0, i1);      // C10 = -C11 A10 Y
}

// ---- solves of sub-matrices with a full leaf (lu.h:30-60)
mnpbem_status rsolve_ss(Ctx& c, const Sub& B, const Sub& A, int i, int j, char uplo, Sub& out) {
  if (B.flag == FLAG_FULL) {
    DMat m;
    MNP_TRY(trsm(c, 'R', mat_view(c, B, i, j), 'N', A, uplo, m));
    out = make_full(i, j, std::move(m));
  } else {
    DMat l, r;
    MNP_TRY(lhs_take(c, B, i, l));
    MNP_TRY(trsm(c, 'L', rhs_view(c, B, j), 'T', A, uplo, r));
    out = make_rk(i, j, std::move(l), std::move(r));
  }
  return MNPBEM_OK;
}
mnpbem_status lsolve_ss(Ctx& c, const Sub& B, const Sub& A, int i, int j, char uplo, Sub& out) {
  if (B.flag == FLAG_FULL) {
    DMat m;
    MNP_TRY(trsm(c, 'L', mat_view(c, B, i, j), 'N', A, uplo, m));
    out = make_full(i, j, std::move(m));
  } else {
    DMat l, r;
    MNP_TRY(trsm(c, 'L', lhs_view(c, B, i), 'N', A, uplo, l));
    MNP_TRY(rhs_take(c, B, j, r));
    out = make_rk(i, j, std::move(l), std::move(r));
  }
  return MNPBEM_OK;
}

// ---- a sub-matrix with an H-matrix factor (lu.h:66-113)
mnpbem_status rsolve_sh(Ctx& c, const Sub& B, const HM& A, int i, int j, char uplo, Sub& out) {
  if (T(c).admiss(j, j)) return rsolve_ss(c, B, at(A, Key(j, j)), i, j, uplo, out);
  const int first = uplo == 'U' ? 0 : 1, second = 1 - first;
  const int j0 = T(c).sons(j, first), j1 = T(c).sons(j, second);
  Sub X[2][2];
  MNP_TRY(rsolve_sh(c, B, A, i, j0, uplo, X[0][first]));
  Sub mb, prod, rhs;
  MNP_TRY(mask(c, B, i, j1, mb));
  MNP_TRY(add_mul2(c, opS(X[0][first]), opH(A), i, j1, j0, B.flag, prod));
  MNP_TRY(sub_minus(c, mb, prod, rhs));
  MNP_TRY(rsolve_sh(c, rhs, A, i, j1, uplo, X[0][second]));
  MNP_TRY(cat(c, X, 1, 2, i, j, out));
  return truncate(c, out);
}
mnpbem_status lsolve_sh(Ctx& c, const Sub& B, const HM& A, int i, int j, char uplo, Sub& out) {
  if (T(c).admiss(i, i)) return lsolve_ss(c, B, at(A, Key(i, i)), i, j, uplo, out);
  const int first = uplo == 'L' ? 0 : 1, second = 1 - first;
  const int i0 = T(c).sons(i, first), i1 = T(c).sons(i, second);
  Sub X[2][2];
  MNP_TRY(lsolve_sh(c, B, A, i0, j, uplo, X[first][0]));
  Sub mb, prod, rhs;
  MNP_TRY(mask(c, B, i1, j, mb));
  MNP_TRY(add_mul2(c, opH(A), opS(X[first][0]), i1, j, i0, B.flag, prod));
  MNP_TRY(sub_minus(c, mb, prod, rhs));
  MNP_TRY(lsolve_sh(c, rhs, A, i1, j, uplo, X[second][0]));
  MNP_TRY(cat(c, X, 2, 1, i, j, out));
  return truncate(c, out);
}

// ---- H-matrix solves (lu.h:118-176); B and X may be the same map
mnpbem_status rsolve_h(Ctx& c, const HM& B, const HM& A, HM& X, int i, int j, char uplo) {
  const Sub* pA = Op{&A, nullptr}.find(j, j);
  const Sub* pB = Op{&B, nullptr}.find(i, j);
  if (pA && pB) {
    Sub s;
    MNP_TRY(rsolve_ss(c, *pB, *pA, i, j, uplo, s));
    X[Key(i, j)] = std::move(s);
    return MNPBEM_OK;
  }
  int bi[2], bj[2];
  if (pA) {
    const int ni = T(c).begin(i, bi);
    for (int a = 0; a < ni; ++a) MNP_TRY(rsolve_h(c, B, A, X, bi[a], j, uplo));
    return MNPBEM_OK;
  }
  if (!pB) {
    const int ni = T(c).begin(i, bi), nj = T(c).begin(j, bj);
    if (uplo != 'U' && nj == 2) std::swap(bj[0], bj[1]);
    const int kf = T(c).sons(j, uplo == 'U' ? 0 : 1);
    for (int q = 0; q < nj; ++q)
      for (int a = 0; a < ni; ++a) {
        if (q == 0) {
          MNP_TRY(rsolve_h(c, B, A, X, bi[a], bj[q], uplo));
        } else {
          HM prod, Bn;
          MNP_TRY(hmul(c, opH(X), opH(A), bi[a], bj[q], kf, prod));
          MNP_TRY(subtract(c, B, prod, bi[a], bj[q], Bn));
          MNP_TRY(rsolve_h(c, Bn, A, X, bi[a], bj[q], uplo));
        }
      }
    return MNPBEM_OK;
  }
  Sub s;
  MNP_TRY(rsolve_sh(c, *pB, A, i, j, uplo, s));
  X[Key(i, j)] = std::move(s);
  return MNPBEM_OK;
}
mnpbem_status lsolve_h(Ctx& c, const HM& B, const HM& A, HM& X, int i, int j, char uplo) {
  const Sub* pA = Op{&A, nullptr}.find(i, i);
  const Sub* pB = Op{&B, nullptr}.find(i, j);
  if (pA && pB) {
    Sub s;
    MNP_TRY(lsolve_ss(c, *pB, *pA, i, j, uplo, s));
    X[Key(i, j)] = std::move(s);
    return MNPBEM_OK;
  }
  int bi[2], bj[2];
  if (pA) {
    const int nj = T(c).begin(j, bj);
    for (int b = 0; b < nj; ++b) MNP_TRY(lsolve_h(c, B, A, X, i, bj[b], uplo));
    return MNPBEM_OK;
  }
  if (!pB) {
    const int ni = T(c).begin(i, bi), nj = T(c).begin(j, bj);
    if (uplo != 'L' && ni == 2) std::swap(bi[0], bi[1]);
    const int kf = T(c).sons(i, uplo == 'L' ? 0 : 1);
    for (int q = 0; q < ni; ++q)
      for (int b = 0; b < nj; ++b) {
        if (q == 0) {
          MNP_TRY(lsolve_h(c, B, A, X, bi[q], bj[b], uplo));
        } else {
          HM prod, Bn;
          MNP_TRY(hmul(c, opH(A), opH(X), bi[q], bj[b], kf, prod));
          MNP_TRY(subtract(c, B, prod, bi[q], bj[b], Bn));
          MNP_TRY(lsolve_h(c, Bn, A, X, bi[q], bj[b], uplo));
        }
      }
    return MNPBEM_OK;
  }
  Sub s;
  MNP_TRY(lsolve_sh(c, *pB, A, i, j, uplo, s));
  X[Key(i, j)] = std::move(s);
  return MNPBEM_OK;
}

mnpbem_status lu_rec(Ctx& c, const HM& B, HM& A, int i) {
  if (T(c).leaf(i)) return lu_dense(c, at(B, Key(i, i)).mat, i, A[Key(i, i)]);
  const int i0 = T(c).sons(i, 0), i1 = T(c).sons(i, 1);
  MNP_TRY(lu_rec(c, B, A, i0));
  MNP_TRY(lsolve_h(c, B, A, A, i0, i1, 'L'));
  MNP_TRY(rsolve_h(c, B, A, A, i1, i0, 'U'));
  HM prod, S;
  MNP_TRY(hmul(c, opH(A), opH(A), i1, i1, i0, prod));
  MNP_TRY(subtract(c, B, prod, i1, i1, S));
  return lu_rec(c, S, A, i1);
}

// y[rows of r] += alpha S x[rows of col]  (x, y ld n, N columns)
mnpbem_status sub_apply(Ctx& c, const Sub& S, double2 alpha, const double2* x, double2* y, int N) {
  const int n = T(c).n;
  const View xv{x + T(c).lo[S.col], n, T(c).size(S.col), N};
  double2* yp = y + T(c).lo[S.row];
  if (S.flag == FLAG_FULL)
    return gemm(c, S.mat.m, N, S.mat.n, alpha, whole(S.mat), 0, xv, 0, ONE, yp, n);
  DMat t;
  MNP_TRY(mul(c, whole(S.rhs), 1, xv, 0, t));   // R^T x
  return gemm(c, S.lhs.m, N, S.lhs.n, alpha, whole(S.lhs), 0, whole(t), 0, ONE, yp, n);
}

mnpbem_status solve_vec(Ctx& c, const HM& A, double2* x, int N, int i, char uplo) {
  if (T(c).admiss(i, i)) {
    const Sub& D = at(A, Key(i, i));
    const DMat& Ti = uplo == 'L' ? D.linv : D.uinv;
    double2* xp = x + T(c).lo[i];
    const int n = T(c).n, m = T(c).size(i);
    if (!Ti.p) return trsm_left(c, D.mat, uplo, 'N', xp, n, N);
    DMat t;
    MNP_TRY(mul(c, whole(Ti), 0, View{xp, n, m, N}, 0, t));
    MNP_CUDA(cudaMemcpy2DAsync(xp, sizeof(double2) * n, t.ptr(), sizeof(double2) * m, sizeof(double2) * m, N,
                               cudaMemcpyDeviceToDevice, c.st));
    return MNPBEM_OK;
  }
  const int i0 = uplo == 'L' ? T(c).sons(i, 0) : T(c).sons(i, 1);
  const int i1 = uplo == 'L' ? T(c).sons(i, 1) : T(c).sons(i, 0);
  MNP_TRY(solve_vec(c, A, x, N, i0, uplo));
  std::vector<Key> ps;
  T(c).pairs(i1, i0, ps);
  for (const Key& p : ps) MNP_TRY(sub_apply(c, at(A, p), MONE, x, x, N));
  return solve_vec(c, A, x, N, i1, uplo);
}

}  // namespace

// ------------------------------------------------------ public operations
mnpbem_status h_lu(Ctx& c, const HM& B, HM& A) {
  A.clear();
  MNP_TRY(lu_rec(c, B, A, 0));
  return check_flags(c);
}

mnpbem_status h_rsolve_lu(Ctx& c, const HM& B, const HM& A, char key, HM& X) {
  X.clear();
  if (key == 'U' || key == 'N') MNP_TRY(rsolve_h(c, B, A, X, 0, 0, 'U'));
  if (key == 'L' || key == 'N') {
    const HM Bx = key == 'N' ? X : B;
    if (key == 'L') X.clear();
    MNP_TRY(rsolve_h(c, Bx, A, X, 0, 0, 'L'));
  }
  return check_flags(c);
}

mnpbem_status h_lsolve_lu(Ctx& c, const HM& B, const HM& A, char key, HM& X) {
  X.clear();
  if (key == 'L' || key == 'N') MNP_TRY(lsolve_h(c, B, A, X, 0, 0, 'L'));
  if (key == 'U' || key == 'N') {
    const HM Bx = key == 'N' ? X : B;
    if (key == 'U') X.clear();
    MNP_TRY(lsolve_h(c, Bx, A, X, 0, 0, 'U'));
  }
  return check_flags(c);
}

mnpbem_status h_mul(Ctx& c, const HM& A, const HM& B, HM& C) {
  MNP_TRY(hmul(c, opH(A), opH(B), 0, 0, 0, C));
  return check_flags(c);
}

mnpbem_status h_inv(Ctx& c, const HM& A, HM& C) {
  MNP_TRY(inv_rec(c, A, 0, C));
  return check_flags(c);
}

mnpbem_status h_add(Ctx& c, const HM& A, const HM& B, HM& C) {
  C.clear();
  return add_into(c, A, B, 0, 0, C);
}

mnpbem_status h_neg(Ctx& c, const HM& A, HM& C) { return uminus(c, A, 0, 0, C); }

mnpbem_status h_scale(Ctx& c, const HM& A, const double2* d, char side, HM& C) {
  C.clear();
  for (const auto& kv : A) {
    const Sub& S = kv.second;
    const int r = S.row, col = S.col;
    const double2* dv = d + T(c).lo[side == 'L' ? r : col];
    auto scaled = [&](const DMat& a, int rows, DMat& out) -> mnpbem_status {
      MNP_TRY(alloc(c, a.m, a.n, out));
      const int64_t cnt = (int64_t)a.m * a.n;
      if (cnt) {
        k_scale_rc<<<eblocks(cnt), 256, 0, c.st>>>(a.ptr(), out.ptr(), a.m, a.n, dv, rows);
        MNP_CHECK_LAUNCH();
      }
      return MNPBEM_OK;
    };
    Sub o;
    if (S.flag == FLAG_FULL) {
      DMat m;
      MNP_TRY(scaled(S.mat, side == 'L' ? 1 : 0, m));
      o = make_full(r, col, std::move(m));
    } else if (side == 'L') {
      DMat l;
      MNP_TRY(scaled(S.lhs, 1, l));
      o = make_rk(r, col, std::move(l), S.rhs);
    } else {
      DMat rr;
      MNP_TRY(scaled(S.rhs, 1, rr));
      o = make_rk(r, col, S.lhs, std::move(rr));
    }
    C[kv.first] = std::move(o);
  }
  return MNPBEM_OK;
}

mnpbem_status h_solve(Ctx& c, const HM& A, char key, double2* x, int N) {
  if (N <= 0) return MNPBEM_OK;
  if (key == 'L' || key == 'N') MNP_TRY(solve_vec(c, A, x, N, 0, 'L'));
  if (key == 'U' || key == 'N') MNP_TRY(solve_vec(c, A, x, N, 0, 'U'));
  return MNPBEM_OK;
}

mnpbem_status h_matvec(Ctx& c, const HM& A, const double2* x, double2* y, int N, bool acc) {
  if (N <= 0) return MNPBEM_OK;
  if (!acc) MNP_CUDA(cudaMemsetAsync(y, 0, sizeof(double2) * (size_t)T(c).n * N, c.st));
  for (const auto& kv : A) MNP_TRY(sub_apply(c, kv.second, ONE, x, y, N));
  return MNPBEM_OK;
}

mnpbem_status h_full(Ctx& c, const HM& A, double2* out) {
  const int n = T(c).n;
  for (const auto& kv : A) {
    const Sub& S = kv.second;
    double2* o = out + T(c).lo[S.row] + (int64_t)T(c).lo[S.col] * n;
    if (S.flag == FLAG_FULL) {
      if (S.mat.m > 0 && S.mat.n > 0)
        MNP_CUDA(cudaMemcpy2DAsync(o, sizeof(double2) * n, S.mat.ptr(), sizeof(double2) * S.mat.m,
                                   sizeof(double2) * S.mat.m, S.mat.n, cudaMemcpyDeviceToDevice, c.st));
    } else {
      MNP_TRY(gemm(c, S.lhs.m, S.rhs.m, S.lhs.n, ONE, whole(S.lhs), 0, whole(S.rhs), 1, ZERO, o, n));
    }
  }
  return MNPBEM_OK;
}

// ------------------------------------------------------ preconditioner
namespace {

__global__ void k_gather(const double2* src, const int* perm, int n, double2* dst) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) dst[c] = src[perm[c]];
}
__global__ void k_gather_nvec(const double* nv, const int* perm, int n, double2* dst) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) dst[c + (int64_t)d * n] = make_double2(nv[3 * (int64_t)perm[c] + d], 0.0);
}
// v[c] = s (e1[c] - e2[c]) (s complex)
__global__ void k_deps(const double2* e1, const double2* e2, double2 s, int n, double2* v) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    v[c] = cmul(s, csub(e1[c], e2[c]));
}
// b-space (face order) -> cluster order, column-major: PHI [n][P], A3 [n][3P]
// (column d P + p), AL [n][3P], DE [n][P]
__global__ void k_pc_in(int n, int P, const int* perm, const double2* phi, const double2* a, const double2* al,
                        const double2* De, double2* PHI, double2* A3, double2* AL, double2* DE) {
  const int64_t cnt = (int64_t)n * 4 * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % n), q = (int)(e / n);
    const int64_t f = perm[c];
    if (q < P) {
      PHI[c + (int64_t)q * n] = phi[f * P + q];
      DE[c + (int64_t)q * n] = De[f * P + q];
    } else {
      const int v = q - P;   // d P + p
      A3[c + (int64_t)v * n] = a[f * 3 * P + v];
      AL[c + (int64_t)v * n] = al[f * 3 * P + v];
    }
  }
}
// mfun.m:37-38: AL' = AL - T1 + ik nvec eps1 PHI;  DE' = DE - eps1 T2 + ik eps1 (nvec . A3)
__global__ void k_pc_mod(int n, int P, double2 ik, const double2* nv, const double2* e1, const double2* PHI,
                         const double2* A3, const double2* T1, const double2* T2, double2* AL, double2* DE) {
  const int64_t cnt = (int64_t)n * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % n), p = (int)(e / n);
    const double2 ep = e1[c], ph = PHI[c + (int64_t)p * n];
    double2 inn = make_double2(0.0, 0.0);
    for (int d = 0; d < 3; ++d) {
      const int64_t o = c + (int64_t)(d * P + p) * n;
      const double2 nd = nv[c + (int64_t)d * n];
      AL[o] = cadd(csub(AL[o], T1[o]), cmul(cmul(ik, nd), cmul(ep, ph)));
      inn = cadd(inn, cmul(nd, A3[o]));
    }
    const int64_t o = c + (int64_t)p * n;
    DE[o] = cadd(csub(DE[o], cmul(ep, T2[o])), cmul(cmul(ik, ep), inn));
  }
}
// rhs = DE' + ik (e1 - e2) (nvec . T3)
__global__ void k_pc_rhs(int n, int P, double2 ik, const double2* nv, const double2* e1, const double2* e2,
                         const double2* DE, const double2* T3, double2* out) {
  const int64_t cnt = (int64_t)n * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % n), p = (int)(e / n);
    double2 inn = make_double2(0.0, 0.0);
    for (int d = 0; d < 3; ++d) inn = cadd(inn, cmul(nv[c + (int64_t)d * n], T3[c + (int64_t)(d * P + p) * n]));
    out[e] = cadd(DE[e], cmul(cmul(ik, csub(e1[c], e2[c])), inn));
  }
}
// out = ik nvec (e1 - e2) sig2 + AL'
__global__ void k_pc_h2in(int n, int P, double2 ik, const double2* nv, const double2* e1, const double2* e2,
                          const double2* S2, const double2* AL, double2* out) {
  const int64_t cnt = (int64_t)n * 3 * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % n), v = (int)(e / n), d = v / P, p = v % P;
    const double2 s = cmul(cmul(ik, nv[c + (int64_t)d * n]), cmul(csub(e1[c], e2[c]), S2[c + (int64_t)p * n]));
    out[e] = cadd(s, AL[e]);
  }
}
// x-space (face order): [n][4P] (S | H) at dst, [n][4P] (S2 | H2) at dst + 4 n P
__global__ void k_pc_out(int n, int P, const int* perm, const double2* S1, const double2* H1, const double2* S2,
                         const double2* H2, double2* dst) {
  const int64_t cnt = (int64_t)n * 4 * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % n), q = (int)(e / n);
    const int64_t f = perm[c], o = f * 4 * P + q;
    if (q < P) {
      dst[o] = S1[c + (int64_t)q * n];
      dst[(int64_t)n * 4 * P + o] = S2[c + (int64_t)q * n];
    } else {
      dst[o] = H1[c + (int64_t)(q - P) * n];
      dst[(int64_t)n * 4 * P + o] = H2[c + (int64_t)(q - P) * n];
    }
  }
}

}  // namespace

mnpbem_status precond_build(std::shared_ptr<Ctx> cp, HM& G1, HM& H1, HM& G2, HM& H2, double k,
                            const double2* eps1_f, const double2* eps2_f, const double* nvec_f, HPrecond& out) {
  Ctx& c = *cp;
  const int n = T(c).n;
  out.c = cp;
  out.k = make_double2(k, 0.0);
  MNP_TRY(alloc_raw(c, sizeof(int) * n, out.perm));
  int* perm = static_cast<int*>(out.perm.get());
  MNP_CUDA(cudaMemcpyAsync(perm, T(c).perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c.st));
  MNP_TRY(alloc(c, n, 1, out.eps1));
  MNP_TRY(alloc(c, n, 1, out.eps2));
  MNP_TRY(alloc(c, n, 3, out.nvec));
  const unsigned nb = eblocks(n);
  k_gather<<<nb, 256, 0, c.st>>>(eps1_f, perm, n, out.eps1.ptr());
  k_gather<<<nb, 256, 0, c.st>>>(eps2_f, perm, n, out.eps2.ptr());
  k_gather_nvec<<<nb, 256, 0, c.st>>>(nvec_f, perm, n, out.nvec.ptr());
  MNP_CHECK_LAUNCH();
  // initprecond.m:29-50
  MNP_TRY(h_lu(c, G1, out.G1i));
  G1.clear();
  MNP_TRY(h_lu(c, G2, out.G2i));
  G2.clear();
  MNP_TRY(h_rsolve_lu(c, H1, out.G1i, 'N', out.Sigma1));
  H1.clear();
  HM Sigma2;
  MNP_TRY(h_rsolve_lu(c, H2, out.G2i, 'N', Sigma2));
  H2.clear();
  HM nS2, D;
  MNP_TRY(h_neg(c, Sigma2, nS2));
  MNP_TRY(h_add(c, out.Sigma1, nS2, D));
  MNP_TRY(h_inv(c, D, out.Deltai));
  D.clear();
  // fun(Deltai, nvec) = sum_d diag(n_d) Deltai diag(n_d)
  HM F;
  for (int d = 0; d < 3; ++d) {
    HM a, b;
    const double2* nd = out.nvec.ptr() + (int64_t)d * n;
    MNP_TRY(h_scale(c, out.Deltai, nd, 'L', a));
    MNP_TRY(h_scale(c, a, nd, 'R', b));
    if (d == 0) F = std::move(b);
    else {
      HM s;
      MNP_TRY(h_add(c, F, b, s));
      F = std::move(s);
    }
  }
  // Sigma = eps1 Sigma1 - eps2 Sigma2 + k^2 deps F deps
  DMat deps, k2deps;
  MNP_TRY(alloc(c, n, 1, deps));
  MNP_TRY(alloc(c, n, 1, k2deps));
  k_deps<<<nb, 256, 0, c.st>>>(out.eps1.ptr(), out.eps2.ptr(), make_double2(1.0, 0.0), n, deps.ptr());
  k_deps<<<nb, 256, 0, c.st>>>(out.eps1.ptr(), out.eps2.ptr(), make_double2(k * k, 0.0), n, k2deps.ptr());
  MNP_CHECK_LAUNCH();
  HM a1, a2, na2, s1, f1, f2, S;
  MNP_TRY(h_scale(c, out.Sigma1, out.eps1.ptr(), 'L', a1));
  MNP_TRY(h_scale(c, Sigma2, out.eps2.ptr(), 'L', a2));
  MNP_TRY(h_neg(c, a2, na2));
  MNP_TRY(h_add(c, a1, na2, s1));
  MNP_TRY(h_scale(c, F, k2deps.ptr(), 'L', f1));
  MNP_TRY(h_scale(c, f1, deps.ptr(), 'R', f2));
  MNP_TRY(h_add(c, s1, f2, S));
  MNP_TRY(h_lu(c, S, out.Sigmai));
  return check_flags(c);
}

mnpbem_status precond_apply(HPrecond& h, int P, const double2* phi, const double2* a, const double2* alpha,
                            const double2* De, double2* dst) {
  Ctx& c = *h.c;
  const int n = T(c).n;
  const int64_t sP = (int64_t)n * P;
  // PHI, A3, AL, DE, T1 (3P), T2 (P), rhs (P), buffer (3P)
  const int64_t need = sP * (1 + 3 + 3 + 1 + 3 + 1 + 1 + 3);
  if (!h.work.p || (int64_t)h.work.m * h.work.n < need) MNP_TRY(alloc(c, (int)need, 1, h.work));
  double2* w = h.work.ptr();
  double2 *PHI = w, *A3 = PHI + sP, *AL = A3 + 3 * sP, *DE = AL + 3 * sP, *T1 = DE + sP, *T2 = T1 + 3 * sP,
          *RHS = T2 + sP, *BUF = RHS + sP;
  const int* perm = static_cast<const int*>(h.perm.get());
  const unsigned nb = eblocks((int64_t)n * 4 * P);
  k_pc_in<<<nb, 256, 0, c.st>>>(n, P, perm, phi, a, alpha, De, PHI, A3, AL, DE);
  MNP_CHECK_LAUNCH();
  const double2 ik = make_double2(0.0, h.k.x);
  const double2* nv = h.nvec.ptr();
  const double2 *e1 = h.eps1.ptr(), *e2 = h.eps2.ptr();
  MNP_TRY(h_matvec(c, h.Sigma1, A3, T1, 3 * P, false));
  MNP_TRY(h_matvec(c, h.Sigma1, PHI, T2, P, false));
  k_pc_mod<<<eblocks(sP), 256, 0, c.st>>>(n, P, ik, nv, e1, PHI, A3, T1, T2, AL, DE);
  MNP_CHECK_LAUNCH();
  MNP_TRY(h_matvec(c, h.Deltai, AL, T1, 3 * P, false));
  k_pc_rhs<<<eblocks(sP), 256, 0, c.st>>>(n, P, ik, nv, e1, e2, DE, T1, RHS);
  MNP_CHECK_LAUNCH();
  MNP_TRY(h_solve(c, h.Sigmai, 'N', RHS, P));                 // sig2
  k_pc_h2in<<<eblocks(3 * sP), 256, 0, c.st>>>(n, P, ik, nv, e1, e2, RHS, AL, BUF);
  MNP_CHECK_LAUNCH();
  MNP_TRY(h_matvec(c, h.Deltai, BUF, T1, 3 * P, false));      // h2
  // sig1 = G1i \ (sig2 + phi) -> PHI;  h1 = G1i \ (h2 + a) -> A3
  k_add2<<<eblocks(sP), 256, 0, c.st>>>(RHS, PHI, PHI, sP, 1.0);
  k_add2<<<eblocks(3 * sP), 256, 0, c.st>>>(T1, A3, A3, 3 * sP, 1.0);
  MNP_CHECK_LAUNCH();
  MNP_TRY(h_solve(c, h.G1i, 'N', PHI, P));
  MNP_TRY(h_solve(c, h.G1i, 'N', A3, 3 * P));
  MNP_TRY(h_solve(c, h.G2i, 'N', RHS, P));
  MNP_TRY(h_solve(c, h.G2i, 'N', T1, 3 * P));
  k_pc_out<<<nb, 256, 0, c.st>>>(n, P, perm, PHI, A3, RHS, T1, dst);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

}  // namespace hl
}  // namespace mnpbem

// ------------------------------------------------------ tree from the C ABI
namespace mnpbem {
namespace hl {

mnpbem_status tree_from_abi(const mnpbem_cluster_tree* t, std::shared_ptr<Tree>& out) {
  auto bad = [](const char* why) {
    set_error("H-matrix: cluster tree %s", why);
    return MNPBEM_ERR_INVALID_ARG;
  };
  if (!t || t->ncluster < 1 || !t->son || !t->cind || !t->perm || t->nfull < 1 || !t->full || t->nlow < 0 ||
      (t->nlow > 0 && !t->low))
    return bad("arrays missing");
  auto T = std::make_shared<Tree>();
  const int nc = t->ncluster;
  T->son0.resize(nc); T->son1.resize(nc); T->lo.resize(nc); T->hi.resize(nc);
  for (int i = 0; i < nc; ++i) {
    T->son0[i] = t->son[2 * i];
    T->son1[i] = t->son[2 * i + 1];
    T->lo[i] = t->cind[2 * i];
    T->hi[i] = t->cind[2 * i + 1] + 1;
    if (T->son0[i] < -1 || T->son0[i] >= nc || T->son1[i] < -1 || T->son1[i] >= nc || (T->son0[i] < 0) != (T->son1[i] < 0))
      return bad("son index out of range");
    if (T->lo[i] < 0 || T->hi[i] <= T->lo[i]) return bad("cluster range invalid");
  }
  T->n = T->hi[0];
  if (T->lo[0] != 0) return bad("root does not start at 0");
  for (int i = 0; i < nc; ++i)
    if (T->son0[i] >= 0) {
      const int a = T->son0[i], b = T->son1[i];
      if (T->lo[a] != T->lo[i] || T->hi[a] != T->lo[b] || T->hi[b] != T->hi[i]) return bad("sons do not split their cluster");
    }
  T->perm.assign(t->perm, t->perm + T->n);
  std::vector<char> seen(T->n, 0);
  for (int f : T->perm) {
    if (f < 0 || f >= T->n || seen[f]) return bad("perm is not a permutation");
    seen[f] = 1;
  }
  double area = 0.0;
  auto add_block = [&](int r, int c, int flag) -> bool {
    if (r < 0 || r >= nc || c < 0 || c >= nc) return false;
    if (!T->ad.emplace(Key(r, c), flag).second) return false;
    area += (double)(T->hi[r] - T->lo[r]) * (T->hi[c] - T->lo[c]);
    return true;
  };
  for (int b = 0; b < t->nfull; ++b) {
    const int r = t->full[2 * b], c = t->full[2 * b + 1];
    if (!add_block(r, c, FLAG_FULL)) return bad("full block invalid or repeated");
    if (r >= 0 && (T->son0[r] >= 0 || T->son0[c] >= 0)) return bad("full blocks must be leaf pairs");
    if (T->hi[r] - T->lo[r] > HL_LEAF_MAX || T->hi[c] - T->lo[c] > HL_LEAF_MAX) return bad("leaf larger than 1024");
    T->full.emplace_back(r, c);
  }
  for (int b = 0; b < t->nlow; ++b) {
    const int r = t->low[2 * b], c = t->low[2 * b + 1];
    if (!add_block(r, c, FLAG_RK)) return bad("low-rank block invalid or repeated");
    T->low.emplace_back(r, c);
  }
  if (area != (double)T->n * T->n) return bad("blocks do not partition the matrix");
  // every leaf pair the recursion reaches must be a block: walk the tree
  std::vector<Key> ps;
  T->pairs(0, 0, ps);
  if (ps.size() != T->ad.size()) return bad("blocks do not match the cluster tree");
  for (int i = 0; i < nc; ++i)
    if (T->son0[i] < 0 && T->admiss(i, i) != FLAG_FULL) return bad("a diagonal leaf block is not full");
  out = std::move(T);
  return MNPBEM_OK;
}

}  // namespace hl
}  // namespace mnpbem

// ====================================================================== C ABI
// Opaque H-matrix of the C ABI: the blocks and the options (htol, kmax) of
// one cluster tree, the arguments the reference's H-matrix MEX functions take
// (mex/hmatlu.cpp, hmatrsolve.cpp, hmatinv.cpp, hmatadd.cpp, hmatsolve.cpp).
struct mnpbem_hm_s {
  std::shared_ptr<mnpbem::hl::Ctx> c;
  mnpbem::hl::HM m;
};

namespace {
using namespace mnpbem;
using namespace mnpbem::hl;

bool same_tree(const Tree& a, const Tree& b) {
  return a.son0 == b.son0 && a.son1 == b.son1 && a.lo == b.lo && a.hi == b.hi && a.ad == b.ad;
}

mnpbem_status hm_check(const mnpbem_hm* h, const char* who) {
  if (!h || !h->c) {
    set_error("%s: invalid H-matrix handle", who);
    return MNPBEM_ERR_INVALID_ARG;
  }
  return MNPBEM_OK;
}

mnpbem_status hm_new(const mnpbem_hm* like, mnpbem_hm** out) {
  if (!out) {
    set_error("H-matrix: output handle is NULL");
    return MNPBEM_ERR_INVALID_ARG;
  }
  auto* h = new (std::nothrow) mnpbem_hm();
  if (!h) return MNPBEM_ERR_OUT_OF_MEMORY;
  mnpbem_status s = ctx_make(like->c->device, like->c->t, like->c->tol, like->c->kmax, h->c);
  if (s != MNPBEM_OK) {
    delete h;
    return s;
  }
  *out = h;
  return MNPBEM_OK;
}

struct DevGuard {
  int prev = -1;
  explicit DevGuard(int d) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(d);
  }
  ~DevGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// run op into a new handle; free it on failure
template <typename F>
mnpbem_status hm_result(const mnpbem_hm* like, mnpbem_hm** out, F op) {
  mnpbem_hm* h = nullptr;
  MNP_TRY(hm_new(like, &h));
  DevGuard g(like->c->device);
  mnpbem_status s = op(*h->c, h->m);
  if (s == MNPBEM_OK) s = check_flags(*h->c);
  if (s != MNPBEM_OK) {
    delete h;
    return s;
  }
  *out = h;
  return MNPBEM_OK;
}

}  // namespace

extern "C" {

MNPBEM_API mnpbem_status mnpbem_hm_create(int32_t device, const mnpbem_cluster_tree* tree, double htol, int32_t kmax,
                                          const double* vals, const int32_t* ranks, const double* lhs,
                                          const double* rhs, mnpbem_hm** out) {
  if (!out || !vals || !(htol > 0) || kmax < 1 || (tree && tree->nlow > 0 && (!ranks || !lhs || !rhs))) {
    set_error("mnpbem_hm_create: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  *out = nullptr;
  int ndev = 0;
  MNP_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) {
    set_error("mnpbem_hm_create: device %d not present", device);
    return MNPBEM_ERR_INVALID_ARG;
  }
  std::shared_ptr<Tree> T;
  MNP_TRY(tree_from_abi(tree, T));
  for (int b = 0; b < tree->nlow; ++b) {
    const int r = tree->low[2 * b], c = tree->low[2 * b + 1];
    if (ranks[b] < 0 || ranks[b] > std::min(T->size(r), T->size(c)) + 4096) {
      set_error("mnpbem_hm_create: rank of low-rank block %d out of range", b);
      return MNPBEM_ERR_INVALID_ARG;
    }
  }
  DevGuard g(device);
  auto* h = new (std::nothrow) mnpbem_hm();
  if (!h) return MNPBEM_ERR_OUT_OF_MEMORY;
  mnpbem_status s = ctx_make(device, T, htol, kmax, h->c);
  const double2* v = reinterpret_cast<const double2*>(vals);
  const double2* l = reinterpret_cast<const double2*>(lhs);
  const double2* rr = reinterpret_cast<const double2*>(rhs);
  for (size_t b = 0; s == MNPBEM_OK && b < T->full.size(); ++b) {
    const Key k = T->full[b];
    const int m = T->size(k.first), n = T->size(k.second);
    Sub S;
    S.row = k.first; S.col = k.second; S.flag = FLAG_FULL;
    s = upload(*h->c, v, m, n, S.mat);
    v += (int64_t)m * n;
    h->m[k] = std::move(S);
  }
  for (size_t b = 0; s == MNPBEM_OK && b < T->low.size(); ++b) {
    const Key k = T->low[b];
    const int m = T->size(k.first), n = T->size(k.second), r = ranks[b];
    Sub S;
    S.row = k.first; S.col = k.second; S.flag = FLAG_RK;
    s = upload(*h->c, l, m, r, S.lhs);
    if (s == MNPBEM_OK) s = upload(*h->c, rr, n, r, S.rhs);
    l += (int64_t)m * r;
    rr += (int64_t)n * r;
    h->m[k] = std::move(S);
  }
  if (s == MNPBEM_OK) s = check_flags(*h->c);
  if (s != MNPBEM_OK) {
    delete h;
    return s;
  }
  *out = h;
  return MNPBEM_OK;
}

MNPBEM_API mnpbem_status mnpbem_hm_set_options(mnpbem_hm* h, double htol, int32_t kmax) {
  MNP_TRY(hm_check(h, "mnpbem_hm_set_options"));
  if (!(htol > 0) || kmax < 1) {
    set_error("mnpbem_hm_set_options: htol must be > 0 and kmax >= 1");
    return MNPBEM_ERR_INVALID_ARG;
  }
  h->c->tol = htol;
  h->c->kmax = kmax;
  return MNPBEM_OK;
}

MNPBEM_API mnpbem_status mnpbem_hm_lu(const mnpbem_hm* a, mnpbem_hm** out) {
  MNP_TRY(hm_check(a, "mnpbem_hm_lu"));
  return hm_result(a, out, [&](Ctx& c, HM& r) { return h_lu(c, a->m, r); });
}

MNPBEM_API mnpbem_status mnpbem_hm_rsolve(const mnpbem_hm* b, const mnpbem_hm* lu, char key, mnpbem_hm** out) {
  MNP_TRY(hm_check(b, "mnpbem_hm_rsolve"));
  MNP_TRY(hm_check(lu, "mnpbem_hm_rsolve"));
  if ((key != 'N' && key != 'L' && key != 'U') || !same_tree(*b->c->t, *lu->c->t) || b->c->device != lu->c->device) {
    set_error("mnpbem_hm_rsolve: key must be 'N', 'L' or 'U' and both H-matrices on one tree and device");
    return MNPBEM_ERR_INVALID_ARG;
  }
  return hm_result(b, out, [&](Ctx& c, HM& r) { return h_rsolve_lu(c, b->m, lu->m, key, r); });
}

MNPBEM_API mnpbem_status mnpbem_hm_lsolve(const mnpbem_hm* b, const mnpbem_hm* lu, char key, mnpbem_hm** out) {
  MNP_TRY(hm_check(b, "mnpbem_hm_lsolve"));
  MNP_TRY(hm_check(lu, "mnpbem_hm_lsolve"));
  if ((key != 'N' && key != 'L' && key != 'U') || !same_tree(*b->c->t, *lu->c->t) || b->c->device != lu->c->device) {
    set_error("mnpbem_hm_lsolve: key must be 'N', 'L' or 'U' and both H-matrices on one tree and device");
    return MNPBEM_ERR_INVALID_ARG;
  }
  return hm_result(b, out, [&](Ctx& c, HM& r) { return h_lsolve_lu(c, b->m, lu->m, key, r); });
}

MNPBEM_API mnpbem_status mnpbem_hm_matmul(const mnpbem_hm* a, const mnpbem_hm* b, mnpbem_hm** out) {
  MNP_TRY(hm_check(a, "mnpbem_hm_matmul"));
  MNP_TRY(hm_check(b, "mnpbem_hm_matmul"));
  if (!same_tree(*a->c->t, *b->c->t) || a->c->device != b->c->device) {
    set_error("mnpbem_hm_matmul: both H-matrices must be on one tree and device");
    return MNPBEM_ERR_INVALID_ARG;
  }
  return hm_result(a, out, [&](Ctx& c, HM& r) { return h_mul(c, a->m, b->m, r); });
}

MNPBEM_API mnpbem_status mnpbem_hm_inv(const mnpbem_hm* a, mnpbem_hm** out) {
  MNP_TRY(hm_check(a, "mnpbem_hm_inv"));
  return hm_result(a, out, [&](Ctx& c, HM& r) { return h_inv(c, a->m, r); });
}

MNPBEM_API mnpbem_status mnpbem_hm_add(const mnpbem_hm* a, const mnpbem_hm* b, double sign, mnpbem_hm** out) {
  MNP_TRY(hm_check(a, "mnpbem_hm_add"));
  MNP_TRY(hm_check(b, "mnpbem_hm_add"));
  if ((sign != 1.0 && sign != -1.0) || !same_tree(*a->c->t, *b->c->t) || a->c->device != b->c->device) {
    set_error("mnpbem_hm_add: sign must be 1 or -1 and both H-matrices on one tree and device");
    return MNPBEM_ERR_INVALID_ARG;
  }
  return hm_result(a, out, [&](Ctx& c, HM& r) -> mnpbem_status {
    if (sign > 0) return h_add(c, a->m, b->m, r);
    HM nb;
    MNP_TRY(h_neg(c, b->m, nb));
    return h_add(c, a->m, nb, r);
  });
}

MNPBEM_API mnpbem_status mnpbem_hm_scale(const mnpbem_hm* a, const double* d, char side, mnpbem_hm** out) {
  MNP_TRY(hm_check(a, "mnpbem_hm_scale"));
  if (!d || (side != 'L' && side != 'R')) {
    set_error("mnpbem_hm_scale: d missing or side not 'L' / 'R'");
    return MNPBEM_ERR_INVALID_ARG;
  }
  return hm_result(a, out, [&](Ctx& c, HM& r) -> mnpbem_status {
    DMat dv;
    MNP_TRY(upload(c, reinterpret_cast<const double2*>(d), c.t->n, 1, dv));
    return h_scale(c, a->m, dv.ptr(), side, r);
  });
}

MNPBEM_API mnpbem_status mnpbem_hm_solve(const mnpbem_hm* lu, char key, double* x, int32_t N) {
  MNP_TRY(hm_check(lu, "mnpbem_hm_solve"));
  if (!x || N < 1 || (key != 'N' && key != 'L' && key != 'U')) {
    set_error("mnpbem_hm_solve: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  Ctx& c = *lu->c;
  DevGuard g(c.device);
  DMat xv;
  MNP_TRY(upload(c, reinterpret_cast<const double2*>(x), c.t->n, N, xv));
  MNP_TRY(h_solve(c, lu->m, key, xv.ptr(), N));
  MNP_CUDA(cudaMemcpyAsync(x, xv.ptr(), sizeof(double2) * (size_t)c.t->n * N, cudaMemcpyDeviceToHost, c.st));
  return check_flags(c);
}

MNPBEM_API mnpbem_status mnpbem_hm_mul(const mnpbem_hm* a, const double* x, double* y, int32_t N) {
  MNP_TRY(hm_check(a, "mnpbem_hm_mul"));
  if (!x || !y || N < 1) {
    set_error("mnpbem_hm_mul: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  Ctx& c = *a->c;
  DevGuard g(c.device);
  DMat xv, yv;
  MNP_TRY(upload(c, reinterpret_cast<const double2*>(x), c.t->n, N, xv));
  MNP_TRY(alloc(c, c.t->n, N, yv));
  MNP_TRY(h_matvec(c, a->m, xv.ptr(), yv.ptr(), N, false));
  MNP_CUDA(cudaMemcpyAsync(y, yv.ptr(), sizeof(double2) * (size_t)c.t->n * N, cudaMemcpyDeviceToHost, c.st));
  return check_flags(c);
}

MNPBEM_API mnpbem_status mnpbem_hm_full(const mnpbem_hm* a, double* out) {
  MNP_TRY(hm_check(a, "mnpbem_hm_full"));
  if (!out) {
    set_error("mnpbem_hm_full: out is NULL");
    return MNPBEM_ERR_INVALID_ARG;
  }
  Ctx& c = *a->c;
  DevGuard g(c.device);
  const int n = c.t->n;
  DMat f;
  MNP_TRY(alloc(c, n, n, f));
  MNP_TRY(h_full(c, a->m, f.ptr()));
  MNP_CUDA(cudaMemcpyAsync(out, f.ptr(), sizeof(double2) * (size_t)n * n, cudaMemcpyDeviceToHost, c.st));
  return check_flags(c);
}

MNPBEM_API mnpbem_status mnpbem_hm_sizes(const mnpbem_hm* a, int64_t* nvals, int64_t* nlhs, int64_t* nrhs) {
  MNP_TRY(hm_check(a, "mnpbem_hm_sizes"));
  const Tree& T = *a->c->t;
  int64_t v = 0, l = 0, r = 0;
  for (const Key& k : T.full) v += (int64_t)T.size(k.first) * T.size(k.second);
  for (const Key& k : T.low) {
    auto it = a->m.find(k);
    if (it == a->m.end() || it->second.flag != FLAG_RK) {
      set_error("mnpbem_hm_sizes: block (%d, %d) is not low-rank", k.first, k.second);
      return MNPBEM_ERR_INVALID_ARG;
    }
    l += (int64_t)it->second.lhs.m * it->second.rank();
    r += (int64_t)it->second.rhs.m * it->second.rank();
  }
  if (nvals) *nvals = v;
  if (nlhs) *nlhs = l;
  if (nrhs) *nrhs = r;
  return MNPBEM_OK;
}

MNPBEM_API mnpbem_status mnpbem_hm_export(const mnpbem_hm* a, double* vals, int32_t* ranks, double* lhs,
                                          double* rhs) {
  MNP_TRY(hm_check(a, "mnpbem_hm_export"));
  const Tree& T = *a->c->t;
  Ctx& c = *a->c;
  DevGuard g(c.device);
  double2* v = reinterpret_cast<double2*>(vals);
  double2* l = reinterpret_cast<double2*>(lhs);
  double2* r = reinterpret_cast<double2*>(rhs);
  for (size_t b = 0; b < T.full.size(); ++b) {
    auto it = a->m.find(T.full[b]);
    if (it == a->m.end() || it->second.flag != FLAG_FULL) {
      set_error("mnpbem_hm_export: block (%d, %d) is not full", T.full[b].first, T.full[b].second);
      return MNPBEM_ERR_INVALID_ARG;
    }
    const DMat& M = it->second.mat;
    if (vals) MNP_CUDA(cudaMemcpyAsync(v, M.ptr(), sizeof(double2) * M.m * M.n, cudaMemcpyDeviceToHost, c.st));
    v += (int64_t)M.m * M.n;
  }
  for (size_t b = 0; b < T.low.size(); ++b) {
    auto it = a->m.find(T.low[b]);
    if (it == a->m.end() || it->second.flag != FLAG_RK) {
      set_error("mnpbem_hm_export: block (%d, %d) is not low-rank", T.low[b].first, T.low[b].second);
      return MNPBEM_ERR_INVALID_ARG;
    }
    const Sub& S = it->second;
    const int k = S.rank();
    if (ranks) ranks[b] = k;
    if (lhs && k) MNP_CUDA(cudaMemcpyAsync(l, S.lhs.ptr(), sizeof(double2) * S.lhs.m * k, cudaMemcpyDeviceToHost, c.st));
    if (rhs && k) MNP_CUDA(cudaMemcpyAsync(r, S.rhs.ptr(), sizeof(double2) * S.rhs.m * k, cudaMemcpyDeviceToHost, c.st));
    l += (int64_t)S.lhs.m * k;
    r += (int64_t)S.rhs.m * k;
  }
  return check_flags(c);
}

MNPBEM_API void mnpbem_hm_free(mnpbem_hm* h) {
  if (!h) return;
  DevGuard g(h->c ? h->c->device : 0);
  delete h;
}

}  // extern "C"
