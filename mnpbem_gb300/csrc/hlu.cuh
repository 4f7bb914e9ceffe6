// H-matrix arithmetic on the GPU: LU, triangular solves, inversion and
// addition of hierarchical matrices with low-rank blocks truncated by ACA,
// as MNPBEM's hlib does on the CPU (mex/hlib/lu.h, hmatrix.h, submatrix.h,
// aca.cpp, lu.cpp).  The recursion over the cluster tree runs on the host;
// every numeric step (products, leaf LU and inverses, triangular solves, ACA,
// copies) is a kernel on one stream, with matrices in a stream-ordered pool.
// The 'hmat' preconditioner of the iterative solver is built from these
// (BEM/@bemretiter/private/initprecond.m, mfun.m).
#pragma once
#include <map>
#include <memory>
#include <mutex>
#include <utility>
#include <vector>

#include "common.cuh"

namespace mnpbem {
namespace hl {

constexpr int FLAG_RK = 1, FLAG_FULL = 2;   // clustertree.h flagRk / flagFull
constexpr int HL_LEAF_MAX = 1024;           // largest leaf cluster (inverse, LU)

// column-major complex128 matrix on the device, leading dimension m
struct DMat {
  std::shared_ptr<double2> p;
  int m = 0, n = 0;
  double2* ptr() const { return p.get(); }
};

// block of cluster pair (row, col): full (mat) or low-rank (lhs rhs^T)
struct Sub {
  int row = -1, col = -1, flag = 0;
  DMat mat, lhs, rhs;
  DMat linv, uinv;   // diagonal leaf of an LU: inverses of its L and U factors
  int rank() const { return lhs.n; }
};
using Key = std::pair<int, int>;
using HM = std::map<Key, Sub>;

// cluster tree with the admissibility of its leaf blocks (clustertree.h)
struct Tree {
  std::vector<int> son0, son1, lo, hi;   // hi: one past the last position
  std::map<Key, int> ad;                 // FLAG_FULL / FLAG_RK of the leaf blocks
  std::vector<int> perm;                 // face at each cluster position
  std::vector<Key> full, low;            // leaf blocks in the order given
  int n = 0;
  bool leaf(int i) const { return son0[i] < 0; }
  int sons(int i, int s) const { return s ? son1[i] : son0[i]; }
  int size(int i) const { return hi[i] - lo[i]; }
  int admiss(int r, int c) const {
    auto it = ad.find(Key(r, c));
    return it == ad.end() ? 0 : it->second;
  }
  // sons of i in order, or i itself for a leaf
  int begin(int i, int* out) const {
    if (leaf(i)) { out[0] = i; return 1; }
    out[0] = son0[i]; out[1] = son1[i];
    return 2;
  }
  // leaf blocks below (r, c) in the order of the pair iterator
  void pairs(int r, int c, std::vector<Key>& out) const;
};

// options of one family of H-matrices.  Every operation runs on one stream
// per device (created on first use, kept for the process), with matrices
// from a stream-ordered pool of that device and freed on that stream.
struct Ctx {
  std::shared_ptr<const Tree> t;
  double tol = 1e-6;     // hopts.tol
  int kmax = 100;        // hopts.kmax
  cudaStream_t st = nullptr;
  int device = 0;
  int* host = nullptr;   // pinned: [0] ACA rank, [1] error flags
  int* dev = nullptr;    // device: the same two words
  ~Ctx();
};

// error flags a kernel raises (dev[1]): a zero pivot of a leaf LU or inverse
constexpr int HL_ERR_PIVOT = 1;

// cluster tree of the C ABI, checked (leaf pairs full, blocks partition the
// matrix and match the tree)
mnpbem_status tree_from_abi(const mnpbem_cluster_tree* t, std::shared_ptr<Tree>& out);

mnpbem_status ctx_make(int device, std::shared_ptr<const Tree> t, double tol, int kmax, std::shared_ptr<Ctx>& out);
// the H-arithmetic stream of a device (created on first use)
mnpbem_status hl_stream(int device, cudaStream_t& st);
// error flags raised since the last call (synchronises the stream)
mnpbem_status check_flags(Ctx& c);

// ---- operations (hmatlu, hmatrsolve, hmatinv, hmatadd, mtimes1, hmatsolve,
// hmatmul1, hmatfull)
mnpbem_status h_lu(Ctx& c, const HM& B, HM& A);
// X (L U) = B for key 'N' ('U' then 'L'), or one factor for 'U' / 'L'
mnpbem_status h_rsolve_lu(Ctx& c, const HM& B, const HM& A, char key, HM& X);
// X with (L U) X = B for key 'N' ('L' then 'U'), or one factor for 'L' / 'U'
mnpbem_status h_lsolve_lu(Ctx& c, const HM& B, const HM& A, char key, HM& X);
// C = A B (hmatrix.h operator*, truncated with the options of c)
mnpbem_status h_mul(Ctx& c, const HM& A, const HM& B, HM& C);
mnpbem_status h_inv(Ctx& c, const HM& A, HM& C);
mnpbem_status h_add(Ctx& c, const HM& A, const HM& B, HM& C);
mnpbem_status h_neg(Ctx& c, const HM& A, HM& C);
// diag(d) A (side 'L') or A diag(d) (side 'R'); d [n] in cluster order (device)
mnpbem_status h_scale(Ctx& c, const HM& A, const double2* d, char side, HM& C);
// x [n][N] column-major (ld n) in cluster order: (L U) x = b in place
mnpbem_status h_solve(Ctx& c, const HM& A, char key, double2* x, int N);
// y = A x (+ y when acc), x, y column-major [n][N] in cluster order
mnpbem_status h_matvec(Ctx& c, const HM& A, const double2* x, double2* y, int N, bool acc);
// expanded matrix [n][n] column-major in cluster order
mnpbem_status h_full(Ctx& c, const HM& A, double2* out);
// device copy of a block given on the host (column-major)
mnpbem_status upload(Ctx& c, const double2* host, int m, int n, DMat& out);
mnpbem_status alloc(Ctx& c, int m, int n, DMat& out);
mnpbem_status alloc_raw(Ctx& c, size_t bytes, std::shared_ptr<void>& out);

// ---- the 'hmat' preconditioner (initprecond.m / mfun.m)
struct HPrecond {
  std::shared_ptr<Ctx> c;
  HM G1i, G2i, Sigma1, Deltai, Sigmai;
  DMat eps1, eps2, nvec;   // cluster order: [n], [n], [n][3] (column d at d n)
  double2 k = {0.0, 0.0};  // wavenumber in vacuum
  DMat work;               // vectors of apply()
  std::shared_ptr<void> perm;   // [n] face at each cluster position (device)
};
// G1, H1, G2, H2 (consumed), per-face eps1 / eps2 (device, face order) and
// normals nvec [n][3] (device, face order)
mnpbem_status precond_build(std::shared_ptr<Ctx> c, HM& G1, HM& H1, HM& G2, HM& H2, double k,
                            const double2* eps1_f, const double2* eps2_f, const double* nvec_f, HPrecond& out);
// mfun.m on b-space vectors in face order (phi, De [n][P]; a, alpha
// [n][3][P]); dst: x-space [n][4P] (sig1 | h1) then [n][4P] (sig2 | h2)
mnpbem_status precond_apply(HPrecond& h, int P, const double2* phi, const double2* a, const double2* alpha,
                            const double2* De, double2* dst);

}  // namespace hl
}  // namespace mnpbem
