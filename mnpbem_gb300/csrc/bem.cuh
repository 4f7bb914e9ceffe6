#pragma once
#include "common.cuh"

namespace mnpbem {

// Per-face data the BEM kernels read (device pointers).
struct FaceData {
  int64_t n = 0;
  const double* pos = nullptr;   // [n][3]
  const double* nvec = nullptr;  // [n][3]
  const double* area = nullptr;  // [n]
  const double2* eps1 = nullptr; // [n] dielectric function inside each face
  const double2* eps2 = nullptr; // [n] outside
  const unsigned char* exc_in = nullptr;   // [n] inside medium == excitation medium
  const unsigned char* exc_out = nullptr;  // [n] outside medium == excitation medium
  // complex64 copies for the complex64 kernels: eps1, eps2, L = eps1 - eps2, nvec
  const float2* eps1f = nullptr;
  const float2* eps2f = nullptr;
  const float2* Lf = nullptr;
  const float* nvecf = nullptr;   // [n][3]
};

// Right-hand side / solution sets of P polarisations:
//   scalar fields [n][P], vector fields [n][3][P].
template <typename R>
struct Fields {
  cplx<R>* s = nullptr;   // phi or sig
  cplx<R>* v = nullptr;   // a or h
};

// planewaveret potential (potential.m:13-57) + bemret excitation (excitation.m:4-29):
// phi [n][P] (= 0), a, alpha [n][3][P], De [n][P]  (FP64)
void launch_excitation(const FaceData& f, int P, const double* pol, const double* dir,
                       const LamParams* lp, double2* phi, double2* a, double2* alpha,
                       double2* De, cudaStream_t st);
// external potentials [4][n][P] + [4][n][3][P] (phi1, phi1p, phi2, phi2p, a1,
// a1p, a2, a2p) -> phi, a, alpha, De (BEM/@bemret/private/excitation.m)
void launch_excitation_ext(const FaceData& f, int P, const double2* pot, const LamParams* lp, double2* phi,
                           double2* a, double2* alpha, double2* De, cudaStream_t st);

// per-face dielectric functions eps1 (inside) / eps2 (outside) of this wavelength,
// plus their complex64 copies, L = eps1 - eps2 and the normals in FP32
void launch_face_eps(int64_t n, const int* med_in, const int* med_out, const LamParams* lp,
                     const double* nvec, double2* eps1, double2* eps2, float2* eps1f, float2* eps2f,
                     float2* Lf, float* nvecf, cudaStream_t st);

// The matrices of the mldivide chain as initmat leaves them: block LDU
// factors (dense.cuh) of G1, G2 and Sigma, explicit Sigma1 and Deltai.  G1 is
// factored per diagonal block (g1_off / g1_n: the particle groups whose
// media do not couple, e.g. the two spheres of a dimer; one block when G1 is
// full), its off-diagonal blocks being zero.
constexpr int CHAIN_MAXBLK = 16;
template <typename R> struct ChainMats {
  const cplx<R>* G1; const cplx<R>* G2; const cplx<R>* Sigma1; const cplx<R>* Deltai;
  const cplx<R>* Sigma; int64_t ld;
  int b = 64;                      // rows of the diagonal blocks of the LDU factors
  unsigned* bar = nullptr;         // grid-barrier words of the one-launch triangular sweeps (per stream)
  int ng1 = 1;
  int64_t g1_off[CHAIN_MAXBLK] = {0};
  int64_t g1_n[CHAIN_MAXBLK] = {0};
};

template <typename R>
using ChainGemm = mnpbem_status (*)(int64_t M, int64_t N, int64_t K, cplx<R> alpha,
                                    const cplx<R>* A, int64_t lda, const cplx<R>* B, int64_t ldb,
                                    cplx<R> beta, cplx<R>* C, int64_t ldc, cudaStream_t st,
                                    void* ctx);

// mldivide.m:12-49 in precision R.  in: phi, a, alpha, De; out: x1 = [sig1 | h1],
// x2 = [sig2 | h2] as [n][4P].  work must hold 32 n P complex values.
template <typename R>
mnpbem_status apply_mldivide(const FaceData& f, int P, const LamParams* lp, const ChainMats<R>& m,
                             const cplx<R>* phi, const cplx<R>* a, const cplx<R>* alpha,
                             const cplx<R>* De, cplx<R>* x1, cplx<R>* x2, cplx<R>* work,
                             ChainGemm<R> gemm, void* ctx, cudaStream_t st);

// r = b - A x with the full BEM operator (BEM/@bemretiter/private/afun.m:6-35), FP64.
// Y1 = G1 x1, Y2 = G2 x2, Z1 = H1 x1, Z2 = H2 x2 already computed ([n][4P]).
// Outputs r_phi, r_a, r_alpha, r_De; accumulates ||r||^2 and ||b||^2 into norms[0..1].
void launch_residual(const FaceData& f, int P, const LamParams* lp, const double2* Y1, const double2* Y2,
                     const double2* Z1, const double2* Z2, const double2* phi, const double2* a,
                     const double2* alpha, const double2* De, double2* rphi, double2* ra,
                     double2* ralpha, double2* rDe, double* norms, cudaStream_t st);

void launch_cvt_d2f(const double2* in, float2* out, int64_t count, cudaStream_t st);
void launch_cvt_f2d(const float2* in, double2* out, int64_t count, cudaStream_t st);
// x += dx (FP64 += from precision R); accumulates ||dx||^2, ||x_new||^2 into norms[0..1]
void launch_axpy_norm(double2* x, const float2* dx, int64_t count, double* norms, cudaStream_t st);
void launch_axpy_norm(double2* x, const double2* dx, int64_t count, double* norms, cudaStream_t st);

// Sigma stage of initmat.m:46-56 (per-face eps, scalar eps as a constant vector):
//   D = S1 - S2 ;  S = S1 diag(e1) - S2 diag(e2)           (launch_delta_sigma)
//   S += k^2 diag(L) (Deltai o (n n^T)) diag(L), L = e1 - e2   (launch_sigma_add)
template <typename R>
void launch_delta_sigma(int64_t n, const cplx<R>* S1, cplx<R>* S2_to_S, cplx<R>* D, int64_t ld,
                        const FaceData& f, cudaStream_t st);
template <typename R>
void launch_sigma_add(int64_t n, cplx<R>* S, const cplx<R>* Di, int64_t ld, const FaceData& f,
                      const LamParams* lp, cudaStream_t st);

// Far fields and cross sections (farfield.m:15-74, scattering.m, extinction.m).
// dirs [ndir][3]: first P rows are the excitation directions (extinction),
// the remaining ninf rows the sphere at infinity with weights inf_area.
// fields: scratch of ndir * 6 * P complex values.
void launch_farfield(const FaceData& f, int P, const double2* x1, const double2* x2,
                     const double* dirs, int ndir, const LamParams* lp, double2* fields,
                     cudaStream_t st);
void launch_cross_sections(int P, const double* pol, const double* inf_nvec, const double* inf_area,
                           int ninf, const double2* fields, double2 k_med, double2 nb1,
                           double* ext, double* sca, cudaStream_t st);
// same, with k_med / nb1 from lp and outputs at ext + lp->w * P, sca + lp->w * P
void launch_cross_sections_lp(int P, const double* pol, const double* inf_nvec,
                              const double* inf_area, int ninf, const double2* fields,
                              const LamParams* lp, double* ext, double* sca, cudaStream_t st);

}  // namespace mnpbem
