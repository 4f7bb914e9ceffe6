// Adjoint gradient of the extinction cross section (device side).
#pragma once
#include "common.cuh"

namespace mnpbem {

constexpr int MAX_ORDER_ADJ = 8;

struct AdjParams {
  int64_t n = 0;
  int order = 5;
  // geometry (device)
  const double* pos = nullptr;    // [n][3] centroids
  const double* nvec = nullptr;   // [n][3]
  const double* area = nullptr;   // [n]
  const double* verts = nullptr;  // [nverts][3]
  const int* faces = nullptr;     // [n][4], -1 = triangle
  const double *xt = nullptr, *yt = nullptr, *wt = nullptr;   // rule-18 points
  int ntri = 0;
  const double *x3 = nullptr, *y3 = nullptr, *w3 = nullptr;   // polar rule, triangles
  int n3 = 0;
  const double *x4 = nullptr, *y4 = nullptr, *w4 = nullptr;   // polar rule, quadrilaterals
  int n4 = 0;
  const int* ref_row = nullptr;
  const int* ref_col = nullptr;
  const int* off_idx = nullptr;   // refined entries with row != col
  int noff = 0;
  // per face and per wavelength
  const double2* eps1 = nullptr;  // [n] inside
  const double2* eps2 = nullptr;  // [n] outside
  const unsigned char* exc_out = nullptr;   // outside medium is the excitation medium
  double2 k1{0, 0}, k2{0, 0}, kb{0, 0};     // inside, outside, excitation medium
  double k0 = 0;
  // weights: U [n][16] = (UG1, UH1, UG2, UH2), X [n][8] = (sig1, h1, sig2, h2), cb [n]
  double2* U = nullptr;
  double2* X = nullptr;
  double* cb = nullptr;
  // gradient accumulators (FP64)
  double* gpos = nullptr;    // [n][3]
  double* gnv = nullptr;     // [n][3]
  double* garea = nullptr;   // [n]
  double* gv = nullptr;      // [nverts][3]
  double* gk1 = nullptr;     // [2]: d(lam^T A x)/dk of the inside medium
};

void adj_transpose(double2* A, int64_t n, int64_t ld, cudaStream_t st);
void adj_transpose(float2* A, int64_t n, int64_t ld, cudaStream_t st);
// general elementwise steps of the transposed chain (see adjoint.cu)
template <typename C>
void adj_chainT(const AdjParams& p, int mode, const C* a, const C* b, C* o1, C* o2, const C* c, const C* d,
                cudaStream_t st);
// y [n][4] = (Ahi + Alo)^T V in double-single arithmetic, V[i][c] = src[i * stride + off + c]
// (vsplit: 8 n complex64 scratch, part: chunks * 4 n complex128 scratch)
void adj_gemm_t_ds(int64_t n, const float2* Ahi, const float2* Alo, int64_t lda, const double2* V, int stride,
                   int off, float2* vsplit, double2* part, int chunks, double2* y, cudaStream_t st, bool accumulate);
// r = w - A^T lam from the two sides' products y1, y2 ([n][4]); norms[0] += |r|^2
void adj_resid(int64_t n, const double2* y1, const double2* y2, const double2* ws2, const double2* wh2, double2* rs1,
               double2* rh1, double2* rs2, double2* rh2, double* norms, cudaStream_t st);
// dJ/dx of ext (adj_rhs) or sca (adj_rhs_sca, which also adds the explicit
// far-field terms of sca to the position / area accumulators)
void adj_rhs(const AdjParams& p, const double* pol, const double* dir, double2* gs2, double2* gh2, cudaStream_t st);
void adj_rhs_sca(const AdjParams& p, const double2* fields, const double* inf_nvec, const double* inf_area,
                 int ninf, int P, int ip, double nb, const double2* x2, double2* gs2, double2* gh2, cudaStream_t st);
// elementwise steps of the transposed bemret chain (see adjoint.cu)
void adj_chain_step(const AdjParams& p, int mode, const double2* a, const double2* b, double2* o1, double2* o2,
                    const double2* c, cudaStream_t st);
void adj_weights(const AdjParams& p, const double2* lphi, const double2* la, const double2* lDe,
                 const double2* lal, const double2* x1, const double2* x2, int P, int ip, cudaStream_t st);
// all geometric contractions and the chain rule to the vertices (which: 0 ext, 1 sca)
void adj_geometry(const AdjParams& p, int which, const double* pol, const double* dir, const double2* lphi,
                  const double2* la, const double2* lDe, const double2* lal, const double2* GX1,
                  const double2* GX2, const double2* HX1, double* geps, cudaStream_t st);

}  // namespace mnpbem
