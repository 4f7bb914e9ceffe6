#pragma once
#include "common.cuh"

namespace mnpbem {

constexpr int ASM_MAXP = 16;    // particles per composite
constexpr int ASM_MAXMED = 16;  // media
constexpr double DBL_EPS_ASM = 2.220446049250313e-16;

struct AsmParams {
  int64_t n = 0;
  int64_t nref = 0;
  int order = 5;
  int64_t ld64 = 0, ld32 = 0;
  const int* part = nullptr;      // [n] particle index of each face
  const double4_32a* src = nullptr;   // [n] (x, y, z, area)
  const double4_32a* nrm = nullptr;   // [n] (nx, ny, nz, 0)
  const float4* srcf = nullptr;   // [n][2] double-single splits of src: (hi x, y, z, area), (lo ...)
  const float4* nrmf = nullptr;   // [n][2] double-single splits of nrm
  const int* ref_row = nullptr;
  const int* ref_col = nullptr;
  const double* ref_g = nullptr;
  const double* ref_f = nullptr;
  const LamParams* lp = nullptr;   // wavenumbers of the media (device)
  int nmed = 1;                    // media used by the blocks (1-based indices <= nmed)
  bool ds = false;                 // mixed outputs from the double-single pass
  // media (1-based, 0 = block not connected) of the four connectivity
  // blocks: 0 -> con{1,1} (+G1), 1 -> con{2,1} (-G1), 2 -> con{2,2} (+G2), 3 -> con{1,2} (-G2)
  signed char med[4][ASM_MAXP][ASM_MAXP];
  double2 *G1 = nullptr, *H1 = nullptr, *G2 = nullptr, *H2 = nullptr;  // complex128 outputs
  float2 *g1 = nullptr, *h1 = nullptr, *g2 = nullptr, *h2 = nullptr;   // complex64 outputs
  // mixed precision: the FP64 value of G1, H1, G2, H2 as complex64 pairs
  // hi = fl32(v), lo = fl32(v - hi) in planes [n][ld32] (used instead of G1..H2)
  float2 *G1lo = nullptr, *H1lo = nullptr, *G2lo = nullptr, *H2lo = nullptr;
  float2 *G1hi = nullptr, *H1hi = nullptr, *G2hi = nullptr, *H2hi = nullptr;
};

// full blocks of the H-matrices of G1, H1, G2, H2 on the leaf pairs of a
// cluster tree (cluster order = perm)
struct LeafAsm {
  int nfull = 0, nleaf = 0;
  int64_t nvals = 0;             // sum of the blocks' entries
  const int4* fblk = nullptr;    // [nfull] (first row, rows, first col, cols) in cluster order
  const int64_t* foff = nullptr; // [nfull] value offsets
  const int* perm = nullptr;     // [n] face at each cluster position
  const int* iperm = nullptr;    // [n] cluster position of each face
  const int* leaf_of = nullptr;  // [n] leaf index of each cluster position
  const int* fidx = nullptr;     // [nleaf][nleaf] full block of a leaf pair, -1 if none
  double2* val[4] = {};          // G1, H1, G2, H2 block values, row-major per block
};
mnpbem_status assemble_leaves(const AsmParams& p, const LeafAsm& la, cudaStream_t st);

void pack_sources(int n, const double* pos, const double* area, const double* nvec, double4_32a* src,
                  double4_32a* nrm, float4* srcf, float4* nrmf, cudaStream_t st);
// w64 && !w32: complex128 outputs; !w64 && w32: complex64 outputs;
// w64 && w32: complex64 working matrices plus hi / lo planes
mnpbem_status assemble_launch(const AsmParams& p, bool w64, bool w32, cudaStream_t st);
// out = hi + lo in FP64 (count complex values)
void hilo_to_c128(const float2* hi, const float2* lo, double2* out, int64_t count, cudaStream_t st);

}  // namespace mnpbem
