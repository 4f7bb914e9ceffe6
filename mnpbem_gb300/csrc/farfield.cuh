// Far fields of one direction, shared by the far-field kernel of the solve
// (bem.cu, charges and currents packed per face) and by the no-allocation
// cross sections (noalloc.cu, the public solution layout).  A CTA of 256
// threads per direction (dx, dy, dz): the phase exp(-i k (r . d)) area of
// every face whose inside (sig1, h1) or outside (sig2, h2) medium is the
// excitation medium, summed over the faces for each polarisation, then
//   e = i k0 Ph - i k (d Ps),   h = i k d x Ph      (@spectrumret/farfield.m)
// into fields [d][6][P].  Src gives sig(side, j, p) and h(side, j, c, p).
#pragma once
#include "common.cuh"

namespace mnpbem {

template <int MAXP, typename Src>
__device__ __forceinline__ void farfield_dir(int64_t n, int P, const double* __restrict__ pos,
                                             const double* __restrict__ area,
                                             const unsigned char* __restrict__ exc_in,
                                             const unsigned char* __restrict__ exc_out, const Src& src,
                                             double dx, double dy, double dz, double2 k, double k0, int d,
                                             double2* fields) {
  double2 Ps[MAXP], Ph[3][MAXP];
  for (int p = 0; p < MAXP; ++p) {
    Ps[p] = make_double2(0, 0);
    for (int c = 0; c < 3; ++c) Ph[c][p] = make_double2(0, 0);
  }
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    const bool in1 = exc_in[j] != 0, in2 = exc_out[j] != 0;
    if (!in1 && !in2) continue;
    const double s = dx * pos[3 * j] + dy * pos[3 * j + 1] + dz * pos[3 * j + 2];
    // exp(-i k s) * area
    double sn, cs;
    sincos(k.x * s, &sn, &cs);
    const double ee = exp(k.y * s) * area[j];
    const double2 ph = make_double2(ee * cs, -ee * sn);
    for (int p = 0; p < P; ++p) {
      double2 sv = make_double2(0, 0);
      double2 hv[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
      if (in1) {
        sv = cadd(sv, src.sig(0, j, p));
        for (int c = 0; c < 3; ++c) hv[c] = cadd(hv[c], src.h(0, j, c, p));
      }
      if (in2) {
        sv = cadd(sv, src.sig(1, j, p));
        for (int c = 0; c < 3; ++c) hv[c] = cadd(hv[c], src.h(1, j, c, p));
      }
      cfma(Ps[p], ph, sv);
      for (int c = 0; c < 3; ++c) cfma(Ph[c][p], ph, hv[c]);
    }
  }
  // block reduction of 4P complex accumulators
  __shared__ double2 red[8][4 * MAXP];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int p = 0; p < P; ++p) {
    for (int q = 0; q < 4; ++q) {
      double2 v = q == 0 ? Ps[p] : Ph[q - 1][p];
      for (int o = 16; o; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) red[wid][q * MAXP + p] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x / 32;
    const double2 ik = make_double2(-k.y, k.x);
    const double2 ik0 = make_double2(0, k0);
    const double dv[3] = {dx, dy, dz};
    for (int p = 0; p < P; ++p) {
      double2 S[4];
      for (int q = 0; q < 4; ++q) {
        S[q] = make_double2(0, 0);
        for (int w = 0; w < nw; ++w) S[q] = cadd(S[q], red[w][q * MAXP + p]);
      }
      const double2 ph3[3] = {S[1], S[2], S[3]};
      for (int c = 0; c < 3; ++c)
        fields[((int64_t)d * 6 + c) * P + p] = csub(cmul(ik0, ph3[c]), cmul(ik, cscale(S[0], dv[c])));
      // h = ik dir x Ph
      double2 cr[3];
      cr[0] = csub(cscale(ph3[2], dv[1]), cscale(ph3[1], dv[2]));
      cr[1] = csub(cscale(ph3[0], dv[2]), cscale(ph3[2], dv[0]));
      cr[2] = csub(cscale(ph3[1], dv[0]), cscale(ph3[0], dv[1]));
      for (int c = 0; c < 3; ++c) fields[((int64_t)d * 6 + 3 + c) * P + p] = cmul(ik, cr[c]);
    }
  }
}

}  // namespace mnpbem
