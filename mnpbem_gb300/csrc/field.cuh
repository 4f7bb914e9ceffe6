// Fields at points off the particle boundary.
#pragma once
#include "geometry.cuh"

namespace mnpbem {

// E and H [npts][3][npol] (complex128, device) at the points pts [npts][3]
// (host) lying in the 1-based media pt_med (host) from the surface charges
// sig1, sig2 [n][npol] and currents h1, h2 [n][3][npol] (device).  face_med:
// device [2][n] 0-based inside / outside media of the faces; kmed [nmed]: the
// media's wavenumbers; k0 = 2 pi / enei.
mnpbem_status point_fields(const GeomDev& g, const int* face_med, int64_t npts, const double* pts,
                           const int* pt_med, const double2* kmed, int nmed, double k0, int npol,
                           const double2* sig1, const double2* sig2, const double2* h1, const double2* h2,
                           double2* e, double2* h, double rel_cut, double abs_cut, cudaStream_t st);

// Fields E, H [n][3][npol] and potentials phi, phip [n][npol], a, ap
// [n][3][npol] (device, complex128; any output may be null) at the faces on
// side `side` (0 inside, 1 outside) from the surface charges and currents
// (device); kmed [nmed] device wavenumbers of the media.
mnpbem_status surface_fields(const GeomDev& g, const int* face_med, const double2* kmed, double k0, int npol,
                             int side, const double2* sig1, const double2* sig2, const double2* h1,
                             const double2* h2, double2* e, double2* h, double2* phi, double2* phip,
                             double2* av, double2* ap, cudaStream_t st);

// Far fields e, h [ndir][3][npol] (device, complex128; either may be null)
// in the unit directions dirs [ndir][3] (device) of the charges and currents
// on the faces bordering the 0-based embedding medium `med` of wavenumber k.
mnpbem_status far_fields(const GeomDev& g, const int* face_med, int med, double2 k, double k0, int npol,
                         int ndir, const double* dirs, const double2* sig1, const double2* sig2,
                         const double2* h1, const double2* h2, double2* e, double2* h, cudaStream_t st);

}  // namespace mnpbem
