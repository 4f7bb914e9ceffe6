// MEX gateway between MNPBEM's MATLAB classes and the C ABI of
// include/mnpbem_gpu.h.  It mirrors the reference's own MEX functions
// (mex/hmatgreenret.cpp:21-61: one mexFunction, inputs read from mxArrays,
// new mxArrays returned to MATLAB) and is called by the bemretgpu class
// (@bemretgpu/bemretgpu.m), which bemsolver selects through
// Base/@bembase/find.m:25-51 when op.sim = 'ret' and op.gpu is set.
//
// Build (MATLAB R2018a or later, interleaved complex API), from this folder:
//   mex -R2018a -I../../include mnpbem_gpu_mex.cpp -L.. -lmnpbem_gpu
// (libmnpbem_gpu.so is built by the package's build step).  Not compiled in
// this repository's tests: neither MATLAB nor mex.h is available there; the
// same C calls are exercised through ctypes by the Python mirror.
//
// Commands (first argument):
//   h = mnpbem_gpu_mex('init', verts', faces', part_nfaces, inout', closed, quad, op)
//       verts' [3 x nv] double; faces' [4 x n] int64, 0-based, -1 for a
//       triangle's 4th corner; part_nfaces [np] int64; inout' [2 x np] int32;
//       closed [np] int32; quad: struct with x, y, w, x3, y3, w3, x4, y4, w4;
//       op: struct with RelCutoff, AbsCutoff, order, device (any may be absent)
//   [ext, sca, sig1, sig2, h1, h2, iters] = mnpbem_gpu_mex('solve', h, pol', dir',
//       medium, pinfty_nvec', pinfty_area, enei, eps_media, precision, refine_tol)
//       eps_media [nmed x nenei] complex; outputs in row-major order of the C
//       ABI: ext, sca [npol x nenei]; sig [npol x n x nenei]; h [npol x 3 x n x nenei]
//       (bemretgpu permutes them into MNPBEM's n x npol / n x 3 x npol layout)
//   [sig1, sig2, h1, h2, iters] = mnpbem_gpu_mex('solve_pot', h, enei, eps_media, precision,
//       refine_tol, phi1, phi1p, phi2, phi2p, a1, a1p, a2, a2p)
//       sig = bem \ exc(p, enei) for MNPBEM's excitation compstruct (any
//       potential may be [] for zero): phi [npol x n], a [npol x 3 x n]
//       complex, i.e. MNPBEM's n x npol / n x 3 x npol arrays permuted
//   mnpbem_gpu_mex('option', h, key, value)     tuning options (mnpbem_geom_set_option)
//   v = mnpbem_gpu_mex('stat', h, key)          statistics (mnpbem_geom_stat)
//   mnpbem_gpu_mex('free', h)
// Errors of the library become MATLAB errors (mexErrMsgIdAndTxt with the
// library's last error message) instead of the reference's exit(1).
#include <cstdint>
#include <set>
#include <string>

#include "mex.h"
#include "mnpbem_gpu.h"

namespace {

std::set<mnpbem_geom*>& handles() {
  static std::set<mnpbem_geom*> h;
  return h;
}

void fail(const char* what) { mexErrMsgIdAndTxt("mnpbem:gpu", "%s: %s", what, mnpbem_last_error()); }

void need(bool ok, const char* msg) {
  if (!ok) mexErrMsgIdAndTxt("mnpbem:gpu:args", "%s", msg);
}

std::string str(const mxArray* a) {
  need(mxIsChar(a), "expected a character array");
  char* c = mxArrayToString(a);
  std::string s(c ? c : "");
  mxFree(c);
  return s;
}

mnpbem_geom* handle_of(const mxArray* a) {
  need(mxIsUint64(a) && mxGetNumberOfElements(a) == 1, "expected a solver handle (uint64 scalar)");
  mnpbem_geom* g = reinterpret_cast<mnpbem_geom*>(static_cast<uintptr_t>(*static_cast<uint64_t*>(mxGetData(a))));
  need(handles().count(g) == 1, "invalid or freed solver handle");
  return g;
}

const double* dbl(const mxArray* a, size_t count, const char* name) {
  if (!(mxIsDouble(a) && !mxIsComplex(a) && mxGetNumberOfElements(a) == count))
    mexErrMsgIdAndTxt("mnpbem:gpu:args", "%s: expected %zu real doubles", name, count);
  return mxGetDoubles(a);
}

const double* field_dbl(const mxArray* s, const char* f, size_t* count) {
  const mxArray* a = mxGetField(s, 0, f);
  if (!a) mexErrMsgIdAndTxt("mnpbem:gpu:args", "quad.%s missing", f);
  need(mxIsDouble(a) && !mxIsComplex(a), "quadrature fields must be real doubles");
  *count = mxGetNumberOfElements(a);
  return mxGetDoubles(a);
}

double opt(const mxArray* op, const char* f, double dflt) {
  if (!op || !mxIsStruct(op)) return dflt;
  const mxArray* a = mxGetField(op, 0, f);
  return (a && mxIsNumeric(a) && mxGetNumberOfElements(a) == 1) ? mxGetScalar(a) : dflt;
}

void cmd_init(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  need(nrhs >= 7 && nlhs == 1, "init: h = mnpbem_gpu_mex('init', verts', faces', part_nfaces, inout', closed, quad[, op])");
  const mxArray *V = prhs[1], *F = prhs[2], *PN = prhs[3], *IO = prhs[4], *CL = prhs[5], *Q = prhs[6];
  const mxArray* op = nrhs > 7 ? prhs[7] : nullptr;
  need(mxIsDouble(V) && mxGetM(V) == 3, "verts' must be 3 x nv double");
  need(mxIsInt64(F) && mxGetM(F) == 4, "faces' must be 4 x n int64 (0-based, -1 for triangles)");
  need(mxIsInt64(PN), "part_nfaces must be int64");
  const int64_t nv = (int64_t)mxGetN(V), n = (int64_t)mxGetN(F);
  const int32_t np = (int32_t)mxGetNumberOfElements(PN);
  need(mxIsInt32(IO) && mxGetM(IO) == 2 && (int32_t)mxGetN(IO) == np, "inout' must be 2 x np int32");
  need(mxIsInt32(CL) && (int32_t)mxGetNumberOfElements(CL) == np, "closed must be np int32");
  need(mxIsStruct(Q), "quad must be a struct");
  size_t nx, ny, nw, nx3, ny3, nw3, nx4 = 0, ny4 = 0, nw4 = 0;
  mnpbem_quad q{};
  q.x = field_dbl(Q, "x", &nx);
  q.y = field_dbl(Q, "y", &ny);
  q.w = field_dbl(Q, "w", &nw);
  q.x3 = field_dbl(Q, "x3", &nx3);
  q.y3 = field_dbl(Q, "y3", &ny3);
  q.w3 = field_dbl(Q, "w3", &nw3);
  if (mxGetField(Q, 0, "x4")) {
    q.x4 = field_dbl(Q, "x4", &nx4);
    q.y4 = field_dbl(Q, "y4", &ny4);
    q.w4 = field_dbl(Q, "w4", &nw4);
  }
  need(nx == ny && ny == nw && nx3 == ny3 && ny3 == nw3 && nx4 == ny4 && ny4 == nw4, "quadrature sizes differ");
  q.n_tri = (int32_t)nx;
  q.n_pol3 = (int32_t)nx3;
  q.n_pol4 = (int32_t)nx4;
  mnpbem_options o{opt(op, "RelCutoff", 3.0), opt(op, "AbsCutoff", 0.0), (int32_t)opt(op, "order", 5),
                   (int32_t)opt(op, "device", 0)};
  mnpbem_geom* g = nullptr;
  if (mnpbem_geom_create(mxGetDoubles(V), nv, static_cast<const int64_t*>(mxGetData(F)), n, np,
                         static_cast<const int64_t*>(mxGetData(PN)), static_cast<const int32_t*>(mxGetData(IO)),
                         static_cast<const int32_t*>(mxGetData(CL)), &q, &o, &g) != MNPBEM_OK)
    fail("mnpbem_geom_create");
  handles().insert(g);
  plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
  *static_cast<uint64_t*>(mxGetData(plhs[0])) = static_cast<uint64_t>(reinterpret_cast<uintptr_t>(g));
}

void cmd_solve(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  need(nrhs == 11, "solve: [ext, sca, sig1, sig2, h1, h2, iters] = mnpbem_gpu_mex('solve', h, pol', dir', medium, "
                   "pinfty_nvec', pinfty_area, enei, eps_media, precision, refine_tol)");
  mnpbem_geom* g = handle_of(prhs[1]);
  int64_t n = 0, nref = 0;
  if (mnpbem_geom_size(g, &n, &nref) != MNPBEM_OK) fail("mnpbem_geom_size");
  const int32_t npol = (int32_t)mxGetN(prhs[2]);
  need(mxGetM(prhs[2]) == 3 && mxGetM(prhs[3]) == 3 && (int32_t)mxGetN(prhs[3]) == npol, "pol', dir' must be 3 x npol");
  const int32_t ninf = (int32_t)mxGetN(prhs[5]);
  mnpbem_planewave pw{};
  pw.npol = npol;
  pw.pol = dbl(prhs[2], 3 * (size_t)npol, "pol");
  pw.dir = dbl(prhs[3], 3 * (size_t)npol, "dir");
  pw.medium = (int32_t)mxGetScalar(prhs[4]);
  pw.ninf = ninf;
  pw.inf_nvec = dbl(prhs[5], 3 * (size_t)ninf, "pinfty_nvec");
  pw.inf_area = dbl(prhs[6], (size_t)ninf, "pinfty_area");
  const int32_t nenei = (int32_t)mxGetNumberOfElements(prhs[7]);
  const double* enei = dbl(prhs[7], (size_t)nenei, "enei");
  const mxArray* E = prhs[8];
  need(mxIsComplex(E) && mxIsDouble(E) && (int32_t)mxGetN(E) == nenei, "eps_media must be complex nmed x nenei");
  const int32_t nmed = (int32_t)mxGetM(E);
  const std::string prec = str(prhs[9]);
  need(prec == "mixed" || prec == "fp64", "precision must be 'mixed' or 'fp64'");
  mnpbem_refine ref{20, mxGetScalar(prhs[10])};
  const mwSize dext[2] = {(mwSize)npol, (mwSize)nenei};
  const mwSize dsig[3] = {(mwSize)npol, (mwSize)n, (mwSize)nenei};
  const mwSize dh[4] = {(mwSize)npol, 3, (mwSize)n, (mwSize)nenei};
  plhs[0] = mxCreateNumericArray(2, dext, mxDOUBLE_CLASS, mxREAL);
  plhs[1] = mxCreateNumericArray(2, dext, mxDOUBLE_CLASS, mxREAL);
  mnpbem_solution sol{};
  sol.ext = mxGetDoubles(plhs[0]);
  sol.sca = mxGetDoubles(plhs[1]);
  mxArray* outs[4] = {nullptr, nullptr, nullptr, nullptr};
  if (nlhs > 2) {
    outs[0] = mxCreateNumericArray(3, dsig, mxDOUBLE_CLASS, mxCOMPLEX);
    outs[1] = mxCreateNumericArray(3, dsig, mxDOUBLE_CLASS, mxCOMPLEX);
    outs[2] = mxCreateNumericArray(4, dh, mxDOUBLE_CLASS, mxCOMPLEX);
    outs[3] = mxCreateNumericArray(4, dh, mxDOUBLE_CLASS, mxCOMPLEX);
    sol.sig1 = reinterpret_cast<double*>(mxGetComplexDoubles(outs[0]));
    sol.sig2 = reinterpret_cast<double*>(mxGetComplexDoubles(outs[1]));
    sol.h1 = reinterpret_cast<double*>(mxGetComplexDoubles(outs[2]));
    sol.h2 = reinterpret_cast<double*>(mxGetComplexDoubles(outs[3]));
  }
  mxArray* it = mxCreateNumericMatrix(1, nenei, mxINT32_CLASS, mxREAL);
  sol.ir_iters = static_cast<int32_t*>(mxGetData(it));
  const mnpbem_status s =
      mnpbem_solve(g, &pw, nenei, enei, reinterpret_cast<const double*>(mxGetComplexDoubles(E)), nmed,
                   prec == "mixed" ? MNPBEM_MIXED : MNPBEM_FP64, &ref, &sol);
  if (s != MNPBEM_OK) {
    for (mxArray* a : outs)
      if (a) mxDestroyArray(a);
    mxDestroyArray(it);
    fail("mnpbem_solve");
  }
  for (int k = 0; k < 4; ++k) {
    if (nlhs > 2 + k) plhs[2 + k] = outs[k];
    else if (outs[k]) mxDestroyArray(outs[k]);
  }
  if (nlhs > 6) plhs[6] = it;
  else mxDestroyArray(it);
}

void cmd_solve_pot(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  need(nrhs == 14, "solve_pot: [sig1, sig2, h1, h2, iters] = mnpbem_gpu_mex('solve_pot', h, enei, eps_media, "
                   "precision, refine_tol, phi1, phi1p, phi2, phi2p, a1, a1p, a2, a2p)");
  mnpbem_geom* g = handle_of(prhs[1]);
  int64_t n = 0, nref = 0;
  if (mnpbem_geom_size(g, &n, &nref) != MNPBEM_OK) fail("mnpbem_geom_size");
  const double enei = mxGetScalar(prhs[2]);
  const mxArray* E = prhs[3];
  need(mxIsComplex(E) && mxIsDouble(E), "eps_media must be complex");
  const int32_t nmed = (int32_t)mxGetNumberOfElements(E);
  const std::string prec = str(prhs[4]);
  need(prec == "mixed" || prec == "fp64", "precision must be 'mixed' or 'fp64'");
  mnpbem_refine ref{20, mxGetScalar(prhs[5])};
  // the number of polarisations from the first non-empty potential
  int32_t npol = 0;
  for (int q = 0; q < 8 && !npol; ++q)
    if (!mxIsEmpty(prhs[6 + q])) npol = (int32_t)mxGetM(prhs[6 + q]);
  need(npol >= 1 && npol <= 4, "one to four polarisations (columns of the potentials) are supported");
  const double* pot[8];
  for (int q = 0; q < 8; ++q) {
    const mxArray* a = prhs[6 + q];
    if (mxIsEmpty(a)) { pot[q] = nullptr; continue; }
    const size_t want = (q < 4 ? 1 : 3) * (size_t)n * npol;
    need(mxIsDouble(a) && mxIsComplex(a) && mxGetNumberOfElements(a) == want,
         "potentials must be complex npol x n (phi) or npol x 3 x n (a), [] for zero");
    pot[q] = reinterpret_cast<const double*>(mxGetComplexDoubles(a));
  }
  mnpbem_potentials P{npol, pot[0], pot[1], pot[2], pot[3], pot[4], pot[5], pot[6], pot[7]};
  const mwSize dsig[2] = {(mwSize)npol, (mwSize)n};
  const mwSize dh[3] = {(mwSize)npol, 3, (mwSize)n};
  mxArray* outs[4] = {mxCreateNumericArray(2, dsig, mxDOUBLE_CLASS, mxCOMPLEX),
                      mxCreateNumericArray(2, dsig, mxDOUBLE_CLASS, mxCOMPLEX),
                      mxCreateNumericArray(3, dh, mxDOUBLE_CLASS, mxCOMPLEX),
                      mxCreateNumericArray(3, dh, mxDOUBLE_CLASS, mxCOMPLEX)};
  mxArray* it = mxCreateNumericMatrix(1, 1, mxINT32_CLASS, mxREAL);
  mnpbem_solution sol{};
  sol.sig1 = reinterpret_cast<double*>(mxGetComplexDoubles(outs[0]));
  sol.sig2 = reinterpret_cast<double*>(mxGetComplexDoubles(outs[1]));
  sol.h1 = reinterpret_cast<double*>(mxGetComplexDoubles(outs[2]));
  sol.h2 = reinterpret_cast<double*>(mxGetComplexDoubles(outs[3]));
  sol.ir_iters = static_cast<int32_t*>(mxGetData(it));
  if (mnpbem_solve_potentials(g, &P, enei, reinterpret_cast<const double*>(mxGetComplexDoubles(E)), nmed,
                              prec == "mixed" ? MNPBEM_MIXED : MNPBEM_FP64, &ref, &sol) != MNPBEM_OK) {
    for (mxArray* a : outs) mxDestroyArray(a);
    mxDestroyArray(it);
    fail("mnpbem_solve_potentials");
  }
  for (int k = 0; k < 4; ++k) {
    if (nlhs > k) plhs[k] = outs[k];
    else mxDestroyArray(outs[k]);
  }
  if (nlhs > 4) plhs[4] = it;
  else mxDestroyArray(it);
}

}  // namespace

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  need(nrhs >= 1, "usage: mnpbem_gpu_mex(command, ...)");
  const std::string cmd = str(prhs[0]);
  if (cmd == "init") {
    cmd_init(nlhs, plhs, nrhs, prhs);
  } else if (cmd == "solve") {
    cmd_solve(nlhs, plhs, nrhs, prhs);
  } else if (cmd == "solve_pot") {
    cmd_solve_pot(nlhs, plhs, nrhs, prhs);
  } else if (cmd == "option") {
    need(nrhs == 4, "option: mnpbem_gpu_mex('option', h, key, value)");
    if (mnpbem_geom_set_option(handle_of(prhs[1]), str(prhs[2]).c_str(), (int32_t)mxGetScalar(prhs[3])) != MNPBEM_OK)
      fail("mnpbem_geom_set_option");
  } else if (cmd == "stat") {
    need(nrhs == 3 && nlhs == 1, "stat: v = mnpbem_gpu_mex('stat', h, key)");
    double v = 0.0;
    if (mnpbem_geom_stat(handle_of(prhs[1]), str(prhs[2]).c_str(), &v) != MNPBEM_OK) fail("mnpbem_geom_stat");
    plhs[0] = mxCreateDoubleScalar(v);
  } else if (cmd == "free") {
    need(nrhs == 2, "free: mnpbem_gpu_mex('free', h)");
    mnpbem_geom* g = handle_of(prhs[1]);
    handles().erase(g);
    if (mnpbem_geom_destroy(g) != MNPBEM_OK) fail("mnpbem_geom_destroy");
  } else {
    mexErrMsgIdAndTxt("mnpbem:gpu:args", "unknown command '%s'", cmd.c_str());
  }
}
