// C ABI of the library: handle management and the per-wavelength solve.
//
// The per-wavelength sequence follows BEM/@bemret/private/initmat.m:5-74 and
// BEM/@bemret/mldivide.m:12-49:
//   assemble G1, H1, G2, H2                    (compgreenret eval, assemble.cu)
//   G1i = inv(G1), G2i = inv(G2)               (blocked Gauss-Jordan, dense.cu)
//   Sigma1 = H1 G1i, Sigma2 = H2 G2i           (GEMM)
//   Deltai = inv(Sigma1 - Sigma2)
//   Sigma = Sigma1 L1 - Sigma2 L2 + k^2 ((L Deltai) .* (n n')) L,  Sigmai = inv(Sigma)
//   excitation, mldivide chain, spectra        (bem.cu)
// MNPBEM_MIXED runs the inversions and products on complex64 operands and
// recovers FP64 accuracy by iterative refinement with the FP64 operator of
// BEM/@bemretiter/private/afun.m:6-35 (the complex64 chain is the preconditioner).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <complex>
#include <vector>

#include "assemble.cuh"
#include "bem.cuh"
#include "dense.cuh"
#include "geometry.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

namespace mnpbem {

static thread_local std::string g_err;
void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}
const char* get_error() { return g_err.c_str(); }

Profiler*& current_profiler() {
  static thread_local Profiler* p = nullptr;
  return p;
}

// binds a handle's profiler to the calling thread for one API call
struct ProfBind {
  Profiler* prev;
  explicit ProfBind(Profiler* p) : prev(current_profiler()) { current_profiler() = p; }
  ~ProfBind() { current_profiler() = prev; }
};

// GEMM adapters
static mnpbem_status gemm64(int64_t M, int64_t N, int64_t K, double2 al, const double2* A,
                            int64_t lda, const double2* B, int64_t ldb, double2 be, double2* C,
                            int64_t ldc, cudaStream_t st, void*) {
  return gemm_simt<double>(M, N, K, al, A, lda, B, ldb, be, C, ldc, st);
}
static mnpbem_status gemm32(int64_t M, int64_t N, int64_t K, float2 al, const float2* A, int64_t lda,
                            const float2* B, int64_t ldb, float2 be, float2* C, int64_t ldc,
                            cudaStream_t st, void* ctx) {
  TcGemmCtx* tc = reinterpret_cast<TcGemmCtx*>(ctx);
  if (tc && tc_gemm_eligible(*tc, M, N, K))
    return tc_gemm_c64(*tc, M, N, K, al, A, lda, B, ldb, be, C, ldc, st);
  return gemm_simt<float>(M, N, K, al, A, lda, B, ldb, be, C, ldc, st);
}

}  // namespace mnpbem

using namespace mnpbem;

struct mnpbem_geom {
  int device = 0;
  cudaStream_t st = nullptr;
  GeomDev g;
  DevBufSet b;
  int nparts = 0;
  std::vector<int64_t> part_off;
  std::vector<int> inout;   // [np][2]
  std::vector<int> face_part;
  int max_medium = 0;
  DevBuf d_part, d_src, d_nrm;
  // workspace
  int64_t ld = 0;
  DevBuf mat[5];      // working-precision matrices
  DevBuf mat64[4];    // FP64 G1, H1, G2, H2 for refinement (MIXED)
  DevBuf vec64, vecw, facebuf, exbuf, fields, norms, outbuf;
  GJWork<float> gj32;
  GJWork<double> gj64;
  TcGemmCtx tc;
  bool tc_enabled = true;
  Profiler prof;
};

namespace {

std::complex<double> cx(const double* p) { return {p[0], p[1]}; }

mnpbem_status check_geom(const mnpbem_geom* g) {
  if (!g) { set_error("null geometry handle"); return MNPBEM_ERR_INVALID_ARG; }
  return MNPBEM_OK;
}

// connectivity media of the four blocks (Particles/@compound/connect.m:40-57)
void fill_media(const mnpbem_geom* G, AsmParams& p) {
  memset(p.med, 0, sizeof(p.med));
  for (int a = 0; a < G->nparts; ++a)
    for (int b = 0; b < G->nparts; ++b) {
      int ia = G->inout[2 * a], oa = G->inout[2 * a + 1];
      int ib = G->inout[2 * b], ob = G->inout[2 * b + 1];
      p.med[0][a][b] = (signed char)(ia == ib ? ia : 0);  // con{1,1}
      p.med[1][a][b] = (signed char)(oa == ib ? oa : 0);  // con{2,1}
      p.med[2][a][b] = (signed char)(oa == ob ? oa : 0);  // con{2,2}
      p.med[3][a][b] = (signed char)(ia == ob ? ia : 0);  // con{1,2}
    }
}

bool con12_zero(const mnpbem_geom* G) {
  for (int a = 0; a < G->nparts; ++a)
    for (int b = 0; b < G->nparts; ++b)
      if (G->inout[2 * a] == G->inout[2 * b + 1]) return false;
  return true;
}

AsmParams base_params(mnpbem_geom* G, const std::vector<std::complex<double>>& kmed) {
  AsmParams p;
  p.n = G->g.n;
  p.nref = G->g.nref;
  p.order = G->g.order;
  p.part = G->d_part.as<int>();
  p.src = G->d_src.as<double4_32a>();
  p.nrm = G->d_nrm.as<double4_32a>();
  p.ref_row = G->g.ref_row;
  p.ref_col = G->g.ref_col;
  p.ref_g = G->g.ref_g;
  p.ref_f = G->g.ref_f;
  for (size_t m = 0; m < kmed.size() && m < (size_t)ASM_MAXMED; ++m)
    p.k[m] = make_double2(kmed[m].real(), kmed[m].imag());
  fill_media(G, p);
  return p;
}

}  // namespace

extern "C" {

const char* mnpbem_last_error(void) { return get_error(); }
const char* mnpbem_version(void) { return "mnpbem-gb300 0.1 (sm_103a)"; }

mnpbem_status mnpbem_geom_create(const double* verts, int64_t nverts, const int64_t* faces,
                                 int64_t nfaces, int32_t nparts, const int64_t* part_nfaces,
                                 const int32_t* inout, const int32_t* closed,
                                 const mnpbem_quad* quad, const mnpbem_options* opts,
                                 mnpbem_geom** out) {
  if (!out || !verts || !faces || !part_nfaces || !inout || !quad || nverts <= 0 || nfaces <= 0 ||
      nparts <= 0) {
    set_error("mnpbem_geom_create: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (nparts > ASM_MAXP) { set_error("at most %d particles", ASM_MAXP); return MNPBEM_ERR_UNSUPPORTED; }
  if (nfaces > (int64_t)1 << 30) { set_error("too many faces"); return MNPBEM_ERR_UNSUPPORTED; }
  int64_t tot = 0;
  for (int i = 0; i < nparts; ++i) {
    if (part_nfaces[i] <= 0) { set_error("particle %d has no faces", i); return MNPBEM_ERR_INVALID_ARG; }
    tot += part_nfaces[i];
  }
  if (tot != nfaces) { set_error("part_nfaces do not sum to nfaces"); return MNPBEM_ERR_INVALID_ARG; }
  for (int64_t k = 0; k < nfaces; ++k) {
    for (int c = 0; c < 4; ++c) {
      int64_t v = faces[4 * k + c];
      if ((c < 3 && (v < 0 || v >= nverts)) || (c == 3 && (v < -1 || v >= nverts))) {
        set_error("face %lld has an invalid vertex index", (long long)k);
        return MNPBEM_ERR_INVALID_ARG;
      }
    }
  }
  int maxmed = 0;
  for (int i = 0; i < 2 * nparts; ++i) {
    if (inout[i] < 1 || inout[i] > ASM_MAXMED) { set_error("media must be in 1..%d", ASM_MAXMED); return MNPBEM_ERR_INVALID_ARG; }
    maxmed = std::max(maxmed, (int)inout[i]);
  }
  if (quad->n_tri <= 0 || !quad->x || !quad->y || !quad->w || quad->n_pol3 <= 0 || !quad->x3 ||
      !quad->y3 || !quad->w3 || quad->n_pol4 < 0) {
    set_error("invalid quadrature rules");
    return MNPBEM_ERR_INVALID_ARG;
  }
  mnpbem_options op = {3.0, 0.0, 5, 0};
  if (opts) op = *opts;
  if (op.order < 0 || op.order > MAX_ORDER) { set_error("order must be 0..%d", MAX_ORDER); return MNPBEM_ERR_INVALID_ARG; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device available");
    return MNPBEM_ERR_CUDA;
  }
  if (op.device < 0 || op.device >= ndev) { set_error("invalid device %d", op.device); return MNPBEM_ERR_INVALID_ARG; }
  MNP_CUDA(cudaSetDevice(op.device));
  mnpbem_geom* G = new mnpbem_geom();
  G->device = op.device;
  if (cudaStreamCreateWithFlags(&G->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete G;
    set_error("cudaStreamCreate failed");
    return MNPBEM_ERR_CUDA;
  }
  ProfBind pb_(&G->prof);
  G->nparts = nparts;
  G->max_medium = maxmed;
  G->inout.assign(inout, inout + 2 * nparts);
  G->part_off.assign(nparts + 1, 0);
  for (int i = 0; i < nparts; ++i) G->part_off[i + 1] = G->part_off[i] + part_nfaces[i];
  G->face_part.resize(nfaces);
  for (int i = 0; i < nparts; ++i)
    for (int64_t k = G->part_off[i]; k < G->part_off[i + 1]; ++k) G->face_part[k] = i;
  std::vector<int> cs, ce;
  for (int i = 0; i < nparts; ++i)
    if (!closed || closed[i]) { cs.push_back((int)G->part_off[i]); ce.push_back((int)G->part_off[i + 1]); }
  G->g.order = op.order;
  mnpbem_status s = geometry_build(G->g, G->b, verts, nverts, faces, nfaces, cs.data(), ce.data(),
                                   (int)cs.size(), quad, op.rel_cutoff, op.abs_cutoff, G->st);
  if (s == MNPBEM_OK) s = G->d_part.ensure(sizeof(int) * nfaces);
  if (s == MNPBEM_OK) s = G->d_src.ensure(sizeof(double4_32a) * nfaces);
  if (s == MNPBEM_OK) s = G->d_nrm.ensure(sizeof(double4_32a) * nfaces);
  if (s == MNPBEM_OK) {
    if (cudaMemcpyAsync(G->d_part.ptr, G->face_part.data(), sizeof(int) * nfaces,
                        cudaMemcpyHostToDevice, G->st) != cudaSuccess) {
      set_error("upload of particle index failed");
      s = MNPBEM_ERR_CUDA;
    } else {
      pack_sources((int)nfaces, G->g.pos, G->g.area, G->g.nvec, G->d_src.as<double4_32a>(),
                   G->d_nrm.as<double4_32a>(), G->st);
      if (cudaStreamSynchronize(G->st) != cudaSuccess) {
        set_error("geometry set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
        s = MNPBEM_ERR_CUDA;
      }
    }
  }
  if (s != MNPBEM_OK) {
    std::string keep = get_error();
    mnpbem_geom_destroy(G);
    set_error("%s", keep.c_str());
    return s;
  }
  G->ld = round_up(nfaces, 32);
  const char* env = getenv("MNPBEM_TC");
  if (env && env[0] == '0') G->tc_enabled = false;
  *out = G;
  return MNPBEM_OK;
}

mnpbem_status mnpbem_geom_destroy(mnpbem_geom* g) {
  if (!g) return MNPBEM_OK;
  cudaSetDevice(g->device);
  if (g->st) cudaStreamSynchronize(g->st);
  tc_release(g->tc);
  if (g->st) cudaStreamDestroy(g->st);
  delete g;
  return MNPBEM_OK;
}

mnpbem_status mnpbem_geom_size(const mnpbem_geom* g, int64_t* nfaces, int64_t* nref) {
  MNP_TRY(check_geom(g));
  if (nfaces) *nfaces = g->g.n;
  if (nref) *nref = g->g.nref;
  return MNPBEM_OK;
}

mnpbem_status mnpbem_geom_export(const mnpbem_geom* g, double* pos, double* nvec, double* tvec1,
                                 double* tvec2, double* area, int64_t* ref_row, int64_t* ref_col,
                                 double* ref_g, double* ref_f) {
  MNP_TRY(check_geom(g));
  MNP_CUDA(cudaSetDevice(g->device));
  const int64_t n = g->g.n, nref = g->g.nref, O = g->g.order;
  auto cp = [&](void* dst, const void* src, size_t bytes) -> mnpbem_status {
    if (dst && bytes) MNP_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return MNPBEM_OK;
  };
  MNP_TRY(cp(pos, g->g.pos, sizeof(double) * 3 * n));
  MNP_TRY(cp(nvec, g->g.nvec, sizeof(double) * 3 * n));
  MNP_TRY(cp(tvec1, g->g.tvec1, sizeof(double) * 3 * n));
  MNP_TRY(cp(tvec2, g->g.tvec2, sizeof(double) * 3 * n));
  MNP_TRY(cp(area, g->g.area, sizeof(double) * n));
  if (ref_row || ref_col) {
    std::vector<int> tmp(nref);
    if (ref_row) {
      MNP_TRY(cp(tmp.data(), g->g.ref_row, sizeof(int) * nref));
      for (int64_t e = 0; e < nref; ++e) ref_row[e] = tmp[e];
    }
    if (ref_col) {
      MNP_TRY(cp(tmp.data(), g->g.ref_col, sizeof(int) * nref));
      for (int64_t e = 0; e < nref; ++e) ref_col[e] = tmp[e];
    }
  }
  MNP_TRY(cp(ref_g, g->g.ref_g, sizeof(double) * nref * (O + 1)));
  MNP_TRY(cp(ref_f, g->g.ref_f, sizeof(double) * nref * 3 * (O + 1)));
  return MNPBEM_OK;
}

mnpbem_status mnpbem_assemble(mnpbem_geom* G, const double* k_media, int32_t nmed,
                              int32_t precision, void* G1, void* H1, void* G2, void* H2) {
  MNP_TRY(check_geom(G));
  if (!k_media || nmed < G->max_medium || nmed > ASM_MAXMED ||
      (precision != MNPBEM_FP64 && precision != MNPBEM_FP32)) {
    set_error("mnpbem_assemble: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  std::vector<std::complex<double>> km(nmed);
  for (int m = 0; m < nmed; ++m) km[m] = cx(k_media + 2 * m);
  AsmParams p = base_params(G, km);
  const int64_t n = G->g.n;
  const bool w64 = precision == MNPBEM_FP64;
  const size_t es = w64 ? sizeof(double2) : sizeof(float2);
  void* hosts[4] = {G1, H1, G2, H2};
  DevBuf tmp[4];
  for (int q = 0; q < 4; ++q)
    if (hosts[q]) MNP_TRY(tmp[q].ensure(es * n * n));
  if (w64) {
    p.ld64 = n;
    p.G1 = tmp[0].as<double2>(); p.H1 = tmp[1].as<double2>();
    p.G2 = tmp[2].as<double2>(); p.H2 = tmp[3].as<double2>();
  } else {
    p.ld32 = n;
    p.g1 = tmp[0].as<float2>(); p.h1 = tmp[1].as<float2>();
    p.g2 = tmp[2].as<float2>(); p.h2 = tmp[3].as<float2>();
  }
  MNP_TRY(assemble_launch(p, w64, !w64, G->st));
  for (int q = 0; q < 4; ++q)
    if (hosts[q]) MNP_CUDA(cudaMemcpyAsync(hosts[q], tmp[q].ptr, es * n * n, cudaMemcpyDeviceToHost, G->st));
  MNP_CUDA(cudaStreamSynchronize(G->st));
  return MNPBEM_OK;
}

mnpbem_status mnpbem_profile_enable(mnpbem_geom* G, int32_t on) {
  MNP_TRY(check_geom(G));
  G->prof.enabled = on != 0;
  return MNPBEM_OK;
}

mnpbem_status mnpbem_profile_reset(mnpbem_geom* G) {
  MNP_TRY(check_geom(G));
  MNP_CUDA(cudaSetDevice(G->device));
  MNP_CUDA(cudaStreamSynchronize(G->st));
  G->prof.reset();
  return MNPBEM_OK;
}

mnpbem_status mnpbem_profile_read(mnpbem_geom* G, int32_t phase, double* ms, double* flops,
                                  double* bytes, int64_t* launches) {
  MNP_TRY(check_geom(G));
  if (phase < 0 || phase >= PH_COUNT) { set_error("invalid phase"); return MNPBEM_ERR_INVALID_ARG; }
  MNP_CUDA(cudaSetDevice(G->device));
  MNP_CUDA(cudaStreamSynchronize(G->st));
  G->prof.flush();
  const PhaseAcc& a = G->prof.acc[phase];
  if (ms) *ms = a.ms;
  if (flops) *flops = a.flops;
  if (bytes) *bytes = a.bytes;
  if (launches) *launches = a.launches;
  return MNPBEM_OK;
}

mnpbem_status mnpbem_gemm_c64(int32_t device, int32_t path, int64_t M, int64_t N, int64_t K,
                              const float* alpha, const float* A, int64_t lda, const float* B,
                              int64_t ldb, const float* beta, float* C, int64_t ldc) {
  if (M <= 0 || N <= 0 || K <= 0 || !alpha || !beta || !A || !B || !C || lda < K || ldb < N ||
      ldc < N || (path != 0 && path != 1)) {
    set_error("mnpbem_gemm_c64: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  MNP_CUDA(cudaSetDevice(device));
  static TcGemmCtx tc[64];
  if (device < 0 || device >= 64) { set_error("invalid device"); return MNPBEM_ERR_INVALID_ARG; }
  cudaStream_t st;
  MNP_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{st};
  DevBuf dA, dB, dC;
  MNP_TRY(dA.ensure(sizeof(float2) * M * lda));
  MNP_TRY(dB.ensure(sizeof(float2) * K * ldb));
  MNP_TRY(dC.ensure(sizeof(float2) * M * ldc));
  MNP_CUDA(cudaMemcpyAsync(dA.ptr, A, sizeof(float2) * M * lda, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(dB.ptr, B, sizeof(float2) * K * ldb, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(dC.ptr, C, sizeof(float2) * M * ldc, cudaMemcpyHostToDevice, st));
  const float2 al = make_float2(alpha[0], alpha[1]), be = make_float2(beta[0], beta[1]);
  if (path == 1) {
    if (!tc_gemm_eligible(tc[device], M, N, K)) {
      set_error("tensor-core GEMM not available for this device or shape");
      return MNPBEM_ERR_UNSUPPORTED;
    }
    MNP_TRY(tc_gemm_c64(tc[device], M, N, K, al, dA.as<float2>(), lda, dB.as<float2>(), ldb, be,
                        dC.as<float2>(), ldc, st));
    MNP_TRY(tc_check_error(tc[device], st));
  } else {
    MNP_TRY(gemm_simt<float>(M, N, K, al, dA.as<float2>(), lda, dB.as<float2>(), ldb, be,
                             dC.as<float2>(), ldc, st));
  }
  MNP_CUDA(cudaMemcpyAsync(C, dC.ptr, sizeof(float2) * M * ldc, cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  return MNPBEM_OK;
}

mnpbem_status mnpbem_geom_stream(const mnpbem_geom* G, void** stream) {
  MNP_TRY(check_geom(G));
  if (!stream) { set_error("null stream pointer"); return MNPBEM_ERR_INVALID_ARG; }
  *stream = (void*)G->st;
  return MNPBEM_OK;
}

}  // extern "C"

// ======================================================================
// per-wavelength solver
// ======================================================================
namespace {

struct SolveCtx {
  mnpbem_geom* G;
  int P;
  double enei, k0;
  std::complex<double> kmed_exc, nb1;
  std::vector<std::complex<double>> kmed;   // per medium
  double2* eps1;   // device per-face
  double2* eps2;
  FaceData fd;
};

// upload per-face eps for this wavelength
mnpbem_status prepare_faces(mnpbem_geom* G, SolveCtx& c, const double* eps_media, int nmed) {
  const int64_t n = G->g.n;
  std::vector<double2> e(2 * n);
  for (int64_t i = 0; i < n; ++i) {
    int p = G->face_part[i];
    int mi = G->inout[2 * p] - 1, mo = G->inout[2 * p + 1] - 1;
    e[i] = make_double2(eps_media[2 * mi], eps_media[2 * mi + 1]);
    e[n + i] = make_double2(eps_media[2 * mo], eps_media[2 * mo + 1]);
  }
  (void)nmed;
  MNP_TRY(G->facebuf.ensure(sizeof(double2) * 2 * n + 2 * n + 64));
  MNP_CUDA(cudaMemcpyAsync(G->facebuf.ptr, e.data(), sizeof(double2) * 2 * n, cudaMemcpyHostToDevice, G->st));
  c.eps1 = G->facebuf.as<double2>();
  c.eps2 = c.eps1 + n;
  c.fd.n = n;
  c.fd.pos = G->g.pos;
  c.fd.nvec = G->g.nvec;
  c.fd.area = G->g.area;
  c.fd.eps1 = c.eps1;
  c.fd.eps2 = c.eps2;
  c.fd.exc_in = reinterpret_cast<const unsigned char*>(c.eps2 + n);
  c.fd.exc_out = c.fd.exc_in + n;
  return MNPBEM_OK;
}

mnpbem_status upload_masks(mnpbem_geom* G, int medium) {
  const int64_t n = G->g.n;
  std::vector<unsigned char> m(2 * n);
  for (int64_t i = 0; i < n; ++i) {
    int p = G->face_part[i];
    m[i] = G->inout[2 * p] == medium;
    m[n + i] = G->inout[2 * p + 1] == medium;
  }
  MNP_TRY(G->facebuf.ensure(sizeof(double2) * 2 * n + 2 * n + 64));
  unsigned char* dst = reinterpret_cast<unsigned char*>(G->facebuf.as<double2>() + 2 * n);
  MNP_CUDA(cudaMemcpyAsync(dst, m.data(), 2 * n, cudaMemcpyHostToDevice, G->st));
  MNP_CUDA(cudaStreamSynchronize(G->st));
  return MNPBEM_OK;
}

template <typename R>
GJWork<R>& gjw(mnpbem_geom* G);
template <> GJWork<float>& gjw<float>(mnpbem_geom* G) { return G->gj32; }
template <> GJWork<double>& gjw<double>(mnpbem_geom* G) { return G->gj64; }

template <typename R>
mnpbem_status gemm_w(int64_t M, int64_t N, int64_t K, cplx<R> al, const cplx<R>* A, int64_t lda,
                     const cplx<R>* B, int64_t ldb, cplx<R> be, cplx<R>* C, int64_t ldc,
                     cudaStream_t st, void* ctx);
template <>
mnpbem_status gemm_w<float>(int64_t M, int64_t N, int64_t K, float2 al, const float2* A, int64_t lda,
                            const float2* B, int64_t ldb, float2 be, float2* C, int64_t ldc,
                            cudaStream_t st, void* ctx) {
  return mnpbem::gemm32(M, N, K, al, A, lda, B, ldb, be, C, ldc, st, ctx);
}
template <>
mnpbem_status gemm_w<double>(int64_t M, int64_t N, int64_t K, double2 al, const double2* A,
                             int64_t lda, const double2* B, int64_t ldb, double2 be, double2* C,
                             int64_t ldc, cudaStream_t st, void* ctx) {
  return mnpbem::gemm64(M, N, K, al, A, lda, B, ldb, be, C, ldc, st, ctx);
}

// initmat in precision R on matrices M0..M4 (assembled G1, G2, H1, H2 in M0..M3)
template <typename R>
mnpbem_status initmat(mnpbem_geom* G, SolveCtx& c) {
  using Cx = cplx<R>;
  const int64_t n = G->g.n, ld = G->ld;
  Cx* M[5];
  for (int q = 0; q < 5; ++q) M[q] = G->mat[q].as<Cx>();
  void* ctx = (sizeof(R) == 4 && G->tc_enabled) ? (void*)&G->tc : nullptr;
  const Cx one = mk<R>(1, 0), zero = mk<R>(0, 0);
  // G1i, G2i
  MNP_TRY(gj_invert<R>(M[0], n, ld, gjw<R>(G), gemm_w<R>, ctx, G->st));
  MNP_TRY(gj_invert<R>(M[1], n, ld, gjw<R>(G), gemm_w<R>, ctx, G->st));
  // Sigma1 = H1 G1i -> M4 ; Sigma2 = H2 G2i -> M2
  MNP_TRY(gemm_w<R>(n, n, n, one, M[2], ld, M[0], ld, zero, M[4], ld, G->st, ctx));
  MNP_TRY(gemm_w<R>(n, n, n, one, M[3], ld, M[1], ld, zero, M[2], ld, G->st, ctx));
  // Delta -> M3, Sigma (partial) -> M2
  launch_delta_sigma<R>(n, M[4], M[2], M[3], ld, c.eps1, c.eps2, G->st);
  MNP_CHECK_LAUNCH();
  MNP_TRY(gj_invert<R>(M[3], n, ld, gjw<R>(G), gemm_w<R>, ctx, G->st));
  launch_sigma_add<R>(n, M[2], M[3], ld, c.eps1, c.eps2, G->g.nvec, c.k0, G->st);
  MNP_CHECK_LAUNCH();
  MNP_TRY(gj_invert<R>(M[2], n, ld, gjw<R>(G), gemm_w<R>, ctx, G->st));
  if (ctx) MNP_TRY(tc_check_error(G->tc, G->st));
  return MNPBEM_OK;
}

template <typename R>
ChainMats<R> chain_mats(mnpbem_geom* G) {
  using Cx = cplx<R>;
  ChainMats<R> m;
  m.G1i = G->mat[0].as<Cx>();
  m.G2i = G->mat[1].as<Cx>();
  m.Sigma1 = G->mat[4].as<Cx>();
  m.Deltai = G->mat[3].as<Cx>();
  m.Sigmai = G->mat[2].as<Cx>();
  m.ld = G->ld;
  return m;
}

mnpbem_status assemble_into(mnpbem_geom* G, SolveCtx& c, int precision) {
  AsmParams p = base_params(G, c.kmed);
  const int64_t ld = G->ld;
  if (precision == MNPBEM_FP64) {
    p.ld64 = ld;
    p.G1 = G->mat[0].as<double2>(); p.G2 = G->mat[1].as<double2>();
    p.H1 = G->mat[2].as<double2>(); p.H2 = G->mat[3].as<double2>();
    return assemble_launch(p, true, false, G->st);
  }
  p.ld32 = ld;
  p.ld64 = ld;
  p.g1 = G->mat[0].as<float2>(); p.g2 = G->mat[1].as<float2>();
  p.h1 = G->mat[2].as<float2>(); p.h2 = G->mat[3].as<float2>();
  p.G1 = G->mat64[0].as<double2>(); p.H1 = G->mat64[1].as<double2>();
  p.G2 = G->mat64[2].as<double2>(); p.H2 = G->mat64[3].as<double2>();
  return assemble_launch(p, true, true, G->st);
}

mnpbem_status ensure_workspace(mnpbem_geom* G, int precision, int P) {
  const int64_t n = G->g.n, ld = G->ld;
  const size_t es = precision == MNPBEM_FP64 ? sizeof(double2) : sizeof(float2);
  for (int q = 0; q < 5; ++q) MNP_TRY(G->mat[q].ensure(es * n * ld));
  if (precision == MNPBEM_MIXED)
    for (int q = 0; q < 4; ++q) MNP_TRY(G->mat64[q].ensure(sizeof(double2) * n * ld));
  // FP64 vectors: b (8nP) x (8nP) r (8nP) YZ (16nP) + chain work for FP64 (32nP)
  MNP_TRY(G->vec64.ensure(sizeof(double2) * n * P * (8 + 8 + 8 + 16 + 32)));
  // working-precision vectors for MIXED: in (8nP) out (8nP) work (32nP)
  MNP_TRY(G->vecw.ensure(sizeof(float2) * n * P * (8 + 8 + 32)));
  MNP_TRY(G->norms.ensure(sizeof(double) * 4));
  return MNPBEM_OK;
}

// one wavelength
mnpbem_status solve_one(mnpbem_geom* G, SolveCtx& c, const mnpbem_planewave* exc, int precision,
                        const mnpbem_refine* ref, double* dext, double* dsca, int32_t* iters,
                        double* resid) {
  const int64_t n = G->g.n;
  const int P = c.P;
  cudaStream_t st = G->st;
  MNP_TRY(assemble_into(G, c, precision));
  if (precision == MNPBEM_FP64) MNP_TRY(initmat<double>(G, c));
  else MNP_TRY(initmat<float>(G, c));
  // FP64 vectors
  double2* V = G->vec64.as<double2>();
  double2 *phi = V, *a = phi + n * P, *alpha = a + 3 * n * P, *De = alpha + 3 * n * P;
  double2 *x1 = De + n * P, *x2 = x1 + 4 * n * P;
  double2 *rphi = x2 + 4 * n * P, *ra = rphi + n * P, *ral = ra + 3 * n * P, *rDe = ral + 3 * n * P;
  double2 *Y1 = rDe + n * P, *Y2 = Y1 + 4 * n * P, *Z1 = Y2 + 4 * n * P, *Z2 = Z1 + 4 * n * P;
  double2* work64 = Z2 + 4 * n * P;
  const double* pol = G->exbuf.as<double>();
  const double* dirs = pol + 3 * P;
  launch_excitation(c.fd, P, pol, dirs, make_double2(c.kmed_exc.real(), c.kmed_exc.imag()), c.k0,
                    phi, a, alpha, De, st);
  MNP_CHECK_LAUNCH();
  double* norms = G->norms.as<double>();
  int used = 0;
  double final_res = -1.0;
  if (precision == MNPBEM_FP64) {
    MNP_TRY(apply_mldivide<double>(c.fd, P, c.k0, chain_mats<double>(G), phi, a, alpha, De, x1, x2,
                                   work64, gemm_w<double>, nullptr, st));
  } else {
    float2* W = G->vecw.as<float2>();
    float2 *fphi = W, *fa = fphi + n * P, *fal = fa + 3 * n * P, *fDe = fal + 3 * n * P;
    float2 *fx1 = fDe + n * P, *fx2 = fx1 + 4 * n * P, *fwork = fx2 + 4 * n * P;
    void* ctx = G->tc_enabled ? (void*)&G->tc : nullptr;
    ChainMats<float> cm = chain_mats<float>(G);
    auto apply32 = [&](const double2* p_, const double2* a_, const double2* al_,
                       const double2* De_) -> mnpbem_status {
      launch_cvt_d2f(p_, fphi, n * P, st);
      launch_cvt_d2f(a_, fa, 3 * n * P, st);
      launch_cvt_d2f(al_, fal, 3 * n * P, st);
      launch_cvt_d2f(De_, fDe, n * P, st);
      MNP_CHECK_LAUNCH();
      return apply_mldivide<float>(c.fd, P, c.k0, cm, fphi, fa, fal, fDe, fx1, fx2, fwork,
                                   gemm_w<float>, ctx, st);
    };
    MNP_TRY(apply32(phi, a, alpha, De));
    launch_cvt_f2d(fx1, x1, 4 * n * P, st);
    launch_cvt_f2d(fx2, x2, 4 * n * P, st);
    MNP_CHECK_LAUNCH();
    const int maxit = ref && ref->max_iter > 0 ? ref->max_iter : 10;
    const double tol = ref && ref->tol > 0 ? ref->tol : 1e-12;
    const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
    const double2* A64[4] = {G->mat64[0].as<double2>(), G->mat64[1].as<double2>(),
                             G->mat64[2].as<double2>(), G->mat64[3].as<double2>()};
    bool conv = false;
    for (int it = 0; it < maxit; ++it) {
      MNP_TRY(gemm_simt<double>(n, 4 * P, n, one, A64[0], G->ld, x1, 4 * P, zero, Y1, 4 * P, st));
      MNP_TRY(gemm_simt<double>(n, 4 * P, n, one, A64[2], G->ld, x2, 4 * P, zero, Y2, 4 * P, st));
      MNP_TRY(gemm_simt<double>(n, 4 * P, n, one, A64[1], G->ld, x1, 4 * P, zero, Z1, 4 * P, st));
      MNP_TRY(gemm_simt<double>(n, 4 * P, n, one, A64[3], G->ld, x2, 4 * P, zero, Z2, 4 * P, st));
      MNP_CUDA(cudaMemsetAsync(norms, 0, sizeof(double) * 4, st));
      launch_residual(c.fd, P, c.k0, Y1, Y2, Z1, Z2, phi, a, alpha, De, rphi, ra, ral, rDe, norms, st);
      MNP_CHECK_LAUNCH();
      MNP_TRY(apply32(rphi, ra, ral, rDe));
      launch_axpy_norm(x1, fx1, 4 * n * P, norms + 2, st);
      launch_axpy_norm(x2, fx2, 4 * n * P, norms + 2, st);
      MNP_CHECK_LAUNCH();
      double hn[4];
      MNP_CUDA(cudaMemcpyAsync(hn, norms, sizeof(hn), cudaMemcpyDeviceToHost, st));
      MNP_CUDA(cudaStreamSynchronize(st));
      used = it + 1;
      final_res = hn[1] > 0 ? sqrt(hn[0] / hn[1]) : 0.0;
      if (!(hn[2] == hn[2])) { set_error("refinement produced NaN"); return MNPBEM_ERR_NOT_CONVERGED; }
      if (sqrt(hn[2]) <= tol * sqrt(hn[3])) { conv = true; break; }
    }
    (void)conv;
  }
  // spectra (FP64)
  const int ndir = P + exc->ninf;
  const double* inf_nvec = dirs + 3 * P;
  const double* inf_area = inf_nvec + 3 * exc->ninf;
  double2* fields = G->fields.as<double2>();
  launch_farfield(c.fd, P, x1, x2, dirs, ndir, make_double2(c.kmed_exc.real(), c.kmed_exc.imag()),
                  c.k0, fields, st);
  MNP_CHECK_LAUNCH();
  launch_cross_sections(P, pol, inf_nvec, inf_area, exc->ninf, fields,
                        make_double2(c.kmed_exc.real(), c.kmed_exc.imag()),
                        make_double2(c.nb1.real(), c.nb1.imag()), dext, dsca, st);
  MNP_CHECK_LAUNCH();
  if (iters) *iters = used;
  if (resid) *resid = final_res;
  if (precision == MNPBEM_MIXED && G->tc_enabled) MNP_TRY(tc_check_error(G->tc, st));
  return MNPBEM_OK;
}

}  // namespace

extern "C" {

mnpbem_status mnpbem_solve(mnpbem_geom* G, const mnpbem_planewave* exc, int32_t nenei,
                           const double* enei, const double* eps_media, int32_t nmed,
                           int32_t precision, const mnpbem_refine* refine, mnpbem_solution* out) {
  MNP_TRY(check_geom(G));
  if (!exc || !enei || !eps_media || nenei <= 0 || nmed < G->max_medium || nmed > ASM_MAXMED ||
      exc->npol <= 0 || exc->npol > 4 || !exc->pol || !exc->dir || exc->medium < 1 ||
      exc->medium > nmed || exc->ninf < 0 || (exc->ninf > 0 && (!exc->inf_nvec || !exc->inf_area)) ||
      (precision != MNPBEM_FP64 && precision != MNPBEM_MIXED) || !out) {
    set_error("mnpbem_solve: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  for (int p = 0; p < exc->npol; ++p) {
    const double* q = exc->pol + 3 * p;
    const double* d = exc->dir + 3 * p;
    if (q[0] * d[0] + q[1] * d[1] + q[2] * d[2] != 0.0) {
      set_error("polarisation and propagation direction must be orthogonal");
      return MNPBEM_ERR_INVALID_ARG;
    }
  }
  for (int w = 0; w < nenei; ++w)
    if (!(enei[w] > 0)) { set_error("wavelengths must be positive"); return MNPBEM_ERR_INVALID_ARG; }
  if (!con12_zero(G)) {
    set_error("nested media (inside medium of one particle equals the outside of another) are not supported");
    return MNPBEM_ERR_UNSUPPORTED;
  }
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  const int P = exc->npol;
  const int64_t n = G->g.n;
  MNP_TRY(ensure_workspace(G, precision, P));
  // excitation buffer: pol, dir, inf nvec, inf area
  {
    std::vector<double> eb;
    eb.insert(eb.end(), exc->pol, exc->pol + 3 * P);
    eb.insert(eb.end(), exc->dir, exc->dir + 3 * P);
    if (exc->ninf) {
      eb.insert(eb.end(), exc->inf_nvec, exc->inf_nvec + 3 * exc->ninf);
      eb.insert(eb.end(), exc->inf_area, exc->inf_area + exc->ninf);
    }
    MNP_TRY(G->exbuf.ensure(sizeof(double) * eb.size()));
    MNP_CUDA(cudaMemcpyAsync(G->exbuf.ptr, eb.data(), sizeof(double) * eb.size(), cudaMemcpyHostToDevice, G->st));
    MNP_TRY(G->fields.ensure(sizeof(double2) * (size_t)(P + exc->ninf) * 6 * P));
  }
  MNP_TRY(upload_masks(G, exc->medium));
  MNP_TRY(G->outbuf.ensure(sizeof(double) * 2 * P * (size_t)nenei));
  double* dext = G->outbuf.as<double>();
  double* dsca = dext + P * (size_t)nenei;
  for (int w = 0; w < nenei; ++w) {
    SolveCtx c;
    c.G = G;
    c.P = P;
    c.enei = enei[w];
    c.k0 = 2 * M_PI / enei[w];
    const double* em = eps_media + 2 * (size_t)nmed * w;
    c.kmed.resize(nmed);
    for (int m = 0; m < nmed; ++m) c.kmed[m] = 2 * M_PI / enei[w] * std::sqrt(cx(em + 2 * m));
    c.kmed_exc = c.kmed[exc->medium - 1];
    c.nb1 = std::sqrt(cx(em));
    MNP_TRY(prepare_faces(G, c, em, nmed));
    int32_t it = 0;
    double res = -1;
    MNP_TRY(solve_one(G, c, exc, precision, refine, dext + (size_t)w * P, dsca + (size_t)w * P, &it, &res));
    if (out->ir_iters) out->ir_iters[w] = it;
    if (out->ir_resid) out->ir_resid[w] = res;
    // field outputs
    double2* x1 = G->vec64.as<double2>() + 8 * n * P;
    double2* x2 = x1 + 4 * n * P;
    const cudaMemcpyKind kind = out->outputs_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t cs = sizeof(double2);
    auto cp2 = [&](double* dst, const double2* src, int off, int width) -> mnpbem_status {
      if (!dst) return MNPBEM_OK;
      MNP_CUDA(cudaMemcpy2DAsync(dst + 2 * (size_t)w * n * width, cs * width, src + off, cs * 4 * P,
                                 cs * width, n, kind, G->st));
      return MNPBEM_OK;
    };
    MNP_TRY(cp2(out->sig1, x1, 0, P));
    MNP_TRY(cp2(out->h1, x1, P, 3 * P));
    MNP_TRY(cp2(out->sig2, x2, 0, P));
    MNP_TRY(cp2(out->h2, x2, P, 3 * P));
  }
  const cudaMemcpyKind kind = out->outputs_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (out->ext) MNP_CUDA(cudaMemcpyAsync(out->ext, dext, sizeof(double) * P * nenei, kind, G->st));
  if (out->sca) MNP_CUDA(cudaMemcpyAsync(out->sca, dsca, sizeof(double) * P * nenei, kind, G->st));
  MNP_CUDA(cudaStreamSynchronize(G->st));
  G->prof.flush();
  return MNPBEM_OK;
}

mnpbem_status mnpbem_bem_matrices(mnpbem_geom* G, double enei, const double* eps_media,
                                  int32_t nmed, int32_t precision, double* G1i, double* G2i,
                                  double* Sigma1, double* Deltai, double* Sigmai) {
  MNP_TRY(check_geom(G));
  if (!eps_media || nmed < G->max_medium || nmed > ASM_MAXMED || !(enei > 0) ||
      (precision != MNPBEM_FP64 && precision != MNPBEM_MIXED)) {
    set_error("mnpbem_bem_matrices: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  if (!con12_zero(G)) { set_error("nested media are not supported"); return MNPBEM_ERR_UNSUPPORTED; }
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  const int64_t n = G->g.n, ld = G->ld;
  MNP_TRY(ensure_workspace(G, precision, 1));
  SolveCtx c;
  c.G = G; c.P = 1; c.enei = enei; c.k0 = 2 * M_PI / enei;
  c.kmed.resize(nmed);
  for (int m = 0; m < nmed; ++m) c.kmed[m] = 2 * M_PI / enei * std::sqrt(cx(eps_media + 2 * m));
  MNP_TRY(prepare_faces(G, c, eps_media, nmed));
  MNP_TRY(assemble_into(G, c, precision));
  if (precision == MNPBEM_FP64) MNP_TRY(initmat<double>(G, c));
  else MNP_TRY(initmat<float>(G, c));
  double* outs[5] = {G1i, G2i, Sigmai, Deltai, Sigma1};  // order of mat[0..4]
  DevBuf conv;
  if (precision == MNPBEM_MIXED) MNP_TRY(conv.ensure(sizeof(double2) * n * ld));
  for (int q = 0; q < 5; ++q) {
    if (!outs[q]) continue;
    const double2* src = G->mat[q].as<double2>();
    if (precision == MNPBEM_MIXED) {
      launch_cvt_f2d(G->mat[q].as<float2>(), conv.as<double2>(), n * ld, G->st);
      MNP_CHECK_LAUNCH();
      src = conv.as<double2>();
    }
    MNP_CUDA(cudaMemcpy2DAsync(outs[q], sizeof(double2) * n, src, sizeof(double2) * ld,
                               sizeof(double2) * n, n, cudaMemcpyDeviceToHost, G->st));
    MNP_CUDA(cudaStreamSynchronize(G->st));
  }
  return MNPBEM_OK;
}

}  // extern "C"
