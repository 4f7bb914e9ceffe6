// C ABI of the library: handle management and the per-wavelength solve.
//
// The per-wavelength sequence follows BEM/@bemret/private/initmat.m:5-74 and
// BEM/@bemret/mldivide.m:12-49, with the inverses of G1, G2 and Sigma replaced
// by block LDU factors (dense.cu) and triangular solves:
//   assemble G1, H1, G2, H2                    (compgreenret eval, assemble.cu)
//   G1 = L D U, G2 = L D U                     (G1 per diagonal block when the
//                                               particles' media do not couple)
//   Sigma1 = H1 G1^-1, Sigma2 = H2 G2^-1       (right-side triangular solves)
//   Deltai = inv(Sigma1 - Sigma2)              (blocked Gauss-Jordan: needed
//                                               elementwise by the Sigma term)
//   Sigma = Sigma1 L1 - Sigma2 L2 + k^2 ((L Deltai) .* (n n')) L,  Sigma = L D U
//   excitation, mldivide chain, spectra        (bem.cu; G1i x, G2i x, Sigmai x
//                                               as triangular solves)
// MNPBEM_MIXED runs the inversions and products on complex64 operands and
// recovers FP64 accuracy by iterative refinement with the FP64 operator of
// BEM/@bemretiter/private/afun.m:6-35 (the complex64 chain is the preconditioner).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <complex>
#include <functional>
#include <algorithm>
#include <memory>
#include <thread>
#include <vector>

#include "adjoint.cuh"
#include "assemble.cuh"
#include "bem.cuh"
#include "dense.cuh"
#include "geometry.cuh"
#include "field.cuh"
#include "hlu.cuh"
#include "hmat.cuh"
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

uint64_t& alloc_generation() {
  static uint64_t gen = 0;
  return gen;
}
bool& capturing_now() {
  static thread_local bool c = false;
  return c;
}

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
  if (tc && tc_gemm_eligible(*tc, M, N, K, A, lda, C, ldc, be))
    return tc_gemm_c64(*tc, M, N, K, al, A, lda, B, ldb, be, C, ldc, st);
  return gemm_simt<float>(M, N, K, al, A, lda, B, ldb, be, C, ldc, st);
}

}  // namespace mnpbem

using namespace mnpbem;

// Per-wavelength working state.  A handle owns one or more lanes; each lane
// has its own stream, matrices, vectors, Gauss-Jordan and tensor-core
// workspaces and captured stage graphs, so that several wavelengths of a
// sweep run concurrently: the latency-bound steps of one wavelength (pivot
// blocks, panel products, refinement vectors) overlap the tensor-core
// updates of the others.  Lane 0 runs on the handle's stream.
constexpr int NSTAGES = 7;   // assemble, initmat, first solve, refine (DS), spectra, refine (FP32), refine (incremental)

struct Lane {
  cudaStream_t st = nullptr;
  bool own_stream = false;
  DevBuf mat[5];      // working-precision matrices
  DevBuf mat64[4];    // G1, H1, G2, H2 for the refinement residual (MIXED): hi / lo complex64 planes
  DevBuf vec64, vecw, facebuf, fields, norms, outbuf, bsplit, lp_dev;
  GJWork<float> gj32;    // block width set per solve (256 on the tensor-core path)
  GJWork<double> gj64;
  LDUWork<float> lu32;   // block LDU factors of G1, G2, Sigma
  LDUWork<double> lu64;
  DevBuf lu_status;      // LDU status words (see dense.cuh)
  DevBuf lu_bar;         // grid-barrier words of the one-launch triangular sweeps
  TcGemmCtx tc;
  int* status_host = nullptr;     // pinned: Gauss-Jordan (4), LDU (2), tensor-core error word (1), spare
  double* norms_host = nullptr;   // pinned: refinement norms (4)
  cudaEvent_t ev = nullptr;       // completion of the work last queued by the scheduler
  struct Graphs {
    bool valid = false;
    int precision = -1, P = 0, ninf = 0;
    bool prof = false;
    uint64_t sig = 0;             // addresses of every buffer the graphs captured
    cudaGraphExec_t exec[NSTAGES] = {};
    cudaGraph_t graph[NSTAGES] = {};   // the captured stages (child graphs of a sweep graph)
    Profiler::GraphRec rec[NSTAGES];
  } graphs;
  DevBuf swctl;                   // device state of the lane in a sweep graph (SweepCtl)
  float cond_max = 0.f;       // largest block condition proxy since the counter was reset
  // scheduler state
  enum { IDLE = 0, ITER, DONE } state = IDLE;
  int w = -1, iters = 0;
  double res = -1.0;
  int last_kind = 0;         // stage of the last refinement step
  bool ds_done = false;      // a double-single residual has been computed for this wavelength
  double bnorm2 = 0.0;       // ||b||^2 of the excitation (from the last full residual)
  // preconditioner of the iterative solver kept for later wavelengths: the
  // dense chain matrices in mat[], the per-face data and parameters of the
  // wavelength it was built at (cleared whenever mat[] is overwritten)
  DevBuf pc_face, pc_lp;
  bool pc_valid = false;
  int pc_precision = -1;
  double pc_enei = 0.0;
  int pc_last_steps = 0;
  const void* pc_mat0 = nullptr;
  // the 'hmat' preconditioner (H-matrix LU factors, FP64) and a signature of
  // the cluster tree it was built on
  std::shared_ptr<hl::HPrecond> hpc;
  uint64_t hpc_sig = 0;
};

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
  int64_t nverts = 0;
  bool all_closed = true;
  bool curved = false;       // curved (6-node / 9-node) elements: interp = 'curv'
  double rel_cut = 3.0, abs_cut = 0.0;   // refinement cutoffs (RelCutoff, AbsCutoff)
  DevBuf d_part, d_src, d_nrm, d_srcf, d_nrmf, face_med, exbuf;
  DevBuf adj, adj2, adj_mats, adj_off;   // adjoint gradient workspace
  int adj_noff = -1;
  int64_t ld = 0;
  std::vector<std::unique_ptr<Lane>> lanes;
  int lanes_req = 0;        // 0: automatic
  int gj_nb = 0;            // Gauss-Jordan step width on the tensor-core path (256 or 512; 0: by size)
  int lu_steps = 0;         // LDU steps of 256 per trailing update on the tensor-core path (1, 2 or 4; 0: by size)
  std::vector<int64_t> g1_off, g1_n;   // diagonal blocks of G1 (one block when G1 is full)
  bool tf32_rna = true;     // round tensor-core A operands to nearest TF32
  bool asm_ds = true;       // mixed-precision assembly in double-single FP32 arithmetic
  bool gj_fused = true;     // fused Gauss-Jordan steps on the tensor-core path
  int tc_stages = 0;        // pipeline depth of the tensor-core GEMM (0: its default)
  int tc_ctas = 0;          // CTAs of the persistent tensor-core GEMM (0: one per SM)
  int tc_pair = 0;          // CTA-pair tensor-core GEMM: 1 always, 0 off, -1 long-K products
  bool tc_f16 = true;       // tensor-core products with scaled FP16 operands (kind::f16) instead of TF32
  bool tc_enabled = true;
  bool use_graphs = true;
  Profiler prof;
  // per-wavelength parameters: pinned host ring (one slot per wavelength)
  LamParams* lp_ring = nullptr;
  int lp_cap = 0;
  // one-graph sweeps (device-side wavelength queue and refinement decisions)
  bool sweep_graph = true;
  int64_t sweep_runs = 0;   // sweeps (or batch members) run as one graph
  int sweep_err = 0;        // CUDA error that turned them off
  cudaGraphExec_t sweep_exec = nullptr;
  uint64_t sweep_key = 0;
  DevBuf sweep_lp, sweep_ctl, sweep_res;   // parameters [nenei], job control, per-wavelength results
};

namespace {

constexpr int MAX_LANES = 16;
constexpr int DEFAULT_LANES = 4;
constexpr int LANE_NSTATUS = 8;

mnpbem_status check_geom(const mnpbem_geom* g) {
  if (!g) { set_error("null geometry handle"); return MNPBEM_ERR_INVALID_ARG; }
  return MNPBEM_OK;
}

void lane_release(Lane& L) {
  if (L.st) cudaStreamSynchronize(L.st);
  tc_release(L.tc);
  for (int q = 0; q < NSTAGES; ++q) {
    if (L.graphs.exec[q]) cudaGraphExecDestroy(L.graphs.exec[q]);
    L.graphs.exec[q] = nullptr;
    if (L.graphs.graph[q]) cudaGraphDestroy(L.graphs.graph[q]);
    L.graphs.graph[q] = nullptr;
    Profiler::release(L.graphs.rec[q]);
  }
  if (L.status_host) cudaFreeHost(L.status_host);
  if (L.norms_host) cudaFreeHost(L.norms_host);
  if (L.ev) cudaEventDestroy(L.ev);
  if (L.own_stream && L.st) cudaStreamDestroy(L.st);
  L.status_host = nullptr;
  L.norms_host = nullptr;
  L.ev = nullptr;
  L.st = nullptr;
}

mnpbem_status add_lane(mnpbem_geom* G) {
  std::unique_ptr<Lane> L(new Lane());
  if (G->lanes.empty()) {
    L->st = G->st;
  } else {
    MNP_CUDA(cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking));
    L->own_stream = true;
  }
  cudaError_t e = cudaMallocHost(&L->status_host, LANE_NSTATUS * sizeof(int));
  if (e == cudaSuccess) e = cudaMallocHost(&L->norms_host, 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L->ev, cudaEventDisableTiming);
  mnpbem_status s = MNPBEM_OK;
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("lane set-up failed: %s", cudaGetErrorString(e));
    s = MNPBEM_ERR_CUDA;
  }
  if (s == MNPBEM_OK) s = L->lp_dev.ensure(sizeof(LamParams));
  if (s == MNPBEM_OK) s = L->lu_status.ensure(2 * sizeof(int));
  if (s == MNPBEM_OK) s = L->lu_bar.ensure(2 * sizeof(unsigned));
  if (s != MNPBEM_OK) {
    lane_release(*L);
    return s;
  }
  for (int q = 0; q < LANE_NSTATUS; ++q) L->status_host[q] = 0;
  if (G->tc_stages) L->tc.stages = G->tc_stages;
  L->tc.max_ctas = G->tc_ctas;
  L->tc.pair = G->tc_pair;
  L->tc.f16 = G->tc_f16;
  G->lanes.push_back(std::move(L));
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

// Diagonal blocks of G1 = G11 - G21 and H1 = H11 - H21 (initmat.m:27-31):
// block (a, b) is non-zero when con{1,1} or con{2,1} connects the particles
// (the same inside medium, or the outside medium of a is the inside medium of
// b; Particles/@compound/connect.m:40-57).  Particles that couple directly
// or through others form one block; when every group is a contiguous range
// of particles, G1 is block-diagonal over their face ranges (e.g. the two
// spheres of a dimer with separate media), otherwise one full block.
void set_g1_blocks(mnpbem_geom* G) {
  const int np = G->nparts;
  std::vector<int> root(np);
  for (int a = 0; a < np; ++a) root[a] = a;
  std::function<int(int)> find = [&](int a) { return root[a] == a ? a : (root[a] = find(root[a])); };
  for (int a = 0; a < np; ++a)
    for (int b = 0; b < np; ++b) {
      const int ia = G->inout[2 * a], oa = G->inout[2 * a + 1], ib = G->inout[2 * b];
      if (a != b && (ia == ib || oa == ib)) root[find(a)] = find(b);
    }
  G->g1_off.clear();
  G->g1_n.clear();
  bool contiguous = true;
  for (int a = 0; a < np && contiguous; ++a) {
    if (a > 0 && find(a) == find(a - 1)) continue;   // same group as the previous particle
    for (int b = 0; b < a; ++b)
      if (find(b) == find(a)) contiguous = false;    // the group appeared before a gap
    G->g1_off.push_back(G->part_off[a]);
  }
  if (!contiguous || (int)G->g1_off.size() > CHAIN_MAXBLK) {
    G->g1_off.assign(1, 0);
    G->g1_n.assign(1, G->part_off[np]);
    return;
  }
  for (size_t q = 0; q < G->g1_off.size(); ++q)
    G->g1_n.push_back((q + 1 < G->g1_off.size() ? G->g1_off[q + 1] : G->part_off[np]) - G->g1_off[q]);
}

bool con12_zero(const mnpbem_geom* G) {
  for (int a = 0; a < G->nparts; ++a)
    for (int b = 0; b < G->nparts; ++b)
      if (G->inout[2 * a] == G->inout[2 * b + 1]) return false;
  return true;
}

AsmParams base_params(mnpbem_geom* G, const LamParams* lp) {
  AsmParams p;
  p.n = G->g.n;
  p.nref = G->g.nref;
  p.order = G->g.order;
  p.part = G->d_part.as<int>();
  p.src = G->d_src.as<double4_32a>();
  p.nrm = G->d_nrm.as<double4_32a>();
  p.srcf = G->d_srcf.as<float4>();
  p.nrmf = G->d_nrmf.as<float4>();
  p.nmed = G->max_medium;
  p.ref_row = G->g.ref_row;
  p.ref_col = G->g.ref_col;
  p.ref_g = G->g.ref_g;
  p.ref_f = G->g.ref_f;
  p.lp = lp;
  fill_media(G, p);
  return p;
}

}  // namespace

extern "C" {

const char* mnpbem_last_error(void) { return get_error(); }
const char* mnpbem_version(void) { return "mnpbem-gb300 0.2 (sm_103a)"; }

static mnpbem_status geom_create_impl(const double* verts, int64_t nverts, const int64_t* faces,
                                      const int64_t* faces2, int64_t nfaces, int32_t nparts,
                                      const int64_t* part_nfaces, const int32_t* inout,
                                      const int32_t* closed, const mnpbem_quad* quad,
                                      const mnpbem_options* opts, mnpbem_geom** out) {
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
  set_g1_blocks(G);
  std::vector<int> cs, ce;
  for (int i = 0; i < nparts; ++i)
    if (!closed || closed[i]) { cs.push_back((int)G->part_off[i]); ce.push_back((int)G->part_off[i + 1]); }
  G->nverts = nverts;
  G->all_closed = (int)cs.size() == nparts;
  G->g.order = op.order;
  G->curved = faces2 != nullptr;
  G->rel_cut = op.rel_cutoff;
  G->abs_cut = op.abs_cutoff;
  mnpbem_status s = geometry_build(G->g, G->b, verts, nverts, faces, faces2, nfaces, cs.data(), ce.data(),
                                   (int)cs.size(), quad, op.rel_cutoff, op.abs_cutoff, G->st);
  if (s == MNPBEM_OK) s = G->face_med.ensure(sizeof(int) * 2 * nfaces);
  if (s == MNPBEM_OK) {
    std::vector<int> fm(2 * nfaces);
    for (int64_t k = 0; k < nfaces; ++k) {
      fm[k] = G->inout[2 * G->face_part[k]] - 1;
      fm[nfaces + k] = G->inout[2 * G->face_part[k] + 1] - 1;
    }
    if (cudaMemcpy(G->face_med.ptr, fm.data(), sizeof(int) * 2 * nfaces, cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      set_error("geometry set-up: upload of face media failed");
      s = MNPBEM_ERR_CUDA;
    }
  }
  if (s == MNPBEM_OK) s = add_lane(G);
  if (s == MNPBEM_OK) s = G->d_part.ensure(sizeof(int) * nfaces);
  if (s == MNPBEM_OK) s = G->d_src.ensure(sizeof(double4_32a) * nfaces);
  if (s == MNPBEM_OK) s = G->d_nrm.ensure(sizeof(double4_32a) * nfaces);
  if (s == MNPBEM_OK) s = G->d_srcf.ensure(sizeof(float4) * 2 * nfaces);
  if (s == MNPBEM_OK) s = G->d_nrmf.ensure(sizeof(float4) * 2 * nfaces);
  if (s == MNPBEM_OK) {
    if (cudaMemcpyAsync(G->d_part.ptr, G->face_part.data(), sizeof(int) * nfaces,
                        cudaMemcpyHostToDevice, G->st) != cudaSuccess) {
      set_error("upload of particle index failed");
      s = MNPBEM_ERR_CUDA;
    } else {
      pack_sources((int)nfaces, G->g.pos, G->g.area, G->g.nvec, G->d_src.as<double4_32a>(),
                   G->d_nrm.as<double4_32a>(), G->d_srcf.as<float4>(), G->d_nrmf.as<float4>(), G->st);
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
  const char* genv = getenv("MNPBEM_GRAPHS");
  if (genv && genv[0] == '0') G->use_graphs = false;
  const char* dsenv = getenv("MNPBEM_ASM_DS");
  if (dsenv && dsenv[0] == '0') G->asm_ds = false;
  const char* rnaenv = getenv("MNPBEM_TF32_RNA");
  if (rnaenv && rnaenv[0] == '0') G->tf32_rna = false;
  const char* gjfenv = getenv("MNPBEM_GJ_FUSED");
  if (gjfenv && gjfenv[0] == '0') G->gj_fused = false;
  const char* nbenv = getenv("MNPBEM_GJ_NB");
  if (nbenv && atoi(nbenv) == 512) G->gj_nb = 512;
  const char* f16env = getenv("MNPBEM_TC_F16");
  if (f16env && f16env[0] == '0') G->tc_f16 = false;
  const char* luenv = getenv("MNPBEM_LU_STEPS");
  if (luenv && (atoi(luenv) == 1 || atoi(luenv) == 2 || atoi(luenv) == 4)) G->lu_steps = atoi(luenv);
  const char* lenv = getenv("MNPBEM_LANES");
  if (lenv && atoi(lenv) > 0) G->lanes_req = std::min(MAX_LANES, atoi(lenv));
  const char* swenv = getenv("MNPBEM_SWEEP_GRAPH");
  if (swenv && swenv[0] == '0') G->sweep_graph = false;
  *out = G;
  return MNPBEM_OK;
}

mnpbem_status mnpbem_geom_create(const double* verts, int64_t nverts, const int64_t* faces,
                                 int64_t nfaces, int32_t nparts, const int64_t* part_nfaces,
                                 const int32_t* inout, const int32_t* closed,
                                 const mnpbem_quad* quad, const mnpbem_options* opts,
                                 mnpbem_geom** out) {
  return geom_create_impl(verts, nverts, faces, nullptr, nfaces, nparts, part_nfaces, inout, closed, quad,
                          opts, out);
}

mnpbem_status mnpbem_geom_create_curved(const double* verts2, int64_t nverts2, const int64_t* faces2,
                                        int64_t nfaces, int32_t nparts, const int64_t* part_nfaces,
                                        const int32_t* inout, const int32_t* closed,
                                        const mnpbem_quad* quad, const mnpbem_options* opts,
                                        mnpbem_geom** out) {
  if (!faces2 || nfaces <= 0 || nverts2 <= 0) {
    set_error("mnpbem_geom_create_curved: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  // corners for the flat-element bookkeeping (bradius, face lists); the curved
  // nodes must all exist: triangles use columns 0-2 and 4-6, quadrilaterals 0-8
  std::vector<int64_t> corners(4 * (size_t)nfaces);
  for (int64_t k = 0; k < nfaces; ++k) {
    const int64_t* f = faces2 + 9 * k;
    const bool quad4 = f[3] >= 0;
    for (int c = 0; c < 9; ++c) {
      const bool used = c < 3 || (c >= 4 && c <= 6) || (quad4 && (c == 3 || c == 7 || c == 8));
      const int64_t v = f[c];
      if ((used && (v < 0 || v >= nverts2)) || (!used && v != -1 && (v < 0 || v >= nverts2))) {
        set_error("curved face %lld has an invalid node index in column %d", (long long)k, c);
        return MNPBEM_ERR_INVALID_ARG;
      }
    }
    for (int c = 0; c < 4; ++c) corners[4 * k + c] = f[c];
  }
  return geom_create_impl(verts2, nverts2, corners.data(), faces2, nfaces, nparts, part_nfaces, inout, closed,
                          quad, opts, out);
}

mnpbem_status mnpbem_geom_destroy(mnpbem_geom* g) {
  if (!g) return MNPBEM_OK;
  cudaSetDevice(g->device);
  if (g->st) cudaStreamSynchronize(g->st);
  g->prof.flush();
  if (g->sweep_exec) cudaGraphExecDestroy(g->sweep_exec);
  g->sweep_exec = nullptr;
  for (auto& L : g->lanes) lane_release(*L);
  g->lanes.clear();
  if (g->lp_ring) cudaFreeHost(g->lp_ring);
  if (g->st) cudaStreamDestroy(g->st);
  delete g;
  return MNPBEM_OK;
}

mnpbem_status mnpbem_geom_set_lanes(mnpbem_geom* g, int32_t lanes) {
  MNP_TRY(check_geom(g));
  if (lanes < 0 || lanes > MAX_LANES) {
    set_error("lanes must be 0 (automatic) .. %d", MAX_LANES);
    return MNPBEM_ERR_INVALID_ARG;
  }
  g->lanes_req = lanes;
  return MNPBEM_OK;
}

mnpbem_status mnpbem_geom_set_option(mnpbem_geom* g, const char* key, int32_t value) {
  MNP_TRY(check_geom(g));
  if (!key) { set_error("null option name"); return MNPBEM_ERR_INVALID_ARG; }
  const std::string k(key);
  if (k == "lanes") return mnpbem_geom_set_lanes(g, value);
  if (k == "gj_block" && (value == 256 || value == 512)) { g->gj_nb = value; return MNPBEM_OK; }
  if (k == "tc_stages" && (value == 3 || value == 4)) {
    g->tc_stages = value;
    for (auto& L : g->lanes) L->tc.stages = value;
    return MNPBEM_OK;
  }
  if (k == "tc_pair" && value == 0) {
    g->tc_pair = 0;
    for (auto& L : g->lanes) L->tc.pair = 0;
    return MNPBEM_OK;
  }
  if (k == "tc_pair" && (value == 1 || value == -1)) {
    // a four-lane sweep with the CTA-pair GEMM once ran until its time limit
    // without a recorded cause; the sweep keeps the single-CTA kernel until the
    // cause is known (the pair kernel stays available to mnpbem_gemm_c64)
    set_error("tc_pair: the CTA-pair GEMM is not enabled inside sweeps");
    return MNPBEM_ERR_UNSUPPORTED;
  }
  if (k == "lu_steps" && (value == 1 || value == 2 || value == 4)) { g->lu_steps = value; return MNPBEM_OK; }
  if (k == "tc_f16" && (value == 0 || value == 1)) {
    g->tc_f16 = value != 0;
    for (auto& L : g->lanes) L->tc.f16 = g->tc_f16;
    return MNPBEM_OK;
  }
  if (k == "tc_ctas" && value >= 0 && value <= 4096) {
    g->tc_ctas = value;
    for (auto& L : g->lanes) L->tc.max_ctas = value;
    return MNPBEM_OK;
  }
  if (k == "sweep_graph" && (value == 0 || value == 1)) { g->sweep_graph = value != 0; return MNPBEM_OK; }
  if (k == "tf32_round" && (value == 0 || value == 1)) { g->tf32_rna = value != 0; return MNPBEM_OK; }
  if (k == "assembly_ds" && (value == 0 || value == 1)) { g->asm_ds = value != 0; return MNPBEM_OK; }
  set_error("unknown option '%s' or value %d out of range", key, value);
  return MNPBEM_ERR_INVALID_ARG;
}

mnpbem_status mnpbem_geom_stat(mnpbem_geom* g, const char* key, double* value) {
  MNP_TRY(check_geom(g));
  if (!key || !value) { set_error("mnpbem_geom_stat: invalid arguments"); return MNPBEM_ERR_INVALID_ARG; }
  const std::string k(key);
  if (k == "block_cond_max") {
    float c = 0.f;
    for (auto& L : g->lanes) c = std::max(c, L->cond_max);
    *value = c;
    return MNPBEM_OK;
  }
  if (k == "block_cond_reset") {
    for (auto& L : g->lanes) L->cond_max = 0.f;
    *value = 0.0;
    return MNPBEM_OK;
  }
  if (k == "g1_blocks") {
    *value = (double)g->g1_off.size();
    return MNPBEM_OK;
  }
  if (k == "sweep_graph_runs") {
    *value = (double)g->sweep_runs;
    return MNPBEM_OK;
  }
  if (k == "sweep_graph_error") {   // CUDA error that turned the one-graph sweep off (0: none)
    *value = (double)g->sweep_err;
    return MNPBEM_OK;
  }
  if (k == "stage_graphs") {        // stages replayed from captured graphs (0: run directly)
    *value = g->use_graphs ? 1.0 : 0.0;
    return MNPBEM_OK;
  }
  set_error("mnpbem_geom_stat: unknown key '%s'", key);
  return MNPBEM_ERR_INVALID_ARG;
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
      (precision != MNPBEM_FP64 && precision != MNPBEM_FP32 && precision != MNPBEM_MIXED)) {
    set_error("mnpbem_assemble: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  Lane& L = *G->lanes[0];
  {
    LamParams lp{};
    for (int m = 0; m < nmed; ++m) lp.k[m] = make_double2(k_media[2 * m], k_media[2 * m + 1]);
    MNP_CUDA(cudaMemcpyAsync(L.lp_dev.ptr, &lp, sizeof(lp), cudaMemcpyHostToDevice, G->st));
    MNP_CUDA(cudaStreamSynchronize(G->st));
  }
  AsmParams p = base_params(G, L.lp_dev.as<LamParams>());
  const int64_t n = G->g.n;
  if (precision == MNPBEM_MIXED) {
    // the mixed-precision pass (double-single far field, hi / lo planes), returned as hi + lo
    DevBuf work, planes, out;
    MNP_TRY(work.ensure(sizeof(float2) * 4 * n * n));
    MNP_TRY(planes.ensure(sizeof(float2) * 8 * n * n));
    MNP_TRY(out.ensure(sizeof(double2) * n * n));
    float2* w = work.as<float2>();
    float2* pl = planes.as<float2>();
    p.ld32 = n;
    p.g1 = w; p.h1 = w + n * n; p.g2 = w + 2 * n * n; p.h2 = w + 3 * n * n;
    p.G1hi = pl; p.G1lo = pl + n * n; p.H1hi = pl + 2 * n * n; p.H1lo = pl + 3 * n * n;
    p.G2hi = pl + 4 * n * n; p.G2lo = pl + 5 * n * n; p.H2hi = pl + 6 * n * n; p.H2lo = pl + 7 * n * n;
    p.ds = G->asm_ds;
    MNP_TRY(assemble_launch(p, true, true, G->st));
    void* hosts[4] = {G1, H1, G2, H2};
    for (int q = 0; q < 4; ++q) {
      if (!hosts[q]) continue;
      hilo_to_c128(pl + 2 * q * n * n, pl + (2 * q + 1) * n * n, out.as<double2>(), n * n, G->st);
      MNP_CHECK_LAUNCH();
      MNP_CUDA(cudaMemcpyAsync(hosts[q], out.ptr, sizeof(double2) * n * n, cudaMemcpyDeviceToHost, G->st));
      MNP_CUDA(cudaStreamSynchronize(G->st));
    }
    return MNPBEM_OK;
  }
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
      ldc < N || path < 0 || path > 4) {
    set_error("mnpbem_gemm_c64: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  MNP_CUDA(cudaSetDevice(device));
  static TcGemmCtx tc[64];
  if (device < 0 || device >= 64) { set_error("invalid device"); return MNPBEM_ERR_INVALID_ARG; }
  // A, B, C all in device memory: the product runs on them on the default
  // stream, without copies; otherwise host arrays go through device buffers
  auto on_device = [](const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
  };
  const bool dev = on_device(A) && on_device(B) && on_device(C);
  cudaStream_t st = nullptr;
  if (!dev) MNP_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { if (s) cudaStreamDestroy(s); } } sg{st};
  DevBuf dA, dB, dC;
  const float2 *pA = reinterpret_cast<const float2*>(A), *pB = reinterpret_cast<const float2*>(B);
  float2* pC = reinterpret_cast<float2*>(C);
  if (!dev) {
    MNP_TRY(dA.ensure(sizeof(float2) * M * lda));
    MNP_TRY(dB.ensure(sizeof(float2) * K * ldb));
    MNP_TRY(dC.ensure(sizeof(float2) * M * ldc));
    MNP_CUDA(cudaMemcpyAsync(dA.ptr, A, sizeof(float2) * M * lda, cudaMemcpyHostToDevice, st));
    MNP_CUDA(cudaMemcpyAsync(dB.ptr, B, sizeof(float2) * K * ldb, cudaMemcpyHostToDevice, st));
    MNP_CUDA(cudaMemcpyAsync(dC.ptr, C, sizeof(float2) * M * ldc, cudaMemcpyHostToDevice, st));
    pA = dA.as<float2>();
    pB = dB.as<float2>();
    pC = dC.as<float2>();
  }
  const float2 al = make_float2(alpha[0], alpha[1]), be = make_float2(beta[0], beta[1]);
  if (path >= 1) {
    tc[device].pair = (path == 2 || path == 3) ? 1 : 0;
    tc[device].pair_epi = path == 3 ? 1 : 0;
    tc[device].f16 = path == 4;
    tc[device].f16_min_k = 1;
    tc[device].f16_min_mn = 1;
    if (!tc_gemm_eligible(tc[device], M, N, K, pA, lda, pC, ldc, be)) {
      set_error("tensor-core GEMM not available for this device or shape");
      return MNPBEM_ERR_UNSUPPORTED;
    }
    MNP_TRY(tc_gemm_c64(tc[device], M, N, K, al, pA, lda, pB, ldb, be, pC, ldc, st));
    if (!dev) MNP_TRY(tc_check_error(tc[device], st));
  } else {
    MNP_TRY(gemm_simt<float>(M, N, K, al, pA, lda, pB, ldb, be, pC, ldc, st));
  }
  if (!dev) {
    MNP_CUDA(cudaMemcpyAsync(C, dC.ptr, sizeof(float2) * M * ldc, cudaMemcpyDeviceToHost, st));
    MNP_CUDA(cudaStreamSynchronize(st));
  }
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
// The work of one wavelength is split into stages that depend on the
// wavelength only through the lane's device parameter block lp_dev:
//   S0 assemble        per-face eps + G1, H1, G2, H2 (complex64 and/or complex128)
//   S1 initmat         inversions, products, Sigma stage
//   S2 first solve     excitation + mldivide chain (+ conversions)
//   S3 refinement step FP64 residual of the full operator + chain + update (MIXED)
//   S4 spectra         far fields + extinction / scattering into a fixed slot
// The first wavelength a lane runs for a configuration goes through the
// stages directly (sizing every buffer); the lane then captures each stage as
// a CUDA graph and replays the graphs for its later wavelengths.
namespace {

struct SolveCtx {
  int P;
  int precision;
  const mnpbem_planewave* exc;
  const double2* ext_pot = nullptr;   // external potentials instead of the plane wave (device)
  bool spectra = true;                // far fields and cross sections of the plane wave
};

size_t lane_bytes_estimate(const mnpbem_geom* G, int precision, int P, int ninf) {
  const size_t n = G->g.n, ld = G->ld;
  const size_t es = precision == MNPBEM_FP64 ? sizeof(double2) : sizeof(float2);
  size_t b = 5 * es * n * ld;
  // hi / lo planes, B' of the rank-1024 products and the LDU panels
  if (precision == MNPBEM_MIXED) b += 4 * 2 * sizeof(float2) * n * ld + 3 * 8 * 1024 * n;
  b += sizeof(double2) * n * P * 80 + sizeof(float2) * n * P * 56;
  b += 3 * es * n * 256 + sizeof(double2) * (size_t)(P + ninf) * 6 * P + 64 * n;
  return b;
}

mnpbem_status ensure_workspace(mnpbem_geom* G, Lane& L, int precision, int P, int ninf) {
  const int64_t n = G->g.n, ld = G->ld;
  const size_t es = precision == MNPBEM_FP64 ? sizeof(double2) : sizeof(float2);
  for (int q = 0; q < 5; ++q) MNP_TRY(L.mat[q].ensure(es * n * ld));
  if (precision == MNPBEM_MIXED)
    for (int q = 0; q < 4; ++q) MNP_TRY(L.mat64[q].ensure(2 * sizeof(float2) * n * ld));
  // FP64 vectors: b (8nP) x (8nP) r (8nP) YZ (16nP) + chain work for FP64 (32nP)
  MNP_TRY(L.vec64.ensure(sizeof(double2) * n * P * (8 + 8 + 8 + 16 + 32 + 8)));
  // working-precision vectors for MIXED: in (8nP) out (8nP) work (32nP)
  MNP_TRY(L.vecw.ensure(sizeof(float2) * n * P * (8 + 8 + 32)));
  MNP_TRY(L.norms.ensure(sizeof(double) * 4));
  MNP_TRY(L.bsplit.ensure(sizeof(float2) * 2 * n * 4 * P));
  MNP_TRY(L.facebuf.ensure(sizeof(double2) * 2 * n + sizeof(float2) * 3 * n + sizeof(float) * 3 * n + 2 * n + 256));
  MNP_TRY(L.fields.ensure(sizeof(double2) * (size_t)(P + ninf) * 6 * P));
  MNP_TRY(L.outbuf.ensure(sizeof(double) * 2 * P));   // ext / sca slot of the current wavelength
  return MNPBEM_OK;
}

// fingerprint of every device address a lane's graphs capture
uint64_t lane_sig(const mnpbem_geom* G, const Lane& L) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](const void* p, size_t b) {
    h = (h ^ (uint64_t)(uintptr_t)p) * 1099511628211ull;
    h = (h ^ (uint64_t)b) * 1099511628211ull;
  };
  auto mixbuf = [&](const DevBuf& d) { mix(d.ptr, d.bytes); };
  for (int q = 0; q < 5; ++q) mixbuf(L.mat[q]);
  for (int q = 0; q < 4; ++q) mixbuf(L.mat64[q]);
  mixbuf(L.vec64); mixbuf(L.vecw); mixbuf(L.facebuf); mixbuf(L.fields); mixbuf(L.norms);
  mixbuf(L.outbuf); mixbuf(L.bsplit); mixbuf(L.lp_dev); mixbuf(G->exbuf);
  mixbuf(L.tc.bexp); mixbuf(L.tc.err);
  auto gj = [&](const auto& w) {
    mixbuf(w.ccol); mixbuf(w.rrow); mixbuf(w.ncol); mixbuf(w.xblk); mixbuf(w.status);
    mix(nullptr, (size_t)w.nb);
    if (w.inner) {
      mixbuf(w.inner->ccol); mixbuf(w.inner->rrow); mixbuf(w.inner->ncol); mixbuf(w.inner->xblk);
      mixbuf(w.inner->status);
    }
  };
  gj(L.gj32);
  gj(L.gj64);
  auto lu = [&](const auto& w) {
    mixbuf(w.ccol); mixbuf(w.rrow); mixbuf(w.xblk); mixbuf(w.tmp);
    mix(nullptr, (size_t)w.b);
    mix(nullptr, (size_t)w.m);
  };
  lu(L.lu32);
  lu(L.lu64);
  mixbuf(L.lu_status);
  mixbuf(L.lu_bar);
  mix(nullptr, (size_t)G->lu_steps);
  mix(nullptr, (size_t)G->gj_nb);
  mix(L.status_host, 0);
  mix(L.norms_host, 0);
  // tuning options baked into the captured launches
  mix(nullptr, (size_t)L.tc.stages);
  mix(nullptr, (size_t)L.tc.max_ctas);
  mix(nullptr, (size_t)(L.tc.pair + 1));
  mix(nullptr, (size_t)L.tc.f16);
  mix(nullptr, (size_t)G->tf32_rna);
  mix(nullptr, (size_t)G->asm_ds);
  mix(nullptr, (size_t)G->gj_fused);
  return h;
}

FaceData face_data_in(mnpbem_geom* G, DevBuf& buf) {
  const int64_t n = G->g.n;
  FaceData f;
  f.n = n;
  f.pos = G->g.pos;
  f.nvec = G->g.nvec;
  f.area = G->g.area;
  double2* e = buf.as<double2>();
  f.eps1 = e;
  f.eps2 = e + n;
  float2* ef = reinterpret_cast<float2*>(e + 2 * n);
  f.eps1f = ef;
  f.eps2f = ef + n;
  f.Lf = ef + 2 * n;
  f.nvecf = reinterpret_cast<const float*>(ef + 3 * n);
  f.exc_in = reinterpret_cast<const unsigned char*>(f.nvecf + 3 * n);
  f.exc_out = f.exc_in + n;
  return f;
}
FaceData face_data(mnpbem_geom* G, Lane& L) { return face_data_in(G, L.facebuf); }

mnpbem_status upload_masks(mnpbem_geom* G, Lane& L, const std::vector<unsigned char>& m) {
  unsigned char* dst = const_cast<unsigned char*>(face_data(G, L).exc_in);
  MNP_CUDA(cudaMemcpyAsync(dst, m.data(), m.size(), cudaMemcpyHostToDevice, L.st));
  MNP_CUDA(cudaStreamSynchronize(L.st));
  return MNPBEM_OK;
}

template <typename R>
GJWork<R>& gjw(Lane& L);
template <> GJWork<float>& gjw<float>(Lane& L) { return L.gj32; }
template <> GJWork<double>& gjw<double>(Lane& L) { return L.gj64; }

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

template <typename R>
LDUWork<R>& luw(Lane& L);
template <> LDUWork<float>& luw<float>(Lane& L) { return L.lu32; }
template <> LDUWork<double>& luw<double>(Lane& L) { return L.lu64; }

void* tc_ctx(mnpbem_geom* G, Lane& L) { return G->tc_enabled ? (void*)&L.tc : nullptr; }

// rows of the diagonal blocks of the LDU factors: 256 on the tensor-core path
// (cluster block inverse), else 64 (single-CTA block inverse with pivoting)
template <typename R>
int lu_block(const mnpbem_geom* G, void* ctx) {
  return (sizeof(R) == 4 && ctx && G->g.n >= 1024) ? 256 : 64;
}

// Lane matrices after initmat: mat[0] LDU(G1), mat[1] LDU(G2), mat[2] Sigma1,
// mat[3] LDU(Sigma), mat[4] Deltai
template <typename R>
ChainMats<R> chain_mats(mnpbem_geom* G, Lane& L) {
  using Cx = cplx<R>;
  ChainMats<R> m;
  m.G1 = L.mat[0].as<Cx>();
  m.G2 = L.mat[1].as<Cx>();
  m.Sigma1 = L.mat[2].as<Cx>();
  m.Sigma = L.mat[3].as<Cx>();
  m.Deltai = L.mat[4].as<Cx>();
  m.ld = G->ld;
  m.b = lu_block<R>(G, sizeof(R) == 4 ? tc_ctx(G, L) : nullptr);
  m.bar = L.lu_bar.as<unsigned>();
  m.ng1 = (int)G->g1_off.size();
  for (int q = 0; q < m.ng1; ++q) {
    m.g1_off[q] = G->g1_off[q];
    m.g1_n[q] = G->g1_n[q];
  }
  return m;
}

// ---------------------------------------------------------------- S0
mnpbem_status stage_assemble(mnpbem_geom* G, Lane& L, int precision) {
  const int64_t n = G->g.n, ld = G->ld;
  L.pc_valid = false;   // mat[] is about to be overwritten
  const int* fm = G->face_med.as<int>();
  FaceData f = face_data(G, L);
  const LamParams* lp = L.lp_dev.as<LamParams>();
  launch_face_eps(n, fm, fm + n, lp, G->g.nvec, const_cast<double2*>(f.eps1),
                  const_cast<double2*>(f.eps2), const_cast<float2*>(f.eps1f), const_cast<float2*>(f.eps2f),
                  const_cast<float2*>(f.Lf), const_cast<float*>(f.nvecf), L.st);
  MNP_CHECK_LAUNCH();
  AsmParams p = base_params(G, lp);
  if (precision == MNPBEM_FP64) {
    p.ld64 = ld;
    p.G1 = L.mat[0].as<double2>(); p.G2 = L.mat[1].as<double2>();
    p.H1 = L.mat[2].as<double2>(); p.H2 = L.mat[3].as<double2>();
    return assemble_launch(p, true, false, L.st);
  }
  p.ld32 = ld;
  p.g1 = L.mat[0].as<float2>(); p.g2 = L.mat[1].as<float2>();
  p.h1 = L.mat[2].as<float2>(); p.h2 = L.mat[3].as<float2>();
  // residual matrices as hi / lo complex64 planes (mat64[q]: hi [n][ld] then lo [n][ld])
  float2* hl[4];
  for (int q = 0; q < 4; ++q) hl[q] = L.mat64[q].as<float2>();
  p.G1hi = hl[0]; p.G1lo = hl[0] + n * ld;
  p.H1hi = hl[1]; p.H1lo = hl[1] + n * ld;
  p.G2hi = hl[2]; p.G2lo = hl[2] + n * ld;
  p.H2hi = hl[3]; p.H2lo = hl[3] + n * ld;
  p.ds = G->asm_ds;
  return assemble_launch(p, true, true, L.st);
}

// ---------------------------------------------------------------- S1
// initmat.m:27-72 with block LDU factors in place of the inverses of G1, G2
// and Sigma (real FLOP per wavelength: 8/3 n^3 per factorisation, 8 n^3 per
// right-side solve, 8 n^3 for the Gauss-Jordan inverse of Delta; with G1
// block-diagonal its factorisation and solve cost the sum over its blocks).
template <typename R>
mnpbem_status stage_initmat(mnpbem_geom* G, Lane& L, bool direct) {
  using Cx = cplx<R>;
  const int64_t n = G->g.n, ld = G->ld;
  Cx* M[5];
  for (int q = 0; q < 5; ++q) M[q] = L.mat[q].as<Cx>();
  void* ctx = sizeof(R) == 4 ? tc_ctx(G, L) : nullptr;
  // wider Gauss-Jordan steps when the rank-nb updates run on tensor cores:
  // fewer passes over the n x n matrix (each step reads and writes it once)
  // By size (measured on GB300, 24 000-face dimer: rank-1024 LDU updates and
  // 512-wide Gauss-Jordan steps 1.365 against 1.265 wavelength-solves/s for
  // rank-512 / 256-wide; at 4000 faces the 256-wide steps were faster)
  const bool large = n >= 12000;
  gjw<R>(L).nb = (ctx && n >= 1024) ? (G->gj_nb ? G->gj_nb : (large ? 512 : 256)) : 64;
  gjw<R>(L).round_a = G->tf32_rna;
  gjw<R>(L).fused = G->gj_fused;
  LDUWork<R>& lw = luw<R>(L);
  lw.b = lu_block<R>(G, ctx);
  lw.m = lw.b == 256 ? (G->lu_steps ? G->lu_steps : (large ? 4 : 2)) : 1;
  lw.round_a = G->tf32_rna;
  int* lus = L.lu_status.as<int>();
  MNP_CUDA(cudaMemsetAsync(lus, 0, 2 * sizeof(int), L.st));
  const FaceData fd = face_data(G, L);
  const LamParams* lp = L.lp_dev.as<LamParams>();
  // G1 = LDU per diagonal block, Sigma1 = H1 G1^-1 (H1 shares G1's blocks:
  // its off-diagonal blocks are zero and stay zero)
  for (size_t q = 0; q < G->g1_off.size(); ++q) {
    const int64_t o = G->g1_off[q], nq = G->g1_n[q];
    MNP_TRY(ldu_factor<R>(M[0] + o * ld + o, nq, ld, lw, lus, gemm_w<R>, ctx, L.st));
    MNP_TRY(ldu_rsolve<R>(M[2] + o * ld + o, nq, ld, M[0] + o * ld + o, ld, lw, gemm_w<R>, ctx, L.st));
  }
  // G2 = LDU, Sigma2 = H2 G2^-1
  MNP_TRY(ldu_factor<R>(M[1], n, ld, lw, lus, gemm_w<R>, ctx, L.st));
  MNP_TRY(ldu_rsolve<R>(M[3], n, ld, M[1], ld, lw, gemm_w<R>, ctx, L.st));
  // Delta -> M4, Sigma (partial) -> M3
  launch_delta_sigma<R>(n, M[2], M[3], M[4], ld, fd, L.st);
  MNP_CHECK_LAUNCH();
  MNP_TRY(gj_invert<R>(M[4], n, ld, gjw<R>(L), gemm_w<R>, ctx, L.st, direct));
  launch_sigma_add<R>(n, M[3], M[4], ld, fd, lp, L.st);
  MNP_CHECK_LAUNCH();
  MNP_TRY(ldu_factor<R>(M[3], n, ld, lw, lus, gemm_w<R>, ctx, L.st));
  if (direct) {
    int hs[2] = {0, 0};
    MNP_CUDA(cudaMemcpyAsync(hs, lus, sizeof(hs), cudaMemcpyDeviceToHost, L.st));
    MNP_CUDA(cudaStreamSynchronize(L.st));
    if (hs[0]) {
      set_error("block LDU factorisation: zero or non-finite pivot in a diagonal block");
      return MNPBEM_ERR_SINGULAR;
    }
  }
  if (direct && ctx) MNP_TRY(tc_check_error(L.tc, L.st));
  if (direct) MNP_TRY(thin_stream_check(L.st));
  return MNPBEM_OK;
}

// FP64 vector arena layout
struct Vec64 {
  double2 *phi, *a, *alpha, *De, *x1, *x2, *rphi, *ra, *ral, *rDe, *Y1, *Y2, *Z1, *Z2, *work, *d1, *d2;
};
Vec64 vec64(const mnpbem_geom* G, Lane& L, int P) {
  const int64_t n = G->g.n;
  Vec64 v;
  double2* V = L.vec64.as<double2>();
  v.phi = V; v.a = v.phi + n * P; v.alpha = v.a + 3 * n * P; v.De = v.alpha + 3 * n * P;
  v.x1 = v.De + n * P; v.x2 = v.x1 + 4 * n * P;
  v.rphi = v.x2 + 4 * n * P; v.ra = v.rphi + n * P; v.ral = v.ra + 3 * n * P; v.rDe = v.ral + 3 * n * P;
  v.Y1 = v.rDe + n * P; v.Y2 = v.Y1 + 4 * n * P; v.Z1 = v.Y2 + 4 * n * P; v.Z2 = v.Z1 + 4 * n * P;
  v.work = v.Z2 + 4 * n * P;
  v.d1 = v.work + 32 * n * P;   // last correction in FP64 (incremental residual)
  v.d2 = v.d1 + 4 * n * P;
  return v;
}

// complex64 chain applied to FP64 inputs, result in fx1/fx2 (per-face data
// and parameters fd / lp: those of the wavelength the matrices belong to)
mnpbem_status apply32_at(mnpbem_geom* G, Lane& L, int P, const FaceData& fd, const LamParams* lp,
                         const double2* p_, const double2* a_, const double2* al_, const double2* De_) {
  const int64_t n = G->g.n;
  cudaStream_t st = L.st;
  float2* W = L.vecw.as<float2>();
  float2 *fphi = W, *fa = fphi + n * P, *fal = fa + 3 * n * P, *fDe = fal + 3 * n * P;
  float2 *fx1 = fDe + n * P, *fx2 = fx1 + 4 * n * P, *fwork = fx2 + 4 * n * P;
  launch_cvt_d2f(p_, fphi, n * P, st);
  launch_cvt_d2f(a_, fa, 3 * n * P, st);
  launch_cvt_d2f(al_, fal, 3 * n * P, st);
  launch_cvt_d2f(De_, fDe, n * P, st);
  MNP_CHECK_LAUNCH();
  return apply_mldivide<float>(fd, P, lp, chain_mats<float>(G, L), fphi, fa, fal, fDe, fx1, fx2, fwork,
                               gemm_w<float>, tc_ctx(G, L), st);
}
mnpbem_status apply32(mnpbem_geom* G, Lane& L, int P, const double2* p_, const double2* a_,
                      const double2* al_, const double2* De_) {
  return apply32_at(G, L, P, face_data(G, L), L.lp_dev.as<LamParams>(), p_, a_, al_, De_);
}
float2* fx_ptr(const mnpbem_geom* G, Lane& L, int P, int which) {
  const int64_t n = G->g.n;
  return L.vecw.as<float2>() + 8 * n * P + (which ? 4 * n * P : 0);
}

// ---------------------------------------------------------------- S2
mnpbem_status stage_first(mnpbem_geom* G, Lane& L, const SolveCtx& c) {
  const int64_t n = G->g.n;
  const int P = c.P;
  Vec64 v = vec64(G, L, P);
  const double* pol = G->exbuf.as<double>();
  const double* dirs = pol + 3 * P;
  const LamParams* lp = L.lp_dev.as<LamParams>();
  const FaceData fd = face_data(G, L);
  if (c.ext_pot)
    launch_excitation_ext(fd, P, c.ext_pot, lp, v.phi, v.a, v.alpha, v.De, L.st);
  else
    launch_excitation(fd, P, pol, dirs, lp, v.phi, v.a, v.alpha, v.De, L.st);
  MNP_CHECK_LAUNCH();
  if (c.precision == MNPBEM_FP64)
    return apply_mldivide<double>(fd, P, lp, chain_mats<double>(G, L), v.phi, v.a, v.alpha, v.De, v.x1, v.x2,
                                  v.work, gemm_w<double>, nullptr, L.st);
  MNP_TRY(apply32(G, L, P, v.phi, v.a, v.alpha, v.De));
  launch_cvt_f2d(fx_ptr(G, L, P, 0), v.x1, 4 * n * P, L.st);
  launch_cvt_f2d(fx_ptr(G, L, P, 1), v.x2, 4 * n * P, L.st);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

// Y = G1 x, Z = H1 x from the hi (and, with ds, lo) planes, one product per
// diagonal block of G1 and H1 (their off-diagonal blocks are zero)
mnpbem_status residual_g1h1(mnpbem_geom* G, const float2* const* hl, bool ds, const double2* x, double2* Y,
                            double2* Z, int N, float2* bs, cudaStream_t st) {
  const int64_t n = G->g.n, ld = G->ld;
  for (size_t q = 0; q < G->g1_off.size(); ++q) {
    const int64_t o = G->g1_off[q], nq = G->g1_n[q], off = o * ld + o;
    MNP_TRY(gemm_thin_ds(nq, N, nq, hl[0] + off, ds ? hl[0] + n * ld + off : nullptr, ld, x + o * N, N, Y + o * N, N,
                         bs, st));
    MNP_TRY(gemm_thin_ds(nq, N, nq, hl[1] + off, ds ? hl[1] + n * ld + off : nullptr, ld, x + o * N, N, Z + o * N, N,
                         bs, st));
  }
  return MNPBEM_OK;
}

// ---------------------------------------------------------------- S3 / S5
// norms[0..1] = ||r||^2, ||b||^2 ; norms[2..3] = ||dx||^2, ||x||^2
// ds: residual products in double-single arithmetic from the hi / lo planes
// (S3); otherwise FP32 products of the hi planes (S5), enough while the
// residual is still large compared with their rounding error.
mnpbem_status stage_iter(mnpbem_geom* G, Lane& L, const SolveCtx& c, bool ds) {
  const int64_t n = G->g.n;
  const int P = c.P;
  cudaStream_t st = L.st;
  Vec64 v = vec64(G, L, P);
  const int64_t ld = G->ld;
  const float2* hl[4];
  for (int q = 0; q < 4; ++q) hl[q] = L.mat64[q].as<float2>();
  double* norms = L.norms.as<double>();
  // G1 x1, H1 x1 (per diagonal block of G1 and H1), G2 x2, H2 x2
  float2* bs = L.bsplit.as<float2>();
  auto lo = [&](int q) -> const float2* { return ds ? hl[q] + n * ld : nullptr; };
  MNP_TRY(residual_g1h1(G, hl, ds, v.x1, v.Y1, v.Z1, 4 * P, bs, st));
  MNP_TRY(gemm_thin_ds(n, 4 * P, n, hl[2], lo(2), ld, v.x2, 4 * P, v.Y2, 4 * P, bs, st));
  MNP_TRY(gemm_thin_ds(n, 4 * P, n, hl[3], lo(3), ld, v.x2, 4 * P, v.Z2, 4 * P, bs, st));
  MNP_CUDA(cudaMemsetAsync(norms, 0, sizeof(double) * 4, st));
  launch_residual(face_data(G, L), P, L.lp_dev.as<LamParams>(), v.Y1, v.Y2, v.Z1, v.Z2, v.phi, v.a, v.alpha,
                  v.De, v.rphi, v.ra, v.ral, v.rDe, norms, st);
  MNP_CHECK_LAUNCH();
  MNP_TRY(apply32(G, L, P, v.rphi, v.ra, v.ral, v.rDe));
  launch_axpy_norm(v.x1, fx_ptr(G, L, P, 0), 4 * n * P, norms + 2, st);
  launch_axpy_norm(v.x2, fx_ptr(G, L, P, 1), 4 * n * P, norms + 2, st);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

// ---------------------------------------------------------------- S6
// incremental refinement step: r <- r - A dx with the last correction dx and
// FP32 products of the hi planes (their rounding, ~1e-7 of |A| |dx|, shrinks
// with dx), then the complex64 chain and x += dx'.  Used after the first full
// residual; one double-single residual in between anchors the accuracy.
mnpbem_status stage_incr(mnpbem_geom* G, Lane& L, const SolveCtx& c) {
  const int64_t n = G->g.n;
  const int P = c.P;
  cudaStream_t st = L.st;
  Vec64 v = vec64(G, L, P);
  const int64_t ld = G->ld;
  const float2* hl[4];
  for (int q = 0; q < 4; ++q) hl[q] = L.mat64[q].as<float2>();
  double* norms = L.norms.as<double>();
  launch_cvt_f2d(fx_ptr(G, L, P, 0), v.d1, 4 * n * P, st);
  launch_cvt_f2d(fx_ptr(G, L, P, 1), v.d2, 4 * n * P, st);
  MNP_CHECK_LAUNCH();
  float2* bs = L.bsplit.as<float2>();
  MNP_TRY(residual_g1h1(G, hl, false, v.d1, v.Y1, v.Z1, 4 * P, bs, st));
  MNP_TRY(gemm_thin_ds(n, 4 * P, n, hl[2], nullptr, ld, v.d2, 4 * P, v.Y2, 4 * P, bs, st));
  MNP_TRY(gemm_thin_ds(n, 4 * P, n, hl[3], nullptr, ld, v.d2, 4 * P, v.Z2, 4 * P, bs, st));
  MNP_CUDA(cudaMemsetAsync(norms, 0, sizeof(double) * 4, st));
  // in place: the residual kernel reads each entry of r before writing it
  launch_residual(face_data(G, L), P, L.lp_dev.as<LamParams>(), v.Y1, v.Y2, v.Z1, v.Z2, v.rphi, v.ra, v.ral,
                  v.rDe, v.rphi, v.ra, v.ral, v.rDe, norms, st);
  MNP_CHECK_LAUNCH();
  MNP_TRY(apply32(G, L, P, v.rphi, v.ra, v.ral, v.rDe));
  launch_axpy_norm(v.x1, fx_ptr(G, L, P, 0), 4 * n * P, norms + 2, st);
  launch_axpy_norm(v.x2, fx_ptr(G, L, P, 1), 4 * n * P, norms + 2, st);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

// ---------------------------------------------------------------- S4
mnpbem_status stage_spectra(mnpbem_geom* G, Lane& L, const SolveCtx& c) {
  const int P = c.P;
  Vec64 v = vec64(G, L, P);
  const double* pol = G->exbuf.as<double>();
  const double* dirs = pol + 3 * P;
  const int ninf = c.exc->ninf;
  const double* inf_nvec = dirs + 3 * P;
  const double* inf_area = inf_nvec + 3 * ninf;
  double2* fields = L.fields.as<double2>();
  const LamParams* lp = L.lp_dev.as<LamParams>();
  launch_farfield(face_data(G, L), P, v.x1, v.x2, dirs, P + ninf, lp, fields, L.st);
  MNP_CHECK_LAUNCH();
  double* slot = L.outbuf.as<double>();
  launch_cross_sections_lp(P, pol, inf_nvec, inf_area, ninf, fields, lp, slot, slot + P, L.st);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

mnpbem_status run_stage(mnpbem_geom* G, Lane& L, const SolveCtx& c, int stage, bool direct) {
  switch (stage) {
    case 0: return stage_assemble(G, L, c.precision);
    case 1: return c.precision == MNPBEM_FP64 ? stage_initmat<double>(G, L, direct) : stage_initmat<float>(G, L, direct);
    case 2: return stage_first(G, L, c);
    case 3: return stage_iter(G, L, c, true);
    case 5: return stage_iter(G, L, c, false);
    case 6: return stage_incr(G, L, c);
    default: return stage_spectra(G, L, c);
  }
}

// capture one stage into a graph; profiling events recorded during the
// capture become event nodes whose timings are read after every replay
mnpbem_status capture_stage(mnpbem_geom* G, Lane& L, const SolveCtx& c, int stage) {
  auto& gr = L.graphs;
  Profiler cap;
  cap.enabled = G->prof.enabled;
  ProfBind pb(&cap);
  capturing_now() = true;
  cudaError_t e = cudaStreamBeginCapture(L.st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    capturing_now() = false;
    MNP_CUDA(e);
  }
  mnpbem_status s = run_stage(G, L, c, stage, false);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(L.st, &graph);
  capturing_now() = false;
  if (s != MNPBEM_OK) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return s;
  }
  MNP_CUDA(e);
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) cudaGraphDestroy(graph);
  MNP_CUDA(e);
  if (gr.exec[stage]) cudaGraphExecDestroy(gr.exec[stage]);
  if (gr.graph[stage]) cudaGraphDestroy(gr.graph[stage]);
  Profiler::release(gr.rec[stage]);
  gr.exec[stage] = exec;
  gr.graph[stage] = graph;
  cap.move_to(gr.rec[stage]);
  return MNPBEM_OK;
}

void drop_graphs(mnpbem_geom* G, Lane& L) {
  auto& gr = L.graphs;
  cudaStreamSynchronize(L.st);
  G->prof.flush();          // replayed records must be read before their events go
  for (int q = 0; q < NSTAGES; ++q) {
    if (gr.exec[q]) cudaGraphExecDestroy(gr.exec[q]);
    gr.exec[q] = nullptr;
    if (gr.graph[q]) cudaGraphDestroy(gr.graph[q]);
    gr.graph[q] = nullptr;
    Profiler::release(gr.rec[q]);
  }
  gr.valid = false;
  cudaGetLastError();
}

bool graphs_match(const mnpbem_geom* G, const Lane& L, const SolveCtx& c) {
  const auto& gr = L.graphs;
  return gr.valid && gr.precision == c.precision && gr.P == c.P && gr.ninf == c.exc->ninf &&
         gr.prof == G->prof.enabled && gr.sig == lane_sig(G, L);
}

mnpbem_status launch_stage(mnpbem_geom* G, Lane& L, const SolveCtx& c, int stage, bool graphs) {
  if (!graphs) return run_stage(G, L, c, stage, true);
  MNP_CUDA(cudaGraphLaunch(L.graphs.exec[stage], L.st));
  G->prof.replayed.push_back(&L.graphs.rec[stage]);
  return MNPBEM_OK;
}

// Status words of a lane's last initmat, copied into pinned host memory after
// the stage is queued and read when the lane's work has completed:
//   [0] [1]  Gauss-Jordan (Deltai): pivot flag, block condition proxy (float bits)
//   [2] [3]  the same for its inner level (pivot blocks wider than 64)
//   [4] [5]  block LDU factors (G1, G2, Sigma): pivot flag, condition proxy
//   [6]      tensor-core GEMM error word (a bounded wait expired)
// The condition proxy of a diagonal block is max|A_kk| * max|inv(A_kk)|; above
// these limits its inverse has lost (nearly) every digit of the precision.
constexpr float COND_LIMIT_32 = 1e6f, COND_LIMIT_64 = 1e13f;

float status_cond(const Lane& L) {
  float c = 0.f;
  for (int q : {1, 3, 5}) {
    float v;
    memcpy(&v, &L.status_host[q], sizeof(float));
    c = std::max(c, v);
  }
  return c;
}

mnpbem_status check_pivots(Lane& L, int precision) {
  const int* h = L.status_host;
  if (h[6]) {
    set_error("tensor-core GEMM: a bounded pipeline wait expired (code %d)", h[6]);
    L.tc.enabled = false;
    return MNPBEM_ERR_TIMEOUT;
  }
  if (h[0] | h[2] | h[4]) {
    set_error("block factorisation: zero or non-finite pivot in a diagonal block");
    return MNPBEM_ERR_SINGULAR;
  }
  const float c = status_cond(L);
  L.cond_max = std::max(L.cond_max, c);
  if (c > (precision == MNPBEM_FP64 ? COND_LIMIT_64 : COND_LIMIT_32)) {
    set_error("block factorisation: a diagonal block is numerically singular (condition proxy %.3g)", (double)c);
    return MNPBEM_ERR_SINGULAR;
  }
  return MNPBEM_OK;
}

mnpbem_status status_copy(Lane& L, int precision) {
  int* h = L.status_host;
  for (int q = 0; q < LANE_NSTATUS; ++q) h[q] = 0;
  auto cp = [&](const DevBuf& b, int slot, int words) -> mnpbem_status {
    if (b.ptr) MNP_CUDA(cudaMemcpyAsync(h + slot, b.ptr, words * sizeof(int), cudaMemcpyDeviceToHost, L.st));
    return MNPBEM_OK;
  };
  if (precision == MNPBEM_FP64) {
    MNP_TRY(cp(L.gj64.status, 0, 2));
    if (L.gj64.inner) MNP_TRY(cp(L.gj64.inner->status, 2, 2));
  } else {
    MNP_TRY(cp(L.gj32.status, 0, 2));
    if (L.gj32.inner) MNP_TRY(cp(L.gj32.inner->status, 2, 2));
  }
  MNP_TRY(cp(L.lu_status, 4, 2));
  if (L.tc.err.ptr && L.tc.err_cleared) MNP_TRY(cp(L.tc.err, 6, 1));
  return MNPBEM_OK;
}

struct Refine {
  int maxit;
  double tol;
};

// Refinement schedule of one wavelength (stages 3, 5, 6):
//   step 1      full residual b - A x with FP32 products of the hi planes (5)
//   then        incremental residuals r - A dx, FP32 products (6)
//   once        a full double-single residual (3), when the relative residual
//               is below 1e-3 or after three steps: it removes the FP32
//               rounding of the first residual (~1e-7 of |A| |x|); taken as
//               early as the FP32 chain's contraction allows, it saves one
//               step against an anchor at 1e-5
//   then        incremental residuals again, whose rounding (~1e-7 of |A| |dx|)
//               is far below the 1e-10 tolerance once dx is small.
// The stopping test (||dx|| <= tol ||x||) counts only after the double-single
// residual.  Relative residuals are measured against ||b|| of the last full one.
// One definition of these rules serves the host scheduler (state in the Lane)
// and the device-side decisions of a sweep graph (state in SweepCtl): S has
// iters, ds_done, res and bnorm2; hn are the four norms a step leaves.
constexpr double DS_SWITCH = 1e-3;
constexpr int STEP_DS = 3, STEP_FP32 = 5, STEP_INCR = 6;
template <typename S>
__host__ __device__ inline int refine_next_kind(const S& s) {
  if (s.iters == 0) return STEP_FP32;
  if (!s.ds_done && (s.res <= DS_SWITCH || s.iters >= 3)) return STEP_DS;
  return STEP_INCR;
}
template <typename S>
__host__ __device__ inline void refine_step_done(S& s, int kind, const double* hn) {
  if (kind != STEP_INCR) s.bnorm2 = hn[1];
  if (kind == STEP_DS) s.ds_done = true;
  s.res = s.bnorm2 > 0 ? sqrt(hn[0] / s.bnorm2) : 0.0;
  ++s.iters;
}
template <typename S>
__host__ __device__ inline bool refine_converged(const S& s, const double* hn, double tol) {
  return s.ds_done && sqrt(hn[2]) <= tol * sqrt(hn[3]);
}
int next_step(const Lane& L) { return refine_next_kind(L); }
void step_done(Lane& L, int kind, const double* hn) { refine_step_done(L, kind, hn); }
bool step_converged(const Lane& L, const double* hn, double tol) { return refine_converged(L, hn, tol); }
void refine_reset(Lane& L) {
  L.iters = 0;
  L.res = -1.0;
  L.ds_done = false;
  L.bnorm2 = 0.0;
}

// one wavelength through all stages, synchronously (graphs == true replays
// captured stages; false runs the stages directly and sizes the buffers)
mnpbem_status solve_one(mnpbem_geom* G, Lane& L, const SolveCtx& c, const Refine& ref, bool graphs,
                        int32_t* iters, double* resid) {
  cudaStream_t st = L.st;
  for (int stage = 0; stage < 3; ++stage) MNP_TRY(launch_stage(G, L, c, stage, graphs));
  MNP_TRY(status_copy(L, c.precision));
  int used = 0;
  double final_res = -1.0;
  if (c.precision == MNPBEM_MIXED) {
    double* hn = L.norms_host;
    refine_reset(L);
    for (int it = 0; it < ref.maxit; ++it) {
      const int kind = next_step(L);
      MNP_TRY(launch_stage(G, L, c, kind, graphs));
      MNP_CUDA(cudaMemcpyAsync(hn, L.norms.ptr, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
      MNP_CUDA(cudaStreamSynchronize(st));
      G->prof.flush();
      MNP_TRY(check_pivots(L, c.precision));
      step_done(L, kind, hn);
      used = L.iters;
      final_res = L.res;
      if (!(hn[2] == hn[2])) { set_error("refinement produced NaN"); return MNPBEM_ERR_NOT_CONVERGED; }
      if (step_converged(L, hn, ref.tol)) break;
    }
  }
  if (c.spectra) MNP_TRY(launch_stage(G, L, c, 4, graphs));
  MNP_CUDA(cudaStreamSynchronize(st));
  G->prof.flush();
  MNP_TRY(check_pivots(L, c.precision));
  if (iters) *iters = used;
  if (resid) *resid = final_res;
  return MNPBEM_OK;
}

void fill_lp(LamParams& lp, double enei, const double* em, int nmed, int medium, int w) {
  lp = LamParams{};
  const double k0 = 2 * M_PI / enei;
  for (int m = 0; m < nmed; ++m) {
    const std::complex<double> e(em[2 * m], em[2 * m + 1]);
    const std::complex<double> k = k0 * std::sqrt(e);
    lp.eps[m] = make_double2(e.real(), e.imag());
    lp.k[m] = make_double2(k.real(), k.imag());
  }
  lp.kexc = lp.k[medium - 1];
  const std::complex<double> nb1 = std::sqrt(std::complex<double>(em[0], em[1]));
  lp.nb1 = make_double2(nb1.real(), nb1.imag());
  lp.k0 = k0;
  lp.w = w;
}

mnpbem_status ensure_lp_ring(mnpbem_geom* G, int count) {
  if (G->lp_cap >= count) return MNPBEM_OK;
  if (G->lp_ring) cudaFreeHost(G->lp_ring);   // every lane was synchronised at the end of the last call
  G->lp_ring = nullptr;
  G->lp_cap = 0;
  MNP_CUDA(cudaMallocHost(&G->lp_ring, sizeof(LamParams) * count));
  G->lp_cap = count;
  return MNPBEM_OK;
}

// ----------------------------------------------------------- sweep scheduler
struct Sweep {
  int nenei;
  const double* enei;
  const double* eps;
  int nmed;
  int medium;
  Refine ref;
  mnpbem_solution* out;
};

mnpbem_status upload_lp(mnpbem_geom* G, Lane& L, const Sweep& s, int w) {
  LamParams& lp = G->lp_ring[w];
  fill_lp(lp, s.enei[w], s.eps + 2 * (size_t)s.nmed * w, s.nmed, s.medium, 0);
  MNP_CUDA(cudaMemcpyAsync(L.lp_dev.ptr, &lp, sizeof(LamParams), cudaMemcpyHostToDevice, L.st));
  return MNPBEM_OK;
}

// copies of wavelength w's results from the lane into the caller's outputs
mnpbem_status write_outputs(mnpbem_geom* G, Lane& L, const SolveCtx& c, const Sweep& s, int w) {
  mnpbem_solution* out = s.out;
  const int P = c.P;
  const int64_t n = G->g.n;
  const cudaMemcpyKind kind = out->outputs_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  const size_t cs = sizeof(double2);
  Vec64 v = vec64(G, L, P);
  auto cp2 = [&](double* dst, const double2* src, int off, int width) -> mnpbem_status {
    if (!dst) return MNPBEM_OK;
    MNP_CUDA(cudaMemcpy2DAsync(dst + 2 * (size_t)w * n * width, cs * width, src + off, cs * 4 * P,
                               cs * width, n, kind, L.st));
    return MNPBEM_OK;
  };
  MNP_TRY(cp2(out->sig1, v.x1, 0, P));
  MNP_TRY(cp2(out->h1, v.x1, P, 3 * P));
  MNP_TRY(cp2(out->sig2, v.x2, 0, P));
  MNP_TRY(cp2(out->h2, v.x2, P, 3 * P));
  const double* slot = L.outbuf.as<double>();
  if (out->ext) MNP_CUDA(cudaMemcpyAsync(out->ext + (size_t)w * P, slot, sizeof(double) * P, kind, L.st));
  if (out->sca) MNP_CUDA(cudaMemcpyAsync(out->sca + (size_t)w * P, slot + P, sizeof(double) * P, kind, L.st));
  if (out->ir_iters) out->ir_iters[w] = L.iters;
  if (out->ir_resid) out->ir_resid[w] = L.res;
  return MNPBEM_OK;
}

mnpbem_status queue_iter(mnpbem_geom* G, Lane& L, const SolveCtx& c) {
  L.last_kind = next_step(L);
  MNP_TRY(launch_stage(G, L, c, L.last_kind, true));
  MNP_CUDA(cudaMemcpyAsync(L.norms_host, L.norms.ptr, 4 * sizeof(double), cudaMemcpyDeviceToHost, L.st));
  MNP_CUDA(cudaEventRecord(L.ev, L.st));
  L.state = Lane::ITER;
  return MNPBEM_OK;
}

mnpbem_status queue_finish(mnpbem_geom* G, Lane& L, const SolveCtx& c) {
  MNP_TRY(launch_stage(G, L, c, 4, true));
  MNP_CUDA(cudaEventRecord(L.ev, L.st));
  L.state = Lane::DONE;
  return MNPBEM_OK;
}

// queue wavelength w on a lane with captured graphs (returns without waiting)
mnpbem_status lane_start(mnpbem_geom* G, Lane& L, const SolveCtx& c, const Sweep& s, int w) {
  L.w = w;
  refine_reset(L);
  MNP_TRY(upload_lp(G, L, s, w));
  for (int stage = 0; stage < 3; ++stage) MNP_TRY(launch_stage(G, L, c, stage, true));
  MNP_TRY(status_copy(L, c.precision));
  if (c.precision == MNPBEM_MIXED && s.ref.maxit > 0) return queue_iter(G, L, c);
  return queue_finish(G, L, c);
}

// the lane's queued work has completed: decide what comes next
mnpbem_status lane_advance(mnpbem_geom* G, Lane& L, const SolveCtx& c, const Sweep& s) {
  if (G->prof.enabled) G->prof.flush();
  MNP_TRY(check_pivots(L, c.precision));
  if (L.state == Lane::ITER) {
    const double* hn = L.norms_host;
    step_done(L, L.last_kind, hn);
    if (!(hn[2] == hn[2])) { set_error("refinement produced NaN"); return MNPBEM_ERR_NOT_CONVERGED; }
    if (step_converged(L, hn, s.ref.tol) || L.iters >= s.ref.maxit) return queue_finish(G, L, c);
    return queue_iter(G, L, c);
  }
  // DONE: results of L.w are in the lane; the stream is idle, so host-side
  // copies into pageable memory do not wait on other work
  MNP_TRY(write_outputs(G, L, c, s, L.w));
  L.state = Lane::IDLE;
  L.w = -1;
  return MNPBEM_OK;
}

// number of lanes for this call: requested (or default), bounded by the
// wavelengths and by the free device memory for lanes not yet allocated
int choose_lanes(mnpbem_geom* G, int precision, int P, int ninf, int nenei) {
  int want = G->lanes_req > 0 ? G->lanes_req : DEFAULT_LANES;
  if (G->prof.enabled || !G->use_graphs) want = 1;
  want = std::max(1, std::min(want, std::min(nenei, MAX_LANES)));
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  const size_t est = lane_bytes_estimate(G, precision, P, ninf);
  const size_t reserve = std::max<size_t>((size_t)2 << 30, tot / 20);
  int nl = 1;
  for (int l = 1; l < want; ++l) {
    size_t have = 0;
    if (l < (int)G->lanes.size()) {
      const Lane& L = *G->lanes[l];
      for (int q = 0; q < 5; ++q) have += L.mat[q].bytes;
      for (int q = 0; q < 4; ++q) have += L.mat64[q].bytes;
    }
    const size_t need = est > have ? est - have : 0;
    if (fr < need + reserve) break;
    fr -= need;
    nl = l + 1;
  }
  return nl;
}

// One wavelength sweep on one handle.  A call of mnpbem_solve is one job; a
// call of mnpbem_solve_batch runs several jobs (particles) through one
// scheduler loop, so that the lanes of every handle stay busy together.
struct Job {
  mnpbem_geom* G = nullptr;
  SolveCtx c;
  Sweep s;
  int nl = 1;
  int next = 0;                 // next wavelength to hand out
  int active = 0;               // lanes with queued work
  std::vector<Lane*> run;       // lanes with graphs for this configuration
};

mnpbem_status validate_job(mnpbem_geom* G, const mnpbem_planewave* exc, int32_t nenei, const double* enei,
                           const double* eps_media, int32_t nmed, int32_t precision, mnpbem_solution* out) {
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
  return MNPBEM_OK;
}

// excitation buffer, lanes, workspaces, masks and the parameter ring of a job
mnpbem_status job_setup(Job& j, const mnpbem_planewave* exc, int32_t nenei, const double* enei,
                        const double* eps_media, int32_t nmed, int32_t precision,
                        const mnpbem_refine* refine, mnpbem_solution* out) {
  mnpbem_geom* G = j.G;
  ProfBind pb_(&G->prof);
  const int P = exc->npol;
  const int64_t n = G->g.n;
  {
    std::vector<double> eb;
    eb.insert(eb.end(), exc->pol, exc->pol + 3 * P);
    eb.insert(eb.end(), exc->dir, exc->dir + 3 * P);
    if (exc->ninf) {
      eb.insert(eb.end(), exc->inf_nvec, exc->inf_nvec + 3 * exc->ninf);
      eb.insert(eb.end(), exc->inf_area, exc->inf_area + exc->ninf);
    }
    for (auto& L : G->lanes) MNP_CUDA(cudaStreamSynchronize(L->st));   // nothing may still read exbuf
    MNP_TRY(G->exbuf.ensure(sizeof(double) * eb.size()));
    MNP_CUDA(cudaMemcpy(G->exbuf.ptr, eb.data(), sizeof(double) * eb.size(), cudaMemcpyHostToDevice));
  }
  j.nl = choose_lanes(G, precision, P, exc->ninf, nenei);
  while ((int)G->lanes.size() < j.nl) MNP_TRY(add_lane(G));
  std::vector<unsigned char> masks(2 * n);
  for (int64_t i = 0; i < n; ++i) {
    const int p = G->face_part[i];
    masks[i] = G->inout[2 * p] == exc->medium;
    masks[n + i] = G->inout[2 * p + 1] == exc->medium;
  }
  for (int l = 0; l < j.nl; ++l) {
    MNP_TRY(ensure_workspace(G, *G->lanes[l], precision, P, exc->ninf));
    MNP_TRY(upload_masks(G, *G->lanes[l], masks));
  }
  MNP_TRY(ensure_lp_ring(G, nenei));
  j.c.P = P;
  j.c.precision = precision;
  j.c.exc = exc;
  j.s.nenei = nenei;
  j.s.enei = enei;
  j.s.eps = eps_media;
  j.s.nmed = nmed;
  j.s.medium = exc->medium;
  j.s.ref.maxit = refine && refine->max_iter > 0 ? refine->max_iter : 10;
  j.s.ref.tol = refine && refine->tol > 0 ? refine->tol : 1e-10;
  j.s.out = out;
  j.next = 0;
  j.active = 0;
  j.run.clear();
  return MNPBEM_OK;
}

// lanes without graphs for this configuration run one wavelength directly
// (sizing every buffer), then capture the stages; without graphs every
// wavelength runs directly on lane 0
mnpbem_status job_prepare(Job& j) {
  mnpbem_geom* G = j.G;
  ProfBind pb_(&G->prof);
  const SolveCtx& c = j.c;
  const Sweep& s = j.s;
  if (c.ext_pot) {
    // external potentials: direct solves on lane 0 (no captured graphs)
    Lane& L = *G->lanes[0];
    for (; j.next < s.nenei; ++j.next) {
      MNP_TRY(upload_lp(G, L, s, j.next));
      L.w = j.next;
      MNP_TRY(solve_one(G, L, c, s.ref, false, &L.iters, &L.res));
      MNP_TRY(write_outputs(G, L, c, s, j.next));
    }
    return MNPBEM_OK;
  }
  std::vector<int> fresh;
  for (int l = 0; l < j.nl && j.next < s.nenei; ++l) {
    Lane& L = *G->lanes[l];
    if (graphs_match(G, L, c)) continue;
    if (L.graphs.valid) drop_graphs(G, L);
    const int w = j.next++;
    MNP_TRY(upload_lp(G, L, s, w));
    L.w = w;
    MNP_TRY(solve_one(G, L, c, s.ref, false, &L.iters, &L.res));
    MNP_TRY(write_outputs(G, L, c, s, w));
    MNP_CUDA(cudaStreamSynchronize(L.st));
    if (!G->use_graphs) break;
    fresh.push_back(l);
  }
  for (int l : fresh) {
    Lane& L = *G->lanes[l];
    bool ok = true;
    for (int stage = 0; stage < NSTAGES && ok; ++stage) {
      if ((stage == 3 || stage == 5 || stage == 6) && c.precision != MNPBEM_MIXED) continue;
      ok = capture_stage(G, L, c, stage) == MNPBEM_OK;
    }
    if (ok) {
      auto& gr = L.graphs;
      gr.valid = true;
      gr.precision = c.precision;
      gr.P = c.P;
      gr.ninf = c.exc->ninf;
      gr.prof = G->prof.enabled;
      gr.sig = lane_sig(G, L);
    } else {
      drop_graphs(G, L);
      G->use_graphs = false;   // run directly from now on
    }
  }
  if (!G->use_graphs) {
    Lane& L = *G->lanes[0];
    for (; j.next < s.nenei; ++j.next) {
      MNP_TRY(upload_lp(G, L, s, j.next));
      L.w = j.next;
      MNP_TRY(solve_one(G, L, c, s.ref, false, &L.iters, &L.res));
      MNP_TRY(write_outputs(G, L, c, s, j.next));
    }
    return MNPBEM_OK;
  }
  for (int l = 0; l < j.nl; ++l)
    if (graphs_match(G, *G->lanes[l], c)) j.run.push_back(G->lanes[l].get());
  return MNPBEM_OK;
}

// the remaining wavelengths of every job go to its lanes as they free up; the
// host polls each lane's completion event and queues the lane's next step
mnpbem_status jobs_poll(std::vector<Job*>& jobs) {
  cudaEvent_t start;
  MNP_CUDA(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  struct EvGuard { cudaEvent_t e; ~EvGuard() { cudaEventDestroy(e); } } eg{start};
  int active = 0;
  for (Job* j : jobs) {
    ProfBind pb_(&j->G->prof);
    MNP_CUDA(cudaEventRecord(start, j->G->st));
    for (Lane* L : j->run) {
      MNP_CUDA(cudaStreamWaitEvent(L->st, start, 0));
      if (j->next < j->s.nenei) {
        MNP_TRY(lane_start(j->G, *L, j->c, j->s, j->next++));
        ++j->active;
        ++active;
      }
    }
  }
  while (active > 0) {
    bool progressed = false;
    for (Job* j : jobs) {
      if (!j->active) continue;
      ProfBind pb_(&j->G->prof);
      for (Lane* L : j->run) {
        if (L->state == Lane::IDLE) continue;
        const cudaError_t q = cudaEventQuery(L->ev);
        if (q == cudaErrorNotReady) continue;
        MNP_CUDA(q);
        progressed = true;
        MNP_TRY(lane_advance(j->G, *L, j->c, j->s));
        if (L->state == Lane::IDLE) {
          if (j->next < j->s.nenei) {
            MNP_TRY(lane_start(j->G, *L, j->c, j->s, j->next++));
          } else {
            --j->active;
            --active;
          }
        }
      }
    }
    if (!progressed) std::this_thread::yield();
  }
  return MNPBEM_OK;
}

// ------------------------------------------------------------ sweep graphs
// The remaining wavelengths of a sweep as one CUDA graph: per lane a WHILE
// node whose body takes the next wavelength from a device counter shared by
// the job's lanes (a work queue), runs the captured stages (child graphs),
// refines in a nested WHILE node whose body picks the step kind on the device
// (a SWITCH over the FP32, double-single and incremental steps) and decides
// on the norms the step left (the host scheduler's rules, restated), and
// writes the wavelength's results into per-wavelength slots.  Every loop is
// bounded: the queue ends at nenei, the refinement at maxit (<= 1000).  The
// host reads the slots once the graph has completed.  Several jobs (the
// particles of a batch) are parallel branches of one graph.
struct SweepCtl {
  int w, iters, ds_done, kind;
  double res, bnorm2;
};
struct JobCtl {
  int next, nenei;
};
// per-wavelength result slots of one job (device)
struct SweepDst {
  double2 *sig1, *h1, *sig2, *h2;   // [w][n][P], [w][n][3P] (NULL: not requested)
  double *ext, *sca;                // [w][P]
  int* iters;                       // [w]
  double* res;                      // [w]
  int* status;                      // [w][LANE_NSTATUS]
  int* nan;                         // set when a refinement step produced NaN
  unsigned long long* stages;       // [NSTAGES] stage runs (the launch accounting of the replays)
  int64_t n;
  int P;
};

// the next wavelength of the job's queue for this lane; the queue stops for
// the lane once a bounded tensor-core wait has expired or a refinement step
// produced NaN (the host reports either after the graph)
__global__ void k_sw_next(JobCtl* jc, SweepCtl* sc, const LamParams* lps, LamParams* lp,
                          cudaGraphConditionalHandle h, const int* tce, const SweepDst* dp) {
  if (threadIdx.x) return;
  const bool failed = (tce && *(volatile const int*)tce) || *(volatile const int*)dp->nan;
  const int w = failed ? jc->nenei : atomicAdd(&jc->next, 1);
  const bool go = w < jc->nenei;
  if (go) {
    sc->w = w;
    *lp = lps[w];
  }
  cudaGraphSetConditional(h, go ? 1u : 0u);
}

// status words of the wavelength's initmat (the layout of Lane::status_host)
__global__ void k_sw_status(const SweepCtl* sc, const int* gj, const int* gji, const int* lu, const int* tce,
                            const SweepDst* dp) {
  if (threadIdx.x) return;
  atomicAdd(dp->stages + 0, 1ull);
  atomicAdd(dp->stages + 1, 1ull);
  atomicAdd(dp->stages + 2, 1ull);
  atomicAdd(dp->stages + 4, 1ull);
  int* o = dp->status + (int64_t)sc->w * LANE_NSTATUS;
  for (int q = 0; q < LANE_NSTATUS; ++q) o[q] = 0;
  if (gj) { o[0] = gj[0]; o[1] = gj[1]; }
  if (gji) { o[2] = gji[0]; o[3] = gji[1]; }
  if (lu) { o[4] = lu[0]; o[5] = lu[1]; }
  if (tce) o[6] = tce[0];
}

__global__ void k_ref_init(SweepCtl* sc, cudaGraphConditionalHandle h, int run, const SweepDst* dp) {
  if (threadIdx.x) return;
  const SweepDst& d = *dp;
  sc->iters = 0;
  sc->ds_done = 0;
  sc->res = -1.0;
  sc->bnorm2 = 0.0;
  d.iters[sc->w] = 0;
  d.res[sc->w] = -1.0;
  if (run) cudaGraphSetConditional(h, 1u);
}

// refine_next_kind(): FP32 first, the double-single step once the FP32
// residual is small (or after three steps), then incremental steps; body
// index 0 / 1 / 2
__global__ void k_ref_pick(SweepCtl* sc, cudaGraphConditionalHandle h, const SweepDst* dp) {
  if (threadIdx.x) return;
  const int kind = refine_next_kind(*sc);
  sc->kind = kind;
  atomicAdd(dp->stages + kind, 1ull);
  cudaGraphSetConditional(h, kind == STEP_FP32 ? 0u : kind == STEP_DS ? 1u : 2u);
}

// refine_step_done() and refine_converged() on the norms the step left
__global__ void k_ref_decide(SweepCtl* sc, const double* hn, double tol, int maxit, cudaGraphConditionalHandle h,
                             const SweepDst* dp) {
  if (threadIdx.x) return;
  const SweepDst& d = *dp;
  refine_step_done(*sc, sc->kind, hn);
  const bool nan = !(hn[2] == hn[2]);
  if (nan) atomicOr(d.nan, 1);
  const bool conv = refine_converged(*sc, hn, tol);
  d.iters[sc->w] = sc->iters;
  d.res[sc->w] = sc->res;
  cudaGraphSetConditional(h, (nan || conv || sc->iters >= maxit) ? 0u : 1u);
}

// the lane's solution and cross sections into the wavelength's slots
__global__ void k_sw_out(const SweepCtl* sc, const double2* x1, const double2* x2, const double* ob,
                         const SweepDst* dp) {
  const SweepDst d = *dp;
  const int w = sc->w, P = d.P;
  const int64_t n = d.n, W = 4 * P;
  const int64_t cnt = n * W;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / W;
    const int c = (int)(e - i * W);
    if (c < P) {
      if (d.sig1) d.sig1[(w * n + i) * P + c] = x1[e];
      if (d.sig2) d.sig2[(w * n + i) * P + c] = x2[e];
    } else {
      if (d.h1) d.h1[(w * n + i) * 3 * P + (c - P)] = x1[e];
      if (d.h2) d.h2[(w * n + i) * 3 * P + (c - P)] = x2[e];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < P) {
    if (d.ext) d.ext[(int64_t)w * P + threadIdx.x] = ob[threadIdx.x];
    if (d.sca) d.sca[(int64_t)w * P + threadIdx.x] = ob[P + threadIdx.x];
  }
}

struct GraphBuild {
  cudaGraph_t top = nullptr;
  ~GraphBuild() {
    if (top) cudaGraphDestroy(top);
  }
};

template <typename... A>
cudaError_t add_kernel(cudaGraphNode_t* node, cudaGraph_t g, const cudaGraphNode_t* dep, int ndep, void (*fn)(A...),
                       dim3 grid, dim3 block, void** args) {
  cudaKernelNodeParams kp = {};
  kp.func = reinterpret_cast<void*>(fn);
  kp.gridDim = grid;
  kp.blockDim = block;
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  kp.extra = nullptr;
  return cudaGraphAddKernelNode(node, g, dep, ndep, &kp);
}

cudaError_t add_cond(cudaGraphNode_t* node, cudaGraph_t g, const cudaGraphNode_t* dep, int ndep,
                     cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, unsigned size,
                     cudaGraph_t* bodies) {
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = size;
  cudaError_t e = cudaGraphAddNode(node, g, dep, nullptr, ndep, &p);
  if (e == cudaSuccess)
    for (unsigned q = 0; q < size; ++q) bodies[q] = p.conditional.phGraph_out[q];
  return e;
}

// the branch of one lane: the queue loop around one wavelength's stages
cudaError_t build_lane_branch(mnpbem_geom* G, Lane& L, const SolveCtx& c, const Sweep& s, cudaGraph_t top,
                              JobCtl* jc, const LamParams* lps, const SweepDst* d) {
  auto& gr = L.graphs;
  SweepCtl* sc = L.swctl.as<SweepCtl>();
  LamParams* lpd = L.lp_dev.as<LamParams>();
  cudaGraphConditionalHandle hq;
  cudaError_t e = cudaGraphConditionalHandleCreate(&hq, top, 0, 0);
  if (e != cudaSuccess) return e;
  const int* stc = (L.tc.err.ptr && L.tc.err_cleared) ? L.tc.err.as<int>() : nullptr;
  cudaGraphNode_t first, loop;
  void* a_next[] = {&jc, &sc, &lps, &lpd, &hq, &stc, &d};
  if ((e = add_kernel(&first, top, nullptr, 0, k_sw_next, 1, 32, a_next)) != cudaSuccess) return e;
  cudaGraph_t body;
  if ((e = add_cond(&loop, top, &first, 1, hq, cudaGraphCondTypeWhile, 1, &body)) != cudaSuccess) return e;
  cudaGraphNode_t n0, n1, n2, nst, last;
  if ((e = cudaGraphAddChildGraphNode(&n0, body, nullptr, 0, gr.graph[0])) != cudaSuccess) return e;
  if ((e = cudaGraphAddChildGraphNode(&n1, body, &n0, 1, gr.graph[1])) != cudaSuccess) return e;
  const bool f64 = c.precision == MNPBEM_FP64;
  const GJWork<float>& g32 = L.gj32;
  const GJWork<double>& g64 = L.gj64;
  const int* sgj = f64 ? g64.status.as<int>() : g32.status.as<int>();
  const int* sgji = f64 ? (g64.inner ? g64.inner->status.as<int>() : nullptr)
                        : (g32.inner ? g32.inner->status.as<int>() : nullptr);
  const int* slu = L.lu_status.as<int>();
  void* a_st[] = {&sc, &sgj, &sgji, &slu, &stc, &d};
  if ((e = add_kernel(&nst, body, &n1, 1, k_sw_status, 1, 32, a_st)) != cudaSuccess) return e;
  if ((e = cudaGraphAddChildGraphNode(&n2, body, &nst, 1, gr.graph[2])) != cudaSuccess) return e;
  const bool refine = c.precision == MNPBEM_MIXED && s.ref.maxit > 0;
  // a handle must belong to a conditional node: created only for the loop
  cudaGraphConditionalHandle hr = 0;
  if (refine && (e = cudaGraphConditionalHandleCreate(&hr, body, 0, 0)) != cudaSuccess) return e;
  int run = refine ? 1 : 0;
  cudaGraphNode_t ni;
  void* a_init[] = {&sc, &hr, &run, &d};
  if ((e = add_kernel(&ni, body, &n2, 1, k_ref_init, 1, 32, a_init)) != cudaSuccess) return e;
  last = ni;
  if (refine) {
    cudaGraphNode_t rl;
    cudaGraph_t rbody;
    if ((e = add_cond(&rl, body, &ni, 1, hr, cudaGraphCondTypeWhile, 1, &rbody)) != cudaSuccess) return e;
    cudaGraphConditionalHandle hs;
    if ((e = cudaGraphConditionalHandleCreate(&hs, rbody, 0, 0)) != cudaSuccess) return e;
    cudaGraphNode_t pk, sw, dc;
    void* a_pick[] = {&sc, &hs, &d};
    if ((e = add_kernel(&pk, rbody, nullptr, 0, k_ref_pick, 1, 32, a_pick)) != cudaSuccess) return e;
    cudaGraph_t sb[3];
    if ((e = add_cond(&sw, rbody, &pk, 1, hs, cudaGraphCondTypeSwitch, 3, sb)) != cudaSuccess) return e;
    const int stage_of[3] = {STEP_FP32, STEP_DS, STEP_INCR};
    for (int q = 0; q < 3; ++q) {
      cudaGraphNode_t cn;
      if ((e = cudaGraphAddChildGraphNode(&cn, sb[q], nullptr, 0, gr.graph[stage_of[q]])) != cudaSuccess) return e;
    }
    const double* hn = L.norms.as<double>();
    double tol = s.ref.tol;
    int maxit = s.ref.maxit;
    void* a_dec[] = {&sc, &hn, &tol, &maxit, &hr, &d};
    if ((e = add_kernel(&dc, rbody, &sw, 1, k_ref_decide, 1, 32, a_dec)) != cudaSuccess) return e;
    last = rl;
  }
  cudaGraphNode_t n4, no, nn;
  if ((e = cudaGraphAddChildGraphNode(&n4, body, &last, 1, gr.graph[4])) != cudaSuccess) return e;
  Vec64 v = vec64(G, L, c.P);
  const double2* x1 = v.x1;
  const double2* x2 = v.x2;
  const double* ob = L.outbuf.as<double>();
  void* a_out[] = {&sc, &x1, &x2, &ob, &d};
  const unsigned ob_blocks = (unsigned)std::min<int64_t>(cdiv_up(G->g.n * 4 * c.P, (int64_t)256), 2048);
  if ((e = add_kernel(&no, body, &n4, 1, k_sw_out, ob_blocks, 256, a_out)) != cudaSuccess) return e;
  void* a_nx[] = {&jc, &sc, &lps, &lpd, &hq, &stc, &d};
  return add_kernel(&nn, body, &no, 1, k_sw_next, 1, 32, a_nx);
}

// is a one-graph sweep usable for these jobs (captured stages, no profiling,
// plane-wave excitation)?
bool sweep_graph_ok(const std::vector<Job*>& jobs) {
  for (const Job* j : jobs) {
    const mnpbem_geom* G = j->G;
    if (!G->sweep_graph || !G->use_graphs || G->prof.enabled || j->c.ext_pot || j->run.empty()) return false;
    if (j->s.ref.maxit > 1000) return false;
    for (const Lane* L : j->run)
      for (int q = 0; q < NSTAGES; ++q) {
        if ((q == 3 || q == 5 || q == 6) && j->c.precision != MNPBEM_MIXED) continue;
        if (!L->graphs.graph[q]) return false;
      }
  }
  return true;
}

// per-job device buffers: wavelength parameters, control word, result slots
struct SweepJobBufs {
  SweepDst d = {};
  SweepDst* dd = nullptr;       // device copy of d (the kernels' view; refreshed before every launch)
  JobCtl* jc = nullptr;
  LamParams* lps = nullptr;
  double2* stage_x = nullptr;   // staging of host-side solution outputs
  double* stage_r = nullptr;    // ext, sca, res
  int* stage_i = nullptr;       // iters, status, nan
  bool staged[6] = {};          // sig1, h1, sig2, h2, ext, sca copied back by the host
};

// the device address of a caller's buffer the graph's kernels may write:
// device or managed memory, or page-locked host memory (mapped); NULL for
// pageable host memory (then the results go through device staging)
void* device_address(void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  return nullptr;
}

mnpbem_status sweep_bufs(Job& j, SweepJobBufs& b) {
  mnpbem_geom* G = j.G;
  const int nenei = j.s.nenei, P = j.c.P;
  const int64_t n = G->g.n;
  const mnpbem_solution* out = j.s.out;
  const bool dev = out->outputs_on_device != 0;
  const int64_t nx = (int64_t)nenei * n * P;
  // host outputs go through device staging
  const int64_t xcount = dev ? 0 : (out->sig1 ? nx : 0) + (out->h1 ? 3 * nx : 0) + (out->sig2 ? nx : 0) +
                                    (out->h2 ? 3 * nx : 0);
  const size_t bytes_lp = ((sizeof(LamParams) * nenei + 255) / 256) * 256;
  MNP_TRY(G->sweep_lp.ensure(bytes_lp + 256 + sizeof(double2) * std::max<int64_t>(1, xcount)));
  MNP_TRY(G->sweep_res.ensure(sizeof(double) * (size_t)nenei * (2 * P + 1) +
                              sizeof(int) * ((size_t)nenei * (1 + LANE_NSTATUS) + 1) + 512));
  char* base = G->sweep_lp.as<char>();
  b.lps = reinterpret_cast<LamParams*>(base);
  b.jc = reinterpret_cast<JobCtl*>(base + bytes_lp);
  b.dd = reinterpret_cast<SweepDst*>(base + bytes_lp + 64);
  b.stage_x = reinterpret_cast<double2*>(base + bytes_lp + 256);
  b.stage_r = G->sweep_res.as<double>();
  b.stage_i = reinterpret_cast<int*>(b.stage_r + (size_t)nenei * (2 * P + 1));
  SweepDst& d = b.d;
  d.n = n;
  d.P = P;
  double2* xs = b.stage_x;
  auto place = [&](double* user, int64_t cnt, int slot) -> double2* {
    if (!user) return nullptr;
    if (dev) return reinterpret_cast<double2*>(user);
    if (void* da = device_address(user)) return reinterpret_cast<double2*>(da);
    b.staged[slot] = true;
    double2* r = xs;
    xs += cnt;
    return r;
  };
  d.sig1 = place(out->sig1, nx, 0);
  d.h1 = place(out->h1, 3 * nx, 1);
  d.sig2 = place(out->sig2, nx, 2);
  d.h2 = place(out->h2, 3 * nx, 3);
  auto place_r = [&](double* user, double* stage, int slot) -> double* {
    if (!user) return nullptr;
    if (dev) return user;
    if (void* da = device_address(user)) return static_cast<double*>(da);
    b.staged[slot] = true;
    return stage;
  };
  d.ext = place_r(out->ext, b.stage_r, 4);
  d.sca = place_r(out->sca, b.stage_r + (size_t)nenei * P, 5);
  d.res = b.stage_r + (size_t)nenei * 2 * P;
  d.iters = b.stage_i;
  d.status = b.stage_i + nenei;
  d.nan = b.stage_i + (size_t)nenei * (1 + LANE_NSTATUS);
  const size_t soff = (((size_t)nenei * (1 + LANE_NSTATUS) + 1) * sizeof(int) + 7) / 8 * 8;
  d.stages = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(b.stage_i) + soff);
  return MNPBEM_OK;
}

// the host's part after the graph: outputs to host buffers, refinement
// counts, status checks (the checks of check_pivots per wavelength)
mnpbem_status sweep_finish(Job& j, SweepJobBufs& b, int w0) {
  mnpbem_geom* G = j.G;
  const int nenei = j.s.nenei, P = j.c.P;
  const int64_t n = G->g.n;
  mnpbem_solution* out = j.s.out;
  std::vector<int> iv((size_t)nenei * (1 + LANE_NSTATUS) + 1);
  std::vector<double> rv((size_t)nenei * (2 * P + 1));
  MNP_CUDA(cudaMemcpy(iv.data(), b.stage_i, sizeof(int) * iv.size(), cudaMemcpyDeviceToHost));
  MNP_CUDA(cudaMemcpy(rv.data(), b.stage_r, sizeof(double) * rv.size(), cudaMemcpyDeviceToHost));
  if (iv.back()) {
    set_error("refinement produced NaN");
    return MNPBEM_ERR_NOT_CONVERGED;
  }
  Lane& L0 = *j.run[0];
  // launch accounting: every stage run as a replay of lane 0's record, plus
  // the graph's control kernels (4 per wavelength, 2 per refinement step)
  {
    unsigned long long cnt[NSTAGES];
    MNP_CUDA(cudaMemcpy(cnt, b.d.stages, sizeof(cnt), cudaMemcpyDeviceToHost));
    Profiler& pr = G->prof;
    for (int q = 0; q < NSTAGES; ++q)
      for (int ph = 0; ph < PH_COUNT; ++ph) {
        const PhaseAcc& r = L0.graphs.rec[q].counts[ph];
        pr.acc[ph].launches += (int64_t)cnt[q] * r.launches;
        pr.acc[ph].flops += (double)cnt[q] * r.flops;
        pr.acc[ph].bytes += (double)cnt[q] * r.bytes;
      }
    for (int w = w0; w < nenei; ++w) pr.acc[PH_ELEMWISE].launches += 4 + 2 * (int64_t)iv[w];
  }
  for (int w = w0; w < nenei; ++w) {
    memcpy(L0.status_host, &iv[(size_t)nenei + (size_t)w * LANE_NSTATUS], sizeof(int) * LANE_NSTATUS);
    MNP_TRY(check_pivots(L0, j.c.precision));
  }
  const int64_t nx = (int64_t)nenei * n * P;
  const size_t skip = (size_t)w0 * n * P;   // wavelengths solved before the graph are already written
  auto back = [&](double* user, const double2* stage, int width, int slot) -> mnpbem_status {
    if (!user || !b.staged[slot] || !stage) return MNPBEM_OK;
    const size_t off = skip * width;
    MNP_CUDA(cudaMemcpy(reinterpret_cast<double2*>(user) + off, stage + off,
                        sizeof(double2) * ((size_t)nx * width - off), cudaMemcpyDeviceToHost));
    return MNPBEM_OK;
  };
  MNP_TRY(back(out->sig1, b.d.sig1, 1, 0));
  MNP_TRY(back(out->h1, b.d.h1, 3, 1));
  MNP_TRY(back(out->sig2, b.d.sig2, 1, 2));
  MNP_TRY(back(out->h2, b.d.h2, 3, 3));
  for (int w = w0; w < nenei; ++w) {
    if (out->ext && b.staged[4]) memcpy(out->ext + (size_t)w * P, &rv[(size_t)w * P], sizeof(double) * P);
    if (out->sca && b.staged[5]) memcpy(out->sca + (size_t)w * P, &rv[(size_t)(nenei + w) * P], sizeof(double) * P);
    if (out->ir_iters) out->ir_iters[w] = iv[w];
    if (out->ir_resid) out->ir_resid[w] = rv[(size_t)nenei * 2 * P + w];
  }
  return MNPBEM_OK;
}

// the remaining wavelengths of every job as one graph launch; returns
// MNPBEM_ERR_UNSUPPORTED (nothing launched) when the graph cannot be built
mnpbem_status jobs_graph(std::vector<Job*>& jobs) {
  if (!sweep_graph_ok(jobs)) return MNPBEM_ERR_UNSUPPORTED;
  bool work = false;
  for (const Job* j : jobs) work = work || j->next < j->s.nenei;
  if (!work) return MNPBEM_OK;
  // job buffers: one set per handle, so one job per handle
  for (size_t a = 0; a < jobs.size(); ++a)
    for (size_t b2 = a + 1; b2 < jobs.size(); ++b2)
      if (jobs[a]->G == jobs[b2]->G) return MNPBEM_ERR_UNSUPPORTED;
  std::vector<SweepJobBufs> bufs(jobs.size());
  std::vector<int> w0(jobs.size());
  for (size_t q = 0; q < jobs.size(); ++q) {
    Job& j = *jobs[q];
    mnpbem_geom* G = j.G;
    ProfBind pb_(&G->prof);
    w0[q] = j.next;
    MNP_TRY(sweep_bufs(j, bufs[q]));
    for (Lane* L : j.run) MNP_TRY(L->swctl.ensure(sizeof(SweepCtl)));
    // parameters of every wavelength, the queue start, zeroed slots
    for (int w = 0; w < j.s.nenei; ++w)
      fill_lp(G->lp_ring[w], j.s.enei[w], j.s.eps + 2 * (size_t)j.s.nmed * w, j.s.nmed, j.s.medium, 0);
    MNP_CUDA(cudaMemcpyAsync(bufs[q].lps, G->lp_ring, sizeof(LamParams) * j.s.nenei, cudaMemcpyHostToDevice,
                             G->st));
    JobCtl jc{j.next, j.s.nenei};
    MNP_CUDA(cudaMemcpyAsync(bufs[q].jc, &jc, sizeof(JobCtl), cudaMemcpyHostToDevice, G->st));
    MNP_CUDA(cudaMemcpyAsync(bufs[q].dd, &bufs[q].d, sizeof(SweepDst), cudaMemcpyHostToDevice, G->st));
    MNP_CUDA(cudaMemsetAsync(G->sweep_res.ptr, 0, G->sweep_res.bytes, G->st));
    MNP_CUDA(cudaStreamSynchronize(G->st));   // jc lives on this stack frame
  }
  // build (or reuse, for a single job on an unchanged handle) the graph
  Job& j0 = *jobs[0];
  mnpbem_geom* G0 = j0.G;
  uint64_t key = 1469598103934665603ull;
  auto mix = [&](uint64_t v) { key = (key ^ v) * 1099511628211ull; };
  for (size_t q = 0; q < jobs.size(); ++q) {
    const Job& j = *jobs[q];
    mix((uint64_t)(uintptr_t)j.G);
    mix((uint64_t)j.c.precision);
    mix((uint64_t)j.c.P);
    mix((uint64_t)j.s.ref.maxit);
    uint64_t tb;
    memcpy(&tb, &j.s.ref.tol, sizeof(tb));
    mix(tb);
    for (const void* ptr : {(const void*)bufs[q].dd, (const void*)bufs[q].lps, (const void*)bufs[q].jc})
      mix((uint64_t)(uintptr_t)ptr);
    for (const Lane* L : j.run) {
      mix((uint64_t)(uintptr_t)L);
      mix(L->graphs.sig);
      for (int s = 0; s < NSTAGES; ++s) mix((uint64_t)(uintptr_t)L->graphs.graph[s]);
    }
  }
  cudaGraphExec_t exec = nullptr;
  const bool cache = jobs.size() == 1;
  if (cache && G0->sweep_exec && G0->sweep_key == key) {
    exec = G0->sweep_exec;
  } else {
    GraphBuild gb;
    cudaError_t e = cudaGraphCreate(&gb.top, 0);
    for (size_t q = 0; q < jobs.size() && e == cudaSuccess; ++q)
      for (Lane* L : jobs[q]->run) {
        e = build_lane_branch(jobs[q]->G, *L, jobs[q]->c, jobs[q]->s, gb.top, bufs[q].jc, bufs[q].lps, bufs[q].dd);
        if (e != cudaSuccess) break;
      }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, gb.top, 0);
    if (e != cudaSuccess) {
      cudaGetLastError();
      for (Job* j : jobs) {   // the host scheduler from now on
        j->G->sweep_graph = false;
        j->G->sweep_err = (int)e;
      }
      return MNPBEM_ERR_UNSUPPORTED;
    }
    if (cache) {
      if (G0->sweep_exec) cudaGraphExecDestroy(G0->sweep_exec);
      G0->sweep_exec = exec;
      G0->sweep_key = key;
    }
  }
  // every lane's stream has finished its earlier work; the graph runs on the
  // first handle's stream after all of them
  cudaEvent_t ev;
  MNP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  struct EvGuard { cudaEvent_t e; ~EvGuard() { cudaEventDestroy(e); } } eg{ev};
  for (Job* j : jobs)
    for (Lane* L : j->run) {
      MNP_CUDA(cudaEventRecord(ev, L->st));
      MNP_CUDA(cudaStreamWaitEvent(G0->st, ev, 0));
    }
  const cudaError_t le = cudaGraphLaunch(exec, G0->st);
  const cudaError_t se = le == cudaSuccess ? cudaStreamSynchronize(G0->st) : le;
  if (!cache) cudaGraphExecDestroy(exec);
  MNP_CUDA(se);
  for (size_t q = 0; q < jobs.size(); ++q) {
    jobs[q]->next = jobs[q]->s.nenei;
    ++jobs[q]->G->sweep_runs;
    ProfBind pb_(&jobs[q]->G->prof);
    MNP_TRY(sweep_finish(*jobs[q], bufs[q], w0[q]));
  }
  return MNPBEM_OK;
}

// join (the handle's stream waits for every lane), synchronise, read the
// pivot and tensor-core status words
mnpbem_status job_finish(Job& j, bool failed) {
  mnpbem_geom* G = j.G;
  if (failed) {
    // leave nothing in flight that writes the caller's buffers
    for (int l = 0; l < j.nl && l < (int)G->lanes.size(); ++l) cudaStreamSynchronize(G->lanes[l]->st);
    cudaGetLastError();
    G->prof.flush();
    return MNPBEM_OK;
  }
  for (int l = 0; l < j.nl; ++l) {
    Lane& L = *G->lanes[l];
    if (L.st == G->st) continue;
    MNP_CUDA(cudaEventRecord(L.ev, L.st));
    MNP_CUDA(cudaStreamWaitEvent(G->st, L.ev, 0));
  }
  for (int l = 0; l < j.nl; ++l) MNP_CUDA(cudaStreamSynchronize(G->lanes[l]->st));
  G->prof.flush();
  for (int l = 0; l < j.nl; ++l) {
    Lane& L = *G->lanes[l];
    MNP_TRY(check_pivots(L, j.c.precision));
    if (j.c.precision == MNPBEM_MIXED && G->tc_enabled) MNP_TRY(tc_check_error(L.tc, L.st));
  }
  MNP_TRY(thin_stream_check(G->st));
  return MNPBEM_OK;
}

mnpbem_status run_jobs(std::vector<Job>& jobs) {
  mnpbem_status st = MNPBEM_OK;
  for (Job& j : jobs)
    for (auto& L : j.G->lanes) L->pc_valid = false;
  for (Job& j : jobs)
    if (st == MNPBEM_OK) st = job_prepare(j);
  if (st == MNPBEM_OK) {
    std::vector<Job*> js;
    for (Job& j : jobs) js.push_back(&j);
    st = jobs_graph(js);
    if (st == MNPBEM_ERR_UNSUPPORTED) st = jobs_poll(js);
  }
  if (st != MNPBEM_OK) {
    const std::string keep = get_error();
    for (Job& j : jobs) job_finish(j, true);
    set_error("%s", keep.c_str());
    return st;
  }
  for (Job& j : jobs) MNP_TRY(job_finish(j, false));
  return MNPBEM_OK;
}

template <typename C>
__global__ void k_set_identity(C* X, int64_t n, int64_t ld) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * n) return;
  const int64_t r = i / n, c = i - r * n;
  X[r * ld + c] = (r == c) ? from_d<C>(make_double2(1, 0)) : from_d<C>(make_double2(0, 0));
}

// inverse of the matrix whose LDU factors lane matrix q holds (0: G1 per
// diagonal block, 1: G2, 3: Sigma), by solves with the identity on CUDA cores
// (export for tests; not on the solve path)
template <typename R>
mnpbem_status ldu_inverse(mnpbem_geom* G, Lane& L, int q, cplx<R>* X, cplx<R>* tmp) {
  using Cx = cplx<R>;
  const int64_t n = G->g.n, ld = G->ld;
  k_set_identity<Cx><<<(unsigned)cdiv_up(n * n, (int64_t)256), 256, 0, L.st>>>(X, n, ld);
  MNP_CHECK_LAUNCH();
  const Cx* F = L.mat[q].as<Cx>();
  const int b = lu_block<R>(G, sizeof(R) == 4 ? tc_ctx(G, L) : nullptr);
  if (q == 0) {
    for (size_t k = 0; k < G->g1_off.size(); ++k) {
      const int64_t o = G->g1_off[k];
      MNP_TRY(ldu_solve<R>(F + o * ld + o, G->g1_n[k], ld, b, X + o * ld, ld, n, tmp, gemm_w<R>, nullptr, L.st));
    }
    return MNPBEM_OK;
  }
  return ldu_solve<R>(F, n, ld, b, X, ld, n, tmp, gemm_w<R>, nullptr, L.st);
}

// y += x (count complex values)
template <typename C>
__global__ void k_cacc(C* __restrict__ y, const C* __restrict__ x, int64_t count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) y[i] = cadd(y[i], x[i]);
}
template <typename C>
void cacc(C* y, const C* x, int64_t count, cudaStream_t st) {
  if (count > 0) k_cacc<C><<<(unsigned)cdiv_up(count, (int64_t)256), 256, 0, st>>>(y, x, count);
}

// A^{-T} applied through the transposed chain of mldivide.m.  The chain
// matrices m are transposed in place beforehand: the LDU factors of G1, G2
// and Sigma then hold the factors of G1^T, G2^T and Sigma^T (their solves are
// the same calls), Sigma1 and Deltai hold Sigma1^T and Deltai^T.
// Unknown-space input (gs1, gh1 may be null: zero), equation-space output
// lam = [phi (n) | a (3n) | De (n) | alpha (3n)]; work holds 11 n values.
template <typename R>
mnpbem_status chain_transpose(const AdjParams& p, const ChainMats<R>& m, const cplx<R>* gs1, const cplx<R>* gh1,
                              const cplx<R>* gs2, const cplx<R>* gh2, cplx<R>* lam, cplx<R>* work,
                              GemmFn<R> gemm, void* ctx, cudaStream_t st) {
  using Cx = cplx<R>;
  const int64_t n = p.n, ld = m.ld;
  const size_t cs = sizeof(Cx);
  const Cx one = mk<R>(1, 0), zero = mk<R>(0, 0);
  Cx *lphi = lam, *la = lam + n, *lDe = lam + 4 * n, *lal = lam + 5 * n;
  Cx *gS2 = work, *gH2p = work + n, *v3 = work + 4 * n, *tS1 = work + 7 * n, *ga0 = work + 8 * n;
  auto g1solve = [&](Cx* x, int N) -> mnpbem_status {
    for (int q = 0; q < m.ng1; ++q)
      MNP_TRY(ldu_solve<R>(m.G1 + m.g1_off[q] * ld + m.g1_off[q], m.g1_n[q], ld, m.b, x + m.g1_off[q] * N, N, N,
                           nullptr, gemm, ctx, st, m.bar));
    return MNPBEM_OK;
  };
  // G2^-T w_sig2, G2^-T w_h2
  MNP_CUDA(cudaMemcpyAsync(gS2, gs2, cs * n, cudaMemcpyDeviceToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(gH2p, gh2, cs * 3 * n, cudaMemcpyDeviceToDevice, st));
  MNP_TRY(ldu_solve<R>(m.G2, n, ld, m.b, gS2, 1, 1, nullptr, gemm, ctx, st, m.bar));
  MNP_TRY(ldu_solve<R>(m.G2, n, ld, m.b, gH2p, 3, 3, nullptr, gemm, ctx, st, m.bar));
  if (gs1) {
    MNP_CUDA(cudaMemcpyAsync(lphi, gs1, cs * n, cudaMemcpyDeviceToDevice, st));
    MNP_TRY(g1solve(lphi, 1));                                                     // G1^-T w_sig1
    cacc(gS2, lphi, n, st);
  } else {
    MNP_CUDA(cudaMemsetAsync(lphi, 0, cs * n, st));
  }
  if (gh1) {
    MNP_CUDA(cudaMemcpyAsync(ga0, gh1, cs * 3 * n, cudaMemcpyDeviceToDevice, st));
    MNP_TRY(g1solve(ga0, 3));                                                      // G1^-T w_h1
    cacc(gH2p, ga0, 3 * n, st);
  }
  MNP_TRY(gemm(n, 3, n, one, m.Deltai, ld, gH2p, 3, zero, lal, 3, st, ctx));        // Deltai^T
  adj_chainT<Cx>(p, 0, lal, nullptr, gS2, nullptr, nullptr, nullptr, st);
  MNP_CUDA(cudaMemcpyAsync(lDe, gS2, cs * n, cudaMemcpyDeviceToDevice, st));
  MNP_TRY(ldu_solve<R>(m.Sigma, n, ld, m.b, lDe, 1, 1, nullptr, gemm, ctx, st, m.bar));   // Sigma^-T
  adj_chainT<Cx>(p, 1, lDe, nullptr, v3, nullptr, nullptr, nullptr, st);
  MNP_TRY(gemm(n, 3, n, one, m.Deltai, ld, v3, 3, one, lal, 3, st, ctx));           // += Deltai^T v
  MNP_TRY(gemm(n, 1, n, one, m.Sigma1, ld, lDe, 1, zero, tS1, 1, st, ctx));         // Sigma1^T
  MNP_TRY(gemm(n, 3, n, one, m.Sigma1, ld, lal, 3, zero, la, 3, st, ctx));
  adj_chainT<Cx>(p, 2, tS1, lal, lphi, la, lDe, gh1 ? ga0 : nullptr, st);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

}  // namespace

extern "C" {

mnpbem_status mnpbem_solve(mnpbem_geom* G, const mnpbem_planewave* exc, int32_t nenei,
                           const double* enei, const double* eps_media, int32_t nmed,
                           int32_t precision, const mnpbem_refine* refine, mnpbem_solution* out) {
  MNP_TRY(validate_job(G, exc, nenei, enei, eps_media, nmed, precision, out));
  MNP_CUDA(cudaSetDevice(G->device));
  std::vector<Job> jobs(1);
  jobs[0].G = G;
  MNP_TRY(job_setup(jobs[0], exc, nenei, enei, eps_media, nmed, precision, refine, out));
  return run_jobs(jobs);
}

mnpbem_status mnpbem_solve_batch(const mnpbem_job* jobs_in, int32_t njobs, int32_t precision,
                                 const mnpbem_refine* refine) {
  if (!jobs_in || njobs <= 0) {
    set_error("mnpbem_solve_batch: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  for (int a = 0; a < njobs; ++a) {
    const mnpbem_job& q = jobs_in[a];
    MNP_TRY(validate_job(q.g, q.exc, q.nenei, q.enei, q.eps_media, q.nmed, precision, q.out));
    if (q.g->device != jobs_in[0].g->device) {
      set_error("mnpbem_solve_batch: all handles must be on one device");
      return MNPBEM_ERR_INVALID_ARG;
    }
    for (int b = 0; b < a; ++b)
      if (jobs_in[b].g == q.g) {
        set_error("mnpbem_solve_batch: a handle appears twice (job %d and %d)", b, a);
        return MNPBEM_ERR_INVALID_ARG;
      }
  }
  MNP_CUDA(cudaSetDevice(jobs_in[0].g->device));
  std::vector<Job> jobs(njobs);
  for (int a = 0; a < njobs; ++a) {
    const mnpbem_job& q = jobs_in[a];
    jobs[a].G = q.g;
    MNP_TRY(job_setup(jobs[a], q.exc, q.nenei, q.enei, q.eps_media, q.nmed, precision, refine, q.out));
  }
  return run_jobs(jobs);
}

mnpbem_status mnpbem_ext_gradient(mnpbem_geom* G, const mnpbem_planewave* exc, int32_t ipol, double enei,
                                  const double* eps_media, int32_t nmed, int32_t precision, double* ext,
                                  double* verts_grad, double* eps_grad) {
  return mnpbem_cross_section_gradient(G, exc, ipol, 0, enei, eps_media, nmed, precision, ext, verts_grad,
                                       eps_grad);
}

mnpbem_status mnpbem_cross_section_gradient(mnpbem_geom* G, const mnpbem_planewave* exc, int32_t ipol,
                                            int32_t which, double enei, const double* eps_media, int32_t nmed,
                                            int32_t precision, double* value, double* verts_grad,
                                            double* eps_grad) {
  MNP_TRY(check_geom(G));
  if (!exc || ipol < 0 || ipol >= exc->npol || !verts_grad || !eps_grad || (which != 0 && which != 1) ||
      (which == 1 && exc->ninf <= 0)) {
    set_error("mnpbem_cross_section_gradient: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  if (G->nparts != 1 || !G->all_closed || G->inout[0] == G->inout[1] || exc->medium != G->inout[1]) {
    set_error("mnpbem_ext_gradient: one closed particle excited from its outside medium is required");
    return MNPBEM_ERR_UNSUPPORTED;
  }
  if (G->curved) {
    set_error("cross-section gradients are implemented for flat elements (norm_flat.m) only");
    return MNPBEM_ERR_UNSUPPORTED;
  }
  double sol_ext[4] = {0, 0, 0, 0}, sol_sca[4] = {0, 0, 0, 0};
  mnpbem_solution sol{};
  sol.ext = sol_ext;
  sol.sca = sol_sca;
  MNP_TRY(validate_job(G, exc, 1, &enei, eps_media, nmed, precision, &sol));
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  std::vector<Job> jobs(1);
  Job& j = jobs[0];
  j.G = G;
  MNP_TRY(job_setup(j, exc, 1, &enei, eps_media, nmed, precision, nullptr, &sol));
  Lane& L = *G->lanes[0];
  cudaStream_t st = L.st;
  // forward solve (direct) on lane 0: FP64, or complex64 with FP64-class refinement
  MNP_TRY(upload_lp(G, L, j.s, 0));
  L.w = 0;
  MNP_TRY(solve_one(G, L, j.c, j.s.ref, false, &L.iters, &L.res));
  MNP_TRY(write_outputs(G, L, j.c, j.s, 0));
  MNP_CUDA(cudaStreamSynchronize(st));
  if (value) *value = which == 0 ? sol_ext[ipol] : sol_sca[ipol];
  const int64_t n = G->g.n, ld = G->ld, nv = G->nverts;
  const int P = exc->npol;
  // refined off-diagonal entries (once per geometry)
  if (G->adj_noff < 0) {
    std::vector<int> rr(G->g.nref), cc(G->g.nref), off;
    MNP_CUDA(cudaMemcpy(rr.data(), G->g.ref_row, sizeof(int) * G->g.nref, cudaMemcpyDeviceToHost));
    MNP_CUDA(cudaMemcpy(cc.data(), G->g.ref_col, sizeof(int) * G->g.nref, cudaMemcpyDeviceToHost));
    for (int64_t e = 0; e < G->g.nref; ++e)
      if (rr[e] != cc[e]) off.push_back((int)e);
    MNP_TRY(G->adj_off.ensure(sizeof(int) * std::max<size_t>(1, off.size())));
    if (!off.empty()) MNP_CUDA(cudaMemcpy(G->adj_off.ptr, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice));
    G->adj_noff = (int)off.size();
  }
  // workspace: complex vectors, weights, accumulators, three FP64 matrices
  const size_t cs = sizeof(double2);
  const size_t nvec_c = 40 * (size_t)n;         // complex vectors of the transposed chain + products
  const size_t nacc = 7 * (size_t)n + 3 * (size_t)nv + 4;
  MNP_TRY(G->adj.ensure(cs * (nvec_c + 24 * (size_t)n) + sizeof(double) * (nacc + (size_t)n) + 256));
  MNP_TRY(G->adj_mats.ensure(cs * 3 * (size_t)n * ld));
  double2* V = G->adj.as<double2>();
  double2 *gs2 = V, *gh2 = gs2 + n, *lam = gh2 + 3 * n, *work = lam + 8 * n;     // 1 + 3 + 8 + 11 n
  double2 *GX1 = work + 11 * n, *GX2 = GX1 + 4 * n, *HX1 = GX2 + 4 * n;          // 32 n
  double2 *gphi = lam, *ga = lam + n, *gDe = lam + 4 * n, *gAl = lam + 5 * n;
  double2* Ub = V + nvec_c;
  double2* Xb = Ub + 16 * n;
  double* acc = reinterpret_cast<double*>(Xb + 8 * n);
  double* cb = acc + nacc;
  MNP_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * nacc, st));
  const LamParams& lp = G->lp_ring[0];
  const int in = G->inout[0], out = G->inout[1];
  AdjParams p;
  p.n = n;
  p.order = G->g.order;
  p.pos = G->g.pos; p.nvec = G->g.nvec; p.area = G->g.area; p.verts = G->g.verts; p.faces = G->g.faces;
  p.xt = G->g.xt; p.yt = G->g.yt; p.wt = G->g.wt; p.ntri = G->g.ntri;
  p.x3 = G->g.x3; p.y3 = G->g.y3; p.w3 = G->g.w3; p.n3 = G->g.n3;
  p.x4 = G->g.x4; p.y4 = G->g.y4; p.w4 = G->g.w4; p.n4 = G->g.n4;
  p.ref_row = G->g.ref_row; p.ref_col = G->g.ref_col;
  p.off_idx = G->adj_off.as<int>(); p.noff = G->adj_noff;
  const FaceData fd = face_data(G, L);
  p.eps1 = fd.eps1; p.eps2 = fd.eps2; p.exc_out = fd.exc_out;
  p.k1 = lp.k[in - 1]; p.k2 = lp.k[out - 1]; p.kb = lp.kexc; p.k0 = lp.k0;
  p.U = Ub; p.X = Xb; p.cb = cb;
  p.gpos = acc; p.gnv = acc + 3 * n; p.garea = acc + 6 * n; p.gv = acc + 7 * n; p.gk1 = acc + 7 * n + 3 * nv;
  double* geps = p.gk1 + 2;
  const double* pol_d = G->exbuf.as<double>() + 3 * ipol;
  const double* dir_d = G->exbuf.as<double>() + 3 * P + 3 * ipol;
  Vec64 vv = vec64(G, L, P);
  // ---- right-hand side w = dJ/dx (sig2, h2; zero on sig1, h1)
  if (which == 0) {
    adj_rhs(p, pol_d, dir_d, gs2, gh2, st);
  } else {
    const double* inf_nvec = G->exbuf.as<double>() + 6 * P;
    const double* inf_area = inf_nvec + 3 * exc->ninf;
    adj_rhs_sca(p, L.fields.as<double2>(), inf_nvec, inf_area, exc->ninf, P, ipol, lp.nb1.x, vv.x2, gs2, gh2, st);
  }
  MNP_CHECK_LAUNCH();
  // ---- adjoint solve A^T lam = w through the transposed chain of mldivide.m
  if (precision == MNPBEM_FP64) {
    for (int q = 0; q < 5; ++q) adj_transpose(L.mat[q].as<double2>(), n, ld, st);   // factors and matrices -> transposes
    MNP_CHECK_LAUNCH();
    MNP_TRY(chain_transpose<double>(p, chain_mats<double>(G, L), nullptr, nullptr, gs2, gh2, lam, work, gemm_w<double>,
                                    nullptr, st));
  } else {
    // complex64 transposed chain as the preconditioner of a refinement on the
    // FP64-class operator: r = w - A^T lam with A^T lam = [G1^T U_G1 + H1^T U_H1 ;
    // G2^T U_G2 + H2^T U_H2] (the weights U of lam), products of the hi / lo
    // planes in double-single arithmetic
    for (int q = 0; q < 5; ++q) adj_transpose(L.mat[q].as<float2>(), n, ld, st);
    const ChainMats<float> mT = chain_mats<float>(G, L);
    const int chunks = 32;
    MNP_TRY(G->adj2.ensure(cs * (8 * (size_t)n + 8 * (size_t)n + chunks * 4 * (size_t)n) +
                           sizeof(float2) * (8 * (size_t)n + 8 * (size_t)n + 11 * (size_t)n + 8 * (size_t)n) +
                           sizeof(double) * 4 + 256));
    double2* r64 = G->adj2.as<double2>();                 // unknown layout: sig1 | h1 | sig2 | h2
    double2* y12 = r64 + 8 * n;                            // y1 [n][4], y2 [n][4]
    double2* part = y12 + 8 * n;
    float2* r32 = reinterpret_cast<float2*>(part + chunks * 4 * n);
    float2* dl32 = r32 + 8 * n;
    float2* w32 = dl32 + 8 * n;
    float2* vsplit = w32 + 11 * n;
    double* nrm = reinterpret_cast<double*>(vsplit + 8 * n);
    const float2* hl[4];
    for (int q = 0; q < 4; ++q) hl[q] = L.mat64[q].as<float2>();
    MNP_CUDA(cudaMemsetAsync(lam, 0, cs * 8 * n, st));
    MNP_CUDA(cudaMemsetAsync(r64, 0, cs * 4 * n, st));
    MNP_CUDA(cudaMemcpyAsync(r64 + 4 * n, gs2, cs * n, cudaMemcpyDeviceToDevice, st));
    MNP_CUDA(cudaMemcpyAsync(r64 + 5 * n, gh2, cs * 3 * n, cudaMemcpyDeviceToDevice, st));
    const double tol = 1e-10;
    for (int it = 0; it < 20; ++it) {
      launch_cvt_d2f(r64, r32, 8 * n, st);
      MNP_CHECK_LAUNCH();
      MNP_TRY(chain_transpose<float>(p, mT, r32, r32 + n, r32 + 4 * n, r32 + 5 * n, dl32, w32, gemm_w<float>,
                                     tc_ctx(G, L), st));
      MNP_CUDA(cudaMemsetAsync(nrm, 0, sizeof(double) * 4, st));
      launch_axpy_norm(lam, dl32, 8 * n, nrm, st);
      MNP_CHECK_LAUNCH();
      double hn[4];
      MNP_CUDA(cudaMemcpyAsync(hn, nrm, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
      MNP_CUDA(cudaStreamSynchronize(st));
      if (!(hn[0] == hn[0])) { set_error("adjoint refinement produced NaN"); return MNPBEM_ERR_NOT_CONVERGED; }
      if (sqrt(hn[0]) <= tol * sqrt(hn[1])) break;
      // residual with the weights of the current lam
      adj_weights(p, gphi, ga, gDe, gAl, vv.x1, vv.x2, P, ipol, st);
      adj_gemm_t_ds(n, hl[0], hl[0] + n * ld, ld, Ub, 16, 0, vsplit, part, chunks, y12, st, false);
      adj_gemm_t_ds(n, hl[1], hl[1] + n * ld, ld, Ub, 16, 4, vsplit, part, chunks, y12, st, true);
      adj_gemm_t_ds(n, hl[2], hl[2] + n * ld, ld, Ub, 16, 8, vsplit, part, chunks, y12 + 4 * n, st, false);
      adj_gemm_t_ds(n, hl[3], hl[3] + n * ld, ld, Ub, 16, 12, vsplit, part, chunks, y12 + 4 * n, st, true);
      adj_resid(n, y12, y12 + 4 * n, gs2, gh2, r64, r64 + n, r64 + 4 * n, r64 + 5 * n, nrm + 2, st);
      MNP_CHECK_LAUNCH();
    }
    MNP_TRY(tc_check_error(L.tc, st));
    MNP_TRY(thin_stream_check(st));
  }
  // ---- weights, then G1 [sig1 h1], G2 [sig2 h2], H1 sig1 from freshly assembled FP64 matrices
  adj_weights(p, gphi, ga, gDe, gAl, vv.x1, vv.x2, P, ipol, st);
  MNP_CHECK_LAUNCH();
  {
    const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
    AsmParams ap = base_params(G, L.lp_dev.as<LamParams>());
    double2* AM = G->adj_mats.as<double2>();
    ap.ld64 = ld;
    ap.G1 = AM; ap.H1 = AM + n * ld; ap.G2 = AM + 2 * n * ld; ap.H2 = nullptr;
    MNP_TRY(assemble_launch(ap, true, false, st));
    MNP_TRY(gemm_simt<double>(n, 4, n, one, ap.G1, ld, Xb, 8, zero, GX1, 4, st));
    MNP_TRY(gemm_simt<double>(n, 4, n, one, ap.G2, ld, Xb + 4, 8, zero, GX2, 4, st));
    MNP_TRY(gemm_simt<double>(n, 1, n, one, ap.H1, ld, Xb, 8, zero, HX1, 1, st));
  }
  // ---- geometric contractions and the chain rule to the vertices
  adj_geometry(p, which, pol_d, dir_d, gphi, ga, gDe, gAl, GX1, GX2, HX1, geps, st);
  MNP_CHECK_LAUNCH();
  MNP_CUDA(cudaMemcpyAsync(verts_grad, p.gv, sizeof(double) * 3 * nv, cudaMemcpyDeviceToHost, st));
  double hk[4];
  MNP_CUDA(cudaMemcpyAsync(hk, p.gk1, sizeof(double) * 4, cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  G->prof.flush();
  // eps of the inside medium: k1 = k0 sqrt(eps) (dk1/deps = k1 / (2 eps)) plus the explicit eps1
  const std::complex<double> gk1(hk[0], hk[1]), gex(hk[2], hk[3]);
  const std::complex<double> k1(p.k1.x, p.k1.y), e1(lp.eps[in - 1].x, lp.eps[in - 1].y);
  const std::complex<double> g = -(gk1 * (k1 / (2.0 * e1)) + gex);
  eps_grad[0] = g.real();     // dJ / dRe(eps)
  eps_grad[1] = -g.imag();    // dJ / dIm(eps)
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
  Lane& L = *G->lanes[0];
  MNP_TRY(ensure_workspace(G, L, precision, 1, 0));
  LamParams lp;
  fill_lp(lp, enei, eps_media, nmed, 1, 0);
  MNP_CUDA(cudaMemcpyAsync(L.lp_dev.ptr, &lp, sizeof(LamParams), cudaMemcpyHostToDevice, L.st));
  MNP_TRY(stage_assemble(G, L, precision));
  if (precision == MNPBEM_FP64) MNP_TRY(stage_initmat<double>(G, L, true));
  else MNP_TRY(stage_initmat<float>(G, L, true));
  MNP_TRY(status_copy(L, precision));
  MNP_CUDA(cudaStreamSynchronize(L.st));
  MNP_TRY(check_pivots(L, precision));
  // Sigma1 and Deltai as stored (mat[2], mat[4]); G1i, G2i and Sigmai from the
  // LDU factors (mat[0], mat[1], mat[3]) by solves with the identity
  double* outs[5] = {G1i, G2i, Sigma1, Sigmai, Deltai};  // order of mat[0..4]
  DevBuf conv, inv, tmp;
  if (precision == MNPBEM_MIXED) MNP_TRY(conv.ensure(sizeof(double2) * n * ld));
  const size_t es = precision == MNPBEM_FP64 ? sizeof(double2) : sizeof(float2);
  for (int q = 0; q < 5; ++q) {
    if (!outs[q]) continue;
    const void* m = L.mat[q].ptr;
    if (q == 0 || q == 1 || q == 3) {
      MNP_TRY(inv.ensure(es * n * ld));
      MNP_TRY(tmp.ensure(es * 256 * n));
      if (precision == MNPBEM_FP64) MNP_TRY(ldu_inverse<double>(G, L, q, inv.as<double2>(), tmp.as<double2>()));
      else MNP_TRY(ldu_inverse<float>(G, L, q, inv.as<float2>(), tmp.as<float2>()));
      m = inv.ptr;
    }
    const double2* src = static_cast<const double2*>(m);
    if (precision == MNPBEM_MIXED) {
      launch_cvt_f2d(static_cast<const float2*>(m), conv.as<double2>(), n * ld, L.st);
      MNP_CHECK_LAUNCH();
      src = conv.as<double2>();
    }
    MNP_CUDA(cudaMemcpy2DAsync(outs[q], sizeof(double2) * n, src, sizeof(double2) * ld,
                               sizeof(double2) * n, n, cudaMemcpyDeviceToHost, L.st));
    MNP_CUDA(cudaStreamSynchronize(L.st));
  }
  G->prof.flush();
  return MNPBEM_OK;
}

}  // extern "C"

mnpbem_status mnpbem_fields(mnpbem_geom* G, int64_t npts, const double* pts, const int32_t* pt_medium,
                            double enei, const double* eps_media, int32_t nmed, int32_t npol,
                            const double* sig1, const double* sig2, const double* h1, const double* h2,
                            double* e, double* h) {
  MNP_TRY(check_geom(G));
  if (npts <= 0 || !pts || !pt_medium || !(enei > 0) || !eps_media || nmed < G->max_medium || npol < 1 ||
      !sig1 || !sig2 || !h1 || !h2 || (!e && !h)) {
    set_error("mnpbem_fields: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  const int64_t n = G->g.n;
  const double k0 = 2 * M_PI / enei;
  std::vector<double2> km(nmed);
  for (int m = 0; m < nmed; ++m) {
    const std::complex<double> kk = k0 * std::sqrt(std::complex<double>(eps_media[2 * m], eps_media[2 * m + 1]));
    km[m] = make_double2(kk.real(), kk.imag());
  }
  DevBuf ds, dout;
  MNP_TRY(ds.ensure(sizeof(double2) * 8 * n * npol));
  MNP_TRY(dout.ensure(sizeof(double2) * 6 * npts * npol));
  double2* S = ds.as<double2>();
  double2 *s1 = S, *s2 = S + n * npol, *q1 = S + 2 * n * npol, *q2 = S + 5 * n * npol;
  cudaStream_t st = G->st;
  MNP_CUDA(cudaMemcpyAsync(s1, sig1, sizeof(double2) * n * npol, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(s2, sig2, sizeof(double2) * n * npol, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(q1, h1, sizeof(double2) * 3 * n * npol, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(q2, h2, sizeof(double2) * 3 * n * npol, cudaMemcpyHostToDevice, st));
  double2* de = dout.as<double2>();
  double2* dh = de + 3 * npts * npol;
  MNP_TRY(point_fields(G->g, G->face_med.as<int>(), npts, pts, pt_medium, km.data(), nmed, k0, npol, s1, s2, q1, q2,
                       de, dh, G->rel_cut, G->abs_cut, st));
  if (e) MNP_CUDA(cudaMemcpyAsync(e, de, sizeof(double2) * 3 * npts * npol, cudaMemcpyDeviceToHost, st));
  if (h) MNP_CUDA(cudaMemcpyAsync(h, dh, sizeof(double2) * 3 * npts * npol, cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  G->prof.flush();
  return MNPBEM_OK;
}

mnpbem_status mnpbem_surface_fields(mnpbem_geom* G, double enei, const double* eps_media, int32_t nmed,
                                    int32_t npol, int32_t inout, const double* sig1, const double* sig2,
                                    const double* h1, const double* h2, double* e, double* h, double* phi,
                                    double* phip, double* a, double* ap) {
  MNP_TRY(check_geom(G));
  if (!(enei > 0) || !eps_media || nmed < G->max_medium || npol < 1 || (inout != 1 && inout != 2) ||
      !sig1 || !sig2 || !h1 || !h2 || (!e && !h && !phi && !phip && !a && !ap)) {
    set_error("mnpbem_surface_fields: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  if (npol > 4) { set_error("mnpbem_surface_fields: npol must be 1..4"); return MNPBEM_ERR_UNSUPPORTED; }
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  const int64_t n = G->g.n;
  const double k0 = 2 * M_PI / enei;
  std::vector<double2> km(nmed);
  for (int m = 0; m < nmed; ++m) {
    const std::complex<double> kk = k0 * std::sqrt(std::complex<double>(eps_media[2 * m], eps_media[2 * m + 1]));
    km[m] = make_double2(kk.real(), kk.imag());
  }
  // inputs: sig1, sig2 [n][npol], h1, h2 [n][3][npol]; outputs: e, h, a, ap
  // [n][3][npol], phi, phip [n][npol]; the wavenumbers of the media last
  DevBuf buf;
  const int64_t np = n * npol;
  MNP_TRY(buf.ensure(sizeof(double2) * (8 * np + 14 * np + nmed)));
  double2* S = buf.as<double2>();
  double2 *s1 = S, *s2 = S + np, *q1 = S + 2 * np, *q2 = S + 5 * np, *O = S + 8 * np;
  double2 *de = O, *dh = O + 3 * np, *dphi = O + 6 * np, *dphip = O + 7 * np, *da = O + 8 * np, *dap = O + 11 * np;
  double2* dk = O + 14 * np;
  cudaStream_t st = G->st;
  MNP_CUDA(cudaMemcpyAsync(s1, sig1, sizeof(double2) * np, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(s2, sig2, sizeof(double2) * np, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(q1, h1, sizeof(double2) * 3 * np, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(q2, h2, sizeof(double2) * 3 * np, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(dk, km.data(), sizeof(double2) * nmed, cudaMemcpyHostToDevice, st));
  MNP_TRY(surface_fields(G->g, G->face_med.as<int>(), dk, k0, npol, inout - 1, s1, s2, q1, q2,
                         e ? de : nullptr, h ? dh : nullptr, phi ? dphi : nullptr, phip ? dphip : nullptr,
                         a ? da : nullptr, ap ? dap : nullptr, st));
  if (e) MNP_CUDA(cudaMemcpyAsync(e, de, sizeof(double2) * 3 * np, cudaMemcpyDeviceToHost, st));
  if (h) MNP_CUDA(cudaMemcpyAsync(h, dh, sizeof(double2) * 3 * np, cudaMemcpyDeviceToHost, st));
  if (phi) MNP_CUDA(cudaMemcpyAsync(phi, dphi, sizeof(double2) * np, cudaMemcpyDeviceToHost, st));
  if (phip) MNP_CUDA(cudaMemcpyAsync(phip, dphip, sizeof(double2) * np, cudaMemcpyDeviceToHost, st));
  if (a) MNP_CUDA(cudaMemcpyAsync(a, da, sizeof(double2) * 3 * np, cudaMemcpyDeviceToHost, st));
  if (ap) MNP_CUDA(cudaMemcpyAsync(ap, dap, sizeof(double2) * 3 * np, cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  G->prof.flush();
  return MNPBEM_OK;
}

mnpbem_status mnpbem_farfield(mnpbem_geom* G, double enei, const double* eps_media, int32_t nmed, int32_t medium,
                              int64_t ndir, const double* dirs, int32_t npol, const double* sig1,
                              const double* sig2, const double* h1, const double* h2, double* e, double* h) {
  MNP_TRY(check_geom(G));
  if (!(enei > 0) || !eps_media || nmed < G->max_medium || medium < 1 || medium > nmed || ndir <= 0 ||
      ndir > ((int64_t)1 << 30) || !dirs || npol < 1 || !sig1 || !sig2 || !h1 || !h2 || (!e && !h)) {
    set_error("mnpbem_farfield: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  if (npol > 4) { set_error("mnpbem_farfield: npol must be 1..4"); return MNPBEM_ERR_UNSUPPORTED; }
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  const int64_t n = G->g.n, np = n * npol, nd = ndir * npol;
  const double k0 = 2 * M_PI / enei;
  const std::complex<double> kk =
      k0 * std::sqrt(std::complex<double>(eps_media[2 * (medium - 1)], eps_media[2 * (medium - 1) + 1]));
  // inputs sig1, sig2 [n][npol], h1, h2 [n][3][npol]; outputs e, h [ndir][3][npol]; directions last
  DevBuf buf;
  MNP_TRY(buf.ensure(sizeof(double2) * (8 * np + 6 * nd) + sizeof(double) * 3 * ndir));
  double2* S = buf.as<double2>();
  double2 *s1 = S, *s2 = S + np, *q1 = S + 2 * np, *q2 = S + 5 * np, *de = S + 8 * np, *dh = de + 3 * nd;
  double* dd = reinterpret_cast<double*>(dh + 3 * nd);
  cudaStream_t st = G->st;
  MNP_CUDA(cudaMemcpyAsync(s1, sig1, sizeof(double2) * np, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(s2, sig2, sizeof(double2) * np, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(q1, h1, sizeof(double2) * 3 * np, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(q2, h2, sizeof(double2) * 3 * np, cudaMemcpyHostToDevice, st));
  MNP_CUDA(cudaMemcpyAsync(dd, dirs, sizeof(double) * 3 * ndir, cudaMemcpyHostToDevice, st));
  MNP_TRY(far_fields(G->g, G->face_med.as<int>(), medium - 1, make_double2(kk.real(), kk.imag()), k0, npol,
                     (int)ndir, dd, s1, s2, q1, q2, e ? de : nullptr, h ? dh : nullptr, st));
  if (e) MNP_CUDA(cudaMemcpyAsync(e, de, sizeof(double2) * 3 * nd, cudaMemcpyDeviceToHost, st));
  if (h) MNP_CUDA(cudaMemcpyAsync(h, dh, sizeof(double2) * 3 * nd, cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  G->prof.flush();
  return MNPBEM_OK;
}

mnpbem_status mnpbem_solve_potentials(mnpbem_geom* G, const mnpbem_potentials* pot, double enei,
                                      const double* eps_media, int32_t nmed, int32_t precision,
                                      const mnpbem_refine* refine, mnpbem_solution* out) {
  MNP_TRY(check_geom(G));
  if (!pot || pot->npol < 1 || pot->npol > 4 || !out || !(enei > 0)) {
    set_error("mnpbem_solve_potentials: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  const int P = pot->npol;
  const double* src[8] = {pot->phi1, pot->phi1p, pot->phi2, pot->phi2p, pot->a1, pot->a1p, pot->a2, pot->a2p};
  // a plane wave without directions stands in for the job's excitation; the
  // potentials replace its excitation and no spectra are computed
  std::vector<double> zero(3 * P, 0.0);
  mnpbem_planewave pw{P, zero.data(), zero.data(), 1, 0, nullptr, nullptr};
  mnpbem_solution o = *out;
  o.ext = o.sca = nullptr;
  MNP_TRY(validate_job(G, &pw, 1, &enei, eps_media, nmed, precision, &o));
  MNP_CUDA(cudaSetDevice(G->device));
  const int64_t n = G->g.n;
  DevBuf dpot;
  MNP_TRY(dpot.ensure(sizeof(double2) * 16 * n * P));
  double2* D = dpot.as<double2>();
  for (int q = 0; q < 8; ++q) {
    const int64_t cnt = (q < 4 ? 1 : 3) * n * P;
    double2* dst = D + (q < 4 ? q * n * P : 4 * n * P + (q - 4) * 3 * n * P);
    if (src[q])
      MNP_CUDA(cudaMemcpyAsync(dst, src[q], sizeof(double2) * cnt, cudaMemcpyHostToDevice, G->st));
    else
      MNP_CUDA(cudaMemsetAsync(dst, 0, sizeof(double2) * cnt, G->st));
  }
  MNP_CUDA(cudaStreamSynchronize(G->st));
  std::vector<Job> jobs(1);
  jobs[0].G = G;
  MNP_TRY(job_setup(jobs[0], &pw, 1, &enei, eps_media, nmed, precision, refine, &o));
  jobs[0].c.ext_pot = D;
  jobs[0].c.spectra = false;
  jobs[0].nl = 1;
  return run_jobs(jobs);
}

// ======================================================================
// iterative solver: H-matrices + preconditioned GMRES
// ======================================================================
namespace {

// index arrays, values and factors of the H-matrices of one cluster tree
struct HmatHost {
  DevBuf idx, vals, fac, fact, used, tbuf, xsbuf;
  HmatDev d;
  LeafAsm la;
  std::vector<int4> lblk;   // host copy of the low-rank blocks
  std::vector<int4> fblk;   // host copy of the full blocks
  std::vector<int64_t> foff, aoff, boff;   // host copies of the value / factor offsets
  std::vector<int> ranks;   // [4][nlow] ACA ranks of the current wavelength
  double mv_bytes = 0.0;    // algorithmic bytes of one product of the four matrices
};

template <typename T>
T* carve(char*& p, size_t count) {
  T* r = reinterpret_cast<T*>(p);
  p += ((sizeof(T) * count + 255) / 256) * 256;
  return r;
}
size_t carve_size(size_t bytes) { return ((bytes + 255) / 256) * 256; }

mnpbem_status hmat_setup(mnpbem_geom* G, const mnpbem_cluster_tree* t, int kmax, double htol, HmatHost& H,
                         cudaStream_t st) {
  const int n = (int)G->g.n;
  const int nc = t ? t->ncluster : 0;
  auto bad = [](const char* why) {
    set_error("cluster tree: %s", why);
    return MNPBEM_ERR_INVALID_ARG;
  };
  if (!t || nc < 1 || !t->son || !t->cind || !t->ipart || !t->perm || t->nfull < 0 || t->nlow < 0 ||
      (t->nfull > 0 && !t->full) || (t->nlow > 0 && !t->low))
    return bad("missing arrays");
  if (kmax < 1 || kmax > ACA_KMAX || !(htol > 0)) {
    set_error("iterative solver: kmax must be 1..%d and htol > 0", ACA_KMAX);
    return MNPBEM_ERR_INVALID_ARG;
  }
  std::vector<int> iperm(n, -1);
  for (int c = 0; c < n; ++c) {
    const int f = t->perm[c];
    if (f < 0 || f >= n || iperm[f] >= 0) return bad("perm is not a permutation of the faces");
    iperm[f] = c;
  }
  for (int c = 0; c < nc; ++c) {
    const int a = t->cind[2 * c], b = t->cind[2 * c + 1];
    if (a < 0 || b < a || b >= n) return bad("cluster range out of bounds");
    for (int s = 0; s < 2; ++s)
      if (t->son[2 * c + s] < -1 || t->son[2 * c + s] >= nc) return bad("son index out of range");
  }
  // leaves tile [0, n)
  std::vector<int> leaves;
  for (int c = 0; c < nc; ++c)
    if (t->son[2 * c] < 0) leaves.push_back(c);
  std::sort(leaves.begin(), leaves.end(), [&](int a, int b) { return t->cind[2 * a] < t->cind[2 * b]; });
  const int nleaf = (int)leaves.size();
  std::vector<int> leaf_id(nc, -1), leaf_of(n, -1);
  {
    int pos = 0;
    for (int l = 0; l < nleaf; ++l) {
      const int c = leaves[l];
      if (t->cind[2 * c] != pos) return bad("leaves do not tile the faces");
      for (int i = t->cind[2 * c]; i <= t->cind[2 * c + 1]; ++i) leaf_of[i] = l;
      pos = t->cind[2 * c + 1] + 1;
      leaf_id[c] = l;
    }
    if (pos != n) return bad("leaves do not tile the faces");
  }
  auto rows = [&](int c) { return t->cind[2 * c + 1] - t->cind[2 * c] + 1; };
  const int nf = t->nfull, nlow = t->nlow;
  std::vector<int4> fblk(nf), lblk(nlow);
  std::vector<int64_t> foff(nf), aoff(nlow), boff(nlow), uoff(nlow), toff(nlow);
  std::vector<int> kcap(nlow), fidx((size_t)nleaf * nleaf, -1);
  double area = 0.0;
  int64_t nvals = 0, asz = 0, bsz = 0, usz = 0, tsz = 0;
  for (int b = 0; b < nf; ++b) {
    const int r = t->full[2 * b], c = t->full[2 * b + 1];
    if (r < 0 || r >= nc || c < 0 || c >= nc || leaf_id[r] < 0 || leaf_id[c] < 0)
      return bad("full blocks must be leaf pairs");
    fblk[b] = make_int4(t->cind[2 * r], rows(r), t->cind[2 * c], rows(c));
    foff[b] = nvals;
    nvals += (int64_t)rows(r) * rows(c);
    fidx[(size_t)leaf_id[r] * nleaf + leaf_id[c]] = b;
    area += (double)rows(r) * rows(c);
  }
  for (int b = 0; b < nlow; ++b) {
    const int r = t->low[2 * b], c = t->low[2 * b + 1];
    if (r < 0 || r >= nc || c < 0 || c >= nc) return bad("low-rank block cluster out of range");
    const int m = rows(r), nb = rows(c);
    // the product walks a block's rows leaf by leaf: its row range must start
    // and end on leaf boundaries
    const int r0 = t->cind[2 * r], r1 = t->cind[2 * r + 1];
    if (t->cind[2 * leaves[leaf_of[r0]]] != r0 || t->cind[2 * leaves[leaf_of[r1]] + 1] != r1)
      return bad("a low-rank block's rows do not start and end on leaf boundaries");
    lblk[b] = make_int4(t->cind[2 * r], m, t->cind[2 * c], nb);
    kcap[b] = std::min(kmax, std::min(m, nb));
    aoff[b] = asz; asz += (int64_t)m * kcap[b];
    boff[b] = bsz; bsz += (int64_t)nb * kcap[b];
    uoff[b] = usz; usz += m;
    toff[b] = tsz; tsz += (int64_t)kcap[b] * HMV_NMAX;
    area += (double)m * nb;
  }
  if (area != (double)n * n) return bad("blocks do not partition the matrix");
  // blocks covering each leaf's rows: full blocks of the leaf, then low-rank
  // blocks whose row cluster contains it
  std::vector<std::vector<int>> cover(nleaf);
  for (int b = 0; b < nf; ++b) cover[leaf_id[t->full[2 * b]]].push_back(b);
  for (int b = 0; b < nlow; ++b)
    for (int i = lblk[b].x; i < lblk[b].x + lblk[b].y;) {
      const int l = leaf_of[i];
      cover[l].push_back(~b);
      i = t->cind[2 * leaves[l] + 1] + 1;
    }
  std::vector<int> lptr(nleaf + 1, 0), lent;
  std::vector<int2> leaf(nleaf);
  for (int l = 0; l < nleaf; ++l) {
    leaf[l] = make_int2(t->cind[2 * leaves[l]], rows(leaves[l]));
    lent.insert(lent.end(), cover[l].begin(), cover[l].end());
    lptr[l + 1] = (int)lent.size();
  }
  // device copies
  const size_t bytes = carve_size(sizeof(int) * 3 * n) + carve_size(sizeof(int) * fidx.size()) +
                       carve_size(sizeof(int4) * (nf + nlow)) + carve_size(sizeof(int64_t) * (nf + 4 * nlow)) +
                       carve_size(sizeof(int) * (2 * nlow + 4 * nlow)) + carve_size(sizeof(int2) * nleaf) +
                       carve_size(sizeof(int) * (nleaf + 1 + lent.size())) + 4096;
  MNP_TRY(H.idx.ensure(bytes));
  char* p = static_cast<char*>(H.idx.ptr);
  std::vector<char> host(bytes, 0);
  char* hp = host.data();
  auto put = [&](const void* src, size_t nbytes) -> void* {
    const size_t off = (size_t)(hp - host.data());
    if (nbytes) memcpy(hp, src, nbytes);
    hp += carve_size(nbytes);
    return p + off;
  };
  std::vector<int> perm(t->perm, t->perm + n);
  H.la.perm = H.d.perm = static_cast<const int*>(put(perm.data(), sizeof(int) * n));
  H.la.iperm = static_cast<const int*>(put(iperm.data(), sizeof(int) * n));
  H.la.leaf_of = static_cast<const int*>(put(leaf_of.data(), sizeof(int) * n));
  H.la.fidx = static_cast<const int*>(put(fidx.data(), sizeof(int) * fidx.size()));
  H.la.fblk = H.d.fblk = static_cast<const int4*>(put(fblk.data(), sizeof(int4) * nf));
  H.la.foff = H.d.foff = static_cast<const int64_t*>(put(foff.data(), sizeof(int64_t) * nf));
  H.d.lblk = static_cast<const int4*>(put(lblk.data(), sizeof(int4) * nlow));
  H.d.kcap = static_cast<const int*>(put(kcap.data(), sizeof(int) * nlow));
  H.d.aoff = static_cast<const int64_t*>(put(aoff.data(), sizeof(int64_t) * nlow));
  H.d.boff = static_cast<const int64_t*>(put(boff.data(), sizeof(int64_t) * nlow));
  H.d.uoff = static_cast<const int64_t*>(put(uoff.data(), sizeof(int64_t) * nlow));
  H.d.toff = static_cast<const int64_t*>(put(toff.data(), sizeof(int64_t) * nlow));
  std::vector<int> zr(4 * (size_t)nlow, 0);
  H.d.rank = static_cast<int*>(put(zr.data(), sizeof(int) * zr.size()));
  H.d.leaf = static_cast<const int2*>(put(leaf.data(), sizeof(int2) * nleaf));
  H.d.lptr = static_cast<const int*>(put(lptr.data(), sizeof(int) * lptr.size()));
  H.d.lent = static_cast<const int*>(put(lent.data(), sizeof(int) * lent.size()));
  if ((size_t)(hp - host.data()) > bytes) return bad("internal: index buffer size");
  MNP_CUDA(cudaMemcpyAsync(H.idx.ptr, host.data(), (size_t)(hp - host.data()), cudaMemcpyHostToDevice, st));
  // values, factors, scratch
  MNP_TRY(H.vals.ensure(sizeof(double2) * 4 * std::max<int64_t>(1, nvals)));
  MNP_TRY(H.fac.ensure(sizeof(double2) * 4 * std::max<int64_t>(1, asz + bsz)));
  MNP_TRY(H.fact.ensure(sizeof(float4) * 4 * std::max<int64_t>(1, asz)));
  MNP_TRY(H.used.ensure(4 * std::max<int64_t>(1, usz)));
  MNP_TRY(H.tbuf.ensure(sizeof(float4) * 4 * std::max<int64_t>(1, tsz)));
  MNP_TRY(H.xsbuf.ensure(sizeof(float4) * 2 * (size_t)n * HMV_NMAX));
  for (int q = 0; q < 4; ++q) {
    H.la.val[q] = H.d.val[q] = H.vals.as<double2>() + q * nvals;
    H.d.A[q] = H.fac.as<double2>() + q * (asz + bsz);
    H.d.B[q] = H.d.A[q] + asz;
    H.d.At[q] = H.fact.as<float4>() + q * asz;
  }
  H.d.used = H.used.as<unsigned char>();
  H.d.T = H.tbuf.as<float4>();
  H.d.xs = H.xsbuf.as<float4>();
  H.d.nvals = nvals;
  H.d.n = n; H.d.nfull = nf; H.d.nlow = nlow; H.d.nleaf = nleaf;
  H.d.tol = htol;
  H.d.usz = usz; H.d.tsz = tsz;
  H.la.nfull = nf; H.la.nleaf = nleaf; H.la.nvals = nvals;
  H.lblk = lblk;
  H.fblk = fblk;
  H.foff = foff;
  H.aoff = aoff;
  H.boff = boff;
  MNP_CUDA(cudaStreamSynchronize(st));
  return MNPBEM_OK;
}

// FP64 values and factors of the four H-matrices as H-arithmetic blocks
// (column-major copies on the H stream, made before hmat_split overwrites the
// right factors); ranks already on the host
__global__ void k_rm_to_cm(const double2* src, int m, int n, double2* dst) {
  const int64_t cnt = (int64_t)m * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % m), j = (int)(e / m);
    dst[e] = src[(int64_t)i * n + j];
  }
}

mnpbem_status hmat_capture(Lane& L, HmatHost& H, hl::Ctx& c, hl::HM out[4]) {
  cudaEvent_t ev[2] = {nullptr, nullptr};
  for (auto& e : ev) MNP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  struct EvFree {
    cudaEvent_t* e;
    ~EvFree() { for (int i = 0; i < 2; ++i) if (e[i]) cudaEventDestroy(e[i]); }
  } ef{ev};
  MNP_CUDA(cudaEventRecord(ev[0], L.st));
  MNP_CUDA(cudaStreamWaitEvent(c.st, ev[0], 0));
  const hl::Tree& T = *c.t;
  for (int q = 0; q < 4; ++q) {
    out[q].clear();
    for (size_t b = 0; b < T.full.size(); ++b) {
      const int4 fb = H.fblk[b];
      hl::Sub S;
      S.row = T.full[b].first; S.col = T.full[b].second; S.flag = hl::FLAG_FULL;
      MNP_TRY(hl::alloc(c, fb.y, fb.w, S.mat));
      const int64_t cnt = (int64_t)fb.y * fb.w;
      k_rm_to_cm<<<(unsigned)std::min<int64_t>(cdiv_up(cnt, 256), 4096), 256, 0, c.st>>>(H.d.val[q] + H.foff[b], fb.y,
                                                                                        fb.w, S.mat.ptr());
      MNP_CHECK_LAUNCH();
      out[q][T.full[b]] = std::move(S);
    }
    for (size_t b = 0; b < T.low.size(); ++b) {
      const int4 lb = H.lblk[b];
      const int k = H.ranks[(size_t)q * H.d.nlow + b];
      hl::Sub S;
      S.row = T.low[b].first; S.col = T.low[b].second; S.flag = hl::FLAG_RK;
      MNP_TRY(hl::alloc(c, lb.y, k, S.lhs));
      MNP_TRY(hl::alloc(c, lb.w, k, S.rhs));
      if (k > 0) {
        MNP_CUDA(cudaMemcpyAsync(S.lhs.ptr(), H.d.A[q] + H.aoff[b], sizeof(double2) * lb.y * k,
                                 cudaMemcpyDeviceToDevice, c.st));
        MNP_CUDA(cudaMemcpyAsync(S.rhs.ptr(), H.d.B[q] + H.boff[b], sizeof(double2) * lb.w * k,
                                 cudaMemcpyDeviceToDevice, c.st));
      }
      out[q][T.low[b]] = std::move(S);
    }
  }
  MNP_CUDA(cudaEventRecord(ev[1], c.st));
  MNP_CUDA(cudaStreamWaitEvent(L.st, ev[1], 0));
  return MNPBEM_OK;
}

// full blocks and ACA of one wavelength (lane parameters lp_dev); ranks to
// the host, bytes of a product with N columns.  cap: copies of the FP64
// blocks for the H-matrix arithmetic (NULL: none)
mnpbem_status hmat_fill(mnpbem_geom* G, Lane& L, HmatHost& H, int N, hl::Ctx* cap = nullptr,
                        hl::HM* out = nullptr) {
  AsmParams p = base_params(G, L.lp_dev.as<LamParams>());
  MNP_TRY(assemble_leaves(p, H.la, L.st));
  MNP_TRY(hmat_aca(p, H.d, L.st));
  H.ranks.assign((size_t)4 * H.d.nlow, 0);
  if (!H.ranks.empty())
    MNP_CUDA(cudaMemcpyAsync(H.ranks.data(), H.d.rank, sizeof(int) * H.ranks.size(), cudaMemcpyDeviceToHost, L.st));
  MNP_CUDA(cudaStreamSynchronize(L.st));
  if (cap) MNP_TRY(hmat_capture(L, H, *cap, out));
  MNP_TRY(hmat_split(H.d, L.st));
  MNP_CUDA(cudaStreamSynchronize(L.st));
  double entries = 4.0 * (double)H.la.nvals;
  for (int q = 0; q < 4; ++q)
    for (int b = 0; b < H.d.nlow; ++b)
      entries += (double)H.ranks[(size_t)q * H.d.nlow + b] * (H.lblk[b].y + H.lblk[b].w);
  H.mv_bytes = 16.0 * (entries + 4.0 * 2.0 * (double)H.d.n * N);
  return MNPBEM_OK;
}

void face_eps(mnpbem_geom* G, Lane& L) {
  const int* fm = G->face_med.as<int>();
  FaceData f = face_data(G, L);
  launch_face_eps(G->g.n, fm, fm + G->g.n, L.lp_dev.as<LamParams>(), G->g.nvec, const_cast<double2*>(f.eps1),
                  const_cast<double2*>(f.eps2), const_cast<float2*>(f.eps1f), const_cast<float2*>(f.eps2f),
                  const_cast<float2*>(f.Lf), const_cast<float*>(f.nvecf), L.st);
}

struct IterOpts {
  int solver = 0;   // 0 gmres, 1 cgs, 2 bicgstab
  double tol = 1e-6, htol = 1e-6;
  int maxit = 100, restart = 0, precond = 1, kmax = 100;
  int kmax_pc = 4;   // rank cap of the 'hmat' preconditioner's arithmetic (compress.m: min(op.kmax))
  double htol_pc = 1e-6;   // its ACA tolerance (compress.m: max(op.htol))
  int reuse = 0, refresh = 0;
};

mnpbem_status iter_opts(const mnpbem_iter_options* op, IterOpts& o) {
  if (op) {
    if (op->solver < 0 || op->solver > 2) {
      set_error("iterative solver: solver must be 0 (gmres), 1 (cgs) or 2 (bicgstab)");
      return MNPBEM_ERR_INVALID_ARG;
    }
    o.solver = op->solver;
    if (op->tol > 0) o.tol = op->tol;
    if (op->maxit > 0) o.maxit = op->maxit;
    if (op->restart > 0) o.restart = op->restart;
    if (op->precond >= 0 && op->precond <= 2) o.precond = op->precond;
    else { set_error("iterative solver: precond must be 0, 1 or 2"); return MNPBEM_ERR_INVALID_ARG; }
    if (op->htol > 0) o.htol = op->htol;
    if (op->kmax > 0) o.kmax = op->kmax;
    if (op->kmax_precond > 0) o.kmax_pc = op->kmax_precond;
    o.htol_pc = op->htol_precond > 0 ? op->htol_precond : o.htol;
    o.reuse = op->reuse_precond != 0;
    o.refresh = std::max(0, op->refresh_steps);
  }
  return MNPBEM_OK;
}

// Restarted, left-preconditioned GMRES on M A x = M b (@bemiter/solve.m with
// the afun / mfun of bemretiter), x-space vectors [x1 | x2] of 8 n P complex:
// classical Gram-Schmidt applied twice, complex Givens rotations, stop when
// ||M (b - A x)|| <= tol ||M b|| (estimated in the cycle, confirmed with the
// true preconditioned residual after it).
struct Gmres {
  mnpbem_geom* G;
  Lane& L;
  const SolveCtx& c;
  HmatHost& H;
  const IterOpts& o;
  int64_t n, len;
  int P;
  DevBuf V, part, hdev, zero, rvec;
  std::vector<double2> hpart;
  std::vector<double> npart;
  FaceData fdp;                // per-face data of the preconditioner's wavelength
  const LamParams* lpp;        // its parameters

  Gmres(mnpbem_geom* G_, Lane& L_, const SolveCtx& c_, HmatHost& H_, const IterOpts& o_)
      : G(G_), L(L_), c(c_), H(H_), o(o_), n(G_->g.n), len(8 * G_->g.n * c_.P), P(c_.P),
        fdp(face_data_in(G_, L_.pc_face)), lpp(L_.pc_lp.as<LamParams>()) {}

  // (rphi, ra, ral, rDe) = b - A x with b = (bphi, ba, bal, bDe); norms[0..1] += ||r||^2, ||b||^2
  mnpbem_status residual(const double2* x, const double2* bphi, const double2* ba, const double2* bal,
                         const double2* bDe) {
    Vec64 v = vec64(G, L, P);
    double2* y[4] = {v.Y1, v.Z1, v.Y2, v.Z2};
    MNP_TRY(hmat_mv(H.d, 4 * P, x, x + 4 * n * P, y, H.mv_bytes, L.st));
    launch_residual(face_data(G, L), P, L.lp_dev.as<LamParams>(), v.Y1, v.Y2, v.Z1, v.Z2, bphi, ba, bal, bDe,
                    v.rphi, v.ra, v.ral, v.rDe, L.norms.as<double>(), L.st);
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  // dst (x-space) = M applied to the b-space vector (phi, a, alpha, De)
  mnpbem_status precond(const double2* phi, const double2* a, const double2* al, const double2* De, double2* dst) {
    Vec64 v = vec64(G, L, P);
    if (!o.precond) {
      kv_pack_bx(n, P, phi, a, al, De, dst, L.st);
    } else if (o.precond == 2) {
      // H-matrix LU preconditioner on the H stream, ordered with the lane
      hl::HPrecond& h = *L.hpc;
      cudaEvent_t ev[2] = {nullptr, nullptr};
      for (auto& e : ev) MNP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      mnpbem_status s = MNPBEM_OK;
      cudaError_t ce = cudaEventRecord(ev[0], L.st);
      if (ce == cudaSuccess) ce = cudaStreamWaitEvent(h.c->st, ev[0], 0);
      if (ce == cudaSuccess) s = hl::precond_apply(h, P, phi, a, al, De, dst);
      if (ce == cudaSuccess && s == MNPBEM_OK) ce = cudaEventRecord(ev[1], h.c->st);
      if (ce == cudaSuccess && s == MNPBEM_OK) ce = cudaStreamWaitEvent(L.st, ev[1], 0);
      for (auto& e : ev) cudaEventDestroy(e);
      MNP_CUDA(ce);
      MNP_TRY(s);
    } else if (c.precision == MNPBEM_FP64) {
      MNP_TRY(apply_mldivide<double>(fdp, P, lpp, chain_mats<double>(G, L), phi, a, al, De, dst, dst + 4 * n * P,
                                     v.work, gemm_w<double>, nullptr, L.st));
    } else {
      MNP_TRY(apply32_at(G, L, P, fdp, lpp, phi, a, al, De));
      launch_cvt_f2d(fx_ptr(G, L, P, 0), dst, 4 * n * P, L.st);
      launch_cvt_f2d(fx_ptr(G, L, P, 1), dst + 4 * n * P, 4 * n * P, L.st);
    }
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  // dst = M A x
  mnpbem_status op(const double2* x, double2* dst) {
    const double2* z = zero.as<double2>();
    MNP_TRY(residual(x, z, z + n * P, z + 4 * n * P, z + 7 * n * P));   // -A x
    Vec64 v = vec64(G, L, P);
    MNP_TRY(precond(v.rphi, v.ra, v.ral, v.rDe, dst));
    kv_scale(dst, len, -1.0, dst, L.st);
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  mnpbem_status norm(const double2* w, double& out) {
    kv_norm2(w, len, part.as<double>(), L.st);
    MNP_CHECK_LAUNCH();
    npart.resize(KV_BLOCKS);
    MNP_CUDA(cudaMemcpyAsync(npart.data(), part.ptr, sizeof(double) * KV_BLOCKS, cudaMemcpyDeviceToHost, L.st));
    MNP_CUDA(cudaStreamSynchronize(L.st));
    double s = 0.0;
    for (double q : npart) s += q;
    out = sqrt(s);
    return MNPBEM_OK;
  }
  mnpbem_status dots(int nv, const double2* w, std::vector<std::complex<double>>& h) {
    kv_dots(V.as<double2>(), nv, len, w, part.as<double2>(), L.st);
    MNP_CHECK_LAUNCH();
    hpart.resize((size_t)nv * KV_BLOCKS);
    MNP_CUDA(cudaMemcpyAsync(hpart.data(), part.ptr, sizeof(double2) * hpart.size(), cudaMemcpyDeviceToHost, L.st));
    MNP_CUDA(cudaStreamSynchronize(L.st));
    h.assign(nv, 0.0);
    for (int i = 0; i < nv; ++i) {
      double2 s = make_double2(0.0, 0.0);
      for (int b = 0; b < KV_BLOCKS; ++b) s = cadd(s, hpart[(size_t)i * KV_BLOCKS + b]);
      h[i] = std::complex<double>(s.x, s.y);
    }
    return MNPBEM_OK;
  }
  // w -= sum_i h_i V_i
  mnpbem_status update(int nv, const std::vector<std::complex<double>>& h, double2* w) {
    MNP_CUDA(cudaMemcpyAsync(hdev.ptr, h.data(), sizeof(double2) * nv, cudaMemcpyHostToDevice, L.st));
    kv_update(V.as<double2>(), nv, len, hdev.as<double2>(), w, L.st);
    MNP_CHECK_LAUNCH();
    MNP_CUDA(cudaStreamSynchronize(L.st));   // h lives in pageable host memory
    return MNPBEM_OK;
  }

  mnpbem_status run(int& flag, int& steps, double& relres) {
    using cd = std::complex<double>;
    // restart 0: cycles of up to maxit steps, maxit steps in all; else cycles
    // of restart steps, at most maxit cycles.  A cycle whose estimated
    // residual reached the tolerance while the true one did not (an inexact
    // complex64 preconditioner) is followed by another within the budget.
    const int inner = o.restart > 0 ? o.restart : o.maxit;
    const int64_t budget = o.restart > 0 ? (int64_t)o.maxit * o.restart : o.maxit;
    if (inner > 4096) {
      set_error("GMRES: at most 4096 steps per cycle (set restart)");
      return MNPBEM_ERR_INVALID_ARG;
    }
    MNP_TRY(V.ensure(sizeof(double2) * (size_t)(inner + 1) * len));
    MNP_TRY(part.ensure(sizeof(double2) * (size_t)(inner + 1) * KV_BLOCKS));
    MNP_TRY(hdev.ensure(sizeof(double2) * (size_t)(inner + 1)));
    MNP_TRY(zero.ensure(sizeof(double2) * len));
    MNP_TRY(rvec.ensure(sizeof(double2) * len));
    MNP_CUDA(cudaMemsetAsync(zero.ptr, 0, sizeof(double2) * len, L.st));
    Vec64 v = vec64(G, L, P);
    double2* x = v.x1;                     // x2 follows x1
    double2* r = rvec.as<double2>();
    double2* Vb = V.as<double2>();
    MNP_CUDA(cudaMemsetAsync(x, 0, sizeof(double2) * len, L.st));
    MNP_TRY(precond(v.phi, v.a, v.alpha, v.De, r));
    double nmb = 0.0;
    MNP_TRY(norm(r, nmb));
    flag = 1;
    steps = 0;
    relres = 0.0;
    if (!(nmb > 0)) {
      flag = nmb == 0 ? 0 : 1;
      if (nmb != 0) { set_error("GMRES: non-finite right-hand side"); return MNPBEM_ERR_NOT_CONVERGED; }
      return MNPBEM_OK;
    }
    const double tolb = o.tol * nmb;
    std::vector<cd> h, h2, g(inner + 1), sn(inner), y;
    std::vector<double> cs(inner);
    std::vector<std::vector<cd>> Hc(inner, std::vector<cd>(inner + 1));
    double rn = nmb;
    while (steps < budget) {
      const double beta = rn;
      if (beta <= tolb) { flag = 0; break; }
      const int inner_c = (int)std::min<int64_t>(inner, budget - steps);
      kv_scale(r, len, 1.0 / beta, Vb, L.st);
      std::fill(g.begin(), g.end(), cd(0.0));
      g[0] = beta;
      int m = 0;
      for (int j = 0; j < inner_c; ++j) {
        double2* w = Vb + (size_t)(j + 1) * len;
        MNP_TRY(op(Vb + (size_t)j * len, w));
        ++steps;
        MNP_TRY(dots(j + 1, w, h));
        MNP_TRY(update(j + 1, h, w));
        MNP_TRY(dots(j + 1, w, h2));
        MNP_TRY(update(j + 1, h2, w));
        for (int i = 0; i <= j; ++i) h[i] += h2[i];
        double hn = 0.0;
        MNP_TRY(norm(w, hn));
        if (!(hn == hn)) { set_error("GMRES: non-finite Krylov vector"); return MNPBEM_ERR_NOT_CONVERGED; }
        std::vector<cd>& col = Hc[j];
        std::fill(col.begin(), col.end(), cd(0.0));
        for (int i = 0; i <= j; ++i) col[i] = h[i];
        col[j + 1] = hn;
        for (int i = 0; i < j; ++i) {
          const cd a0 = col[i], a1 = col[i + 1];
          col[i] = cs[i] * a0 + sn[i] * a1;
          col[i + 1] = -std::conj(sn[i]) * a0 + cs[i] * a1;
        }
        const cd a = col[j], bb = col[j + 1];
        const double t = std::hypot(std::abs(a), std::abs(bb));
        if (std::abs(a) == 0.0) {
          cs[j] = 0.0;
          sn[j] = 1.0;
        } else {
          cs[j] = std::abs(a) / t;
          sn[j] = (a / std::abs(a)) * std::conj(bb) / t;
        }
        col[j] = cs[j] * a + sn[j] * bb;
        col[j + 1] = 0.0;
        g[j + 1] = -std::conj(sn[j]) * g[j];
        g[j] = cs[j] * g[j];
        m = j + 1;
        if (hn == 0.0 || std::abs(g[j + 1]) <= tolb) break;
        kv_scale(w, len, 1.0 / hn, w, L.st);
      }
      // x += V y with H y = g (upper triangular)
      y.assign(m, 0.0);
      for (int i = m - 1; i >= 0; --i) {
        cd s = g[i];
        for (int k = i + 1; k < m; ++k) s -= Hc[k][i] * y[k];
        y[i] = s / Hc[i][i];
      }
      for (int i = 0; i < m; ++i) y[i] = -y[i];
      MNP_TRY(update(m, y, x));
      // true preconditioned residual
      MNP_TRY(residual(x, v.phi, v.a, v.alpha, v.De));
      MNP_TRY(precond(v.rphi, v.ra, v.ral, v.rDe, r));
      MNP_TRY(norm(r, rn));
      if (rn <= tolb) { flag = 0; break; }
    }
    if (rn <= tolb) flag = 0;
    relres = rn / nmb;
    return MNPBEM_OK;
  }

  // ---- cgs / bicgstab (@bemiter/solve.m): preconditioner on the search
  // directions, unpreconditioned residuals in the equation layout
  // (phi, a, alpha, De; 8 n P values), unknowns in [x1 | x2]
  DevBuf kw;
  std::complex<double> dot(const double2* u, const double2* w) {
    kv_dots(u, 1, len, w, part.as<double2>(), L.st);
    hpart.resize(KV_BLOCKS);
    cudaMemcpyAsync(hpart.data(), part.ptr, sizeof(double2) * KV_BLOCKS, cudaMemcpyDeviceToHost, L.st);
    cudaStreamSynchronize(L.st);
    double2 s = make_double2(0.0, 0.0);
    for (int b = 0; b < KV_BLOCKS; ++b) s = cadd(s, hpart[b]);
    return std::complex<double>(s.x, s.y);
  }
  static double2 c2(std::complex<double> z) { return make_double2(z.real(), z.imag()); }
  void comb(double2* out, std::initializer_list<std::pair<std::complex<double>, const double2*>> terms) {
    KvTerms t;
    for (const auto& pr : terms) {
      t.c[t.n] = c2(pr.first);
      t.v[t.n] = pr.second;
      ++t.n;
    }
    kv_lincomb(t, len, out, L.st);
  }
  // bdst = A x (equation layout)
  mnpbem_status aop(const double2* x, double2* bdst) {
    const double2* z = zero.as<double2>();
    MNP_TRY(residual(x, z, z + n * P, z + 4 * n * P, z + 7 * n * P));
    Vec64 v = vec64(G, L, P);
    kv_scale(v.rphi, len, -1.0, bdst, L.st);
    MNP_CHECK_LAUNCH();
    return MNPBEM_OK;
  }
  // xdst = M b
  mnpbem_status mop(const double2* b, double2* xdst) {
    return precond(b, b + n * P, b + 4 * n * P, b + 7 * n * P, xdst);
  }
  mnpbem_status run_cgs_bicg(int& flag, int& steps, double& relres) {
    using cd = std::complex<double>;
    MNP_TRY(part.ensure(sizeof(double2) * KV_BLOCKS));
    MNP_TRY(zero.ensure(sizeof(double2) * len));
    MNP_TRY(kw.ensure(sizeof(double2) * 10 * len));
    MNP_CUDA(cudaMemsetAsync(zero.ptr, 0, sizeof(double2) * len, L.st));
    Vec64 v = vec64(G, L, P);
    double2* x = v.x1;
    double2* W = kw.as<double2>();
    double2 *r = W, *rt = W + len, *p = W + 2 * len, *u = W + 3 * len, *q = W + 4 * len, *vv = W + 5 * len;
    double2 *ph = W + 6 * len, *uh = W + 7 * len, *t = W + 8 * len, *tmp = W + 9 * len;
    const double2* b = v.phi;   // phi, a, alpha, De are contiguous
    MNP_CUDA(cudaMemsetAsync(x, 0, sizeof(double2) * len, L.st));
    double nb = 0.0;
    MNP_TRY(norm(b, nb));
    flag = 1;
    steps = 0;
    relres = 0.0;
    if (!(nb > 0)) {
      if (nb != 0) { set_error("iterative solver: non-finite right-hand side"); return MNPBEM_ERR_NOT_CONVERGED; }
      flag = 0;
      return MNPBEM_OK;
    }
    const double tolb = o.tol * nb;
    comb(r, {{1.0, b}});
    comb(rt, {{1.0, b}});
    cd rho = 1.0, rho1, alpha = 1.0, omega = 1.0;
    double rn = nb;
    for (int ii = 1; ii <= o.maxit; ++ii) {
      rho1 = rho;
      rho = dot(rt, r);
      if (rho == 0.0 || !(std::abs(rho) == std::abs(rho))) break;
      steps = ii;
      if (o.solver == 1) {                                   // cgs
        if (ii == 1) {
          comb(u, {{1.0, r}});
          comb(p, {{1.0, u}});
        } else {
          const cd beta = rho / rho1;
          comb(u, {{1.0, r}, {beta, q}});
          comb(p, {{1.0, u}, {beta, q}, {beta * beta, p}});
        }
        MNP_TRY(mop(p, ph));
        MNP_TRY(aop(ph, vv));
        const cd rtv = dot(rt, vv);
        if (rtv == 0.0) break;
        alpha = rho / rtv;
        comb(q, {{1.0, u}, {-alpha, vv}});
        comb(tmp, {{1.0, u}, {1.0, q}});
        MNP_TRY(mop(tmp, uh));
        comb(x, {{1.0, x}, {alpha, uh}});
        MNP_TRY(aop(uh, t));
        comb(r, {{1.0, r}, {-alpha, t}});
        MNP_TRY(norm(r, rn));
        if (rn <= tolb) { flag = 0; break; }
      } else {                                               // bicgstab
        if (ii == 1) {
          comb(p, {{1.0, r}});
        } else {
          const cd beta = (rho / rho1) * (alpha / omega);
          comb(p, {{1.0, r}, {beta, p}, {-beta * omega, vv}});
        }
        MNP_TRY(mop(p, ph));
        MNP_TRY(aop(ph, vv));
        const cd rtv = dot(rt, vv);
        if (rtv == 0.0) break;
        alpha = rho / rtv;
        comb(q, {{1.0, r}, {-alpha, vv}});                  // s
        double sn = 0.0;
        MNP_TRY(norm(q, sn));
        if (sn <= tolb) {
          comb(x, {{1.0, x}, {alpha, ph}});
          flag = 0;
          break;
        }
        MNP_TRY(mop(q, uh));                                 // sh
        MNP_TRY(aop(uh, t));
        const cd tt = dot(t, t);
        if (tt == 0.0) break;
        omega = dot(t, q) / tt;
        comb(x, {{1.0, x}, {alpha, ph}, {omega, uh}});
        comb(r, {{1.0, q}, {-omega, t}});
        MNP_TRY(norm(r, rn));
        if (rn <= tolb) { flag = 0; break; }
      }
    }
    // true residual
    MNP_TRY(aop(x, tmp));
    comb(tmp, {{1.0, b}, {-1.0, tmp}});
    MNP_TRY(norm(tmp, rn));
    relres = rn / nb;
    return MNPBEM_OK;
  }
};

// the cluster tree and options an 'hmat' preconditioner was built with
uint64_t tree_signature(const mnpbem_cluster_tree* t, const IterOpts& o) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ull; };
  auto mix_arr = [&](const int32_t* a, int64_t cnt) {
    for (int64_t i = 0; a && i < cnt; ++i) mix((uint32_t)a[i]);
  };
  if (!t) return 0;
  mix((uint32_t)t->ncluster);
  mix_arr(t->son, 2 * (int64_t)t->ncluster);
  mix_arr(t->cind, 2 * (int64_t)t->ncluster);
  mix_arr(t->full, 2 * (int64_t)t->nfull);
  mix_arr(t->low, 2 * (int64_t)t->nlow);
  uint64_t ht;
  memcpy(&ht, &o.htol_pc, sizeof(ht));
  mix(ht);
  mix((uint32_t)o.kmax_pc);
  mix((uint32_t)o.kmax);
  return h;
}

// one wavelength on lane 0: excitation, H-matrices, optional preconditioner
mnpbem_status iter_prepare(mnpbem_geom* G, Job& j, const double2* ext_pot, HmatHost& H, const IterOpts& o,
                           const mnpbem_cluster_tree* tree) {
  Lane& L = *G->lanes[0];
  MNP_TRY(upload_lp(G, L, j.s, 0));
  L.w = 0;
  MNP_TRY(hmat_setup(G, tree, o.kmax, o.htol, H, L.st));
  const bool refresh_due = o.refresh > 0 && L.pc_last_steps > o.refresh;
  const bool keep = o.precond == 1 && o.reuse && L.pc_valid && L.pc_precision == j.c.precision &&
                    L.pc_mat0 == L.mat[0].ptr && !refresh_due;
  const uint64_t tsig = tree_signature(tree, o);
  const bool keep_h = o.precond == 2 && o.reuse && L.hpc && L.hpc_sig == tsig && !refresh_due;
  if (o.precond == 1 && !keep) {
    MNP_TRY(run_stage(G, L, j.c, 0, true));   // per-face eps + dense matrices
    MNP_TRY(run_stage(G, L, j.c, 1, true));   // dense inverses of bemret (initmat.m)
    MNP_TRY(L.pc_face.ensure(L.facebuf.bytes));
    MNP_TRY(L.pc_lp.ensure(sizeof(LamParams)));
    MNP_CUDA(cudaMemcpyAsync(L.pc_face.ptr, L.facebuf.ptr, L.facebuf.bytes, cudaMemcpyDeviceToDevice, L.st));
    MNP_CUDA(cudaMemcpyAsync(L.pc_lp.ptr, L.lp_dev.ptr, sizeof(LamParams), cudaMemcpyDeviceToDevice, L.st));
    L.pc_valid = true;
    L.pc_precision = j.c.precision;
    L.pc_enei = j.s.enei[0];
    L.pc_mat0 = L.mat[0].ptr;
  } else {
    face_eps(G, L);
    MNP_CHECK_LAUNCH();
    if (o.precond != 1) {   // the dense preconditioner's per-face data (unused)
      MNP_TRY(L.pc_face.ensure(L.facebuf.bytes));
      MNP_TRY(L.pc_lp.ensure(sizeof(LamParams)));
    }
  }
  const int P = j.c.P;
  if (o.precond == 2 && !keep_h) {
    // initprecond.m ('hmat'): H-matrix LU of G1, G2 and Sigma, Sigma1 and
    // Deltai as H-matrices, truncated with htol and min(op.kmax)
    std::shared_ptr<hl::Tree> T;
    MNP_TRY(hl::tree_from_abi(tree, T));
    std::shared_ptr<hl::Ctx> hc;
    MNP_TRY(hl::ctx_make(G->device, T, o.htol_pc, o.kmax_pc, hc));
    hl::HM m4[4];
    L.hpc.reset();
    MNP_TRY(hmat_fill(G, L, H, 4 * P, hc.get(), m4));
    auto hp = std::make_shared<hl::HPrecond>();
    const FaceData fd = face_data(G, L);
    MNP_CUDA(cudaStreamSynchronize(L.st));   // per-face eps of this wavelength
    MNP_TRY(hl::precond_build(hc, m4[0], m4[1], m4[2], m4[3], 2.0 * M_PI / j.s.enei[0], fd.eps1, fd.eps2,
                              G->g.nvec, *hp));
    L.hpc = hp;
    L.hpc_sig = tsig;
    L.pc_enei = j.s.enei[0];
  } else {
    MNP_TRY(hmat_fill(G, L, H, 4 * P));
  }
  Vec64 v = vec64(G, L, P);
  const FaceData fd = face_data(G, L);
  const LamParams* lp = L.lp_dev.as<LamParams>();
  if (ext_pot) {
    launch_excitation_ext(fd, P, ext_pot, lp, v.phi, v.a, v.alpha, v.De, L.st);
  } else {
    const double* pol = G->exbuf.as<double>();
    launch_excitation(fd, P, pol, pol + 3 * P, lp, v.phi, v.a, v.alpha, v.De, L.st);
  }
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

// ranks and the stored entries of the four H-matrices against 4 n^2
void hmat_stats(const HmatHost& H, const std::vector<int>& ranks, int64_t n, mnpbem_iter_info* info) {
  int rmax = 0;
  double rs = 0.0, stored = 4.0 * (double)H.la.nvals;
  for (int q = 0; q < 4; ++q)
    for (int b = 0; b < H.d.nlow; ++b) {
      const int r = ranks[(size_t)q * H.d.nlow + b];
      rmax = std::max(rmax, r);
      rs += r;
      stored += (double)r * (H.lblk[b].y + H.lblk[b].w);
    }
  info->rank_max = rmax;
  info->rank_mean = ranks.empty() ? 0.0 : rs / ranks.size();
  info->compression = stored / (4.0 * (double)n * n);
}

}  // namespace

mnpbem_status mnpbem_solve_iter(mnpbem_geom* G, const mnpbem_cluster_tree* tree, const mnpbem_iter_options* op,
                                const mnpbem_planewave* exc, const mnpbem_potentials* pot, double enei,
                                const double* eps_media, int32_t nmed, int32_t precision, mnpbem_solution* out,
                                mnpbem_iter_info* info) {
  MNP_TRY(check_geom(G));
  IterOpts o;
  MNP_TRY(iter_opts(op, o));
  if (!out || !(enei > 0) || (!exc && !pot) || (pot && (pot->npol < 1 || pot->npol > 4))) {
    set_error("mnpbem_solve_iter: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  const int P = pot ? pot->npol : exc->npol;
  std::vector<double> zero(3 * P, 0.0);
  mnpbem_planewave pw{P, zero.data(), zero.data(), 1, 0, nullptr, nullptr};
  mnpbem_solution so = *out;
  if (pot) so.ext = so.sca = nullptr;
  const mnpbem_planewave* ex = pot ? &pw : exc;
  MNP_TRY(validate_job(G, ex, 1, &enei, eps_media, nmed, precision, &so));
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  const int64_t n = G->g.n;
  DevBuf dpot;
  if (pot) {
    const double* src[8] = {pot->phi1, pot->phi1p, pot->phi2, pot->phi2p, pot->a1, pot->a1p, pot->a2, pot->a2p};
    MNP_TRY(dpot.ensure(sizeof(double2) * 16 * n * P));
    double2* D = dpot.as<double2>();
    for (int q = 0; q < 8; ++q) {
      const int64_t cnt = (q < 4 ? 1 : 3) * n * P;
      double2* dst = D + (q < 4 ? q * n * P : 4 * n * P + (q - 4) * 3 * n * P);
      if (src[q]) MNP_CUDA(cudaMemcpy(dst, src[q], sizeof(double2) * cnt, cudaMemcpyHostToDevice));
      else MNP_CUDA(cudaMemset(dst, 0, sizeof(double2) * cnt));
    }
  }
  std::vector<Job> jobs(1);
  Job& j = jobs[0];
  j.G = G;
  MNP_TRY(job_setup(j, ex, 1, &enei, eps_media, nmed, precision, nullptr, &so));
  j.c.spectra = !pot;
  Lane& L = *G->lanes[0];
  HmatHost H;
  MNP_TRY(iter_prepare(G, j, pot ? dpot.as<double2>() : nullptr, H, o, tree));
  Gmres gm(G, L, j.c, H, o);
  int flag = 1, steps = 0;
  double relres = 0.0;
  if (o.solver == 0) MNP_TRY(gm.run(flag, steps, relres));
  else MNP_TRY(gm.run_cgs_bicg(flag, steps, relres));
  L.pc_last_steps = steps;
  // true relative residual ||b - A x|| / ||b|| with the H-matrix operator
  Vec64 v = vec64(G, L, P);
  MNP_CUDA(cudaMemsetAsync(L.norms.ptr, 0, sizeof(double) * 4, L.st));
  MNP_TRY(gm.residual(v.x1, v.phi, v.a, v.alpha, v.De));
  double hn[4];
  MNP_CUDA(cudaMemcpyAsync(hn, L.norms.ptr, sizeof(double) * 4, cudaMemcpyDeviceToHost, L.st));
  if (j.c.spectra) MNP_TRY(run_stage(G, L, j.c, 4, true));
  MNP_CUDA(cudaStreamSynchronize(L.st));
  L.iters = steps;
  L.res = hn[1] > 0 ? sqrt(hn[0] / hn[1]) : 0.0;
  MNP_TRY(write_outputs(G, L, j.c, j.s, 0));
  G->prof.flush();
  if (info) {
    info->flag = flag;
    info->iter = steps;
    info->relres = relres;
    info->true_relres = L.res;
    info->precond_enei = o.precond ? L.pc_enei : 0.0;
    hmat_stats(H, H.ranks, n, info);
  }
  return MNPBEM_OK;
}

mnpbem_status mnpbem_hmat_full(mnpbem_geom* G, const mnpbem_cluster_tree* tree, const mnpbem_iter_options* op,
                               double enei, const double* eps_media, int32_t nmed, int32_t which, double* out,
                               int32_t* ranks) {
  MNP_TRY(check_geom(G));
  IterOpts o;
  MNP_TRY(iter_opts(op, o));
  if (!out || which < 0 || which > 3 || !(enei > 0)) {
    set_error("mnpbem_hmat_full: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  const double pol[3] = {1, 0, 0}, dir[3] = {0, 0, 1};
  mnpbem_planewave pw{1, pol, dir, 1, 0, nullptr, nullptr};
  mnpbem_solution so{};
  MNP_TRY(validate_job(G, &pw, 1, &enei, eps_media, nmed, MNPBEM_FP64, &so));
  MNP_CUDA(cudaSetDevice(G->device));
  ProfBind pb_(&G->prof);
  std::vector<Job> jobs(1);
  Job& j = jobs[0];
  j.G = G;
  MNP_TRY(job_setup(j, &pw, 1, &enei, eps_media, nmed, MNPBEM_FP64, nullptr, &so));
  Lane& L = *G->lanes[0];
  MNP_TRY(upload_lp(G, L, j.s, 0));
  HmatHost H;
  MNP_TRY(hmat_setup(G, tree, o.kmax, o.htol, H, L.st));
  MNP_TRY(hmat_fill(G, L, H, 4));
  const int64_t n = G->g.n;
  DevBuf full;
  MNP_TRY(full.ensure(sizeof(double2) * n * n));
  MNP_TRY(hmat_full(H.d, which, full.as<double2>(), L.st));
  MNP_CUDA(cudaMemcpyAsync(out, full.ptr, sizeof(double2) * n * n, cudaMemcpyDeviceToHost, L.st));
  if (ranks && H.d.nlow > 0)
    MNP_CUDA(cudaMemcpyAsync(ranks, H.d.rank, sizeof(int) * 4 * H.d.nlow, cudaMemcpyDeviceToHost, L.st));
  MNP_CUDA(cudaStreamSynchronize(L.st));
  return MNPBEM_OK;
}
