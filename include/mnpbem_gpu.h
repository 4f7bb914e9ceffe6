/*
 * mnpbem_gpu.h — C ABI of the GB300-native retarded BEM path of MNPBEM.
 *
 * The library replaces, behind MNPBEM's own calling surface, the MATLAB code of
 *   bem = bemsolver(p, op)            (Base/bemsolver.m:18-27 -> BEM/@bemret/private/init.m:16-31
 *                                      -> Greenfun/@compgreenret/private/init.m:5-31)
 *   sig = bem \ exc(p, enei)          (BEM/@bemret/mldivide.m:12-49, private/initmat.m:5-74,
 *                                      Simulation/retarded/@planewaveret/potential.m:13-57)
 *   exc.ext(sig), exc.sca(sig)        (Simulation/retarded/@planewaveret/extinction.m:12-16,
 *                                      scattering.m:13-19, @spectrumret/farfield.m:15-74)
 * A MATLAB MEX gateway (the pattern of mex/hmatgreenret.cpp:21-61) or a Python
 * ctypes harness calls these symbols.  Conventions:
 *   - every function returns an mnpbem_status; nothing calls exit();
 *     mnpbem_last_error() gives a message for the last failure on this thread;
 *   - arrays are C order (row-major); complex numbers are interleaved
 *     (re, im) doubles; face and vertex indices are 0-based; the 4th face
 *     column is -1 for triangles (MNPBEM uses NaN there);
 *   - the caller owns host buffers, the library owns device buffers and the
 *     handle; one CUDA stream per handle; a handle is not shared across threads.
 */
#ifndef MNPBEM_GPU_H
#define MNPBEM_GPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define MNPBEM_API __declspec(dllexport)
#else
#define MNPBEM_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mnpbem_status {
  MNPBEM_OK = 0,
  MNPBEM_ERR_INVALID_ARG = 1,
  MNPBEM_ERR_CUDA = 2,
  MNPBEM_ERR_OUT_OF_MEMORY = 3,
  MNPBEM_ERR_SINGULAR = 4,      /* pivot guard of the block inversion tripped      */
  MNPBEM_ERR_NOT_CONVERGED = 5, /* FP64 refinement did not reach its tolerance     */
  MNPBEM_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up              */
  MNPBEM_ERR_UNSUPPORTED = 7
} mnpbem_status;

typedef enum mnpbem_precision {
  MNPBEM_FP64 = 0,  /* all assembly / inversion / products in FP64 (plain FP64 path)  */
  MNPBEM_MIXED = 1, /* complex64 TF32 tensor-core inversion + FP64 refinement         */
  MNPBEM_FP32 = 2   /* assembly output only: complex64 matrices                        */
} mnpbem_precision;

/* Quadrature rules carried by a particle (p.quad, Misc/integration/@quadface):
 * the triangle rule (rule 18: 28 points, weights summing to 1) and the polar
 * rules around the centroid for triangles (x3, y3, w3) and quadrilaterals
 * (x4, y4, w4) (@quadface/private/init.m:25-80). */
typedef struct mnpbem_quad {
  int32_t n_tri;
  const double *x, *y, *w;
  int32_t n_pol3;
  const double *x3, *y3, *w3;
  int32_t n_pol4;
  const double *x4, *y4, *w4;
} mnpbem_quad;

/* Options of the Green function (Misc/bemoptions.m:16-25). */
typedef struct mnpbem_options {
  double rel_cutoff; /* RelCutoff (3)                         */
  double abs_cutoff; /* AbsCutoff (0)                         */
  int32_t order;     /* order of the exp(ikr) expansion (5)   */
  int32_t device;    /* CUDA device ordinal                   */
} mnpbem_options;

typedef struct mnpbem_geom mnpbem_geom;

/* comparticle(eps, {p1..pnp}, inout, closed) + compgreenret(p, p, op):
 * flat-face geometry (Particles/@particle/private/norm_flat.m:8-62), the
 * refinement pattern (Greenfun/+green/refinematrix.m:28-68), the Taylor
 * coefficients of the near elements (Greenfun/@greenret/private/init.m:42-177)
 * and the closed-surface sum rule (Greenfun/@compgreenret/private/initclosed.m:19-89).
 *   verts  [nverts][3];  faces [nfaces][4] (concatenated particles)
 *   part_nfaces [nparts]: faces of each particle, in order
 *   inout [nparts][2]: 1-based media (inside, outside)
 *   closed [nparts]: 1 when particle i is a closed surface by itself           */
MNPBEM_API mnpbem_status mnpbem_geom_create(const double* verts, int64_t nverts,
                                 const int64_t* faces, int64_t nfaces,
                                 int32_t nparts, const int64_t* part_nfaces,
                                 const int32_t* inout, const int32_t* closed,
                                 const mnpbem_quad* quad, const mnpbem_options* opts,
                                 mnpbem_geom** out);
/* Same for curved boundary elements (particle with interp = 'curv'): 6-node
 * triangles and 9-node quadrilaterals (Particles/@particle/private/norm_curv.m:8-62,
 * quad_curv.m:13-59, quadpol_curv.m:15-88, totriangles_curv.m:14-31).
 *   verts2 [nverts2][3]: corners and the extra nodes (p.verts2)
 *   faces2 [nfaces][9] (p.faces2, 0-based, -1 for NaN): corners 0-3 (3 = -1 for
 *   triangles), midpoints of edges 12, 23, 34 (31 for triangles), 41 in 4-7,
 *   quadrilateral centre in 8.  Gradients (mnpbem_cross_section_gradient)
 *   return MNPBEM_ERR_UNSUPPORTED on curved handles.                           */
MNPBEM_API mnpbem_status mnpbem_geom_create_curved(const double* verts2, int64_t nverts2,
                                        const int64_t* faces2, int64_t nfaces,
                                        int32_t nparts, const int64_t* part_nfaces,
                                        const int32_t* inout, const int32_t* closed,
                                        const mnpbem_quad* quad, const mnpbem_options* opts,
                                        mnpbem_geom** out);
MNPBEM_API mnpbem_status mnpbem_geom_destroy(mnpbem_geom* g);

/* Sizes: number of faces and of refined (near + self) elements. */
MNPBEM_API mnpbem_status mnpbem_geom_size(const mnpbem_geom* g, int64_t* nfaces, int64_t* nref);

/* Copy geometry and refinement data to host (any pointer may be NULL).
 *   pos, nvec, tvec1, tvec2 [n][3]; area [n];
 *   ref_row, ref_col [nref] in MATLAB's find() order (column-major);
 *   ref_g [nref][order+1]; ref_f [nref][3][order+1]   (greenret obj.g, obj.f)   */
MNPBEM_API mnpbem_status mnpbem_geom_export(const mnpbem_geom* g, double* pos, double* nvec,
                                 double* tvec1, double* tvec2, double* area,
                                 int64_t* ref_row, int64_t* ref_col, double* ref_g,
                                 double* ref_f);

/* compgreenret matrices of bemret (BEM/@bemret/private/initmat.m:27-31):
 *   G1 = G{1,1} - G{2,1}, H1 = H1{1,1} - H1{2,1}, G2 = G{2,2} - G{1,2}, H2 = H2{2,2} - H2{1,2}
 * for wavenumbers k_media [nmed] (complex, interleaved) of the media.
 * precision MNPBEM_FP64 -> complex128 [n][n] outputs, MNPBEM_FP32 -> complex64,
 * MNPBEM_MIXED -> complex128 hi + lo of the mixed-precision pass (far field in
 * double-single FP32 arithmetic, refined entries in FP64).
 * Outputs are host pointers (NULL to skip).                                     */
MNPBEM_API mnpbem_status mnpbem_assemble(mnpbem_geom* g, const double* k_media, int32_t nmed,
                              int32_t precision, void* G1, void* H1, void* G2, void* H2);

/* Plane-wave excitation (planewaveret(pol, dir, op)) plus the unit sphere at
 * infinity used for the scattering cross section (op.pinfty, default
 * trisphere(256, 2); Simulation/retarded/@planewaveret/init.m:26-30). */
typedef struct mnpbem_planewave {
  int32_t npol;
  const double* pol; /* [npol][3] */
  const double* dir; /* [npol][3] */
  int32_t medium;    /* 1-based excitation medium (default 1) */
  int32_t ninf;
  const double* inf_nvec; /* [ninf][3] outer normals of the sphere at infinity */
  const double* inf_area; /* [ninf] */
} mnpbem_planewave;

/* Outputs of a wavelength sweep (NULL to skip any of them). */
typedef struct mnpbem_solution {
  double* ext;      /* [nenei][npol]  extinction cross section  */
  double* sca;      /* [nenei][npol]  scattering cross section  */
  double* sig1;     /* [nenei][n][npol]    complex  */
  double* sig2;     /* [nenei][n][npol]    complex  */
  double* h1;       /* [nenei][n][3][npol] complex  */
  double* h2;       /* [nenei][n][3][npol] complex  */
  int32_t* ir_iters;  /* [nenei] refinement iterations used (MIXED) */
  double* ir_resid;   /* [nenei] final relative FP64 residual of the BEM equations */
  int32_t outputs_on_device; /* 1: sig1/sig2/h1/h2/ext/sca are device pointers */
} mnpbem_solution;

/* Refinement control for MNPBEM_MIXED (ignored for FP64). */
typedef struct mnpbem_refine {
  int32_t max_iter; /* default 10 */
  double tol;       /* stop when ||dx|| <= tol * ||x|| (default 1e-10) */
} mnpbem_refine;

/* Wavelength sweep: for each enei[w] (nm) with dielectric functions
 * eps_media [nenei][nmed] (complex; eps of medium m at enei[w]):
 * excitation (planewaveret/potential.m), bemret initmat + mldivide, and
 * ext / sca.  precision: MNPBEM_FP64 or MNPBEM_MIXED.  refine may be NULL. */
MNPBEM_API mnpbem_status mnpbem_solve(mnpbem_geom* g, const mnpbem_planewave* exc, int32_t nenei,
                           const double* enei, const double* eps_media, int32_t nmed,
                           int32_t precision, const mnpbem_refine* refine,
                           mnpbem_solution* out);

/* One particle's sweep inside mnpbem_solve_batch (fields as in mnpbem_solve). */
typedef struct mnpbem_job {
  mnpbem_geom* g;
  const mnpbem_planewave* exc;
  int32_t nenei;
  const double* enei;       /* [nenei] nm */
  const double* eps_media;  /* [nenei][nmed] complex */
  int32_t nmed;
  mnpbem_solution* out;
} mnpbem_job;

/* Several independent sweeps (e.g. particles of uneven size, each its own
 * handle) solved together: every handle's lanes are branches of one CUDA
 * graph whose device-side queues hand out each handle's wavelengths and whose
 * refinement decisions are taken on the device ("sweep_graph" option), so the
 * small particles' wavelengths fill the GPU while the large ones run.
 * Same results as one mnpbem_solve per job.  The handles must be distinct and
 * on one device.  The reference has no batch call: its user code loops over
 * particles and wavelengths (Demo/planewave/ret/demospecret*.m).             */
MNPBEM_API mnpbem_status mnpbem_solve_batch(const mnpbem_job* jobs, int32_t njobs, int32_t precision,
                                            const mnpbem_refine* refine);

/* Gradient of the extinction cross section of polarisation ipol at one
 * wavelength by the adjoint method: a transposed solve through the transposed
 * inverses of the forward solve, then the derivatives of G, F (far pairs,
 * refined near pairs, self elements, closed-surface diagonal), of the
 * excitation and of the far field contracted with the adjoint and forward
 * surface charges, chained to the vertices through norm_flat.m.  No
 * counterpart in the reference (MNPBEM has no derivatives).  The refinement
 * pattern is held fixed.  Scope: one closed particle excited from its outside
 * medium.  precision MNPBEM_FP64: FP64 solves; MNPBEM_MIXED: complex64
 * (TF32) forward and transposed solves, each refined on the FP64-class
 * operator (double-single products of the hi / lo planes).
 *   ext: the cross section (may be NULL); verts_grad [nverts][3] (host):
 *   dext / dvertex; eps_grad [2] (host): dext / dRe(eps), dext / dIm(eps) of
 *   the medium inside the particle.                                          */
MNPBEM_API mnpbem_status mnpbem_ext_gradient(mnpbem_geom* g, const mnpbem_planewave* exc, int32_t ipol,
                                             double enei, const double* eps_media, int32_t nmed,
                                             int32_t precision, double* ext, double* verts_grad,
                                             double* eps_grad);

/* Same for the extinction (which = 0) or the scattering cross section
 * (which = 1, scattering.m:14-31 over the sphere at infinity of exc, whose
 * ninf must be > 0); value receives the cross section.  No counterpart in
 * the reference.                                                             */
MNPBEM_API mnpbem_status mnpbem_cross_section_gradient(mnpbem_geom* g, const mnpbem_planewave* exc,
                                                       int32_t ipol, int32_t which, double enei,
                                                       const double* eps_media, int32_t nmed,
                                                       int32_t precision, double* value,
                                                       double* verts_grad, double* eps_grad);

/* The matrices bemret stores per wavelength (initmat.m:27-72), copied to host
 * as complex128 [n][n] (NULL to skip): G1i, G2i, Sigma1, Deltai, Sigmai.       */
MNPBEM_API mnpbem_status mnpbem_bem_matrices(mnpbem_geom* g, double enei, const double* eps_media,
                                  int32_t nmed, int32_t precision, double* G1i,
                                  double* G2i, double* Sigma1, double* Deltai,
                                  double* Sigmai);

/* Per-phase accounting of the library's kernels on a handle (the tracing that
 * the reference does with named timer maps, mex/hlib/hoptions.h:65-72, and
 * BEM/@bemiter/tocout.m).  Phases: 0 assembly, 1 O(n^3) GEMMs, 2 thin/panel GEMMs,
 * 3 pivot-block inversions, 4 element-wise kernels, 5 spectra, 6 geometry set-up,
 * 7 H-matrix construction (full blocks + ACA), 8 H-matrix products.
 * Launch counts are always kept; with profiling enabled each launch is also
 * bracketed by CUDA events on the handle's stream (durations in ms) and the
 * algorithmic FLOPs / bytes of the launches are accumulated.                */
MNPBEM_API mnpbem_status mnpbem_profile_enable(mnpbem_geom* g, int32_t on);
MNPBEM_API mnpbem_status mnpbem_profile_reset(mnpbem_geom* g);
MNPBEM_API mnpbem_status mnpbem_profile_read(mnpbem_geom* g, int32_t phase, double* ms,
                                             double* flops, double* bytes, int64_t* launches);

/* Complex64 GEMM C = alpha A B + beta C (row-major, interleaved complex,
 * leading dimensions in elements) on host buffers, or, when A, B and C are all
 * device pointers, on them directly and asynchronously on the default stream
 * (the caller synchronises; an expired wait shows at the next host-buffer
 * call): path 0 = CUDA-core kernel, path 1 =
 * tcgen05 tensor-core kernel (TF32 inputs, FP32 accumulation), path 2 = the
 * same on CTA pairs (cta_group::2, 256 x 256 tiles; M >= 256, else path 1)
 * with a TMA store / reduce-add epilogue, path 3 = CTA pairs with vector
 * stores / reductions from the load-store path, path 4 = single-CTA
 * tensor-core kernel on FP16 operands (kind::f16) scaled per row of A and per
 * column of B by powers of two, FP32 accumulation.
 * The building block of the factorisations and products of initmat.m (MATLAB
 * mtimes on complex matrices); beta must be real for paths 1 to 4.           */
MNPBEM_API mnpbem_status mnpbem_gemm_c64(int32_t device, int32_t path, int64_t M, int64_t N,
                                         int64_t K, const float* alpha, const float* A,
                                         int64_t lda, const float* B, int64_t ldb,
                                         const float* beta, float* C, int64_t ldc);

/* Extinction and scattering cross sections of given surface charges and
 * currents, like mnpbem_solve's ext/sca, for callers that cannot allocate GPU
 * memory (a MEX gateway inside a MATLAB session whose GPU memory belongs to
 * MATLAB, a plugin whose host application owns all device memory through its
 * own pool, a real-time loop that must not meet allocation failures).
 * It calls no cudaMalloc/cudaFree: every input and output is a caller-owned
 * DEVICE pointer and the scratch (far fields) is a fixed __device__ array in
 * the library, shared by all calls on a device and held until process exit.
 * No counterpart in the reference.  Limits: npol <= 4 and npol + ninf <= 2048
 * directions (larger sizes return MNPBEM_ERR_INVALID_ARG).  Each call looks up
 * the scratch address in the current context (valid after a device reset); the
 * first call on a device loads the module: make it before any stream capture.
 * Calls whose kernels overlap on the GPU race on the shared scratch.
 * Asynchronous on `stream` (cudaStream_t, NULL = default stream).
 *   pos [n][3], area [n]; exc_in / exc_out [n]: 1 where the inside / outside
 *   medium of a face is the excitation medium; sig1, sig2 [n][npol] and
 *   h1, h2 [n][3][npol] complex; pol, dir [npol][3]; inf_nvec [ninf][3],
 *   inf_area [ninf]; eps_exc, eps_1: complex dielectric function of the
 *   excitation medium and of medium 1 at enei (host, 2 doubles each);
 *   ext, sca [npol] (device outputs).                                          */
MNPBEM_API mnpbem_status mnpbem_cross_sections_noalloc(
    int32_t device, void* stream, int64_t n, int32_t npol, const double* pos, const double* area,
    const unsigned char* exc_in, const unsigned char* exc_out, const double* sig1, const double* h1,
    const double* sig2, const double* h2, const double* pol, const double* dir, int32_t ninf,
    const double* inf_nvec, const double* inf_area, double enei, const double* eps_exc,
    const double* eps_1, double* ext, double* sca);

/* Number of wavelengths a sweep keeps in flight at once (0 = automatic: 4,
 * fewer when device memory is short; 1 while profiling).  Each lane owns its
 * own stream and per-wavelength workspace (the five working matrices, the
 * refinement matrices and vectors), so device memory grows with the lane
 * count.  No counterpart in the reference, which solves one wavelength at a
 * time (Simulation/retarded/@spectrumret and the demo loops over enei).      */
MNPBEM_API mnpbem_status mnpbem_geom_set_lanes(mnpbem_geom* g, int32_t lanes);

/* Tuning options of a handle (the autotuner of mnpbem_gb300/autotune.py picks
 * them per problem size): "lanes" (0..16), "gj_block" (Gauss-Jordan step of
 * the tensor-core inversions: 256 or 512), "tc_stages" (TMA pipeline depth of
 * the tensor-core GEMM: 3 or 4), "tc_ctas" (CTAs of the persistent
 * tensor-core GEMM, 0 = one per SM; fewer leave SMs to the pivot-block
 * clusters of other lanes), "tc_pair" (only 0: the CTA-pair tensor-core GEMM
 * is not used inside sweeps; 1 / -1 return MNPBEM_ERR_UNSUPPORTED),
 * "lu_steps" (256-row LDU steps gathered into one trailing update: 1, 2 or
 * 4, i.e. updates of rank 256, 512 or 1024), "tc_f16" (tensor-core products
 * on FP16 operands scaled per row / column by powers of two, kind::f16, 1 =
 * default, or on TF32 operands, 0), "tf32_round" (round A operands to nearest
 * TF32: 0/1), "assembly_ds" (mixed-precision assembly in double-single FP32
 * arithmetic: 0/1), "sweep_graph" (1 = default: the wavelengths of a sweep
 * after each lane's first run as one CUDA graph with a device-side
 * wavelength queue and device-side refinement decisions; 0: the host
 * scheduler polls the lanes and queues every stage; results are identical).
 * Unknown keys or values return MNPBEM_ERR_INVALID_ARG.
 * No counterpart in the reference.                                          */
MNPBEM_API mnpbem_status mnpbem_geom_set_option(mnpbem_geom* g, const char* key, int32_t value);

/* Statistics of a handle: "block_cond_max" (largest condition proxy
 * max|A_kk| * max|inv(A_kk)| over the diagonal blocks of every factorisation
 * and inversion since the last "block_cond_reset"; a block above 1e6
 * (complex64) or 1e13 (FP64) fails the solve with MNPBEM_ERR_SINGULAR),
 * "block_cond_reset", "g1_blocks" (number of diagonal blocks G1 is factored
 * in), "sweep_graph_runs" (sweeps, or batch members, run as one graph),
 * "sweep_graph_error" (the CUDA error that turned one-graph sweeps off for
 * the handle, 0: none), "stage_graphs" (1: stages replay captured graphs, 0:
 * they run directly).  No counterpart in the reference (MATLAB's inv reports a near-singular
 * matrix as a warning).                                                      */
MNPBEM_API mnpbem_status mnpbem_geom_stat(mnpbem_geom* g, const char* key, double* value);

/* The handle's CUDA stream (cudaStream_t).  mnpbem_solve runs lane 0 on it
 * and makes it wait for the other lanes before returning, so work queued on
 * this stream after a call is ordered after all of the call's kernels.       */
MNPBEM_API mnpbem_status mnpbem_geom_stream(const mnpbem_geom* g, void** stream);

/* External potentials of one wavelength (MNPBEM's compstruct exc of any
 * excitation, e.g. dipoleret.potential): scalar potentials phi1, phi2 and
 * their surface derivatives phi1p, phi2p [n][npol] complex, vector potentials
 * a1, a2 and derivatives a1p, a2p [n][3][npol] complex (index 1: inside
 * of the faces, 2: outside); NULL = 0.                                      */
typedef struct mnpbem_potentials {
  int32_t npol;
  const double *phi1, *phi1p, *phi2, *phi2p;
  const double *a1, *a1p, *a2, *a2p;
} mnpbem_potentials;

/* sig = bem \ exc for external potentials at one wavelength: the excitation
 * variables of BEM/@bemret/private/excitation.m, then the solve of
 * mnpbem_solve (same precision and refinement).  out->sig1, sig2, h1, h2,
 * ir_iters, ir_resid are filled (ext, sca are not: no plane wave).          */
MNPBEM_API mnpbem_status mnpbem_solve_potentials(mnpbem_geom* g, const mnpbem_potentials* pot, double enei,
                                                 const double* eps_media, int32_t nmed, int32_t precision,
                                                 const mnpbem_refine* refine, mnpbem_solution* out);

/* Electric and magnetic fields at points off the particle boundary
 * (Greenfun/@compgreenret/field.m:17-38 on the Green function between a
 * compoint and the particle; Simulation/misc/@meshfield): for a point in
 * medium m, the faces whose inside (outside) medium is m contribute through
 * sig1 / h1 (sig2 / h2); points within RelCutoff element radii of a face use
 * the refined Taylor coefficients of the pair (refinematrix.m with the face's
 * radius, greenret/private/init.m:98-177).
 *   pts [npts][3]; pt_medium [npts] 1-based (compoint's inout)
 *   eps_media [nmed] complex; sig1, sig2 [n][npol], h1, h2 [n][3][npol]
 *   complex (mnpbem_solve's outputs for wavelength enei), host
 *   e, h [npts][3][npol] complex (host; either may be NULL)                  */
MNPBEM_API mnpbem_status mnpbem_fields(mnpbem_geom* g, int64_t npts, const double* pts,
                                       const int32_t* pt_medium, double enei, const double* eps_media,
                                       int32_t nmed, int32_t npol, const double* sig1, const double* sig2,
                                       const double* h1, const double* h2, double* e, double* h);

/* Far fields of the surface charges and currents in the unit directions
 * dirs [ndir][3] (replaces Simulation/retarded/@spectrumret/farfield.m:15-74):
 * with ph_j = exp(-i k dir . r_j) A_j over the faces whose inside (outside)
 * medium is `medium` (1-based; k its wavenumber), through sig1 / h1 (sig2 /
 * h2):  e = i k0 sum ph h - i k dir sum ph sig,  h = i k dir x sum ph h.
 *   eps_media [nmed] complex; sig1, sig2 [n][npol], h1, h2 [n][3][npol]
 *   complex, host; npol 1..4
 *   e, h [ndir][3][npol] complex (host; either may be NULL)                  */
MNPBEM_API mnpbem_status mnpbem_farfield(mnpbem_geom* g, double enei, const double* eps_media, int32_t nmed,
                                         int32_t medium, int64_t ndir, const double* dirs, int32_t npol,
                                         const double* sig1, const double* sig2, const double* h1,
                                         const double* h2, double* e, double* h);

/* Fields and potentials on the particle boundary itself, at the face
 * centroids on side inout (1 inside, 2 outside; MNPBEM's bemret default is
 * 2): replaces Greenfun/@compgreenret/field.m:14-38 and potential.m:16-48
 * as called by BEM/@bemret/field.m:8-11 and potential.m:14-15 ('cart'
 * derivative).  Faces whose inside (outside) medium is the observation
 * face's side-inout medium contribute through sig1 / h1 (sig2 / h2);
 *   E = i k0 (G h1 + G h2) - Hp sig1 - Hp sig2,   H = Hp x h1 + Hp x h2,
 *   phi = G sig1 + G sig2,   phip = H sig1 + H sig2,   a, ap likewise on h,
 * with Hp = H1p (H2p) = Gp +- 2 pi nvec [d == 0] and H = nvec . Hp (eval1.m
 * 140-149), refined pairs from the near-field Taylor coefficients.
 *   eps_media [nmed] complex; sig1, sig2 [n][npol], h1, h2 [n][3][npol]
 *   complex, host; npol 1..4
 *   e, h, a, ap [n][3][npol] and phi, phip [n][npol] complex (host; any may
 *   be NULL, not all)                                                       */
MNPBEM_API mnpbem_status mnpbem_surface_fields(mnpbem_geom* g, double enei, const double* eps_media, int32_t nmed,
                                               int32_t npol, int32_t inout, const double* sig1, const double* sig2,
                                               const double* h1, const double* h2, double* e, double* h,
                                               double* phi, double* phip, double* a, double* ap);

/* Cluster tree and block partition of an H-matrix (the arguments
 * Greenfun/hmatrices/@hmatrix/treemex.m hands to the H-matrix MEX functions,
 * mex/hmatgreenret.cpp:21-61, 0-based): clusters in the order of
 * @clustertree/private/bisection.m, positions in cluster order.
 *   son [ncluster][2]   sons, -1 for leaves
 *   cind [ncluster][2]  first and last cluster-order position (inclusive)
 *   ipart [ncluster]    particle of the cluster (0-based), -1 if several
 *   perm [n]            face at each cluster-order position (tree.ind(:,1) - 1)
 *   full [nfull][2]     (row, column) clusters of the full blocks (leaf pairs)
 *   low [nlow][2]       (row, column) clusters of the low-rank blocks        */
typedef struct mnpbem_cluster_tree {
  int32_t ncluster;
  const int32_t* son;
  const int32_t* cind;
  const int32_t* ipart;
  const int32_t* perm;
  int32_t nfull;
  const int32_t* full;
  int32_t nlow;
  const int32_t* low;
} mnpbem_cluster_tree;

/* Options of the iterative solver (BEM/@bemiter/options.m; defaults in
 * brackets).  solver: 0 GMRES [0], 1 CGS, 2 BiCGStab (the preconditioner
 * applied to the search directions; relres then is ||b - A x|| / ||b||);
 * precond: 0 none, 1 'full' [1] (the dense inverses of bemret in the
 * solve's precision: FP64, or complex64 on the tensor cores for MIXED),
 * 2 'hmat' (initprecond.m / mfun.m with H-matrices: LU of G1, G2 and Sigma,
 * Sigma1 and Deltai as H-matrices, FP64, low-rank blocks truncated by ACA
 * with htol_precond and kmax_precond, as compress.m sets them: max(op.htol),
 * min(op.kmax); no dense n x n matrix is formed);
 * restart 0 = no restarts (one cycle of up to maxit steps); at most 4096
 * steps per cycle.
 * reuse_precond 1 (not in the reference, which rebuilds the preconditioner
 * at every wavelength): keep the preconditioner ('full' or 'hmat') of an earlier
 * iterative solve on this handle (same precision) for this wavelength; it
 * changes the number of GMRES steps, not the solution (tol).  It is rebuilt
 * when the previous solve needed more than refresh_steps steps
 * (refresh_steps 0: never) and after any direct solve on the handle.       */
typedef struct mnpbem_iter_options {
  int32_t solver;
  double tol;        /* [1e-6] on ||M (b - A x)|| / ||M b||  */
  int32_t maxit;     /* [100] */
  int32_t restart;   /* [0]   */
  int32_t precond;   /* [1]   */
  double htol;       /* [1e-6] ACA tolerance */
  int32_t kmax;      /* [100] largest rank of a low-rank block (<= 512) */
  int32_t reuse_precond;  /* [0] */
  int32_t refresh_steps;  /* [0] */
  int32_t kmax_precond;   /* [4] (0: default) rank cap of the 'hmat' preconditioner */
  double htol_precond;    /* [htol] (0: htol) ACA tolerance of the 'hmat' preconditioner */
} mnpbem_iter_options;

/* Statistics of one iterative solve. */
typedef struct mnpbem_iter_info {
  int32_t flag;          /* 0 converged, 1 maxit reached */
  int32_t iter;          /* GMRES steps */
  double relres;         /* ||M (b - A x)|| / ||M b|| */
  double true_relres;    /* ||b - A x|| / ||b|| with the H-matrix operator */
  int32_t rank_max;      /* largest ACA rank over the four matrices */
  double rank_mean;
  double compression;    /* stored entries of the four H-matrices / 4 n^2 */
  double precond_enei;   /* wavelength the preconditioner was built at (0: none) */
} mnpbem_iter_info;

/* sig = bem \ exc with the iterative solver (BEM/@bemretiter/solve.m:11-36,
 * @bemiter/solve.m): H-matrices of G1, H1, G2, H2 (full blocks of the
 * complete Green function on leaf pairs, low-rank blocks by ACA of the far
 * field kernel, Greenfun/+aca/@compgreenret/eval.m), the operator of
 * afun.m with H-matrix products (entries assembled and compressed in FP64,
 * products in double-single FP32 arithmetic, ~1e-14 relative), GMRES
 * preconditioned by mfun.m.
 * Excitation: the plane wave exc (ext / sca filled when exc->ninf > 0 for
 * sca), or the potentials pot when pot is not NULL (exc ignored).  One
 * wavelength; out as mnpbem_solve (ir_iters: GMRES steps, ir_resid: true
 * relative residual); info may be NULL.                                     */
MNPBEM_API mnpbem_status mnpbem_solve_iter(mnpbem_geom* g, const mnpbem_cluster_tree* tree,
                                           const mnpbem_iter_options* op, const mnpbem_planewave* exc,
                                           const mnpbem_potentials* pot, double enei, const double* eps_media,
                                           int32_t nmed, int32_t precision, mnpbem_solution* out,
                                           mnpbem_iter_info* info);

/* H-matrix `which` (0 G1, 1 H1, 2 G2, 3 H2) of wavelength enei expanded to a
 * dense [n][n] complex host array (Greenfun/hmatrices/@hmatrix/full.m).
 * ranks [4][nlow] (may be NULL) receives the ACA ranks.                     */
MNPBEM_API mnpbem_status mnpbem_hmat_full(mnpbem_geom* g, const mnpbem_cluster_tree* tree,
                                          const mnpbem_iter_options* op, double enei, const double* eps_media,
                                          int32_t nmed, int32_t which, double* out, int32_t* ranks);

/* ---------------------------------------------------------------------------
 * H-matrix arithmetic (LU, triangular solves, inversion, addition with ACA
 * truncation), the operations behind bemretiter's 'hmat' preconditioner
 * (BEM/@bemretiter/private/initprecond.m).  Each call replaces one MEX
 * function of the reference and takes the same data: a cluster tree, the full
 * blocks and the low-rank factors (Greenfun/hmatrices/@hmatrix val / lhs /
 * rhs), htol and kmax (hopts of mex/hlib/hoptions.h).
 *   vals   full blocks in tree->full order, each rows x cols column-major
 *          complex (interleaved re / im), concatenated
 *   ranks  [nlow] ranks of the low-rank blocks (tree->low order)
 *   lhs    low-rank blocks' left factors, rows x rank column-major, concatenated
 *   rhs    right factors, cols x rank column-major (block = lhs rhs^T)
 * Rows and columns are cluster positions (tree->cind).  Leaves hold at most
 * 1024 positions.  The arithmetic runs in FP64 on the GPU, on one stream per
 * device; results are new handles (free with mnpbem_hm_free).  A zero pivot
 * in a leaf's LU or inverse returns MNPBEM_ERR_SINGULAR.                    */
typedef struct mnpbem_hm_s mnpbem_hm;

MNPBEM_API mnpbem_status mnpbem_hm_create(int32_t device, const mnpbem_cluster_tree* tree, double htol, int32_t kmax,
                                          const double* vals, const int32_t* ranks, const double* lhs,
                                          const double* rhs, mnpbem_hm** out);
/* options of later operations on h (BEM/@bemretiter/private/compress.m)  */
MNPBEM_API mnpbem_status mnpbem_hm_set_options(mnpbem_hm* h, double htol, int32_t kmax);
/* L U of a (mex/hmatlu.cpp; mex/hlib/lu.h:180-198): L lower with its
 * diagonal, U unit upper, both in the returned blocks                        */
MNPBEM_API mnpbem_status mnpbem_hm_lu(const mnpbem_hm* a, mnpbem_hm** out);
/* X with X (L U) = b, lu from mnpbem_hm_lu (mex/hmatrsolve.cpp): key 'N'
 * both factors ('U' then 'L'), 'U' or 'L' one of them; options of b         */
MNPBEM_API mnpbem_status mnpbem_hm_rsolve(const mnpbem_hm* b, const mnpbem_hm* lu, char key, mnpbem_hm** out);
/* X with (L U) X = b, lu from mnpbem_hm_lu (mex/hmatlsolve.cpp): key 'N'
 * both factors ('L' then 'U'), 'L' or 'U' one of them; options of b         */
MNPBEM_API mnpbem_status mnpbem_hm_lsolve(const mnpbem_hm* b, const mnpbem_hm* lu, char key, mnpbem_hm** out);
/* a b (mex/hmatmul2.cpp; mex/hlib/hmatrix.h operator*), options of a        */
MNPBEM_API mnpbem_status mnpbem_hm_matmul(const mnpbem_hm* a, const mnpbem_hm* b, mnpbem_hm** out);
/* inverse of a (mex/hmatinv.cpp; mex/hlib/hmatrix.h inv)                    */
MNPBEM_API mnpbem_status mnpbem_hm_inv(const mnpbem_hm* a, mnpbem_hm** out);
/* a + sign b, sign 1 or -1 (mex/hmatadd.cpp; @hmatrix/plus.m, minus.m)     */
MNPBEM_API mnpbem_status mnpbem_hm_add(const mnpbem_hm* a, const mnpbem_hm* b, double sign, mnpbem_hm** out);
/* diag(d) a (side 'L') or a diag(d) (side 'R'), d [n] complex in cluster
 * order (@hmatrix/private/mtimes1.m)                                        */
MNPBEM_API mnpbem_status mnpbem_hm_scale(const mnpbem_hm* a, const double* d, char side, mnpbem_hm** out);
/* (L U) x = b in place, x [N][n] complex (column-major n x N, cluster order),
 * key 'N' (L then U), 'L' or 'U' (mex/hmatsolve.cpp)                        */
MNPBEM_API mnpbem_status mnpbem_hm_solve(const mnpbem_hm* lu, char key, double* x, int32_t N);
/* y = a x, x and y column-major n x N complex in cluster order (hmatmul1)   */
MNPBEM_API mnpbem_status mnpbem_hm_mul(const mnpbem_hm* a, const double* x, double* y, int32_t N);
/* a expanded to out, n x n column-major complex in cluster order (hmatfull) */
MNPBEM_API mnpbem_status mnpbem_hm_full(const mnpbem_hm* a, double* out);
/* sizes of mnpbem_hm_export's arrays in complex entries                     */
MNPBEM_API mnpbem_status mnpbem_hm_sizes(const mnpbem_hm* a, int64_t* nvals, int64_t* nlhs, int64_t* nrhs);
/* blocks of a in mnpbem_hm_create's layout (any pointer may be NULL)        */
MNPBEM_API mnpbem_status mnpbem_hm_export(const mnpbem_hm* a, double* vals, int32_t* ranks, double* lhs,
                                          double* rhs);
MNPBEM_API void mnpbem_hm_free(mnpbem_hm* h);

/* Self test of the bounded device-side waits that every pipelined kernel of
 * the library uses (mbarrier waits with a wall-clock limit): one CTA waits,
 * with a limit of limit_us microseconds (1 .. 1e6), on a barrier that nothing
 * completes; the wait expires, the kernel records an error code and returns.
 * Returns MNPBEM_ERR_TIMEOUT (the expected outcome), and the context stays
 * usable.  No counterpart in the reference (its MEX code has no device waits). */
MNPBEM_API mnpbem_status mnpbem_selftest_bounded_wait(int32_t device, int32_t limit_us);

/* Message of the last failure on the calling thread ("" if none). */
MNPBEM_API const char* mnpbem_last_error(void);

/* Library version string. */
MNPBEM_API const char* mnpbem_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MNPBEM_GPU_H */
