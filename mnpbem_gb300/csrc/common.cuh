// Shared device/host helpers for the MNPBEM retarded-BEM GPU library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/mnpbem_gpu.h"

namespace mnpbem {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
const char* get_error();

#define MNP_CUDA(call)                                                         \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ::mnpbem::set_error("%s:%d CUDA error %s: %s", __FILE__, __LINE__,       \
                          cudaGetErrorName(e_), cudaGetErrorString(e_));       \
      return MNPBEM_ERR_CUDA;                                                  \
    }                                                                          \
  } while (0)

#define MNP_CHECK_LAUNCH() MNP_CUDA(cudaGetLastError())

#define MNP_TRY(expr)                                                          \
  do {                                                                         \
    mnpbem_status s_ = (expr);                                                 \
    if (s_ != MNPBEM_OK) return s_;                                            \
  } while (0)

// ------------------------------------------------------------ complex math
template <typename R> struct cplx_t;
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<double> { using type = double2; };
template <typename R> using cplx = typename cplx_t<R>::type;

template <typename R> __host__ __device__ __forceinline__ cplx<R> mk(R x, R y) {
  cplx<R> c; c.x = x; c.y = y; return c;
}
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) {
  C c; c.x = a.x + b.x; c.y = a.y + b.y; return c;
}
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) {
  C c; c.x = a.x - b.x; c.y = a.y - b.y; return c;
}
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
template <typename C, typename R> __host__ __device__ __forceinline__ C cscale(C a, R s) {
  C c; c.x = a.x * s; c.y = a.y * s; return c;
}
// c += a * b
template <typename C> __host__ __device__ __forceinline__ void cfma(C& c, C a, C b) {
  c.x = fma(a.x, b.x, c.x); c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y); c.y = fma(a.y, b.x, c.y);
}
template <typename C> __host__ __device__ __forceinline__ C cdiv(C a, C b) {
  // Smith's algorithm
  C c;
  if (fabs(b.x) >= fabs(b.y)) {
    auto r = b.y / b.x; auto den = b.x + b.y * r;
    c.x = (a.x + a.y * r) / den; c.y = (a.y - a.x * r) / den;
  } else {
    auto r = b.x / b.y; auto den = b.x * r + b.y;
    c.x = (a.x * r + a.y) / den; c.y = (a.y * r - a.x) / den;
  }
  return c;
}
template <typename C> __host__ __device__ __forceinline__ double cabs2(C a) {
  return (double)a.x * a.x + (double)a.y * a.y;
}

__host__ __device__ __forceinline__ float2 to_f(double2 a) { return make_float2((float)a.x, (float)a.y); }
__host__ __device__ __forceinline__ double2 to_d(float2 a) { return make_double2(a.x, a.y); }
__host__ __device__ __forceinline__ double2 to_d(double2 a) { return a; }
template <typename C> __host__ __device__ __forceinline__ C from_d(double2 a);
template <> __host__ __device__ __forceinline__ double2 from_d<double2>(double2 a) { return a; }
template <> __host__ __device__ __forceinline__ float2 from_d<float2>(double2 a) { return to_f(a); }

// Per-wavelength scalars, kept in device memory so that the kernels of one
// wavelength can be captured once in CUDA graphs and replayed for the next.
constexpr int LAM_MAXMED = 16;
struct LamParams {
  double2 k[LAM_MAXMED];    // wavenumber 2 pi / enei sqrt(eps_m) of each medium
  double2 eps[LAM_MAXMED];  // dielectric function of each medium
  double2 kexc;             // wavenumber in the excitation medium
  double2 nb1;              // refractive index sqrt(eps_1) of medium 1
  double k0;                // vacuum wavenumber 2 pi / enei
  int w;                    // index of the wavelength in the sweep (output slot)
  int pad;
};

// Area of the triangle (v1, v2, v3) as norm_flat.m computes it: N = (v1 - v2) x
// (v3 - v2), 0.5 sqrt(N . N), every product and sum rounded on its own in that
// order (no fused multiply-add).  A quadrilateral takes the basis of the
// larger of its two triangles; for symmetric warped quadrilaterals (rounded
// cube edges) the two areas agree to the last bits, so the choice must follow
// the same roundings as the reference's (and the oracle's) evaluation.
#ifdef __CUDACC__
__device__ __forceinline__ double tri_area_rn(double3 v1, double3 v2, double3 v3) {
  const double ax = __dsub_rn(v1.x, v2.x), ay = __dsub_rn(v1.y, v2.y), az = __dsub_rn(v1.z, v2.z);
  const double bx = __dsub_rn(v3.x, v2.x), by = __dsub_rn(v3.y, v2.y), bz = __dsub_rn(v3.z, v2.z);
  const double nx = __dsub_rn(__dmul_rn(ay, bz), __dmul_rn(az, by));
  const double ny = __dsub_rn(__dmul_rn(az, bx), __dmul_rn(ax, bz));
  const double nz = __dsub_rn(__dmul_rn(ax, by), __dmul_rn(ay, bx));
  const double nn = __dadd_rn(__dadd_rn(__dmul_rn(nx, nx), __dmul_rn(ny, ny)), __dmul_rn(nz, nz));
  return __dmul_rn(0.5, __dsqrt_rn(nn));
}
#endif

inline int64_t cdiv_up(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return cdiv_up(a, b) * b; }

// ------------------------------------------------------- device buffers
// Every (re)allocation bumps alloc_generation(), which invalidates CUDA graphs
// that captured buffer addresses; during a capture no allocation may happen.
uint64_t& alloc_generation();
bool& capturing_now();

struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr; bytes = 0;
  }
  mnpbem_status ensure(size_t nbytes) {
    if (bytes >= nbytes && ptr) return MNPBEM_OK;
    if (capturing_now()) {
      set_error("internal: device allocation of %zu bytes requested during graph capture", nbytes);
      return MNPBEM_ERR_CUDA;
    }
    release();
    ++alloc_generation();
    if (nbytes == 0) return MNPBEM_OK;
    cudaError_t e = cudaMalloc(&ptr, nbytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMalloc of %zu bytes failed: %s", nbytes, cudaGetErrorString(e));
      ptr = nullptr;
      return MNPBEM_ERR_OUT_OF_MEMORY;
    }
    bytes = nbytes;
    return MNPBEM_OK;
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(ptr); }
};

}  // namespace mnpbem
