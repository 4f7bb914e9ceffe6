// Extinction and scattering cross sections of given surface charges and
// currents (exc.ext(sig), exc.sca(sig):
// Simulation/retarded/@planewaveret/extinction.m:12-16, scattering.m:13-19,
// @spectrumret/farfield.m:15-74) with no device allocation at all.
//
// Some callers cannot call cudaMalloc: a MEX gateway running inside a MATLAB
// session whose GPU memory is owned by MATLAB's own allocator, a plugin inside
// a host application that owns all device memory through its own pool, or a
// real-time loop that must not meet allocation latency or an out-of-memory
// failure in the middle of a run.  For them this entry point takes only
// caller-owned device pointers for its inputs and outputs, and keeps its one
// piece of scratch — the far fields e and h of every direction and
// polarisation — in a file-scope __device__ array of fixed size
// (NOALLOC_MAX_DIRS directions x 6 components x NOALLOC_MAX_POL
// polarisations of complex128 = 768 KB), which every GPU that loads the
// library holds until the process exits.
//
// Host code cannot use the array's name as a device address (in host code it
// is only a stand-in).  Every call, with its device current, looks the address
// up with cudaGetSymbolAddress (a host-side query that allocates nothing), so
// that a context re-created after cudaDeviceReset (MATLAB's reset(gpuDevice))
// never leaves a stale address behind.  The first call on a device also loads
// the library's module into that context: make it before any stream capture.
// Every call shares the array and it
// keeps the previous call's contents: each call first writes every entry it
// later reads, so nothing needs clearing, but calls whose kernels overlap on
// the GPU (different streams, or threads sharing a device) race on it.
#include <complex>

#include "bem.cuh"
#include "farfield.cuh"

namespace mnpbem {

constexpr int NOALLOC_MAX_POL = 4;
constexpr int NOALLOC_MAX_DIRS = 2048;   // excitation directions + sphere-at-infinity directions

static __device__ __align__(256) double2 g_noalloc_fields[NOALLOC_MAX_DIRS * 6 * NOALLOC_MAX_POL];


// Far fields of one direction per block, inputs in the public solution layout
// (sig [n][P], h [n][3][P] per side); direction d < P is dir[d], else
// inf_nvec[d - P].  The far-field routine of the solve (farfield.cuh) with
// this layout.
struct SplitSrc {
  const double2 *s1, *h1, *s2, *h2;
  int P;
  __device__ double2 sig(int side, int64_t j, int p) const { return (side ? s2 : s1)[j * P + p]; }
  __device__ double2 h(int side, int64_t j, int c, int p) const { return (side ? h2 : h1)[(j * 3 + c) * P + p]; }
};

__global__ void __launch_bounds__(256) k_farfield_noalloc(
    int64_t n, int P, const double* __restrict__ pos, const double* __restrict__ area,
    const unsigned char* __restrict__ exc_in, const unsigned char* __restrict__ exc_out,
    const double2* __restrict__ sig1, const double2* __restrict__ h1, const double2* __restrict__ sig2,
    const double2* __restrict__ h2, const double* __restrict__ dir, const double* __restrict__ inf_nvec,
    double2 k, double k0, double2* fields) {
  const int d = blockIdx.x;
  const double* dv = d < P ? dir + 3 * d : inf_nvec + 3 * (d - P);
  farfield_dir<NOALLOC_MAX_POL>(n, P, pos, area, exc_in, exc_out, SplitSrc{sig1, h1, sig2, h2, P}, dv[0], dv[1],
                                dv[2], k, k0, d, fields);
}

// device address of the scratch array in the current context, looked up on
// every call: a cached address would outlive a reset of the device's context
static mnpbem_status noalloc_scratch(double2** out) {
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_fields);
  if (e != cudaSuccess || !ptr) {
    cudaGetLastError();
    set_error("cudaGetSymbolAddress of the cross-section scratch failed: %s", cudaGetErrorString(e));
    return MNPBEM_ERR_CUDA;
  }
  *out = static_cast<double2*>(ptr);
  return MNPBEM_OK;
}

}  // namespace mnpbem

using namespace mnpbem;

extern "C" mnpbem_status mnpbem_cross_sections_noalloc(
    int32_t device, void* stream, int64_t n, int32_t npol, const double* pos, const double* area,
    const unsigned char* exc_in, const unsigned char* exc_out, const double* sig1, const double* h1,
    const double* sig2, const double* h2, const double* pol, const double* dir, int32_t ninf,
    const double* inf_nvec, const double* inf_area, double enei, const double* eps_exc,
    const double* eps_1, double* ext, double* sca) {
  if (n <= 0 || npol <= 0 || ninf < 0 || !pos || !area || !exc_in || !exc_out || !sig1 || !h1 || !sig2 ||
      !h2 || !pol || !dir || (ninf > 0 && (!inf_nvec || !inf_area)) || !eps_exc || !eps_1 || !ext ||
      !sca || !(enei > 0)) {
    set_error("mnpbem_cross_sections_noalloc: invalid arguments");
    return MNPBEM_ERR_INVALID_ARG;
  }
  if (npol > NOALLOC_MAX_POL) {
    set_error("mnpbem_cross_sections_noalloc: npol = %d exceeds the maximum of %d polarisations",
              (int)npol, NOALLOC_MAX_POL);
    return MNPBEM_ERR_INVALID_ARG;
  }
  if ((int64_t)npol + ninf > NOALLOC_MAX_DIRS) {
    set_error("mnpbem_cross_sections_noalloc: npol + ninf = %lld directions exceed the maximum of %d",
              (long long)npol + ninf, NOALLOC_MAX_DIRS);
    return MNPBEM_ERR_INVALID_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess) cudaGetLastError();
  if (device < 0 || device >= ndev) {
    set_error("mnpbem_cross_sections_noalloc: invalid device %d", (int)device);
    return MNPBEM_ERR_INVALID_ARG;
  }
  MNP_CUDA(cudaSetDevice(device));
  double2* fields = nullptr;
  MNP_TRY(noalloc_scratch(&fields));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double k0 = 2 * M_PI / enei;
  const std::complex<double> kmed = k0 * std::sqrt(std::complex<double>(eps_exc[0], eps_exc[1]));
  const std::complex<double> nb1 = std::sqrt(std::complex<double>(eps_1[0], eps_1[1]));
  const double2 k = make_double2(kmed.real(), kmed.imag());
  k_farfield_noalloc<<<npol + ninf, 256, 0, st>>>(
      n, npol, pos, area, exc_in, exc_out, reinterpret_cast<const double2*>(sig1),
      reinterpret_cast<const double2*>(h1), reinterpret_cast<const double2*>(sig2),
      reinterpret_cast<const double2*>(h2), dir, inf_nvec, k, k0, fields);
  MNP_CHECK_LAUNCH();
  launch_cross_sections(npol, pol, inf_nvec, inf_area, ninf, fields, k,
                        make_double2(nb1.real(), nb1.imag()), ext, sca, st);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}
