// Standalone timing of the library's thin complex64 GEMM (gemm_simt<float>,
// N <= 4 right-hand sides) on n x n matrices that stream from HBM: five
// matrices alternate so that no launch finds its matrix in L2.  CUDA-event
// timing over 30 launches after 3 warm-ups; MNPBEM_THIN_STREAM=0 selects the
// register-tiled kernel instead of the streamed one.  Build after the library:
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -lineinfo -Iinclude \
//        mnpbem_gb300/csrc/probes/thin_gemm_probe.cu mnpbem_gb300/_build/*.o -lcuda -o thin_gemm_probe
#include <cstdio>
#include <cstdlib>
#include "../common.cuh"
#include "../dense.cuh"
using namespace mnpbem;
__global__ void fill(float2* p, size_t n, unsigned seed) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)(i * 2654435761u) ^ seed; h ^= h >> 13; h *= 0x5bd1e995u; h ^= h >> 15;
    p[i] = make_float2((h & 0xffff) / 65536.f - 0.5f, (h >> 16) / 65536.f - 0.5f);
  }
}
int main(int argc, char** argv) {
  // optional argument: a single matrix size n (default: 4000 and 12000)
  const int64_t only = argc > 1 ? atoll(argv[1]) : 0;
  const int NM = 5;
  for (int64_t n : {(int64_t)4000, (int64_t)12000}) {
    if (only && n != only) continue;
    const int64_t ld = (n + 31) / 32 * 32;
    float2* A[NM];
    for (int m = 0; m < NM; ++m) { cudaMalloc(&A[m], n * ld * 8); fill<<<2048, 256>>>(A[m], n * ld, m + 1); }
    float2 *B, *C; cudaMalloc(&B, ld * 4 * 8); cudaMalloc(&C, ld * 4 * 8); fill<<<64, 256>>>(B, ld * 4, 9);
    cudaStream_t st; cudaStreamCreate(&st);
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    for (int N : {1, 3, 4}) {
      for (int w = 0; w < 3; ++w) gemm_simt<float>(n, N, n, make_float2(1, 0), A[w % NM], ld, B, N, make_float2(0, 0), C, N, st);
      const int reps = 30;
      cudaEventRecord(e0, st);
      for (int r = 0; r < reps; ++r) gemm_simt<float>(n, N, n, make_float2(1, 0), A[r % NM], ld, B, N, make_float2(0, 0), C, N, st);
      cudaEventRecord(e1, st); cudaEventSynchronize(e1);
      float ms; cudaEventElapsedTime(&ms, e0, e1);
      const double us = 1e3 * ms / reps;
      printf("n %6lld N %d : %8.1f us  %6.2f TB/s  %s\n", (long long)n, N, us, n * n * 8 / (us * 1e-6) / 1e12, cudaGetErrorString(cudaGetLastError()));
    }
    for (int m = 0; m < NM; ++m) cudaFree(A[m]);
    cudaFree(B); cudaFree(C);
  }
  printf("stream check %d\n", (int)thin_stream_check(0));
  return 0;
}
