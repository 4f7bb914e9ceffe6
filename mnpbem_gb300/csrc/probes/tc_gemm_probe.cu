// Standalone timing of the tensor-core complex64 GEMM variants (one CTA per
// 128 x 256 tile, CTA pairs per 256 x 256 tile with TMA or load-store
// epilogue; beta 0 and 1) on the shapes of the solver: the rank-256 Gauss-
// Jordan update at n = 4000 and 12000, the 256-row panel product and the n^3
// Sigma product.  CUDA-event timing of 10 launches (B expansion included)
// after 3 warm-ups.  Build after the library:
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -Iinclude \
//        mnpbem_gb300/csrc/probes/tc_gemm_probe.cu mnpbem_gb300/_build/*.o -lcuda -o tc_gemm_probe
#include <cstdio>
#include <cstdlib>
#include "../common.cuh"
#include "../tc_gemm.cuh"
using namespace mnpbem;
__global__ void fill(float2* p, size_t n, unsigned seed) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)(i * 2654435761u) ^ seed;
    h ^= h >> 13; h *= 0x5bd1e995u; h ^= h >> 15;
    p[i] = make_float2(((h & 0xffff) / 65536.f - 0.5f) * 1e-2f, ((h >> 16) / 65536.f - 0.5f) * 1e-2f);
  }
}
int main(int argc, char** argv) {
  struct Shape { int64_t M, N, K; const char* name; };
  Shape shapes[] = {{4000, 4000, 256, "rank256 update"}, {256, 4000, 256, "panel product"},
                    {4000, 4000, 4000, "Sigma product"}, {12000, 12000, 256, "rank256 update 12k"}};
  cudaStream_t st; cudaStreamCreate(&st);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  for (auto& sh : shapes) {
    const int64_t M = sh.M, N = sh.N, K = sh.K, lda = K, ldb = N, ldc = N;
    float2 *A, *B, *C;
    cudaMalloc(&A, sizeof(float2) * M * lda); cudaMalloc(&B, sizeof(float2) * K * ldb); cudaMalloc(&C, sizeof(float2) * M * ldc);
    fill<<<1024, 256, 0, st>>>(A, M * lda, 1); fill<<<1024, 256, 0, st>>>(B, K * ldb, 2); fill<<<1024, 256, 0, st>>>(C, M * ldc, 3);
    for (int cfg = 0; cfg < 3; ++cfg)
      for (int stages = 4; stages <= 4; ++stages)
        for (int beta = 0; beta < 2; ++beta) {
          const int pair = cfg > 0;
          TcGemmCtx c; c.pair = pair ? 1 : 0; c.pair_epi = cfg == 2 ? 1 : 0;
          if (!tc_gemm_eligible(c, M, N, K, A, lda, C, ldc, make_float2((float)beta, 0.f))) { printf("not eligible\n"); return 1; }
          c.stages = stages;
          const float2 al = make_float2(-1.f, 0.f), be = make_float2((float)beta, 0.f);
          for (int w = 0; w < 3; ++w) tc_gemm_c64(c, M, N, K, al, A, lda, B, ldb, be, C, ldc, st);
          const int reps = 10;
          cudaEventRecord(e0, st);
          for (int r = 0; r < reps; ++r) tc_gemm_c64(c, M, N, K, al, A, lda, B, ldb, be, C, ldc, st);
          cudaEventRecord(e1, st);
          cudaStreamSynchronize(st);
          float ms = 0; cudaEventElapsedTime(&ms, e0, e1);
          int s = tc_check_error(c, st);
          const double us = 1e3 * ms / reps;
          printf("%-20s cfg %d stages %d beta %d : %8.1f us  %7.1f TFLOP/s (incl. B expansion)  status %d\n", sh.name, cfg, stages, beta,
                 us, 8.0 * M * N * K / (us * 1e-6) / 1e12, s);
          tc_release(c);
        }
    cudaFree(A); cudaFree(B); cudaFree(C);
  }
  printf("last error: %s\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
