// Complex64 GEMM on the 5th-generation tensor cores (tcgen05, kind::tf32).
#pragma once
#include "common.cuh"

namespace mnpbem {

struct TcGemmCtx {
  bool checked = false;   // device capability probed
  bool usable = false;    // sm_103 device, driver entry point and kernel attributes available
  bool enabled = true;    // switched off after a device-side error
  bool err_cleared = false;
  DevBuf bexp;            // expanded B operand [2N][2K] (real, K-major, tf32 or fp16)
  DevBuf a16, scales;     // FP16 path: A operand [M][2K] in fp16, row / column scales
  bool f16 = false;       // FP16 operands with power-of-two row / column scaling (kind::f16)
  int f16_min_k = 512;    // ... for products with K >= f16_min_k
  int f16_min_mn = 512;   //     and M, N >= f16_min_mn
  DevBuf err;             // device error word of the bounded waits
  DevBuf ctr;             // tile counter of the persistent kernel (zeroed before each launch)
  int num_sms = 0;
  int stages = 4;         // pipeline depth of the persistent kernel (3 or 4)
  int pair = 0;           // CTA-pair kernel (tcgen05 cta_group::2, 256 x 256 tiles) for M >= 256:
                          // 1 always, 0 never, -1 for long K (at least 1024), where it is faster
  int pair_epi = 0;       // epilogue of the pair kernel: 0 TMA store / reduce-add, 1 vector stores / reductions
  int pair_nb = 2;        // epilogue staging buffers per warp of the pair kernel (2: 6 stages, 4: 5 stages)
  int max_ctas = 0;       // CTAs of the persistent kernel (0: one per SM); fewer leave SMs
                          // to the pivot-block clusters of other wavelengths in flight
  void* encode_fn = nullptr;
};

// true when the tensor-core path can run this product (device, shape and layout:
// even leading dimensions and 16-byte aligned A and C, real beta)
bool tc_gemm_eligible(TcGemmCtx& c, int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                      const void* C, int64_t ldc, float2 beta);
// B's columns [bz0, bz1) are read as zero (the B operand is copied, expanded,
// before the product runs, so C may overlap B)
mnpbem_status tc_gemm_c64(TcGemmCtx& c, int64_t M, int64_t N, int64_t K, float2 alpha,
                          const float2* A, int64_t lda, const float2* B, int64_t ldb, float2 beta,
                          float2* C, int64_t ldc, cudaStream_t st, int64_t bz0 = 0, int64_t bz1 = 0);
// reads (and clears) the device error word; MNPBEM_ERR_TIMEOUT if a wait expired
mnpbem_status tc_check_error(TcGemmCtx& c, cudaStream_t st);
void tc_release(TcGemmCtx& c);

}  // namespace mnpbem
