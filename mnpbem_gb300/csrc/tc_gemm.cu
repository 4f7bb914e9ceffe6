// Complex64 GEMM on the 5th-generation tensor cores: tcgen05.mma kind::tf32
// with operands staged by TMA (cp.async.bulk.tensor) into 128-byte-swizzled
// shared memory, the accumulator in tensor memory, and an mbarrier pipeline.
//
// A complex product C = alpha A B + beta C (row-major, interleaved complex)
// is one real GEMM on the interleaved view:
//     C_r[M][2N] = A_r[M][2K] * B'[2N][2K]^T (+ beta C_r)
// A_r is the complex64 matrix A read as floats (K-major, no copy).  B' is built
// from alpha * B by k_expand_b (O(K N) work):
//     B'[2j  ][2l] =  Re b_lj   B'[2j  ][2l+1] = -Im b_lj
//     B'[2j+1][2l] =  Im b_lj   B'[2j+1][2l+1] =  Re b_lj
// so that C_r[i][2j] = sum_l (Re a Re b - Im a Im b) and
// C_r[i][2j+1] = sum_l (Re a Im b + Im a Re b).  B' is rounded to TF32.
//
// Tile: 128 x 256 real outputs, K chunks of 32 floats (one 128-byte swizzle
// row), 3 or 4 pipeline stages (48 KB each), two TMEM accumulators; the kernel is
// persistent with warp-specialised producer / MMA / epilogue roles (below).
// Every mbarrier wait is bounded by a wall-clock limit; on expiry the kernel
// records an error code, waits (bounded) for its own copies in flight, frees
// its tensor memory and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include "mbarrier.cuh"
#include "profile.cuh"
#include "tc_gemm.cuh"

#include <algorithm>

namespace mnpbem {

constexpr int TC_BM = 128, TC_BN = 256, TC_BK = 32;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 4;   // 16 KB
constexpr int TC_B_BYTES = TC_BN * TC_BK * 4;   // 32 KB
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
constexpr uint32_t TC_TMEM_COLS = 256;
constexpr unsigned long long TC_WAIT_NS = MBAR_WAIT_NS;

// instruction descriptor: D f32, A/B tf32, K-major A and B, N = 256, M = 128
// kind::f16 with FP16 A and B (the same type for both), FP32 accumulator
constexpr uint32_t TC_IDESC_F16 = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(TC_BN >> 3) << 17) |
                                  ((uint32_t)(TC_BM >> 4) << 24);
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_BN >> 3) << 17) |
                              ((uint32_t)(TC_BM >> 4) << 24);

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(dst), "l"((unsigned long long)map), "r"(bar), "r"(x), "r"(y)
      : "memory");
}
// L2 prefetch of one C tile (128 rows x 256 floats, unswizzled map) so that the
// epilogue's reduce-add finds C in L2 instead of waiting for HBM
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap* map, int x, int y) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];"
               ::"l"((unsigned long long)map), "r"(x), "r"(y)
               : "memory");
}
// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused with one swizzle atom along K)
  d |= (uint64_t)(1024u >> 4) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;             // descriptor version
  d |= (uint64_t)2 << 61;             // 128-byte swizzle
  return d;
}
__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(dtmem), "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(dtmem), "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}
// Tile order of the persistent kernels: groups of TC_GROUP_M row tiles, and
// within a group the column tiles one after another (the group's row tiles
// fastest).  The CTAs in flight then share a few A row panels (TC_GROUP_M x
// 128 rows) and a few B' tiles, which stay in L2; with the plain row-fastest
// order every column of tiles sweeps the whole A panel, which at n = 24 000
// and K = 512 (98 MB) does not stay in L2 next to the streamed C tiles and is
// read again from HBM for every column.
constexpr int TC_GROUP_M = 32;
__device__ __forceinline__ void tile_coords(int t, int MT, int NT, int& mt, int& nt) {
  const int per_group = TC_GROUP_M * NT;
  const int g = t / per_group;
  const int m_first = g * TC_GROUP_M;
  const int gm = min(TC_GROUP_M, MT - m_first);
  const int r = t - g * per_group;
  mt = m_first + r % gm;
  nt = r / gm;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
      "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
        "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// C_r[M][N2] = A_r[M][K2] * B'[N2][K2]^T + beta * C_r        (all row-major floats)
//
// Persistent kernel, one CTA per SM, 192 threads in three roles:
//   warp 0      TMA producer: takes tile indices from a global counter
//               (dynamic schedule: CTAs that start late take fewer tiles) and
//               streams the K chunks of A and B' through ST buffers (3 or 4:
//               with 3 the kernel leaves ~50 KB of shared memory per SM to
//               kernels of other streams),
//               running ahead across tile boundaries;
//   warp 1      MMA issuer: accumulates each tile into one of two TMEM
//               accumulators (2 x 256 columns) so that the next tile's MMAs
//               overlap the previous tile's epilogue;
//   warps 2-5   epilogue: TMEM -> registers -> shared staging -> TMA bulk
//               tensor store (beta = 0) or reduce-add (beta = 1) into C.
// The tile indices pass from the producer to the other roles through a
// four-slot ring in shared memory guarded by mbarriers.
constexpr int TC_EPI_WARPS = 4;
constexpr int TC_THREADS = 32 * (2 + TC_EPI_WARPS);
constexpr int TC_STAGE_SMEM = TC_EPI_WARPS * 2 * 4096;   // two 32 x 32 float staging tiles per epilogue warp
constexpr int tc_psmem(int stages) { return stages * TC_STAGE_BYTES + TC_STAGE_SMEM + 1024; }
constexpr int TC_TQ = 4;                                  // tile-index ring slots

// One 32 x 32 accumulator chunk (row = lane, r = its 32 columns) stored from
// the SM's load-store path: transposed through the warp's 4 KB staging tile
// (row per lane in, eight lanes per 128-byte row out) and written with
// coalesced vector stores (beta = 0) or vector reductions (beta = 1).  Used
// where the TMA store cannot be: a row length of 2N floats that is not a
// multiple of 16 bytes (TMA writes whole 16-byte granules at the right edge).
__device__ __forceinline__ void epi_chunk_lsu(const uint32_t (&r)[32], float* stage, int lane, float* __restrict__ Cp,
                                              long long ldcf, int row0, int col0, int M, int N2, int accumulate) {
  float4* st = reinterpret_cast<float4*>(stage) + lane * 8;
#pragma unroll
  for (int c4 = 0; c4 < 8; ++c4)
    st[c4 ^ (lane & 7)] = make_float4(__uint_as_float(r[4 * c4]), __uint_as_float(r[4 * c4 + 1]),
                                      __uint_as_float(r[4 * c4 + 2]), __uint_as_float(r[4 * c4 + 3]));
  __syncwarp();
  const int q4 = lane & 7, col = col0 + 4 * q4;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int rr = 4 * i + (lane >> 3), grow = row0 + rr;
    const float4 v = reinterpret_cast<const float4*>(stage)[rr * 8 + (q4 ^ (rr & 7))];
    if (grow < M && col < N2) {
      float* dst = Cp + (long long)grow * ldcf + col;
      if (col + 4 <= N2) {
        if (accumulate)
          asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(v.x), "f"(v.y), "f"(v.z),
                       "f"(v.w)
                       : "memory");
        else
          *reinterpret_cast<float4*>(dst) = v;
      } else {                                          // N2 is even: a last pair of columns
        if (accumulate)
          asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(dst), "f"(v.x), "f"(v.y) : "memory");
        else
          *reinterpret_cast<float2*>(dst) = make_float2(v.x, v.y);
      }
    }
  }
  __syncwarp();
}

// F16: A and B' are FP16 (kind::f16), scaled per row of A and per complex
// column of B' into FP16's range; the epilogue multiplies each accumulator by
// inv_r[row] * inv_c[column / 2] before storing.  K2 counts elements of the
// operand type (TF32 floats or halves); a K chunk is one 128-byte swizzle row
// either way (32 floats or 64 halves).
template <int ST, int EPI, bool F16>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
              const __grid_constant__ CUtensorMap mapC, const __grid_constant__ CUtensorMap mapP,
              float* __restrict__ Cp, long long ldcf, int M, int N2, int K2, int accumulate, int* tile_ctr, int* err,
              const float* __restrict__ inv_r, const float* __restrict__ inv_c) {
  constexpr int BK = F16 ? 64 : TC_BK;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bars[2 * ST + 4 + 2 * TC_TQ];
  __shared__ int tq[TC_TQ];
  __shared__ uint32_t tmem_slot;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int KT = (K2 + BK - 1) / BK;
  const int MT = (M + TC_BM - 1) / TC_BM, NT = (N2 + TC_BN - 1) / TC_BN;
  const int ntiles = MT * NT;
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[ST]);
  const uint32_t accf0 = smem_u32(&bars[2 * ST]), acce0 = smem_u32(&bars[2 * ST + 2]);
  const uint32_t tqf0 = smem_u32(&bars[2 * ST + 4]), tqe0 = smem_u32(&bars[2 * ST + 4 + TC_TQ]);
  const uint32_t stage_base = base + ST * TC_STAGE_BYTES;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, TC_EPI_WARPS);
    }
    for (int q = 0; q < TC_TQ; ++q) {
      mbar_init(tqf0 + 8 * q, 1);
      mbar_init(tqe0 + 8 * q, 1 + TC_EPI_WARPS);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(2 * TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  int issued = 0;   // producer: K chunks issued (for the drain after an error)
  if (warp == 0) {
    if (lane == 0) {
      // ---------------- tile scheduler + TMA producer
      int it = 0;
      // the tile counter is read one tile ahead: the atomic's round trip
      // overlaps the current tile's copies instead of stalling the pipeline
      int t_next = atomicAdd(tile_ctr, 1);
      for (int j = 0;; ++j) {
        const int q = j % TC_TQ;
        if (j >= TC_TQ && !mbar_wait(tqe0 + 8 * q, ((j / TC_TQ) - 1) & 1, err, 16)) break;
        int t = *(volatile int*)err ? -1 : t_next;
        if (t >= ntiles) t = -1;
        if (t >= 0) t_next = atomicAdd(tile_ctr, 1);
        tq[q] = t;
        mbar_arrive(tqf0 + 8 * q);
        if (t < 0) break;
        int mt, nt;
        tile_coords(t, MT, NT, mt, nt);
        const int m0 = mt * TC_BM, n0 = nt * TC_BN;
        if (accumulate) tma_prefetch_2d(&mapP, n0, m0);
        bool ok = true;
        for (int kt = 0; kt < KT; ++kt, ++it) {
          const int s = it % ST;
          if (it >= ST && !mbar_wait(empty0 + 8 * s, ((it / ST) - 1) & 1, err, 1)) { ok = false; break; }
          const uint32_t sa = base + s * TC_STAGE_BYTES, sb = sa + TC_A_BYTES;
          mbar_expect_tx(full0 + 8 * s, TC_STAGE_BYTES);
          tma_load_2d(sa, &mapA, full0 + 8 * s, kt * BK, m0);
          tma_load_2d(sb, &mapB, full0 + 8 * s, kt * BK, n0);
          issued = it + 1;
        }
        if (!ok) {
          // hand out an end marker in the next slot so that the other roles stop
          const int q2 = (j + 1) % TC_TQ;
          if (j + 1 < TC_TQ || mbar_wait(tqe0 + 8 * q2, (((j + 1) / TC_TQ) - 1) & 1, err, 16)) {
            tq[q2] = -1;
            mbar_arrive(tqf0 + 8 * q2);
          }
          break;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      int it = 0;
      for (int j = 0;; ++j) {
        const int q = j % TC_TQ;
        if (!mbar_wait(tqf0 + 8 * q, (j / TC_TQ) & 1, err, 32)) break;
        const int t = *(volatile int*)&tq[q];
        mbar_arrive(tqe0 + 8 * q);
        if (t < 0) break;
        const int b = j & 1;
        if (j >= 2 && !mbar_wait(acce0 + 8 * b, ((j >> 1) - 1) & 1, err, 64)) break;
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)(b * TC_TMEM_COLS);
        bool ok = true;
        for (int kt = 0; kt < KT; ++kt, ++it) {
          const int s = it % ST;
          if (!mbar_wait(full0 + 8 * s, (it / ST) & 1, err, 2)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sa = base + s * TC_STAGE_BYTES, sb = sa + TC_A_BYTES;
          const uint64_t da = desc_sw128(sa), db = desc_sw128(sb);
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            // advance 8 tf32 or 16 halves = 32 bytes along K inside the swizzle row
            if constexpr (F16)
              mma_f16(dt, da + 2 * kk, db + 2 * kk, TC_IDESC_F16, (kt > 0 || kk > 0) ? 1u : 0u);
            else
              mma_tf32(dt, da + 2 * kk, db + 2 * kk, TC_IDESC, (kt > 0 || kk > 0) ? 1u : 0u);
          }
          mma_commit(empty0 + 8 * s);
        }
        if (!ok) break;
        mma_commit(accf0 + 8 * b);
      }
    }
  } else {
    // ---------------- epilogue warps: TMEM lane quarter (warp % 4) = 32 rows of the tile
    const int ew = warp - 2;                 // staging slot
    const int quarter = warp & 3;
    const uint32_t stage0 = stage_base + (uint32_t)ew * 2u * 4096u;
    float* stage_gen = reinterpret_cast<float*>(smem_raw + (stage_base - smem_u32(smem_raw))) + ew * 2 * 1024;
    int nstores = 0;
    for (int j = 0;; ++j) {
      const int q = j % TC_TQ;
      int t = -1;
      const bool okq = __all_sync(0xffffffffu, mbar_wait(tqf0 + 8 * q, (j / TC_TQ) & 1, err, 128) ? 1 : 0) != 0;
      if (okq) t = *(volatile int*)&tq[q];
      __syncwarp();
      if (lane == 0 && okq) mbar_arrive(tqe0 + 8 * q);
      if (!okq || t < 0) break;
      const int b = j & 1;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(accf0 + 8 * b, (j >> 1) & 1, err, 4) ? 1 : 0) != 0;
      if (!ok) break;
      tc_fence_after();
      int mt, nt;
      tile_coords(t, MT, NT, mt, nt);
      const int m0 = mt * TC_BM, n0 = nt * TC_BN;
      const int row0 = m0 + quarter * 32;
      for (int c = 0; c < TC_BN / 32; ++c) {
        const int col0 = n0 + c * 32;
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * TC_TMEM_COLS + c * 32), r);
        if (col0 >= N2 || row0 >= M) continue;            // warp-uniform
        if constexpr (F16) {
          // undo the operand scaling: row scale of this lane's row, column
          // scale of each complex column (two floats)
          const float rs = (row0 + lane < M) ? __ldg(inv_r + row0 + lane) : 0.f;
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int cc = (col0 >> 1) + q;
            const float sc = rs * ((2 * cc < N2) ? __ldg(inv_c + cc) : 0.f);
            r[2 * q] = __float_as_uint(__uint_as_float(r[2 * q]) * sc);
            r[2 * q + 1] = __float_as_uint(__uint_as_float(r[2 * q + 1]) * sc);
          }
        }
        if constexpr (EPI == 1) {
          epi_chunk_lsu(r, stage_gen, lane, Cp, ldcf, row0, col0, M, N2, accumulate);
          continue;
        }
        const int buf = nstores & 1;
        if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        __syncwarp();
        // row = lane of a 32 x 32 tile in the 128-byte swizzled layout of the
        // C tensor map: 16-byte chunk c of row l sits at chunk c ^ (l & 7)
        float4* st = reinterpret_cast<float4*>(stage_gen + buf * 1024) + lane * 8;
#pragma unroll
        for (int c4 = 0; c4 < 8; ++c4)
          st[c4 ^ (lane & 7)] = make_float4(__uint_as_float(r[4 * c4]), __uint_as_float(r[4 * c4 + 1]),
                                            __uint_as_float(r[4 * c4 + 2]), __uint_as_float(r[4 * c4 + 3]));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          const uint32_t src = stage0 + (uint32_t)buf * 4096u;
          if (accumulate)
            asm volatile(
                "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.bulk_group [%0, {%1, %2}], [%3];"
                ::"l"((unsigned long long)&mapC), "r"(col0), "r"(row0), "r"(src)
                : "memory");
          else
            asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];"
                         ::"l"((unsigned long long)&mapC), "r"(col0), "r"(row0), "r"(src)
                         : "memory");
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
        ++nstores;
      }
      // this accumulator has been read: the MMA warp may overwrite it
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce0 + 8 * b);
    }
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    __syncwarp();
  }
  // ---------------- drain loads still in flight after an error, free TMEM
  if (warp == 0 && lane == 0 && *(volatile int*)err) {
    for (int i = issued - ST > 0 ? issued - ST : 0; i < issued; ++i) {
      const int s = i % ST;
      mbar_wait(full0 + 8 * s, (i / ST) & 1, err, 8);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_TMEM_COLS) : "memory");
  }
}

// ------------------------------------------------------------- CTA-pair kernel
// The same product with a cluster of two CTAs per 256 x 256 output tile:
// tcgen05.mma.cta_group::2 (M = 256, N = 256), issued by the even CTA, reads
// 128 rows of A and 128 rows of B' from the shared memory of each CTA, so a CTA
// streams 32 KB per K chunk for the tensor work that costs 48 KB in the
// single-CTA kernel, and 5 or 6 chunks fit in flight.  Each CTA's tensor memory
// holds its 128 rows of the tile (two 256-column accumulators, allocated for
// the pair) and its four epilogue warps store them.
// Signalling across the pair:
//   full[s]   even CTA, 1 arrival + 64 KB: the TMA copies of both CTAs complete
//             on the even CTA's barrier (cta_group::2 copies);
//   empty[s]  each CTA: MMA completion, committed to both CTAs (multicast);
//   accf[b]   each CTA: accumulator complete, committed to both CTAs;
//   acce[b]   even CTA, 8 arrivals: the epilogue warps of both CTAs;
//   tile ring the even CTA's producer takes a tile index from the counter and
//             writes it into both CTAs' slot; the consumers of both CTAs
//             release the slot on the even CTA's barrier (10 arrivals).
// Waits are bounded as in the single-CTA kernel.  Before exiting, each producer
// waits for the MMA completions of its last stages (so that no commit arrives in
// shared memory of an exited CTA), and both CTAs meet at a cluster barrier.
constexpr int TP_ROWS = 128;                          // A and B' rows per CTA and K chunk
constexpr int TP_A_BYTES = TP_ROWS * TC_BK * 4;       // 16 KB
constexpr int TP_B_BYTES = TP_ROWS * TC_BK * 4;       // 16 KB
constexpr int TP_STAGE_BYTES = TP_A_BYTES + TP_B_BYTES;
constexpr int TP_TILE = 2 * TP_ROWS;
constexpr uint32_t TP_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TP_TILE >> 3) << 17) |
                              ((uint32_t)(TP_TILE >> 4) << 24);
constexpr int tp_psmem(int stages, int nbuf) { return stages * TP_STAGE_BYTES + TC_EPI_WARPS * nbuf * 4096 + 1024; }
static_assert(tp_psmem(6, 2) <= 232448 && tp_psmem(5, 4) <= 232448, "pair kernel shared memory");

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// shared::cluster address of the same shared-memory offset in CTA `rank`
__device__ __forceinline__ uint32_t mapa_rank(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t caddr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(caddr) : "memory");
}
__device__ __forceinline__ void st_cluster_u32(uint32_t caddr, uint32_t v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(caddr), "r"(v) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cl(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait on a barrier that receives arrivals from the other CTA
__device__ __forceinline__ bool mbar_wait_cl(uint32_t bar, uint32_t parity, int* err, int code) {
  if (mbar_try_wait_cl(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (true) {
    if (mbar_try_wait_cl(bar, parity)) return true;
    if (gtimer() - t0 > TC_WAIT_NS) {
      atomicOr(err, code);
      return false;
    }
  }
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// TMA copy into this CTA's shared memory, completing on the even CTA's barrier
__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap* map, uint32_t cbar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(dst), "l"((unsigned long long)map), "r"(cbar), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void mma_tf32_pair(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(dtmem), "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// arrive on the barrier at this offset in both CTAs when the MMAs issued so far complete
__device__ __forceinline__ void mma_commit_pair(uint32_t bar) {
  const uint16_t mask = 3;
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
               ::"r"(bar), "h"(mask)
               : "memory");
}

template <int ST, int NB, int EPI>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(TC_THREADS, 1)
    k_tc_gemm_pair(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   const __grid_constant__ CUtensorMap mapC, const __grid_constant__ CUtensorMap mapP,
                   float* __restrict__ Cp, long long ldcf, int M, int N2, int K2, int accumulate,
                   int* tile_ctr, int* err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long bars[2 * ST + 4 + 2 * TC_TQ];
  __shared__ int tq[TC_TQ];
  __shared__ uint32_t tmem_slot;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t crank = cluster_rank();
  const bool lead = crank == 0;
  const int KT = (K2 + TC_BK - 1) / TC_BK;
  const int MT = (M + TP_TILE - 1) / TP_TILE, NT = (N2 + TP_TILE - 1) / TP_TILE;
  const int ntiles = MT * NT;
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[ST]);
  const uint32_t accf0 = smem_u32(&bars[2 * ST]), acce0 = smem_u32(&bars[2 * ST + 2]);
  const uint32_t tqf0 = smem_u32(&bars[2 * ST + 4]), tqe0 = smem_u32(&bars[2 * ST + 4 + TC_TQ]);
  const uint32_t stage_base = base + ST * TP_STAGE_BYTES;
  // the even CTA's barriers, the odd CTA's ring (cluster addresses)
  const uint32_t full0_l = mapa_rank(full0, 0), acce0_l = mapa_rank(acce0, 0), tqe0_l = mapa_rank(tqe0, 0);
  const uint32_t tq_p = mapa_rank(smem_u32(&tq[0]), 1), tqf0_p = mapa_rank(tqf0, 1);

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, 2 * TC_EPI_WARPS);
    }
    for (int q = 0; q < TC_TQ; ++q) {
      mbar_init(tqf0 + 8 * q, 1);
      mbar_init(tqe0 + 8 * q, 2 + 2 * TC_EPI_WARPS);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    // one warp of each CTA allocates the pair's tensor memory collectively
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(2 * TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  cluster_sync_all();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- tile scheduler (even CTA) + TMA producer (both CTAs)
      int it = 0, issued = 0;
      int t_next = lead ? atomicAdd(tile_ctr, 1) : -1;   // one tile ahead (see the single-CTA kernel)
      for (int j = 0;; ++j) {
        const int q = j % TC_TQ;
        int t;
        if (lead) {
          if (j >= TC_TQ && !mbar_wait_cl(tqe0 + 8 * q, ((j / TC_TQ) - 1) & 1, err, 16)) break;
          t = *(volatile int*)err ? -1 : t_next;
          if (t >= ntiles) t = -1;
          if (t >= 0) t_next = atomicAdd(tile_ctr, 1);
          tq[q] = t;
          st_cluster_u32(tq_p + 4 * q, (uint32_t)t);
          mbar_arrive(tqf0 + 8 * q);
          mbar_arrive_cluster(tqf0_p + 8 * q);
        } else {
          if (!mbar_wait_cl(tqf0 + 8 * q, (j / TC_TQ) & 1, err, 16)) break;
          t = *(volatile int*)&tq[q];
          mbar_arrive_cluster(tqe0_l + 8 * q);
        }
        if (t < 0) break;
        const int m0 = (t % MT) * TP_TILE + (int)crank * TP_ROWS;
        const int n0 = (t / MT) * TP_TILE + (int)crank * TP_ROWS;
        if (accumulate) tma_prefetch_2d(&mapP, (t / MT) * TP_TILE, m0);
        bool ok = true;
        for (int kt = 0; kt < KT; ++kt, ++it) {
          const int s = it % ST;
          if (it >= ST && !mbar_wait(empty0 + 8 * s, ((it / ST) - 1) & 1, err, 1)) { ok = false; break; }
          const uint32_t sa = base + s * TP_STAGE_BYTES, sb = sa + TP_A_BYTES;
          if (lead) mbar_expect_tx(full0 + 8 * s, 2 * TP_STAGE_BYTES);
          tma_load_2d_pair(sa, &mapA, full0_l + 8 * s, kt * TC_BK, m0);
          tma_load_2d_pair(sb, &mapB, full0_l + 8 * s, kt * TC_BK, n0);
          issued = it + 1;
        }
        if (!ok) {
          if (lead) {
            // hand out an end marker in the next slot so that the other roles stop
            const int j2 = j + 1, q2 = j2 % TC_TQ;
            if (j2 < TC_TQ || mbar_wait_cl(tqe0 + 8 * q2, ((j2 / TC_TQ) - 1) & 1, err, 16)) {
              tq[q2] = -1;
              st_cluster_u32(tq_p + 4 * q2, 0xffffffffu);
              mbar_arrive(tqf0 + 8 * q2);
              mbar_arrive_cluster(tqf0_p + 8 * q2);
            }
          }
          break;
        }
      }
      if (!*(volatile int*)err) {
        for (int i = issued - ST > 0 ? issued - ST : 0; i < issued; ++i)
          mbar_wait(empty0 + 8 * (i % ST), (i / ST) & 1, err, 8);
      } else {
        // copies may still be in flight towards a barrier that never completes:
        // give them time to land before the shared memory is released
        const unsigned long long t0 = gtimer();
        while (gtimer() - t0 < 200000ull) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && lead) {
      // ---------------- MMA issuer (even CTA)
      int it = 0;
      for (int j = 0;; ++j) {
        const int q = j % TC_TQ;
        if (!mbar_wait(tqf0 + 8 * q, (j / TC_TQ) & 1, err, 32)) break;
        const int t = *(volatile int*)&tq[q];
        mbar_arrive(tqe0 + 8 * q);
        if (t < 0) break;
        const int b = j & 1;
        if (j >= 2 && !mbar_wait_cl(acce0 + 8 * b, ((j >> 1) - 1) & 1, err, 64)) break;
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)(b * TC_TMEM_COLS);
        bool ok = true;
        for (int kt = 0; kt < KT; ++kt, ++it) {
          const int s = it % ST;
          if (!mbar_wait(full0 + 8 * s, (it / ST) & 1, err, 2)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sa = base + s * TP_STAGE_BYTES, sb = sa + TP_A_BYTES;
          const uint64_t da = desc_sw128(sa), db = desc_sw128(sb);
#pragma unroll
          for (int kk = 0; kk < TC_BK / 8; ++kk)
            mma_tf32_pair(dt, da + 2 * kk, db + 2 * kk, TP_IDESC, (kt > 0 || kk > 0) ? 1u : 0u);
          mma_commit_pair(empty0 + 8 * s);
        }
        if (!ok) break;
        mma_commit_pair(accf0 + 8 * b);
      }
    }
  } else {
    // ---------------- epilogue warps (both CTAs): TMEM lane quarter = 32 rows
    const int ew = warp - 2;
    const int quarter = warp & 3;
    const uint32_t stage0 = stage_base + (uint32_t)ew * (uint32_t)NB * 4096u;
    float* stage_gen = reinterpret_cast<float*>(smem_raw + (stage_base - smem_u32(smem_raw))) + ew * NB * 1024;
    int nstores = 0;
    for (int j = 0;; ++j) {
      const int q = j % TC_TQ;
      int t = -1;
      const bool okq = __all_sync(0xffffffffu, mbar_wait_cl(tqf0 + 8 * q, (j / TC_TQ) & 1, err, 128) ? 1 : 0) != 0;
      if (okq) t = *(volatile int*)&tq[q];
      __syncwarp();
      if (lane == 0 && okq) {
        if (lead) mbar_arrive(tqe0 + 8 * q);
        else mbar_arrive_cluster(tqe0_l + 8 * q);
      }
      if (!okq || t < 0) break;
      const int b = j & 1;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(accf0 + 8 * b, (j >> 1) & 1, err, 4) ? 1 : 0) != 0;
      if (!ok) break;
      tc_fence_after();
      const int m0 = (t % MT) * TP_TILE + (int)crank * TP_ROWS, n0 = (t / MT) * TP_TILE;
      const int row0 = m0 + quarter * 32;
      for (int c = 0; c < TP_TILE / 32; ++c) {
        const int col0 = n0 + c * 32;
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * TC_TMEM_COLS + c * 32), r);
        if constexpr (EPI == 1) {
          if (c == TP_TILE / 32 - 1) {
            // the accumulator has been read: the MMA warp may overwrite it
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
              if (lead) mbar_arrive(acce0 + 8 * b);
              else mbar_arrive_cluster(acce0_l + 8 * b);
            }
          }
          if (col0 >= N2 || row0 >= M) continue;          // warp-uniform
          epi_chunk_lsu(r, stage_gen, lane, Cp, ldcf, row0, col0, M, N2, accumulate);
          continue;
        }
        if (col0 >= N2 || row0 >= M) continue;            // warp-uniform
        const int buf = nstores % NB;
        if (lane == 0) asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(NB - 1) : "memory");
        __syncwarp();
        float4* st = reinterpret_cast<float4*>(stage_gen + buf * 1024) + lane * 8;
#pragma unroll
        for (int c4 = 0; c4 < 8; ++c4)
          st[c4 ^ (lane & 7)] = make_float4(__uint_as_float(r[4 * c4]), __uint_as_float(r[4 * c4 + 1]),
                                            __uint_as_float(r[4 * c4 + 2]), __uint_as_float(r[4 * c4 + 3]));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          const uint32_t src = stage0 + (uint32_t)buf * 4096u;
          if (accumulate)
            asm volatile(
                "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.bulk_group [%0, {%1, %2}], [%3];"
                ::"l"((unsigned long long)&mapC), "r"(col0), "r"(row0), "r"(src)
                : "memory");
          else
            asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];"
                         ::"l"((unsigned long long)&mapC), "r"(col0), "r"(row0), "r"(src)
                         : "memory");
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
        ++nstores;
      }
      if constexpr (EPI == 0) {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          if (lead) mbar_arrive(acce0 + 8 * b);
          else mbar_arrive_cluster(acce0_l + 8 * b);
        }
      }
    }
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  __syncwarp();
  tc_fence_before();
  cluster_sync_all();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_TMEM_COLS) : "memory");
  }
}

// B'[2N][K2p] from alpha * B (B: K x N complex, row-major ldb), tf32-rounded,
// zero-padded for 2K <= k < K2p.
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
__global__ void k_expand_b(int K, int N, float2 alpha, const float2* __restrict__ B, int64_t ldb, float* __restrict__ Bp,
                           int K2p, int bz0, int bz1) {
  __shared__ float2 tile[32][33];
  const int l0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    int l = l0 + r, j = j0 + tx;
    float2 v = make_float2(0.f, 0.f);
    if (l < K && j < N && (j < bz0 || j >= bz1)) {
      float2 b = B[(int64_t)l * ldb + j];
      v = make_float2(alpha.x * b.x - alpha.y * b.y, alpha.x * b.y + alpha.y * b.x);
    }
    tile[r][tx] = v;
  }
  __syncthreads();
  // write: rows 2j, 2j+1; columns 2l, 2l+1 (coalesced along l)
  for (int r = ty; r < 32; r += 8) {
    int j = j0 + r, l = l0 + tx;
    if (j >= N) continue;
    float2 v = tile[tx][r];
    float re = to_tf32(v.x), im = to_tf32(v.y);
    if (l < K) {
      float2* r0 = reinterpret_cast<float2*>(Bp + (int64_t)(2 * j) * K2p) + l;
      float2* r1 = reinterpret_cast<float2*>(Bp + (int64_t)(2 * j + 1) * K2p) + l;
      *r0 = make_float2(re, -im);
      *r1 = make_float2(im, re);
    } else if (2 * l < K2p) {
      float2* r0 = reinterpret_cast<float2*>(Bp + (int64_t)(2 * j) * K2p) + l;
      float2* r1 = reinterpret_cast<float2*>(Bp + (int64_t)(2 * j + 1) * K2p) + l;
      *r0 = make_float2(0.f, 0.f);
      *r1 = make_float2(0.f, 0.f);
    }
  }
}

// ------------------------------------------------ FP16 operands with scaling
// A power of two s with s * mx in [2^14, 2^15) (1 for mx = 0): FP16's largest
// finite value is 65504, so every scaled entry is representable, and the
// scaling is exact.
__device__ __forceinline__ float pow2_scale(float mx) {
  if (!(mx > 0.f) || !isfinite(mx)) return 1.f;
  return ldexpf(1.f, 14 - ilogbf(mx));
}

// A16[i][0 .. K2p) = fp16(s_i A_r[i][k]) for k < 2K (A_r: the complex64 row read as
// floats), zero beyond; inv_r[i] = 1 / s_i with s_i from the row's largest entry.
// One warp per row.
__global__ void k_a_to_f16(const float2* __restrict__ A, int64_t lda, int M, int K, __half* __restrict__ A16,
                           int K2p, float* __restrict__ inv_r) {
  const int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= M) return;
  const float* a = reinterpret_cast<const float*>(A + (int64_t)row * lda);
  float mx = 0.f;
  for (int k = lane; k < 2 * K; k += 32) mx = fmaxf(mx, fabsf(a[k]));
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const float sc = pow2_scale(mx);
  if (lane == 0) inv_r[row] = 1.f / sc;
  __half* dst = A16 + (int64_t)row * K2p;
  for (int k = lane; k < K2p; k += 32) dst[k] = __float2half_rn(k < 2 * K ? a[k] * sc : 0.f);
}

// per complex column j of alpha * B (K x N, row stride ldb): the largest real
// or imaginary part, as the bits of a non-negative float (colmax zeroed
// beforehand); columns [bz0, bz1) stay zero.  CTA (32 x 8 threads) = 32
// columns x 128 rows of B.
__global__ void k_b_colmax(const float2* __restrict__ B, int64_t ldb, int K, int N, float2 alpha, int bz0, int bz1,
                           unsigned* __restrict__ colmax) {
  __shared__ float red[8][32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int j = blockIdx.x * 32 + tx, l0 = blockIdx.y * 128;
  float mx = 0.f;
  if (j < N && (j < bz0 || j >= bz1)) {
    for (int l = l0 + ty; l < min(K, l0 + 128); l += 8) {
      const float2 b = B[(int64_t)l * ldb + j];
      const float vr = alpha.x * b.x - alpha.y * b.y, vi = alpha.x * b.y + alpha.y * b.x;
      mx = fmaxf(mx, fmaxf(fabsf(vr), fabsf(vi)));
    }
  }
  red[ty][tx] = mx;
  __syncthreads();
  if (ty == 0 && j < N) {
    for (int r = 1; r < 8; ++r) mx = fmaxf(mx, red[r][tx]);
    if (mx > 0.f) atomicMax(colmax + j, __float_as_uint(mx));
  }
}

// B'[2N][K2p] in FP16 from c_j alpha B (c_j from colmax), the same real layout
// as k_expand_b; the CTAs of the first row of tiles write inv_c
__global__ void k_expand_b16(int K, int N, float2 alpha, const float2* __restrict__ B, int64_t ldb,
                             __half* __restrict__ Bp, int K2p, int bz0, int bz1, const unsigned* __restrict__ colmax,
                             float* __restrict__ inv_c) {
  __shared__ float2 tile[32][33];
  const int l0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
  {
    const int j = j0 + tx;
    if (blockIdx.y == 0 && ty == 0 && j < N) inv_c[j] = 1.f / pow2_scale(__uint_as_float(colmax[j]));
  }
  for (int r = ty; r < 32; r += 8) {
    const int l = l0 + r, j = j0 + tx;
    float2 v = make_float2(0.f, 0.f);
    if (l < K && j < N && (j < bz0 || j >= bz1)) {
      const float2 b = B[(int64_t)l * ldb + j];
      const float s = pow2_scale(__uint_as_float(colmax[j]));
      v = make_float2((alpha.x * b.x - alpha.y * b.y) * s, (alpha.x * b.y + alpha.y * b.x) * s);
    }
    tile[r][tx] = v;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int j = j0 + r, l = l0 + tx;
    if (j >= N || 2 * l >= K2p) continue;
    const float2 v = tile[tx][r];
    __half2* r0 = reinterpret_cast<__half2*>(Bp + (int64_t)(2 * j) * K2p) + l;
    __half2* r1 = reinterpret_cast<__half2*>(Bp + (int64_t)(2 * j + 1) * K2p) + l;
    if (l < K) {
      *r0 = __floats2half2_rn(v.x, -v.y);
      *r1 = __floats2half2_rn(v.y, v.x);
    } else {
      *r0 = __floats2half2_rn(0.f, 0.f);
      *r1 = __floats2half2_rn(0.f, 0.f);
    }
  }
}

// ------------------------------------------------------------------ host
static PFN_cuTensorMapEncodeTiled_v12000 get_encode(TcGemmCtx& c) {
  if (!c.encode_fn) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      c.encode_fn = fn;
    else
      cudaGetLastError();
  }
  return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(c.encode_fn);
}

static bool make_map(PFN_cuTensorMapEncodeTiled_v12000 enc, CUtensorMap* map, const void* ptr, uint64_t inner,
                     uint64_t rows, uint64_t row_bytes, uint32_t box_rows, bool swizzle = true,
                     uint32_t box_inner = TC_BK, bool f16 = false) {
  cuuint64_t dims[2] = {inner, rows};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {box_inner, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                   const_cast<void*>(ptr), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

bool tc_gemm_eligible(TcGemmCtx& c, int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                      const void* C, int64_t ldc, float2 beta) {
  if (!c.checked) {
    c.checked = true;
    int dev = 0, major = 0, minor = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    c.usable = (major == 10 && minor == 3) && get_encode(c) != nullptr &&
               cudaFuncSetAttribute(k_tc_gemm<3, 0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_psmem(3)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm<4, 0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_psmem(4)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm<3, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_psmem(3)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm<4, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_psmem(4)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm<3, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_psmem(3)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm<4, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_psmem(4)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm<3, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_psmem(3)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm<4, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_psmem(4)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm_pair<5, 4, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, tp_psmem(5, 4)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm_pair<6, 2, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, tp_psmem(6, 2)) == cudaSuccess &&
               cudaFuncSetAttribute(k_tc_gemm_pair<6, 2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tp_psmem(6, 2)) == cudaSuccess &&
               cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess;
    if (!c.usable) cudaGetLastError();
    const char* env = getenv("MNPBEM_TC_STAGES");
    if (env && (env[0] == '3' || env[0] == '4')) c.stages = env[0] - '0';
    if (c.stages != 3 && c.stages != 4) c.stages = 4;
    const char* penv = getenv("MNPBEM_TC_PAIR");
    if (penv && (penv[0] == '0' || penv[0] == '1')) c.pair = penv[0] - '0';
  }
  if (!c.usable || !c.enabled) return false;
  if ((lda & 1) || (ldc & 1) || (reinterpret_cast<uintptr_t>(A) & 15) ||
      (reinterpret_cast<uintptr_t>(C) & 15) || beta.y != 0.0f || (beta.x != 0.0f && beta.x != 1.0f))
    return false;
  return M >= 128 && N >= 64 && K >= 16 && M < (1 << 30) && 2 * N < (1 << 30) && 2 * K < (1 << 30);
}

// The product with FP16 operands: A converted row by row and B' column by
// column into FP16 with power-of-two scales (k_a_to_f16, k_b_colscale,
// k_expand_b16), kind::f16 MMAs with FP32 accumulation, the scales undone in
// the epilogue.  FP16 keeps TF32's 10-bit significand and issues at twice the
// TF32 rate with half the operand bytes per multiply-add.
static mnpbem_status tc_gemm_f16(TcGemmCtx& c, int64_t M, int64_t N, int64_t K, float2 alpha, const float2* A,
                                 int64_t lda, const float2* B, int64_t ldb, float2 beta, float2* C, int64_t ldc,
                                 cudaStream_t st, int64_t bz0, int64_t bz1) {
  constexpr int BK = 64;
  const int64_t K2 = 2 * K, N2 = 2 * N, K2p = round_up(K2, BK);
  MNP_TRY(c.bexp.ensure(sizeof(__half) * N2 * K2p));
  MNP_TRY(c.a16.ensure(sizeof(__half) * M * K2p));
  MNP_TRY(c.scales.ensure(sizeof(float) * (M + 2 * N)));
  MNP_TRY(c.err.ensure(sizeof(int)));
  __half* Bp = c.bexp.as<__half>();
  __half* A16 = c.a16.as<__half>();
  float* inv_r = c.scales.as<float>();
  unsigned* colmax = reinterpret_cast<unsigned*>(inv_r + M);
  float* inv_c = inv_r + M + N;
  {
    ProfScope ps(PH_ELEMWISE, st, 0.0, 16.0 * K * N + 8.0 * M * K + 4.0 * M * K + 8.0 * N * K);
    MNP_CUDA(cudaMemsetAsync(colmax, 0, sizeof(unsigned) * N, st));
    k_a_to_f16<<<(unsigned)cdiv_up(M, (int64_t)8), 256, 0, st>>>(A, lda, (int)M, (int)K, A16, (int)K2p, inv_r);
    k_b_colmax<<<dim3((unsigned)cdiv_up(N, 32), (unsigned)cdiv_up(K, 128)), dim3(32, 8), 0, st>>>(
        B, ldb, (int)K, (int)N, alpha, (int)bz0, (int)bz1, colmax);
    dim3 g((unsigned)cdiv_up(N, 32), (unsigned)cdiv_up(K2p / 2, 32));
    k_expand_b16<<<g, dim3(32, 8), 0, st>>>((int)K, (int)N, alpha, B, ldb, Bp, (int)K2p, (int)bz0, (int)bz1, colmax,
                                            inv_c);
    MNP_CHECK_LAUNCH();
  }
  auto enc = get_encode(c);
  CUtensorMap ma, mb, mc, mp;
  if (!make_map(enc, &ma, A16, (uint64_t)K2p, (uint64_t)M, (uint64_t)K2p * 2, TC_BM, true, BK, true) ||
      !make_map(enc, &mb, Bp, (uint64_t)K2p, (uint64_t)N2, (uint64_t)K2p * 2, TC_BN, true, BK, true) ||
      !make_map(enc, &mc, C, (uint64_t)N2, (uint64_t)M, (uint64_t)ldc * 8, 32, true) ||
      !make_map(enc, &mp, C, (uint64_t)N2, (uint64_t)M, (uint64_t)ldc * 8, TC_BM, false, TC_BN)) {
    set_error("cuTensorMapEncodeTiled failed");
    return MNPBEM_ERR_CUDA;
  }
  if (!c.err_cleared) {
    MNP_CUDA(cudaMemsetAsync(c.err.ptr, 0, sizeof(int), st));
    c.err_cleared = true;
  }
  const int64_t MT = cdiv_up(M, TC_BM), NT = cdiv_up(N2, TC_BN);
  if (MT * NT >= (1ll << 31)) { set_error("tc_gemm_c64: too many tiles"); return MNPBEM_ERR_INVALID_ARG; }
  MNP_TRY(c.ctr.ensure(sizeof(int)));
  MNP_CUDA(cudaMemsetAsync(c.ctr.ptr, 0, sizeof(int), st));
  const bool lsu = c.pair_epi == 1 || (N2 & 3) != 0;
  float* Cf = reinterpret_cast<float*>(C);
  const long long ldcf = 2ll * ldc;
  const int acc = beta.x != 0.0f ? 1 : 0;
  int ctas = c.num_sms > 0 ? c.num_sms : 148;
  if (c.max_ctas > 0 && c.max_ctas < ctas) ctas = c.max_ctas;
  ProfScope ps(M >= 128 && N >= 128 ? PH_GEMM_BIG : PH_GEMM_SMALL, st, 8.0 * M * N * K,
               8.0 * ((double)M * K + (double)K * N + 2.0 * M * N));
  const unsigned grid = (unsigned)std::min<int64_t>(MT * NT, ctas);
  auto kern = c.stages == 3 ? (lsu ? k_tc_gemm<3, 1, true> : k_tc_gemm<3, 0, true>)
                            : (lsu ? k_tc_gemm<4, 1, true> : k_tc_gemm<4, 0, true>);
  kern<<<grid, TC_THREADS, tc_psmem(c.stages == 3 ? 3 : 4), st>>>(ma, mb, mc, mp, Cf, ldcf, (int)M, (int)N2, (int)K2p,
                                                                  acc, c.ctr.as<int>(), c.err.as<int>(), inv_r, inv_c);
  MNP_CHECK_LAUNCH();
  return MNPBEM_OK;
}

mnpbem_status tc_gemm_c64(TcGemmCtx& c, int64_t M, int64_t N, int64_t K, float2 alpha, const float2* A,
                          int64_t lda, const float2* B, int64_t ldb, float2 beta, float2* C, int64_t ldc,
                          cudaStream_t st, int64_t bz0, int64_t bz1) {
  if (beta.y != 0.0f || (beta.x != 0.0f && beta.x != 1.0f) || (lda & 1) || (ldc & 1) ||
      (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(C) & 15)) {
    set_error("tc_gemm_c64: unsupported layout (odd leading dimension, misaligned base, beta not 0 or 1)");
    return MNPBEM_ERR_UNSUPPORTED;
  }
  // FP16 for the rank-512 and wider updates, where the n^3 work is; the
  // narrower panel products keep TF32 operands and skip the three conversion
  // passes (their launches dominated them at 4000 faces)
  if (c.f16 && c.pair != 1 && K >= c.f16_min_k && M >= c.f16_min_mn && N >= c.f16_min_mn)
    return tc_gemm_f16(c, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, st, bz0, bz1);
  const int64_t K2 = 2 * K, N2 = 2 * N;
  const int64_t K2p = round_up(K2, TC_BK);
  MNP_TRY(c.bexp.ensure(sizeof(float) * N2 * K2p));
  MNP_TRY(c.err.ensure(sizeof(int)));
  float* Bp = c.bexp.as<float>();
  {
    ProfScope ps(PH_ELEMWISE, st, 0.0, 8.0 * K * N + 16.0 * K * N);
    dim3 g((unsigned)cdiv_up(N, 32), (unsigned)cdiv_up(K2p / 2, 32));
    k_expand_b<<<g, dim3(32, 8), 0, st>>>((int)K, (int)N, alpha, B, ldb, Bp, (int)K2p, (int)bz0, (int)bz1);
    MNP_CHECK_LAUNCH();
  }
  auto enc = get_encode(c);
  // CTA pairs for products with at least 256 rows (the pair tile is 256 x 256)
  // measured on GB300 (complex 4000 x 4000 products): the pair kernel reaches
  // 870 TFLOP/s at K = 4000 against 745 for the single-CTA kernel, and ties or
  // trails it at K = 256 (rank updates, panel products)
  const bool pair = M >= TP_TILE && (c.pair == 1 || (c.pair < 0 && K >= 1024));
  CUtensorMap ma, mb, mc, mp;
  if (!make_map(enc, &ma, A, (uint64_t)K2, (uint64_t)M, (uint64_t)lda * 8, pair ? TP_ROWS : TC_BM) ||
      !make_map(enc, &mb, Bp, (uint64_t)K2p, (uint64_t)N2, (uint64_t)K2p * 4, pair ? TP_ROWS : TC_BN) ||
      !make_map(enc, &mc, C, (uint64_t)N2, (uint64_t)M, (uint64_t)ldc * 8, 32, true) ||
      !make_map(enc, &mp, C, (uint64_t)N2, (uint64_t)M, (uint64_t)ldc * 8, TC_BM, false, TC_BN)) {
    set_error("cuTensorMapEncodeTiled failed");
    return MNPBEM_ERR_CUDA;
  }
  if (!c.err_cleared) {
    MNP_CUDA(cudaMemsetAsync(c.err.ptr, 0, sizeof(int), st));
    c.err_cleared = true;
  }
  const int64_t MT = cdiv_up(M, pair ? TP_TILE : TC_BM), NT = cdiv_up(N2, pair ? TP_TILE : TC_BN);
  if (MT * NT >= (1ll << 31)) { set_error("tc_gemm_c64: too many tiles"); return MNPBEM_ERR_INVALID_ARG; }
  MNP_TRY(c.ctr.ensure(sizeof(int)));
  MNP_CUDA(cudaMemsetAsync(c.ctr.ptr, 0, sizeof(int), st));
  // 2N floats per row that are not a multiple of 16 bytes: vector stores, not TMA
  const bool lsu = c.pair_epi == 1 || (N2 & 3) != 0;
  float* Cf = reinterpret_cast<float*>(C);
  const long long ldcf = 2ll * ldc;
  const int acc = beta.x != 0.0f ? 1 : 0;
  int ctas = c.num_sms > 0 ? c.num_sms : 148;
  if (c.max_ctas > 0 && c.max_ctas < ctas) ctas = c.max_ctas;
  {
    ProfScope ps(M >= 128 && N >= 128 ? PH_GEMM_BIG : PH_GEMM_SMALL, st, 8.0 * M * N * K,
                 8.0 * ((double)M * K + (double)K * N + 2.0 * M * N));
    if (pair) {
      // one cluster of two CTAs per pair tile, at most one CTA per SM
      const unsigned grid = 2u * (unsigned)std::min<int64_t>(MT * NT, std::max(1, ctas / 2));
      if (c.pair_nb == 4 && !lsu)
        k_tc_gemm_pair<5, 4, 0><<<grid, TC_THREADS, tp_psmem(5, 4), st>>>(ma, mb, mc, mp, Cf, ldcf, (int)M, (int)N2,
                                                                          (int)K2, acc, c.ctr.as<int>(), c.err.as<int>());
      else if (lsu)
        k_tc_gemm_pair<6, 2, 1><<<grid, TC_THREADS, tp_psmem(6, 2), st>>>(ma, mb, mc, mp, Cf, ldcf, (int)M, (int)N2,
                                                                          (int)K2, acc, c.ctr.as<int>(), c.err.as<int>());
      else
        k_tc_gemm_pair<6, 2, 0><<<grid, TC_THREADS, tp_psmem(6, 2), st>>>(ma, mb, mc, mp, Cf, ldcf, (int)M, (int)N2,
                                                                          (int)K2, acc, c.ctr.as<int>(), c.err.as<int>());
      MNP_CHECK_LAUNCH();
      return MNPBEM_OK;
    }
    const unsigned grid = (unsigned)std::min<int64_t>(MT * NT, ctas);
    auto kern = c.stages == 3 ? (lsu ? k_tc_gemm<3, 1, false> : k_tc_gemm<3, 0, false>)
                              : (lsu ? k_tc_gemm<4, 1, false> : k_tc_gemm<4, 0, false>);
    kern<<<grid, TC_THREADS, tc_psmem(c.stages == 3 ? 3 : 4), st>>>(ma, mb, mc, mp, Cf, ldcf, (int)M, (int)N2, (int)K2,
                                                                    acc, c.ctr.as<int>(), c.err.as<int>(), nullptr,
                                                                    nullptr);
    MNP_CHECK_LAUNCH();
  }
  return MNPBEM_OK;
}

mnpbem_status tc_check_error(TcGemmCtx& c, cudaStream_t st) {
  if (!c.err.ptr || !c.err_cleared) return MNPBEM_OK;
  int h = 0;
  MNP_CUDA(cudaMemcpyAsync(&h, c.err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  MNP_CUDA(cudaStreamSynchronize(st));
  c.err_cleared = false;
  if (h) {
    set_error("tensor-core GEMM: a bounded pipeline wait expired (code %d)", h);
    c.enabled = false;
    return MNPBEM_ERR_TIMEOUT;
  }
  return MNPBEM_OK;
}

// ---------------------------------------------------- bounded-wait self test
// One CTA waits on an mbarrier that nothing arrives at, through the same
// bounded-wait helper as the pipelines above but with a short limit: the wait
// expires, the error word records the code and the kernel returns, leaving
// the context usable.  Tests check that the host then sees MNPBEM_ERR_TIMEOUT.
__global__ void k_wait_selftest(int* err, unsigned long long limit_ns) {
  __shared__ __align__(8) unsigned long long bar;
  const uint32_t b = smem_u32(&bar);
  if (threadIdx.x == 0) {
    mbar_init(b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait_ns(b, 0, err, 32, limit_ns);   // phase 0 never completes
  __syncthreads();
}

void tc_release(TcGemmCtx& c) {
  c.bexp.release();
  c.a16.release();
  c.scales.release();
  c.err.release();
  c.ctr.release();
}

}  // namespace mnpbem

extern "C" mnpbem_status mnpbem_selftest_bounded_wait(int32_t device, int32_t limit_us) {
  using namespace mnpbem;
  if (limit_us < 1 || limit_us > 1000000) {
    set_error("mnpbem_selftest_bounded_wait: limit must be 1 us .. 1 s");
    return MNPBEM_ERR_INVALID_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess) cudaGetLastError();
  if (device < 0 || device >= ndev) {
    set_error("mnpbem_selftest_bounded_wait: invalid device %d", (int)device);
    return MNPBEM_ERR_INVALID_ARG;
  }
  MNP_CUDA(cudaSetDevice(device));
  DevBuf err;
  MNP_TRY(err.ensure(sizeof(int)));
  MNP_CUDA(cudaMemset(err.ptr, 0, sizeof(int)));
  k_wait_selftest<<<1, 32>>>(err.as<int>(), 1000ull * (unsigned long long)limit_us);
  MNP_CHECK_LAUNCH();
  int h = 0;
  MNP_CUDA(cudaMemcpy(&h, err.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    set_error("bounded wait self test: the wait expired after %d us (code %d)", (int)limit_us, h);
    return MNPBEM_ERR_TIMEOUT;
  }
  return MNPBEM_OK;
}
