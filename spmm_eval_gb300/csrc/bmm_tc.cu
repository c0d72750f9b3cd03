// Dense binary matmul on the 5th-generation tensor cores (tcgen05).
//
// and(r, c) = sum_k a_rk b_ck with a, b in {0, 1} is an ordinary GEMM of 0/1
// matrices.  The bits of the reference's word-major operands (ToBit32ColUd
// layout, spmm.cu:93-111) are expanded to FP8 e4m3 bytes (0x38 = 1.0,
// 0x00 = 0.0), K-major and zero-padded to a multiple of 128, and multiplied
// with tcgen05.mma.kind::f8f6f4 into FP32 accumulators in tensor memory.
// Every product is 0 or 1 and every partial sum an integer <= K < 2^24, so
// the FP32 accumulation is exact; XOR counts come from row popcounts as
// popc(a) + popc(b) - 2 and(a, b).
//
// Two launch forms share the tile machinery.  k_bmm_tc: one 128-thread
// CTA per 128 x 256 output tile.  Thread 0 of warp 0 streams 128-byte K
// slices of A (128 rows) and B (256 rows) into a 4-stage shared-memory ring
// with TMA (cp.async.bulk.tensor, 128B swizzle, mbarrier complete_tx);
// thread 0 of warp 1 issues four K=32 MMAs per slice (tcgen05.mma,
// cta_group::1, M=128, N=256) and releases each slot with tcgen05.commit;
// after the last slice all four warps read their 32 TMEM lanes (= output
// rows) with tcgen05.ld and write int32 C.  k_bmm_tc_persist (the default):
// the same roles in a persistent warp-specialised CTA per SM with two TMEM
// accumulators.  Every mbarrier wait is bounded: on timeout the
// kernel records an error flag, skips the remaining work, frees its tensor
// memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"
#include "util.cuh"

namespace gbs {

constexpr int TC_BM = 128, TC_BN = 256, TC_BK = 128, TC_STAGES = 4;
constexpr int TC_A_BYTES = TC_BM * TC_BK;  // 16 KiB per stage
constexpr int TC_B_BYTES = TC_BN * TC_BK;  // 32 KiB per stage
constexpr int TC_SMEM = TC_STAGES * (TC_A_BYTES + TC_B_BYTES) + 1024 + 256;  // ring + barriers
constexpr uint32_t TC_WAIT_LIMIT = 1u << 22;

// kind::f8f6f4 instruction descriptor: D = F32 (bits 4-5 = 1), A = B = E4M3
// (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
constexpr uint32_t TC_IDESC = (1u << 4) | ((uint32_t)(TC_BN >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);

struct BmmTcArgs {
  int M, N, Kw, Kp;
  int mode;
  const int *pa;
  const int *pb;
  int32_t *C;
  float *Cf;
  int ldc;
  int *err;
  // sign-word output (instead of C / Cf): bit = (nbits - 2 xor >= 0), 32
  // columns per word, first column in bit 31; layout 0 = BMM32_BIN
  // (Cbits[(c / 32) * M + r]), 1 = BMM32S_BIN (Cbits[(r / 32) * N * 32 +
  // c / 32 * 32 + r % 32]); M, N multiples of 32
  uint32_t *Cbits;
  int bin_layout;
  int nbits;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait; false (and the error flag set) when the phase never completes.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err) {
  for (uint32_t i = 0; i < TC_WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(err, 1);
  return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor, K-major operand with 128-byte swizzle:
// start address >> 4 (bits 0-13), leading offset 16 B (unused for this
// layout), stride 1024 B between 8-row groups (bits 32-45), version 1
// (bits 46-47), swizzle mode 2 = 128B (bits 61-63).  Tile bases are
// 1024-byte aligned, so the base-offset field stays 0.
__device__ __forceinline__ uint64_t sdesc_k_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void mma_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Epilogue of one 128 x 256 tile held in TMEM accumulator b: warp quarter
// q4 reads its 32 lanes (= rows m0 + 32 q4 + lane) 32 columns at a time and
// writes the counts (int32 or float C), or -- with Cbits -- thresholds the
// 32 XOR counts a lane holds for its row into one sign word (the lane owns
// the whole word, so no shuffle or ballot) and writes only the words: 1/32
// of the int32 count matrix, and no second pass over it.
__device__ __forceinline__ void epilogue_tile(const BmmTcArgs &a, uint32_t tmem, int b, int q4, int lane, int m0,
                                              int n0) {
  const int Kbits = 32 * a.Kw;
  const int row = m0 + q4 * 32 + lane;
  const int par = (a.mode != 1 && row < a.M) ? __ldg(a.pa + row) : 0;
#pragma unroll 1
  for (int cb = 0; cb < TC_BN / 32; ++cb) {
    uint32_t v[32];
    tmem_ld32(tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(b * TC_BN + cb * 32), v);
    const int c0 = n0 + cb * 32;
    if (a.Cbits) {
      if (row < a.M && c0 < a.N) {
        uint32_t word = 0;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int andc = (int)__uint_as_float(v[q]);
          const int xr = par + __ldg(a.pb + c0 + q) - 2 * andc;
          word = (word << 1) | (a.nbits - 2 * xr >= 0 ? 1u : 0u);
        }
        if (a.bin_layout == 0) a.Cbits[(size_t)(c0 >> 5) * a.M + row] = word;
        else a.Cbits[(size_t)(row >> 5) * a.N * 32 + (size_t)c0 + (row & 31)] = word;
      }
      continue;
    }
    if (row < a.M) {
#pragma unroll
      for (int q = 0; q < 32; q += 4) {
        const int c = c0 + q;
        if (c >= a.N) break;
        int x[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int andc = (int)__uint_as_float(v[q + e]);
          int val = andc;
          if (a.mode != 1) {
            const int xr = par + __ldg(a.pb + c + e) - 2 * andc;
            val = a.mode == 0 ? xr : Kbits - 2 * xr;
          }
          x[e] = val;
        }
        if (a.Cf)
          *reinterpret_cast<float4 *>(a.Cf + (size_t)row * a.ldc + c) =
              make_float4((float)x[0], (float)x[1], (float)x[2], (float)x[3]);
        else
          *reinterpret_cast<int4 *>(a.C + (size_t)row * a.ldc + c) = make_int4(x[0], x[1], x[2], x[3]);
      }
    }
  }
}

__global__ void __launch_bounds__(128, 1)
    k_bmm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, BmmTcArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *sA = base;
  uint8_t *sB = base + TC_STAGES * TC_A_BYTES;
  uint64_t *full = reinterpret_cast<uint64_t *>(sB + TC_STAGES * TC_B_BYTES);
  uint64_t *empty = full + TC_STAGES;
  uint64_t *accf = empty + TC_STAGES;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accf + 1);
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_BN;
  const int nk = a.Kp / TC_BK;

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    mbar_init(accf, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"((uint32_t)TC_BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer: K slices of A and B into the ring
    int issued = 0;
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % TC_STAGES, r = kb / TC_STAGES;
      if (kb >= TC_STAGES && !mbar_wait(empty + s, (uint32_t)((r - 1) & 1), a.err)) {
        s_fail = 1;
        break;
      }
      mbar_expect_tx(full + s, TC_A_BYTES + TC_B_BYTES);
      tma_load_2d(sA + s * TC_A_BYTES, &tmA, kb * TC_BK, m0, full + s);
      tma_load_2d(sB + s * TC_B_BYTES, &tmB, kb * TC_BK, n0, full + s);
      issued = kb + 1;
    }
    if (s_fail) {  // let the copies already in flight land before leaving
      for (int kb = issued - TC_STAGES < 0 ? 0 : issued - TC_STAGES; kb < issued; ++kb)
        mbar_wait(full + kb % TC_STAGES, (uint32_t)((kb / TC_STAGES) & 1), a.err);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = true;
    for (int kb = 0; kb < nk && ok; ++kb) {
      const int s = kb % TC_STAGES, r = kb / TC_STAGES;
      if (!mbar_wait(full + s, (uint32_t)(r & 1), a.err)) {
        ok = false;
        s_fail = 1;
        break;
      }
      tc_fence_after();
      const uint64_t ad = sdesc_k_sw128(smem_u32(sA + s * TC_A_BYTES));
      const uint64_t bd = sdesc_k_sw128(smem_u32(sB + s * TC_B_BYTES));
#pragma unroll
      for (int k = 0; k < TC_BK / 32; ++k)  // K = 32 bytes per MMA; +32 B = +2 in the address field
        mma_f8(tmem, ad + 2 * k, bd + 2 * k, TC_IDESC, (kb | k) != 0 ? 1u : 0u);
      mma_commit(empty + s);
    }
    mma_commit(accf);
  }
  __syncwarp();

  // epilogue: warp w owns TMEM lanes (= tile rows) 32w .. 32w + 31; lane 0
  // waits and decides for the warp (the TMEM loads need a converged warp)
  int have = 0;
  if (lane == 0) have = mbar_wait(accf, 0, a.err) && !s_fail;
  have = __shfl_sync(0xffffffffu, have, 0);
  tc_fence_after();
  if (have) epilogue_tile(a, tmem, 0, warp, lane, m0, n0);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)TC_BN)
                 : "memory");
  }
}

// Grouped tile order of the persistent kernel: tiles run in groups of
// TC_GROUP_M tile rows, down the group's rows first and across N second, so
// the CTAs resident at any moment share a few A row-blocks and a few B
// column-blocks; both stay in L2 across consecutive tiles instead of all of
// B being re-read from DRAM for every wave of tiles.
constexpr int TC_GROUP_M = 16;
__device__ __forceinline__ void tile_origin(int t, int tiles_m, int tiles_n, int *m0, int *n0) {
  const int per_group = TC_GROUP_M * tiles_n;
  const int grp = t / per_group, first = grp * TC_GROUP_M;
  const int gm = tiles_m - first < TC_GROUP_M ? tiles_m - first : TC_GROUP_M;
  const int local = t - grp * per_group;
  *m0 = (first + local % gm) * TC_BM;
  *n0 = (local / gm) * TC_BN;
}

// Persistent, warp-specialised version: one CTA per SM walks output tiles
// tile = blockIdx.x, blockIdx.x + gridDim.x, ...  Warp 0 (one thread) feeds
// the shared-memory ring with TMA, warp 1 (one thread) issues the MMAs, warps
// 2-5 drain accumulators.  Tensor memory holds two 128 x 256 FP32
// accumulators (all 512 columns), so the epilogue of tile i (tcgen05.ld +
// stores) overlaps the MMAs of tile i + 1.  Barriers: full/empty per ring
// slot (TMA -> MMA -> TMA), tfull/tempty per accumulator (MMA -> epilogue ->
// MMA); every wait is bounded.
__global__ void __launch_bounds__(192, 1)
    k_bmm_tc_persist(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, BmmTcArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t *sA = base;
  uint8_t *sB = base + TC_STAGES * TC_A_BYTES;
  uint64_t *full = reinterpret_cast<uint64_t *>(sB + TC_STAGES * TC_B_BYTES);
  uint64_t *empty = full + TC_STAGES;
  uint64_t *tfull = empty + TC_STAGES;  // [2]
  uint64_t *tempty = tfull + 2;         // [2]
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tempty + 2);
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_n = (a.N + TC_BN - 1) / TC_BN, tiles_m = (a.M + TC_BM - 1) / TC_BM;
  const int tiles = tiles_n * tiles_m;
  const int nk = a.Kp / TC_BK;

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull + b, 1);
      mbar_init(tempty + b, 4);  // one arrival per epilogue warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2u * TC_BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int g = 0;  // k-blocks issued so far (ring position)
      for (int t = blockIdx.x; t < tiles && !s_fail; t += gridDim.x) {
        int m0, n0;
        tile_origin(t, tiles_m, tiles_n, &m0, &n0);
        for (int kb = 0; kb < nk; ++kb, ++g) {
          const int s = g % TC_STAGES, r = g / TC_STAGES;
          if (g >= TC_STAGES && !mbar_wait(empty + s, (uint32_t)((r - 1) & 1), a.err)) {
            s_fail = 1;
            break;
          }
          mbar_expect_tx(full + s, TC_A_BYTES + TC_B_BYTES);
          tma_load_2d(sA + s * TC_A_BYTES, &tmA, kb * TC_BK, m0, full + s);
          tma_load_2d(sB + s * TC_B_BYTES, &tmB, kb * TC_BK, n0, full + s);
        }
      }
      // leave only after the copies in flight have landed
      for (int q = g - TC_STAGES < 0 ? 0 : g - TC_STAGES; q < g; ++q)
        if (!mbar_try_wait(full + q % TC_STAGES, (uint32_t)((q / TC_STAGES) & 1)))
          mbar_wait(full + q % TC_STAGES, (uint32_t)((q / TC_STAGES) & 1), a.err);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int g = 0, i = 0;
      for (int t = blockIdx.x; t < tiles && !s_fail; t += gridDim.x, ++i) {
        const int b = i & 1, u = i >> 1;
        if (u >= 1 && !mbar_wait(tempty + b, (uint32_t)((u - 1) & 1), a.err)) {
          s_fail = 1;
          break;
        }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * TC_BN);
        for (int kb = 0; kb < nk; ++kb, ++g) {
          const int s = g % TC_STAGES, r = g / TC_STAGES;
          if (!mbar_wait(full + s, (uint32_t)(r & 1), a.err)) {
            s_fail = 1;
            break;
          }
          tc_fence_after();
          const uint64_t ad = sdesc_k_sw128(smem_u32(sA + s * TC_A_BYTES));
          const uint64_t bd = sdesc_k_sw128(smem_u32(sB + s * TC_B_BYTES));
#pragma unroll
          for (int k = 0; k < TC_BK / 32; ++k) mma_f8(acc, ad + 2 * k, bd + 2 * k, TC_IDESC, (kb | k) != 0 ? 1u : 0u);
          mma_commit(empty + s);
        }
        mma_commit(tfull + b);
        if (s_fail) break;
      }
    }
  } else {
    // epilogue warps 2..5: TMEM lane quarter = warp % 4
    const int q4 = warp & 3;
    int i = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++i) {
      const int b = i & 1, u = i >> 1;
      // lane 0 waits and decides for the warp, so the .sync.aligned TMEM
      // loads below run on a converged warp even when a wait gives up
      int go = 0;
      if (lane == 0) go = mbar_wait(tfull + b, (uint32_t)(u & 1), a.err) && !s_fail;
      go = __shfl_sync(0xffffffffu, go, 0);
      tc_fence_after();
      if (!go) break;
      int m0, n0;
      tile_origin(t, tiles_m, tiles_n, &m0, &n0);
      epilogue_tile(a, tmem, b, q4, lane, m0, n0);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(tempty + b)) : "memory");
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2u * TC_BN) : "memory");
  }
}

// Word-major bits -> K-major e4m3 bytes, plus row popcounts.
// out[r][32 kw + b] = bit b of G[kw][r] ? 1.0 (0x38) : 0.0, columns Kw*32 ..
// Kp zero; pop[r] += popc of the row's words (pop zeroed by the caller).  A
// 256-thread block transposes a 32-word x 32-row tile through shared
// memory: loads run along rows (contiguous in the word-major input), stores
// along K (each row's 32 words are 1 KiB contiguous in the output).
__global__ void __launch_bounds__(256) k_bits_to_e4m3(const uint32_t *__restrict__ G, int rows, int Kw, int Kp,
                                                      uint8_t *__restrict__ out, int *__restrict__ pop) {
  __shared__ uint32_t tile[32][33];
  const int r0 = blockIdx.x * 32, kw0 = blockIdx.y * 32;
  const int words = Kp / 32;
  for (int i = threadIdx.x; i < 32 * 32; i += 256) {
    const int kk = i >> 5, rr = i & 31;
    const int kw = kw0 + kk, r = r0 + rr;
    tile[kk][rr] = (kw < Kw && r < rows) ? __ldg(G + (size_t)kw * rows + r) : 0u;
  }
  __syncthreads();
  if (threadIdx.x < 32 && r0 + (int)threadIdx.x < rows && kw0 < Kw) {
    int c = 0;
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) c += __popc(tile[kk][threadIdx.x]);
    atomicAdd(pop + r0 + threadIdx.x, c);
  }
  // 32 rows x 32 words x 2 halves of 16 bits -> 16-byte stores
  for (int i = threadIdx.x; i < 32 * 64; i += 256) {
    const int rr = i >> 6, q = i & 63, kk = q >> 1, h = q & 1;
    const int r = r0 + rr, kw = kw0 + kk;
    if (r >= rows || kw >= words) continue;
    const uint32_t w = tile[kk][rr] >> (16 * h);
    uint32_t o[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      // spread the 4 bits of a nibble to the low bit of 4 bytes (bit b ->
      // bit 8b; the four shifted copies occupy disjoint bit ranges, so the
      // product has no carries), then scale each 0/1 byte to 0x38
      const uint32_t nib = (w >> (4 * n)) & 0xFu;
      o[n] = ((nib * 0x00204081u) & 0x01010101u) * 0x38u;
    }
    *reinterpret_cast<uint4 *>(out + (size_t)r * Kp + (size_t)kw * 32 + h * 16) = make_uint4(o[0], o[1], o[2], o[3]);
  }
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::mutex mu;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

gbs_status make_map(CUtensorMap *map, void *base, int rows, int Kp, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return fail(GBS_ERR_CUDA, "bmm tc: cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp};
  cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(GBS_ERR_CUDA, "bmm tc: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return GBS_OK;
}

}  // namespace

static __device__ int g_bmm_tc_err;

// launch forms of bmm_tc_run
constexpr int kTcPerTile = 0, kTcPersistent = 1;

gbs_status bmm_tc_run(const uint32_t *A, const uint32_t *B, int M, int N, int Kw, int mode, int32_t *C, float *Cf,
                      int ldc, cudaStream_t s, int form, uint32_t *Cbits, int bin_layout, int nbits) {
  GBS_REQUIRE(M % 4 == 0 && N % 4 == 0 && ldc % 4 == 0, "bmm tc: M, N (and ldc) must be multiples of 4");
  GBS_REQUIRE(!Cbits || (M % 32 == 0 && N % 32 == 0 && mode == 0),
              "bmm tc: sign words need M, N multiples of 32 and XOR counts");
  GBS_REQUIRE((long long)Kw * 32 < (1ll << 24), "bmm tc: K must be < 2^24 bits (exact FP32 accumulation)");
  const int Kp = (Kw * 32 + TC_BK - 1) / TC_BK * TC_BK;
  DevBuf A8, B8, pa, pb;
  GBS_TRY(A8.alloc((size_t)M * Kp, s));
  GBS_TRY(B8.alloc((size_t)N * Kp, s));
  GBS_TRY(pa.alloc(sizeof(int) * (size_t)M, s));
  GBS_TRY(pb.alloc(sizeof(int) * (size_t)N, s));
  GBS_CUDA_TRY(cudaMemsetAsync(pa.p, 0, sizeof(int) * (size_t)M, s));
  GBS_CUDA_TRY(cudaMemsetAsync(pb.p, 0, sizeof(int) * (size_t)N, s));
  const int wb = (Kp / 32 + 31) / 32;
  k_bits_to_e4m3<<<dim3((M + 31) / 32, wb), 256, 0, s>>>(A, M, Kw, Kp, A8.as<uint8_t>(), pa.as<int>());
  k_bits_to_e4m3<<<dim3((N + 31) / 32, wb), 256, 0, s>>>(B, N, Kw, Kp, B8.as<uint8_t>(), pb.as<int>());
  GBS_TRY(check_launch("bmm tc prologue"));
  CUtensorMap ma, mb;
  GBS_TRY(make_map(&ma, A8.p, M, Kp, TC_BM));
  GBS_TRY(make_map(&mb, B8.p, N, Kp, TC_BN));
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_bmm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (attr_err == cudaSuccess)
      attr_err = cudaFuncSetAttribute(k_bmm_tc_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
  });
  if (attr_err != cudaSuccess) return cuda_fail(attr_err, "cudaFuncSetAttribute(k_bmm_tc)");
  int *err = nullptr;
  GBS_CUDA_TRY(cudaGetSymbolAddress((void **)&err, g_bmm_tc_err));
  BmmTcArgs args{M, N, Kw, Kp, mode, pa.as<int>(), pb.as<int>(), C, Cf, ldc, err, Cbits, bin_layout, nbits};
  const int tiles = ((N + TC_BN - 1) / TC_BN) * ((M + TC_BM - 1) / TC_BM);
  DeviceInfo di;
  GBS_TRY(device_info(&di));
  if (form == kTcPersistent) {
    const int grid = tiles < di.sm_count ? tiles : di.sm_count;
    k_bmm_tc_persist<<<grid, 192, TC_SMEM, s>>>(ma, mb, args);
  } else {
    dim3 grid((N + TC_BN - 1) / TC_BN, (M + TC_BM - 1) / TC_BM);
    k_bmm_tc<<<grid, 128, TC_SMEM, s>>>(ma, mb, args);
  }
  return check_launch("k_bmm_tc");
}

gbs_status bmm_tc_error_count(int *out) {
  int v = 0;
  GBS_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_bmm_tc_err, sizeof(int)));
  *out = v;
  return GBS_OK;
}

}  // namespace gbs
