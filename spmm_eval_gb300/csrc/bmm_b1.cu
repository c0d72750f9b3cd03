// Dense binary matmul (backend/mm.cu semantics) on sm_103a.
//
// Operands are in the reference's word-major layout (ToBit32ColUd,
// spmm.cu:93-111): A[kw][M] and B[kw][N] uint32 words, word kw of row r
// holding K-bits 32kw..32kw+31.  For rows r of A and c of B:
//   xor(r,c) = sum_kw popc(A[kw][r] ^ B[kw][c])
//   and(r,c) = sum_kw popc(A[kw][r] & B[kw][c])
// BMM32_Arow_Brow / BMM32_MT_M_S store 32*Kw - 2*xor (mm.cu:44-51, :74).
//
// Two kernels, same tiling (128 x 128 output tile per 256-thread CTA,
// 16-word K slices staged in shared memory with a 2-stage cp.async
// pipeline, padded rows so fragment reads are bank-conflict free):
//   * popc : CUDA cores, each thread 8 x 8 outputs, XOR + POPC + ADD.
//   * mma  : tensor cores, mma.sync.aligned.m16n8k256 .b1 AND-popc; XOR is
//            recovered as popc(a) + popc(b) - 2 * and from row popcounts.
// Of these two, popc is the faster on GB300 (8192^3: 3.6 ms against 7.5 ms
// for the .b1 tensor path); the default is the persistent tcgen05 kernel in
// bmm_tc.cu (0.39 ms), which multiplies the bits expanded to FP8.
// Bit order inside a word does not matter to either (popcount of matching
// K positions), so the reference layout is consumed as is.
#include <cstdint>

#include "common.cuh"
#include "util.cuh"

namespace gbs {

constexpr int BM = 128, BN = 128, BKW = 16, PAD = 8;
constexpr int SROW = BM + PAD;  // words per staged K-word row

enum { MODE_XOR = 0, MODE_AND = 1, MODE_SIGNED = 2 };

struct BmmArgs {
  const uint32_t *A;  // [Kw][lda]
  const uint32_t *B;  // [Kw][ldb]
  int M, N, Kw, lda, ldb;
  int32_t *C;  // row-major M x N (ldc), or
  float *Cf;   // float output (BMM32_Arow_Brow)
  int ldc;
  int mode;
  const int *pa;  // row popcounts (mma XOR / SIGNED)
  const int *pb;
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 16 : 0;  // zero-fill outside the matrix
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Stage K-words [k0, k0+BKW) of the 128-row block starting at row0 into
// S[kw][SROW].  256 threads x 2 chunks of 4 words.
__device__ __forceinline__ void stage(uint32_t *S, const uint32_t *G, int ld, int rows, int Kw, int k0,
                                      int row0, int tid) {
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int chunk = tid + q * 256;  // 0..511
    const int kw = chunk >> 5;        // 32 chunks of 4 rows per K-word
    const int r4 = (chunk & 31) * 4;
    const bool valid = (k0 + kw < Kw) && (row0 + r4 < rows);
    const uint32_t *src = valid ? G + (size_t)(k0 + kw) * ld + row0 + r4 : G;
    cp_async16(S + kw * SROW + r4, src, valid);
  }
}

// ----------------------------------------------------------------------------
template <bool MMA>
__global__ void __launch_bounds__(256) k_bmm(BmmArgs a) {
  __shared__ __align__(16) uint32_t As[2][BKW * SROW];
  __shared__ __align__(16) uint32_t Bs[2][BKW * SROW];
  const int tid = threadIdx.x;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int nk = (a.Kw + BKW - 1) / BKW;

  stage(As[0], a.A, a.lda, a.M, a.Kw, 0, m0, tid);
  stage(Bs[0], a.B, a.ldb, a.N, a.Kw, 0, n0, tid);
  cp_async_commit();

  if constexpr (MMA) {
    const int warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, tig = lane & 3;
    const int wm = (warp >> 2) * 64, wn = (warp & 3) * 32;
    int acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][j][q] = 0;
    for (int kt = 0; kt < nk; ++kt) {
      const int cur = kt & 1;
      if (kt + 1 < nk) {
        stage(As[cur ^ 1], a.A, a.lda, a.M, a.Kw, (kt + 1) * BKW, m0, tid);
        stage(Bs[cur ^ 1], a.B, a.ldb, a.N, a.Kw, (kt + 1) * BKW, n0, tid);
      }
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
      const uint32_t *as = As[cur], *bs = Bs[cur];
#pragma unroll
      for (int kk = 0; kk < BKW; kk += 8) {
        uint32_t af[4][4], bf[4][2];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = wm + i * 16 + g;
          af[i][0] = as[(kk + tig) * SROW + r];
          af[i][1] = as[(kk + tig) * SROW + r + 8];
          af[i][2] = as[(kk + 4 + tig) * SROW + r];
          af[i][3] = as[(kk + 4 + tig) * SROW + r + 8];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int c = wn + j * 8 + g;
          bf[j][0] = bs[(kk + tig) * SROW + c];
          bf[j][1] = bs[(kk + 4 + tig) * SROW + c];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j)
            asm volatile(
                "mma.sync.aligned.m16n8k256.row.col.s32.b1.b1.s32.and.popc "
                "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                : "+r"(acc[i][j][0]), "+r"(acc[i][j][1]), "+r"(acc[i][j][2]), "+r"(acc[i][j][3])
                : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bf[j][0]),
                  "r"(bf[j][1]));
      }
      __syncthreads();
    }
    const int Kbits = 32 * a.Kw;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = m0 + wm + i * 16 + g + 8 * h;
        if (r >= a.M) continue;
        const int par = (a.mode != MODE_AND) ? __ldg(a.pa + r) : 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int c = n0 + wn + j * 8 + tig * 2;
          int v[2];
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int andc = acc[i][j][2 * h + e];
            int x = andc;
            if (a.mode != MODE_AND && c + e < a.N) {
              const int xr = par + __ldg(a.pb + c + e) - 2 * andc;
              x = a.mode == MODE_XOR ? xr : Kbits - 2 * xr;
            }
            v[e] = x;
          }
          if (a.Cf) {
            if (c < a.N) a.Cf[(size_t)r * a.ldc + c] = (float)v[0];
            if (c + 1 < a.N) a.Cf[(size_t)r * a.ldc + c + 1] = (float)v[1];
          } else {
            if (c < a.N) a.C[(size_t)r * a.ldc + c] = v[0];
            if (c + 1 < a.N) a.C[(size_t)r * a.ldc + c + 1] = v[1];
          }
        }
      }
  } else {
    // popc: thread (ty, tx) owns rows ty*8..+7 and columns tx*8..+7.
    const int ty = tid >> 4, tx = tid & 15;
    int acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0;
    const bool use_and = a.mode == MODE_AND;
    for (int kt = 0; kt < nk; ++kt) {
      const int cur = kt & 1;
      if (kt + 1 < nk) {
        stage(As[cur ^ 1], a.A, a.lda, a.M, a.Kw, (kt + 1) * BKW, m0, tid);
        stage(Bs[cur ^ 1], a.B, a.ldb, a.N, a.Kw, (kt + 1) * BKW, n0, tid);
      }
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
      const uint32_t *as = As[cur], *bs = Bs[cur];
#pragma unroll 4
      for (int kw = 0; kw < BKW; ++kw) {
        const uint4 a0 = *reinterpret_cast<const uint4 *>(as + kw * SROW + ty * 8);
        const uint4 a1 = *reinterpret_cast<const uint4 *>(as + kw * SROW + ty * 8 + 4);
        const uint4 b0 = *reinterpret_cast<const uint4 *>(bs + kw * SROW + tx * 8);
        const uint4 b1 = *reinterpret_cast<const uint4 *>(bs + kw * SROW + tx * 8 + 4);
        const uint32_t av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const uint32_t bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
        if (use_and) {
#pragma unroll
          for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] += __popc(av[i] & bv[j]);
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] += __popc(av[i] ^ bv[j]);
        }
      }
      __syncthreads();
    }
    const int Kbits = 32 * a.Kw;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = m0 + ty * 8 + i;
      if (r >= a.M) continue;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = n0 + tx * 8 + j;
        if (c >= a.N) continue;
        const int x = a.mode == MODE_SIGNED ? Kbits - 2 * acc[i][j] : acc[i][j];
        if (a.Cf) a.Cf[(size_t)r * a.ldc + c] = (float)x;
        else a.C[(size_t)r * a.ldc + c] = x;
      }
    }
  }
}

// Row popcounts of a word-major matrix: p[r] = sum_kw popc(G[kw][r]).
__global__ void k_row_popc(const uint32_t *__restrict__ G, int rows, int Kw, int ld, int *__restrict__ p) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  int s = 0;
  for (int k = 0; k < Kw; ++k) s += __popc(__ldg(G + (size_t)k * ld + r));
  p[r] = s;
}

// Sign words of a count matrix: bit = (nbits - 2 * xor >= 0), 32 columns per
// word, first column in bit 31.  layout 0 = BMM32_BIN (word of row r over
// columns 32*by.. at C[by*m + r], mm.cu:84, :97-104); layout 1 = BMM32S_BIN
// (at C[(r/32)*k*32 + by*32 + r%32], mm.cu:114, :123-124).
__global__ void k_sign_words(const int32_t *__restrict__ X, int m, int k, int nbits, int layout,
                             uint32_t *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // (r, by) pair
  const int kb = k / 32;
  if (w >= (long long)m * kb) return;
  const int r = (int)(w / kb), by = (int)(w % kb);
  const int32_t x = X[(size_t)r * k + by * 32 + lane];
  const float t = (float)nbits - 2.0f * (float)x;
  const uint32_t word = __brev(__ballot_sync(0xffffffffu, t >= 0.0f));
  if (lane == 0) {
    if (layout == 0) out[(size_t)by * m + r] = word;
    else out[(size_t)(r / 32) * k * 32 + (size_t)by * 32 + (r % 32)] = word;
  }
}

// form: 0 = one CTA per tile, 1 = persistent
gbs_status bmm_tc_run(const uint32_t *A, const uint32_t *B, int M, int N, int Kw, int mode, int32_t *C, float *Cf,
                      int ldc, cudaStream_t s, int form, uint32_t *Cbits = nullptr, int bin_layout = 0,
                      int nbits = 0);
gbs_status bmm_tc_error_count(int *out);

gbs_status bmm_run(const uint32_t *A, const uint32_t *B, int M, int N, int Kw, int mode, int algo,
                   int32_t *C, float *Cf, int ldc, cudaStream_t s) {
  if (algo == 0 || algo == 4) return bmm_tc_run(A, B, M, N, Kw, mode, C, Cf, ldc, s, 1);
  if (algo == 3) return bmm_tc_run(A, B, M, N, Kw, mode, C, Cf, ldc, s, 0);
  GBS_REQUIRE(M % 4 == 0 && N % 4 == 0, "bmm: M and N must be multiples of 4");
  GBS_REQUIRE((reinterpret_cast<uintptr_t>(A) & 15u) == 0 && (reinterpret_cast<uintptr_t>(B) & 15u) == 0,
              "bmm: A and B must be 16-byte aligned");
  BmmArgs a{};
  a.A = A;
  a.B = B;
  a.M = M;
  a.N = N;
  a.Kw = Kw;
  a.lda = M;
  a.ldb = N;
  a.C = C;
  a.Cf = Cf;
  a.ldc = ldc;
  a.mode = mode;
  DevBuf pa, pb;
  const bool mma = algo == 2;
  if (mma && mode != MODE_AND) {
    GBS_TRY(pa.alloc(sizeof(int) * (size_t)M, s));
    GBS_TRY(pb.alloc(sizeof(int) * (size_t)N, s));
    k_row_popc<<<(M + 255) / 256, 256, 0, s>>>(A, M, Kw, M, pa.as<int>());
    k_row_popc<<<(N + 255) / 256, 256, 0, s>>>(B, N, Kw, N, pb.as<int>());
    GBS_TRY(check_launch("k_row_popc"));
    a.pa = pa.as<int>();
    a.pb = pb.as<int>();
  }
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  if (mma) k_bmm<true><<<grid, 256, 0, s>>>(a);
  else k_bmm<false><<<grid, 256, 0, s>>>(a);
  return check_launch("k_bmm");
}

}  // namespace gbs

using namespace gbs;

// algo: 0 = default (the fastest measured on GB300: persistent tcgen05 on
// FP8 {0,1}), 1 = popc CUDA cores, 2 = tensor-core mma.sync .b1, 3 = tcgen05
// one CTA per tile, 4 = persistent tcgen05.  8192^3 XOR counts on GB300,
// each incl. the bit expansion: 0.39 / 0.60 ms for 4 / 3 (2.8 P bit-ops/s
// for 4), popc 3.59 ms
// (306 T), mma.sync .b1 7.51 ms (146 T).
extern "C" gbs_status gbs_bmm_b1(const uint32_t *A, const uint32_t *B, int M, int N, int Kw, int mode,
                                 int algo, int32_t *C, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(M >= 0 && N >= 0 && Kw >= 1, "bmm: bad sizes");
  GBS_REQUIRE(mode >= 0 && mode <= 2, "bmm: mode must be 0 (xor), 1 (and) or 2 (32*Kw - 2*xor)");
  GBS_REQUIRE(algo >= 0 && algo <= 4, "bmm: algo must be 0..4");
  if (M == 0 || N == 0) return GBS_OK;
  GBS_REQUIRE(A && B && C, "bmm: null pointer");
  return bmm_run(A, B, M, N, Kw, mode, algo, C, nullptr, N, (cudaStream_t)stream);
}

extern "C" gbs_status gbs_bmm_tc_timeouts(int *count) {
  clear_error();
  GBS_REQUIRE(count != nullptr, "bmm tc timeouts: null output");
  return bmm_tc_error_count(count);
}

extern "C" gbs_status gbs_bmm32_arow_brow(const uint32_t *A, const uint32_t *B, float *C, int A_height,
                                          int A_width, int B_width, gbs_stream_t stream) {
  clear_error();
  GBS_REQUIRE(A_height >= 0 && B_width >= 0 && A_width >= 1, "bmm32_arow_brow: bad sizes");
  if (A_height == 0 || B_width == 0) return GBS_OK;
  GBS_REQUIRE(A && B && C, "bmm32_arow_brow: null pointer");
  return bmm_run(A, B, A_height, B_width, A_width, MODE_SIGNED, 0, nullptr, C, B_width,
                 (cudaStream_t)stream);
}

// Sign words of the binary GEMM.  algo 0 (default): the persistent tcgen05
// kernel thresholds the counts in its epilogue and writes only the words;
// algo 1: the int32 XOR counts of the default GEMM into an m x k temporary,
// then k_sign_words (kept as the cross-check and the timing baseline).
static gbs_status bin_run(const uint32_t *A, const uint32_t *B, uint32_t *C, int m, int n, int k,
                          int layout, int algo, cudaStream_t s) {
  GBS_REQUIRE(m >= 0 && k >= 0 && n >= 1, "bmm32 bin: bad sizes");
  GBS_REQUIRE(m % 32 == 0 && k % 32 == 0, "bmm32 bin: m and k must be multiples of 32 (as the reference's grid)");
  GBS_REQUIRE(layout == 0 || layout == 1, "bmm bin: layout must be 0 (BMM32_BIN) or 1 (BMM32S_BIN)");
  GBS_REQUIRE(algo == 0 || algo == 1, "bmm bin: algo must be 0 (fused) or 1 (counts, then sign words)");
  if (m == 0 || k == 0) return GBS_OK;
  GBS_REQUIRE(A && B && C, "bmm32 bin: null pointer");
  const int Kw = (n + 31) / 32;
  if (algo == 0) return bmm_tc_run(A, B, m, k, Kw, MODE_XOR, nullptr, nullptr, k, s, 1, C, layout, n);
  DevBuf X;
  GBS_TRY(X.alloc(sizeof(int32_t) * (size_t)m * k, s));
  GBS_TRY(bmm_run(A, B, m, k, Kw, MODE_XOR, 0, X.as<int32_t>(), nullptr, k, s));
  const long long warps = (long long)m * (k / 32);
  k_sign_words<<<(int)((warps * 32 + 255) / 256), 256, 0, s>>>(X.as<int32_t>(), m, k, n, layout, C);
  return check_launch("k_sign_words");
}

static gbs_status bin_common(const uint32_t *A, const uint32_t *B, uint32_t *C, int m, int n, int k,
                             int layout, cudaStream_t s) {
  return bin_run(A, B, C, m, n, k, layout, 0, s);
}

extern "C" gbs_status gbs_bmm_bin(const uint32_t *A, const uint32_t *B, uint32_t *C, int m, int n, int k,
                                  int layout, int algo, gbs_stream_t stream) {
  clear_error();
  return bin_run(A, B, C, m, n, k, layout, algo, (cudaStream_t)stream);
}

extern "C" gbs_status gbs_bmm32_bin(const uint32_t *A, const uint32_t *B, uint32_t *C, int m, int n, int k,
                                    gbs_stream_t stream) {
  clear_error();
  return bin_common(A, B, C, m, n, k, 0, (cudaStream_t)stream);
}

extern "C" gbs_status gbs_bmm32s_bin(const uint32_t *A, const uint32_t *B, uint32_t *C, int m, int n, int k,
                                     gbs_stream_t stream) {
  clear_error();
  return bin_common(A, B, C, m, n, k, 1, (cudaStream_t)stream);
}
