// Drop-in executables for the reference's driver surface:
//   {kernel_name} {matrix.mtx} {hidden_size}
// (test_spmm_full.cu:474-514, Makefile:17-30, README.md:8).  One binary;
// the behaviour is chosen by the name it is run under (bin/ holds links):
//
//   spmmfbf      B2SR-4 x float FBF SpMM (gbs_spmm4_full_full) -- the
//                reference's spmm/spmmfbf
//   spmmcsr      merge-path CSR SpMM, FP32 features
//   spmmcsr_bf16 merge-path CSR SpMM, BF16 features
//   spmmb2sr8 / spmmb2sr16 / spmmb2sr32   B2SR x float at that tile size
//   spmmbmm      B2SR-4 x packed +-1 features -> int32 (signed form)
//
// As in the reference: A is read from the .mtx file (gbs_mtx_read, the
// readMtx + coo2csr semantics), B is nrows x hidden of random +-1 values,
// the result is checked against cusparseSpMM (CSR, FP32, column-major
// copies, alpha = 1, beta = 0) and the first two lines printed are
//   "<name>: <ms>, csr-float: <ms>"   and   "TEST PASSED: <0|1>".
// Exact equality is required (+-1 features make every partial sum an
// integer), except for spmmcsr (max |diff| <= 1e-5 * (|A| |B|)) and
// spmmcsr_bf16 (1e-2).  A JSON line with the details follows.
// Differences from the reference: B comes from a seeded generator
// (GBS_SEED, default 0x5EED) instead of srand(time(0)); times are the median
// of 10 launches after one warm-up instead of one cold launch; the exit
// status is 0 on pass, 1 on a failed check, 2 on bad input.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cusparse.h>
#include <libgen.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbspmm.h"

#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      std::fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), \
                   __FILE__, __LINE__);                                        \
      std::exit(2);                                                            \
    }                                                                          \
  } while (0)
#define GK(x)                                                                   \
  do {                                                                          \
    gbs_status s_ = (x);                                                        \
    if (s_ != GBS_OK) {                                                         \
      std::fprintf(stderr, "gbs error %d: %s (%s:%d)\n", (int)s_,               \
                   gbs_last_error(), __FILE__, __LINE__);                       \
      std::exit(2);                                                             \
    }                                                                           \
  } while (0)
#define SK(x)                                                                      \
  do {                                                                             \
    cusparseStatus_t s_ = (x);                                                     \
    if (s_ != CUSPARSE_STATUS_SUCCESS) {                                           \
      std::fprintf(stderr, "cuSPARSE error %d at %s:%d\n", (int)s_, __FILE__, __LINE__); \
      std::exit(2);                                                                \
    }                                                                              \
  } while (0)

template <typename T>
static T *dalloc(size_t n) {
  T *p = nullptr;
  CK(cudaMalloc(&p, sizeof(T) * (n ? n : 1)));
  return p;
}

struct Timer {
  cudaEvent_t a, b;
  Timer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  template <typename F>
  float median_ms(F f, int reps = 10) {
    f();  // warm-up
    CK(cudaDeviceSynchronize());
    std::vector<float> t;
    for (int i = 0; i < reps; ++i) {
      cudaEventRecord(a);
      f();
      cudaEventRecord(b);
      CK(cudaEventSynchronize(b));
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      t.push_back(ms);
    }
    std::sort(t.begin(), t.end());
    return t[t.size() / 2];
  }
};

static uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int main(int argc, char **argv) {
  std::string name = basename(argv[0]);
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <matrix.mtx> <hidden_size>\n", name.c_str());
    return 2;
  }
  const int F = std::atoi(argv[2]);
  if (F < 1) {
    std::fprintf(stderr, "%s: hidden_size must be >= 1\n", name.c_str());
    return 2;
  }
  const bool is_fbf = name == "spmmfbf", is_csr = name == "spmmcsr", is_bf16 = name == "spmmcsr_bf16",
             is_bmm = name == "spmmbmm";
  int tile = 4;
  if (name == "spmmb2sr8") tile = 8;
  else if (name == "spmmb2sr16") tile = 16;
  else if (name == "spmmb2sr32") tile = 32;
  else if (!is_fbf && !is_csr && !is_bf16 && !is_bmm) {
    std::fprintf(stderr, "unknown kernel name '%s'\n", name.c_str());
    return 2;
  }
  CK(cudaSetDevice(0));

  gbs_host_csr A{};
  GK(gbs_mtx_read(argv[1], &A));
  const int n = A.nrows, m = A.ncols, nnz = A.nnz;

  // random +-1 features (rows = ncols of A; the reference uses nrows, which
  // is the same for its square graphs)
  uint64_t seed = 0x5EED;
  if (const char *e = std::getenv("GBS_SEED")) seed = std::strtoull(e, nullptr, 0);
  std::vector<float> B((size_t)m * F), Bcol((size_t)m * F);
  for (size_t i = 0; i < B.size(); ++i) B[i] = (splitmix(seed) >> 63) ? 1.0f : -1.0f;
  for (int j = 0; j < F; ++j)
    for (int i = 0; i < m; ++i) Bcol[(size_t)j * m + i] = B[(size_t)i * F + j];

  int *d_rp = dalloc<int>(n + 1), *d_ci = dalloc<int>(nnz);
  float *d_v = dalloc<float>(nnz), *d_B = dalloc<float>((size_t)m * F), *d_Bcol = dalloc<float>((size_t)m * F);
  float *d_Ccol = dalloc<float>((size_t)n * F), *d_C = dalloc<float>((size_t)n * F);
  CK(cudaMemcpy(d_rp, A.rowptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_ci, A.colind, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_v, A.vals, sizeof(float) * (size_t)nnz, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_B, B.data(), sizeof(float) * B.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_Bcol, Bcol.data(), sizeof(float) * Bcol.size(), cudaMemcpyHostToDevice));

  // baseline: cusparseSpMM as evalCSRSpmmFloatCuSPARSE (test_spmm_full.cu:212-342)
  Timer tm;
  cusparseHandle_t h;
  SK(cusparseCreate(&h));
  cusparseSpMatDescr_t sA;
  cusparseDnMatDescr_t sB, sC;
  float alpha = 1.f, beta = 0.f;
  SK(cusparseCreateCsr(&sA, n, m, nnz, d_rp, d_ci, d_v, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                       CUSPARSE_INDEX_BASE_ZERO, CUDA_R_32F));
  SK(cusparseCreateDnMat(&sB, m, F, m, d_Bcol, CUDA_R_32F, CUSPARSE_ORDER_COL));
  SK(cusparseCreateDnMat(&sC, n, F, n, d_Ccol, CUDA_R_32F, CUSPARSE_ORDER_COL));
  size_t bsz = 0;
  SK(cusparseSpMM_bufferSize(h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, sA,
                             sB, &beta, sC, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, &bsz));
  void *sbuf = dalloc<char>(bsz);
  const float ms_ref = tm.median_ms([&] {
    SK(cusparseSpMM(h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, sA, sB, &beta,
                    sC, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, sbuf));
  });
  std::vector<float> Cref_col((size_t)n * F), Cref((size_t)n * F);
  CK(cudaMemcpy(Cref_col.data(), d_Ccol, sizeof(float) * Cref_col.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < F; ++j) Cref[(size_t)i * F + j] = Cref_col[(size_t)j * n + i];

  float ms = 0, ms_pack = 0;
  std::vector<float> C((size_t)n * F);
  double tol = 0.0;
  int nnzb = 0;
  if (is_csr || is_bf16) {
    const void *Bk = d_B;
    __nv_bfloat16 *d_Bh = nullptr;
    if (is_bf16) {
      std::vector<__nv_bfloat16> Bh(B.size());
      for (size_t i = 0; i < B.size(); ++i) Bh[i] = __float2bfloat16(B[i]);
      d_Bh = dalloc<__nv_bfloat16>(B.size());
      CK(cudaMemcpy(d_Bh, Bh.data(), sizeof(__nv_bfloat16) * Bh.size(), cudaMemcpyHostToDevice));
      Bk = d_Bh;
    }
    size_t wsb = 0;
    GK(gbs_csr_spmm_workspace_size(n, nnz, F, is_bf16 ? GBS_BF16 : GBS_F32, &wsb));
    void *ws = dalloc<char>(wsb);
    GK(gbs_csr_spmm_workspace_init(ws, wsb, nullptr));
    ms = tm.median_ms([&] {
      GK(gbs_csr_spmm(n, m, nnz, d_rp, d_ci, d_v, Bk, is_bf16 ? GBS_BF16 : GBS_F32, F, d_C, ws, wsb, nullptr));
    });
    CK(cudaMemcpy(C.data(), d_C, sizeof(float) * C.size(), cudaMemcpyDeviceToHost));
    tol = is_bf16 ? 1e-2 : 1e-5;
    cudaFree(ws);
    if (d_Bh) cudaFree(d_Bh);
  } else {
    const int mb = (n + tile - 1) / tile;
    int *d_brp = dalloc<int>(mb + 1);
    const float t0 = tm.median_ms([&] { GK(gbs_csr2b2sr_nnzb(n, m, nnz, d_rp, d_ci, tile, d_brp, &nnzb, nullptr)); }, 3);
    int *d_bci = dalloc<int>(nnzb);
    void *d_bv = dalloc<char>((size_t)nnzb * tile * (tile <= 8 ? 1 : tile / 8));
    const float t1 = tm.median_ms([&] { GK(gbs_csr2b2sr(n, m, nnz, d_rp, d_ci, tile, d_brp, d_bci, d_bv, nullptr)); }, 3);
    ms_pack = t0 + t1;
    if (is_bmm) {
      uint32_t *d_X = dalloc<uint32_t>((size_t)m * ((F + 31) / 32));
      int32_t *d_Ci = dalloc<int32_t>((size_t)n * F);
      GK(gbs_pack_sign_rows(d_B, m, F, d_X, nullptr));
      ms = tm.median_ms([&] { GK(gbs_b2sr_bmm(tile, n, mb, d_brp, d_bci, d_bv, d_X, F, 1, d_Ci, nullptr)); });
      std::vector<int32_t> Ci((size_t)n * F);
      CK(cudaMemcpy(Ci.data(), d_Ci, sizeof(int32_t) * Ci.size(), cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < C.size(); ++i) C[i] = (float)Ci[i];
      cudaFree(d_X);
      cudaFree(d_Ci);
    } else if (is_fbf) {
      // C zero-filled once, as evalB2SRSpmmFull32 does before its timer
      // (test_spmm_full.cu:347-348); repeated launches store the same values.
      CK(cudaMemset(d_C, 0, sizeof(float) * C.size()));
      ms = tm.median_ms([&] {
        GK(gbs_spmm4_full_full((const uint8_t *)d_bv, d_B, d_C, d_brp, d_bci, mb, F, nullptr));
      });
      CK(cudaMemcpy(C.data(), d_C, sizeof(float) * C.size(), cudaMemcpyDeviceToHost));
    } else {
      ms = tm.median_ms([&] { GK(gbs_b2sr_spmm(tile, n, mb, d_brp, d_bci, d_bv, d_B, GBS_F32, F, d_C, nullptr)); });
      CK(cudaMemcpy(C.data(), d_C, sizeof(float) * C.size(), cudaMemcpyDeviceToHost));
    }
    cudaFree(d_brp);
    cudaFree(d_bci);
    cudaFree(d_bv);
  }

  // verify (verifyResultFull, test_spmm_full.cu:412-431)
  bool pass = true;
  double worst = 0.0;
  if (tol == 0.0) {
    for (size_t i = 0; i < C.size(); ++i)
      if (C[i] != Cref[i]) pass = false;
  } else {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < F; ++j) {
        double mag = 0.0;
        for (int e = A.rowptr[i]; e < A.rowptr[i + 1]; ++e)
          mag += std::fabs((double)A.vals[e]) * std::fabs((double)B[(size_t)A.colind[e] * F + j]);
        const double d = std::fabs((double)C[(size_t)i * F + j] - (double)Cref[(size_t)i * F + j]);
        const double r = mag > 0 ? d / mag : (d == 0 ? 0.0 : INFINITY);
        worst = std::max(worst, r);
      }
    pass = worst <= tol;
  }
  const char *label = is_fbf ? "b2sr" : name.c_str();
  std::printf("%s: %.3f, csr-float: %.3f\n", label, ms, ms_ref);
  std::printf("TEST PASSED: %d\n", pass ? 1 : 0);
  std::printf("{\"kernel\": \"%s\", \"matrix\": \"%s\", \"nrows\": %d, \"nnz\": %d, \"F\": %d, \"ms\": %.4f, "
              "\"csr_float_cusparse_ms\": %.4f, \"pack_ms\": %.4f, \"tile\": %d, \"nnzb\": %d, "
              "\"max_rel_err\": %.3e, \"pass\": %s}\n",
              name.c_str(), argv[1], n, nnz, F, ms, ms_ref, ms_pack, (is_csr || is_bf16) ? 0 : tile, nnzb, worst,
              pass ? "true" : "false");

  cusparseDestroySpMat(sA);
  cusparseDestroyDnMat(sB);
  cusparseDestroyDnMat(sC);
  cusparseDestroy(h);
  gbs_host_csr_free(&A);
  return pass ? 0 : 1;
}
