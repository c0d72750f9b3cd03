// Harness that runs the reference's own ingest path -- readMtx<float>(...,
// directed = 0, ...) then coo2csr (test_spmm_full.cu:99-113 calling
// backend/readMtx.hpp:351-422 and :246-304) -- on one .mtx file and prints
// the CSR it builds.  Compiled by oracle/Makefile against the reference's
// sources where they lie; the binary goes to oracle/_ref/ and is used only to
// make the golden fixtures under tests/golden/.
#include <cstdio>
#include <vector>

#include "readMtx.hpp"

int main(int argc, char **argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: readmtx_ref file.mtx\n");
    return 2;
  }
  std::vector<int> rows, cols;
  std::vector<float> vals;
  int nrows = 0, ncols = 0, nnz = 0;
  char *dat_name = nullptr;
  readMtx(argv[1], &rows, &cols, &vals, &nrows, &ncols, &nnz, 0, false, &dat_name);
  std::vector<int> rowptr(nrows + 1), colind(rows.size());
  std::vector<float> csrval(rows.size());
  coo2csr(rowptr.data(), colind.data(), csrval.data(), rows, cols, vals, nrows, ncols);
  std::printf("%d %d %d %zu\n", nrows, ncols, nnz, rows.size());
  for (int i = 0; i <= nrows; ++i) std::printf("%d%c", rowptr[i], i == nrows ? '\n' : ' ');
  for (size_t i = 0; i < colind.size(); ++i) std::printf("%d ", colind[i]);
  std::printf("\n");
  for (size_t i = 0; i < csrval.size(); ++i) std::printf("%.9g ", csrval[i]);
  std::printf("\n");
  return 0;
}
