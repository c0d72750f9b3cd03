"""GPU test of gbs_csr_spmm_noalloc, the CSR SpMM entry point that allocates
no device memory (for callers that may not call cudaMalloc while they run,
e.g. a framework that owns all device memory through its own pool, or a
serving loop that forbids allocation on the request path).

It is called twice in a row through the C ABI on a power-law graph whose
hub rows are split across warps (so the shared scratch array's partial
slots and arrival counters are exercised, and the second call starts from
whatever the first left behind), and each result is compared with the
workspace-based gbs_csr_spmm on the same inputs, within the tolerance the
other SpMM tests use (max |diff| / (|A| |B|) <= 1e-5).  This file is named
to be collected last.
"""
import pytest
import torch

from spmm_eval_gb300 import _lib
from spmm_eval_gb300 import graphs as G
from spmm_eval_gb300 import ops

pytestmark = pytest.mark.gpu


def _noalloc(A, B, out):
    _lib.call("gbs_csr_spmm_noalloc", A.nrows, A.ncols, A.nnz, A.rowptr.data_ptr(),
              A.colind.data_ptr(), A.vals.data_ptr(), B.data_ptr(), ops._DT[B.dtype],
              int(B.shape[1]), out.data_ptr(), torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("F, dtype", [(64, torch.float32), (256, torch.float32),
                                      (256, torch.bfloat16)])
def test_noalloc_matches_workspace_entry_point(cuda, F, dtype):
    g = G.flickr_like()
    A = ops.CSR(g.rowptr.to(cuda), g.colind.to(cuda), g.vals.to(cuda), g.nrows, g.ncols)
    B = G.normal(F, 6, (g.ncols, F)).to(dtype).to(cuda)
    ref = ops.csr_spmm(A, B)
    absA = ops.CSR(A.rowptr, A.colind, A.vals.abs(), g.nrows, g.ncols)
    scale = ops.csr_spmm(absA, B.float().abs()).clamp_min(1e-30)
    for _ in range(2):
        out = torch.full((g.nrows, F), float("nan"), device=cuda)
        _noalloc(A, B, out)
        torch.cuda.synchronize()
        rel = ((out - ref).abs() / scale).max().item()
        assert rel <= 1e-5, rel


def test_noalloc_rejects_unsupported_width(cuda):
    g = G.uniform_rows(64, 4)
    A = ops.CSR(g.rowptr.to(cuda), g.colind.to(cuda), g.vals.to(cuda), g.nrows, g.ncols)
    B = torch.zeros(64, 4096, device=cuda)
    out = torch.empty(64, 4096, device=cuda)
    with pytest.raises(_lib.GbsError):
        _noalloc(A, B, out)
