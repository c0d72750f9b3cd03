"""GPU test of gbs_csr_spmm_noalloc, the CSR SpMM entry point that allocates
no device memory (for callers that may not call cudaMalloc while they run,
e.g. a framework that owns all device memory through its own pool, or a
serving loop that forbids allocation on the request path).

It is called twice in a row through the C ABI on a power-law graph whose
hub rows are split across warps (so the shared scratch array's partial
slots and arrival counters are exercised, and the second call starts from
whatever the first left behind), and each result is compared with the
workspace-based gbs_csr_spmm on the same inputs, within the tolerance the
other SpMM tests use (max |diff| / (|A| |B|) <= 1e-5).  The widths cover
FP32 (16-byte and scalar loads), BF16 and FP16, and rows wide enough that
the warp count is cut to fit the 8 MiB array.  This file is named to be
collected last.
"""
import pytest
import torch

from spmm_eval_gb300 import _lib
from spmm_eval_gb300 import graphs as G
from spmm_eval_gb300 import ops

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 8 << 20


def _noalloc(A, B, out):
    _lib.call("gbs_csr_spmm_noalloc", A.nrows, A.ncols, A.nnz, A.rowptr.data_ptr(),
              A.colind.data_ptr(), A.vals.data_ptr(), B.data_ptr(), ops._DT[B.dtype],
              int(B.shape[1]), out.data_ptr(), torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("F, dtype", [(64, torch.float32), (256, torch.float32), (33, torch.float32),
                                      (1024, torch.float32), (256, torch.bfloat16),
                                      (2048, torch.bfloat16), (128, torch.float16)])
def test_noalloc_matches_workspace_entry_point(cuda, F, dtype):
    g = G.flickr_like()
    A = ops.CSR(g.rowptr.to(cuda), g.colind.to(cuda), g.vals.to(cuda), g.nrows, g.ncols)
    B = G.normal(F, 6, (g.ncols, F)).to(dtype).to(cuda)
    if F >= 1024:
        # the smallest resident wave (one 8-warp CTA per SM) would need more
        # partial-sum rows than the array holds, so the warp count is cut
        sms = torch.cuda.get_device_properties(cuda).multi_processor_count
        assert 2 * sms * 8 * F * 4 > SCRATCH_BYTES
        assert (g.nrows + g.nnz) // 256 > sms * 8
    ref = ops.csr_spmm(A, B)
    absA = ops.CSR(A.rowptr, A.colind, A.vals.abs(), g.nrows, g.ncols)
    # FP32 rows wider than 1024 columns run in column blocks of 1024
    scale = ops.csr_spmm(absA, B.float().abs(), col_block=1024 if F > 1024 else 0).clamp_min(1e-30)
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
