"""GPU parity of the merge-path CSR SpMM against the FP64 CPU oracle and
against cuSPARSE (the library the reference verifies with,
test_spmm_full.cu:279-307).

Tolerances (stated per test):
  * FP32 features: max relative error <= 1e-5 against FP64, where the error
    of C[i,k] is scaled by M[i,k] = sum_j |A_ij| |B_jk| (the scale of the
    rounding bound of a sum of products; |C| itself can be ~0 by
    cancellation).
  * BF16 / FP16 features: the same measure against the FP64 product of the
    *rounded* features <= 1e-5 (accumulation), and against the FP64 product
    of the FP32 features <= 1e-2 (incl. the storage rounding).
"""
import numpy as np
import pytest
import torch

import oracle
from spmm_eval_gb300 import graphs as G
from spmm_eval_gb300 import ops

pytestmark = pytest.mark.gpu


def dev_csr(g, dev, with_vals=True):
    return ops.CSR(g.rowptr.to(dev), g.colind.to(dev), g.vals.to(dev) if with_vals else None,
                   g.nrows, g.ncols)


def check_f32(g, B, C, vals=True, tol=1e-5):
    ref, mag = oracle.csr_spmm_f64(g.rowptr.numpy(), g.colind.numpy(),
                                   g.vals.numpy() if vals else None, B.numpy())
    mx, mean = oracle.rel_err(C.cpu().numpy(), ref, mag)
    assert mx <= tol, (mx, mean)
    return mx, mean


def small_graph(n, m, density, seed, empty_rows=()):
    rng = np.random.default_rng(seed)
    mask = rng.random((n, m)) < density
    for r in empty_rows:
        mask[r] = False
    rows, cols = np.nonzero(mask)
    counts = np.bincount(rows, minlength=n)
    rowptr = np.zeros(n + 1, np.int32)
    rowptr[1:] = np.cumsum(counts)
    vals = rng.uniform(-1, 1, rows.size).astype(np.float32)
    return G.Graph(torch.from_numpy(rowptr), torch.from_numpy(cols.astype(np.int32)),
                   torch.from_numpy(vals), n, m)


def test_uniform_4096x16_f32(cuda):
    """4096 x 4096, 16 distinct uniform columns per row, B 4096 x 32 N(0,1)."""
    g = G.uniform_rows(4096, 16)
    B = G.normal(0x5EED + 1, 3, (4096, 32))
    C = ops.csr_spmm(dev_csr(g, cuda), B.to(cuda))
    check_f32(g, B, C)


def test_matches_cusparse(cuda):
    """Agreement with cusparseSpMM (reached through torch's CSR matmul)."""
    g = G.uniform_rows(4096, 16)
    B = G.normal(7, 3, (4096, 64)).to(cuda)
    A = torch.sparse_csr_tensor(g.rowptr.long(), g.colind.long(), g.vals, (4096, 4096)).to(cuda)
    ref = (A @ B).float()
    C = ops.csr_spmm(dev_csr(g, cuda), B)
    scale = (torch.sparse_csr_tensor(g.rowptr.long(), g.colind.long(), g.vals.abs(),
                                     (4096, 4096)).to(cuda) @ B.abs())
    rel = ((C - ref).abs() / scale.clamp_min(1e-30)).max().item()
    assert rel <= 2e-6, rel


@pytest.mark.parametrize("F", [1, 3, 4, 8, 16, 24, 32, 40, 64, 100, 128, 136, 152, 200, 252, 256, 260, 512,
                               1024])
def test_feature_widths_f32(cuda, F):
    g = small_graph(300, 257, 0.05, F, empty_rows=(0, 17, 299))
    B = G.normal(F, 1, (257, F))
    C = ops.csr_spmm(dev_csr(g, cuda), B.to(cuda))
    check_f32(g, B, C)


def test_binary_values_null(cuda):
    g = small_graph(200, 200, 0.1, 5)
    B = G.normal(5, 1, (200, 64))
    C = ops.csr_spmm(dev_csr(g, cuda, with_vals=False), B.to(cuda))
    check_f32(g, B, C, vals=False)


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("F", [8, 32, 64, 136, 200, 256, 264, 1024, 2048])
def test_half_features(cuda, dtype, F):
    g = small_graph(257, 300, 0.04, F + 1)
    B32 = G.normal(F, 2, (300, F))
    Bh = B32.to(dtype)
    C = ops.csr_spmm(dev_csr(g, cuda), Bh.to(cuda))
    # accumulation error alone (against the rounded features)
    check_f32(g, Bh.float(), C, tol=1e-5)
    # total error including storage rounding
    check_f32(g, B32, C, tol=1e-2)


def test_power_law_rows_split_across_warps(cuda):
    """flickr-shaped graph: hub rows are cut by merge-path boundaries."""
    g = G.flickr_like()
    for F in (32, 64, 128, 256):
        B = G.normal(F, 4, (g.ncols, F))
        C = ops.csr_spmm(dev_csr(g, cuda), B.to(cuda))
        check_f32(g, B, C)


def test_one_long_row_many_warps(cuda):
    """A single row holding every nonzero spans every warp's share."""
    n, m, deg = 3, 5000, 4999
    rowptr = torch.tensor([0, 0, deg, deg], dtype=torch.int32)
    colind = torch.arange(deg, dtype=torch.int32)
    vals = torch.ones(deg)
    g = G.Graph(rowptr, colind, vals, n, m)
    B = G.normal(11, 1, (m, 64))
    C = ops.csr_spmm(dev_csr(g, cuda), B.to(cuda))
    check_f32(g, B, C)
    assert torch.all(C[0] == 0) and torch.all(C[2] == 0)


def test_no_nonzeros_writes_zeros(cuda):
    g = G.Graph(torch.zeros(6, dtype=torch.int32), torch.zeros(0, dtype=torch.int32),
                torch.zeros(0), 5, 4)
    out = torch.full((5, 16), 7.0, device=cuda)
    ops.csr_spmm(dev_csr(g, cuda), torch.zeros(4, 16, device=cuda), out=out)
    assert torch.all(out == 0)


def test_deterministic_and_workspace_left_zero(cuda):
    """Two calls on one workspace and one on a fresh zero workspace agree
    bitwise: the arrival counters are back to zero after every call."""
    g = G.flickr_like()
    B = G.normal(3, 4, (g.ncols, 128)).to(cuda)
    ws = ops.SpmmWorkspace()
    A = dev_csr(g, cuda)
    c1 = ops.csr_spmm(A, B, workspace=ws).clone()
    c2 = ops.csr_spmm(A, B, workspace=ws).clone()
    c3 = ops.csr_spmm(A, B, workspace=ops.SpmmWorkspace())
    assert torch.equal(c1, c2) and torch.equal(c1, c3)


def test_reddit_scale_properties(cuda):
    """Full-size power-law graph (232,965 nodes, ~114.6M edges, F = 256):
    linearity in B and an FP64 check on sampled rows incl. the largest hubs."""
    g = G.reddit_like(device=cuda)
    g = G.gcn_normalize(g)
    A = ops.CSR(g.rowptr, g.colind, g.vals, g.nrows, g.ncols)
    B1 = G.normal(1, 5, (g.ncols, 256), device=cuda)
    B2 = G.normal(2, 5, (g.ncols, 256), device=cuda)
    C1 = ops.csr_spmm(A, B1)
    C2 = ops.csr_spmm(A, B2)
    C12 = ops.csr_spmm(A, B1 + B2)
    scale = ops.csr_spmm(ops.CSR(g.rowptr, g.colind, g.vals.abs(), g.nrows, g.ncols),
                         B1.abs() + B2.abs())
    lin = ((C12 - (C1 + C2)).abs() / scale.clamp_min(1e-30)).max().item()
    assert lin <= 1e-5, lin
    deg = (g.rowptr[1:] - g.rowptr[:-1]).cpu()
    rows = torch.cat([torch.topk(deg, 16).indices, torch.arange(0, g.nrows, 997)]).numpy()
    ref, mag = oracle.csr_spmm_f64(g.rowptr.cpu().numpy(), g.colind.cpu().numpy(),
                                   g.vals.cpu().numpy(), B1.cpu().numpy(), rows=rows)
    mx, _ = oracle.rel_err(C1.cpu().numpy()[rows], ref, mag)
    assert mx <= 1e-5, mx


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16, torch.float32])
def test_reddit_scale_feature_types(cuda, dtype):
    """The 232,965-node graph at F = 256 with FP32, BF16 or FP16 features
    through the planned SpMM, on sampled rows incl. the 16 largest hubs:
    scaled error <= 1e-5 against the FP64 product of the features as stored
    (accumulation), <= 1e-2 for 16-bit features against the FP64 product of
    the FP32 features (incl. the storage rounding), and the plain relative
    error |C - C64| / |C64| <= 1e-2 (16-bit) / 1e-5 (FP32) over the entries
    whose |C64| is at least the RMS of C64 on those rows."""
    g = G.gcn_normalize(G.reddit_like(device=cuda))
    A = ops.CSR(g.rowptr, g.colind, g.vals, g.nrows, g.ncols)
    B32 = G.normal(4, 5, (g.ncols, 256), device=cuda)
    Bx = B32.to(dtype)
    C = ops.SpmmPlan(A, 256, dtype).run(Bx)
    deg = (g.rowptr[1:] - g.rowptr[:-1]).cpu()
    rows = torch.cat([torch.topk(deg, 16).indices, torch.arange(0, g.nrows, 1999)]).numpy()
    rp, ci, va = g.rowptr.cpu().numpy(), g.colind.cpu().numpy(), g.vals.cpu().numpy()
    got = C.cpu().numpy()[rows]
    ref_s, mag_s = oracle.csr_spmm_f64(rp, ci, va, Bx.float().cpu().numpy(), rows=rows)
    assert oracle.rel_err(got, ref_s, mag_s)[0] <= 1e-5
    ref, mag = oracle.csr_spmm_f64(rp, ci, va, B32.cpu().numpy(), rows=rows)
    assert oracle.rel_err(got, ref, mag)[0] <= (1e-2 if dtype != torch.float32 else 1e-5)
    floor = float(np.sqrt(np.mean(ref ** 2)))
    keep = np.abs(ref) >= floor
    plain = float(np.max(np.abs(got[keep] - ref[keep]) / np.abs(ref[keep])))
    assert plain <= (1e-2 if dtype != torch.float32 else 1e-5), plain


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("cb", [8, 32, 64, 128, 256])
def test_column_blocks(cuda, dtype, cb):
    """Forced column-block widths give the same result as one full-width
    launch (each column is summed in the same order in both)."""
    g = G.flickr_like()
    B = G.normal(9, 4, (g.ncols, 256)).to(dtype)
    A = dev_csr(g, cuda)
    full = ops.csr_spmm(A, B.to(cuda), col_block=256)
    if dtype == torch.bfloat16 and cb == 8:
        cb = 16
    part = ops.csr_spmm(A, B.to(cuda), col_block=cb)
    # The lane split of a row changes with the block width (sub-group count),
    # so both are checked against FP64, not bitwise against each other.
    check_f32(g, B.float(), part)
    check_f32(g, B.float(), full)


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("dtype, vals", [(torch.float32, True), (torch.bfloat16, True), (torch.float32, False)])
def test_host_buffer_pipelined(cuda, pinned, dtype, vals):
    """gbs_csr_spmm_host (host A/B in, host C out, copies overlapped in row
    ranges) against the FP64 oracle."""
    g = G.flickr_like()
    B32 = G.normal(21, 4, (g.ncols, 128))
    Bh = B32.to(dtype)
    args = [g.rowptr, g.colind, g.vals if vals else None, Bh]
    if pinned:
        args = [a.pin_memory() if a is not None else None for a in args]
    C = ops.csr_spmm_host(*args, g.nrows, g.ncols)
    assert not C.is_cuda
    check_f32(g, Bh.float(), C, vals=vals)
    ctx = ops.HostSpmmContext()
    for _ in range(2):  # buffers kept in the context
        C2 = ops.csr_spmm_host(*args, g.nrows, g.ncols, ctx=ctx)
        check_f32(g, Bh.float(), C2, vals=vals)


@pytest.mark.parametrize("dtype, F", [(torch.float32, 256), (torch.float32, 512), (torch.bfloat16, 512)])
def test_host_buffer_wide_features(cuda, dtype, F):
    """Host-buffer SpMM with B larger than half of L2 (FP32 F = 256, 512;
    BF16 F = 512) against the FP64 oracle."""
    g = G.flickr_like()
    B32 = G.normal(F, 5, (g.ncols, F))
    Bh = B32.to(dtype)
    args = [t.pin_memory() for t in (g.rowptr, g.colind, g.vals, Bh)]
    ctx = ops.HostSpmmContext()
    C = ops.csr_spmm_host(*args, g.nrows, g.ncols, ctx=ctx)
    check_f32(g, Bh.float(), C)


def test_workspace_reused_across_shapes(cuda):
    """One workspace serving different shapes (different warp counts and
    slot widths) in sequence: each result still matches FP64."""
    ws = ops.SpmmWorkspace()
    big = G.flickr_like()
    small = small_graph(300, 257, 0.05, 3)
    for g, F in ((big, 256), (small, 64), (big, 32), (small, 256), (big, 128)):
        B = G.normal(F, 9, (g.ncols, F))
        C = ops.csr_spmm(dev_csr(g, cuda), B.to(cuda), workspace=ws)
        check_f32(g, B, C)


@pytest.mark.parametrize("parts", [1, 2, 3, 4, 8])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_column_partitioned_plan(cuda, parts, dtype):
    """Column-partitioned plan: K accumulating passes equal the FP64 product
    (hub rows split across warps in every pass)."""
    g = G.flickr_like()
    B = G.normal(parts, 12, (g.ncols, 128)).to(dtype)
    A = dev_csr(g, cuda)
    plan = ops.SpmmPlan(A, 128, dtype, parts=parts)
    assert plan.parts == parts
    C = plan.run(B.to(cuda))
    check_f32(g, B.float(), C)
    C2 = plan.run(B.to(cuda))  # reusable
    assert torch.equal(C, C2)


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_column_partitioned_plan_f256(cuda, dtype):
    """F = 256 (the half-warp variants run when a part's B slice fits in half
    of L2): the automatic split and an explicit one against FP64."""
    g = G.flickr_like()
    B = G.normal(7, 12, (g.ncols, 256)).to(dtype)
    A = dev_csr(g, cuda)
    for parts in (0, 3):
        plan = ops.SpmmPlan(A, 256, dtype, parts=parts)
        check_f32(g, B.float(), plan.run(B.to(cuda)))


def test_plan_auto_parts(cuda):
    g = G.uniform_rows(4096, 16)
    plan = ops.SpmmPlan(dev_csr(g, cuda), 32)
    assert plan.parts == 1  # B is tiny: no split
    fl = G.flickr_like()
    assert ops.SpmmPlan(dev_csr(fl, cuda), 256).parts == 1  # ~10 nonzeros per column: no split
