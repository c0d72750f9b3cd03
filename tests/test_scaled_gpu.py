"""GPU parity of the degree-normalised SpMM (gbs_csr_spmm_scaled and its
plan): C[r] = rowscale[r] * sum_c colscale[c] B[c] over the stored entries
of a binary A -- the GCN propagation D^-1/2 A D^-1/2 B with the
normalisation folded into the kernel instead of a value array.

Checked against the FP64 oracle of the valued product with values
d[r] * d[c] computed in FP64 (the normalised graphs of the evaluation),
scaled error |C - C64| / (|A| |B|) <= 1e-5 for FP32 features and against
the rounded features for BF16 / FP16; and the FP64-computed D^-1/2 factors
bit for bit against numpy's FP64 1/sqrt rounded to FP32.
"""
import numpy as np
import pytest
import torch

import oracle
from spmm_eval_gb300 import graphs as G
from spmm_eval_gb300 import ops

pytestmark = pytest.mark.gpu


def dinv_np(rp):
    deg = np.diff(rp).astype(np.float64)
    with np.errstate(divide="ignore"):
        d = np.where(deg > 0, 1.0 / np.sqrt(deg), 0.0)
    return d


def valued(rp, ci, rs, cs):
    """FP32 values rs[r] * cs[c] computed in FP64 (the oracle's A)."""
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    r = np.ones(rows.size) if rs is None else rs.astype(np.float64)[rows]
    c = np.ones(ci.size) if cs is None else cs.astype(np.float64)[ci]
    return r * c


def check(rp, ci, rs, cs, Bq, got, rows=None, tol=1e-5):
    v = valued(rp, ci, rs, cs)
    ref, mag = oracle.csr_spmm_f64(rp, ci, v.astype(np.float32), Bq, rows=rows)
    # the oracle's FP32 values round d[r] d[c] once; bound that against the
    # FP64 product of the FP64 values on the same rows
    mx = oracle.rel_err(got, ref, mag)[0]
    assert mx <= tol, mx


def small_graph(n, m, density, seed):
    rng = np.random.default_rng(seed)
    mask = rng.random((n, m)) < density
    mask[3] = False  # an empty row
    rows, cols = np.nonzero(mask)
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(np.bincount(rows, minlength=n))
    return rp, cols.astype(np.int32)


def test_degree_rsqrt_bitwise(cuda):
    g = G.flickr_like()
    A = ops.CSR(g.rowptr.to(cuda), g.colind.to(cuda), None, g.nrows, g.ncols)
    got = ops.degree_rsqrt(A).cpu().numpy()
    want = dinv_np(g.rowptr.numpy()).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("F", [1, 8, 33, 64, 256, 1024])
@pytest.mark.parametrize("which", ["both", "row", "col", "none"])
def test_scaled_small(cuda, F, which):
    n, m = 300, 257
    rp, ci = small_graph(n, m, 0.05, F)
    rng = np.random.default_rng(F + 1)
    rs = rng.uniform(0.1, 2.0, n).astype(np.float32) if which in ("both", "row") else None
    cs = rng.uniform(0.1, 2.0, m).astype(np.float32) if which in ("both", "col") else None
    B = G.normal(F, 3, (m, F))
    A = ops.CSR(torch.from_numpy(rp).to(cuda), torch.from_numpy(ci).to(cuda), None, n, m)
    t = (lambda x: None if x is None else torch.from_numpy(x).to(cuda))
    C = ops.csr_spmm_scaled(A, t(rs), t(cs), B.to(cuda))
    check(rp, ci, rs, cs, B.numpy(), C.cpu().numpy())
    assert torch.all(C[3] == 0)


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16, torch.float16])
@pytest.mark.parametrize("F", [64, 128, 256])
def test_gcn_normalised_flickr(cuda, dtype, F):
    """The normalised 89,250-node graph of the GCN-layer configuration, one
    launch and the plan, FP32 / BF16 / FP16 features."""
    g = G.flickr_like()
    rp, ci = g.rowptr.numpy(), g.colind.numpy()
    A = ops.CSR(g.rowptr.to(cuda), g.colind.to(cuda), None, g.nrows, g.ncols)
    d = ops.degree_rsqrt(A)
    B = G.normal(F, 7, (g.ncols, F)).to(dtype)
    Bq = B.float().numpy()
    dn = d.cpu().numpy()
    C1 = ops.csr_spmm_scaled(A, d, d, B.to(cuda))
    check(rp, ci, dn, dn, Bq, C1.cpu().numpy())
    C2 = ops.SpmmPlan(A, F, dtype, rowscale=d, colscale=d).run(B.to(cuda))
    check(rp, ci, dn, dn, Bq, C2.cpu().numpy())
    # the same graph with FP32 values D^-1/2 A D^-1/2 through the valued path
    gn = G.gcn_normalize(g)
    Cv = ops.csr_spmm(ops.CSR(A.rowptr, A.colind, gn.vals.to(cuda), g.nrows, g.ncols), B.to(cuda))
    absd = ops.csr_spmm_scaled(A, d, d, B.to(cuda).float().abs())
    assert float(((C1 - Cv).abs() / absd.clamp_min(1e-30)).max()) <= 2e-6


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_reddit_scale_planned(cuda, dtype):
    """The 232,965-node graph at F = 256 through the column-partitioned plan
    (2 parts, so later parts accumulate row-scaled partials): sampled rows
    incl. the 16 largest hubs against FP64."""
    g = G.reddit_like(device=cuda)
    A = ops.CSR(g.rowptr, g.colind, None, g.nrows, g.ncols)
    d = ops.degree_rsqrt(A)
    B = G.normal(4, 5, (g.ncols, 256), device=cuda).to(dtype)
    plan = ops.SpmmPlan(A, 256, dtype, parts=2, rowscale=d, colscale=d)
    assert plan.parts == 2
    C = plan.run(B)
    deg = (g.rowptr[1:] - g.rowptr[:-1]).cpu()
    rows = torch.cat([torch.topk(deg, 16).indices, torch.arange(0, g.nrows, 1999)]).numpy()
    rp, ci = g.rowptr.cpu().numpy(), g.colind.cpu().numpy()
    dn = d.cpu().numpy()
    check(rp, ci, dn, dn, B.float().cpu().numpy(), C.cpu().numpy()[rows], rows=rows)
