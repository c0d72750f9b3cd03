"""GPU tests of the backward kernels: CSR transpose (exact vs the oracle),
A^T dC and SDDMM (vs FP64 CPU oracles), and the GCN layer
Y = A_hat (X W), loss = sum(Y * G) on the normalised flickr-shaped graph:
gradients vs an FP64 reference, and a gradcheck against FP64 central finite
differences (eps 1e-6) on a 512-node induced subgraph, in FP32 and
BF16-feature modes.

Error measure: |got - ref| / S with S the matching magnitude sum
(|A| |B| for products); tolerances are stated per test."""
import numpy as np
import pytest
import torch

import oracle
from spmm_eval_gb300 import graphs as G
from spmm_eval_gb300 import ops
from tests.gcn_autograd import gcn_layer

pytestmark = pytest.mark.gpu


def rand_csr(n, m, dens, seed):
    rng = np.random.default_rng(seed)
    mask = rng.random((n, m)) < dens
    mask[::11] = False
    mask[:, ::13] = False
    r, c = np.nonzero(mask)
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(np.bincount(r, minlength=n))
    return G.Graph(torch.from_numpy(rp), torch.from_numpy(c.astype(np.int32)),
                   torch.from_numpy(rng.uniform(-1, 1, r.size).astype(np.float32)), n, m)


def dev(g, d, vals=True):
    return ops.CSR(g.rowptr.to(d), g.colind.to(d), g.vals.to(d) if vals else None, g.nrows, g.ncols)


@pytest.mark.parametrize("which", ["rand", "flickr"])
def test_transpose_exact(cuda, which):
    g = rand_csr(300, 170, 0.05, 1) if which == "rand" else G.flickr_like()
    T = ops.CSRTranspose(dev(g, cuda))
    rp, ci, pm = T.arrays()
    wrp, wci, wpm = oracle.csr_transpose(g.nrows, g.ncols, g.rowptr.numpy(), g.colind.numpy())
    assert np.array_equal(rp.cpu().numpy(), wrp)
    assert np.array_equal(ci.cpu().numpy(), wci)
    assert np.array_equal(pm.cpu().numpy(), wpm)
    tv = T.values(g.vals.to(cuda)).cpu().numpy()
    assert np.array_equal(tv, g.vals.numpy()[wpm])


@pytest.mark.parametrize("F", [16, 64, 256])
def test_transposed_spmm(cuda, F):
    g = rand_csr(400, 250, 0.04, F)
    T = ops.CSRTranspose(dev(g, cuda))
    dC = G.normal(F, 1, (400, F))
    dB = T.spmm(T.values(g.vals.to(cuda)), dC.to(cuda)).cpu().numpy()
    wrp, wci, wpm = oracle.csr_transpose(400, 250, g.rowptr.numpy(), g.colind.numpy())
    ref, mag = oracle.csr_spmm_f64(wrp, wci, g.vals.numpy()[wpm], dC.numpy())
    assert oracle.rel_err(dB, ref, mag)[0] <= 1e-5


def sddmm_scale(rp, ci, Gm, Hm):
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    return np.einsum("ek,ek->e", np.abs(Gm[rows]).astype(np.float64), np.abs(Hm[ci]).astype(np.float64))


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16, torch.float16])
@pytest.mark.parametrize("F", [8, 64, 128, 256])
def test_sddmm(cuda, dtype, F):
    g = G.flickr_like()
    Gm = G.normal(F, 2, (g.nrows, F))
    Hm = G.normal(F, 3, (g.ncols, F))
    out = ops.sddmm(dev(g, cuda, False), Gm.to(dtype).to(cuda), Hm.to(dtype).to(cuda)).cpu().numpy()
    rp, ci = g.rowptr.numpy(), g.colind.numpy()
    Gr, Hr = Gm.to(dtype).float().numpy(), Hm.to(dtype).float().numpy()
    ref = oracle.sddmm_f64(rp, ci, Gr, Hr)
    S = sddmm_scale(rp, ci, Gr, Hr)
    assert np.max(np.abs(out - ref) / np.maximum(S, 1e-30)) <= 1e-5  # accumulation
    ref32 = oracle.sddmm_f64(rp, ci, Gm.numpy(), Hm.numpy())
    S32 = sddmm_scale(rp, ci, Gm.numpy(), Hm.numpy())
    tol = 1e-5 if dtype == torch.float32 else 1e-2
    assert np.max(np.abs(out - ref32) / np.maximum(S32, 1e-30)) <= tol  # incl. feature rounding


class Pattern:
    def __init__(self, g, d):
        self.rowptr, self.colind = g.rowptr.to(d), g.colind.to(d)
        self.nrows, self.ncols = g.nrows, g.ncols


@pytest.mark.parametrize("feat_dtype, tol", [(torch.float32, 1e-5), (torch.bfloat16, 1e-2)])
def test_gcn_layer_grads_vs_fp64(cuda, feat_dtype, tol):
    """89,250-node normalised graph, X 89,250 x 512, W 512 x 128 (Glorot
    uniform), loss = sum(Y * G): dvals, dH (and dX, dW through torch) against
    FP64 CPU references."""
    g = G.gcn_normalize(G.flickr_like())
    n = g.nrows
    X = G.normal(51, 1, (n, 512)).to(cuda)
    bound = (6.0 / (512 + 128)) ** 0.5
    W = (torch.rand(512, 128, generator=torch.Generator().manual_seed(52)) * 2 - 1) * bound
    W = W.to(cuda)
    Gm = G.normal(53, 1, (n, 128)).to(cuda)
    pat = Pattern(g, cuda)
    T = ops.CSRTranspose(ops.CSR(pat.rowptr, pat.colind, None, n, n))
    vals = g.vals.to(cuda).requires_grad_(True)
    Xr, Wr = X.clone().requires_grad_(True), W.clone().requires_grad_(True)
    Y = gcn_layer(vals, Xr, Wr, pat, T, feat_dtype)
    (Y * Gm).sum().backward()
    # FP64 references on the CPU
    H = (X @ W).double().cpu().numpy()
    Gn = Gm.double().cpu().numpy()
    rp, ci, v = g.rowptr.numpy(), g.colind.numpy(), g.vals.numpy()
    wrp, wci, wpm = oracle.csr_transpose(n, n, rp, ci)
    dH, magH = oracle.csr_spmm_f64(wrp, wci, v[wpm], Gn.astype(np.float32))
    dv = oracle.sddmm_f64(rp, ci, Gn.astype(np.float32), H.astype(np.float32))
    Sv = sddmm_scale(rp, ci, Gn, H)
    got_dv = vals.grad.cpu().numpy()
    assert np.max(np.abs(got_dv - dv) / np.maximum(Sv, 1e-30)) <= tol
    dX_ref = dH @ W.double().cpu().numpy().T
    dW_ref = X.double().cpu().numpy().T @ dH
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    assert rel(Xr.grad.cpu().numpy(), dX_ref) <= max(tol, 1e-4)
    assert rel(Wr.grad.cpu().numpy(), dW_ref) <= max(tol, 1e-4)


@pytest.mark.parametrize("feat_dtype, rtol", [(torch.float32, 1e-4), (torch.bfloat16, 2e-2)])
def test_gradcheck_fd_512_subgraph(cuda, feat_dtype, rtol):
    """Gradients from the kernels vs FP64 central finite differences
    (eps = 1e-6) of the FP64 loss on a 512-node induced subgraph, and vs
    the dense FP64 analytic gradient."""
    full = G.gcn_normalize(G.flickr_like())
    deg = full.degrees()
    nodes = torch.argsort(deg, descending=True)[:512]  # well-connected block
    g = G.induced_subgraph(full, nodes)
    n, Fi, Fo = g.nrows, 16, 8
    X = G.normal(61, 1, (n, Fi)).double().to(cuda)
    W = G.normal(62, 1, (Fi, Fo)).double().to(cuda) * 0.3
    Gm = G.normal(63, 1, (n, Fo)).double().to(cuda)
    rows = torch.repeat_interleave(torch.arange(n), g.degrees()).to(cuda)
    cols = g.colind.long().to(cuda)

    def loss64(vals, X, W):
        A = torch.zeros(n, n, dtype=torch.float64, device=cuda)
        A[rows, cols] = vals
        return ((A @ (X @ W)) * Gm).sum()

    v64 = g.vals.double().to(cuda)
    # kernels (FP32 / BF16 features)
    pat = Pattern(g, cuda)
    T = ops.CSRTranspose(ops.CSR(pat.rowptr, pat.colind, None, n, n))
    vals = g.vals.to(cuda).requires_grad_(True)
    Xr, Wr = X.float().clone().requires_grad_(True), W.float().clone().requires_grad_(True)
    (gcn_layer(vals, Xr, Wr, pat, T, feat_dtype) * Gm.float()).sum().backward()
    # dense FP64 analytic
    va, Xa, Wa = v64.clone().requires_grad_(True), X.clone().requires_grad_(True), W.clone().requires_grad_(True)
    loss64(va, Xa, Wa).backward()
    for got, ref in ((vals.grad, va.grad), (Xr.grad, Xa.grad), (Wr.grad, Wa.grad)):
        assert (got.double() - ref).abs().max() <= rtol * ref.abs().max(), (got, ref)
    # FP64 central differences on a sample of coordinates
    eps = 1e-6
    rng = np.random.default_rng(0)
    for name, base, grad in (("vals", v64, vals.grad), ("X", X, Xr.grad), ("W", W, Wr.grad)):
        flat = base.reshape(-1)
        for idx in rng.choice(flat.numel(), size=12, replace=False):
            e = torch.zeros_like(flat)
            e[idx] = eps
            args_p = {"vals": v64, "X": X, "W": W}
            args_m = dict(args_p)
            args_p[name] = (flat + e).reshape(base.shape)
            args_m[name] = (flat - e).reshape(base.shape)
            fd = (loss64(**args_p) - loss64(**args_m)) / (2 * eps)
            g_k = grad.reshape(-1)[idx].double()
            scale = grad.abs().max().double()
            assert abs(g_k - fd) <= rtol * scale + 1e-7, (name, idx, float(g_k), float(fd))


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("F", [8, 32, 64, 256])
def test_fused_backward_matches_separate(cuda, dtype, F):
    """gbs_spmm_backward (A^T SpMM + SDDMM in one pass) against FP64 oracles
    of both outputs."""
    g = G.gcn_normalize(G.flickr_like())
    n = g.nrows
    Gm = G.normal(F, 21, (n, F))
    Hm = G.normal(F, 22, (n, F))
    Gd, Hd = Gm.to(dtype).to(cuda), Hm.to(dtype).to(cuda)
    T = ops.CSRTranspose(dev(g, cuda, False))
    tv = T.values(g.vals.to(cuda))
    dB, dv = ops.spmm_backward(T, tv, Gd, Hd)
    rp, ci, v = g.rowptr.numpy(), g.colind.numpy(), g.vals.numpy()
    Gr, Hr = Gd.float().cpu().numpy(), Hd.float().cpu().numpy()
    wrp, wci, wpm = oracle.csr_transpose(n, n, rp, ci)
    ref, mag = oracle.csr_spmm_f64(wrp, wci, v[wpm], Gr)
    assert oracle.rel_err(dB.cpu().numpy(), ref, mag)[0] <= 1e-5
    refv = oracle.sddmm_f64(rp, ci, Gr, Hr)
    S = sddmm_scale(rp, ci, Gr, Hr)
    assert np.max(np.abs(dv.cpu().numpy() - refv) / np.maximum(S, 1e-30)) <= 1e-5


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("parts", [1, 2, 3, 4])
def test_planned_backward(cuda, dtype, parts):
    """gbs_spmm_backward_planned (A^T split by row ranges of A, accumulating
    dB passes) against FP64 oracles of both outputs and against the one-pass
    fused backward."""
    g = G.gcn_normalize(G.flickr_like())
    n, F = g.nrows, 64
    Gm = G.normal(F, 23, (n, F))
    Hm = G.normal(F, 24, (n, F))
    Gd, Hd = Gm.to(dtype).to(cuda), Hm.to(dtype).to(cuda)
    T = ops.CSRTranspose(dev(g, cuda, False))
    tv = T.values(g.vals.to(cuda))
    plan = ops.BackwardPlan(T, tv, F, dtype, parts)
    assert plan.parts == parts
    dB, dv = plan.run(Gd, Hd)
    dB1, dv1 = ops.spmm_backward(T, tv, Gd, Hd)
    rp, ci, v = g.rowptr.numpy(), g.colind.numpy(), g.vals.numpy()
    Gr, Hr = Gd.float().cpu().numpy(), Hd.float().cpu().numpy()
    wrp, wci, wpm = oracle.csr_transpose(n, n, rp, ci)
    ref, mag = oracle.csr_spmm_f64(wrp, wci, v[wpm], Gr)
    assert oracle.rel_err(dB.cpu().numpy(), ref, mag)[0] <= 1e-5
    refv = oracle.sddmm_f64(rp, ci, Gr, Hr)
    S = sddmm_scale(rp, ci, Gr, Hr)
    assert np.max(np.abs(dv.cpu().numpy() - refv) / np.maximum(S, 1e-30)) <= 1e-5
    assert torch.allclose(dB, dB1, rtol=1e-5, atol=1e-6)
    assert torch.allclose(dv, dv1, rtol=1e-5, atol=1e-6)
    if parts == 1:
        assert torch.equal(dB, dB1) and torch.equal(dv, dv1)


@pytest.mark.parametrize("dtype, F", [(torch.float32, 4), (torch.float32, 200), (torch.float32, 1024),
                                      (torch.bfloat16, 8), (torch.bfloat16, 136), (torch.bfloat16, 2048)])
def test_planned_backward_widths(cuda, dtype, F):
    """Feature widths across the backward variants (3 parts)."""
    g = G.gcn_normalize(G.uniform_rows(3000, 12))
    n = g.nrows
    Gd = G.normal(F, 41, (n, F)).to(dtype).to(cuda)
    Hd = G.normal(F, 42, (n, F)).to(dtype).to(cuda)
    T = ops.CSRTranspose(dev(g, cuda, False))
    tv = T.values(g.vals.to(cuda))
    dB, dv = ops.BackwardPlan(T, tv, F, dtype, 3).run(Gd, Hd)
    rp, ci, v = g.rowptr.numpy(), g.colind.numpy(), g.vals.numpy()
    Gr, Hr = Gd.float().cpu().numpy(), Hd.float().cpu().numpy()
    wrp, wci, wpm = oracle.csr_transpose(n, n, rp, ci)
    ref, mag = oracle.csr_spmm_f64(wrp, wci, v[wpm], Gr)
    assert oracle.rel_err(dB.cpu().numpy(), ref, mag)[0] <= 1e-5
    refv = oracle.sddmm_f64(rp, ci, Gr, Hr)
    S = sddmm_scale(rp, ci, Gr, Hr)
    assert np.max(np.abs(dv.cpu().numpy() - refv) / np.maximum(S, 1e-30)) <= 1e-5


@pytest.mark.parametrize("dtype, K", [(torch.float32, 4), (torch.bfloat16, 2)])
def test_planned_backward_auto_reddit(cuda, dtype, K):
    """The 232,965-node graph at F = 256 through the automatic split (the
    fewest equal row ranges of A whose dC slice fits in half of L2: 4 for
    FP32 dC, 2 for BF16): dB on sampled rows of A^T (incl. the 16 largest)
    and dvals on the entries of sampled rows of A against FP64, and both
    against the plan with one more range."""
    g = G.gcn_normalize(G.reddit_like(device=cuda))
    n, F = g.nrows, 256
    T = ops.CSRTranspose(ops.CSR(g.rowptr, g.colind, None, n, n))
    tv = T.values(g.vals)
    Gd = G.normal(4, 51, (n, F), device=cuda).to(dtype)
    Hd = G.normal(4, 52, (n, F), device=cuda).to(dtype)
    plan = ops.BackwardPlan(T, tv, F, dtype, 0)
    assert plan.parts == K
    dB, dv = plan.run(Gd, Hd)
    dBe, dve = ops.BackwardPlan(T, tv, F, dtype, K + 1).run(Gd, Hd)
    assert torch.allclose(dB, dBe, rtol=1e-5, atol=1e-6)
    assert torch.allclose(dv, dve, rtol=1e-6, atol=1e-7)
    Gr, Hr = Gd.float().cpu().numpy(), Hd.float().cpu().numpy()
    trp, tci, _ = (x.cpu().numpy() for x in T.arrays())
    tdeg = torch.from_numpy(np.diff(trp))
    rows = torch.cat([torch.topk(tdeg, 16).indices, torch.arange(0, n, 1999)]).numpy()
    ref, mag = oracle.csr_spmm_f64(trp, tci, tv.cpu().numpy(), Gr, rows=rows)
    assert oracle.rel_err(dB.cpu().numpy()[rows], ref, mag)[0] <= 1e-5
    rp, ci = g.rowptr.cpu().numpy(), g.colind.cpu().numpy()
    sel = np.arange(7, n, 2999)
    cnt = rp[sel + 1] - rp[sel]
    srp = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    idx = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in sel])
    refv = oracle.sddmm_f64(srp, ci[idx], Gr[sel], Hr)
    S = sddmm_scale(srp, ci[idx], Gr[sel], Hr)
    assert np.max(np.abs(dv.cpu().numpy()[idx] - refv) / np.maximum(S, 1e-30)) <= 1e-5


def test_planned_backward_auto_parts_and_reuse(cuda):
    """Automatic part count (1 when dC fits in half of L2) and a plan reused
    across calls with a shared workspace."""
    g = G.gcn_normalize(G.flickr_like())
    n, F = g.nrows, 32
    T = ops.CSRTranspose(dev(g, cuda, False))
    tv = T.values(g.vals.to(cuda))
    plan = ops.BackwardPlan(T, tv, F, torch.float32, 0)
    assert plan.parts == 1
    ws = ops.SpmmWorkspace()
    outs = []
    for seed in (1, 2):
        Gd = G.normal(seed, 30, (n, F)).to(cuda)
        Hd = G.normal(seed, 31, (n, F)).to(cuda)
        outs.append((plan.run(Gd, Hd, workspace=ws), ops.spmm_backward(T, tv, Gd, Hd, workspace=ws)))
    for (a, b) in outs:
        assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])
