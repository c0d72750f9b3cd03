"""GPU parity of the B2SR path: packing (bit-exact vs the oracle, vs the
hand-derived known answers, and vs cuSPARSE csr2bsr -- the library call the
reference's packer is built on), B2SR x dense SpMM (the tile-4 drop-in bitwise equal to
the reference's summation order; the order-free entry point, whose hub
block-rows are split and summed with atomics, bit-exact against the CSR
product on 0/1 and +-1 features at every tile and within FP32 rounding of
FP64 on float features, and equal to cusparseSpMM on +-1 features
as the reference driver checks, test_spmm_full.cu:421-431), B2SR x bits BMM
(bit-exact int32), the aligned formats and the dense sign packers."""
import ctypes as C
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle
from spmm_eval_gb300 import _lib
from spmm_eval_gb300 import graphs as G
from spmm_eval_gb300 import ops

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent
TILES = [4, 8, 16, 32]
NPDT = {4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}


@pytest.fixture(scope="session")
def cusparse_ref(cuda):
    so = HERE / "native" / "libcusparse_ref.so"
    src = HERE / "native" / "cusparse_ref.cu"
    if not so.exists() or so.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared",
                        "-Xcompiler", "-fPIC", "-Wno-deprecated-declarations", "-o", str(so), str(src),
                        "-lcusparse"], check=True)
    return C.CDLL(str(so))


def graphs():
    rng = np.random.default_rng(0)
    out = []
    d = json.loads((HERE / "golden" / "b2sr_kat.json").read_text())
    rp = np.zeros(d["nrows"] + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in d["rows"]])
    ci = np.array([c for r in d["rows"] for c in r], np.int32)
    out.append(("kat", d["nrows"], d["ncols"], rp, ci))
    for n, m, dens, dup in [(101, 77, 0.08, False), (257, 300, 0.03, True), (64, 64, 0.5, False)]:
        rows = []
        for r in range(n):
            k = rng.binomial(m, dens) if r % 7 else 0
            cols = np.sort(rng.choice(m, size=k, replace=False)) if k else np.zeros(0, np.int64)
            if dup and k:
                cols = np.sort(np.concatenate([cols, cols[:1]]))
            rows.append(cols)
        rp = np.zeros(n + 1, np.int32)
        rp[1:] = np.cumsum([len(x) for x in rows])
        out.append((f"rand{n}", n, m, rp, np.concatenate(rows).astype(np.int32)))
    g = G.flickr_like()
    out.append(("flickr_like", g.nrows, g.ncols, g.rowptr.numpy(), g.colind.numpy()))
    return out


GRAPHS = graphs()


def dev_csr(n, m, rp, ci, dev):
    return ops.CSR(torch.from_numpy(rp).to(dev), torch.from_numpy(ci).to(dev), None, n, m)


def host_val(Ab):
    v = Ab.val.cpu().numpy()
    return v.view(NPDT[Ab.tile]) if v.dtype.itemsize == np.dtype(NPDT[Ab.tile]).itemsize else v


@pytest.mark.parametrize("ts", TILES)
@pytest.mark.parametrize("gi", range(len(GRAPHS)))
def test_pack_bit_exact_vs_oracle(cuda, ts, gi):
    name, n, m, rp, ci = GRAPHS[gi]
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
    assert np.array_equal(Ab.rowptr.cpu().numpy(), brp)
    assert np.array_equal(Ab.colind.cpu().numpy(), bci)
    assert np.array_equal(host_val(Ab), bv)


@pytest.mark.parametrize("ts", TILES)
def test_pack_known_answers(cuda, ts):
    d = json.loads((HERE / "golden" / "b2sr_kat.json").read_text())
    _, n, m, rp, ci = GRAPHS[0]
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    want = d["packings"][str(ts)]
    assert Ab.rowptr.cpu().tolist() == want["rowptr"]
    assert Ab.colind.cpu().tolist() == want["colind"]
    assert [int(x) for x in host_val(Ab)] == want["val"]


@pytest.mark.parametrize("ts", TILES)
@pytest.mark.parametrize("gi", [1, 2, 4])
def test_pack_vs_cusparse_csr2bsr(cuda, cusparse_ref, ts, gi):
    """cusparseXcsr2bsrNnz + cusparseScsr2bsr on the same CSR with values
    1.0 (as csr2bsr_batch_bsrbmv.cu:296-311 does), then bit = (value > 0) in
    the ToBit*Col layout, must equal our packing."""
    name, n, m, rp, ci = GRAPHS[gi]
    drp = torch.from_numpy(rp).to(cuda)
    dci = torch.from_numpy(ci).to(cuda)
    mb = (n + ts - 1) // ts
    crp = torch.zeros(mb + 1, dtype=torch.int32, device=cuda)
    nnzb = C.c_int(0)
    assert cusparse_ref.ref_csr2bsr_nnz(n, m, C.c_void_p(drp.data_ptr()), C.c_void_p(dci.data_ptr()), ts,
                                        C.c_void_p(crp.data_ptr()), C.byref(nnzb)) == 0
    nb = nnzb.value
    ccol = torch.zeros(max(nb, 1), dtype=torch.int32, device=cuda)
    cval = torch.zeros(max(nb * ts * ts, 1), dtype=torch.float32, device=cuda)
    ones = torch.ones(max(len(ci), 1), dtype=torch.float32, device=cuda)
    assert cusparse_ref.ref_csr2bsr_fill(n, m, C.c_void_p(ones.data_ptr()), C.c_void_p(drp.data_ptr()),
                                         C.c_void_p(dci.data_ptr()), ts, C.c_void_p(cval.data_ptr()),
                                         C.c_void_p(crp.data_ptr()), C.c_void_p(ccol.data_ptr())) == 0
    dense = (cval[: nb * ts * ts].reshape(nb, ts, ts) > 0).cpu().numpy().astype(np.uint64)
    weights = (1 << np.arange(ts - 1, -1, -1, dtype=np.uint64))
    want_val = (dense * weights[None, None, :]).sum(-1).reshape(-1)
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    assert np.array_equal(Ab.rowptr.cpu().numpy(), crp.cpu().numpy())
    assert np.array_equal(Ab.colind.cpu().numpy(), ccol[:nb].cpu().numpy())
    assert np.array_equal(host_val(Ab).astype(np.uint64), want_val)


@pytest.mark.parametrize("ts", TILES)
def test_csr2bsr_batch_dropin(cuda, ts):
    name, n, m, rp, ci = GRAPHS[2]
    brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
    mb = (n + ts - 1) // ts
    d_rp = torch.zeros(mb + 1, dtype=torch.int32, device=cuda)
    d_ci = torch.zeros(len(bci), dtype=torch.int32, device=cuda)
    d_v = torch.zeros(len(bv), dtype=ops._TILE_DT[ts], device=cuda)
    ops.csr2bsr_batch(rp, ci, n, m, len(ci), d_rp, d_ci, d_v, ts, mb, len(bci))
    assert np.array_equal(d_rp.cpu().numpy(), brp)
    assert np.array_equal(d_ci.cpu().numpy(), bci)
    assert np.array_equal(d_v.cpu().numpy().view(NPDT[ts]), bv)
    with pytest.raises(_lib.GbsError):  # wrong nblocks is reported, not written past
        ops.csr2bsr_batch(rp, ci, n, m, len(ci), d_rp, d_ci, d_v, ts, mb, len(bci) + 1)


def test_pack_rejects_bad_csr(cuda):
    rp = torch.tensor([0, 2, 3], dtype=torch.int32, device=cuda)
    bad_order = ops.CSR(rp, torch.tensor([5, 3, 1], dtype=torch.int32, device=cuda), None, 2, 10)
    with pytest.raises(_lib.GbsError, match="ascending"):
        ops.csr2b2sr(bad_order, 4)
    bad_range = ops.CSR(rp, torch.tensor([1, 3, 10], dtype=torch.int32, device=cuda), None, 2, 10)
    with pytest.raises(_lib.GbsError, match="range"):
        ops.csr2b2sr(bad_range, 8)


def hub_matrix(n=8192, m=9000, hub_row=4101, hub_deg=3000, seed=5):
    """n x m CSR, 3 entries per row, one row of hub_deg entries (its strip
    goes to the packer's hub pass)."""
    rng = np.random.default_rng(seed)
    rows = []
    for r in range(n):
        k = hub_deg if r == hub_row else 3
        rows.append(np.sort(rng.choice(m, size=k, replace=False)))
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(x) for x in rows])
    return rp, np.concatenate(rows).astype(np.int32)


@pytest.mark.parametrize("ts", TILES)
def test_pack_hub_strip_bit_exact(cuda, ts):
    """A strip with thousands of entries (shared-memory bitmap pass) packs
    exactly like the oracle, beside thousands of ordinary strips."""
    n, m = 8192, 9000
    rp, ci = hub_matrix(n, m)
    brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    assert np.array_equal(Ab.rowptr.cpu().numpy(), brp)
    assert np.array_equal(Ab.colind.cpu().numpy(), bci)
    assert np.array_equal(host_val(Ab), bv)


def test_pack_hub_strip_rejects_bad_csr(cuda):
    """The hub pass validates its strips like the lane-group walk."""
    n, m = 8192, 9000
    rp, ci = hub_matrix(n, m)
    hub0 = int(rp[4101])
    bad = ci.copy()
    bad[hub0 + 10], bad[hub0 + 11] = ci[hub0 + 11], ci[hub0 + 10]  # descending pair in the hub row
    with pytest.raises(_lib.GbsError, match="ascending"):
        ops.csr2b2sr(dev_csr(n, m, rp, bad, cuda), 4)
    bad = ci.copy()
    bad[int(rp[4102]) - 1] = m  # last entry of the hub row out of range
    with pytest.raises(_lib.GbsError, match="range"):
        ops.csr2b2sr(dev_csr(n, m, rp, bad, cuda), 8)


@pytest.mark.parametrize("gi", range(len(GRAPHS)))
@pytest.mark.parametrize("F", [32, 64, 128, 256])
def test_fbf_tile4_bitwise_reference_order(cuda, gi, F):
    """Arbitrary FP32 features: the drop-in (only nonzero results stored into
    a zero-filled C) equals the reference's addition order bit for bit on
    every graph.  The full-output entry point equals it too where no hub is
    split (fewer than 1024 block-rows: one pass); on the 89,250-node graph
    its hubs are split and summed with atomics, so it is held to FP32
    rounding against FP64 there."""
    name, n, m, rp, ci = GRAPHS[gi]
    brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, 4)
    rng = np.random.default_rng(F + gi)
    B = (rng.standard_normal((m, F)) * 10.0 ** rng.integers(-3, 4, (m, 1))).astype(np.float32)
    want = oracle.b2sr4_spmm_ref(n, brp, bci, bv, B)
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), 4)
    Bd = torch.from_numpy(B).to(cuda)
    got = ops.b2sr_spmm(Ab, Bd).cpu().numpy()
    mb = (n + 3) // 4
    if mb < 1024:
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    else:
        ref, mag = oracle.csr_spmm_f64(rp, ci, None, B)
        assert oracle.rel_err(got, ref, mag)[0] <= 1e-5
    Cd = torch.zeros((mb * 4, F), device=cuda)
    ops.spmm4_full_full(Ab.val, Bd, Cd, Ab.rowptr, Ab.colind, mb, F)
    assert np.array_equal(Cd[:n].cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert torch.count_nonzero(Cd[n:]) == 0


@pytest.mark.parametrize("ts", TILES)
@pytest.mark.parametrize("F", [8, 32, 96, 256, 1024])
def test_b2sr_spmm_exact_on_binary_features(cuda, ts, F):
    """0/1 and +-1 features: every tile size equals the CSR product exactly
    (all partial sums are small integers)."""
    g = G.flickr_like()
    A = ops.CSR(g.rowptr.to(cuda), g.colind.to(cuda), None, g.nrows, g.ncols)
    Ab = ops.csr2b2sr(A, ts)
    rng = np.random.default_rng(ts * F)
    B01 = torch.from_numpy(rng.integers(0, 2, (g.ncols, F)).astype(np.float32)).to(cuda)
    assert torch.equal(ops.b2sr_spmm(Ab, B01), ops.csr_spmm(A, B01))
    Bpm = 2 * B01 - 1
    assert torch.equal(ops.b2sr_spmm(Ab, Bpm), ops.csr_spmm(A, Bpm))


@pytest.mark.parametrize("ts", TILES)
@pytest.mark.parametrize("F", [64, 512])
def test_b2sr_spmm_bf16_features_hub_split(cuda, ts, F):
    """16-bit features through both passes (block-rows of more than 256 tiles
    go to the sliced hub pass): +-1 values, so the result equals the FP32
    CSR product exactly."""
    g = G.flickr_like()
    A = ops.CSR(g.rowptr.to(cuda), g.colind.to(cuda), None, g.nrows, g.ncols)
    Ab = ops.csr2b2sr(A, ts)
    rng = np.random.default_rng(7 * ts + F)
    Bpm = torch.from_numpy(rng.integers(0, 2, (g.ncols, F)).astype(np.float32) * 2 - 1).to(cuda)
    got = ops.b2sr_spmm(Ab, Bpm.to(torch.bfloat16))
    assert torch.equal(got, ops.csr_spmm(A, Bpm))


@pytest.mark.parametrize("ts", TILES)
@pytest.mark.parametrize("F,dtype", [(64, torch.float32), (33, torch.float32), (1024, torch.float32),
                                     (256, torch.bfloat16), (128, torch.float16)])
def test_b2sr_spmm_float_features_vs_oracle(cuda, ts, F, dtype):
    """Float features on the 89,250-node graph, whose hub block-rows are cut
    into segments summed with atomics at tiles 4 and 8 (and kept whole, with
    plain stores, where the mean work per warp is larger than any hub): FP32
    rounding against FP64, for the 4-wide, scalar (F = 33) and 16-bit
    feature loads and up to 8 feature slices (F = 1024)."""
    name, n, m, rp, ci = GRAPHS[4]
    B = G.normal(ts + F, 3, (m, F)).to(dtype)
    Bq = B.float().numpy()
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    got = ops.b2sr_spmm(Ab, B.to(cuda)).cpu().numpy()
    ref, mag = oracle.csr_spmm_f64(rp, ci, None, Bq)
    assert oracle.rel_err(got, ref, mag)[0] <= 1e-5
    if F == 64 and dtype == torch.float32:
        brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
        want = oracle.b2sr_spmm(ts, n, brp, bci, bv, Bq)
        assert oracle.rel_err(want, ref, mag)[0] <= 1e-5


@pytest.mark.parametrize("ts", [16, 32])
@pytest.mark.parametrize("F,dtype", [(64, torch.float32), (256, torch.float32), (256, torch.bfloat16)])
def test_b2sr_spmm_dense_tiles(cuda, ts, F, dtype):
    """Fully dense tiles: rows 0..63 hold every column of a 9,000-column
    matrix, so a 32-tile step of the tile-wide pass holds more bits than its
    entry list (the tile-by-tile path) and those block-rows are longer than
    the cut (segments summed with atomics); the other rows are sparse.
    Exact against the CSR product on 0/1 features, FP32 rounding against
    FP64 on float features."""
    n, m = 500, 9000
    rng = np.random.default_rng(ts + F)
    rows = [np.arange(m) if r < 64 else np.sort(rng.choice(m, size=rng.integers(0, 40), replace=False))
            for r in range(n)]
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(x) for x in rows])
    ci = np.concatenate(rows).astype(np.int32)
    A = dev_csr(n, m, rp, ci, cuda)
    Ab = ops.csr2b2sr(A, ts)
    B01 = torch.from_numpy(rng.integers(0, 2, (m, F)).astype(np.float32)).to(cuda)
    assert torch.equal(ops.b2sr_spmm(Ab, B01.to(dtype)), ops.csr_spmm(A, B01))
    B = G.normal(ts + F, 3, (m, F)).to(dtype)
    got = ops.b2sr_spmm(Ab, B.to(cuda)).cpu().numpy()
    ref, mag = oracle.csr_spmm_f64(rp, ci, None, B.float().numpy())
    assert oracle.rel_err(got, ref, mag)[0] <= 1e-5


@pytest.mark.parametrize("F", [32, 64, 256])
def test_fbf_equals_cusparse_on_pm1(cuda, cusparse_ref, F):
    """The reference driver's own check: B2SR-4 FBF == cusparseSpMM (FP32,
    column-major copies) exactly, for +-1 features and 0/1 A."""
    g = G.flickr_like()
    n = g.nrows
    rng = np.random.default_rng(F)
    Bh = np.where(rng.random((n, F)) > 0.5, 1.0, -1.0).astype(np.float32)
    ones = torch.ones(g.nnz, device=cuda)
    drp, dci = g.rowptr.to(cuda), g.colind.to(cuda)
    Bcol = torch.from_numpy(np.ascontiguousarray(Bh.T)).to(cuda)
    Ccol = torch.zeros((F, n), device=cuda)
    assert cusparse_ref.ref_spmm_colmajor(n, n, g.nnz, C.c_void_p(drp.data_ptr()), C.c_void_p(dci.data_ptr()),
                                          C.c_void_p(ones.data_ptr()), C.c_void_p(Bcol.data_ptr()), F,
                                          C.c_void_p(Ccol.data_ptr())) == 0
    Ab = ops.csr2b2sr(ops.CSR(drp, dci, None, n, n), 4)
    mb = Ab.nblockrows
    Cd = torch.zeros((mb * 4, F), device=cuda)
    ops.spmm4_full_full(Ab.val, torch.from_numpy(Bh).to(cuda), Cd, Ab.rowptr, Ab.colind, mb, F)
    assert torch.equal(Cd[:n], Ccol.T.contiguous())


@pytest.mark.parametrize("ts", TILES)
@pytest.mark.parametrize("F", [1, 32, 64, 96, 256, 512, 1024])
def test_bmm_bit_exact(cuda, ts, F):
    """Every width on the flickr-shaped graph, whose hub block-rows go to the
    hub pass (k_b2sr_bmm_hubs, up to 32 words per row at F = 1024), and on a
    small random graph."""
    for gi in (4, 2):
        _bmm_case(cuda, ts, F, gi)


def _bmm_case(cuda, ts, F, gi):
    name, n, m, rp, ci = GRAPHS[gi]
    brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
    X = G.normal(F + ts, 8, (m, F))
    Xw = ops.pack_sign_rows(X.to(cuda))
    assert np.array_equal(Xw.cpu().numpy().view(np.uint32), oracle.pack_sign_rows(X.numpy()))
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    for signed in (False, True):
        got = ops.b2sr_bmm(Ab, Xw, F, signed).cpu().numpy()
        want = oracle.b2sr_bmm(ts, n, brp, bci, bv, Xw.cpu().numpy().view(np.uint32), F, signed)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("ts", [16, 32])
@pytest.mark.parametrize("F", [32, 200, 1024])
def test_bmm_dense_tiles_bit_exact(cuda, ts, F):
    """Fully dense tiles through the BMM (tile 32: the tile-wide pass): rows
    0..63 hold every one of 9,000 columns (steps that overflow the entry
    list, block-rows cut into segments added with integer atomics), the
    rest sparse; F = 200 leaves a partial last word.  Unsigned and +-1
    counts bit for bit against the oracle."""
    n, m = 500, 9000
    rng = np.random.default_rng(ts * F)
    rows = [np.arange(m) if r < 64 else np.sort(rng.choice(m, size=rng.integers(0, 40), replace=False))
            for r in range(n)]
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(x) for x in rows])
    ci = np.concatenate(rows).astype(np.int32)
    brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
    X = G.normal(F + ts, 8, (m, F))
    Xw = ops.pack_sign_rows(X.to(cuda))
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    for signed in (False, True):
        got = ops.b2sr_bmm(Ab, Xw, F, signed).cpu().numpy()
        want = oracle.b2sr_bmm(ts, n, brp, bci, bv, Xw.cpu().numpy().view(np.uint32), F, signed)
        assert np.array_equal(got, want)


def test_bmm_signed_matches_fbf_on_pm1(cuda):
    """signed BMM == float FBF product with the +-1 features it encodes."""
    g = G.flickr_like()
    A = ops.CSR(g.rowptr.to(cuda), g.colind.to(cuda), None, g.nrows, g.ncols)
    Ab = ops.csr2b2sr(A, 4)
    X = G.normal(1, 8, (g.ncols, 128)).to(cuda)
    pm = torch.where(X >= 0, 1.0, -1.0)
    assert torch.equal(ops.b2sr_bmm(Ab, ops.pack_sign_rows(X), 128, True).float(), ops.b2sr_spmm(Ab, pm))


@pytest.mark.parametrize("ts", [8, 16])
def test_aligned_formats(cuda, ts):
    for gi in (1, 4):
        name, n, m, rp, ci = GRAPHS[gi]
        brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
        nrp, nci, nv = oracle.b2sr_aligned(ts, brp, bci, bv)
        Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
        grp, gci, gv = ops.b2sr_aligned(Ab)
        assert np.array_equal(grp.cpu().numpy(), nrp)
        assert np.array_equal(gci.cpu().numpy(), nci)
        assert np.array_equal(gv.cpu().numpy().view(np.uint32), nv)


@pytest.mark.parametrize("ts", [8, 16])
@pytest.mark.parametrize("F", [1, 32, 96, 256, 1024])
def test_bmm_on_aligned_formats(cuda, ts, F):
    """The BMM that reads the aligned B2SR-8/16 words equals the BMM on the
    plain arrays and the oracle, bit for bit, on the flickr-shaped graph (hub
    block-rows included) and a small random graph, signed and unsigned."""
    for gi in (4, 2):
        name, n, m, rp, ci = GRAPHS[gi]
        Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
        al = ops.b2sr_aligned(Ab)
        X = G.normal(F + 3 * ts, 8, (m, F))
        Xw = ops.pack_sign_rows(X.to(cuda))
        brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
        for signed in (False, True):
            got = ops.b2sr_bmm_aligned(Ab, al, Xw, F, signed)
            assert torch.equal(got, ops.b2sr_bmm(Ab, Xw, F, signed))
            if gi == 2 or F <= 96:
                want = oracle.b2sr_bmm(ts, n, brp, bci, bv, Xw.cpu().numpy().view(np.uint32), F, signed)
                assert np.array_equal(got.cpu().numpy(), want)


def test_pack_sign_colud(cuda):
    X = G.normal(4, 4, (70, 100))
    got = ops.pack_sign_colud(X.to(cuda)).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, oracle.pack_sign_colud(X.numpy()))


@pytest.mark.parametrize("ts", TILES)
def test_b2sr_cache_roundtrip_on_device(cuda, tmp_path, ts):
    """A device B2SR written to the binary cache and loaded back gives the
    same arrays and the same SpMM result bit for bit."""
    _, n, m, rp, ci = GRAPHS[1]
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    f = tmp_path / f"a{ts}.b2sr"
    ops.write_b2sr_bin(f, Ab)
    Lb = ops.load_b2sr(f, cuda)
    assert (Lb.nrows, Lb.ncols, Lb.tile, Lb.nnzb) == (Ab.nrows, Ab.ncols, Ab.tile, Ab.nnzb)
    assert torch.equal(Lb.rowptr, Ab.rowptr) and torch.equal(Lb.colind, Ab.colind)
    assert Lb.val.dtype == Ab.val.dtype and torch.equal(Lb.val, Ab.val)
    B = G.normal(ts, 5, (m, 64), device=cuda)
    assert torch.equal(ops.b2sr_spmm(Lb, B), ops.b2sr_spmm(Ab, B))
