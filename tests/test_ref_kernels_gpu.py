"""Parity against the reference's own CUDA kernels, run on the same device
buffers as the library's.

The kernels come from ``oracle/_ref/ref_kernels.fatbin``, compiled from the
reference sources where they lie (``oracle/ref_kernels.cu`` lists them with
their file:line) and loaded through the driver API (``oracle/refkern.py``),
each launched with the grid the reference uses.  Checked bit for bit:

* ``spmm4_full_full_new2`` (backend/spmm.cu:877-956, launched as
  test_spmm_full.cu:351-361) against ``gbs_spmm4_full_full`` on arbitrary
  FP32 features (and ``gbs_b2sr_spmm`` tile 4 where it splits no hub), and
  against the oracle's restatement of its addition order;
* ``ToBit{4,8,16,32}Col<float>`` applied to cuSPARSE csr2bsr blocks (the
  chain inside csr2bsr_batch_{4,8,16,32}, csr2bsr_batch_bsrbmv.cu:296-339)
  against the library's packer;
* ``packUchar2AlignedUnsigned`` / ``packUshort2AlignedUnsigned``
  (csr2bsr_batch_bsrbmv.cu:608-648, :859-888) against
  ``gbs_b2sr_pack_aligned`` and the oracle;
* ``ToBit32ColUd`` / ``ToBit32RowDenseSign`` (spmm.cu:93-111, :75-91)
  against the library's sign packers and the oracle;
* ``BMM32_Arow_Brow<float>``, ``BMM32_MT_M_S``, ``BMM32_BIN``,
  ``BMM32S_BIN`` (mm.cu:17-125) against the library's drop-ins and the
  oracle, including the full 8192 x 8192 x 8192-bit product.

The fatbin is built where the reference sources are (``__graft_entry__.build``
in the development container) and travels with the repository's built files;
without it these tests skip with that reason.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from oracle import refkern
from spmm_eval_gb300 import graphs as G
from spmm_eval_gb300 import ops

from test_b2sr_gpu import GRAPHS, NPDT, TILES, cusparse_ref, dev_csr, host_val  # noqa: F401

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refkern.available(),
                                 reason="oracle/_ref/ref_kernels.fatbin not built (needs the reference sources)")]


@pytest.fixture(scope="module")
def rk(cuda):
    return refkern.kernels()


def ref_fbf(rk, Ab, B, F):
    """spmm4_full_full_new2 with the reference driver's launch shape."""
    mb = Ab.nblockrows
    tiles_per_tb = 1024 // F
    Cd = torch.zeros((mb * 4, F), device=B.device)
    rk.launch("spmm4_full_full_new2", ((mb + tiles_per_tb - 1) // tiles_per_tb,), (1024,),
              Ab.val, B, Cd, Ab.rowptr, Ab.colind, mb, F)
    return Cd


@pytest.mark.parametrize("gi", range(len(GRAPHS)))
@pytest.mark.parametrize("F", [32, 64, 128, 256])
def test_fbf_bitwise_vs_reference_kernel(cuda, rk, gi, F):
    name, n, m, rp, ci = GRAPHS[gi]
    rng = np.random.default_rng(100 + F + gi)
    B = (rng.standard_normal((m, F)) * 10.0 ** rng.integers(-3, 4, (m, 1))).astype(np.float32)
    Bd = torch.from_numpy(B).to(cuda)
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), 4)
    ref = ref_fbf(rk, Ab, Bd, F)
    mine = torch.zeros_like(ref)
    ops.spmm4_full_full(Ab.val, Bd, mine, Ab.rowptr, Ab.colind, Ab.nblockrows, F)
    torch.cuda.synchronize()
    assert torch.equal(mine.view(torch.int32), ref.view(torch.int32))
    full = ops.b2sr_spmm(Ab, Bd)
    if Ab.nblockrows < 1024:  # one pass, no hub split: the reference's order
        assert torch.equal(full.view(torch.int32), ref[:n].view(torch.int32))
    else:  # split hubs summed with atomics: FP32 rounding against FP64
        r64, mag = oracle.csr_spmm_f64(rp, ci, None, B)
        assert oracle.rel_err(full.cpu().numpy(), r64, mag)[0] <= 1e-5
    if m * F <= 4_000_000:  # the oracle's restatement of the order, pinned
        brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, 4)
        want = oracle.b2sr4_spmm_ref(n, brp, bci, bv, B)
        assert np.array_equal(want.view(np.uint32), ref[:n].cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("ts", TILES)
@pytest.mark.parametrize("gi", [1, 2, 3, 4])
def test_tile_packers_vs_reference_kernels(cuda, rk, cusparse_ref, ts, gi):
    """cuSPARSE csr2bsr (values 1.0, row-major blocks) + the reference's own
    ToBit*Col kernel with its launch shape: the tile rows the reference packer
    produces, against the library's packer.  (The 6 x 9 known-answer matrix
    is left out: cusparseXcsr2bsrNnz rejects block sizes above its
    dimensions.)"""
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
    # the reference's tile-packer launch shapes (csr2bsr_batch_bsrbmv.cu:320,
    # :513, :764, :1004): g blocks per 32-thread CTA along grid y; it
    # launches once per block-row strip, here in pieces of at most 65,535
    # CTAs (the grid-y limit), each piece starting on a CTA boundary
    g, kern, tdt = {4: (64, "ToBit4Col", torch.uint8), 8: (16, "ToBit8Col", torch.uint8),
                    16: (4, "ToBit16Col", torch.int16), 32: (1, "ToBit32Col", torch.int32)}[ts]
    groups = (nb + g - 1) // g
    out = torch.zeros(max(groups, 1) * g * ts, dtype=tdt, device=cuda)
    step = g * 65535
    for b0 in range(0, nb, step):
        cnt = min(step, nb - b0)
        sizes = (32, cnt * 32) if ts == 32 else (cnt,)  # ToBit32Col takes (height, width)
        rk.launch(kern, (1, (cnt + g - 1) // g), (32,), cval[b0 * ts * ts:], out[b0 * ts:], *sizes)
    torch.cuda.synchronize()
    want = out[: nb * ts].cpu().numpy().view(NPDT[ts])
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    assert np.array_equal(Ab.rowptr.cpu().numpy(), crp.cpu().numpy())
    assert np.array_equal(Ab.colind.cpu().numpy(), ccol[:nb].cpu().numpy())
    assert np.array_equal(host_val(Ab), want)


@pytest.mark.parametrize("ts", [8, 16])
@pytest.mark.parametrize("gi", [0, 1, 2, 3])
def test_aligned_formats_vs_reference_kernels(cuda, rk, ts, gi):
    name, n, m, rp, ci = GRAPHS[gi]
    Ab = ops.csr2b2sr(dev_csr(n, m, rp, ci, cuda), ts)
    grp, gci, gv = ops.b2sr_aligned(Ab)
    mb = Ab.nblockrows
    ntiles = int(grp[-1].item())
    nrp = torch.full((mb + 1,), -7, dtype=torch.int32, device=cuda)
    nci = torch.full((max(ntiles, 1),), -7, dtype=torch.int32, device=cuda)
    nv = torch.full((max(ntiles * ts // (4 if ts == 8 else 2), 1),), -7, dtype=torch.int32, device=cuda)
    kern = "packUchar2AlignedUnsigned" if ts == 8 else "packUshort2AlignedUnsigned"
    rk.launch(kern, (1,), (1,), Ab.rowptr, Ab.colind, Ab.val, mb, nrp, nci, nv)
    torch.cuda.synchronize()
    assert torch.equal(nrp, grp)
    assert torch.equal(nci[:ntiles], gci)
    assert torch.equal(nv[: gv.numel()], gv)
    brp, bci, bv = oracle.b2sr_pack(n, m, rp, ci, ts)
    orp, oci, ov = oracle.b2sr_aligned(ts, brp, bci, bv)
    assert np.array_equal(nv[: gv.numel()].cpu().numpy().view(np.uint32), ov)


@pytest.mark.parametrize("H, W", [(70, 100), (64, 32), (33, 129), (1000, 1024)])
def test_sign_packers_vs_reference_kernels(cuda, rk, H, W):
    X = G.normal(H, W, (H, W)).to(cuda)
    gx, gy = (H + 31) // 32, (W + 31) // 32
    ud = torch.zeros(gy * gx * 32, dtype=torch.int32, device=cuda)
    rk.launch("ToBit32ColUd", (gx, gy), (32,), X, ud, H, W)
    rows = torch.zeros(gx * 32 * gy, dtype=torch.int32, device=cuda)
    rk.launch("ToBit32RowDenseSign", (gx, gy), (32,), X, rows, H, W)
    torch.cuda.synchronize()
    assert torch.equal(ops.pack_sign_colud(X).reshape(-1), ud)
    assert torch.equal(ops.pack_sign_rows(X).reshape(-1), rows[: H * gy])
    assert np.array_equal(ud.cpu().numpy().view(np.uint32), oracle.pack_sign_colud(X.cpu().numpy()).reshape(-1))


def words(rng, kw, rows):
    return torch.from_numpy(rng.integers(0, 2 ** 32, (kw, rows), dtype=np.uint64).astype(np.uint32).view(np.int32))


@pytest.mark.parametrize("M, N, Kw", [(32, 32, 1), (64, 96, 3), (256, 512, 40), (1024, 2048, 7)])
def test_binary_gemm_vs_reference_kernels(cuda, rk, M, N, Kw):
    rng = np.random.default_rng(M + N + Kw)
    A, B = words(rng, Kw, M).to(cuda), words(rng, Kw, N).to(cuda)
    # BMM32_Arow_Brow<float>: grid (M/32, N/32), one warp per block
    ref = torch.zeros((M, N), device=cuda)
    rk.launch("BMM32_Arow_Brow", (M // 32, N // 32), (32,), A, B, ref, M, Kw, N)
    # BMM32_MT_M_S: same product, 32 warps per block
    ref2 = torch.zeros((M, N), device=cuda)
    rk.launch("BMM32_MT_M_S", (M // 32, N // 32), (1024,), A, B, ref2, M, Kw, N)
    mine = torch.zeros((M, N), device=cuda)
    ops.bmm32_arow_brow(A, B, mine, M, Kw, N)
    torch.cuda.synchronize()
    assert torch.equal(ref, ref2)
    assert torch.equal(mine, ref)
    An, Bn = A.cpu().numpy().view(np.uint32), B.cpu().numpy().view(np.uint32)
    assert np.array_equal(oracle.bmm32_arow_brow(An, Bn, M, Kw, N), ref.cpu().numpy())
    # BIN layouts: n = the number of K bits
    nbits = 32 * Kw
    rb = torch.zeros((N // 32) * M, dtype=torch.int32, device=cuda)
    rk.launch("BMM32_BIN", (M // 32, N // 32), (32,), A, B, rb, M, nbits, N)
    rs = torch.zeros(M * N, dtype=torch.int32, device=cuda)
    rk.launch("BMM32S_BIN", (M // 32, N // 32), (1024,), A, B, rs, M, nbits, N)
    mb = torch.zeros_like(rb)
    ops.bmm32_bin(A, B, mb, M, nbits, N)
    ms = torch.zeros_like(rs)
    ops.bmm32_bin(A, B, ms, M, nbits, N, s_layout=True)
    torch.cuda.synchronize()
    assert torch.equal(mb, rb)
    assert torch.equal(ms, rs)
    assert np.array_equal(oracle.bmm32_bin(An, Bn, M, nbits, N), rb.cpu().numpy().view(np.uint32))
    assert np.array_equal(oracle.bmm32s_bin(An, Bn, M, nbits, N), rs.cpu().numpy().view(np.uint32))


def test_binary_gemm_8192_vs_reference_kernel(cuda, rk):
    """The full binary-GEMM workload: 8192 x 8192 bit matrices (Bernoulli
    0.5), K = 8192 bits.  The reference kernel's float C against the library's
    default tcgen05 path (XOR counts and the float drop-in), the popc path,
    and the oracle on a sampled 256 x 256 block; no bounded wait ran out."""
    M = N = 8192
    Kw = 256
    rng = np.random.default_rng(8192)
    A, B = words(rng, Kw, M).to(cuda), words(rng, Kw, N).to(cuda)
    ref = torch.empty((M, N), device=cuda)
    rk.launch("BMM32_Arow_Brow", (M // 32, N // 32), (32,), A, B, ref, M, Kw, N)
    xor_tc = ops.bmm_b1(A, B, ops.BMM_XOR)
    torch.cuda.synchronize()
    assert torch.equal((32 * Kw - 2 * xor_tc).float(), ref)
    del xor_tc
    xor_popc = ops.bmm_b1(A, B, ops.BMM_XOR, ops.BMM_ALGO_POPC)
    assert torch.equal((32 * Kw - 2 * xor_popc).float(), ref)
    del xor_popc
    mine = torch.empty_like(ref)
    ops.bmm32_arow_brow(A, B, mine, M, Kw, N)
    assert torch.equal(mine, ref)
    assert ops.bmm_tc_timeouts() == 0
    r0, c0 = 4096 - 128, 8192 - 256
    An, Bn = A.cpu().numpy().view(np.uint32), B.cpu().numpy().view(np.uint32)
    want = oracle.bmm_counts(np.ascontiguousarray(An[:, r0:r0 + 256]), np.ascontiguousarray(Bn[:, c0:c0 + 256]),
                             256, 256, Kw, ops.BMM_XOR)
    assert np.array_equal((32 * Kw - 2 * want).astype(np.float32), ref[r0:r0 + 256, c0:c0 + 256].cpu().numpy())
