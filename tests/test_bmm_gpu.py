"""GPU parity of the dense binary matmul (backend/mm.cu semantics): both
kernels (tensor-core mma.sync .b1 AND-popc, CUDA-core __popc) bit-exact
against the oracle for XOR / AND / signed counts, the float drop-in of
BMM32_Arow_Brow, and the BMM32_BIN / BMM32S_BIN sign-word layouts."""
import numpy as np
import pytest
import torch

import oracle
from spmm_eval_gb300 import ops

pytestmark = pytest.mark.gpu


def words(rng, kw, rows):
    return rng.integers(0, 2 ** 32, (kw, rows), dtype=np.uint64).astype(np.uint32)


@pytest.mark.parametrize("algo", [ops.BMM_ALGO_POPC, ops.BMM_ALGO_MMA])
@pytest.mark.parametrize("M, N, Kw", [(128, 128, 8), (256, 384, 16), (132, 100, 17), (64, 36, 1),
                                      (512, 256, 40)])
def test_bmm_counts_bit_exact(cuda, algo, M, N, Kw):
    rng = np.random.default_rng(M + N + Kw)
    A, B = words(rng, Kw, M), words(rng, Kw, N)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dB = torch.from_numpy(B.view(np.int32)).to(cuda)
    for mode in (ops.BMM_XOR, ops.BMM_AND, ops.BMM_SIGNED):
        got = ops.bmm_b1(dA, dB, mode, algo).cpu().numpy()
        want = oracle.bmm_counts(A, B, M, N, Kw, mode)
        assert np.array_equal(got, want), (mode, algo)


def test_bmm_sparse_bits_and_known_answers(cuda):
    """Identity-like patterns with known counts: A = B -> xor 0 on the
    diagonal; complement -> xor = 32*Kw."""
    Kw, M = 4, 128
    rng = np.random.default_rng(3)
    A = words(rng, Kw, M)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dN = torch.from_numpy((~A).view(np.int32)).to(cuda)
    for algo in (ops.BMM_ALGO_POPC, ops.BMM_ALGO_MMA):
        x = ops.bmm_b1(dA, dA, ops.BMM_XOR, algo).cpu().numpy()
        assert np.all(np.diag(x) == 0)
        y = ops.bmm_b1(dA, dN, ops.BMM_XOR, algo).cpu().numpy()
        assert np.all(np.diag(y) == 32 * Kw)


def test_bmm32_arow_brow_dropin(cuda):
    rng = np.random.default_rng(7)
    M, N, Kw = 256, 192, 9
    A, B = words(rng, Kw, M), words(rng, Kw, N)
    C = torch.zeros((M, N), device=cuda)
    ops.bmm32_arow_brow(torch.from_numpy(A.view(np.int32)).to(cuda),
                        torch.from_numpy(B.view(np.int32)).to(cuda), C, M, Kw, N)
    assert np.array_equal(C.cpu().numpy(), oracle.bmm32_arow_brow(A, B, M, Kw, N))


@pytest.mark.parametrize("s_layout", [False, True])
def test_bmm32_bin_layouts(cuda, s_layout):
    rng = np.random.default_rng(9)
    m, k, Kw = 96, 64, 5
    nbits = 32 * Kw - 7  # n not a multiple of 32: the reference reads ceil(n/32) words
    A, B = words(rng, Kw, m), words(rng, Kw, k)
    size = m * k if s_layout else (k // 32) * m
    C = torch.zeros(size, dtype=torch.int32, device=cuda)
    ops.bmm32_bin(torch.from_numpy(A.view(np.int32)).to(cuda), torch.from_numpy(B.view(np.int32)).to(cuda),
                  C, m, nbits, k, s_layout)
    want = (oracle.bmm32s_bin if s_layout else oracle.bmm32_bin)(A, B, m, nbits, k)
    assert np.array_equal(C.cpu().numpy().view(np.uint32), want)


@pytest.mark.parametrize("s_layout", [False, True])
@pytest.mark.parametrize("m, k, nbits", [(32, 32, 1), (96, 64, 153), (256, 512, 1024), (416, 288, 33),
                                         (1024, 2080, 4096)])
def test_bin_fused_epilogue_vs_counts_and_oracle(cuda, s_layout, m, k, nbits):
    """Sign words thresholded in the tcgen05 epilogue equal the two-pass
    form (int32 counts, then sign words) and the oracle, at sizes with
    partial output tiles and n not a multiple of 32."""
    rng = np.random.default_rng(m + k + nbits)
    Kw = (nbits + 31) // 32
    A, B = words(rng, Kw, m), words(rng, Kw, k)
    dA, dB = torch.from_numpy(A.view(np.int32)).to(cuda), torch.from_numpy(B.view(np.int32)).to(cuda)
    size = m * k if s_layout else (k // 32) * m
    fused = torch.full((size,), 7, dtype=torch.int32, device=cuda)
    two = torch.full((size,), 7, dtype=torch.int32, device=cuda)
    ops.bmm_bin(dA, dB, fused, m, nbits, k, s_layout, ops.BIN_FUSED)
    ops.bmm_bin(dA, dB, two, m, nbits, k, s_layout, ops.BIN_COUNTS)
    assert torch.equal(fused, two)
    want = (oracle.bmm32s_bin if s_layout else oracle.bmm32_bin)(A, B, m, nbits, k)
    got = fused.cpu().numpy().view(np.uint32)
    if s_layout:  # the reference's S layout writes k of every k * 32 words
        used = (np.arange(m * k) % (k * 32)) < k
        assert np.array_equal(got[used], want[used])
        assert np.all(got[~used] == 7)
    else:
        assert np.array_equal(got, want)
    assert ops.bmm_tc_timeouts() == 0


def test_bin_fused_8192(cuda):
    """The 8192 x 8192 x 8192-bit configuration: fused sign words equal the
    two-pass form over the whole output, and the oracle on a sampled block."""
    m = k = nbits = 8192
    Kw = nbits // 32
    rng = np.random.default_rng(8193)
    A, B = words(rng, Kw, m), words(rng, Kw, k)
    dA, dB = torch.from_numpy(A.view(np.int32)).to(cuda), torch.from_numpy(B.view(np.int32)).to(cuda)
    fused = torch.zeros((k // 32) * m, dtype=torch.int32, device=cuda)
    two = torch.zeros_like(fused)
    ops.bmm_bin(dA, dB, fused, m, nbits, k, False, ops.BIN_FUSED)
    ops.bmm_bin(dA, dB, two, m, nbits, k, False, ops.BIN_COUNTS)
    assert torch.equal(fused, two)
    r0, c0 = 4096, 8192 - 256
    sub = oracle.bmm32_bin(np.ascontiguousarray(A[:, r0:r0 + 256]), np.ascontiguousarray(B[:, c0:c0 + 256]),
                           256, nbits, 256)  # words [by][r] of the 256 x 256 block
    got = fused.reshape(k // 32, m)[c0 // 32:(c0 + 256) // 32, r0:r0 + 256].cpu().numpy().view(np.uint32)
    assert np.array_equal(got.reshape(-1), sub)
    assert ops.bmm_tc_timeouts() == 0


def test_sign_packed_dense_operands(cuda):
    """End to end from dense +-1 matrices: pack with ToBit32ColUd semantics,
    multiply, compare with the float product."""
    rng = np.random.default_rng(1)
    M, N, K = 96, 64, 160
    Xa = rng.standard_normal((M, K)).astype(np.float32)
    Xb = rng.standard_normal((N, K)).astype(np.float32)
    pa = ops.pack_sign_colud(torch.from_numpy(Xa).to(cuda))
    pb = ops.pack_sign_colud(torch.from_numpy(Xb).to(cuda))
    got = ops.bmm_b1(pa, pb, ops.BMM_SIGNED).cpu().numpy()
    sa, sb = np.where(Xa >= 0, 1, -1), np.where(Xb >= 0, 1, -1)
    assert np.array_equal(got, sa @ sb.T)


def test_default_algo_matches_popc(cuda):
    rng = np.random.default_rng(17)
    M, N, Kw = 256, 320, 12
    A, B = words(rng, Kw, M), words(rng, Kw, N)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dB = torch.from_numpy(B.view(np.int32)).to(cuda)
    for mode in (ops.BMM_XOR, ops.BMM_AND, ops.BMM_SIGNED):
        assert torch.equal(ops.bmm_b1(dA, dB, mode, ops.BMM_ALGO_DEFAULT), ops.bmm_b1(dA, dB, mode, ops.BMM_ALGO_POPC))
