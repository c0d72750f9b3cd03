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
