"""GPU tests of the tcgen05 binary GEMM (algo 3: bits expanded to FP8
{0, 1}, tcgen05.mma kind::f8f6f4 into TMEM, TMA-staged operands):
bit-exact against the oracle, partial tiles, and no bounded wait ran out."""
import numpy as np
import pytest
import torch

import oracle
from spmm_eval_gb300 import ops

pytestmark = pytest.mark.gpu


def words(rng, kw, rows):
    return rng.integers(0, 2 ** 32, (kw, rows), dtype=np.uint64).astype(np.uint32)


@pytest.mark.parametrize("M, N, Kw", [(128, 256, 4), (256, 512, 8), (132, 100, 17), (64, 36, 1),
                                      (384, 768, 40)])
def test_tc_counts_bit_exact(cuda, M, N, Kw):
    rng = np.random.default_rng(M * 7 + N + Kw)
    A, B = words(rng, Kw, M), words(rng, Kw, N)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dB = torch.from_numpy(B.view(np.int32)).to(cuda)
    for mode in (ops.BMM_XOR, ops.BMM_AND, ops.BMM_SIGNED):
        got = ops.bmm_b1(dA, dB, mode, ops.BMM_ALGO_TC).cpu().numpy()
        want = oracle.bmm_counts(A, B, M, N, Kw, mode)
        assert np.array_equal(got, want), (mode, int((got != want).sum()))
    assert ops.bmm_tc_timeouts() == 0


def test_tc_known_answers(cuda):
    Kw, M = 4, 256
    rng = np.random.default_rng(3)
    A = words(rng, Kw, M)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dN = torch.from_numpy((~A).view(np.int32)).to(cuda)
    x = ops.bmm_b1(dA, dA, ops.BMM_XOR, ops.BMM_ALGO_TC).cpu().numpy()
    assert np.all(np.diag(x) == 0)
    y = ops.bmm_b1(dA, dN, ops.BMM_XOR, ops.BMM_ALGO_TC).cpu().numpy()
    assert np.all(np.diag(y) == 32 * Kw)
    z = ops.bmm_b1(dA, dA, ops.BMM_AND, ops.BMM_ALGO_TC).cpu().numpy()
    pop = np.array([sum(bin(int(A[k, r])).count("1") for k in range(Kw)) for r in range(M)])
    assert np.array_equal(np.diag(z), pop)
    assert ops.bmm_tc_timeouts() == 0
