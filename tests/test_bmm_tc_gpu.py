"""GPU tests of the tcgen05 binary GEMM (bits expanded to FP8 {0, 1},
tcgen05.mma kind::f8f6f4 into TMEM, TMA-staged operands) in both launch
forms -- one CTA per tile (algo 3) and the persistent warp-specialised
kernel with two TMEM accumulators (algo 4, the default): bit-exact against
the oracle, partial tiles, more tiles than SMs, and no bounded wait ran
out."""
import numpy as np
import pytest
import torch

import oracle
from spmm_eval_gb300 import ops

pytestmark = pytest.mark.gpu


def words(rng, kw, rows):
    return rng.integers(0, 2 ** 32, (kw, rows), dtype=np.uint64).astype(np.uint32)


TC_ALGOS = [ops.BMM_ALGO_TC, ops.BMM_ALGO_TC_PERSIST]


@pytest.mark.parametrize("algo", TC_ALGOS)
@pytest.mark.parametrize("M, N, Kw", [(128, 256, 4), (256, 512, 8), (132, 100, 17), (64, 36, 1),
                                      (384, 768, 40), (2176, 5120, 6)])
def test_tc_counts_bit_exact(cuda, M, N, Kw, algo):
    rng = np.random.default_rng(M * 7 + N + Kw)
    A, B = words(rng, Kw, M), words(rng, Kw, N)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dB = torch.from_numpy(B.view(np.int32)).to(cuda)
    for mode in (ops.BMM_XOR, ops.BMM_AND, ops.BMM_SIGNED):
        got = ops.bmm_b1(dA, dB, mode, algo).cpu().numpy()
        want = oracle.bmm_counts(A, B, M, N, Kw, mode)
        assert np.array_equal(got, want), (mode, int((got != want).sum()))
    assert ops.bmm_tc_timeouts() == 0


@pytest.mark.parametrize("algo", TC_ALGOS)
def test_tc_known_answers(cuda, algo):
    Kw, M = 4, 256
    rng = np.random.default_rng(3)
    A = words(rng, Kw, M)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dN = torch.from_numpy((~A).view(np.int32)).to(cuda)
    x = ops.bmm_b1(dA, dA, ops.BMM_XOR, algo).cpu().numpy()
    assert np.all(np.diag(x) == 0)
    y = ops.bmm_b1(dA, dN, ops.BMM_XOR, algo).cpu().numpy()
    assert np.all(np.diag(y) == 32 * Kw)
    z = ops.bmm_b1(dA, dA, ops.BMM_AND, algo).cpu().numpy()
    pop = np.array([sum(bin(int(A[k, r])).count("1") for k in range(Kw)) for r in range(M)])
    assert np.array_equal(np.diag(z), pop)
    assert ops.bmm_tc_timeouts() == 0


def test_default_is_persistent_tc(cuda):
    """The default algorithm gives the same counts as the explicit forms."""
    rng = np.random.default_rng(11)
    A, B = words(rng, 9, 640), words(rng, 9, 1100)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dB = torch.from_numpy(B.view(np.int32)).to(cuda)
    d = ops.bmm_b1(dA, dB, ops.BMM_XOR)
    p = ops.bmm_b1(dA, dB, ops.BMM_XOR, ops.BMM_ALGO_TC_PERSIST)
    t = ops.bmm_b1(dA, dB, ops.BMM_XOR, ops.BMM_ALGO_TC)
    assert torch.equal(d, p) and torch.equal(d, t)
    assert ops.bmm_tc_timeouts() == 0


def test_pool_trim_between_calls(cuda):
    """Temporaries come from the library pool; trimming it between calls
    changes nothing in the results."""
    rng = np.random.default_rng(5)
    A, B = words(rng, 5, 256), words(rng, 5, 512)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dB = torch.from_numpy(B.view(np.int32)).to(cuda)
    x = ops.bmm_b1(dA, dB, ops.BMM_AND)
    ops.pool_trim()
    y = ops.bmm_b1(dA, dB, ops.BMM_AND)
    assert torch.equal(x, y)
    assert np.array_equal(x.cpu().numpy(), oracle.bmm_counts(A, B, 256, 512, 5, ops.BMM_AND))


def test_tc_8192_cube_vs_popc_and_oracle(cuda):
    """The full binary-GEMM workload: 8192 x 8192 bit matrices (Bernoulli
    0.5), K = 8192 bits.  The default tcgen05 kernel equals the CUDA-core
    popc kernel over the whole int32 matrix, both equal the oracle on a
    sampled 256 x 256 block, and no bounded wait ran out."""
    M = N = 8192
    Kw = 256
    rng = np.random.default_rng(81)
    A, B = words(rng, Kw, M), words(rng, Kw, N)
    dA = torch.from_numpy(A.view(np.int32)).to(cuda)
    dB = torch.from_numpy(B.view(np.int32)).to(cuda)
    tc = ops.bmm_b1(dA, dB, ops.BMM_XOR)
    popc = ops.bmm_b1(dA, dB, ops.BMM_XOR, ops.BMM_ALGO_POPC)
    assert torch.equal(tc, popc)
    assert ops.bmm_tc_timeouts() == 0
    r0, c0 = 8192 - 256, 4096 - 128
    want = oracle.bmm_counts(np.ascontiguousarray(A[:, r0:r0 + 256]), np.ascontiguousarray(B[:, c0:c0 + 256]),
                             256, 256, Kw, ops.BMM_XOR)
    assert np.array_equal(tc[r0:r0 + 256, c0:c0 + 256].cpu().numpy(), want)
