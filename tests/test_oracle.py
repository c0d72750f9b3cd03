"""CPU tests of the oracle (oracle/oracle.c) against hand-derived known
answers and against independent pure-Python transcriptions of the
reference's loops.  No GPU."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"


def kat():
    d = json.loads((GOLD / "b2sr_kat.json").read_text())
    rowptr = np.zeros(d["nrows"] + 1, np.int32)
    rowptr[1:] = np.cumsum([len(r) for r in d["rows"]])
    colind = np.array([c for r in d["rows"] for c in r], np.int32)
    return d, rowptr, colind


@pytest.mark.parametrize("ts", [4, 8, 16, 32])
def test_b2sr_pack_known_answers(oracle_lib, ts):
    d, rowptr, colind = kat()
    brp, bci, bv = oracle.b2sr_pack(d["nrows"], d["ncols"], rowptr, colind, ts)
    want = d["packings"][str(ts)]
    assert brp.tolist() == want["rowptr"]
    assert bci.tolist() == want["colind"]
    assert [int(x) for x in bv] == want["val"]


def random_csr(n, m, density, seed, dup=False):
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(n):
        k = rng.binomial(m, density)
        cols = np.sort(rng.choice(m, size=k, replace=False)) if k else np.zeros(0, np.int64)
        if dup and k:
            cols = np.sort(np.concatenate([cols, cols[: max(1, k // 3)]]))
        rows.append(cols)
    rowptr = np.zeros(n + 1, np.int32)
    rowptr[1:] = np.cumsum([len(r) for r in rows])
    colind = np.concatenate(rows).astype(np.int32) if rows else np.zeros(0, np.int32)
    return rowptr, colind


def py_pack(nrows, ncols, rowptr, colind, ts):
    """Independent transcription of the strip loop + ToBit*Col layout."""
    mb = (nrows + ts - 1) // ts
    brp, bci, bv = [0], [], []
    for i in range(mb):
        tiles = {}
        for r in range(i * ts, min((i + 1) * ts, nrows)):
            for e in range(rowptr[r], rowptr[r + 1]):
                c = int(colind[e])
                t = tiles.setdefault(c // ts, [0] * ts)
                t[r - i * ts] |= 1 << (ts - 1 - c % ts)
        for tc in sorted(tiles):
            bci.append(tc)
            bv.extend(tiles[tc])
        brp.append(len(bci))
    return brp, bci, bv


@pytest.mark.parametrize("ts", [4, 8, 16, 32])
@pytest.mark.parametrize("n, m, dens, dup", [(37, 50, 0.1, False), (64, 64, 0.3, True),
                                               (5, 200, 0.05, False), (33, 7, 0.5, True)])
def test_b2sr_pack_matches_transcription(oracle_lib, ts, n, m, dens, dup):
    rowptr, colind = random_csr(n, m, dens, n * 100 + m + ts, dup)
    brp, bci, bv = oracle.b2sr_pack(n, m, rowptr, colind, ts)
    w = py_pack(n, m, rowptr, colind, ts)
    assert brp.tolist() == w[0] and bci.tolist() == w[1] and [int(x) for x in bv] == w[2]


def test_b2sr_pack_rejects_unsorted(oracle_lib):
    rowptr = np.array([0, 2], np.int32)
    with pytest.raises(ValueError):
        oracle.b2sr_pack(1, 10, rowptr, np.array([5, 3], np.int32), 4)


def py_fbf_ref(nrows, brp, bci, bv, B):
    """spmm4_full_full_new2 (spmm.cu:900-954) transcribed loop by loop in
    float32: groups of 8 tiles, j outer, tile inner, store if nonzero."""
    F = B.shape[1]
    C = np.zeros((nrows, F), np.float32)
    for r in range(len(brp) - 1):
        for i in range(4):
            if 4 * r + i >= nrows:
                continue
            for c in range(F):
                res = np.float32(0.0)
                for g in range(brp[r], brp[r + 1], 8):
                    for j in range(4):
                        for l in range(8):
                            t = g + l
                            if t < brp[r + 1] and (int(bv[4 * t + i]) >> (3 - j)) & 1:
                                res = np.float32(res + B[4 * bci[t] + j, c])
                if res != 0:
                    C[4 * r + i, c] = res
    return C


def test_fbf_reference_order_is_bitwise(oracle_lib):
    rowptr, colind = random_csr(23, 61, 0.4, 3)
    brp, bci, bv = oracle.b2sr_pack(23, 61, rowptr, colind, 4)
    rng = np.random.default_rng(1)
    # values of very different magnitude make the result order-sensitive
    B = (rng.standard_normal((61, 5)) * 10.0 ** rng.integers(-4, 5, (61, 1))).astype(np.float32)
    got = oracle.b2sr4_spmm_ref(23, brp, bci, bv, B)
    want = py_fbf_ref(23, brp, bci, bv, B)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # and the natural (column) order differs somewhere: the order matters
    nat = oracle.b2sr_spmm(4, 23, brp, bci, bv, B)
    assert np.allclose(nat, got, rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("ts", [4, 8, 16, 32])
def test_b2sr_spmm_equals_csr_product_on_binary(oracle_lib, ts):
    rowptr, colind = random_csr(70, 90, 0.2, ts)
    brp, bci, bv = oracle.b2sr_pack(70, 90, rowptr, colind, ts)
    B = np.random.default_rng(ts).integers(0, 2, (90, 33)).astype(np.float32)
    A = np.zeros((70, 90), np.float32)
    for r in range(70):
        A[r, colind[rowptr[r]:rowptr[r + 1]]] = 1
    assert np.array_equal(oracle.b2sr_spmm(ts, 70, brp, bci, bv, B), A @ B)


def test_pack_sign_rows_and_colud(oracle_lib):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((37, 70)).astype(np.float32)
    X[3, 5] = 0.0  # zero is >= 0 -> bit 1
    w = oracle.pack_sign_rows(X)
    assert w.shape == (37, 3)
    for r in range(37):
        for c in range(96):
            bit = (int(w[r, c // 32]) >> (31 - c % 32)) & 1
            assert bit == (1 if c < 70 and X[r, c] >= 0 else 0)
    u = oracle.pack_sign_colud(X)
    assert u.shape == (3, 64)
    for r in range(64):
        for c in range(96):
            bit = (int(u[c // 32, r]) >> (31 - c % 32)) & 1
            assert bit == (1 if r < 37 and c < 70 and X[r, c] >= 0 else 0)


@pytest.mark.parametrize("ts", [4, 8, 16, 32])
@pytest.mark.parametrize("F", [32, 45, 64])
def test_b2sr_bmm_matches_dense(oracle_lib, ts, F):
    rowptr, colind = random_csr(41, 41, 0.2, ts + F)
    brp, bci, bv = oracle.b2sr_pack(41, 41, rowptr, colind, ts)
    rng = np.random.default_rng(F)
    X = rng.standard_normal((41, F)).astype(np.float32)
    bits = (X >= 0).astype(np.int64)
    A = np.zeros((41, 41), np.int64)
    for r in range(41):
        A[r, colind[rowptr[r]:rowptr[r + 1]]] = 1
    Xw = oracle.pack_sign_rows(X)
    c01 = oracle.b2sr_bmm(ts, 41, brp, bci, bv, Xw, F)
    assert np.array_equal(c01, A @ bits)
    cpm = oracle.b2sr_bmm(ts, 41, brp, bci, bv, Xw, F, signed_form=True)
    assert np.array_equal(cpm, A @ (2 * bits - 1))


def py_aligned(ts, brp, bci, bv):
    g = 4 if ts == 8 else 2
    nrp, nci, words = [0], [], []
    for r in range(len(brp) - 1):
        nt, st = brp[r + 1] - brp[r], brp[r]
        padded = (nt + g - 1) // g * g
        for i in range(0, padded, g):
            for j in range(ts):
                w = 0
                for q in range(g):
                    a = int(bv[(st + i + q) * ts + j]) if i + q < nt else 0
                    w |= a << ((g - 1 - q) * (32 // g))
                words.append(w)
        nci.extend(list(bci[st:st + nt]) + [0] * (padded - nt))
        nrp.append(nrp[-1] + padded)
    return nrp, nci, words


@pytest.mark.parametrize("ts", [8, 16])
def test_aligned_formats(oracle_lib, ts):
    rowptr, colind = random_csr(53, 120, 0.15, ts)
    brp, bci, bv = oracle.b2sr_pack(53, 120, rowptr, colind, ts)
    nrp, nci, nv = oracle.b2sr_aligned(ts, brp, bci, bv)
    w = py_aligned(ts, brp, bci, bv)
    assert nrp.tolist() == w[0] and nci.tolist() == w[1] and [int(x) for x in nv] == w[2]


def test_csr_transpose_and_sddmm(oracle_lib):
    rowptr, colind = random_csr(30, 17, 0.3, 9)
    trp, tci, perm = oracle.csr_transpose(30, 17, rowptr, colind)
    A = np.zeros((30, 17), np.int64)
    for r in range(30):
        A[r, colind[rowptr[r]:rowptr[r + 1]]] = 1 + np.arange(rowptr[r + 1] - rowptr[r])
    T = np.zeros((17, 30), np.int64)
    vals = A[A != 0]  # row-major order = CSR order
    for c in range(17):
        for e in range(trp[c], trp[c + 1]):
            T[c, tci[e]] = vals[perm[e]]
        assert list(tci[trp[c]:trp[c + 1]]) == sorted(tci[trp[c]:trp[c + 1]])
    assert np.array_equal(T, A.T)
    rng = np.random.default_rng(2)
    G = rng.standard_normal((30, 8)).astype(np.float32)
    H = rng.standard_normal((17, 8)).astype(np.float32)
    out = oracle.sddmm_f64(rowptr, colind, G, H)
    rows = np.repeat(np.arange(30), np.diff(rowptr))
    want = np.einsum("ek,ek->e", G[rows].astype(np.float64), H[colind].astype(np.float64))
    assert np.allclose(out, want, rtol=1e-12)


def test_bmm_counts_and_bin_layouts(oracle_lib):
    rng = np.random.default_rng(11)
    M, N, Kw = 64, 96, 3
    A = rng.integers(0, 2 ** 32, (Kw, M), dtype=np.uint64).astype(np.uint32)
    B = rng.integers(0, 2 ** 32, (Kw, N), dtype=np.uint64).astype(np.uint32)

    def bits(words):  # [Kw][rows] -> rows x (32 Kw) 0/1, column 0 = bit 31 of word 0
        out = np.zeros((words.shape[1], 32 * words.shape[0]), np.int64)
        for w in range(words.shape[0]):
            for b in range(32):
                out[:, 32 * w + b] = (words[w].astype(np.int64) >> (31 - b)) & 1
        return out

    a, b = bits(A), bits(B)
    xor = (a[:, None, :] != b[None, :, :]).sum(-1)
    andc = (a[:, None, :] & b[None, :, :]).sum(-1)
    assert np.array_equal(oracle.bmm_counts(A, B, M, N, Kw, 0), xor)
    assert np.array_equal(oracle.bmm_counts(A, B, M, N, Kw, 1), andc)
    assert np.array_equal(oracle.bmm_counts(A, B, M, N, Kw, 2), 32 * Kw - 2 * xor)
    f = oracle.bmm32_arow_brow(A, B, M, Kw, N)
    assert np.array_equal(f, (32 * Kw - 2 * xor).astype(np.float32))
    nbits = 32 * Kw
    sign = (nbits - 2 * xor) >= 0
    cb = oracle.bmm32_bin(A, B, M, nbits, N)
    for by in range(N // 32):
        for row in range(M):
            w = int(cb[by * M + row])
            assert [(w >> (31 - j)) & 1 for j in range(32)] == list(sign[row, by * 32:by * 32 + 32])
    cs = oracle.bmm32s_bin(A, B, M, nbits, N)
    for bx in range(M // 32):
        for by in range(N // 32):
            for wi in range(32):
                w = int(cs[bx * N * 32 + by * 32 + wi])
                assert [(w >> (31 - l)) & 1 for l in range(32)] == list(sign[bx * 32 + wi, by * 32:by * 32 + 32])
