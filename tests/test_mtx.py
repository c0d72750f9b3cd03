"""CPU tests of the library's .mtx reader (gbs_mtx_read) against golden
CSR fixtures produced by the reference's own readMtx + coo2csr
(tests/golden/make_mtx_golden.py), and of its error reporting."""
import json
from pathlib import Path

import numpy as np
import pytest

from spmm_eval_gb300 import _lib, ops

GOLD = Path(__file__).resolve().parent / "golden"
FIXTURES = json.loads((GOLD / "mtx_csr.json").read_text())


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_reader_matches_reference(built_lib, name):
    want = FIXTURES[name]
    nrows, ncols, rowptr, colind, vals = ops.read_mtx(GOLD / "mtx" / name)
    assert (nrows, ncols) == (want["nrows"], want["ncols"])
    assert rowptr.tolist() == want["rowptr"]
    assert colind.tolist() == want["colind"]
    assert np.array_equal(vals, np.array(want["vals"], np.float32))


@pytest.mark.parametrize("body, frag", [
    ("%%MatrixMarket matrix coordinate real general\n3 3 4\n1 1 1\n2 2 2\n", "fewer entries"),
    ("%%MatrixMarket matrix coordinate real general\n3 3 1\n4 1 1\n", "outside"),
    ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n", "data type"),
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", "coordinate"),
    ("not a banner\n", "banner"),
])
def test_reader_errors(built_lib, tmp_path, body, frag):
    f = tmp_path / "bad.mtx"
    f.write_text(body)
    with pytest.raises(_lib.GbsError, match=frag):
        ops.read_mtx(f)


def test_reader_roundtrip_generated_graph(built_lib, tmp_path):
    from spmm_eval_gb300 import graphs as G
    g = G.chung_lu(500, 2.0, 2.0, 60.0, 5)
    rows = np.repeat(np.arange(g.nrows), g.degrees().numpy())
    order = np.random.default_rng(0).permutation(g.nnz)  # file order scrambled
    lines = [f"{rows[i] + 1} {g.colind[i].item() + 1}" for i in order]
    f = tmp_path / "g.mtx"
    f.write_text("%%MatrixMarket matrix coordinate pattern general\n"
                 f"{g.nrows} {g.ncols} {g.nnz}\n" + "\n".join(lines) + "\n")
    nrows, ncols, rowptr, colind, vals = ops.read_mtx(f)
    assert np.array_equal(rowptr, g.rowptr.numpy()) and np.array_equal(colind, g.colind.numpy())
    assert np.all(vals == 1.0)


def _big_file(tmp_path, name, n=60000, deg=20, seed=3, sep=" ", value=True, extra=""):
    """A file of n * deg entries (> 8 MB, parsed by several threads) in
    scrambled order, and the CSR a front-to-back read must give."""
    rng = np.random.default_rng(seed)
    rows = np.repeat(np.arange(n), deg)
    cols = rng.integers(0, n, rows.size)
    vals = rng.integers(-9, 10, rows.size).astype(np.float32) / 4
    order = rng.permutation(rows.size)
    r, c, v = rows[order], cols[order], vals[order]
    kind = "real" if value else "pattern"
    body = [f"%%MatrixMarket matrix coordinate {kind} general", f"{n} {n} {rows.size}"]
    if value:
        body += [f"{a + 1}{sep}{b + 1}{sep}{x:g}" for a, b, x in zip(r, c, v)]
    else:
        body += [f"{a + 1}{sep}{b + 1}" for a, b in zip(r, c)]
    f = tmp_path / name
    f.write_text("\n".join(body) + "\n" + extra)
    key = np.lexsort((np.arange(r.size), c, r))  # by (row, col), file order on ties
    rowptr = np.zeros(n + 1, np.int64)
    rowptr[1:] = np.cumsum(np.bincount(r, minlength=n))
    return f, rowptr, c[key], (v[key] if value else np.ones(r.size, np.float32))


@pytest.mark.parametrize("sep, value", [(" ", True), (" ", False), ("\n", True)])
def test_reader_large_file_threads(built_lib, tmp_path, sep, value):
    """Several parse threads (and, with one token per line, the front-to-back
    fallback when an entry spans a cut) give the front-to-back result; extra
    entries and trailing junk after the stated count are ignored."""
    f, rowptr, colind, vals = _big_file(tmp_path, "big.mtx", sep=sep, value=value, extra="1 1 1\njunk\n")
    assert f.stat().st_size > 8 << 20
    nrows, ncols, rp, ci, vv = ops.read_mtx(f)
    assert np.array_equal(rp, rowptr) and np.array_equal(ci, colind)
    assert np.array_equal(vv, vals)


def test_reader_large_file_errors(built_lib, tmp_path):
    """The first bad entry is reported by its position in the file, also when
    it sits in a later thread's piece."""
    f, *_ = _big_file(tmp_path, "big.mtx")
    lines = f.read_text().split("\n")
    bad = 2 + 1_000_000  # header lines + index of the bad entry
    lines[bad] = "999999 1 1"
    f.write_text("\n".join(lines))
    with pytest.raises(_lib.GbsError, match="entry 1000001 outside"):
        ops.read_mtx(f)
    lines[bad] = "12 1 1"
    f.write_text("\n".join(lines[:-50000]) + "\n")  # truncated
    with pytest.raises(_lib.GbsError, match="fewer entries"):
        ops.read_mtx(f)


@pytest.mark.parametrize("with_vals", [True, False])
def test_csr_bin_roundtrip(built_lib, tmp_path, with_vals):
    """A CSR written to the binary cache reads back identically; a pattern
    (no values) reads back as 1.0 like a pattern .mtx."""
    f, rowptr, colind, vals = _big_file(tmp_path, "g.mtx", n=3000, deg=7, value=with_vals)
    n, m, rp, ci, vv = ops.read_mtx(f)
    b = tmp_path / "g.bin"
    ops.write_csr_bin(b, n, m, rp, ci, vv if with_vals else None)
    assert b.stat().st_size == 24 + 4 * (n + 1) + 4 * ci.size * (2 if with_vals else 1)
    n2, m2, rp2, ci2, vv2 = ops.read_csr_bin(b)
    assert (n2, m2) == (n, m)
    assert np.array_equal(rp2, rp) and np.array_equal(ci2, ci)
    assert np.array_equal(vv2, vv if with_vals else np.ones_like(vv))


def test_csr_bin_empty(built_lib, tmp_path):
    b = tmp_path / "e.bin"
    ops.write_csr_bin(b, 5, 3, np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    n, m, rp, ci, vv = ops.read_csr_bin(b)
    assert (n, m) == (5, 3) and np.array_equal(rp, np.zeros(6)) and ci.size == 0 and vv.size == 0


def test_csr_bin_rejects_bad_files(built_lib, tmp_path):
    """Wrong magic, truncation, a row pointer out of order and a column
    outside [0, ncols) are errors, never a CSR handed to the kernels."""
    b = tmp_path / "g.bin"
    rp = np.array([0, 2, 3, 5], np.int32)
    ci = np.array([0, 3, 1, 2, 3], np.int32)
    ops.write_csr_bin(b, 3, 4, rp, ci, np.arange(5, dtype=np.float32))
    good = b.read_bytes()
    cases = {
        "magic": b"XBSCSR1\0" + good[8:],
        "trunc": good[:-3],
        "header": good[:8] + np.array([3, 4, 5, 7], np.int32).tobytes() + good[24:],
        "rowptr": good[:24] + np.array([0, 3, 2, 5], np.int32).tobytes() + good[40:],
        "column": good[:40] + np.array([0, 4, 1, 2, 3], np.int32).tobytes() + good[60:],
    }
    for name, data in cases.items():
        bad = tmp_path / f"{name}.bin"
        bad.write_bytes(data)
        with pytest.raises(_lib.GbsError, match="csr bin"):
            ops.read_csr_bin(bad)
    with pytest.raises(_lib.GbsError, match="cannot open"):
        ops.read_csr_bin(tmp_path / "missing.bin")


@pytest.mark.parametrize("tile", [4, 8, 16, 32])
def test_b2sr_bin_roundtrip(built_lib, tmp_path, tile):
    """Packed tiles (the oracle's packing of a ragged power-law graph) written
    to the B2SR cache read back identically."""
    import oracle
    from spmm_eval_gb300 import graphs as G
    g = G.chung_lu(1003, 2.0, 2.0, 60.0, 11)
    rp, ci = g.rowptr.numpy(), g.colind.numpy()
    brp, bci, bv = oracle.b2sr_pack(g.nrows, g.ncols, rp, ci, tile)
    f = tmp_path / f"g{tile}.b2sr"
    ops.write_b2sr_bin(f, (g.nrows, g.ncols, tile, brp, bci, bv))
    n, m, T, rp2, ci2, v2 = ops.read_b2sr_bin(f)
    assert (n, m, T) == (g.nrows, g.ncols, tile)
    assert np.array_equal(rp2, brp) and np.array_equal(ci2, bci)
    assert v2.dtype == bv.dtype and np.array_equal(v2, bv)
    assert f.stat().st_size == 28 + 4 * brp.size + 4 * bci.size + bv.nbytes


def test_b2sr_bin_rejects_bad_tiles(built_lib, tmp_path):
    """A bit past the last column or row, a tile column out of order, a
    wrong magic or a truncated file is an error on write or on read."""
    # 6 x 6 matrix, tile 4: block rows {0, 1}, tile columns {0, 1}
    rp = np.array([0, 2, 3], np.int32)
    ci = np.array([0, 1, 1], np.int32)
    val = np.zeros(12, np.uint8)
    val[0] = 0b1000       # row 0, column 0
    val[4 + 1] = 0b1100   # row 1, columns 4, 5 of tile column 1
    val[8 + 1] = 0b0100   # row 5, column 5
    good = (6, 6, 4, rp, ci, val)
    f = tmp_path / "ok.b2sr"
    ops.write_b2sr_bin(f, good)
    assert np.array_equal(ops.read_b2sr_bin(f)[5], val)
    bad_col = val.copy()
    bad_col[4 + 1] = 0b1110       # column 6 does not exist
    bad_row = val.copy()
    bad_row[8 + 2] = 0b0100       # row 6 does not exist
    bad_nibble = val.copy()
    bad_nibble[0] = 0x18          # tile 4 rows use the low nibble only
    for v, rp_, ci_ in ((bad_col, rp, ci), (bad_row, rp, ci), (bad_nibble, rp, ci),
                        (val, rp, np.array([1, 0, 1], np.int32)), (val, np.array([0, 2, 4], np.int32), ci)):
        with pytest.raises(_lib.GbsError, match="b2sr bin"):
            ops.write_b2sr_bin(tmp_path / "x.b2sr", (6, 6, 4, rp_, ci_, v))
    data = f.read_bytes()
    for name, blob in {"magic": b"GBSB2SR2" + data[8:], "trunc": data[:-1],
                       "header": data[:16] + np.int32(5).tobytes() + data[20:]}.items():
        p = tmp_path / f"{name}.b2sr"
        p.write_bytes(blob)
        with pytest.raises(_lib.GbsError, match="b2sr bin"):
            ops.read_b2sr_bin(p)
    # a flipped bit past the last column inside an otherwise intact file
    p = tmp_path / "flip.b2sr"
    p.write_bytes(data[:-3] + bytes([data[-3] | 0b0010]) + data[-2:])
    with pytest.raises(_lib.GbsError, match="b2sr bin"):
        ops.read_b2sr_bin(p)


def test_reader_float_tokens_match_strtof(built_lib, tmp_path):
    """The threaded parser's fast number scanning gives exactly what the C
    library's strtof (the reference's %f) gives, for every token form: signs,
    leading dot, exponents, denormals, overflow, halfway cases, hex floats,
    inf / nan spellings."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.strtof.restype = ctypes.c_float
    libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
    toks = ["1.5", "-0.1", ".5", "-.5", "5.", "+2.5", "1e-40", "-1e-45", "1e-50", "3.4028236e38",
            "-3.5e38", "1.00000005960464477539", "16777217", "0.333333343267440796", "0x1p-3",
            "-0x1.8p1", "inf", "-Infinity", "nan", "1E+3", "007", "-0", "123456789012345678901234567890"]
    per_tok = {t: libc.strtof(t.encode(), None) for t in toks}
    reps = 560000 // len(toks) + 1  # an entry section over 8 MB: the threaded parser
    n = 1000
    rng = np.random.default_rng(5)
    rc = rng.integers(1, n + 1, (reps * len(toks), 2))
    lines = [f"{a} {b} {toks[i % len(toks)]}" for i, (a, b) in enumerate(rc)]
    want = [per_tok[toks[i % len(toks)]] for i in range(len(lines))]
    body = "\n".join(lines) + "\n"
    assert len(body) > 8 << 20
    f = tmp_path / "tok.mtx"
    f.write_text("%%MatrixMarket matrix coordinate real general\n" + f"{n} {n} {len(lines)}\n" + body)
    # the CSR orders entries by (row, col, file order); map back by that order
    r, c = rc[:, 0] - 1, rc[:, 1] - 1
    key = np.lexsort((np.arange(len(lines)), c, r))
    want = np.array(want, np.float32)[key]
    _, _, rp, ci, vv = ops.read_mtx(f)
    assert np.array_equal(ci, c[key])
    same = (vv.view(np.uint32) == want.view(np.uint32)) | (np.isnan(vv) & np.isnan(want))
    assert same.all(), [toks[i % len(toks)] for i in np.nonzero(~same)[0][:5]]


def test_reader_few_heavy_rows_stable(built_lib, tmp_path):
    """Few rows and many duplicate (row, col) pairs: the threaded counting
    sort and the per-row sorts keep file order among equal columns, as the
    reference's stable sorts do."""
    rng = np.random.default_rng(9)
    nz, n, m = 1_200_000, 7, 50
    r = rng.integers(0, n, nz)
    c = rng.integers(0, m, nz)
    v = (np.arange(nz) % 1000).astype(np.float32)  # distinct along file order within a pair
    f = tmp_path / "heavy.mtx"
    f.write_text("%%MatrixMarket matrix coordinate real general\n" + f"{n} {m} {nz}\n" +
                 "\n".join(f"{a + 1} {b + 1} {x:g}" for a, b, x in zip(r, c, v)) + "\n")
    assert f.stat().st_size > 8 << 20
    key = np.lexsort((np.arange(nz), c, r))
    _, _, rp, ci, vv = ops.read_mtx(f)
    assert np.array_equal(rp, np.concatenate([[0], np.cumsum(np.bincount(r, minlength=n))]))
    assert np.array_equal(ci, c[key]) and np.array_equal(vv, v[key])
