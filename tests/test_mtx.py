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
