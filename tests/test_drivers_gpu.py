"""GPU tests of the drop-in executables ({kernel_name} {matrix.mtx}
{hidden_size}, as the reference's spmm/spmmfbf): each runs on a synthetic
power-law graph written as a pattern .mtx, prints the reference's two
result lines first, verifies against cusparseSpMM and exits 0."""
import json
import re
import subprocess

import numpy as np
import pytest

from spmm_eval_gb300 import build as B
from spmm_eval_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mtx_file(tmp_path_factory, cuda):
    B.build_apps()
    g = G.chung_lu(20_003, 2.0, 1.5, 800.0, 77)  # nrows not a multiple of 4
    rows = np.repeat(np.arange(g.nrows), g.degrees().numpy()) + 1
    cols = g.colind.numpy() + 1
    f = tmp_path_factory.mktemp("mtx") / "plaw.mtx"
    with open(f, "w") as fh:
        fh.write("%%MatrixMarket matrix coordinate pattern general\n")
        fh.write(f"{g.nrows} {g.ncols} {g.nnz}\n")
        np.savetxt(fh, np.stack([rows, cols], 1), fmt="%d")
    return f


@pytest.mark.parametrize("name, F", [("spmmfbf", 32), ("spmmfbf", 64), ("spmmfbf", 256), ("spmmcsr", 64),
                                     ("spmmcsr_bf16", 128), ("spmmb2sr8", 64), ("spmmb2sr16", 64),
                                     ("spmmb2sr32", 96), ("spmmbmm", 64)])
def test_driver(mtx_file, name, F):
    exe = B.BIN / name
    r = subprocess.run([str(exe), str(mtx_file), str(F)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.strip().split("\n")
    label = "b2sr" if name == "spmmfbf" else name
    assert re.fullmatch(rf"{label}: \d+\.\d{{3}}, csr-float: \d+\.\d{{3}}", lines[0]), lines[0]
    assert lines[1] == "TEST PASSED: 1"
    info = json.loads(lines[2])
    assert info["pass"] and info["F"] == F and info["nrows"] == 20_003


def test_driver_usage_error(mtx_file):
    r = subprocess.run([str(B.BIN / "spmmfbf"), str(mtx_file)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
