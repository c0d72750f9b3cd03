"""Regenerates tests/golden/mtx_csr.json: runs the reference's own ingest
path (readMtx + coo2csr from the reference sources, built by
`make -C oracle REF=<checkout> ref` into oracle/_ref/readmtx_ref) on every
tests/golden/mtx/*.mtx and records the CSR it produces.  Needs the reference
sources, so it is run by hand in the development container, not by tests."""
import json
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF = ROOT / "oracle" / "_ref" / "readmtx_ref"


def main() -> int:
    # the reference checkout: first argument, SPMM_EVAL_REFERENCE, or beside the repository
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPMM_EVAL_REFERENCE", str(ROOT.parent / "reference"))
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), f"REF={ref}", "ref"], check=True)
    out = {}
    for f in sorted((HERE / "mtx").glob("*.mtx")):
        txt = subprocess.run([str(REF), str(f)], check=True, capture_output=True, text=True).stdout.split("\n")
        nrows, ncols, nnz_hdr, nnz = map(int, txt[0].split())
        rowptr = [int(x) for x in txt[1].split()]
        colind = [int(x) for x in txt[2].split()]
        vals = [float(x) for x in txt[3].split()]
        out[f.name] = {"nrows": nrows, "ncols": ncols, "nnz": nnz, "rowptr": rowptr,
                       "colind": colind, "vals": vals}
    (HERE / "mtx_csr.json").write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {len(out)} fixtures")
    return 0


if __name__ == "__main__":
    sys.exit(main())
