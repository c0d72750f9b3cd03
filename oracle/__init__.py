"""CPU oracle for the spmm_eval path -- TEST INFRASTRUCTURE ONLY.

numpy/ctypes wrapper over ``oracle/oracle.c`` (built by ``oracle/Makefile``).
Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use it, and only as the checker / the timed CPU baseline;
the library in ``spmm_eval_gb300`` never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_READMTX = HERE / "_ref" / "readmtx_ref"

_lock = threading.Lock()
_lib = None


def build(ref_dir: str | None = None) -> None:
    """make the oracle; with ref_dir (a reference checkout), also the
    reference-built checkers in _ref/ (the readMtx harness and the fatbin of
    the reference's CUDA kernels)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if ref_dir:
        subprocess.run(["make", "-s", "-C", str(HERE), f"REF={ref_dir}", "ref", "refkern"], check=True)


def lib() -> C.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            if not LIB.exists() or LIB.stat().st_mtime < (HERE / "oracle.c").stat().st_mtime:
                build()
            _lib = C.CDLL(str(LIB))
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def max_threads() -> int:
    f = lib().orc_max_threads
    f.restype = C.c_int
    return int(f())


def csr_spmm_f64(rowptr, colind, vals, B, rows=None, with_mag=True):
    """FP64 C = A@B (rows subset optional) and magnitude sum |A|@|B|."""
    rowptr, colind, B = _i32(rowptr), _i32(colind), _f32(B)
    vals = None if vals is None else _f32(vals)
    n = rowptr.size - 1
    F = B.shape[1]
    rows_a = None if rows is None else _i32(rows)
    cnt = n if rows is None else rows_a.size
    Cout = np.empty((cnt, F), np.float64)
    M = np.empty((cnt, F), np.float64) if with_mag else None
    lib().orc_csr_spmm_f64(C.c_int(n), _p(rowptr), _p(colind), _p(vals), _p(B), C.c_int(F),
                           _p(rows_a), C.c_int(cnt), _p(Cout), _p(M))
    return Cout, M


def csr_spmm_f32(rowptr, colind, vals, B, r0=0, r1=None, nthreads=0, out=None):
    """FP32 C[r0:r1] = A[r0:r1] @ B, OpenMP over rows (out: optional
    preallocated (r1 - r0, F) float32 C-contiguous array)."""
    rowptr, colind, B = _i32(rowptr), _i32(colind), _f32(B)
    vals = None if vals is None else _f32(vals)
    n = rowptr.size - 1
    r1 = n if r1 is None else r1
    F = B.shape[1]
    if out is None:
        out = np.empty((r1 - r0, F), np.float32)
    elif out.shape != (r1 - r0, F) or out.dtype != np.float32 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float32 array of shape (r1 - r0, F)")
    lib().orc_csr_spmm_f32(C.c_int(r0), C.c_int(r1), _p(rowptr), _p(colind), _p(vals), _p(B),
                           C.c_int(F), _p(out), C.c_int(nthreads))
    return out


_VAL_DT = {4: np.uint8, 8: np.uint8, 16: np.uint16, 32: np.uint32}


def b2sr_pack(nrows, ncols, rowptr, colind, ts):
    """CSR -> B2SR (rowptr, colind, packed vals) with the reference layout."""
    rowptr, colind = _i32(rowptr), _i32(colind)
    mb = (nrows + ts - 1) // ts
    brp = np.empty(mb + 1, np.int32)
    f = lib().orc_b2sr_count
    f.restype = C.c_longlong
    nnzb = f(C.c_int(nrows), C.c_int(ncols), _p(rowptr), _p(colind), C.c_int(ts), _p(brp))
    if nnzb < 0:
        raise ValueError("CSR columns unsorted or out of range")
    bci = np.empty(nnzb, np.int32)
    bv = np.empty(nnzb * ts, _VAL_DT[ts])
    lib().orc_b2sr_fill(C.c_int(nrows), C.c_int(ncols), _p(rowptr), _p(colind), C.c_int(ts),
                        _p(brp), _p(bci), _p(bv))
    return brp, bci, bv


def b2sr_aligned(ts, bsr_rowptr, bsr_colind, bsr_val):
    bsr_rowptr, bsr_colind = _i32(bsr_rowptr), _i32(bsr_colind)
    bsr_val = np.ascontiguousarray(bsr_val, _VAL_DT[ts])
    mb = bsr_rowptr.size - 1
    f = lib().orc_b2sr_aligned
    f.restype = C.c_longlong
    nwords = f(C.c_int(ts), C.c_int(mb), _p(bsr_rowptr), _p(bsr_colind), _p(bsr_val), None, None, None)
    g = 4 if ts == 8 else 2
    ntiles = int(sum(((bsr_rowptr[i + 1] - bsr_rowptr[i]) + g - 1) // g * g for i in range(mb)))
    nrp = np.empty(mb + 1, np.int32)
    nci = np.empty(ntiles, np.int32)
    nv = np.empty(nwords, np.uint32)
    f(C.c_int(ts), C.c_int(mb), _p(bsr_rowptr), _p(bsr_colind), _p(bsr_val), _p(nrp), _p(nci), _p(nv))
    return nrp, nci, nv


def b2sr4_spmm_ref(nrows, bsr_rowptr, bsr_colind, bsr_val, B):
    """spmm4_full_full_new2 restated: C zero-filled, nonzero results stored."""
    bsr_rowptr, bsr_colind, B = _i32(bsr_rowptr), _i32(bsr_colind), _f32(B)
    bsr_val = np.ascontiguousarray(bsr_val, np.uint8)
    F = B.shape[1]
    out = np.zeros((nrows, F), np.float32)
    lib().orc_b2sr4_spmm_ref(C.c_int(bsr_rowptr.size - 1), _p(bsr_rowptr), _p(bsr_colind),
                             _p(bsr_val), _p(B), C.c_int(F), _p(out), C.c_longlong(nrows))
    return out


def b2sr_spmm(ts, nrows, bsr_rowptr, bsr_colind, bsr_val, B):
    bsr_rowptr, bsr_colind, B = _i32(bsr_rowptr), _i32(bsr_colind), _f32(B)
    bsr_val = np.ascontiguousarray(bsr_val, _VAL_DT[ts])
    F = B.shape[1]
    out = np.empty((nrows, F), np.float32)
    lib().orc_b2sr_spmm(C.c_int(ts), C.c_int(nrows), C.c_int(bsr_rowptr.size - 1), _p(bsr_rowptr),
                        _p(bsr_colind), _p(bsr_val), _p(B), C.c_int(F), _p(out))
    return out


def pack_sign_rows(X):
    X = _f32(X)
    n, F = X.shape
    out = np.empty((n, (F + 31) // 32), np.uint32)
    lib().orc_pack_sign_rows(_p(X), C.c_int(n), C.c_int(F), _p(out))
    return out


def pack_sign_colud(A):
    A = _f32(A)
    H, Wd = A.shape
    out = np.empty(((Wd + 31) // 32, (H + 31) // 32 * 32), np.uint32)
    lib().orc_pack_sign_colud(_p(A), C.c_int(H), C.c_int(Wd), _p(out))
    return out


def b2sr_bmm(ts, nrows, bsr_rowptr, bsr_colind, bsr_val, Xbits, F, signed_form=False):
    bsr_rowptr, bsr_colind = _i32(bsr_rowptr), _i32(bsr_colind)
    bsr_val = np.ascontiguousarray(bsr_val, _VAL_DT[ts])
    Xbits = np.ascontiguousarray(Xbits, np.uint32)
    out = np.empty((nrows, F), np.int32)
    lib().orc_b2sr_bmm(C.c_int(ts), C.c_int(nrows), C.c_int(bsr_rowptr.size - 1), _p(bsr_rowptr),
                       _p(bsr_colind), _p(bsr_val), _p(Xbits), C.c_int(F), C.c_int(int(signed_form)),
                       _p(out))
    return out


def bmm_counts(A, B, M, N, Kw, mode):
    A = np.ascontiguousarray(A, np.uint32)
    B = np.ascontiguousarray(B, np.uint32)
    out = np.empty((M, N), np.int32)
    lib().orc_bmm_counts(_p(A), _p(B), C.c_int(M), C.c_int(N), C.c_int(Kw), C.c_int(mode), _p(out))
    return out


def bmm32_arow_brow(A, B, M, Kw, N):
    A = np.ascontiguousarray(A, np.uint32)
    B = np.ascontiguousarray(B, np.uint32)
    out = np.empty((M, N), np.float32)
    lib().orc_bmm32_arow_brow(_p(A), _p(B), C.c_int(M), C.c_int(Kw), C.c_int(N), _p(out))
    return out


def bmm32_bin(A, B, m, n, k):
    A = np.ascontiguousarray(A, np.uint32)
    B = np.ascontiguousarray(B, np.uint32)
    out = np.zeros((k // 32) * m, np.uint32)
    lib().orc_bmm32_bin(_p(A), _p(B), C.c_int(m), C.c_int(n), C.c_int(k), _p(out))
    return out


def bmm32s_bin(A, B, m, n, k):
    A = np.ascontiguousarray(A, np.uint32)
    B = np.ascontiguousarray(B, np.uint32)
    out = np.zeros(m * k, np.uint32)
    lib().orc_bmm32s_bin(_p(A), _p(B), C.c_int(m), C.c_int(n), C.c_int(k), _p(out))
    return out


def csr_transpose(nrows, ncols, rowptr, colind):
    rowptr, colind = _i32(rowptr), _i32(colind)
    nnz = int(rowptr[-1])
    trp = np.empty(ncols + 1, np.int32)
    tci = np.empty(nnz, np.int32)
    perm = np.empty(nnz, np.int32)
    lib().orc_csr_transpose(C.c_int(nrows), C.c_int(ncols), _p(rowptr), _p(colind), _p(trp),
                            _p(tci), _p(perm))
    return trp, tci, perm


def sddmm_f64(rowptr, colind, G, H):
    rowptr, colind, G, H = _i32(rowptr), _i32(colind), _f32(G), _f32(H)
    out = np.empty(colind.size, np.float64)
    lib().orc_sddmm_f64(C.c_int(rowptr.size - 1), _p(rowptr), _p(colind), _p(G), _p(H),
                        C.c_int(G.shape[1]), _p(out))
    return out


def rel_err(got, ref64, mag):
    """max / mean of |got - ref| / max(M, tiny), M = |A|@|B| (the scale of
    the rounding-error bound of a sum of products); entries with M == 0 must
    match exactly (they are returned as inf otherwise)."""
    got = np.asarray(got, np.float64)
    d = np.abs(got - ref64)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(mag > 0, d / np.where(mag > 0, mag, 1.0), np.where(d == 0, 0.0, np.inf))
    return float(r.max()) if r.size else 0.0, float(r.mean()) if r.size else 0.0
