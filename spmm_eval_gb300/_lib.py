"""ctypes binding of ``lib/libgbspmm.so`` (the C ABI in ``include/gbspmm.h``).

The shared library is the only compute path: if it is missing this module
raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libgbspmm.so"

GBS_OK, GBS_ERR_INVALID_ARG, GBS_ERR_UNSUPPORTED, GBS_ERR_CUDA, GBS_ERR_OOM, GBS_ERR_INTERNAL = range(6)
GBS_F32, GBS_BF16, GBS_F16 = 0, 1, 2

_STATUS_NAMES = {
    GBS_OK: "GBS_OK",
    GBS_ERR_INVALID_ARG: "GBS_ERR_INVALID_ARG",
    GBS_ERR_UNSUPPORTED: "GBS_ERR_UNSUPPORTED",
    GBS_ERR_CUDA: "GBS_ERR_CUDA",
    GBS_ERR_OOM: "GBS_ERR_OOM",
    GBS_ERR_INTERNAL: "GBS_ERR_INTERNAL",
}

p = C.c_void_p
i32 = C.c_int
i64 = C.c_int64
sz = C.c_size_t
st = C.c_int  # gbs_status
pi32 = C.POINTER(C.c_int)
psz = C.POINTER(C.c_size_t)

class HostB2SR(C.Structure):
    _fields_ = [("nrows", C.c_int), ("ncols", C.c_int), ("tile", C.c_int), ("nblockrows", C.c_int),
                ("nnzb", C.c_int), ("rowptr", C.POINTER(C.c_int)), ("colind", C.POINTER(C.c_int)),
                ("val", C.c_void_p)]


class HostCSR(C.Structure):
    _fields_ = [("nrows", C.c_int), ("ncols", C.c_int), ("nnz", C.c_int),
                ("rowptr", C.POINTER(C.c_int)), ("colind", C.POINTER(C.c_int)),
                ("vals", C.POINTER(C.c_float))]


# name -> (restype, argtypes); every entry point declared in include/gbspmm.h
SIGNATURES: dict[str, tuple] = {
    "gbs_last_error": (C.c_char_p, []),
    "gbs_abi_version": (C.c_int, []),
    "gbs_pool_trim": (st, []),
    "gbs_mtx_read": (st, [C.c_char_p, C.POINTER(HostCSR)]),
    "gbs_host_csr_free": (None, [C.POINTER(HostCSR)]),
    "gbs_csr_write_bin": (st, [C.c_char_p, C.POINTER(HostCSR)]),
    "gbs_csr_read_bin": (st, [C.c_char_p, C.POINTER(HostCSR)]),
    "gbs_b2sr_write_bin": (st, [C.c_char_p, C.POINTER(HostB2SR)]),
    "gbs_b2sr_read_bin": (st, [C.c_char_p, C.POINTER(HostB2SR)]),
    "gbs_host_b2sr_free": (None, [C.POINTER(HostB2SR)]),
    "gbs_csr_spmm_workspace_size": (st, [i32, i32, i32, i32, psz]),
    "gbs_csr_spmm_workspace_init": (st, [p, sz, p]),
    "gbs_csr_spmm": (st, [i32, i32, i32, p, p, p, p, i32, i32, p, p, sz, p]),
    "gbs_csr_spmm_cb": (st, [i32, i32, i32, p, p, p, p, i32, i32, i32, p, p, sz, p]),
    "gbs_csr_spmm_f32": (st, [i32, i32, i32, p, p, p, p, i32, p, p]),
    "gbs_spmm_host_ctx_create": (st, [C.POINTER(p)]),
    "gbs_spmm_host_ctx_destroy": (st, [p]),
    "gbs_csr_spmm_host": (st, [p, i32, i32, i32, p, p, p, p, i32, i32, p, p]),
    "gbs_csr_spmm_plan_create": (st, [i32, i32, i32, p, p, p, i32, i32, i32, p, C.POINTER(p)]),
    "gbs_csr_spmm_plan_create_scaled": (st, [i32, i32, i32, p, p, p, p, i32, i32, i32, p, C.POINTER(p)]),
    "gbs_csr_spmm_scaled": (st, [i32, i32, i32, p, p, p, p, p, i32, i32, p, p, sz, p]),
    "gbs_degree_rsqrt": (st, [i32, p, p, p]),
    "gbs_csr_spmm_plan_parts": (st, [p, pi32]),
    "gbs_csr_spmm_planned": (st, [p, p, p, p, sz, p]),
    "gbs_csr_spmm_plan_destroy": (st, [p]),
    "gbs_csr_spmm_noalloc": (st, [i32, i32, i32, p, p, p, p, i32, i32, p, p]),
    "gbs_csr_transpose_create": (st, [i32, i32, i32, p, p, p, C.POINTER(p)]),
    "gbs_csr_transpose_arrays": (st, [p, C.POINTER(p), C.POINTER(p), C.POINTER(p)]),
    "gbs_csr_transpose_copy": (st, [p, p, p, p, p]),
    "gbs_csr_transpose_values": (st, [p, p, p, p]),
    "gbs_csr_transpose_destroy": (st, [p]),
    "gbs_csr_spmm_transposed": (st, [p, p, p, i32, i32, p, p, sz, p]),
    "gbs_spmm_backward": (st, [p, p, p, p, i32, i32, p, p, p, sz, p]),
    "gbs_spmm_backward_plan_create": (st, [p, p, i32, i32, i32, p, C.POINTER(p)]),
    "gbs_spmm_backward_plan_parts": (st, [p, pi32]),
    "gbs_spmm_backward_plan_destroy": (st, [p]),
    "gbs_spmm_backward_planned": (st, [p, p, p, p, p, p, sz, p]),
    "gbs_sddmm": (st, [i32, i32, i32, p, p, p, p, i32, i32, p, p]),
    "gbs_csr2b2sr_nnzb": (st, [i32, i32, i32, p, p, i32, p, pi32, p]),
    "gbs_csr2b2sr": (st, [i32, i32, i32, p, p, i32, p, p, p, p]),
    "gbs_csr2bsr_batch": (st, [p, p, i32, i32, i32, p, p, p, i32, i32, i32]),
    "gbs_b2sr_aligned_nnzb": (st, [i32, i32, p, p, pi32, p]),
    "gbs_b2sr_pack_aligned": (st, [i32, i32, p, p, p, p, p, p, p]),
    "gbs_b2sr_spmm": (st, [i32, i32, i32, p, p, p, p, i32, i32, p, p]),
    "gbs_spmm4_full_full": (st, [p, p, p, p, p, i32, i32, p]),
    "gbs_b2sr_bmm": (st, [i32, i32, i32, p, p, p, p, i32, i32, p, p]),
    "gbs_pack_sign_rows": (st, [p, i32, i32, p, p]),
    "gbs_pack_sign_colud": (st, [p, i32, i32, p, p]),
    "gbs_bmm_b1": (st, [p, p, i32, i32, i32, i32, i32, p, p]),
    "gbs_bmm_tc_timeouts": (st, [pi32]),
    "gbs_bmm32_arow_brow": (st, [p, p, p, i32, i32, i32, p]),
    "gbs_bmm32_bin": (st, [p, p, p, i32, i32, i32, p]),
    "gbs_bmm32s_bin": (st, [p, p, p, i32, i32, i32, p]),
    "gbs_bmm_bin": (st, [p, p, p, i32, i32, i32, i32, i32, p]),
    "gbs_b2sr_bmm_aligned": (st, [i32, i32, i32, p, p, p, p, i32, i32, p, p]),
}


class GbsError(RuntimeError):
    """A non-zero gbs_status returned by the library."""

    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: {_STATUS_NAMES.get(status, status)}: {message}")


_lock = threading.Lock()
_lib: C.CDLL | None = None


def load() -> C.CDLL:
    """Load libgbspmm.so once and attach the argument types."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is not built; run spmm_eval_gb300.build.build() "
                    "(there is no CPU fallback for any operation)")
            lib = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def call(name: str, *args) -> None:
    """Call an entry point and raise GbsError on a non-zero status."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != GBS_OK:
        msg = lib.gbs_last_error().decode(errors="replace")
        raise GbsError(rc, name, msg)
