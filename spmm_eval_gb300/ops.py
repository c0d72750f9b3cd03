"""Torch-facing wrappers over the C ABI.

Torch provides device memory and streams only; every operation runs the
sm_103a kernels in ``lib/libgbspmm.so`` through ``_lib.call``.  Inputs must
already be CUDA tensors of the documented dtypes: nothing here converts,
copies to the device or computes on the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib

_DT = {torch.float32: _lib.GBS_F32, torch.bfloat16: _lib.GBS_BF16, torch.float16: _lib.GBS_F16}


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _check_cuda(name: str, t: torch.Tensor, dtype: torch.dtype | tuple | None = None) -> None:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor (no CPU path exists)")
    if dtype is not None:
        ok = t.dtype in dtype if isinstance(dtype, tuple) else t.dtype == dtype
        if not ok:
            raise TypeError(f"{name} has dtype {t.dtype}, expected {dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


@dataclass
class CSR:
    """A CSR matrix on the device (int32 indices, FP32 values or None)."""

    rowptr: torch.Tensor
    colind: torch.Tensor
    vals: torch.Tensor | None
    nrows: int
    ncols: int

    @property
    def nnz(self) -> int:
        return int(self.colind.numel())

    def validate_layout(self) -> None:
        _check_cuda("rowptr", self.rowptr, torch.int32)
        _check_cuda("colind", self.colind, torch.int32)
        if self.vals is not None:
            _check_cuda("vals", self.vals, torch.float32)
        if self.rowptr.numel() != self.nrows + 1:
            raise ValueError("rowptr must have nrows + 1 entries")


class SpmmWorkspace:
    """Zero-filled workspace for ``csr_spmm``, grown on demand and reused.

    The kernels leave it zero-filled after every call; one workspace must not
    serve two calls that can overlap on the GPU.
    """

    def __init__(self) -> None:
        self.buf: torch.Tensor | None = None

    def get(self, nbytes: int, device: torch.device) -> torch.Tensor:
        if self.buf is None or self.buf.numel() < nbytes or self.buf.device != device:
            self.buf = torch.zeros(max(nbytes, 256), dtype=torch.uint8, device=device)
        return self.buf


_WS_CACHE: dict[tuple, int] = {}


def spmm_workspace_bytes(nrows: int, nnz: int, F: int, dtype: torch.dtype) -> int:
    key = (torch.cuda.current_device(), nrows, nnz, F, dtype)
    if key not in _WS_CACHE:
        out = C.c_size_t(0)
        _lib.call("gbs_csr_spmm_workspace_size", nrows, nnz, F, _DT[dtype], C.byref(out))
        _WS_CACHE[key] = int(out.value)
    return _WS_CACHE[key]


def csr_spmm(A: CSR, B: torch.Tensor, out: torch.Tensor | None = None,
             workspace: SpmmWorkspace | None = None, col_block: int = 0) -> torch.Tensor:
    """C = A @ B with A in CSR, B (ncols x F) FP32/BF16/FP16, C FP32.

    col_block > 0 forces the column-block width (must divide F)."""
    A.validate_layout()
    _check_cuda("B", B, tuple(_DT))
    if B.dim() != 2 or B.shape[0] != A.ncols:
        raise ValueError(f"B must be ({A.ncols}, F), got {tuple(B.shape)}")
    F = int(B.shape[1])
    if out is None:
        out = torch.empty((A.nrows, F), dtype=torch.float32, device=B.device)
    else:
        _check_cuda("out", out, torch.float32)
        if tuple(out.shape) != (A.nrows, F):
            raise ValueError("out has the wrong shape")
    ws = workspace or SpmmWorkspace()
    nbytes = spmm_workspace_bytes(A.nrows, A.nnz, F, B.dtype)
    buf = ws.get(nbytes, B.device)
    _lib.call("gbs_csr_spmm_cb", A.nrows, A.ncols, A.nnz, _ptr(A.rowptr), _ptr(A.colind),
              _ptr(A.vals), _ptr(B), _DT[B.dtype], F, int(col_block), _ptr(out), _ptr(buf),
              buf.numel(), _stream(B.device))
    return out


def degree_rsqrt(A: CSR) -> torch.Tensor:
    """D^-1/2 of A's row counts (FP64 on the device, rounded to FP32; 0 for
    an empty row)."""
    A.validate_layout()
    out = torch.empty(A.nrows, dtype=torch.float32, device=A.rowptr.device)
    _lib.call("gbs_degree_rsqrt", A.nrows, _ptr(A.rowptr), _ptr(out), _stream(A.rowptr.device))
    return out


def csr_spmm_scaled(A: CSR, rowscale: torch.Tensor | None, colscale: torch.Tensor | None, B: torch.Tensor,
                    out: torch.Tensor | None = None, workspace: SpmmWorkspace | None = None) -> torch.Tensor:
    """C[r] = rowscale[r] * sum over A's stored entries (r, c) of
    colscale[c] * B[c] (A's values are not used; None = all ones)."""
    A.validate_layout()
    _check_cuda("B", B, tuple(_DT))
    for name, t, n in (("rowscale", rowscale, A.nrows), ("colscale", colscale, A.ncols)):
        if t is not None:
            _check_cuda(name, t, torch.float32)
            if t.numel() != n:
                raise ValueError(f"{name} must have {n} entries")
    F = int(B.shape[1])
    if out is None:
        out = torch.empty((A.nrows, F), dtype=torch.float32, device=B.device)
    ws = workspace or SpmmWorkspace()
    buf = ws.get(spmm_workspace_bytes(A.nrows, A.nnz, F, B.dtype), B.device)
    _lib.call("gbs_csr_spmm_scaled", A.nrows, A.ncols, A.nnz, _ptr(A.rowptr), _ptr(A.colind), _ptr(rowscale),
              _ptr(colscale), _ptr(B), _DT[B.dtype], F, _ptr(out), _ptr(buf), buf.numel(), _stream(B.device))
    return out


class SpmmPlan:
    """Column-partitioned SpMM plan for a fixed A, feature width and type
    (parts = 0 lets the library choose from B's size against L2).  With
    rowscale / colscale the plan computes the degree-normalised product of
    csr_spmm_scaled (A's values unused)."""

    def __init__(self, A: CSR, F: int, dtype: torch.dtype = torch.float32, parts: int = 0,
                 rowscale: torch.Tensor | None = None, colscale: torch.Tensor | None = None):
        A.validate_layout()
        self.A, self.F, self.dtype = A, F, dtype
        h = C.c_void_p()
        if rowscale is not None or colscale is not None:
            _lib.call("gbs_csr_spmm_plan_create_scaled", A.nrows, A.ncols, A.nnz, _ptr(A.rowptr),
                      _ptr(A.colind), _ptr(rowscale), _ptr(colscale), _DT[dtype], F, parts,
                      _stream(A.rowptr.device), C.byref(h))
        else:
            _lib.call("gbs_csr_spmm_plan_create", A.nrows, A.ncols, A.nnz, _ptr(A.rowptr), _ptr(A.colind),
                      _ptr(A.vals), _DT[dtype], F, parts, _stream(A.rowptr.device), C.byref(h))
        self._h = h
        k = C.c_int(0)
        _lib.call("gbs_csr_spmm_plan_parts", h, C.byref(k))
        self.parts = int(k.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().gbs_csr_spmm_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    def run(self, B: torch.Tensor, out: torch.Tensor | None = None,
            workspace: SpmmWorkspace | None = None) -> torch.Tensor:
        _check_cuda("B", B, self.dtype)
        if tuple(B.shape) != (self.A.ncols, self.F):
            raise ValueError("B does not match the plan")
        if out is None:
            out = torch.empty((self.A.nrows, self.F), dtype=torch.float32, device=B.device)
        ws = workspace or SpmmWorkspace()
        buf = ws.get(spmm_workspace_bytes(self.A.nrows, self.A.nnz, self.F, self.dtype), B.device)
        _lib.call("gbs_csr_spmm_planned", self._h, _ptr(B), _ptr(out), _ptr(buf), buf.numel(), _stream(B.device))
        return out


class HostSpmmContext:
    """Device buffers, streams and events kept between csr_spmm_host calls."""

    def __init__(self):
        h = C.c_void_p()
        _lib.call("gbs_spmm_host_ctx_create", C.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().gbs_spmm_host_ctx_destroy(h)
            except Exception:
                pass
            self._h = None


def csr_spmm_host(rowptr: torch.Tensor, colind: torch.Tensor, vals: torch.Tensor | None, B: torch.Tensor,
                  nrows: int, ncols: int, out: torch.Tensor | None = None,
                  ctx: HostSpmmContext | None = None) -> torch.Tensor:
    """C = A @ B from host (CPU) tensors to a host tensor, copies overlapped
    with the kernels (pin the tensors for the overlap)."""
    for name, t in (("rowptr", rowptr), ("colind", colind), ("B", B)):
        if t.is_cuda or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous host tensor")
    if B.dtype not in _DT:
        raise TypeError("B must be float32, bfloat16 or float16")
    F = int(B.shape[1])
    if out is None:
        out = torch.empty((nrows, F), dtype=torch.float32, pin_memory=B.is_pinned())
    dev = torch.device("cuda", torch.cuda.current_device())
    _lib.call("gbs_csr_spmm_host", ctx._h if ctx is not None else None, nrows, ncols, int(colind.numel()),
              _ptr(rowptr), _ptr(colind), _ptr(vals), _ptr(B), _DT[B.dtype], F, _ptr(out), _stream(dev))
    return out


# ---------------------------------------------------------------------------
# B2SR
# ---------------------------------------------------------------------------
_TILE_DT = {4: torch.uint8, 8: torch.uint8, 16: torch.int16, 32: torch.int32}


@dataclass
class B2SR:
    """B2SR matrix on the device: tile rows as uint8 (tile 4, 8), 16-bit
    (tile 16) or 32-bit (tile 32) words held in torch tensors of that width."""

    rowptr: torch.Tensor
    colind: torch.Tensor
    val: torch.Tensor
    tile: int
    nrows: int
    ncols: int

    @property
    def nblockrows(self) -> int:
        return (self.nrows + self.tile - 1) // self.tile

    @property
    def nnzb(self) -> int:
        return int(self.colind.numel())


def csr2b2sr(A: CSR, tile: int) -> B2SR:
    """Pack a CSR matrix (values ignored) into B2SR with the given tile."""
    A.validate_layout()
    dev = A.rowptr.device
    mb = (A.nrows + tile - 1) // tile
    rowptr = torch.empty(mb + 1, dtype=torch.int32, device=dev)
    nnzb = C.c_int(0)
    s = _stream(dev)
    _lib.call("gbs_csr2b2sr_nnzb", A.nrows, A.ncols, A.nnz, _ptr(A.rowptr), _ptr(A.colind), tile,
              _ptr(rowptr), C.byref(nnzb), s)
    nb = int(nnzb.value)
    colind = torch.empty(max(nb, 1), dtype=torch.int32, device=dev)[:nb]
    val = torch.empty(max(nb * tile, 1), dtype=_TILE_DT[tile], device=dev)[:nb * tile]
    _lib.call("gbs_csr2b2sr", A.nrows, A.ncols, A.nnz, _ptr(A.rowptr), _ptr(A.colind), tile,
              _ptr(rowptr), _ptr(colind), _ptr(val), s)
    return B2SR(rowptr, colind, val, tile, A.nrows, A.ncols)


def b2sr_spmm(Ab: B2SR, B: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """C = A01 @ B (FP32 out).  Hub block-rows are split and summed with
    atomics (order-free: exact on 0/1 and +-1 features, FP32 rounding
    otherwise); ``spmm4_full_full`` keeps spmm4_full_full_new2's addition
    order for every row."""
    _check_cuda("B", B, tuple(_DT))
    F = int(B.shape[1])
    if out is None:
        out = torch.empty((Ab.nrows, F), dtype=torch.float32, device=B.device)
    _lib.call("gbs_b2sr_spmm", Ab.tile, Ab.nrows, Ab.nblockrows, _ptr(Ab.rowptr), _ptr(Ab.colind),
              _ptr(Ab.val), _ptr(B), _DT[B.dtype], F, _ptr(out), _stream(B.device))
    return out


def spmm4_full_full(A: torch.Tensor, B: torch.Tensor, C_: torch.Tensor, rowptr: torch.Tensor,
                    colind: torch.Tensor, nblockrows: int, B_cols: int) -> None:
    """Mirror of the reference launch spmm4_full_full_new2<<<...>>>(A, B, C,
    rowptr, colind, nblockrows, B_cols): C must be zero-filled; only nonzero
    results are stored."""
    _lib.call("gbs_spmm4_full_full", _ptr(A), _ptr(B), _ptr(C_), _ptr(rowptr), _ptr(colind),
              int(nblockrows), int(B_cols), _stream(B.device))


def csr2bsr_batch(h_rowptr, h_colind, nrows: int, ncols: int, nnz: int, bsrRowPtr: torch.Tensor,
                  bsrColInd: torch.Tensor, bsrVal: torch.Tensor, blocksize: int, nblockrows: int,
                  nblocks: int) -> None:
    """Mirror of csr2bsr_batch_{4,8,16,32}: host CSR (numpy int32 arrays),
    caller-allocated device outputs."""
    import numpy as np
    h_rowptr = np.ascontiguousarray(h_rowptr, dtype=np.int32)
    h_colind = np.ascontiguousarray(h_colind, dtype=np.int32)
    _lib.call("gbs_csr2bsr_batch", h_rowptr.ctypes.data, h_colind.ctypes.data if h_colind.size else None,
              nrows, ncols, nnz, _ptr(bsrRowPtr), _ptr(bsrColInd), _ptr(bsrVal), blocksize,
              nblockrows, nblocks)


def pack_sign_rows(X: torch.Tensor) -> torch.Tensor:
    """bit = (x >= 0) packed along columns, ceil(F/32) int32-held words/row."""
    _check_cuda("X", X, torch.float32)
    n, F = X.shape
    out = torch.empty((n, (F + 31) // 32), dtype=torch.int32, device=X.device)
    _lib.call("gbs_pack_sign_rows", _ptr(X), n, F, _ptr(out), _stream(X.device))
    return out


def pack_sign_colud(X: torch.Tensor) -> torch.Tensor:
    """ToBit32ColUd layout: [ceil(W/32)][32*ceil(H/32)] words."""
    _check_cuda("X", X, torch.float32)
    H, W = X.shape
    out = torch.empty(((W + 31) // 32, (H + 31) // 32 * 32), dtype=torch.int32, device=X.device)
    _lib.call("gbs_pack_sign_colud", _ptr(X), H, W, _ptr(out), _stream(X.device))
    return out


def b2sr_bmm(Ab: B2SR, Xbits: torch.Tensor, F: int, signed_form: bool = False) -> torch.Tensor:
    """int32 C[i][k] = sum_j A_ij bit_jk (or 2*C - deg(i) when signed)."""
    _check_cuda("Xbits", Xbits, torch.int32)
    out = torch.empty((Ab.nrows, F), dtype=torch.int32, device=Xbits.device)
    _lib.call("gbs_b2sr_bmm", Ab.tile, Ab.nrows, Ab.nblockrows, _ptr(Ab.rowptr), _ptr(Ab.colind),
              _ptr(Ab.val), _ptr(Xbits), F, int(signed_form), _ptr(out), _stream(Xbits.device))
    return out


def b2sr_bmm_aligned(Ab: B2SR, aligned, Xbits: torch.Tensor, F: int, signed_form: bool = False) -> torch.Tensor:
    """b2sr_bmm on the aligned arrays (rowptr, colind, words) that
    b2sr_aligned(Ab) returns (tile 8 or 16)."""
    _check_cuda("Xbits", Xbits, torch.int32)
    nrp, ncol, nval = aligned
    out = torch.empty((Ab.nrows, F), dtype=torch.int32, device=Xbits.device)
    _lib.call("gbs_b2sr_bmm_aligned", Ab.tile, Ab.nrows, Ab.nblockrows, _ptr(nrp), _ptr(ncol), _ptr(nval),
              _ptr(Xbits), F, int(signed_form), _ptr(out), _stream(Xbits.device))
    return out


def b2sr_aligned(Ab: B2SR):
    """Aligned B2SR-8/16: (rowptr, colind, uint32-held words)."""
    dev = Ab.rowptr.device
    mb = Ab.nblockrows
    nrp = torch.empty(mb + 1, dtype=torch.int32, device=dev)
    nt = C.c_int(0)
    s = _stream(dev)
    _lib.call("gbs_b2sr_aligned_nnzb", Ab.tile, mb, _ptr(Ab.rowptr), _ptr(nrp), C.byref(nt), s)
    g = 4 if Ab.tile == 8 else 2
    ntiles = int(nt.value)
    ncol = torch.empty(max(ntiles, 1), dtype=torch.int32, device=dev)[:ntiles]
    nval = torch.empty(max(ntiles * Ab.tile // g, 1), dtype=torch.int32, device=dev)[:ntiles * Ab.tile // g]
    _lib.call("gbs_b2sr_pack_aligned", Ab.tile, mb, _ptr(Ab.rowptr), _ptr(Ab.colind), _ptr(Ab.val),
              _ptr(nrp), _ptr(ncol), _ptr(nval), s)
    return nrp, ncol, nval


# ---------------------------------------------------------------------------
# Dense binary matmul (word-major operands, ToBit32ColUd layout)
# ---------------------------------------------------------------------------
BMM_XOR, BMM_AND, BMM_SIGNED = 0, 1, 2
BMM_ALGO_DEFAULT, BMM_ALGO_POPC, BMM_ALGO_MMA, BMM_ALGO_TC, BMM_ALGO_TC_PERSIST = 0, 1, 2, 3, 4


def bmm_tc_timeouts() -> int:
    n = C.c_int(0)
    _lib.call("gbs_bmm_tc_timeouts", C.byref(n))
    return int(n.value)


def bmm_b1(A: torch.Tensor, B: torch.Tensor, mode: int = BMM_XOR, algo: int = BMM_ALGO_DEFAULT,
           out: torch.Tensor | None = None) -> torch.Tensor:
    """A: (Kw, M), B: (Kw, N) int32-held words -> int32 (M, N) counts."""
    _check_cuda("A", A, torch.int32)
    _check_cuda("B", B, torch.int32)
    Kw, M = A.shape
    N = B.shape[1]
    if out is None:
        out = torch.empty((M, N), dtype=torch.int32, device=A.device)
    _lib.call("gbs_bmm_b1", _ptr(A), _ptr(B), M, N, Kw, mode, algo, _ptr(out), _stream(A.device))
    return out


def bmm32_arow_brow(A: torch.Tensor, B: torch.Tensor, C_: torch.Tensor, A_height: int, A_width: int,
                    B_width: int) -> None:
    """Mirror of BMM32_Arow_Brow<float>(A, B, C, A_height, A_width, B_width)."""
    _lib.call("gbs_bmm32_arow_brow", _ptr(A), _ptr(B), _ptr(C_), A_height, A_width, B_width,
              _stream(A.device))


def bmm32_bin(A: torch.Tensor, B: torch.Tensor, C_: torch.Tensor, m: int, n: int, k: int,
              s_layout: bool = False) -> None:
    """Mirror of BMM32_BIN (or BMM32S_BIN with s_layout=True)."""
    _lib.call("gbs_bmm32s_bin" if s_layout else "gbs_bmm32_bin", _ptr(A), _ptr(B), _ptr(C_), m, n, k,
              _stream(A.device))


BIN_FUSED, BIN_COUNTS = 0, 1


def bmm_bin(A: torch.Tensor, B: torch.Tensor, C_: torch.Tensor, m: int, n: int, k: int,
            s_layout: bool = False, algo: int = BIN_FUSED) -> None:
    """Sign words of the binary GEMM in the BMM32_BIN (or BMM32S_BIN) layout
    with the algorithm chosen: BIN_FUSED thresholds in the tcgen05 epilogue,
    BIN_COUNTS writes int32 counts first and packs them in a second pass."""
    _lib.call("gbs_bmm_bin", _ptr(A), _ptr(B), _ptr(C_), m, n, k, int(s_layout), algo, _stream(A.device))


# ---------------------------------------------------------------------------
# Backward: cached transpose, A^T dC, SDDMM
# ---------------------------------------------------------------------------
class CSRTranspose:
    """A^T of a CSR pattern (device arrays owned by the library handle)."""

    def __init__(self, A: CSR):
        A.validate_layout()
        self.nrows, self.ncols, self.nnz = A.nrows, A.ncols, A.nnz
        self.device = A.rowptr.device
        h = C.c_void_p()
        _lib.call("gbs_csr_transpose_create", A.nrows, A.ncols, A.nnz, _ptr(A.rowptr), _ptr(A.colind),
                  _stream(self.device), C.byref(h))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().gbs_csr_transpose_destroy(h)
            except Exception:
                pass
            self._h = None

    def arrays(self):
        """(t_rowptr, t_colind, perm) copied into new torch tensors."""
        rp = torch.empty(self.ncols + 1, dtype=torch.int32, device=self.device)
        ci = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=self.device)
        pm = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=self.device)
        _lib.call("gbs_csr_transpose_copy", self._h, _ptr(rp), _ptr(ci), _ptr(pm), _stream(self.device))
        return rp, ci[: self.nnz], pm[: self.nnz]

    def values(self, vals: torch.Tensor) -> torch.Tensor:
        _check_cuda("vals", vals, torch.float32)
        out = torch.empty_like(vals)
        _lib.call("gbs_csr_transpose_values", self._h, _ptr(vals), _ptr(out), _stream(self.device))
        return out

    def spmm(self, t_vals: torch.Tensor | None, dC: torch.Tensor, out: torch.Tensor | None = None,
             workspace: SpmmWorkspace | None = None) -> torch.Tensor:
        """dB = A^T dC (FP32 out)."""
        _check_cuda("dC", dC, tuple(_DT))
        F = int(dC.shape[1])
        if out is None:
            out = torch.empty((self.ncols, F), dtype=torch.float32, device=dC.device)
        ws = workspace or SpmmWorkspace()
        nbytes = spmm_workspace_bytes(self.ncols, self.nnz, F, dC.dtype)
        buf = ws.get(nbytes, dC.device)
        _lib.call("gbs_csr_spmm_transposed", self._h, _ptr(t_vals), _ptr(dC), _DT[dC.dtype], F, _ptr(out),
                  _ptr(buf), buf.numel(), _stream(dC.device))
        return out


def spmm_backward(T: "CSRTranspose", t_vals: torch.Tensor | None, dC: torch.Tensor, H: torch.Tensor,
                  dB: torch.Tensor | None = None, dvals: torch.Tensor | None = None,
                  workspace: SpmmWorkspace | None = None):
    """Fused backward of C = A H: (dB = A^T dC, dvals[e] = <dC[row e], H[col e]>)."""
    _check_cuda("dC", dC, tuple(_DT))
    _check_cuda("H", H, dC.dtype)
    F = int(dC.shape[1])
    if dB is None:
        dB = torch.empty((T.ncols, F), dtype=torch.float32, device=dC.device)
    if dvals is None:
        dvals = torch.empty(T.nnz, dtype=torch.float32, device=dC.device)
    ws = workspace or SpmmWorkspace()
    buf = ws.get(spmm_workspace_bytes(T.ncols, T.nnz, F, dC.dtype), dC.device)
    _lib.call("gbs_spmm_backward", T._h, _ptr(t_vals), _ptr(dC), _ptr(H), _DT[dC.dtype], F, _ptr(dB),
              _ptr(dvals), _ptr(buf), buf.numel(), _stream(dC.device))
    return dB, dvals


class BackwardPlan:
    """Planned fused backward (gbs_spmm_backward_plan_*): A^T split by row
    ranges of A so that each pass's dC gathers stay in L2 (parts = 0: the
    library chooses from dC's size against L2).  t_vals is copied at
    creation; with one part the plan keeps references to T and t_vals."""

    def __init__(self, T: "CSRTranspose", t_vals: torch.Tensor | None, F: int,
                 dtype: torch.dtype = torch.float32, parts: int = 0):
        if t_vals is not None:
            _check_cuda("t_vals", t_vals, torch.float32)
        self.T, self.t_vals, self.F, self.dtype = T, t_vals, F, dtype
        h = C.c_void_p()
        _lib.call("gbs_spmm_backward_plan_create", T._h, _ptr(t_vals), _DT[dtype], F, parts,
                  _stream(T.device), C.byref(h))
        self._h = h
        k = C.c_int(0)
        _lib.call("gbs_spmm_backward_plan_parts", h, C.byref(k))
        self.parts = int(k.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().gbs_spmm_backward_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    def run(self, dC: torch.Tensor, H: torch.Tensor, dB: torch.Tensor | None = None,
            dvals: torch.Tensor | None = None, workspace: SpmmWorkspace | None = None):
        _check_cuda("dC", dC, self.dtype)
        _check_cuda("H", H, self.dtype)
        T = self.T
        if tuple(dC.shape) != (T.nrows, self.F) or tuple(H.shape) != (T.ncols, self.F):
            raise ValueError("dC / H do not match the plan")
        if dB is None:
            dB = torch.empty((T.ncols, self.F), dtype=torch.float32, device=dC.device)
        if dvals is None:
            dvals = torch.empty(T.nnz, dtype=torch.float32, device=dC.device)
        ws = workspace or SpmmWorkspace()
        buf = ws.get(spmm_workspace_bytes(T.ncols, T.nnz, self.F, self.dtype), dC.device)
        _lib.call("gbs_spmm_backward_planned", self._h, _ptr(dC), _ptr(H), _ptr(dB), _ptr(dvals), _ptr(buf),
                  buf.numel(), _stream(dC.device))
        return dB, dvals


def sddmm(A: CSR, G: torch.Tensor, H: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """out[e] = <G[row(e)], H[col(e)]> on A's pattern (FP32)."""
    A.validate_layout()
    _check_cuda("G", G, tuple(_DT))
    _check_cuda("H", H, tuple(_DT))
    if G.dtype != H.dtype:
        raise TypeError("G and H must have the same dtype")
    F = int(G.shape[1])
    if out is None:
        out = torch.empty(A.nnz, dtype=torch.float32, device=G.device)
    _lib.call("gbs_sddmm", A.nrows, A.ncols, A.nnz, _ptr(A.rowptr), _ptr(A.colind), _ptr(G), _ptr(H),
              _DT[G.dtype], F, _ptr(out), _stream(G.device))
    return out


# ---------------------------------------------------------------------------
# Matrix Market ingest (host)
# ---------------------------------------------------------------------------
def pool_trim() -> None:
    """Return the unused memory of the library's temporaries pool on the
    current device (gbs_pool_trim)."""
    _lib.call("gbs_pool_trim")


def _host_csr_arrays(fn: str, path) -> tuple:
    import numpy as np
    h = _lib.HostCSR()
    _lib.call(fn, str(path).encode(), C.byref(h))
    try:
        n, nnz = h.nrows, h.nnz
        rowptr = np.ctypeslib.as_array(h.rowptr, shape=(n + 1,)).copy()
        colind = np.ctypeslib.as_array(h.colind, shape=(max(nnz, 1),))[:nnz].copy()
        vals = np.ctypeslib.as_array(h.vals, shape=(max(nnz, 1),))[:nnz].copy()
        return h.nrows, h.ncols, rowptr, colind, vals
    finally:
        _lib.load().gbs_host_csr_free(C.byref(h))


def read_mtx(path) -> tuple:
    """(nrows, ncols, rowptr, colind, vals) as numpy arrays, with the
    reference's readMtx + coo2csr semantics."""
    return _host_csr_arrays("gbs_mtx_read", path)


def read_csr_bin(path) -> tuple:
    """(nrows, ncols, rowptr, colind, vals) from a binary CSR cache file."""
    return _host_csr_arrays("gbs_csr_read_bin", path)


def write_csr_bin(path, nrows: int, ncols: int, rowptr, colind, vals=None) -> None:
    """Write a host CSR (numpy arrays; vals None = pattern) as a binary
    cache file (gbs_csr_write_bin)."""
    import numpy as np
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colind, dtype=np.int32)
    va = None if vals is None else np.ascontiguousarray(vals, dtype=np.float32)
    h = _lib.HostCSR()
    h.nrows, h.ncols, h.nnz = int(nrows), int(ncols), int(ci.size)
    h.rowptr = rp.ctypes.data_as(C.POINTER(C.c_int))
    h.colind = ci.ctypes.data_as(C.POINTER(C.c_int))
    h.vals = va.ctypes.data_as(C.POINTER(C.c_float)) if va is not None else C.POINTER(C.c_float)()
    _lib.call("gbs_csr_write_bin", str(path).encode(), C.byref(h))


_TILE_NP = {4: "uint8", 8: "uint8", 16: "uint16", 32: "uint32"}


def write_b2sr_bin(path, Ab) -> None:
    """Write a B2SR matrix as a binary cache file (gbs_b2sr_write_bin).  Ab is
    a device B2SR or a host tuple (nrows, ncols, tile, rowptr, colind, val)
    of numpy arrays."""
    import numpy as np
    if isinstance(Ab, B2SR):
        nrows, ncols, tile = Ab.nrows, Ab.ncols, Ab.tile
        rowptr, colind = Ab.rowptr.cpu().numpy(), Ab.colind.cpu().numpy()
        val = Ab.val.cpu().numpy().view(_TILE_NP[tile])
    else:
        nrows, ncols, tile, rowptr, colind, val = Ab
    if tile not in _TILE_NP:
        raise ValueError("tile must be 4, 8, 16 or 32")
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colind, dtype=np.int32)
    va = np.ascontiguousarray(val)
    if va.dtype.itemsize != np.dtype(_TILE_NP[tile]).itemsize:
        raise ValueError(f"tile {tile} rows are {np.dtype(_TILE_NP[tile]).itemsize}-byte words")
    va = va.view(_TILE_NP[tile])
    if va.size != ci.size * tile:
        raise ValueError("val must hold nnzb * tile rows")
    h = _lib.HostB2SR()
    h.nrows, h.ncols, h.tile = int(nrows), int(ncols), int(tile)
    h.nblockrows, h.nnzb = int(rp.size - 1), int(ci.size)
    h.rowptr = rp.ctypes.data_as(C.POINTER(C.c_int))
    h.colind = ci.ctypes.data_as(C.POINTER(C.c_int))
    h.val = va.ctypes.data_as(C.c_void_p)
    _lib.call("gbs_b2sr_write_bin", str(path).encode(), C.byref(h))


def read_b2sr_bin(path) -> tuple:
    """(nrows, ncols, tile, rowptr, colind, val) as numpy arrays from a
    binary B2SR cache file (checked on load)."""
    import numpy as np
    h = _lib.HostB2SR()
    _lib.call("gbs_b2sr_read_bin", str(path).encode(), C.byref(h))
    try:
        mb, nb, T = h.nblockrows, h.nnzb, h.tile
        rowptr = np.ctypeslib.as_array(h.rowptr, (mb + 1,)).copy()
        colind = np.ctypeslib.as_array(h.colind, (max(nb, 1),))[:nb].copy() if nb else np.zeros(0, np.int32)
        dt = np.dtype(_TILE_NP[T])
        raw = (C.c_char * (nb * T * dt.itemsize)).from_address(h.val) if nb else b""
        val = np.frombuffer(bytes(raw), dtype=dt).copy() if nb else np.zeros(0, dt)
        return h.nrows, h.ncols, T, rowptr, colind, val
    finally:
        _lib.load().gbs_host_b2sr_free(C.byref(h))


def load_b2sr(path, device) -> B2SR:
    """A B2SR cache file as a device B2SR, ready for b2sr_spmm / b2sr_bmm."""
    nrows, ncols, tile, rowptr, colind, val = read_b2sr_bin(path)
    t = torch.from_numpy(val.view({1: "uint8", 2: "int16", 4: "int32"}[val.dtype.itemsize]))
    return B2SR(torch.from_numpy(rowptr).to(device), torch.from_numpy(colind).to(device), t.to(device),
                tile, nrows, ncols)
