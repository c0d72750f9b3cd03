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
