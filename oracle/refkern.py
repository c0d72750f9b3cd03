"""The reference's own CUDA kernels as GPU checkers -- TEST INFRASTRUCTURE ONLY.

``oracle/_ref/ref_kernels.fatbin`` is built from the reference's sources
where they lie (``make -C oracle REF=<checkout> refkern``; see
``oracle/ref_kernels.cu`` for the list of kernels and the file:line each
comes from).  This module loads it into the current CUDA context with the
driver API (``libcuda`` through ctypes) and launches its kernels with the
reference's own grid shapes on torch's current stream, so a test can run the
reference kernel and the library's kernel on the same device buffers and
compare the results bit for bit.  Nothing in ``spmm_eval_gb300`` imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
FATBIN = HERE / "_ref" / "ref_kernels.fatbin"

# kernel -> Itanium-mangled name prefix: "_Z" + len + identifier, plus the
# template argument list for the instantiated templates
_NAMES = {
    "spmm4_full_full_new2": None,
    "BMM32_Arow_Brow": "IfE",
    "BMM32_MT_M_S": None,
    "BMM32_BIN": None,
    "BMM32S_BIN": None,
    "ToBit4Col": "IfE",
    "ToBit8Col": "IfE",
    "ToBit16Col": "IfE",
    "ToBit32Col": "IfE",
    "ToBit32ColUd": "IfE",
    "ToBit32RowDenseSign": "IfE",
    "packUchar2AlignedUnsigned": None,
    "packUshort2AlignedUnsigned": None,
}


def available() -> bool:
    return FATBIN.exists()


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed with CUresult {rc}")


class RefKernels:
    """Handle to the loaded fatbin; ``launch(name, grid, block, *args)``."""

    def __init__(self):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # the primary context is current on this thread
        self._cu = C.CDLL("libcuda.so.1")
        cu = self._cu
        cu.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_void_p]
        cu.cuModuleGetFunctionCount.argtypes = [C.POINTER(C.c_uint), C.c_void_p]
        cu.cuModuleEnumerateFunctions.argtypes = [C.POINTER(C.c_void_p), C.c_uint, C.c_void_p]
        cu.cuFuncGetName.argtypes = [C.POINTER(C.c_char_p), C.c_void_p]
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]
        self._image = C.create_string_buffer(FATBIN.read_bytes())
        self._mod = C.c_void_p()
        _check(cu.cuModuleLoadData(C.byref(self._mod), self._image), "cuModuleLoadData(ref_kernels.fatbin)")
        n = C.c_uint(0)
        _check(cu.cuModuleGetFunctionCount(C.byref(n), self._mod), "cuModuleGetFunctionCount")
        fns = (C.c_void_p * n.value)()
        _check(cu.cuModuleEnumerateFunctions(fns, n, self._mod), "cuModuleEnumerateFunctions")
        by_name = {}
        for f in fns:
            nm = C.c_char_p()
            _check(cu.cuFuncGetName(C.byref(nm), f), "cuFuncGetName")
            by_name[nm.value.decode()] = f
        self._fn = {}
        for short, targs in _NAMES.items():
            pre = f"_Z{len(short)}{short}" + (targs or "")
            hits = [f for m, f in by_name.items() if m.startswith(pre)
                    and (targs is not None or not m[len(pre):].startswith("I"))]
            if len(hits) != 1:
                raise RuntimeError(f"reference kernel {short}: {len(hits)} matches in the fatbin")
            self._fn[short] = hits[0]

    def launch(self, name: str, grid, block, *args) -> None:
        """args: torch tensors (passed as device pointers) or Python ints
        (passed as int32), in the kernel's parameter order."""
        import torch
        vals = []
        for a in args:
            if isinstance(a, torch.Tensor):
                vals.append(C.c_uint64(a.data_ptr()))
            elif isinstance(a, int):
                vals.append(C.c_int32(a))
            else:
                raise TypeError(f"unsupported kernel argument {type(a)}")
        ptrs = (C.c_void_p * len(vals))(*[C.addressof(v) for v in vals])
        g = tuple(grid) + (1,) * (3 - len(tuple(grid)))
        b = tuple(block) + (1,) * (3 - len(tuple(block)))
        stream = torch.cuda.current_stream().cuda_stream
        _check(self._cu.cuLaunchKernel(self._fn[name], g[0], g[1], g[2], b[0], b[1], b[2], 0, stream, ptrs, None),
               f"cuLaunchKernel({name})")


_inst: RefKernels | None = None


def kernels() -> RefKernels:
    global _inst
    if _inst is None:
        _inst = RefKernels()
    return _inst
