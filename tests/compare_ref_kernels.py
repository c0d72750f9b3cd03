"""Same-box timing of the library against the kernels it replaces: the
reference's own CUDA kernels (from the fatbin compiled out of the reference
sources, oracle/_ref/ref_kernels.fatbin) and cuSPARSE SpMM as the reference
calls it (CSR, ALG_DEFAULT, FP32, column-major B / C,
test_spmm_full.cu:279-307; also with row-major B / C).

Run on a GPU machine after the library is built:

    python tests/compare_ref_kernels.py > comparators.json

Every time is the median of CUDA-event-timed launches on the default stream
with L2 flushed (a 512 MiB write) before each one.  Prints one JSON object.
Workloads: the 89,250-node flickr-shaped graph (values 1.0) at F = 32..256;
the 232,965-node reddit-shaped graph at F = 256 (values D^-1/2 A D^-1/2 for
the CSR products, its 0/1 pattern for the B2SR ones); 8192^3-bit binary
GEMM.  Results are checked for agreement before they are timed.
"""
from __future__ import annotations

import ctypes as C
import json
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

import torch  # noqa: E402

from oracle import refkern  # noqa: E402
from spmm_eval_gb300 import graphs as G  # noqa: E402
from spmm_eval_gb300 import ops  # noqa: E402


def cusparse_lib():
    so = HERE / "native" / "libcusparse_ref.so"
    src = HERE / "native" / "cusparse_ref.cu"
    if not so.exists() or so.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared", "-Xcompiler",
                        "-fPIC", "-Wno-deprecated-declarations", "-o", str(so), str(src), "-lcusparse"], check=True)
    lib = C.CDLL(str(so))
    lib.ref_spmm_handle_create.restype = C.c_void_p
    lib.ref_spmm_handle_create.argtypes = ([C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 4
                                           + [C.c_int, C.c_void_p, C.c_int])
    lib.ref_spmm_handle_run.argtypes = [C.c_void_p]
    lib.ref_spmm_handle_destroy.argtypes = [C.c_void_p]
    return lib


def timer(reps=7):
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def t(fn):
        fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            fn()
            e.record(stream)
            torch.cuda.synchronize()
            ms.append(s.elapsed_time(e))
        return round(sorted(ms)[len(ms) // 2], 4)
    return t


def ref_fbf(rk, Ab, B, F, Cd):
    tiles_per_tb = 1024 // F
    mb = Ab.nblockrows
    rk.launch("spmm4_full_full_new2", ((mb + tiles_per_tb - 1) // tiles_per_tb,), (1024,),
              Ab.val, B, Cd, Ab.rowptr, Ab.colind, mb, F)


def spmm_block(name, g, Fs, cs, rk, t, out):
    dev = torch.device("cuda")
    n = g.nrows
    A = ops.CSR(g.rowptr, g.colind, g.vals, n, n)
    Ab = ops.csr2b2sr(ops.CSR(g.rowptr, g.colind, None, n, n), 4)
    ws = ops.SpmmWorkspace()
    res = {}
    for F in Fs:
        B = G.normal(F, 3, (n, F), device=dev)
        Bcol = B.t().contiguous()
        C_ours = torch.empty((n, F), device=dev)
        r = {}
        plan = ops.SpmmPlan(A, F, torch.float32)
        r["ours_planned_csr"] = t(lambda: plan.run(B, out=C_ours, workspace=ws))
        r["ours_planned_parts"] = plan.parts
        r["ours_csr"] = t(lambda: ops.csr_spmm(A, B, out=C_ours, workspace=ws))
        scale = ops.csr_spmm(ops.CSR(g.rowptr, g.colind, g.vals.abs(), n, n), B.abs()).clamp_min(1e-30)
        for order, key in ((0, "cusparse_csr_colmajor"), (1, "cusparse_csr_rowmajor")):
            Bx = Bcol if order == 0 else B
            Cx = torch.empty((F, n) if order == 0 else (n, F), device=dev)
            h = cs.ref_spmm_handle_create(n, n, g.nnz, g.rowptr.data_ptr(), g.colind.data_ptr(), g.vals.data_ptr(),
                                          Bx.data_ptr(), F, Cx.data_ptr(), order)
            if not h:
                r[key] = None
                continue
            assert cs.ref_spmm_handle_run(h) == 0
            torch.cuda.synchronize()
            got = Cx.t() if order == 0 else Cx
            r[key + "_agree"] = float(((got - C_ours).abs() / scale).max())
            r[key] = t(lambda: cs.ref_spmm_handle_run(h))
            cs.ref_spmm_handle_destroy(h)
            del Cx
        Cr = torch.zeros((Ab.nblockrows * 4, F), device=dev)
        Cm = torch.zeros_like(Cr)
        if rk is not None:
            ref_fbf(rk, Ab, B, F, Cr)
            ops.spmm4_full_full(Ab.val, B, Cm, Ab.rowptr, Ab.colind, Ab.nblockrows, F)
            torch.cuda.synchronize()
            r["fbf_bitwise_equal"] = bool(torch.equal(Cr.view(torch.int32), Cm.view(torch.int32)))
            r["reference_fbf_b2sr4"] = t(lambda: ref_fbf(rk, Ab, B, F, Cr))
        r["ours_fbf_dropin_b2sr4"] = t(lambda: ops.spmm4_full_full(Ab.val, B, Cm, Ab.rowptr, Ab.colind,
                                                                   Ab.nblockrows, F))
        r["ours_b2sr4_spmm"] = t(lambda: ops.b2sr_spmm(Ab, B, out=C_ours))
        res[str(F)] = r
        del B, Bcol, C_ours, Cr, Cm, plan, scale
        torch.cuda.empty_cache()
    out[name] = {"nodes": n, "nnz": g.nnz, "nnzb_tile4": Ab.nnzb, "ms": res}


def main() -> int:
    torch.cuda.init()
    rk = refkern.kernels() if refkern.available() else None
    cs = cusparse_lib()
    t = timer()
    out = {"device": torch.cuda.get_device_name(0), "reference_kernels": rk is not None,
           "timing": "median of 7 CUDA-event-timed launches, L2 flushed before each"}
    g = G.flickr_like(device="cuda")
    spmm_block("flickr_like", g, (32, 64, 128, 256), cs, rk, t, out)
    del g
    g = G.gcn_normalize(G.reddit_like(device="cuda"))
    spmm_block("reddit_like", g, (256,), cs, rk, t, out)
    del g
    torch.cuda.empty_cache()
    # binary GEMM 8192^3 bits
    M = N = 8192
    Kw = 256
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1)
    A = torch.randint(-2 ** 31, 2 ** 31 - 1, (Kw, M), dtype=torch.int32, device="cuda", generator=gen)
    B = torch.randint(-2 ** 31, 2 ** 31 - 1, (Kw, N), dtype=torch.int32, device="cuda", generator=gen)
    Cf = torch.empty((M, N), device="cuda")
    Cr = torch.empty((M, N), device="cuda")
    words = torch.empty((N // 32) * M, dtype=torch.int32, device="cuda")
    wref = torch.empty_like(words)
    r = {"ours_bmm32_arow_brow": t(lambda: ops.bmm32_arow_brow(A, B, Cf, M, Kw, N)),
         "ours_bmm32_bin": t(lambda: ops.bmm32_bin(A, B, words, M, 32 * Kw, N))}
    if rk is not None:
        rk.launch("BMM32_Arow_Brow", (M // 32, N // 32), (32,), A, B, Cr, M, Kw, N)
        rk.launch("BMM32_BIN", (M // 32, N // 32), (32,), A, B, wref, M, 32 * Kw, N)
        torch.cuda.synchronize()
        r["bitwise_equal"] = bool(torch.equal(Cf, Cr)) and bool(torch.equal(words, wref))
        r["reference_bmm32_arow_brow"] = t(lambda: rk.launch("BMM32_Arow_Brow", (M // 32, N // 32), (32,), A, B,
                                                             Cr, M, Kw, N))
        r["reference_bmm32_bin"] = t(lambda: rk.launch("BMM32_BIN", (M // 32, N // 32), (32,), A, B, wref, M,
                                                       32 * Kw, N))
    out["binary_gemm_8192"] = r
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
