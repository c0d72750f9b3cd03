"""Benchmark of the SpMM hot path on GB300.

Workload (one "step"): C = A @ B with the merge-path CSR SpMM (column-
partitioned plan built once outside the timed region: one accumulating
launch per column range of A whose slice of B fits in L2), A the
reddit-shaped power-law graph (232,965 nodes, ~114.6M directed edges,
Chung-Lu, exponent 1.8, degrees capped at 20,000, values D^-1/2 A D^-1/2 in
FP32), B 232,965 x 256 FP32 N(0,1).  Inputs are synthetic and seeded (the
reference's reddit.mtx is not distributed).

metric: SpMM achieved GB/s by the gather model -- every nonzero reads one
whole feature row: bytes = 4(n+1) + 8 nnz + nnz*F*sizeof(B) + n*F*4 -- per
step, divided by the step's CUDA-event time.  L2 is flushed (a 512 MiB
write) before every timed step.  Most of those row gathers are served by L2,
so the line carries two rooflines: `roofline` (HBM: the step's measured DRAM
bytes from an ncu capture over its time, against the measured copy peak) and
`l2_gather` (the row-gather bytes over time against the L2 -> SM gather
ceiling measured by bin/gather_ceiling in the same run).  Extra keys: BF16 and
FP16 features (time, error), errors vs FP64 on sampled rows, forward +
backward, the end-to-end number through the public API with host buffers,
the other evaluation configurations (`configs`), the CPU baseline, clocks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SpMM achieved HBM GB/s (% of peak), fwd+bwd time BF16 vs FP32 at stated error"
WORKLOAD = "reddit_like_csr_spmm_f256"


def gather_bytes(n, nnz, F, bsz):
    return 4 * (n + 1) + 8 * nnz + nnz * F * bsz + n * F * 4


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes of one bench step (the planned SpMM's accumulating
    launches together) from the committed ncu summary (None until one
    exists)."""
    p = ROOT / "profiles" / "csr_spmm_plan_reddit_f256.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("dram_bytes_per_step")
        except Exception:
            return None
    return None


def gather_ceiling():
    """L2 -> SM gather ceiling (TB/s) of this GPU for random 1 KB FP32 and
    512 B BF16 feature rows of an L2-resident 32 MB table, measured now by
    bin/gather_ceiling (the SpMM's own access pattern and nothing else; the
    best of its variants per row type).  None if the probe cannot run."""
    exe = ROOT / "spmm_eval_gb300" / "bin" / "gather_ceiling"
    try:
        if not exe.exists():
            from spmm_eval_gb300 import build as b
            b.build_apps()
        r = subprocess.run([str(exe), "--json"], capture_output=True, text=True, timeout=300)
        d = json.loads(r.stdout)
        best = {}
        for x in d["results"]:
            if x["table_rows"] == 32768:
                k = "f32" if x["kernel"].startswith("fp32") else "bf16"
                best[k] = max(best.get(k, 0.0), x["tbs"])
        return best or None
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi sampled every 100 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def make_inputs(device):
    import torch
    from spmm_eval_gb300 import graphs as G
    g = G.gcn_normalize(G.reddit_like(device=device))
    B = G.normal(0x5EED + 4, 9, (g.ncols, 256), device=device)
    return g, B


def make_grad(shape, device):
    from spmm_eval_gb300 import graphs as G
    return G.normal(0x5EED + 5, 11, tuple(shape), device=device)


def sample_rows_for_error(g, k=192):
    import torch
    deg = (g.rowptr[1:] - g.rowptr[:-1]).to("cpu")
    top = torch.topk(deg, 32).indices
    spread = torch.linspace(0, g.nrows - 1, k - 32).long()
    return torch.unique(torch.cat([top, spread]))


def fp64_rows(g_cpu, B_cpu, rows):
    """FP64 products and |A||B| magnitudes of the sampled rows (torch CPU)."""
    import torch
    out, mag = [], []
    Bd = B_cpu.double()
    for r in rows.tolist():
        s, e = int(g_cpu.rowptr[r]), int(g_cpu.rowptr[r + 1])
        cols = g_cpu.colind[s:e].long()
        v = g_cpu.vals[s:e].double()
        out.append(v @ Bd[cols])
        mag.append(v.abs() @ Bd[cols].abs())
    return torch.stack(out), torch.stack(mag)


def rel_err(got, ref, mag):
    """max and mean of |C - C64| / (|A| |B|) elementwise (the scale of the
    rounding bound of a sum of products; |C64| itself can cancel to ~0)."""
    d = (got.double() - ref).abs()
    r = d / mag.clamp_min(1e-300)
    return float(r.max()), float(r.mean())


def plain_rel_err(got, ref):
    """max of the plain relative error |C - C64| / |C64| over the entries
    with |C64| >= the RMS of C64 over the sampled rows (the stated floor:
    below it the relative error of a cancelling sum is unbounded), and the
    fraction of entries that pass the floor."""
    ref = ref.double()
    floor = float(ref.pow(2).mean().sqrt())
    keep = ref.abs() >= floor
    r = (got.double() - ref).abs()[keep] / ref.abs()[keep]
    return {"max": float(r.max()) if r.numel() else 0.0, "floor": floor,
            "entries": int(keep.sum()), "of": int(ref.numel())}


def cpu_baseline(g_cpu, B_cpu, budget_s=10.0):
    """OpenMP FP32 CSR SpMM of the oracle on a bounded row sample."""
    import numpy as np
    import oracle
    rp = g_cpu.rowptr.numpy()
    target = 4_000_000
    r1 = int(np.searchsorted(rp, target))
    r1 = max(1, min(r1, g_cpu.nrows))
    nnz = int(rp[r1])
    ci, va, Bn = g_cpu.colind.numpy(), g_cpu.vals.numpy(), B_cpu.numpy()
    threads = oracle.max_threads()
    Cn = np.empty((r1, B_cpu.shape[1]), np.float32)
    oracle.csr_spmm_f32(rp, ci, va, Bn, 0, r1, out=Cn)  # warm-up
    times = []
    t_end = time.perf_counter() + budget_s
    while True:
        t0 = time.perf_counter()
        oracle.csr_spmm_f32(rp, ci, va, Bn, 0, r1, out=Cn)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() > t_end or len(times) >= 50:
            break
    t = statistics.median(times)
    gb = gather_bytes(r1, nnz, B_cpu.shape[1], 4) / 1e9
    return {"value": round(gb / t, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"rows [0,{r1}) = {nnz} nonzeros of the same graph, F=256 FP32, "
                      f"median of {len(times)} passes ({t*1e3:.1f} ms/pass)"}, t


def dist_setup(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, device):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """The reference has no CPU path of its own; its semantics (FP32 CSR
    SpMM, per-row in-order accumulation) are timed as the oracle's OpenMP
    port on the host cores, over the whole bench graph every step (rank 0
    only)."""
    world, rank, local = dist_setup(args)
    if rank != 0:
        return
    import torch
    import oracle
    oracle.build()
    dev = torch.device(f"cuda:{local}") if torch.cuda.is_available() else torch.device("cpu")
    g, B = make_inputs(dev)
    g_cpu, B_cpu = g.to("cpu"), B.to("cpu")
    del g, B
    n, nnz, F = g_cpu.nrows, g_cpu.nnz, 256
    rp, ci, va, Bn = g_cpu.rowptr.numpy(), g_cpu.colind.numpy(), g_cpu.vals.numpy(), B_cpu.numpy()
    import numpy as np
    Cn = np.empty((n, F), np.float32)
    for _ in range(args.warmup):
        oracle.csr_spmm_f32(rp, ci, va, Bn, out=Cn)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.csr_spmm_f32(rp, ci, va, Bn, out=Cn)
        times.append(time.perf_counter() - t0)
    t = sum(times) / len(times)
    value = gather_bytes(n, nnz, F, 4) / 1e9 / t
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "nodes": n, "nnz": nnz, "F": F},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": oracle.max_threads(),
                         "kind": "port",
                         "sample": f"the whole graph ({nnz} nonzeros) per step, F=256 FP32"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def event_timer(dev, stream, flush):
    """timed(fn, steps, tag) -> per-step CUDA-event times (ms) on `stream`,
    with L2 flushed (a 512 MiB write) before every step."""
    import torch

    def timed(fn, steps, tag):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        torch.cuda.nvtx.range_push(tag)
        for s, e in evs:
            flush.zero_()
            s.record(stream)
            fn()
            e.record(stream)
        torch.cuda.synchronize(dev)
        torch.cuda.nvtx.range_pop()
        return [s.elapsed_time(e) for s, e in evs]
    return timed


def mean_ms(timed, fn, steps, tag, warm=2):
    for _ in range(warm):
        fn()
    t = timed(fn, steps, tag)
    return sum(t) / len(t)


def other_configs(dev, timed, reps):
    """The other evaluation configurations, event-timed (L2 flushed before
    each rep): the 4096-row uniform matrix (F = 32); the 89,250-node
    flickr-shaped graph (CSR SpMM at F = 32..256, CSR -> B2SR packing and
    B2SR x FP32 SpMM at tiles 4/8/16/32, B2SR x bits BMM at F = 32..1024); the
    8192^3-bit binary GEMM beside cuBLASLt's dense FP8 GEMM of the same shape
    (its tensor-pipe ceiling); one GCN layer Y = A (X W) forward + backward on
    the normalised flickr-shaped graph (X 89,250 x 512, W 512 x 128)."""
    import torch
    from spmm_eval_gb300 import graphs as G
    from spmm_eval_gb300 import ops
    out = {}
    ws = ops.SpmmWorkspace()

    # uniform 4096 x 4096, 16 columns per row, values U[-1, 1], F = 32
    g = G.uniform_rows(4096, 16, device=dev)
    A = ops.CSR(g.rowptr, g.colind, g.vals, g.nrows, g.ncols)
    B = G.normal(0x5EED + 1, 3, (4096, 32), device=dev)
    C = torch.empty((4096, 32), device=dev)
    ms = mean_ms(timed, lambda: ops.csr_spmm(A, B, out=C, workspace=ws), reps, "uniform4096")
    out["uniform4096_f32_f32"] = {"ms": round(ms, 4),
                                  "gbs_gather_model": round(gather_bytes(4096, g.nnz, 32, 4) / (ms * 1e-3) / 1e9, 1)}

    # flickr-shaped graph
    g = G.flickr_like(device=dev)
    n, nnz = g.nrows, g.nnz
    A = ops.CSR(g.rowptr, g.colind, g.vals, n, n)
    Ap = ops.CSR(g.rowptr, g.colind, None, n, n)
    fl = {"nodes": n, "nnz": nnz, "csr_spmm_f32": {}, "pack_ms": {}, "b2sr_spmm_f256_ms": {},
          "fbf_tile4_ms": {}, "bmm_ms": {}}
    Ab4 = ops.csr2b2sr(Ap, 4)
    for F in (32, 64, 128, 256):
        B = G.normal(F, 3, (n, F), device=dev)
        C = torch.empty((n, F), device=dev)
        ms = mean_ms(timed, lambda: ops.csr_spmm(A, B, out=C, workspace=ws), reps, f"flickr_csr_{F}")
        fl["csr_spmm_f32"][str(F)] = {"ms": round(ms, 4),
                                      "gbs_gather_model": round(gather_bytes(n, nnz, F, 4) / (ms * 1e-3) / 1e9, 1)}
        fl["fbf_tile4_ms"][str(F)] = round(mean_ms(timed, lambda: ops.b2sr_spmm(Ab4, B, out=C), reps,
                                                   f"flickr_fbf_{F}"), 4)
    B = G.normal(256, 3, (n, 256), device=dev)
    C = torch.empty((n, 256), device=dev)
    for ts in (4, 8, 16, 32):
        holder = {}

        def pack():
            holder["Ab"] = ops.csr2b2sr(Ap, ts)
        fl["pack_ms"][str(ts)] = round(mean_ms(timed, pack, reps, f"flickr_pack_{ts}"), 4)
        Ab = holder["Ab"]
        fl["b2sr_spmm_f256_ms"][str(ts)] = round(mean_ms(timed, lambda: ops.b2sr_spmm(Ab, B, out=C), reps,
                                                         f"flickr_b2sr_{ts}"), 4)
        fl.setdefault("nnzb", {})[str(ts)] = Ab.nnzb
        bm, bal = {}, {}
        al = ops.b2sr_aligned(Ab) if ts in (8, 16) else None
        for F in (32, 64, 128, 256, 512, 1024):
            X = G.normal(F + 1, 8, (n, F), device=dev)
            Xw = ops.pack_sign_rows(X)
            bm[str(F)] = round(mean_ms(timed, lambda: ops.b2sr_bmm(Ab, Xw, F), reps, f"flickr_bmm_{ts}_{F}"), 4)
            if al is not None:
                bal[str(F)] = round(mean_ms(timed, lambda: ops.b2sr_bmm_aligned(Ab, al, Xw, F), reps,
                                            f"flickr_bmm_aligned_{ts}_{F}"), 4)
        fl["bmm_ms"][str(ts)] = bm
        if bal:
            fl.setdefault("bmm_aligned_ms", {})[str(ts)] = bal
    out["flickr_like"] = fl

    # binary GEMM 8192 x 8192 x 8192 bits (default: persistent tcgen05)
    gen = torch.Generator(device=dev)
    gen.manual_seed(8192)
    Aw = torch.randint(-2 ** 31, 2 ** 31 - 1, (256, 8192), dtype=torch.int32, device=dev, generator=gen)
    Bw = torch.randint(-2 ** 31, 2 ** 31 - 1, (256, 8192), dtype=torch.int32, device=dev, generator=gen)
    Co = torch.empty((8192, 8192), dtype=torch.int32, device=dev)
    ms = mean_ms(timed, lambda: ops.bmm_b1(Aw, Bw, ops.BMM_XOR, out=Co), reps, "bmm8192")
    ms_popc = mean_ms(timed, lambda: ops.bmm_b1(Aw, Bw, ops.BMM_XOR, ops.BMM_ALGO_POPC, out=Co), reps,
                      "bmm8192_popc")
    del Co
    words = torch.empty(256 * 8192, dtype=torch.int32, device=dev)
    ms_bin = mean_ms(timed, lambda: ops.bmm_bin(Aw, Bw, words, 8192, 8192, 8192, False, ops.BIN_FUSED), reps,
                     "bin8192_fused")
    ms_bin2 = mean_ms(timed, lambda: ops.bmm_bin(Aw, Bw, words, 8192, 8192, 8192, False, ops.BIN_COUNTS), reps,
                      "bin8192_counts")
    out["bmm_8192"] = {"ms": round(ms, 4), "pbitops": round(2 * 8192 ** 3 / (ms * 1e-3) / 1e15, 3),
                       "popc_ms": round(ms_popc, 4),
                       "bin_words_fused_ms": round(ms_bin, 4), "bin_words_two_pass_ms": round(ms_bin2, 4),
                       "timeouts": ops.bmm_tc_timeouts()}
    del Aw, Bw, words
    # The tensor-pipe rate the bit GEMM (bits expanded to e4m3) can reach on this GPU: cuBLASLt's
    # dense FP8 GEMM of the same shape (torch._scaled_mm, e4m3 x e4m3 -> bf16), measured here.
    try:
        fa = torch.randn(8192, 8192, device=dev).to(torch.float8_e4m3fn)
        fb = torch.randn(8192, 8192, device=dev).to(torch.float8_e4m3fn).t()
        one = torch.tensor(1.0, device=dev)
        ms_fp8 = mean_ms(timed, lambda: torch._scaled_mm(fa, fb, scale_a=one, scale_b=one,
                                                         out_dtype=torch.bfloat16), reps, "fp8_gemm8192")
        out["bmm_8192"]["fp8_gemm_cublaslt"] = {
            "ms": round(ms_fp8, 4), "pflops": round(2 * 8192 ** 3 / (ms_fp8 * 1e-3) / 1e15, 3),
            "bit_gemm_frac": round(ms_fp8 / ms, 3)}
        del fa, fb
    except (RuntimeError, AttributeError, TypeError) as ex:
        out["bmm_8192"]["fp8_gemm_cublaslt"] = {"unavailable": repr(ex)[:160]}

    # GCN layer on the normalised flickr-shaped graph
    gn = G.gcn_normalize(g)
    An = ops.CSR(gn.rowptr, gn.colind, gn.vals, n, n)
    T = ops.CSRTranspose(ops.CSR(gn.rowptr, gn.colind, None, n, n))
    tv = T.values(gn.vals)
    X = G.normal(51, 1, (n, 512), device=dev)
    lim = (6.0 / (512 + 128)) ** 0.5
    W = ((2 * G.uniform01(52, 0, torch.arange(512 * 128, device=dev)).reshape(512, 128) - 1) * lim).float()
    Gr = G.normal(53, 2, (n, 128), device=dev)
    gcn = {}
    for dt in (torch.float32, torch.bfloat16):
        pf = ops.SpmmPlan(An, 128, dt)
        pb = ops.BackwardPlan(T, tv, 128, dt)
        Y = torch.empty((n, 128), device=dev)
        dH = torch.empty((n, 128), device=dev)
        dv = torch.empty_like(gn.vals)
        Gx = Gr.to(dt)

        def layer():
            H = (X @ W).to(dt)            # dense X W (cuBLAS, in the harness)
            pf.run(H, out=Y, workspace=ws)  # Y = A H
            pb.run(Gx, H, dB=dH, dvals=dv, workspace=ws)  # dH = A^T G, dvals = SDDMM(G, H)
            return H

        def sparse_only(H):
            pf.run(H, out=Y, workspace=ws)
            pb.run(Gx, H, dB=dH, dvals=dv, workspace=ws)
        H = layer()
        gcn[str(dt)[6:]] = {"layer_ms": round(mean_ms(timed, layer, reps, "gcn_layer"), 4),
                            "sparse_ms": round(mean_ms(timed, lambda: sparse_only(H), reps, "gcn_sparse"), 4)}
    gcn["what"] = ("forward Y = A (X W) + backward dH = A^T G and dvals = SDDMM(G, X W); X W by torch "
                   "matmul (FP32); sparse_ms = the library's planned SpMM + planned fused backward only")
    out["gcn_layer_flickr"] = gcn
    return out


def run_ours(args):
    import torch
    from spmm_eval_gb300 import ops
    world, rank, local = dist_setup(args)
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)

    # the L2 -> SM gather ceiling of this GPU, measured before anything else
    ceil = gather_ceiling()

    g, B = make_inputs(dev)
    n, nnz, F = g.nrows, g.nnz, 256
    A = ops.CSR(g.rowptr, g.colind, g.vals, n, n)
    Bh = B.to(torch.bfloat16)
    Bf = B.to(torch.float16)
    C = torch.empty((n, F), dtype=torch.float32, device=dev)
    Ch = torch.empty_like(C)
    Cf = torch.empty_like(C)
    ws = ops.SpmmWorkspace()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    timed = event_timer(dev, stream, flush)

    # column-partitioned plans (built once, like cuSPARSE's SpMM preprocessing;
    # the library picks the number of column ranges from B's size against L2)
    plan32 = ops.SpmmPlan(A, F, torch.float32)
    plan16 = ops.SpmmPlan(A, F, torch.bfloat16)
    planh = ops.SpmmPlan(A, F, torch.float16)

    def step_f32():
        plan32.run(B, out=C, workspace=ws)

    def step_bf16():
        plan16.run(Bh, out=Ch, workspace=ws)

    def step_f16():
        planh.run(Bf, out=Cf, workspace=ws)

    for _ in range(max(3, args.warmup)):
        step_f32()
        step_bf16()
        step_f16()
    torch.cuda.synchronize(dev)

    barrier(world)
    torch.cuda.synchronize(dev)
    with ClockSampler(dev.index if dev.index is not None else 0) as clk:
        t0 = time.perf_counter()
        ms = timed(step_f32, args.steps, "timed_f32")
        barrier(world)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    ms_f32 = sum(ms) / len(ms)
    ms_f32 = max_over_ranks(ms_f32, world, dev)
    ms_bf16 = sum(timed(step_bf16, args.steps, "timed_bf16")) / args.steps
    ms_f16 = sum(timed(step_f16, args.steps, "timed_f16")) / args.steps

    # the same product with the normalisation in the kernel: binary A plus
    # the D^-1/2 factors (no value stream), FP32 and BF16 features
    Apat = ops.CSR(g.rowptr, g.colind, None, n, n)
    dinv = ops.degree_rsqrt(Apat)
    pn32 = ops.SpmmPlan(Apat, F, torch.float32, rowscale=dinv, colscale=dinv)
    pn16 = ops.SpmmPlan(Apat, F, torch.bfloat16, rowscale=dinv, colscale=dinv)
    Cn = torch.empty_like(C)
    Cnh = torch.empty_like(C)
    ms_n32 = mean_ms(timed, lambda: pn32.run(B, out=Cn, workspace=ws), args.steps, "timed_norm_f32", warm=3)
    ms_n16 = mean_ms(timed, lambda: pn16.run(Bh, out=Cnh, workspace=ws), args.steps, "timed_norm_bf16", warm=3)
    del pn32, pn16

    # forward + backward of Y = A H: fwd SpMM, bwd A^T dY (cached transpose)
    # and SDDMM for d(values); FP32 vs BF16 features (H, dY), FP32 accumulate
    T = ops.CSRTranspose(ops.CSR(g.rowptr, g.colind, None, n, n))
    t_vals = T.values(g.vals)
    Gd = make_grad(B.shape, dev)
    Gh = Gd.to(torch.bfloat16)
    dH = torch.empty_like(C)
    dvals = torch.empty_like(g.vals)

    # planned fused backward: A^T dY and SDDMM(dY, H) in one pass over each
    # row-range piece of A^T (pieces chosen so the dY slice fits in L2)
    bplans = {torch.float32: ops.BackwardPlan(T, t_vals, F, torch.float32),
              torch.bfloat16: ops.BackwardPlan(T, t_vals, F, torch.bfloat16)}

    def fwd_bwd(Hx, Gx, Cx):
        pf = plan32 if Hx.dtype == torch.float32 else plan16
        pf.run(Hx, out=Cx, workspace=ws)
        bplans[Hx.dtype].run(Gx, Hx, dB=dH, dvals=dvals, workspace=ws)

    for _ in range(3):
        fwd_bwd(B, Gd, C)
        fwd_bwd(Bh, Gh, Ch)
    torch.cuda.synchronize(dev)
    fb_steps = max(3, min(args.steps, 20))
    ms_fb32 = sum(timed(lambda: fwd_bwd(B, Gd, C), fb_steps, "timed_fwdbwd_f32")) / fb_steps
    ms_fb16 = sum(timed(lambda: fwd_bwd(Bh, Gh, Ch), fb_steps, "timed_fwdbwd_bf16")) / fb_steps
    del Gd, Gh, T

    bytes_f32 = gather_bytes(n, nnz, F, 4)
    bytes_bf16 = gather_bytes(n, nnz, F, 2)
    value = world * bytes_f32 / (ms_f32 * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = profile_traffic()
    # the row gathers (nnz * F elements) against the L2 -> SM ceiling measured above
    l2_gather = None
    if ceil:
        g32 = nnz * F * 4 / (ms_f32 * 1e-3) / 1e12
        g16 = nnz * F * 2 / (ms_bf16 * 1e-3) / 1e12
        l2_gather = {"unit": "TB/s", "f32": {"achieved": round(g32, 2), "ceiling": ceil.get("f32"),
                                              "frac": round(g32 / ceil["f32"], 3) if ceil.get("f32") else None},
                     "bf16": {"achieved": round(g16, 2), "ceiling": ceil.get("bf16"),
                              "frac": round(g16 / ceil["bf16"], 3) if ceil.get("bf16") else None},
                     "what": "row-gather bytes (nnz*F*elem) per second vs the ceiling bin/gather_ceiling "
                             "measured in this run (random rows of an L2-resident 32 MB table)"}

    # errors vs FP64 on sampled rows (incl. the 32 largest hubs)
    rows = sample_rows_for_error(g)
    g_cpu = g.to("cpu")
    B_cpu = B.to("cpu")
    ref, mag = fp64_rows(g_cpu, B_cpu, rows)
    rd = rows.to(dev)
    errs = {}
    for tag, Cx in (("f32", C), ("bf16_features", Ch), ("fp16_features", Cf), ("normalized_f32", Cn),
                    ("normalized_bf16_features", Cnh)):
        got = Cx[rd].cpu()
        mx, mean = rel_err(got, ref, mag)
        errs[tag] = {"max": mx, "mean": mean, "plain": plain_rel_err(got, ref)}
    del Ch, Cf, Bh, Bf, Cn, Cnh

    # the other configurations
    others = None
    if not args.no_configs:
        others = other_configs(dev, timed, max(3, min(args.steps, 5)))
        torch.cuda.empty_cache()

    # end to end through the public host-buffer entry point (gbs_csr_spmm_host):
    # pinned host A and B in, host C out, copies overlapped with the kernels
    h_rowptr = g_cpu.rowptr.pin_memory()
    h_colind = g_cpu.colind.pin_memory()
    h_vals = g_cpu.vals.pin_memory()
    h_B = B_cpu.pin_memory()
    h_C = torch.empty((n, F), dtype=torch.float32).pin_memory()

    hctx = ops.HostSpmmContext()

    def e2e_step():
        ops.csr_spmm_host(h_rowptr, h_colind, h_vals, h_B, n, n, out=h_C, ctx=hctx)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize(dev)
    e2e_steps = max(3, min(args.steps, 10))
    ms_e2e = sum(timed(e2e_step, e2e_steps, "timed_e2e")) / e2e_steps
    ms_e2e = max_over_ranks(ms_e2e, world, dev)
    e2e_err = rel_err(h_C[rows].clone(), ref, mag)[0]
    h2d = (h_rowptr.numel() * 4 + h_colind.numel() * 4 + h_vals.numel() * 4 + h_B.numel() * 4)
    d2h = h_C.numel() * 4

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu, _ = cpu_baseline(g_cpu, B_cpu)

    if rank != 0:
        return
    # HBM roofline of the step: the DRAM bytes ncu measured for one step of
    # these launches, over this run's step time (the gather-model bytes would
    # read ~3x the copy peak, since L2 serves most row gathers)
    hbm_achieved = traffic / (ms_f32 * 1e-3) / 1e9 if traffic else None
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_f32, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "nodes": n, "nnz": nnz, "F": F,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed before every timed step (512 MiB write)"},
        "roofline": {"bound": "hbm", "achieved": round(hbm_achieved, 1) if hbm_achieved else None,
                     "peak": peak, "unit": "GB/s",
                     "frac": round(hbm_achieved / peak, 4) if hbm_achieved else None,
                     "traffic": traffic, "peak_source": peak_kind,
                     "achieved_is": "measured DRAM bytes per step (ncu dram__bytes_read.sum + "
                                    "dram__bytes_write.sum, profiles/csr_spmm_plan_reddit_f256.md) / ms_per_step",
                     "gather_model_bytes_per_step": bytes_f32,
                     "per": "step = one SpMM = %d accumulating launches of k_csr_spmm_merge" % plan32.parts,
                     "binding_roofline": "l2_gather"},
        "l2_gather": l2_gather,
        "fwd_bwd": {"what": "planned SpMM A H + planned fused backward (A^T dY and SDDMM(dY, H) in one pass "
                            "per row-range piece of A^T), F=256",
                    "backward_parts": {"f32": bplans[torch.float32].parts, "bf16": bplans[torch.bfloat16].parts},
                    "f32_ms": round(ms_fb32, 4), "bf16_ms": round(ms_fb16, 4),
                    "bf16_speedup": round(ms_fb32 / ms_fb16, 3)},
        "bf16": {"ms_per_step": round(ms_bf16, 4),
                 "gbs_gather_model": round(bytes_bf16 / (ms_bf16 * 1e-3) / 1e9, 1),
                 "speedup_vs_f32": round(ms_f32 / ms_bf16, 3)},
        "normalized": {"what": "the same SpMM with binary A and the D^-1/2 factors applied in the kernel "
                                "(gbs_csr_spmm_plan_create_scaled: no value stream), planned",
                       "f32_ms": round(ms_n32, 4), "bf16_ms": round(ms_n16, 4),
                       "f32_speedup_vs_valued": round(ms_f32 / ms_n32, 3),
                       "bf16_speedup_vs_valued": round(ms_bf16 / ms_n16, 3)},
        "fp16": {"ms_per_step": round(ms_f16, 4),
                 "gbs_gather_model": round(bytes_bf16 / (ms_f16 * 1e-3) / 1e9, 1),
                 "speedup_vs_f32": round(ms_f32 / ms_f16, 3)},
        "error_vs_fp64": {"rows_sampled": int(rows.numel()),
                          "scale": "max/mean: |C-C64| / (|A| |B|) elementwise; plain: |C-C64| / |C64| over "
                                   "entries with |C64| >= floor = RMS of C64 on the sampled rows",
                          **errs},
        "e2e": {"value": round(world * bytes_f32 / (ms_e2e * 1e-3) / 1e9, 2), "unit": "GB/s",
                "ms_per_step": round(ms_e2e, 3), "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "api": "gbs_csr_spmm_host (pinned host A, B -> host C)",
                "max_rel_err": e2e_err},
        "gpu_launches": args.steps * plan32.parts,
        "plan": {"f32_column_parts": plan32.parts, "bf16_column_parts": plan16.parts,
                 "fp16_column_parts": planh.parts},
        "configs": others,
        "timed_region_wall_s": round(wall, 3),
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def run_profile_case(args):
    """Short fixed launch sequences for ncu (2 warm-up launches, then
    `--steps` launches of each kernel, nothing else heavy):
      full   : bench graph, FP32 then BF16 planned merge-path SpMM, F = 256
               (FP32: 2 column parts = 2 launches per step)
      eighth : same nodes (B still larger than L2), 1/8 of the degree
      fwdbwd : eighth graph, planned SpMM + planned fused backward (FP32, then
               BF16)
      l2resident : 232,965 rows x 492 nonzeros, columns uniform over 8K / 32K /
               128K rows (B in L2), planned FP32 and BF16 SpMM, event-timed
               medians printed (not an ncu case)
      b2sr   : flickr-shaped graph, for tiles 4 / 8 / 16 / 32: CSR->B2SR
               packing, B2SR SpMM F = 256 (tile 4 also the ordered drop-in),
               B2SR BMM F = 256
      bmm    : 4096^3 binary GEMM, popc, mma .b1, tcgen05 per tile, tcgen05
               persistent (XOR counts)
      bmmtc  : 8192^3 binary GEMM, default (persistent tcgen05) only"""
    import torch
    from spmm_eval_gb300 import graphs as G
    from spmm_eval_gb300 import ops
    dev = torch.device("cuda:0")
    case = args.profile_case
    out = {"profile_case": case}
    if case in ("full", "eighth", "fwdbwd"):
        if case == "full":
            g = G.gcn_normalize(G.reddit_like(device=dev))
        else:
            g = G.gcn_normalize(G.chung_lu(232_965, 1.8, 59.9 / 8, 20_000.0 / 8, 0x5EED + 4, dev,
                                           "reddit_like_eighth"))
        B = G.normal(0x5EED + 4, 9, (g.ncols, 256), device=dev)
        Bh = B.to(torch.bfloat16)
        A = ops.CSR(g.rowptr, g.colind, g.vals, g.nrows, g.ncols)
        C = torch.empty((g.nrows, 256), device=dev)
        ws = ops.SpmmWorkspace()
        if case == "fwdbwd":
            T = ops.CSRTranspose(ops.CSR(g.rowptr, g.colind, None, g.nrows, g.ncols))
            tv = T.values(g.vals)
            Gd = G.normal(0x5EED + 5, 11, (g.nrows, 256), device=dev)
            Gh = Gd.to(torch.bfloat16)
            dH = torch.empty_like(C)
            dv = torch.empty_like(g.vals)
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            plans = {dt: (ops.SpmmPlan(A, 256, dt), ops.BackwardPlan(T, tv, 256, dt))
                     for dt in (torch.float32, torch.bfloat16)}
            for Hx, Gx in ((B, Gd), (Bh, Gh)):
                pf, pb = plans[Hx.dtype]
                for _ in range(2 + args.steps):
                    pf.run(Hx, out=C, workspace=ws)
                    pb.run(Gx, Hx, dB=dH, dvals=dv, workspace=ws)
            out["parts"] = {str(k): [v[0].parts, v[1].parts] for k, v in plans.items()}
        else:
            plans = {torch.float32: ops.SpmmPlan(A, 256, torch.float32),
                     torch.bfloat16: ops.SpmmPlan(A, 256, torch.bfloat16)}
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            for Bx in (B, Bh):
                for _ in range(2 + args.steps):
                    plans[Bx.dtype].run(Bx, out=C, workspace=ws)
            out["parts"] = {"f32": plans[torch.float32].parts, "bf16": plans[torch.bfloat16].parts}
        out.update(nodes=g.nrows, nnz=g.nnz)
    elif case == "l2resident":
        # the bench graph's row count and mean degree with columns uniform over
        # a table that fits L2: the planned SpMM against the gather ceiling
        n, deg, F = 232_965, 492, 256
        gen = torch.Generator(device=dev)
        gen.manual_seed(5)
        res = []
        for ncols in (8192, 32768, 131072):
            ci = torch.randint(0, ncols, (n, deg), device=dev, generator=gen, dtype=torch.int32)
            ci = torch.sort(ci, dim=1)[0].reshape(-1).contiguous()
            rp = torch.arange(n + 1, device=dev, dtype=torch.int32) * deg
            A = ops.CSR(rp, ci, torch.full((n * deg,), 0.5, device=dev), n, ncols)
            C = torch.empty((n, F), device=dev)
            ws = ops.SpmmWorkspace()
            for dt in (torch.float32, torch.bfloat16):
                B = G.normal(7, 7, (ncols, F), device=dev).to(dt)
                plan = ops.SpmmPlan(A, F, dt)
                for _ in range(3):
                    plan.run(B, out=C, workspace=ws)
                ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                      for _ in range(max(args.steps, 5))]
                for s0, s1 in ev:
                    s0.record()
                    plan.run(B, out=C, workspace=ws)
                    s1.record()
                torch.cuda.synchronize()
                ms = sorted(s0.elapsed_time(s1) for s0, s1 in ev)[len(ev) // 2]
                gathered = n * deg * F * (4 if dt == torch.float32 else 2)
                res.append({"ncols": ncols, "dtype": str(dt)[6:], "parts": plan.parts, "ms": round(ms, 4),
                            "gather_tbs": round(gathered / (ms * 1e-3) / 1e12, 3)})
            del A, ci, rp, C
        out["results"] = res
    elif case == "b2sr":
        g = G.flickr_like(device=dev)
        A = ops.CSR(g.rowptr, g.colind, None, g.nrows, g.ncols)
        B = G.normal(3, 3, (g.ncols, 256), device=dev)
        Xw = ops.pack_sign_rows(B)
        for ts in (4, 8, 16, 32):
            for _ in range(2 + args.steps):
                Ab = ops.csr2b2sr(A, ts)
            for _ in range(2 + args.steps):
                ops.b2sr_spmm(Ab, B)
            if ts == 4:
                Cd = torch.zeros((Ab.nblockrows * 4, 256), device=dev)
                for _ in range(2 + args.steps):
                    ops.spmm4_full_full(Ab.val, B, Cd, Ab.rowptr, Ab.colind, Ab.nblockrows, 256)
            for _ in range(2 + args.steps):
                ops.b2sr_bmm(Ab, Xw, 256)
            out.setdefault("nnzb", {})[ts] = Ab.nnzb
        out.update(nodes=g.nrows, nnz=g.nnz)
    elif case in ("bmm", "bmmtc"):
        gen = torch.Generator(device=dev)
        gen.manual_seed(0)
        Kw, M = (128, 4096) if case == "bmm" else (256, 8192)
        Aw = torch.randint(-2**31, 2**31 - 1, (Kw, M), dtype=torch.int32, device=dev, generator=gen)
        Bw = torch.randint(-2**31, 2**31 - 1, (Kw, M), dtype=torch.int32, device=dev, generator=gen)
        Co = torch.empty((M, M), dtype=torch.int32, device=dev)
        algos = ((ops.BMM_ALGO_POPC, ops.BMM_ALGO_MMA, ops.BMM_ALGO_TC, ops.BMM_ALGO_TC_PERSIST)
                 if case == "bmm" else (ops.BMM_ALGO_DEFAULT,))
        for algo in algos:
            for _ in range(2 + args.steps):
                ops.bmm_b1(Aw, Bw, ops.BMM_XOR, algo, out=Co)
    torch.cuda.synchronize()
    out["device_bytes"] = torch.cuda.max_memory_allocated()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the other evaluation configurations")
    ap.add_argument("--profile-case", choices=["full", "eighth", "fwdbwd", "l2resident", "b2sr", "bmm", "bmmtc"],
                    default=None,
                    help="run a short fixed launch sequence for ncu instead of the bench")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
