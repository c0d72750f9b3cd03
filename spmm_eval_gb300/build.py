"""In-tree build of the sm_103a library ``lib/libgbspmm.so`` and the drop-in
executables.

Every ``csrc/*.cu`` file is compiled by nvcc for ``sm_103a`` only (one
``-gencode``), in parallel, then linked into one shared library with a plain
C ABI (``include/gbspmm.h``).  Objects are rebuilt only when a source or
header is newer than the object.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libgbspmm.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbspmm")


def _newest_header() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, hdr_mtime: float, verbose: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile csrc/*.cu and link lib/libgbspmm.so; returns the library path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    hdr = _newest_header()
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr, verbose), srcs))
    newest_obj = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest_obj:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs),
               "-o", str(tmp), "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libgbspmm.so failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


APPS = PKG / "apps"
BIN = PKG / "bin"
# {kernel_name} executables of the reference's driver surface, all links to
# one binary that dispatches on its program name
DRIVER_NAMES = ["spmmfbf", "spmmcsr", "spmmcsr_bf16", "spmmb2sr8", "spmmb2sr16", "spmmb2sr32", "spmmbmm"]


def build_apps(verbose: bool = False) -> Path:
    """Compile apps/spmm_driver.cu into bin/spmm_driver (linked against
    lib/libgbspmm.so and cuSPARSE, the reference's verifier), the
    per-kernel links and bin/gather_ceiling (apps/gather_ceiling.cu)."""
    lib = build(verbose)
    BIN.mkdir(parents=True, exist_ok=True)
    exe = BIN / "spmm_driver"
    src = APPS / "spmm_driver.cu"
    newest = max(src.stat().st_mtime, lib.stat().st_mtime, _newest_header())
    if not exe.exists() or exe.stat().st_mtime < newest:
        cmd = [nvcc(), *ARCH, "-O2", "-std=c++17", f"-I{INCLUDE}", str(src), "-o", str(exe),
               f"-L{LIBDIR}", "-lgbspmm", "-lcusparse", "-Xlinker", "-rpath,$ORIGIN/../lib"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    # the L2 -> SM gather ceiling probe quoted beside the SpMM's gather rate
    probe = BIN / "gather_ceiling"
    psrc = APPS / "gather_ceiling.cu"
    if not probe.exists() or probe.stat().st_mtime < psrc.stat().st_mtime:
        cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", str(psrc), "-o", str(probe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"gather_ceiling build failed:\n{r.stdout}\n{r.stderr}")
    for name in DRIVER_NAMES:
        link = BIN / name
        if not link.is_symlink():
            if link.exists():
                link.unlink()
            link.symlink_to("spmm_driver")
    return exe


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    if "--apps" in sys.argv:
        print(build_apps(verbose="-v" in sys.argv))
