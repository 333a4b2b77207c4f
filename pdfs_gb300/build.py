"""Builds libpdfs.so (and the PDFS command-line tool) in-tree for sm_103a.

Every CUDA translation unit is compiled by its own nvcc process in parallel
into pdfs_gb300/_build/, then linked into pdfs_gb300/libpdfs.so.  The C
sources (VTI I/O, the run_fsm shim, the CLI) are compiled by gcc.  A target
is rebuilt only when a source or header is newer than it.

    python -m pdfs_gb300.build          # or: import pdfs_gb300.build as b; b.build()
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpdfs.so")
CLI = os.path.join(PKG, "PDFS")
INC = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpdfs")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INC, "*.h"))


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    hdrs = _headers()
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    lib_c = [p for p in sorted(glob.glob(os.path.join(CSRC, "*.c"))) if not p.endswith("cli.c")]
    jobs, objs = [], []
    nv_flags = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INC, "-I" + CSRC,
                       "--expt-relaxed-constexpr"]
    # the sweep kernels' FP32 arithmetic uses approximate sqrt/divide (the
    # FP64 polish removes the difference); FP64 arithmetic is unaffected
    fast = ["-prec-sqrt=false", "-prec-div=false"]
    per_tu = {"sweep.cu": fast, "tile3d.cu": fast, "pencil.cu": fast, "pencil_batch.cu": fast, "lanecol.cu": fast,
              "lanecol_pmin.cu": fast, "lanecol_prep.cu": fast, "lanecol_pmin4.cu": fast, "lanecol_prep4.cu": fast}
    for src in cu:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append(([nvcc] + nv_flags + per_tu.get(os.path.basename(src), []) + ["-c", src, "-o", obj], src))
    c_flags = ["-O2", "-fPIC", "-std=gnu99", "-ffp-contract=off", "-I" + INC, "-I" + CSRC]
    for src in lib_c:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            jobs.append((["gcc"] + c_flags + ["-c", src, "-o", obj], src))
    procs = []
    for cmd, src in jobs:
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), src))
    failed = []
    for p, src in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError("libpdfs build failed:\n" + msg)
    if force or jobs or _newer(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-L" + os.path.join(cuda, "lib64"), "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    cli_src = os.path.join(CSRC, "cli.c")
    if os.path.exists(cli_src) and (force or _newer(CLI, [cli_src, LIB] + hdrs)):
        cmd = ["gcc", "-O2", "-std=gnu99", "-I" + INC, cli_src, "-o", CLI, "-L" + PKG, "-lpdfs",
               "-Wl,-rpath,$ORIGIN", "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
