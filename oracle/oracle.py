"""ctypes front end of the CPU oracle (test infrastructure only).

Libraries:
  * oracle/_build/liboracle.so  -- this project's C restatement of the FSM
    (fsm_oracle.c), built by `make -C oracle`; available on every machine.
  * oracle/_ref/libref_fsm.so   -- the reference's own mpi_openacc/src/phi3D_fsm.c,
    built unmodified by `make -C oracle ref` where the reference sources exist.
  * oracle/_ref/ref_fsm_cuda*.cubin -- the reference's own CUDA sweep kernel
    (single_gpu_cuda/src/phi3D_fsm.cu), built unmodified by `make -C oracle
    refcu`, and oracle/_build/libref_cuda.so (ref_cuda_host.c), the host
    level loop that runs it on a GPU through the driver API.

Only tests, the smoke check and the benchmark's CPU-baseline leg import this
module, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_fsm.so")
REF_OMP_PATH = os.path.join(HERE, "_ref", "libref_fsm_omp.so")
REF_CUBIN = {"nvcc": os.path.join(HERE, "_ref", "ref_fsm_cuda.cubin"),
             "nofma": os.path.join(HERE, "_ref", "ref_fsm_cuda_nofma.cubin")}
RC_PATH = os.path.join(HERE, "_build", "libref_cuda.so")


def ref_root() -> str:
    """The reference tree: $PDFS_REF_ROOT, else the default of oracle/Makefile
    (the recipe that builds the reference's own solver from its sources)."""
    r = os.environ.get("PDFS_REF_ROOT")
    if r:
        return r
    try:
        out = subprocess.run(["make", "-s", "-C", HERE, "print-ref-root"], check=True, capture_output=True,
                             text=True).stdout.strip()
        return out.splitlines()[-1] if out else ""
    except (OSError, subprocess.CalledProcessError):
        return ""


def ref_src() -> str:
    """Directory of the reference's MPI/OpenACC solver sources (may not exist)."""
    return os.path.join(ref_root(), "mpi_openacc", "src")

_lib = None
_ref = {}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build(ref: bool = True) -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    # the host driver of the reference's CUDA kernel: needs only the CUDA
    # toolkit's header and driver stub, so it builds wherever the library does
    if os.path.exists(os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include", "cuda.h")):
        subprocess.run(["make", "-s", "-C", HERE, "cudahost"], check=True)
    if ref and os.path.isdir(ref_src()):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF_ROOT=" + ref_root()], check=True)
        if os.path.isdir(os.path.join(ref_root(), "single_gpu_cuda", "src")):
            subprocess.run(["make", "-s", "-C", HERE, "refcu", "REF_ROOT=" + ref_root()], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = C.CDLL(LIB_PATH)
        L.orc_godunov.restype = C.c_double
        L.orc_godunov.argtypes = [C.c_double] * 6
        L.orc_godunov_f32.restype = C.c_float
        L.orc_godunov_f32.argtypes = [C.c_float] * 6
        L.orc_sweep.restype = C.c_double
        L.orc_sweep.argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [_dp, C.c_void_p, C.c_int, C.c_int]
        L.orc_sweep_replace.restype = C.c_double
        L.orc_sweep_replace.argtypes = ([C.c_int] * 3 + [C.c_double] * 3 +
                                        [_dp, C.c_void_p, _dp, C.c_int, C.c_int])
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = ([C.c_int] * 3 + [C.c_double] * 3 +
                                [_dp, C.c_void_p, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_double)])
        L.orc_sweep_f32.restype = C.c_float
        L.orc_sweep_f32.argtypes = [C.c_int] * 3 + [C.c_float] * 3 + [_fp, C.c_void_p, C.c_int]
        L.orc_max_threads.restype = C.c_int
        _lib = L
    return _lib


def have_ref(omp: bool = False) -> bool:
    return os.path.exists(REF_OMP_PATH if omp else REF_PATH)


def ref(omp: bool = False):
    key = "omp" if omp else "serial"
    if key not in _ref:
        L = C.CDLL(REF_OMP_PATH if omp else REF_PATH)
        L.ref_sweep.restype = None
        L.ref_sweep.argtypes = [C.c_int] * 3 + [C.c_double] * 3 + [_dp, C.c_int]
        _ref[key] = L
    return _ref[key]


def _mask_ptr(frozen):
    if frozen is None:
        return None
    assert frozen.dtype == np.uint8 and frozen.flags.c_contiguous
    return frozen.ctypes.data


def _dims(u):
    nz, ny, nx = (s - 2 for s in u.shape)
    return nx, ny, nz


def godunov(mx, my, mz, dx, dy, dz) -> float:
    return lib().orc_godunov(mx, my, mz, dx, dy, dz)


def sweep(u, spacing, sn, frozen=None, threads=1) -> float:
    """One ordering sn in 1..8, in place.  Returns the sweep's max change."""
    nx, ny, nz = _dims(u)
    return lib().orc_sweep(nx, ny, nz, *spacing, u, _mask_ptr(frozen), sn, threads)


def sweep_replace(u, spacing, sn, cap, frozen=None, threads=1) -> float:
    nx, ny, nz = _dims(u)
    return lib().orc_sweep_replace(nx, ny, nz, *spacing, u, _mask_ptr(frozen), cap, sn, threads)


def solve(u, spacing, tol=0.0, max_sweeps=10_000, frozen=None, threads=1):
    """Plain FSM to the first sweep with max change <= tol.  In place.
    Returns (sweeps, last_change)."""
    nx, ny, nz = _dims(u)
    last = C.c_double(0.0)
    s = lib().orc_solve(nx, ny, nz, *spacing, u, _mask_ptr(frozen), tol, max_sweeps, threads, C.byref(last))
    return s, last.value


def sweep_f32(u, spacing, sn, frozen=None) -> float:
    nx, ny, nz = _dims(u)
    return lib().orc_sweep_f32(nx, ny, nz, *spacing, u, _mask_ptr(frozen), sn)


def ref_sweep(u, spacing, sn, omp=False) -> float:
    """The reference's runFSM(pf, sn) on u, in place; returns the max change."""
    nx, ny, nz = _dims(u)
    before = u.copy()
    ref(omp).ref_sweep(nx, ny, nz, *spacing, u, sn)
    with np.errstate(invalid="ignore"):
        d = np.abs(u - before)
    d = d[np.isfinite(d)]
    return float(d.max()) if d.size else 0.0


def ref_sweep_raw(u, spacing, sn, omp=False) -> None:
    """The reference's runFSM(pf, sn) on u, in place, without measuring the
    change (for timing)."""
    nx, ny, nz = _dims(u)
    ref(omp).ref_sweep(nx, ny, nz, *spacing, u, sn)


def ref_solve(u, spacing, tol=0.0, max_sweeps=10_000, omp=False):
    s, c = 0, 0.0
    while s < max_sweeps:
        c = ref_sweep(u, spacing, (s % 8) + 1, omp=omp)
        s += 1
        if c <= tol:
            break
    return s, c


def max_threads() -> int:
    return lib().orc_max_threads()


# ---------------- the reference's own CUDA kernel (single_gpu_cuda) ----------------
_rc = {"lib": None, "cubin": None}


def have_ref_cuda(variant: str = "nvcc") -> bool:
    """True where the reference's CUDA kernel was built (oracle/_ref) and its
    host driver too; the GPU itself is checked by ref_cuda_run."""
    return os.path.exists(REF_CUBIN[variant]) and os.path.exists(RC_PATH)


def _rc_lib(variant: str):
    if _rc["lib"] is None:
        L = C.CDLL(RC_PATH)
        L.rc_error.restype = C.c_char_p
        L.rc_open.argtypes = [C.c_char_p]
        L.rc_run.argtypes = ([_dp] + [C.c_int] * 3 + [C.c_double] * 3 + [C.c_int] * 3 +
                             [C.POINTER(C.c_double)] * 2)
        _rc["lib"] = L
    L = _rc["lib"]
    if _rc["cubin"] != variant:
        if L.rc_open(REF_CUBIN[variant].encode()) != 0:
            raise RuntimeError("reference CUDA kernel: " + L.rc_error().decode())
        _rc["cubin"] = variant
    return L


def ref_cuda_run(u, spacing, first=1, nsweeps=8, sync_each=True, variant="nvcc"):
    """nsweeps orderings from `first` (the reference's run_fsm round is 1, 8)
    by the reference's own CUDA kernel and level loop, in place on u (the
    reference layout).  variant "nvcc": built as the reference's Makefile
    builds it; "nofma": without multiply-add contraction.  Returns
    (sweep ms on the device, whole-call ms)."""
    nx, ny, nz = _dims(u)
    L = _rc_lib(variant)
    a, b = C.c_double(0.0), C.c_double(0.0)
    r = L.rc_run(u, nx, ny, nz, *spacing, int(first), int(nsweeps), 1 if sync_each else 0, C.byref(a), C.byref(b))
    if r != 0:
        raise RuntimeError("reference CUDA kernel: " + L.rc_error().decode())
    return a.value, b.value
