"""ctypes binding of libpdfs.so (include/pdfs.h).  No fallback: if the CUDA
library cannot be loaded, every call raises."""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libpdfs.so")

PDFS_OK = 0
PDFS_ERR_INVALID = -1
PDFS_ERR_OOM = -2
PDFS_ERR_CUDA = -3
PDFS_ERR_TIMEOUT = -4
PDFS_ERR_NOT_CONVERGED = -5
PDFS_ERR_IO = -6
PDFS_ERR_NO_DEVICE = -7
PDFS_ERR_TOO_LARGE = -8
STATIC_SCRATCH_BYTES = 32 << 20

PREC_FP64, PREC_FP32, PREC_FP32_POLISH64 = 0, 1, 2
ARITH_REFERENCE, ARITH_FAST, ARITH_MIXED, ARITH_PAIR = 0, 1, 2, 3
FREEZE_NONE, FREEZE_MASK = 0, 1
SCHED_NONE, SCHED_CHANGE, SCHED_LEARNED, SCHED_OCTANT = 0, 1, 2, 3

# Every function declared in include/pdfs.h (the CPU tests check the exports).
EXPORTS = [
    "pdfs_default_opts", "pdfs_solve", "pdfs_sweep", "pdfs_ctx_create", "pdfs_ctx_load", "pdfs_ctx_run",
    "pdfs_ctx_store", "pdfs_ctx_destroy", "pdfs_release_cached", "pdfs_status_string", "pdfs_version",
    "run_fsm", "pdfs_vti_read", "pdfs_vti_write", "pdfs_phi_free", "pdfs_calc_dist_field",
    "pdfs_solve_batch", "pdfs_autotune", "pdfs_static_layout", "pdfs_sweep_static",
    "pdfs_ctx_blocks", "pdfs_ctx_sweep", "pdfs_ctx_orderings",
    "pdfs_mlp_trainer_create", "pdfs_mlp_trainer_add_solve", "pdfs_mlp_trainer_fit", "pdfs_mlp_trainer_weights",
    "pdfs_mlp_trainer_destroy", "pdfs_mlp_grad", "pdfs_mlp_adam", "pdfs_mlp_infer",
]
MLP_IN, MLP_HIDDEN = 16, 64
MLP_PARAMS = MLP_HIDDEN * MLP_IN + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN + MLP_HIDDEN + 1
MLP_BLOB = MLP_PARAMS + 1


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]


class Opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("arith", C.c_int), ("freeze", C.c_int), ("scheduler", C.c_int),
                ("tol", C.c_double), ("max_sweeps", C.c_int), ("fixed_sweeps", C.c_int),
                ("first_ordering", C.c_int), ("tile", C.c_int), ("device", C.c_int),
                ("mlp_weights", C.c_void_p), ("spin_limit", C.c_longlong), ("verbose", C.c_int),
                ("reserved", C.c_int * 8)]


class Stats(C.Structure):
    _fields_ = [("status", C.c_int), ("sweeps_fp32", C.c_int), ("sweeps_fp64", C.c_int),
                ("full_sweeps", C.c_int), ("voxel_updates", C.c_longlong), ("blocks_skipped", C.c_longlong),
                ("final_change", C.c_double), ("ms_total", C.c_double), ("ms_h2d", C.c_double),
                ("ms_d2h", C.c_double), ("ms_fp32", C.c_double), ("ms_fp64", C.c_double),
                ("ms_sched", C.c_double), ("ms_kern_fp32", C.c_double),
                ("ms_kern_fp64", C.c_double), ("tile", C.c_int), ("launches", C.c_int),
                ("ms_device", C.c_double), ("voxel_updates_fp64", C.c_longlong),
                ("ms_kern_masked_fp32", C.c_double), ("ms_kern_masked_fp64", C.c_double),
                ("updates_masked_fp32", C.c_longlong), ("updates_masked_fp64", C.c_longlong),
                ("masked_sweeps_fp32", C.c_int), ("masked_sweeps_fp64", C.c_int)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}
        d["voxel_updates_fp32"] = d["voxel_updates"] - d["voxel_updates_fp64"]
        return d


class Phi(C.Structure):
    """Layout of the reference's Phi (single_gpu_cuda/src/phi3D.h:45-55)."""
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int), ("dx", C.c_double), ("dy", C.c_double),
                ("dz", C.c_double), ("location", C.POINTER(C.c_int)), ("distance", C.POINTER(C.c_double)),
                ("F", C.c_double)]


_lib = None


def load(path: str = LIB_PATH):
    """Loads libpdfs.so (built in-tree by pdfs_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libpdfs.so not found at {path}: run `python -m pdfs_gb300.build` "
                           "(the solver has no CPU fallback)")
    L = C.CDLL(path)
    vp, ip = C.c_void_p, C.c_int
    L.pdfs_default_opts.argtypes = [C.POINTER(Opts)]
    L.pdfs_default_opts.restype = None
    L.pdfs_solve.argtypes = [C.POINTER(Grid), vp, vp, C.POINTER(Opts), C.POINTER(Stats)]
    L.pdfs_solve.restype = ip
    L.pdfs_sweep.argtypes = [C.POINTER(Grid), vp, vp, ip, C.POINTER(Opts), C.POINTER(C.c_double)]
    L.pdfs_sweep.restype = ip
    L.pdfs_ctx_create.argtypes = [C.POINTER(Grid), C.POINTER(Opts), C.POINTER(vp)]
    L.pdfs_ctx_create.restype = ip
    L.pdfs_ctx_load.argtypes = [vp, vp, vp]
    L.pdfs_ctx_load.restype = ip
    L.pdfs_ctx_run.argtypes = [vp, C.POINTER(Stats)]
    L.pdfs_ctx_run.restype = ip
    L.pdfs_ctx_store.argtypes = [vp, vp]
    L.pdfs_ctx_store.restype = ip
    L.pdfs_ctx_destroy.argtypes = [vp]
    L.pdfs_ctx_destroy.restype = None
    L.pdfs_release_cached.argtypes = [ip]
    L.pdfs_release_cached.restype = ip
    L.pdfs_status_string.argtypes = [ip]
    L.pdfs_status_string.restype = C.c_char_p
    L.pdfs_version.argtypes = []
    L.pdfs_version.restype = C.c_char_p
    L.run_fsm.argtypes = [C.POINTER(Phi), ip]
    L.run_fsm.restype = None
    L.pdfs_vti_read.argtypes = [C.c_char_p, C.POINTER(Phi)]
    L.pdfs_vti_read.restype = ip
    L.pdfs_vti_write.argtypes = [C.c_char_p, C.POINTER(Phi)]
    L.pdfs_vti_write.restype = ip
    L.pdfs_phi_free.argtypes = [C.POINTER(Phi)]
    L.pdfs_phi_free.restype = None
    L.pdfs_calc_dist_field.argtypes = [C.POINTER(Phi), ip, C.POINTER(Opts), C.POINTER(Stats)]
    L.pdfs_calc_dist_field.restype = ip
    L.pdfs_solve_batch.argtypes = [ip, C.POINTER(Grid), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                   C.POINTER(Opts), C.POINTER(Stats)]
    L.pdfs_solve_batch.restype = ip
    L.pdfs_autotune.argtypes = [C.POINTER(Grid), C.POINTER(Opts), C.POINTER(ip)]
    L.pdfs_autotune.restype = ip
    L.pdfs_static_layout.argtypes = [C.POINTER(Grid)] + [C.POINTER(C.c_longlong)] * 4
    L.pdfs_static_layout.restype = ip
    L.pdfs_sweep_static.argtypes = [C.POINTER(Grid), vp, ip, C.POINTER(C.c_double), vp]
    L.pdfs_sweep_static.restype = ip
    L.pdfs_ctx_blocks.argtypes = [vp, C.POINTER(ip), C.POINTER(ip), C.POINTER(ip)]
    L.pdfs_ctx_blocks.restype = ip
    L.pdfs_ctx_sweep.argtypes = [vp, ip, vp, vp, C.POINTER(C.c_double)]
    L.pdfs_ctx_sweep.restype = ip
    L.pdfs_ctx_orderings.argtypes = [vp, vp]
    L.pdfs_ctx_orderings.restype = ip
    fp = C.POINTER(C.c_float)
    L.pdfs_mlp_trainer_create.argtypes = [ip, C.c_uint, C.POINTER(vp)]
    L.pdfs_mlp_trainer_create.restype = ip
    L.pdfs_mlp_trainer_add_solve.argtypes = [vp, C.POINTER(Grid), vp, vp, C.POINTER(Opts), C.POINTER(C.c_longlong)]
    L.pdfs_mlp_trainer_add_solve.restype = ip
    L.pdfs_mlp_trainer_fit.argtypes = [vp, ip, ip, C.c_float, C.c_float, fp]
    L.pdfs_mlp_trainer_fit.restype = ip
    L.pdfs_mlp_trainer_weights.argtypes = [vp, C.c_float, vp, fp, fp]
    L.pdfs_mlp_trainer_weights.restype = ip
    L.pdfs_mlp_trainer_destroy.argtypes = [vp]
    L.pdfs_mlp_trainer_destroy.restype = None
    L.pdfs_mlp_grad.argtypes = [vp, vp, vp, ip, C.c_float, vp, fp]
    L.pdfs_mlp_grad.restype = ip
    L.pdfs_mlp_adam.argtypes = [vp, vp, vp, vp, ip, C.c_float, C.c_float, C.c_float, C.c_float, vp]
    L.pdfs_mlp_adam.restype = ip
    L.pdfs_mlp_infer.argtypes = [vp, vp, ip, vp]
    L.pdfs_mlp_infer.restype = ip
    _lib = L
    return L
