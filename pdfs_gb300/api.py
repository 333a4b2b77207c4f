"""Python front end of the GB300 FSM solver (thin layer over the C ABI).

Mirrors the reference's solve entry points: ``sweep(field, spacing, sn)`` is
runFSM(pf, sn) (mpi_openacc/src/phi3D_fsm.c:67), ``run_fsm(field, spacing,
rounds)`` is run_fsm(pf, iterations) (single_gpu_cuda/src/phi3D_fsm.cu:64),
``solve`` iterates to convergence.  Fields are numpy float64 arrays of shape
(nz+2, ny+2, nx+2) in the reference's halo-padded layout; they are updated in
place.  Errors raise PdfsError carrying the C status code.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class PdfsError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = L.load().pdfs_status_string(status).decode()
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


def _grid(field: np.ndarray, spacing) -> L.Grid:
    if field.ndim != 3:
        raise ValueError("field must be 3-D (nz+2, ny+2, nx+2)")
    nz, ny, nx = (s - 2 for s in field.shape)
    return L.Grid(nx, ny, nz, float(spacing[0]), float(spacing[1]), float(spacing[2]))


def _check_field(field):
    if field.dtype != np.float64 or not field.flags.c_contiguous:
        raise ValueError("field must be a C-contiguous float64 array")


def make_opts(precision=L.PREC_FP64, arith=L.ARITH_REFERENCE, freeze=L.FREEZE_NONE, scheduler=L.SCHED_NONE,
              tol=0.0, max_sweeps=0, fixed_sweeps=0, first_ordering=0, tile=0, device=0, verbose=0,
              wait_ms=0, mlp_weights=None) -> L.Opts:
    """pdfs_opts from keyword arguments.  mlp_weights: a float32 blob of
    MLP_BLOB values (kept alive by the caller while the options are used)."""
    o = L.Opts()
    L.load().pdfs_default_opts(C.byref(o))
    o.precision, o.arith, o.freeze, o.scheduler = precision, arith, freeze, scheduler
    o.tol, o.max_sweeps, o.fixed_sweeps, o.first_ordering = tol, max_sweeps, fixed_sweeps, first_ordering
    o.tile, o.device, o.verbose, o.spin_limit = tile, device, verbose, wait_ms
    if mlp_weights is not None:
        if mlp_weights.dtype != np.float32 or mlp_weights.size != L.MLP_BLOB or not mlp_weights.flags.c_contiguous:
            raise ValueError("mlp_weights must be a contiguous float32 array of MLP_BLOB values")
        o.mlp_weights = mlp_weights.ctypes.data
    return o


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data if isinstance(a, np.ndarray) else int(a))


def solve(field: np.ndarray, spacing, frozen: np.ndarray | None = None, **kw) -> dict:
    """Solves in place; returns the stats as a dict.  Keyword arguments are
    the pdfs_opts fields (see make_opts)."""
    _check_field(field)
    if frozen is not None:
        if frozen.shape != field.shape or frozen.dtype != np.uint8:
            raise ValueError("frozen must be a uint8 array shaped like field")
        frozen = np.ascontiguousarray(frozen)
    g = _grid(field, spacing)
    o = make_opts(**kw)
    st = L.Stats()
    s = L.load().pdfs_solve(C.byref(g), _ptr(field), _ptr(frozen), C.byref(o), C.byref(st))
    if s != L.PDFS_OK:
        raise PdfsError(s, "pdfs_solve")
    return st.as_dict()


def sweep(field: np.ndarray, spacing, sn: int, frozen=None, arith=L.ARITH_REFERENCE, freeze=L.FREEZE_NONE,
          tile=0) -> float:
    """One ordering sn (1..8) in place; returns the sweep's max change."""
    _check_field(field)
    g = _grid(field, spacing)
    o = make_opts(arith=arith, freeze=freeze, tile=tile)
    ch = C.c_double(0.0)
    s = L.load().pdfs_sweep(C.byref(g), _ptr(field), _ptr(frozen), int(sn), C.byref(o), C.byref(ch))
    if s != L.PDFS_OK:
        raise PdfsError(s, "pdfs_sweep")
    return ch.value


def run_fsm(field: np.ndarray, spacing, rounds: int = 1, **kw) -> dict:
    """`rounds` rounds of the 8 orderings with no convergence test, as the
    reference's run_fsm(pf, iterations)."""
    return solve(field, spacing, fixed_sweeps=8 * int(rounds), **kw)


def _data_ptr(a, itemsize):
    """Address of a C-contiguous numpy array, or of a contiguous device tensor
    (any object with data_ptr(), e.g. a torch CUDA tensor)."""
    if isinstance(a, np.ndarray):
        if a.itemsize != itemsize or not a.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous with %d-byte elements" % itemsize)
        return a.ctypes.data
    if a.element_size() != itemsize or not a.is_contiguous():
        raise ValueError("tensors must be contiguous with %d-byte elements" % itemsize)
    return int(a.data_ptr())


def solve_batch(fields, spacings, frozen=None, **kw):
    """Solves many grids in one batched solve (pdfs_solve_batch), in place.
    Fields (float64) and frozen masks (uint8) are numpy arrays or device
    tensors.  Returns the per-grid stats dicts."""
    n = len(fields)
    grids = (L.Grid * n)()
    fptr = (C.c_void_p * n)()
    mptr = (C.c_void_p * n)()
    for i, f in enumerate(fields):
        if isinstance(f, np.ndarray):
            _check_field(f)
        g = _grid(f, spacings[i])
        grids[i] = g
        fptr[i] = _data_ptr(f, 8)
        mptr[i] = _data_ptr(frozen[i], 1) if frozen is not None and frozen[i] is not None else None
    o = make_opts(**kw)
    st = (L.Stats * n)()
    s = L.load().pdfs_solve_batch(n, grids, fptr, mptr if frozen is not None else None, C.byref(o), st)
    if s != L.PDFS_OK:
        raise PdfsError(s, "pdfs_solve_batch")
    return [x.as_dict() for x in st]


def release_cached(device: int = 0) -> None:
    """Returns the device blocks that destroyed contexts left in the library's
    cache to CUDA (pdfs_release_cached)."""
    s = L.load().pdfs_release_cached(int(device))
    if s != L.PDFS_OK:
        raise PdfsError(s, "pdfs_release_cached")


def autotune(nx, ny, nz, spacing, **kw) -> int:
    """Fastest tile pair for this grid shape (an opts.tile value)."""
    g = L.Grid(nx, ny, nz, *map(float, spacing))
    o = make_opts(**kw)
    t = C.c_int(0)
    s = L.load().pdfs_autotune(C.byref(g), C.byref(o), C.byref(t))
    if s != L.PDFS_OK:
        raise PdfsError(s, "pdfs_autotune")
    return t.value


class Context:
    """Device-resident solve context (pdfs_ctx_*)."""

    def __init__(self, nx, ny, nz, spacing, **kw):
        self._lib = L.load()
        self.grid = L.Grid(nx, ny, nz, *map(float, spacing))
        self.opts = make_opts(**kw)
        h = C.c_void_p()
        s = self._lib.pdfs_ctx_create(C.byref(self.grid), C.byref(self.opts), C.byref(h))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_ctx_create")
        self.h = h

    def load(self, field, frozen=None):
        s = self._lib.pdfs_ctx_load(self.h, _ptr(field), _ptr(frozen))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_ctx_load")

    def run(self) -> dict:
        st = L.Stats()
        s = self._lib.pdfs_ctx_run(self.h, C.byref(st))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_ctx_run")
        return st.as_dict()

    def store(self, field):
        s = self._lib.pdfs_ctx_store(self.h, _ptr(field))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_ctx_store")

    def blocks(self):
        """(nbx, nby, nbz): the grid's 8^3 node blocks."""
        b = [C.c_int() for _ in range(3)]
        s = self._lib.pdfs_ctx_blocks(self.h, *(C.byref(x) for x in b))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_ctx_blocks")
        return tuple(x.value for x in b)

    def orderings(self) -> np.ndarray:
        """Per 8^3 block (nbz, nby, nbx), the bit set of the orderings that
        matter to it, from the FP32 working field (pdfs_ctx_orderings)."""
        nbx, nby, nbz = self.blocks()
        out = np.zeros((nbz, nby, nbx), dtype=np.uint8)
        s = self._lib.pdfs_ctx_orderings(self.h, out.ctypes.data)
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_ctx_orderings")
        return out

    def sweep(self, sn: int, active=None, block_change=None) -> float:
        """One ordering on the working field (pdfs_ctx_sweep); active and
        block_change are uint8 / float32 arrays with one entry per block,
        (nbz, nby, nbx), or device pointers.  Returns the max change."""
        if isinstance(active, np.ndarray):
            active = np.ascontiguousarray(active, dtype=np.uint8)
        if isinstance(block_change, np.ndarray):
            if block_change.dtype != np.float32 or not block_change.flags.c_contiguous:
                raise ValueError("block_change must be a C-contiguous float32 array")
        ch = C.c_double(0.0)
        s = self._lib.pdfs_ctx_sweep(self.h, int(sn), _ptr(active), _ptr(block_change), C.byref(ch))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_ctx_sweep")
        return ch.value

    def close(self):
        if getattr(self, "h", None):
            self._lib.pdfs_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- learned block scheduler ---------------------------------------------------------
class Trainer:
    """The scheduler network's trainer (pdfs_mlp_trainer_*): samples come from
    plain solves on the GPU, fitting runs the library's bf16 kernels."""

    def __init__(self, device=0, seed=0):
        self._lib = L.load()
        h = C.c_void_p()
        s = self._lib.pdfs_mlp_trainer_create(int(device), int(seed), C.byref(h))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_mlp_trainer_create")
        self.h = h

    def add_solve(self, field, spacing, frozen=None, **kw) -> int:
        _check_field(field)
        g = _grid(field, spacing)
        o = make_opts(**kw)
        n = C.c_longlong(0)
        s = self._lib.pdfs_mlp_trainer_add_solve(self.h, C.byref(g), _ptr(field), _ptr(frozen), C.byref(o),
                                                 C.byref(n))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_mlp_trainer_add_solve")
        return n.value

    def fit(self, epochs=4, batch=8192, lr=2e-3, pos_weight=4.0) -> float:
        loss = C.c_float(0.0)
        s = self._lib.pdfs_mlp_trainer_fit(self.h, int(epochs), int(batch), float(lr), float(pos_weight),
                                           C.byref(loss))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_mlp_trainer_fit")
        return loss.value

    def weights(self, recall=0.99):
        """(blob, recall, active fraction) with the threshold set for `recall`."""
        blob = np.zeros(L.MLP_BLOB, dtype=np.float32)
        r, a = C.c_float(0.0), C.c_float(0.0)
        s = self._lib.pdfs_mlp_trainer_weights(self.h, float(recall), _ptr(blob), C.byref(r), C.byref(a))
        if s != L.PDFS_OK:
            raise PdfsError(s, "pdfs_mlp_trainer_weights")
        return blob, r.value, a.value

    def close(self):
        if getattr(self, "h", None):
            self._lib.pdfs_mlp_trainer_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mlp_grad(params, x_bits, y, pos_weight=1.0):
    """GPU gradient (pdfs_mlp_grad): params float32[MLP_PARAMS], x_bits
    uint16[n, 16] bf16 features, y uint8[n].  Returns (grad, loss)."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    x_bits = np.ascontiguousarray(x_bits, dtype=np.uint16)
    y = np.ascontiguousarray(y, dtype=np.uint8)
    g = np.zeros(L.MLP_PARAMS, dtype=np.float32)
    loss = C.c_float(0.0)
    s = L.load().pdfs_mlp_grad(_ptr(params), _ptr(x_bits), _ptr(y), len(y), float(pos_weight), _ptr(g),
                               C.byref(loss))
    if s != L.PDFS_OK:
        raise PdfsError(s, "pdfs_mlp_grad")
    return g, loss.value


def mlp_adam(params, m, v, grad, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One GPU Adam step (pdfs_mlp_adam) on copies; returns (params, m, v, bf16 bits)."""
    p, m, v = (np.array(a, dtype=np.float32) for a in (params, m, v))
    grad = np.ascontiguousarray(grad, dtype=np.float32)
    pb = np.zeros(L.MLP_PARAMS, dtype=np.uint16)
    s = L.load().pdfs_mlp_adam(_ptr(p), _ptr(m), _ptr(v), _ptr(grad), int(step), float(lr), float(beta1),
                               float(beta2), float(eps), _ptr(pb))
    if s != L.PDFS_OK:
        raise PdfsError(s, "pdfs_mlp_adam")
    return p, m, v, pb


def mlp_infer(blob, x_bits):
    """Logits of bf16 features under a weight blob (pdfs_mlp_infer)."""
    blob = np.ascontiguousarray(blob, dtype=np.float32)
    x_bits = np.ascontiguousarray(x_bits, dtype=np.uint16)
    out = np.zeros(len(x_bits), dtype=np.float32)
    s = L.load().pdfs_mlp_infer(_ptr(blob), _ptr(x_bits), len(x_bits), _ptr(out))
    if s != L.PDFS_OK:
        raise PdfsError(s, "pdfs_mlp_infer")
    return out
