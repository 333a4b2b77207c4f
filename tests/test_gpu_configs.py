"""Parity at the workloads' real sizes, against the oracle (the CPU
restatement pinned bit for bit to the reference's own phi3D_fsm.c), on the
same seeded inputs (pdfs_gb300/workloads.py):

  C2  512 x 512 x 128 heightmap, dz = 0.5
  C4  768^3, 150 spheres (the headline workload)
  C5  a 12-grid batch from the batch workload's size distribution (32..256)

Bars (relative error |a - b| / max(|b|, h) over interior nodes):
  * FP64 reference arithmetic: bit-exact, with the oracle's sweep count;
  * FP64 fast arithmetic: <= 1e-12;
  * FP32 bulk + polish (pair, or FP64 fast arithmetic): <= 1e-6 max, with
    the RMS error reported in the message and bounded by 1e-7;
  * FP32 alone: <= 2e-5 (no polish).
The oracle solves at the tolerance the GPU solve uses (1e-12), with OpenMP
over each hyperplane on every host core."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1
INNER = (slice(1, -1),) * 3


def errs(a, b, h):
    e = np.abs(a[INNER] - b[INNER]) / np.maximum(np.abs(b[INNER]), h)
    return float(e.max()), float(np.sqrt(np.mean(e * e)))


def oracle_solution(w, tol=1e-12):
    ref = w.field.copy()
    sweeps, _ = O.solve(ref, (w.dx, w.dy, w.dz), tol=tol, frozen=w.frozen, threads=THREADS)
    return ref, sweeps


FZ = dict(freeze=L.FREEZE_MASK)
POLISH = {
    "pair": dict(precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR),
    "fp64": dict(precision=L.PREC_FP32_POLISH64, arith=L.ARITH_FAST),
}


@pytest.fixture(scope="module")
def c2():
    w = W.config("C2")
    ref, sweeps = oracle_solution(w)
    return w, ref, sweeps


@pytest.fixture(scope="module")
def c4():
    w = W.config("C4")
    ref, sweeps = oracle_solution(w)
    return w, ref, sweeps


@pytest.mark.parametrize("cfg", ["c2", "c4"])
def test_fp64_reference_arith_bit_exact(cfg, request):
    w, ref, sweeps = request.getfixturevalue(cfg)
    a = w.field.copy()
    st = api.solve(a, (w.dx, w.dy, w.dz), frozen=w.frozen, precision=L.PREC_FP64, arith=L.ARITH_REFERENCE,
                   tol=1e-12, **FZ)
    assert st["sweeps_fp64"] == sweeps
    assert a.tobytes() == ref.tobytes(), "max diff %g" % float(np.max(np.abs(a - ref)))


@pytest.mark.parametrize("cfg", ["c2", "c4"])
def test_fp64_fast_arith_within_1e12(cfg, request):
    w, ref, _ = request.getfixturevalue(cfg)
    a = w.field.copy()
    api.solve(a, (w.dx, w.dy, w.dz), frozen=w.frozen, precision=L.PREC_FP64, arith=L.ARITH_FAST, tol=1e-12, **FZ)
    mx, rms = errs(a, ref, min(w.dx, w.dy, w.dz))
    assert mx <= 1e-12, (mx, rms)


@pytest.mark.parametrize("sched", [L.SCHED_NONE, L.SCHED_LEARNED])
@pytest.mark.parametrize("polish", ["pair", "fp64"])
@pytest.mark.parametrize("cfg", ["c2", "c4"])
def test_fp32_polish_within_1e6(cfg, polish, sched, request):
    w, ref, _ = request.getfixturevalue(cfg)
    h = min(w.dx, w.dy, w.dz)
    a = w.field.copy()
    api.solve(a, (w.dx, w.dy, w.dz), frozen=w.frozen, tol=1e-5 * h, scheduler=sched, **POLISH[polish], **FZ)
    mx, rms = errs(a, ref, h)
    assert mx <= 1e-6 and rms <= 1e-7, (mx, rms)


@pytest.mark.parametrize("cfg", ["c2", "c4"])
def test_fp32_alone_within_2e5(cfg, request):
    w, ref, _ = request.getfixturevalue(cfg)
    a = w.field.copy()
    api.solve(a, (w.dx, w.dy, w.dz), frozen=w.frozen, precision=L.PREC_FP32, **FZ)
    mx, rms = errs(a, ref, min(w.dx, w.dy, w.dz))
    assert mx <= 2e-5, (mx, rms)


def test_batch_c5_sizes_bit_exact_per_grid():
    """Twelve grids drawn from the batch workload's size distribution (per
    axis log-uniform 32..256, 1-20 spheres): one batched FP64 solve in the
    reference arithmetic, each grid bit-exact with the oracle."""
    ws = W.batch_c5(count=12, seed=11)
    assert max(max(w.nx, w.ny, w.nz) for w in ws) > 128
    fields = [w.field.copy() for w in ws]
    st = api.solve_batch(fields, [(w.dx, w.dy, w.dz) for w in ws], frozen=[w.frozen for w in ws],
                         precision=L.PREC_FP64, arith=L.ARITH_REFERENCE, tol=0.0, **FZ)
    for w, f, s in zip(ws, fields, st):
        ref = w.field.copy()
        O.solve(ref, (w.dx, w.dy, w.dz), tol=0.0, frozen=w.frozen, threads=THREADS)
        assert s["status"] == 0
        assert f.tobytes() == ref.tobytes(), w.name


def test_batch_c5_sizes_polish_within_1e6():
    """The same twelve grids, batched FP32 + polish: each within 1e-6 of the
    oracle's FP64 fixed point."""
    ws = W.batch_c5(count=12, seed=11)
    fields = [w.field.copy() for w in ws]
    api.solve_batch(fields, [(w.dx, w.dy, w.dz) for w in ws], frozen=[w.frozen for w in ws],
                    precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-5, **FZ)
    for w, f in zip(ws, fields):
        ref, _ = oracle_solution(w)
        mx, rms = errs(f, ref, 1.0)
        assert mx <= 1e-6, (w.name, mx, rms)
