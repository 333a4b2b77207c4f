"""Batched solves (pdfs_solve_batch) and the tile autotuner."""
import numpy as np
import pytest

from oracle import oracle as O
from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def uneven_batch(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = rng.integers(1, 70, size=3)
        if i == 0:
            n = np.array([1, 1, 1])
        if i == 1:
            n = np.array([37, 3, 41])
        k = int(rng.integers(1, 5))
        out.append(W.random_spheres(int(n[0]), int(n[1]), int(n[2]), 1.0, 1.0, 1.0, k, 1.5, 8.0,
                                    seed=int(rng.integers(0, 1 << 30)), log_radii=False))
    return out


def test_batch_fp64_bit_exact_per_grid():
    ws = uneven_batch(12, 3)
    fields = [w.field.copy() for w in ws]
    st = api.solve_batch(fields, [(w.dx, w.dy, w.dz) for w in ws], frozen=[w.frozen for w in ws],
                         freeze=L.FREEZE_MASK, tol=0.0)
    for w, f, s in zip(ws, fields, st):
        ref = w.field.copy()
        O.solve(ref, (w.dx, w.dy, w.dz), tol=0.0, frozen=w.frozen, threads=4)
        assert f.tobytes() == ref.tobytes(), w.name
        assert s["sweeps_fp64"] % 8 == 0 and s["status"] == 0


def test_batch_polish_within_tolerance():
    ws = uneven_batch(10, 9)
    fields = [w.field.copy() for w in ws]
    st = api.solve_batch(fields, [(w.dx, w.dy, w.dz) for w in ws], frozen=[w.frozen for w in ws],
                         freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_FAST, tol=1e-12)
    for w, f in zip(ws, fields):
        ref = w.field.copy()
        O.solve(ref, (w.dx, w.dy, w.dz), tol=0.0, frozen=w.frozen, threads=4)
        i = (slice(1, -1),) * 3
        # tolerance: polish to a 1e-12 max change, 1e-10 relative to the plain FP64 fixed point
        err = np.max(np.abs(f[i] - ref[i]) / np.maximum(np.abs(ref[i]), 1.0))
        assert err <= 1e-10, (w.name, err)


def test_batch_without_masks_and_invalid_args():
    ws = uneven_batch(4, 5)
    fields = [w.field.copy() for w in ws]
    api.solve_batch(fields, [(1.0, 1.0, 1.0)] * 4, tol=0.0)
    for w, f in zip(ws, fields):
        ref = w.field.copy()
        O.solve(ref, (1.0, 1.0, 1.0), tol=0.0, threads=4)
        assert f.tobytes() == ref.tobytes()
    with pytest.raises(api.PdfsError):
        api.solve_batch(fields, [(1.0, 1.0, 1.0)] * 4, fixed_sweeps=8)


def test_autotune_returns_valid_tiles():
    t = api.autotune(96, 80, 64, (1.0, 1.0, 1.0), precision=L.PREC_FP32_POLISH64)
    # FP32: columns 1-7, bricks 8, 9, 11, pencils 10; FP64 polish, reference
    # arithmetic: columns 1-2, bricks 5, 7, 8, pencils 6
    assert 1 <= (t & 0xFF) <= 11 and (t >> 8) in (1, 2, 5, 6, 7, 8)
    w = W.random_spheres(96, 80, 64, 1.0, 1.0, 1.0, 5, 3.0, 10.0, seed=2)
    a = w.field.copy()
    api.solve(a, (1.0, 1.0, 1.0), frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64,
              arith=L.ARITH_FAST, tile=t, tol=1e-12)
    ref = w.field.copy()
    O.solve(ref, (1.0, 1.0, 1.0), tol=0.0, frozen=w.frozen, threads=4)
    i = (slice(1, -1),) * 3
    assert np.max(np.abs(a[i] - ref[i]) / np.maximum(np.abs(ref[i]), 1.0)) <= 1e-10
