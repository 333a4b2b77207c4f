"""Batched solves (pdfs_solve_batch) and the tile autotuner.

A batch runs on pencils by default: one launch per round of 8 orderings
over every grid (pencil.cuh's batched mode).  Column tiles, asked for
explicitly, run one launch per sweep."""
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


def test_batch_device_tensors_equal_host_arrays():
    """Fields and masks handed over as device tensors (the inputs already in
    HBM): the same bits as host arrays, solved in place on the device."""
    torch = pytest.importorskip("torch")
    ws = uneven_batch(9, 21)
    sps = [(w.dx, w.dy, w.dz) for w in ws]
    kw = dict(freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-9)
    host = [w.field.copy() for w in ws]
    api.solve_batch(host, sps, frozen=[w.frozen for w in ws], **kw)
    dev = [torch.from_numpy(w.field).cuda() for w in ws]
    api.solve_batch(dev, sps, frozen=[torch.from_numpy(w.frozen).cuda() for w in ws], **kw)
    for h, d in zip(host, dev):
        assert h.tobytes() == d.cpu().numpy().tobytes()


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
    # FP32: columns 1-7, bricks 8, 9, 11, pencils 10, lane columns 12-13; FP64
    # polish, reference arithmetic: columns 1-2, bricks 5, 7, 8, pencils 6
    assert 1 <= (t & 0xFF) <= 13 and (t >> 8) in (1, 2, 5, 6, 7, 8)
    w = W.random_spheres(96, 80, 64, 1.0, 1.0, 1.0, 5, 3.0, 10.0, seed=2)
    a = w.field.copy()
    api.solve(a, (1.0, 1.0, 1.0), frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64,
              arith=L.ARITH_FAST, tile=t, tol=1e-12)
    ref = w.field.copy()
    O.solve(ref, (1.0, 1.0, 1.0), tol=0.0, frozen=w.frozen, threads=4)
    i = (slice(1, -1),) * 3
    assert np.max(np.abs(a[i] - ref[i]) / np.maximum(np.abs(ref[i]), 1.0)) <= 1e-10


COLUMNS = 4 | (1 << 8)  # column tiles: the per-sweep batched launch


def test_batch_on_columns_still_bit_exact():
    ws = uneven_batch(8, 21)
    fields = [w.field.copy() for w in ws]
    api.solve_batch(fields, [(w.dx, w.dy, w.dz) for w in ws], frozen=[w.frozen for w in ws],
                    freeze=L.FREEZE_MASK, tol=0.0, tile=COLUMNS)
    for w, f in zip(ws, fields):
        ref = w.field.copy()
        O.solve(ref, (w.dx, w.dy, w.dz), tol=0.0, frozen=w.frozen, threads=4)
        assert f.tobytes() == ref.tobytes(), w.name


def test_pencil_rounds_mixed_spacings_and_sizes():
    """Isotropic and anisotropic grids, tiny and taller than a pencil's ring,
    in one batch: the round kernel stages each grid's description per ticket."""
    rng = np.random.default_rng(4)
    ws = []
    for i, (n, sp) in enumerate([((1, 1, 1), (1.0, 1.0, 1.0)), ((17, 33, 5), (0.7, 1.0, 0.5)),
                                 ((48, 40, 96), (1.0, 1.0, 1.0)), ((33, 16, 70), (0.5, 0.5, 1.0)),
                                 ((64, 64, 64), (1.0, 1.0, 1.0))]):
        ws.append(W.random_spheres(*n, *sp, 3, 1.5, 8.0, seed=int(rng.integers(1 << 30)), log_radii=False))
    fields = [w.field.copy() for w in ws]
    st = api.solve_batch(fields, [(w.dx, w.dy, w.dz) for w in ws], frozen=[w.frozen for w in ws],
                         freeze=L.FREEZE_MASK, tol=0.0)
    for w, f, s in zip(ws, fields, st):
        ref = w.field.copy()
        O.solve(ref, (w.dx, w.dy, w.dz), tol=0.0, frozen=w.frozen, threads=4)
        na, nb = np.isnan(f), np.isnan(ref)  # the reference arithmetic's NaN (far nodes, anisotropic)
        assert np.array_equal(na, nb) and f[~na].tobytes() == ref[~nb].tobytes(), w.name
        assert s["status"] == 0 and s["launches"] > 0


def test_pencil_rounds_pair_polish_within_1e6():
    ws = uneven_batch(10, 13)
    fields = [w.field.copy() for w in ws]
    st = api.solve_batch(fields, [(w.dx, w.dy, w.dz) for w in ws], frozen=[w.frozen for w in ws],
                         freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-5)
    i = (slice(1, -1),) * 3
    for w, f, s in zip(ws, fields, st):
        ref = w.field.copy()
        O.solve(ref, (w.dx, w.dy, w.dz), tol=1e-12, frozen=w.frozen, threads=4)
        err = np.max(np.abs(f[i] - ref[i]) / np.maximum(np.abs(ref[i]), 1.0)) if f[i].size else 0.0
        assert err <= 1e-6, (w.name, err)
        assert s["tile"] == 10 | (6 << 8)


def test_pencil_round_timeout_then_clean_batch(monkeypatch):
    """A pencil that never publishes its faces (the test hook) makes its
    downwind pencils' bounded waits give up: PDFS_ERR_TIMEOUT, and the next
    batch is bit-exact."""
    ws = [W.random_spheres(64, 48, 40, 1.0, 1.0, 1.0, 3, 2.0, 9.0, seed=s) for s in (1, 2, 3)]
    monkeypatch.setenv("PDFS_TEST_POISON_COLUMN", "0")
    monkeypatch.setenv("PDFS_WAIT_MS", "200")
    fields = [w.field.copy() for w in ws]
    with pytest.raises(api.PdfsError) as ei:
        api.solve_batch(fields, [(1.0, 1.0, 1.0)] * 3, frozen=[w.frozen for w in ws], freeze=L.FREEZE_MASK,
                        tol=0.0)
    assert ei.value.status == L.PDFS_ERR_TIMEOUT
    monkeypatch.delenv("PDFS_TEST_POISON_COLUMN")
    monkeypatch.delenv("PDFS_WAIT_MS")
    fields = [w.field.copy() for w in ws]
    api.solve_batch(fields, [(1.0, 1.0, 1.0)] * 3, frozen=[w.frozen for w in ws], freeze=L.FREEZE_MASK, tol=0.0)
    for w, f in zip(ws, fields):
        ref = w.field.copy()
        O.solve(ref, (1.0, 1.0, 1.0), tol=0.0, frozen=w.frozen, threads=4)
        assert f.tobytes() == ref.tobytes()
