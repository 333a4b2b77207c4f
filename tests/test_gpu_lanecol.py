"""Lane-column tiles (FP32 tile 12, FP32-pair tile 9 << 8; lanecol.cuh):
every ordering is a topological order of the same dependency DAG, so their
results must equal the pencils' and bricks' bit for bit -- sweep by sweep,
including the sweep's max change, on ragged shapes, both spacing kinds, with
frozen nodes, block masks and per-block change outputs -- and their solves
must take the same number of sweeps.  FP64 reference arithmetic is pinned
to the oracle elsewhere (test_gpu_parity.py, test_gpu_configs.py); these
kernels carry the FP32 and FP32-pair arithmetic."""
import numpy as np
import pytest

from oracle import oracle as O
from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W

pytestmark = pytest.mark.gpu

LC32, LC64 = 12, 9 << 8   # lane-column tiles, 8 rows
LC32_4, LC64_4 = 13, 10 << 8  # lane-column tiles, 4 rows
P32, P64 = 10, 6 << 8     # pencils (their masked sweeps run on bricks)

SHAPES = [(1, 1, 1), (2, 3, 5), (31, 1, 1), (32, 2, 2), (33, 40, 7), (70, 1, 9), (1, 70, 6), (65, 31, 47)]


def grid(shape, aniso, seed=0):
    nx, ny, nz = shape
    sp = (0.7, 1.0, 0.5) if aniso else (1.0, 1.0, 1.0)
    k = max(1, min(6, (nx * ny * nz) // 4000 + 1))
    rmax = max(1.5, min(nx * sp[0], ny * sp[1], nz * sp[2]) / 3)
    return W.random_spheres(nx, ny, nz, *sp, k, 0.8, rmax, seed=seed)


def sweeps(w, tile, seq, **kw):
    """Runs the orderings seq on a context; returns the fields after each
    sweep and the sweeps' max changes."""
    out, ch = [], []
    with api.Context(w.nx, w.ny, w.nz, (w.dx, w.dy, w.dz), freeze=L.FREEZE_MASK, tile=tile, **kw) as c:
        c.load(w.field, w.frozen)
        for sn in seq:
            ch.append(c.sweep(sn))
            f = np.empty_like(w.field)
            c.store(f)
            out.append(f)
    return out, ch


@pytest.mark.parametrize("lc", [LC32, LC32_4])
@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("shape", SHAPES)
def test_fp32_sweeps_equal_pencils(shape, aniso, lc):
    w = grid(shape, aniso, seed=3)
    seq = [1, 2, 3, 4, 5, 6, 7, 8, 3, 6]
    a, ca = sweeps(w, lc, seq, precision=L.PREC_FP32)
    b, cb = sweeps(w, P32, seq, precision=L.PREC_FP32)
    for k in range(len(seq)):
        assert a[k].tobytes() == b[k].tobytes(), f"sweep {k} ordering {seq[k]}"
        assert ca[k] == cb[k], f"max change of sweep {k}"


@pytest.mark.parametrize("lc", [LC64, LC64_4])
@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("shape", SHAPES)
def test_pair_min_sweeps_equal_pencils(shape, aniso, lc):
    """FP32-pair min-update sweeps (an FP64-precision solve in pairs)."""
    w = grid(shape, aniso, seed=4)
    seq = [1, 2, 3, 4, 5, 6, 7, 8]
    kw = dict(precision=L.PREC_FP64, arith=L.ARITH_PAIR)
    a, ca = sweeps(w, lc, seq, **kw)
    b, cb = sweeps(w, P64, seq, **kw)
    for k in range(len(seq)):
        assert a[k].tobytes() == b[k].tobytes(), f"sweep {k} ordering {seq[k]}"
        assert ca[k] == cb[k]


@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("shape", [(33, 40, 7), (65, 31, 47), (96, 80, 72)])
def test_polish_solve_equals_pencils(shape, aniso):
    """FP32 bulk + FP32-pair polish (the headline solve): same sweeps, same bits."""
    w = grid(shape, aniso, seed=5)
    sp = (w.dx, w.dy, w.dz)
    res = []
    for tile in (LC32 | LC64, LC32_4 | LC64_4, P32 | P64):
        a = w.field.copy()
        st = api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64,
                       arith=L.ARITH_PAIR, tol=1e-5 * min(sp), tile=tile)
        res.append((a, st["sweeps_fp32"], st["sweeps_fp64"]))
    for r in res[1:]:
        assert res[0][1:] == r[1:]
        assert res[0][0].tobytes() == r[0].tobytes()
    ref = w.field.copy()
    O.solve(ref, sp, tol=1e-12, frozen=w.frozen, threads=8)
    i = (slice(1, -1),) * 3
    err = float(np.max(np.abs(res[0][0][i] - ref[i]) / np.maximum(np.abs(ref[i]), min(sp))))
    assert err <= 1e-6, err


@pytest.mark.parametrize("rows", [8, 4])
@pytest.mark.parametrize("prec", ["fp32", "pair"])
@pytest.mark.parametrize("shape", [(33, 40, 7), (65, 31, 47)])
def test_masked_sweeps_equal_pencils(shape, prec, rows):
    """Block-masked sweeps with per-block change output: the lane columns
    against the pencils' masked path (bricks), sweep by sweep, the field and
    every block's change word."""
    w = grid(shape, True, seed=6)
    kw = dict(precision=L.PREC_FP32) if prec == "fp32" else dict(precision=L.PREC_FP64, arith=L.ARITH_PAIR)
    tiles = ((LC32 if rows == 8 else LC32_4), P32) if prec == "fp32" else ((LC64 if rows == 8 else LC64_4), P64)
    rng = np.random.default_rng(7)
    outs = []
    for tile in tiles:
        with api.Context(w.nx, w.ny, w.nz, (w.dx, w.dy, w.dz), freeze=L.FREEZE_MASK, tile=tile, **kw) as c:
            c.load(w.field, w.frozen)
            nbx, nby, nbz = c.blocks()
            rng = np.random.default_rng(7)
            rec = []
            for sn in (1, 2, 5, 8, 3):
                act = (rng.random(nbx * nby * nbz) < 0.6).astype(np.uint8)
                bc = np.zeros(nbx * nby * nbz, dtype=np.float32)
                ch = c.sweep(sn, active=act, block_change=bc)
                f = np.empty_like(w.field)
                c.store(f)
                rec.append((f, bc.copy(), ch))
            outs.append(rec)
    for k, (a, b) in enumerate(zip(*outs)):
        assert a[0].tobytes() == b[0].tobytes(), f"sweep {k}"
        assert a[1].tobytes() == b[1].tobytes(), f"block changes of sweep {k}"
        assert a[2] == b[2]


@pytest.mark.parametrize("sched", [L.SCHED_CHANGE, L.SCHED_LEARNED])
def test_schedulers_on_lane_columns(sched):
    """Scheduled solves on lane columns reach the unscheduled fixed point."""
    w = grid((96, 80, 72), False, seed=8)
    sp = (w.dx, w.dy, w.dz)
    a, b = w.field.copy(), w.field.copy()
    kw = dict(frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR,
              tol=1e-5, tile=LC32 | LC64)
    api.solve(a, sp, **kw)
    api.solve(b, sp, scheduler=sched, **kw)
    i = (slice(1, -1),) * 3
    assert float(np.max(np.abs(a[i] - b[i]) / np.maximum(np.abs(a[i]), 1.0))) <= 1e-6


def test_lane_column_timeout_then_clean_solve(monkeypatch):
    """A tile that never publishes (the test hook) makes its downstream tiles'
    bounded waits give up: PDFS_ERR_TIMEOUT, and the next solve is bit-exact."""
    w = grid((65, 31, 47), False, seed=9)
    sp = (w.dx, w.dy, w.dz)
    monkeypatch.setenv("PDFS_TEST_POISON_COLUMN", "0")
    a = w.field.copy()
    with pytest.raises(api.PdfsError) as ei:
        api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32, wait_ms=200, tile=LC32)
    assert ei.value.status == L.PDFS_ERR_TIMEOUT
    monkeypatch.delenv("PDFS_TEST_POISON_COLUMN")
    a, b = w.field.copy(), w.field.copy()
    api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32, tile=LC32)
    api.solve(b, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32, tile=P32)
    assert a.tobytes() == b.tobytes()
