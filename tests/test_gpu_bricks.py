"""The brick sweep kernel (16 x 16 x BZ bricks held in shared memory, swept
level by level, ordered across bricks by completion flags) through the C
ABI.  Its update order is another topological order of each ordering's
dependency DAG, so FP64 reference arithmetic must match the oracle bit for
bit, and every arithmetic must match the column kernels bit for bit; block
masks must equal freezing the inactive blocks' nodes; a brick that never
publishes must end in the bounded-wait error."""
import numpy as np
import pytest

from oracle import oracle as O
from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W
from test_gpu_blocks import block_max, node_mask, patterned_mask

pytestmark = pytest.mark.gpu

B64 = 5 << 8     # FP64 bricks, 16 x 16 x 16
B32 = (8, 9)     # FP32 bricks, 16 x 16 x 16 and 16 x 16 x 32
P64 = 6 << 8     # FP64 pencils, 16 x 16 along z (block-masked sweeps on bricks)
P32 = 10         # FP32 pencils


def same(a, b):
    return a.tobytes() == b.tobytes()


def inner(a):
    return a[1:-1, 1:-1, 1:-1]


# ragged in every axis, bricks of one node, single rows, exact multiples
SHAPES = [(1, 1, 1), (2, 3, 5), (16, 16, 16), (17, 16, 15), (1, 40, 1), (70, 1, 1), (1, 1, 33), (33, 17, 9),
          (65, 31, 47), (48, 50, 35)]


@pytest.mark.parametrize("tile", [B64, P64])
@pytest.mark.parametrize("shape", SHAPES)
def test_bricks_bit_exact_odd_shapes(shape, tile):
    nx, ny, nz = shape
    f = W.random_field(nx, ny, nz, seed=nx * 5 + ny * 11 + nz, frac_known=0.1)
    for sp in [(1.0, 1.0, 1.0), (0.7, 1.3, 0.4)]:
        a, b = f.copy(), f.copy()
        s, _ = O.solve(b, sp, tol=0.0, threads=8)
        st = api.solve(a, sp, tol=0.0, tile=tile)
        assert same(a, b)
        assert st["sweeps_fp64"] == s
        assert st["tile"] >> 8 == tile >> 8


@pytest.mark.parametrize("tile", [B64, P64])
@pytest.mark.parametrize("sn", range(1, 9))
def test_brick_orderings_multisphere_frozen(sn, tile):
    """One sweep of each ordering on a frozen-mask multi-sphere grid whose
    sizes are not brick or pencil multiples."""
    w = W.random_spheres(75, 41, 38, 1.0, 1.0, 0.5, 6, 3.0, 12.0, seed=40 + sn)
    sp = (w.dx, w.dy, w.dz)
    a, b = w.field.copy(), w.field.copy()
    api.sweep(a, sp, sn, frozen=w.frozen, freeze=L.FREEZE_MASK, tile=tile)
    O.sweep(b, sp, sn, frozen=w.frozen)
    assert same(a, b)


@pytest.mark.parametrize("tall", [False, True])
def test_pencil_fp32_equals_column_fp32(tall):
    """FP32 solves on pencils and on 32 x 8 columns agree bit for bit (a
    tall grid recycles every ring slot many times)."""
    nz = 300 if tall else 40
    w = W.random_spheres(50, 37, nz, 1.0, 1.0, 1.0, 6, 3.0, 12.0, seed=17)
    sp = (w.dx, w.dy, w.dz)
    out = []
    for t in (P32, 4):
        a = w.field.copy()
        st = api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32, tile=t)
        out.append((a, st["sweeps_fp32"]))
    assert same(out[0][0], out[1][0]) and out[0][1] == out[1][1]


@pytest.mark.parametrize("arith", [L.ARITH_MIXED, L.ARITH_PAIR])
def test_pencil_polish_equals_bricks(arith):
    """The polish on pencils and on bricks: the same topological order
    class, so the same bits."""
    w = W.random_spheres(70, 66, 90, 1.0, 1.0, 0.5, 8, 3.0, 14.0, seed=78)
    sp = (w.dx, w.dy, w.dz)
    out = []
    for tile in (P32 | P64, 9 | B64):
        a = w.field.copy()
        api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=arith,
                  tol=1e-6 * min(sp), max_sweeps=200, tile=tile)
        out.append(a)
    assert same(out[0], out[1])


def test_pencil_bounded_wait_times_out_cleanly(monkeypatch):
    w = W.random_spheres(64, 64, 48, 1.0, 1.0, 1.0, 4, 3.0, 10.0, seed=2)
    sp = (w.dx, w.dy, w.dz)
    monkeypatch.setenv("PDFS_TEST_POISON_COLUMN", "0")
    a = w.field.copy()
    with pytest.raises(api.PdfsError) as ei:
        api.solve(a, sp, tol=0.0, wait_ms=200, tile=P64)
    assert ei.value.status == L.PDFS_ERR_TIMEOUT
    monkeypatch.delenv("PDFS_TEST_POISON_COLUMN")
    a, b = w.field.copy(), w.field.copy()
    api.solve(a, sp, tol=0.0, tile=P64)
    O.solve(b, sp, tol=0.0, threads=8)
    assert same(a, b)


@pytest.mark.parametrize("sched", [L.SCHED_CHANGE, L.SCHED_LEARNED])
def test_pencil_tiles_with_schedulers(sched):
    """Scheduled solves on pencil tiles: full sweeps record block changes and
    masked sweeps skip blocks, both on bricks; the fixed point is the plain one."""
    w = W.random_spheres(96, 80, 72, 1.0, 1.0, 1.0, 6, 3.0, 16.0, seed=5)
    sp = (w.dx, w.dy, w.dz)
    a, b = w.field.copy(), w.field.copy()
    st = api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, arith=L.ARITH_FAST, tol=0.0,
                   scheduler=sched, tile=P64)
    O.solve(b, sp, tol=0.0, frozen=w.frozen, threads=8)
    h = min(sp)
    err = float(np.max(np.abs(inner(a) - inner(b)) / np.maximum(np.abs(inner(b)), h)))
    assert err <= 1e-13, err
    assert st["blocks_skipped"] > 0


@pytest.fixture(scope="module", params=[37, 150])
def grid(request):
    return W.random_spheres(70, 45, request.param, 1.0, 1.0, 1.0, 5, 3.0, 12.0, seed=23)


def ctx_for(w, **kw):
    c = api.Context(w.nx, w.ny, w.nz, (w.dx, w.dy, w.dz), freeze=L.FREEZE_MASK, **kw)
    c.load(w.field, w.frozen)
    return c


@pytest.mark.parametrize("sn", range(1, 9))
def test_brick_masked_sweep_equals_frozen_fp64(grid, sn):
    w = grid
    rng = np.random.default_rng(500 + sn)
    with ctx_for(w, precision=L.PREC_FP64, arith=L.ARITH_REFERENCE, tile=B64) as c:
        nb = c.blocks()[::-1]
        act = patterned_mask(nb, rng)
        bc = np.zeros(nb, np.float32)
        ch = c.sweep(sn, act, bc)
        got = np.empty_like(w.field)
        c.store(got)
    exp = w.field.copy()
    O.sweep(exp, (w.dx, w.dy, w.dz), sn, frozen=w.frozen | node_mask(act, w.field.shape))
    assert same(got, exp)
    diff = np.abs(exp - w.field)
    assert ch == float(inner(diff).max())
    assert np.array_equal(bc, block_max(diff, nb))
    assert not bc[act == 0].any()


def test_brick_masked_chain_and_empty(grid):
    """Eight masked orderings in a row on one context (the brick flags carry
    increasing epochs across launches), then an all-inactive sweep."""
    w = grid
    rng = np.random.default_rng(9)
    exp = w.field.copy()
    with ctx_for(w, precision=L.PREC_FP64, arith=L.ARITH_REFERENCE, tile=B64) as c:
        nb = c.blocks()[::-1]
        for sn in range(1, 9):
            act = patterned_mask(nb, rng)
            c.sweep(sn, act)
            O.sweep(exp, (w.dx, w.dy, w.dz), sn, frozen=w.frozen | node_mask(act, w.field.shape))
        assert c.sweep(3, np.zeros(nb, np.uint8)) == 0.0
        got = np.empty_like(w.field)
        c.store(got)
    assert same(got, exp)


@pytest.mark.parametrize("tile", B32)
@pytest.mark.parametrize("sn", [1, 6])
def test_brick_fp32_equals_column_fp32(grid, tile, sn):
    """FP32 sweeps: the bricks and the 32 x 8 columns run the same local
    solver on the same inputs, so results agree bit for bit, masked too."""
    w = grid
    outs = []
    for t in (tile, 4):
        with ctx_for(w, precision=L.PREC_FP32, tile=t) as c:
            nb = c.blocks()[::-1]
            act = patterned_mask(nb, np.random.default_rng(600 + sn))
            for k in range(3):
                c.sweep((sn + k - 1) % 8 + 1, act if k == 1 else None)
            got = np.empty_like(w.field)
            c.store(got)
            outs.append(got)
    assert same(outs[0], outs[1])


@pytest.mark.parametrize("iso", [True, False])
def test_brick_mixed_polish_equals_column(iso):
    """FP32 bulk + mixed FP64 polish on bricks against the column kernels
    (bit for bit) and against the FP64 oracle (1e-6 relative)."""
    sz = 0.5 if not iso else 1.0
    w = W.random_spheres(80, 66, 52, 1.0, 1.0, sz, 8, 3.0, 14.0, seed=77)
    sp = (w.dx, w.dy, w.dz)
    res = []
    for tile in (8 | (5 << 8), 4 | (4 << 8)):
        a = w.field.copy()
        api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64,
                  arith=L.ARITH_MIXED, tol=1e-6 * min(sp), max_sweeps=200, tile=tile)
        res.append(a)
    assert same(res[0], res[1])
    b = w.field.copy()
    O.solve(b, sp, tol=0.0, frozen=w.frozen, threads=8)
    h = min(sp)
    err = float(np.max(np.abs(inner(res[0]) - inner(b)) / np.maximum(np.abs(inner(b)), h)))
    assert err <= 1e-6, err


@pytest.mark.parametrize("sched", [L.SCHED_CHANGE, L.SCHED_LEARNED])
def test_brick_schedulers_same_fixed_point(sched):
    """Scheduled solves skip inactive bricks; the fixed point is the plain one."""
    w = W.random_spheres(96, 80, 72, 1.0, 1.0, 1.0, 6, 3.0, 16.0, seed=5)
    sp = (w.dx, w.dy, w.dz)
    a, b = w.field.copy(), w.field.copy()
    st = api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, arith=L.ARITH_FAST, tol=0.0,
                   scheduler=sched, tile=B64)
    O.solve(b, sp, tol=0.0, frozen=w.frozen, threads=8)
    h = min(sp)
    err = float(np.max(np.abs(inner(a) - inner(b)) / np.maximum(np.abs(inner(b)), h)))
    assert err <= 1e-13, err
    assert st["blocks_skipped"] > 0


def test_brick_bounded_wait_times_out_cleanly(monkeypatch):
    """A brick that never publishes (test hook) makes its downwind bricks give
    up after the wait bound: PDFS_ERR_TIMEOUT, and the device stays usable."""
    w = W.random_spheres(64, 64, 48, 1.0, 1.0, 1.0, 4, 3.0, 10.0, seed=2)
    sp = (w.dx, w.dy, w.dz)
    monkeypatch.setenv("PDFS_TEST_POISON_COLUMN", "0")
    a = w.field.copy()
    with pytest.raises(api.PdfsError) as ei:
        api.solve(a, sp, tol=0.0, wait_ms=200, tile=B64)
    assert ei.value.status == L.PDFS_ERR_TIMEOUT
    monkeypatch.delenv("PDFS_TEST_POISON_COLUMN")
    a, b = w.field.copy(), w.field.copy()
    api.solve(a, sp, tol=0.0, tile=B64)
    O.solve(b, sp, tol=0.0, threads=8)
    assert same(a, b)


# ---- FP32-pair arithmetic (FP64 bricks) --------------------------------------------------
def rel_err(a, b, h):
    return float(np.max(np.abs(inner(a) - inner(b)) / np.maximum(np.abs(inner(b)), h)))


@pytest.mark.parametrize("iso", [True, False])
def test_pair_polish_within_1e6(iso):
    """FP32 bulk + FP32-pair polish against the FP64 oracle; frozen nodes and
    the halo come back as the exact input."""
    sz = 1.0 if iso else 0.5
    w = W.random_spheres(90, 70, 60, 1.0, 1.0, sz, 8, 3.0, 14.0, seed=91)
    sp = (w.dx, w.dy, w.dz)
    a = w.field.copy()
    st = api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64,
                   arith=L.ARITH_PAIR, tol=1e-6 * min(sp), max_sweeps=200)
    assert (st["tile"] >> 8) in (5, 6, 7, 8, 9) and st["sweeps_fp64"] > 0  # bricks, pencils or lane columns
    b = w.field.copy()
    O.solve(b, sp, tol=0.0, frozen=w.frozen, threads=8)
    # tolerance: 1e-6 relative, as for the mixed arithmetic
    assert rel_err(a, b, min(sp)) <= 1e-6
    fz = w.frozen.astype(bool)
    assert same(a[fz], w.field[fz])
    halo = np.ones(a.shape, bool)
    halo[1:-1, 1:-1, 1:-1] = False
    assert same(a[halo], w.field[halo])


def test_pair_agrees_with_mixed():
    """Both keep an FP32 increment over a wide base; their fixed points agree
    to a few 1e-8 relative."""
    w = W.random_spheres(64, 64, 64, 1.0, 1.0, 1.0, 6, 3.0, 12.0, seed=92)
    sp = (w.dx, w.dy, w.dz)
    out = []
    for ar in (L.ARITH_PAIR, L.ARITH_MIXED):
        a = w.field.copy()
        api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=ar,
                  tol=1e-6, max_sweeps=200)
        out.append(a)
    assert rel_err(out[0], out[1], 1.0) <= 3e-7


def test_pair_fp64_precision_solve():
    """PREC_FP64 in pair arithmetic from the input (no FP32 phase)."""
    w = W.random_spheres(72, 50, 40, 1.0, 1.0, 1.0, 5, 3.0, 12.0, seed=93)
    sp = (w.dx, w.dy, w.dz)
    a, b = w.field.copy(), w.field.copy()
    api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP64, arith=L.ARITH_PAIR,
              tol=1e-6, max_sweeps=200)
    O.solve(b, sp, tol=0.0, frozen=w.frozen, threads=8)
    assert rel_err(a, b, 1.0) <= 1e-6


@pytest.mark.parametrize("sn", [3, 8])
def test_pair_masked_sweep_equals_frozen(grid, sn):
    """A block-masked pair sweep equals the same sweep with the inactive
    blocks' nodes frozen, bit for bit, and reports the same block changes."""
    w = grid
    act = patterned_mask(tuple(np.array(((w.nz + 7) // 8, (w.ny + 7) // 8, (w.nx + 7) // 8))),
                         np.random.default_rng(700 + sn))
    kw = dict(precision=L.PREC_FP64, arith=L.ARITH_PAIR)
    with ctx_for(w, **kw) as c:
        bc = np.zeros(act.shape, np.float32)
        c.sweep(sn, act, bc)
        got = np.empty_like(w.field)
        c.store(got)
    fz = (w.frozen | node_mask(act, w.field.shape)).astype(np.uint8)
    with api.Context(w.nx, w.ny, w.nz, (w.dx, w.dy, w.dz), freeze=L.FREEZE_MASK, **kw) as c2:
        c2.load(w.field, fz)
        c2.sweep(sn)
        exp = np.empty_like(w.field)
        c2.store(exp)
    assert same(got, exp)
    assert not bc[act == 0].any()


def test_pair_learned_scheduler_polish():
    w = W.random_spheres(96, 80, 72, 1.0, 1.0, 1.0, 6, 3.0, 16.0, seed=5)
    sp = (w.dx, w.dy, w.dz)
    a, b = w.field.copy(), w.field.copy()
    api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR,
              tol=1e-6, max_sweeps=200, scheduler=L.SCHED_LEARNED)
    O.solve(b, sp, tol=0.0, frozen=w.frozen, threads=8)
    assert rel_err(a, b, 1.0) <= 1e-6


@pytest.mark.parametrize("arith", [L.ARITH_MIXED, L.ARITH_PAIR])
def test_polish_binding_caps(arith):
    """Replace-update where the caps bind: 3 % of the updated nodes start from
    small finite values.  Bricks and pencils read a cap only when the new value
    is not below its block's smallest cap; the result must not depend on it
    (bricks, pencils and, for the mixed arithmetic, columns give the same bits)."""
    w = W.random_spheres(70, 60, 50, 1.0, 1.0, 1.0, 6, 3.0, 12.0, seed=81)
    f = w.field.copy()
    rng = np.random.default_rng(3)
    free = (w.frozen == 0)
    free[0, :, :] = free[-1, :, :] = False
    free[:, 0, :] = free[:, -1, :] = False
    free[:, :, 0] = free[:, :, -1] = False
    pick = free & (rng.random(f.shape) < 0.03)
    f[pick] = rng.uniform(0.0, 6.0, int(pick.sum()))
    sp = (w.dx, w.dy, w.dz)
    tiles = [9 | B64, P32 | P64] + ([4 | (4 << 8)] if arith == L.ARITH_MIXED else [])
    out = []
    for tile in tiles:
        a = f.copy()
        api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=arith,
                  tol=1e-6, max_sweeps=200, tile=tile)
        out.append(a)
    for o in out[1:]:
        assert same(out[0], o)
    b = f.copy()
    O.solve(b, sp, tol=0.0, frozen=w.frozen, threads=8)
    assert rel_err(out[0], b, 1.0) <= 1e-6

