"""Block-masked sweeps (pdfs_ctx_sweep with an active-block mask) through the
C ABI.  Skipping a block must be exactly the same as freezing its nodes: the
kernel skips whole z ranges of a column and copies the faces of the skipped
part from the field, so these tests check that the copies and the shortened
step range leave no trace.  FP64 reference arithmetic is compared bit for
bit with the oracle sweeping with the inactive blocks' nodes frozen."""
import numpy as np
import pytest

from oracle import oracle as O
from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def node_mask(active, shape):
    """(nbz, nby, nbx) block flags -> reference-layout uint8 mask of the
    nodes in inactive blocks."""
    Z, Y, X = shape
    a = np.repeat(np.repeat(np.repeat(active, 8, 0), 8, 1), 8, 2)[:Z - 2, :Y - 2, :X - 2]
    out = np.zeros(shape, np.uint8)
    out[1:-1, 1:-1, 1:-1] = (a == 0)
    return out


def block_max(diff, nb):
    """Per-block max of |diff| over interior nodes, as float32 (nbz, nby, nbx)."""
    nbz, nby, nbx = nb
    d = np.zeros((nbz * 8, nby * 8, nbx * 8))
    i = diff[1:-1, 1:-1, 1:-1]
    d[:i.shape[0], :i.shape[1], :i.shape[2]] = i
    return d.reshape(nbz, 8, nby, 8, nbx, 8).max(axis=(1, 3, 5)).astype(np.float32)


def patterned_mask(nb, rng):
    """Random block flags with whole inactive columns, single active z
    ranges and isolated holes, so every path of the range logic runs."""
    nbz, nby, nbx = nb
    a = (rng.random(nb) < 0.6).astype(np.uint8)
    for _ in range(3):  # whole (x, y) columns off
        a[:, rng.integers(nby), rng.integers(nbx)] = 0
    for _ in range(3):  # one z range on, the rest of the column off
        by, bx = rng.integers(nby), rng.integers(nbx)
        lo = rng.integers(nbz)
        hi = rng.integers(lo, nbz) + 1
        a[:, by, bx] = 0
        a[lo:hi, by, bx] = 1
    return a


@pytest.fixture(scope="module", params=[37, 150])
def grid(request):
    """A short grid (all planes fit the kernel's plane ring) and a tall one
    (ring slots are reused, so a column that starts late must still hand
    back the slots of the planes below its range)."""
    return W.random_spheres(70, 45, request.param, 1.0, 1.0, 1.0, 5, 3.0, 12.0, seed=23)


def ctx_for(w, **kw):
    c = api.Context(w.nx, w.ny, w.nz, (w.dx, w.dy, w.dz), freeze=L.FREEZE_MASK, **kw)
    c.load(w.field, w.frozen)
    return c


@pytest.mark.parametrize("sn", range(1, 9))
def test_masked_sweep_equals_frozen_sweep_fp64(grid, sn):
    w = grid
    rng = np.random.default_rng(100 + sn)
    with ctx_for(w, precision=L.PREC_FP64, arith=L.ARITH_REFERENCE) as c:
        nb = c.blocks()[::-1]
        act = patterned_mask(nb, rng)
        bc = np.zeros(nb, np.float32)
        ch = c.sweep(sn, act, bc)
        got = np.empty_like(w.field)
        c.store(got)
    exp = w.field.copy()
    O.sweep(exp, (w.dx, w.dy, w.dz), sn, frozen=w.frozen | node_mask(act, w.field.shape))
    assert got.tobytes() == exp.tobytes()  # bit-exact
    diff = np.abs(exp - w.field)
    assert ch == float(diff[1:-1, 1:-1, 1:-1].max())
    assert np.array_equal(bc, block_max(diff, nb))
    assert not bc[act == 0].any()


def test_masked_sweeps_chain_fp64(grid):
    """Eight orderings in a row on one context, a new mask each time."""
    w = grid
    rng = np.random.default_rng(7)
    exp = w.field.copy()
    with ctx_for(w, precision=L.PREC_FP64, arith=L.ARITH_REFERENCE) as c:
        nb = c.blocks()[::-1]
        for sn in range(1, 9):
            act = patterned_mask(nb, rng)
            c.sweep(sn, act)
            O.sweep(exp, (w.dx, w.dy, w.dz), sn, frozen=w.frozen | node_mask(act, w.field.shape))
        got = np.empty_like(w.field)
        c.store(got)
    assert got.tobytes() == exp.tobytes()


def test_all_and_no_blocks(grid):
    w = grid
    with ctx_for(w, precision=L.PREC_FP64, arith=L.ARITH_REFERENCE) as c:
        nb = c.blocks()[::-1]
        assert c.sweep(4, np.zeros(nb, np.uint8)) == 0.0
        got = np.empty_like(w.field)
        c.store(got)
        assert got.tobytes() == w.field.tobytes()
        c.sweep(4, np.ones(nb, np.uint8))
        c.store(got)
    exp = w.field.copy()
    api.sweep(exp, (w.dx, w.dy, w.dz), 4, frozen=w.frozen, freeze=L.FREEZE_MASK)
    assert got.tobytes() == exp.tobytes()


@pytest.mark.parametrize("sn", [1, 5, 8])
def test_masked_sweep_equals_frozen_sweep_fp32(grid, sn):
    """FP32: the masked sweep against the same kernel with the inactive
    blocks frozen instead (bit-exact); frozen nodes come back as the exact
    FP64 input, skipped ones as their FP32 value."""
    w = grid
    rng = np.random.default_rng(200 + sn)
    with ctx_for(w, precision=L.PREC_FP32) as c:
        nb = c.blocks()[::-1]
        act = patterned_mask(nb, rng)
        c.sweep(sn, act)
        got = np.empty_like(w.field)
        c.store(got)
    off = node_mask(act, w.field.shape)
    fz = (w.frozen | off).astype(np.uint8)
    with api.Context(w.nx, w.ny, w.nz, (w.dx, w.dy, w.dz), freeze=L.FREEZE_MASK, precision=L.PREC_FP32) as c2:
        c2.load(w.field, fz)
        c2.sweep(sn)
        exp = np.empty_like(w.field)
        c2.store(exp)
    keep = (off == 0)
    assert got[keep].tobytes() == exp[keep].tobytes()
    sk = (off == 1) & (w.frozen == 0)
    assert got[sk].tobytes() == w.field[sk].astype(np.float32).astype(np.float64).tobytes()


@pytest.mark.parametrize("sn", [2, 7])
def test_masked_sweep_mixed_tile6(grid, sn):
    """The 32 x 6 FP64 tile (mixed arithmetic): its frozen-mask words are
    loaded from a 16-byte aligned start and indexed from the column's
    offset; a masked sweep must equal the same kernel with the inactive
    blocks frozen, bit for bit."""
    w = grid
    rng = np.random.default_rng(300 + sn)
    kw = dict(precision=L.PREC_FP64, arith=L.ARITH_MIXED, tile=4 << 8)
    with ctx_for(w, **kw) as c:
        nb = c.blocks()[::-1]
        act = patterned_mask(nb, rng)
        c.sweep(sn, act)
        got = np.empty_like(w.field)
        c.store(got)
    fz = (w.frozen | node_mask(act, w.field.shape)).astype(np.uint8)
    with api.Context(w.nx, w.ny, w.nz, (w.dx, w.dy, w.dz), freeze=L.FREEZE_MASK, **kw) as c2:
        c2.load(w.field, fz)
        c2.sweep(sn)
        exp = np.empty_like(w.field)
        c2.store(exp)
    assert got.tobytes() == exp.tobytes()
