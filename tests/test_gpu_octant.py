"""Octant masks of the polish's first cycle (k_octant_mask, k_octant_union in
sched.cu, read through pdfs_ctx_orderings): per 8^3 block, the orderings
that matter to it, computed from the FP32 working field.  Checked bit for bit
against a numpy restatement of the rule in the same FP32 arithmetic, on
ragged grids with both spacing kinds and frozen nodes, and through the
scheduled polish solve itself (same answer as the unscheduled one)."""
import numpy as np
import pytest

from oracle import oracle as O
from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SLACK = np.float32(0.25)  # kOctSlack


def signs(sn):
    """Sweep directions of ordering sn (+1 ascending), makeSweepInfo's table."""
    desc = -1 if sn in (2, 5, 7, 8) else 1
    return ((-1 if sn in (4, 8) else 1) * desc, (-1 if sn in (2, 6) else 1) * desc, (-1 if sn in (3, 7) else 1) * desc)


def orderings_ref(u32, frozen, spacing, widen=True):
    """u32: the FP32 field in the reference layout (nz+2, ny+2, nx+2)."""
    u = np.abs(u32.astype(np.float32))
    c = u[1:-1, 1:-1, 1:-1]
    nz, ny, nx = c.shape

    def axis(lo, hi, h):
        m = np.minimum(lo, hi)
        tie = np.float32(SLACK * np.float32(h))
        both = ~(m < c) | (np.abs(lo - hi) <= tie)
        return np.where(both, 3, np.where(lo < hi, 1, 2)).astype(np.uint8)

    ax = axis(u[1:-1, 1:-1, :-2], u[1:-1, 1:-1, 2:], spacing[0])
    ay = axis(u[1:-1, :-2, 1:-1], u[1:-1, 2:, 1:-1], spacing[1])
    az = axis(u[:-2, 1:-1, 1:-1], u[2:, 1:-1, 1:-1], spacing[2])
    ok = np.isfinite(c)
    if frozen is not None:
        ok &= frozen[1:-1, 1:-1, 1:-1] == 0
    bits = np.zeros(c.shape, dtype=np.uint8)
    for sn in range(1, 9):
        sx, sy, sz = signs(sn)
        m = ((ax & (1 if sx > 0 else 2)) > 0) & ((ay & (1 if sy > 0 else 2)) > 0) & ((az & (1 if sz > 0 else 2)) > 0)
        bits |= (m & ok).astype(np.uint8) << (sn - 1)
    nbz, nby, nbx = (nz + 7) // 8, (ny + 7) // 8, (nx + 7) // 8
    pad = np.zeros((nbz * 8, nby * 8, nbx * 8), dtype=np.uint8)
    pad[:nz, :ny, :nx] = bits
    blk = np.bitwise_or.reduce(pad.reshape(nbz, 8, nby, 8, nbx, 8), axis=(1, 3, 5))
    if not widen:
        return blk
    # ordering sn also where it holds in the face neighbour sn sweeps into the block from
    up = [np.uint8(sum(1 << (sn - 1) for sn in range(1, 9) if signs(sn)[a] > 0)) for a in range(3)]
    out = blk.copy()
    out[:, :, 1:] |= blk[:, :, :-1] & up[0]
    out[:, :, :-1] |= blk[:, :, 1:] & ~up[0]
    out[:, 1:] |= blk[:, :-1] & up[1]
    out[:, :-1] |= blk[:, 1:] & ~up[1]
    out[1:] |= blk[:-1] & up[2]
    out[:-1] |= blk[1:] & ~up[2]
    return out


@pytest.mark.parametrize("aniso", [False, True])
@pytest.mark.parametrize("shape", [(1, 1, 1), (9, 17, 8), (33, 40, 7), (65, 31, 47), (70, 64, 40)])
def test_orderings_equal_numpy_rule(shape, aniso):
    sp = (0.7, 1.0, 0.5) if aniso else (1.0, 1.0, 1.0)
    w = W.random_spheres(*shape, *sp, 4, 1.5, 8.0, seed=sum(shape))
    with api.Context(w.nx, w.ny, w.nz, sp, freeze=L.FREEZE_MASK, precision=L.PREC_FP32) as c:
        c.load(w.field, w.frozen)
        c.run()
        f = np.empty_like(w.field)
        c.store(f)
        got = c.orderings()
    want = orderings_ref(f.astype(np.float32), w.frozen, sp)
    assert got.shape == want.shape
    assert np.array_equal(got, want), int((got != want).sum())


def test_orderings_need_an_fp32_field():
    w = W.random_spheres(20, 20, 20, 1.0, 1.0, 1.0, 2, 2.0, 5.0, seed=3)
    with api.Context(w.nx, w.ny, w.nz, (1.0, 1.0, 1.0), precision=L.PREC_FP64) as c:
        c.load(w.field)
        c.run()
        with pytest.raises(api.PdfsError):
            c.orderings()


def test_scheduled_polish_same_answer():
    """The octant-masked first polish cycle then full sweeps to the tolerance:
    the answer is the unscheduled polish's to within the FP32-pair rounding,
    and both are within 1e-6 of the oracle."""
    w = W.random_spheres(128, 112, 96, 1.0, 1.0, 1.0, 10, 3.0, 20.0, seed=44)
    sp = (w.dx, w.dy, w.dz)
    kw = dict(frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-5)
    a, b = w.field.copy(), w.field.copy()
    sa = api.solve(a, sp, scheduler=L.SCHED_LEARNED, **kw)
    api.solve(b, sp, **kw)
    ref = w.field.copy()
    O.solve(ref, sp, tol=1e-12, frozen=w.frozen, threads=8)
    i = (slice(1, -1),) * 3
    for x in (a, b):
        assert float(np.max(np.abs(x[i] - ref[i]) / np.maximum(np.abs(ref[i]), 1.0))) <= 1e-6
    assert sa["masked_sweeps_fp64"] == 8 and sa["updates_masked_fp64"] < 8 * w.interior


@pytest.mark.parametrize("aniso", [False, True])
def test_octant_round_equals_sequential_masked_sweeps(aniso):
    """The polish's first cycle as one launch (16 x 16 x 16 bricks, the
    octant round: a brick of sweep j starts once it and its face neighbours
    finished their latest earlier sweep) against the same 8 masked sweeps
    run one launch each (16 x 16 x 32 bricks, which have no round): the
    same bits, the same sweep counts."""
    sp = (0.8, 1.0, 0.6) if aniso else (1.0, 1.0, 1.0)
    w = W.random_spheres(112, 96, 120, *sp, 12, 3.0, 18.0, seed=45)
    kw = dict(frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-5,
              scheduler=L.SCHED_LEARNED)
    a, b = w.field.copy(), w.field.copy()
    sa = api.solve(a, sp, tile=10 | (6 << 8), **kw)
    sb = api.solve(b, sp, tile=10 | (7 << 8), **kw)
    assert (sa["sweeps_fp32"], sa["sweeps_fp64"]) == (sb["sweeps_fp32"], sb["sweeps_fp64"])
    assert sa["masked_sweeps_fp64"] == sb["masked_sweeps_fp64"] == 8
    assert a.tobytes() == b.tobytes()


def test_fp32_octant_rounds_equal_sweep_by_sweep():
    """PDFS_SCHED_OCTANT on an FP32 solve: a full first cycle, then cycles as
    one-launch octant rounds (16 x 16 x 32 bricks) until a round's last two
    sweeps change by at most 16 x 4e-6, then full sweeps to the tolerance.
    Replayed here sweep by sweep through pdfs_ctx_sweep with the masks of
    pdfs_ctx_orderings: the same bits."""
    w = W.random_spheres(96, 80, 112, 1.0, 1.0, 1.0, 12, 3.0, 16.0, seed=46)
    sp = (w.dx, w.dy, w.dz)
    a = w.field.copy()
    st = api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32, scheduler=L.SCHED_OCTANT)
    assert st["masked_sweeps_fp32"] >= 8
    with api.Context(w.nx, w.ny, w.nz, sp, freeze=L.FREEZE_MASK, precision=L.PREC_FP32) as c:
        c.load(w.field, w.frozen)
        s = 0
        for _ in range(8):
            c.sweep(s % 8 + 1)
            s += 1
        for _ in range(3):
            bits = c.orderings()
            ch = []
            for _ in range(8):
                sn = s % 8 + 1
                ch.append(c.sweep(sn, active=((bits >> (sn - 1)) & 1).astype(np.uint8)))
                s += 1
            if max(ch[6], ch[7]) <= 16 * np.float32(4e-6):
                break
        while True:
            chg = c.sweep(s % 8 + 1)
            s += 1
            if chg <= np.float32(4e-6):
                break
        b = np.empty_like(w.field)
        c.store(b)
    assert st["sweeps_fp32"] == s
    assert a.tobytes() == b.tobytes()


def test_octant_scheduler_headline_accuracy():
    """The FP32 + pair polish solve under PDFS_SCHED_OCTANT: within 1e-6 of the
    oracle's FP64 fixed point, fewer node updates than the unscheduled solve."""
    w = W.random_spheres(128, 112, 96, 1.0, 1.0, 1.0, 10, 3.0, 20.0, seed=44)
    sp = (w.dx, w.dy, w.dz)
    kw = dict(frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-5)
    a, b = w.field.copy(), w.field.copy()
    sa = api.solve(a, sp, scheduler=L.SCHED_OCTANT, **kw)
    sb = api.solve(b, sp, **kw)
    ref = w.field.copy()
    O.solve(ref, sp, tol=1e-12, frozen=w.frozen, threads=8)
    i = (slice(1, -1),) * 3
    err = float(np.max(np.abs(a[i] - ref[i]) / np.maximum(np.abs(ref[i]), 1.0)))
    assert err <= 1e-6, err
    assert sa["masked_sweeps_fp32"] >= 8 and sa["masked_sweeps_fp64"] == 8
    assert sa["voxel_updates"] < sb["voxel_updates"]


@pytest.mark.parametrize("shape", [(12, 200, 30), (150, 9, 40), (40, 36, 300), (16, 16, 16), (5, 3, 7)])
def test_octant_rounds_on_thin_grids(shape):
    """Grids one brick thick (or one brick in all) along some axis: the
    rounds' ticket keys and waits degenerate there (one level per axis), and
    the solve still ends on a certified fixed point within 1e-6 of the
    oracle's, with the octant rounds run (FP32 first cycle, FP32 round, polish
    round) and every wait ending."""
    nx, ny, nz = shape
    w = W.random_spheres(nx, ny, nz, 1.0, 1.0, 1.0, 3, 2.0, 9.0, seed=sum(shape) + 5)
    sp = (w.dx, w.dy, w.dz)
    a = w.field.copy()
    st = api.solve(a, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64,
                   arith=L.ARITH_PAIR, tol=1e-5, scheduler=L.SCHED_OCTANT)
    ref = w.field.copy()
    O.solve(ref, sp, tol=1e-12, frozen=w.frozen, threads=8)
    i = (slice(1, -1),) * 3
    err = float(np.max(np.abs(a[i] - ref[i]) / np.maximum(np.abs(ref[i]), 1.0)))
    assert err <= 1e-6, err
    assert st["masked_sweeps_fp64"] == 8 and st["sweeps_fp32"] >= 8

