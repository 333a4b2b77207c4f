"""The octant round's ticket order (k_oct_tickets, k_oct_plan, k_oct_merge in
tile3d.cu), restated in Python and checked on the CPU: for random masks,
grids of bricks and first orderings the merged list is a permutation of the
round's tickets, and every brick of sweep j comes after its active upwind
bricks of sweep j and after itself and its six face neighbours in their
latest earlier active sweep -- the waits of the round kernel, so every wait
is on a smaller ticket (the round cannot deadlock)."""
import random

import pytest


def signs(sn):
    """Sweep directions of ordering sn (the reference's makeSweepInfo table)."""
    desc = -1 if sn in (2, 5, 7, 8) else 1
    return ((-1 if sn in (4, 8) else 1) * desc, (-1 if sn in (2, 6) else 1) * desc, (-1 if sn in (3, 7) else 1) * desc)


def brick_order(ntx, nty, ntz):
    """Local brick ids by level li + lj + lk (brick_order in tile3d.cu)."""
    o = []
    for lev in range(ntx + nty + ntz - 2):
        for z in range(ntz):
            for y in range(nty):
                for x in range(ntx):
                    if x + y + z == lev:
                        o.append((z * nty + y) * ntx + x)
    return o


def oriented(t, s, n):
    """Global brick t <-> its local id in a sweep with directions s (an involution)."""
    ntx, nty, ntz = n
    x, y, z = t % ntx, (t // ntx) % nty, t // (ntx * nty)
    a = x if s[0] > 0 else ntx - 1 - x
    b = y if s[1] > 0 else nty - 1 - y
    c = z if s[2] > 0 else ntz - 1 - z
    return (c * nty + b) * ntx + a


def merged_tickets(n, first, tbits, full=0):
    ntx, nty, ntz = n
    nb, WL = ntx * nty * ntz, ntx + nty + ntz - 2
    torder = brick_order(*n)
    sg = [signs((first + j) % 8 + 1) for j in range(8)]
    lists = []
    for j in range(8):  # k_oct_tickets
        bit = 1 << ((first + j) % 8)
        lists.append([lt for lt in torder if (full >> j) & 1 or tbits[oriented(lt, sg[j], n)] & bit])
    T = [0] * 8  # the host's key offsets (launch_octant_round)
    ext = (ntx - 1, nty - 1, ntz - 1)
    for j in range(8):
        for q in range(j):
            T[j] = max(T[j], T[q] + 2 + sum(ext[a] for a in range(3) if sg[q][a] != sg[j][a]))

    def level(lt):
        return lt % ntx + (lt // ntx) % nty + lt // (ntx * nty)

    start = [[0] * (WL + 1) for _ in range(8)]  # k_oct_plan
    for j in range(8):
        for w in range(WL + 1):
            lo, hi = 0, len(lists[j])
            while lo < hi:
                mid = (lo + hi) // 2
                if level(lists[j][mid]) < w:
                    lo = mid + 1
                else:
                    hi = mid
            start[j][w] = lo
    base = [[None] * WL for _ in range(8)]
    pos = 0
    for c in range((T[7] + WL) * 8):
        j, w = c % 8, c // 8 - T[c % 8]
        if 0 <= w < WL:
            base[j][w] = pos
            pos += start[j][w + 1] - start[j][w]
    assert pos == sum(len(x) for x in lists)
    merged = [None] * pos  # k_oct_merge
    for j in range(8):
        for i, lt in enumerate(lists[j]):
            w = level(lt)
            p = base[j][w] + i - start[j][w]
            assert merged[p] is None
            merged[p] = (j, lt)
    return merged, sg


@pytest.mark.parametrize("n", [(1, 1, 1), (2, 1, 1), (3, 4, 2), (5, 5, 5), (7, 3, 6), (6, 6, 3)])
@pytest.mark.parametrize("first", [0, 3, 6])
@pytest.mark.parametrize("density", [0.3, 0.7, 1.0])
def test_every_wait_is_on_an_earlier_ticket(n, first, density):
    rng = random.Random(hash((n, first, density)) & 0xffff)
    ntx, nty, ntz = n
    nb = ntx * nty * ntz
    tbits = [sum(1 << k for k in range(8) if rng.random() < density) for _ in range(nb)]
    full = 0xff if density == 1.0 and first == 0 else 0
    merged, sg = merged_tickets(n, first, tbits, full)
    pos = {e: i for i, e in enumerate(merged)}
    assert len(pos) == len(merged)

    def active(j, t):
        return (full >> j) & 1 or tbits[t] & (1 << ((first + j) % 8))

    for tk, (j, lt) in enumerate(merged):
        s = sg[j]
        tile = oriented(lt, s, n)
        bi, bj, bk = tile % ntx, (tile // ntx) % nty, tile // (ntx * nty)
        li, lj, lk = lt % ntx, (lt // ntx) % nty, lt // (ntx * nty)
        faces = [tile]
        if bi > 0: faces.append(tile - 1)
        if bi < ntx - 1: faces.append(tile + 1)
        if bj > 0: faces.append(tile - ntx)
        if bj < nty - 1: faces.append(tile + ntx)
        if bk > 0: faces.append(tile - ntx * nty)
        if bk < ntz - 1: faces.append(tile + ntx * nty)
        for t in faces:  # the latest earlier sweep in which t is active
            for j2 in range(j - 1, -1, -1):
                if active(j2, t):
                    assert pos[(j2, oriented(t, sg[j2], n))] < tk
                    break
        ups = []
        if li > 0: ups.append(tile - s[0])
        if lj > 0: ups.append(tile - s[1] * ntx)
        if lk > 0: ups.append(tile - s[2] * ntx * nty)
        for t in ups:
            if active(j, t):
                assert pos[(j, oriented(t, s, n))] < tk


def diag_column(tid, bx=16, by=16):
    """diag_column in tile3d.cuh: thread tid's brick column when the bx x by
    columns are listed by diagonal lx + ly, then by ly."""
    base = 0
    for d in range(bx + by - 1):
        lo, hi = max(0, d - (bx - 1)), min(d, by - 1)
        if tid < base + hi - lo + 1:
            ly = lo + tid - base
            return d - ly, ly
        base += hi - lo + 1
    return 0, 0


@pytest.mark.parametrize("bz", [16, 32])
def test_diagonal_columns(bz):
    """Every column of a 16 x 16 brick has one thread, and a warp's 32 columns
    span at most 8 diagonals: its level body runs on bz + 2 .. bz + 7 levels
    (158 warp-level bodies per 16^3 brick, 286 per 16 x 16 x 32, against 256 and
    384 for warps of two rows)."""
    cols = [diag_column(t) for t in range(256)]
    assert sorted(cols) == sorted((x, y) for x in range(16) for y in range(16))
    spans = []
    for w in range(8):
        d = [x + y for x, y in cols[32 * w:32 * w + 32]]
        spans.append(max(d) - min(d))
    assert max(spans) <= 7 and min(spans) >= 2
    bodies = sum(bz + s for s in spans)
    assert bodies == {16: 158, 32: 286}[bz]
    assert bodies < 8 * (bz + 16)
