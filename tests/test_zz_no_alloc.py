"""pdfs_sweep_static: the allocation-free sweep for callers that cannot call
the device allocator while they run (code confined to a pool handed over by
a host application, real-time loops that must not call cudaMalloc, plugins
whose host forbids allocation after set-up).  Checked through the C ABI
against the allocating entry point pdfs_sweep on two calls in a row.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def layout(nx, ny, nz):
    g = L.Grid(nx, ny, nz, 1.0, 1.0, 1.0)
    px, ry, el, sb = (C.c_longlong() for _ in range(4))
    s = L.load().pdfs_static_layout(C.byref(g), C.byref(px), C.byref(ry), C.byref(el), C.byref(sb))
    return s, px.value, ry.value, el.value, sb.value


def to_internal(field, px, ry, elems):
    """Reference layout (z, y, x) with halo -> the static sweep's layout:
    node (x, y, z) at z*ry*px + y*px + x + 1, +inf elsewhere."""
    Z, Y, X = field.shape
    out = np.full(elems, np.inf)
    v = out.reshape(Z, ry, px)
    v[:, :Y, 1:1 + X] = field
    return out


def from_internal(buf, shape, px, ry):
    Z, Y, X = shape
    return buf.reshape(Z, ry, px)[:, :Y, 1:1 + X].copy()


def test_static_sweep_matches_allocating_sweep_twice():
    torch = pytest.importorskip("torch")
    w = W.random_spheres(71, 45, 33, 0.7, 1.0, 0.5, 6, 2.0, 9.0, seed=17)
    sp = (w.dx, w.dy, w.dz)
    s, px, ry, elems, scratch = layout(w.nx, w.ny, w.nz)
    assert s == L.PDFS_OK and scratch <= L.STATIC_SCRATCH_BYTES
    g = L.Grid(w.nx, w.ny, w.nz, *sp)
    dev = torch.from_numpy(to_internal(w.field, px, ry, elems)).cuda()
    expect = w.field.copy()
    for sn in (3, 6):  # two calls in a row, each checked against pdfs_sweep
        ch_ref = api.sweep(expect, sp, sn)
        ch = C.c_double(-1.0)
        s = L.load().pdfs_sweep_static(C.byref(g), C.c_void_p(dev.data_ptr()), sn, C.byref(ch), None)
        assert s == L.PDFS_OK, L.load().pdfs_status_string(s)
        torch.cuda.synchronize()
        got = from_internal(dev.cpu().numpy(), w.field.shape, px, ry)
        # tolerance: the same FP64 arithmetic as pdfs_sweep, so bit-exact
        assert got.tobytes() == expect.tobytes(), f"ordering {sn}"
        assert ch.value == ch_ref


def test_static_sweep_rejects_grids_beyond_its_scratch():
    s, px, ry, elems, scratch = layout(512, 512, 512)
    assert s == L.PDFS_ERR_TOO_LARGE and scratch > L.STATIC_SCRATCH_BYTES
    g = L.Grid(512, 512, 512, 1.0, 1.0, 1.0)
    # rejected before any device work: a dummy, never-dereferenced pointer is enough
    s = L.load().pdfs_sweep_static(C.byref(g), C.c_void_p(256), 1, None, None)
    assert s == L.PDFS_ERR_TOO_LARGE
    assert b"too large" in L.load().pdfs_status_string(s)
