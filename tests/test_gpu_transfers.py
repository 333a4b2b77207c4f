"""Host transfers and context memory on the GPU: the slab-pipelined load and
store of fields of 256 MB and more must give the same bits as device-resident
input and output (and as a field small enough to load in one slab), and a
destroyed context's device blocks must be reused by the next context of the
same size and handed back by pdfs_release_cached."""
import numpy as np
import pytest

from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def same(a, b):
    return a.tobytes() == b.tobytes()


@pytest.mark.parametrize("arith", [L.ARITH_PAIR, L.ARITH_MIXED])
def test_slab_pipeline_equals_device_buffers(arith):
    """A 340 x 330 x 320 field (293 MB: 21 slabs of 16 planes on the way in
    and out, cap bounds per slab) through host buffers equals the same solve
    on device buffers, which load and store in one pass."""
    torch = pytest.importorskip("torch")
    w = W.random_spheres(340, 330, 320, 1.0, 1.0, 1.0, 12, 4.0, 30.0, seed=41)
    assert w.field.nbytes >= 256 << 20
    sp = (w.dx, w.dy, w.dz)
    kw = dict(freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=arith, tol=1e-5)
    host = w.field.copy()
    api.solve(host, sp, frozen=w.frozen, **kw)
    with api.Context(w.nx, w.ny, w.nz, sp, **kw) as c:
        df = torch.from_numpy(w.field).cuda()
        dm = torch.from_numpy(w.frozen).cuda()
        c.load(df.data_ptr(), dm.data_ptr())
        c.run()
        do = torch.zeros_like(df)
        c.store(do.data_ptr())
        torch.cuda.synchronize()
        dev = do.cpu().numpy()
        # and a host load with a device store, and the reverse
        c.load(w.field, w.frozen)
        c.run()
        do.zero_()
        c.store(do.data_ptr())
        torch.cuda.synchronize()
        mixed = do.cpu().numpy()
    assert same(host, dev) and same(host, mixed)


def test_pinned_and_pageable_host_buffers_agree():
    torch = pytest.importorskip("torch")
    w = W.random_spheres(330, 330, 330, 1.0, 1.0, 1.0, 8, 4.0, 25.0, seed=43)
    assert w.field.nbytes >= 256 << 20  # the pipelined path
    sp = (w.dx, w.dy, w.dz)
    kw = dict(freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-5)
    pageable = w.field.copy()
    api.solve(pageable, sp, frozen=w.frozen, **kw)
    pf = torch.from_numpy(w.field.copy()).pin_memory()
    pm = torch.from_numpy(w.frozen.copy()).pin_memory()
    pinned = pf.numpy()
    api.solve(pinned, sp, frozen=pm.numpy(), **kw)
    assert same(pageable, pinned)


def test_block_cache_reuse_and_release():
    torch = pytest.importorskip("torch")
    w = W.random_spheres(200, 200, 200, 1.0, 1.0, 1.0, 6, 4.0, 20.0, seed=44)
    sp = (w.dx, w.dy, w.dz)
    kw = dict(freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-5)
    mib = 1 << 20
    api.release_cached(0)
    free0 = torch.cuda.mem_get_info(0)[0]
    a = w.field.copy()
    api.solve(a, sp, frozen=w.frozen, **kw)  # the context's blocks stay cached
    free1 = torch.cuda.mem_get_info(0)[0]
    assert free0 - free1 >= 200 * mib  # the field alone is 65 MB in each of 3 copies, plus the stage
    b = w.field.copy()
    api.solve(b, sp, frozen=w.frozen, **kw)  # takes the cached blocks
    free2 = torch.cuda.mem_get_info(0)[0]
    assert abs(free2 - free1) <= 16 * mib
    assert same(a, b)
    api.release_cached(0)
    free3 = torch.cuda.mem_get_info(0)[0]
    assert free3 - free2 >= 200 * mib
    with pytest.raises(api.PdfsError):
        api.release_cached(-1)
