"""pdfs_sweep_static: the allocation-free sweep for callers that cannot call
the device allocator while they run (code confined to a pool handed over by
a host application, real-time loops that must not call cudaMalloc, plugins
whose host forbids allocation after set-up).  Checked through the C ABI
against the allocating entry point pdfs_sweep and the oracle on two calls in
a row (bit-exact: both run the reference's FP64 arithmetic; against the
oracle every NaN counts as one value, see same()), with the
device's free memory unchanged across the second call; against the bounded
wait's timeout path; and across a cudaDeviceReset in a child process.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from pdfs_gb300 import _lib as L  # noqa: E402
from pdfs_gb300 import api  # noqa: E402
from pdfs_gb300 import workloads as W  # noqa: E402

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


def case():
    return W.random_spheres(71, 45, 33, 0.7, 1.0, 0.5, 6, 2.0, 9.0, seed=17)


def same(a, b):
    """Bit-exact, with every NaN counted as one value.  On this anisotropic
    grid the reference's own arithmetic (phi3D_fsm.c:167-177, the expanded
    quadratic) turns far nodes (1e10) into NaN, and the GPU and the host CPU
    give NaN different sign bits; the oracle reproduces the reference's NaNs
    where they arise."""
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and a[~na].tobytes() == b[~nb].tobytes())


def test_static_sweep_matches_allocating_sweep_twice():
    torch = pytest.importorskip("torch")
    w = case()
    sp = (w.dx, w.dy, w.dz)
    s, px, ry, elems, scratch = layout(w.nx, w.ny, w.nz)
    assert s == L.PDFS_OK and scratch <= L.STATIC_SCRATCH_BYTES
    g = L.Grid(w.nx, w.ny, w.nz, *sp)
    dev = torch.from_numpy(to_internal(w.field, px, ry, elems)).cuda()
    expect = w.field.copy()
    orc = w.field.copy()
    for k, sn in enumerate((3, 6)):  # two calls in a row, each checked against pdfs_sweep and the oracle
        ch_ref = api.sweep(expect, sp, sn)
        O.sweep(orc, sp, sn)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        ch = C.c_double(-1.0)
        s = L.load().pdfs_sweep_static(C.byref(g), C.c_void_p(dev.data_ptr()), sn, C.byref(ch), None)
        assert s == L.PDFS_OK, L.load().pdfs_status_string(s)
        torch.cuda.synchronize()
        if k == 1:  # after the first call has loaded the module: nothing is allocated
            assert torch.cuda.mem_get_info()[0] == free0
        got = from_internal(dev.cpu().numpy(), w.field.shape, px, ry)
        # tolerance: the same FP64 reference arithmetic as pdfs_sweep and the oracle, so bit-exact
        assert got.tobytes() == expect.tobytes(), f"ordering {sn} vs pdfs_sweep"
        assert same(got, orc), f"ordering {sn} vs the oracle"
        assert ch.value == ch_ref


def test_static_sweep_rejects_grids_beyond_its_scratch():
    s, px, ry, elems, scratch = layout(512, 512, 512)
    assert s == L.PDFS_ERR_TOO_LARGE and scratch > L.STATIC_SCRATCH_BYTES
    g = L.Grid(512, 512, 512, 1.0, 1.0, 1.0)
    # rejected before any device work: a dummy, never-dereferenced pointer is enough
    s = L.load().pdfs_sweep_static(C.byref(g), C.c_void_p(256), 1, None, None)
    assert s == L.PDFS_ERR_TOO_LARGE
    assert b"too large" in L.load().pdfs_status_string(s)


def test_static_sweep_timeout_then_clean_call(monkeypatch):
    """A column that never publishes (the test hook) makes the downstream
    columns' bounded waits give up: PDFS_ERR_TIMEOUT, and the next call on the
    same scratch is bit-exact again."""
    torch = pytest.importorskip("torch")
    w = case()
    sp = (w.dx, w.dy, w.dz)
    s, px, ry, elems, _ = layout(w.nx, w.ny, w.nz)
    g = L.Grid(w.nx, w.ny, w.nz, *sp)
    dev = torch.from_numpy(to_internal(w.field, px, ry, elems)).cuda()
    monkeypatch.setenv("PDFS_WAIT_MS", "300")
    monkeypatch.setenv("PDFS_TEST_POISON_COLUMN", "0")
    s = L.load().pdfs_sweep_static(C.byref(g), C.c_void_p(dev.data_ptr()), 1, None, None)
    assert s == L.PDFS_ERR_TIMEOUT, L.load().pdfs_status_string(s)
    monkeypatch.delenv("PDFS_TEST_POISON_COLUMN")
    monkeypatch.delenv("PDFS_WAIT_MS")
    dev.copy_(torch.from_numpy(to_internal(w.field, px, ry, elems)))
    s = L.load().pdfs_sweep_static(C.byref(g), C.c_void_p(dev.data_ptr()), 1, None, None)
    assert s == L.PDFS_OK, L.load().pdfs_status_string(s)
    torch.cuda.synchronize()
    expect = w.field.copy()
    O.sweep(expect, sp, 1)
    assert same(from_internal(dev.cpu().numpy(), w.field.shape, px, ry), expect)


def _reset_check() -> None:
    """Child process: call, cudaDeviceReset, call again; each result against
    the oracle.  The CUDA runtime is the one libpdfs links (libcudart.so.13)."""
    rt = C.CDLL("libcudart.so.13")
    lib = L.load()
    w = case()
    sp = (w.dx, w.dy, w.dz)
    s, px, ry, elems, _ = layout(w.nx, w.ny, w.nz)
    g = L.Grid(w.nx, w.ny, w.nz, *sp)
    host = to_internal(w.field, px, ry, elems)
    expect = w.field.copy()
    for k, sn in enumerate((2, 5)):
        if k == 1:
            assert rt.cudaDeviceReset() == 0
        p = C.c_void_p()
        assert rt.cudaMalloc(C.byref(p), C.c_size_t(host.nbytes)) == 0
        assert rt.cudaMemcpy(p, host.ctypes.data_as(C.c_void_p), C.c_size_t(host.nbytes), 1) == 0
        st = lib.pdfs_sweep_static(C.byref(g), p, sn, None, None)
        assert st == L.PDFS_OK, lib.pdfs_status_string(st)
        out = np.empty_like(host)
        assert rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), p, C.c_size_t(host.nbytes), 2) == 0
        assert rt.cudaFree(p) == 0
        O.sweep(expect, sp, sn)
        assert same(from_internal(out, w.field.shape, px, ry), expect), f"call {k + 1}"
        host = out
    print("reset check ok")


def test_static_sweep_after_device_reset():
    """After a cudaDeviceReset the scratch's address is looked up again in
    the new context (run in a child process: the reset would end this
    process's other CUDA state)."""
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "reset-check"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0 and "reset check ok" in r.stdout, r.stdout + r.stderr


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "reset-check":
    _reset_check()
