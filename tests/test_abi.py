"""CPU checks of the C ABI: the library loads, exports every function that
include/pdfs.h declares, validates its arguments before touching a device,
and has no CPU fallback."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pdfs_gb300 import _lib as L
from pdfs_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(pdfs_\w+|run_fsm\w*)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = L.load()
    decl = declared_functions()
    assert decl, "no declarations parsed"
    for name in decl:
        assert hasattr(lib, name), name
    assert set(L.EXPORTS) <= set(decl)


def test_status_strings_and_version():
    lib = L.load()
    for s in range(0, -8, -1):
        assert lib.pdfs_status_string(s)
    assert b"sm_103a" in lib.pdfs_version()


def test_default_opts():
    o = L.Opts()
    L.load().pdfs_default_opts(C.byref(o))
    assert o.precision == L.PREC_FP64 and o.arith == L.ARITH_REFERENCE and o.freeze == L.FREEZE_NONE
    assert o.tol == 0.0


@pytest.mark.parametrize("grid", [(0, 4, 4, 1, 1, 1), (4, 4, 4, 0, 1, 1), (4, 4, 4, 1, -1, 1),
                                  (4, 4, 4, 1, 1, float("nan"))])
def test_invalid_grid_rejected_before_device(grid):
    g = L.Grid(*grid)
    o = api.make_opts()
    f = np.zeros(100, dtype=np.float64)
    assert L.load().pdfs_solve(C.byref(g), f.ctypes.data, None, C.byref(o), None) == L.PDFS_ERR_INVALID


def test_invalid_options_rejected():
    g = L.Grid(4, 4, 4, 1.0, 1.0, 1.0)
    f = np.zeros(6 * 6 * 6, dtype=np.float64)
    for k, v in [("precision", 7), ("arith", 4), ("freeze", -1), ("tol", -1.0), ("first_ordering", 9),
                 ("tile", 99)]:
        o = api.make_opts()
        setattr(o, k, v)
        assert L.load().pdfs_solve(C.byref(g), f.ctypes.data, None, C.byref(o), None) == L.PDFS_ERR_INVALID, k
    # FP32 pairs run on the FP64 bricks and pencils (tiles 5-8) only
    o = api.make_opts(arith=L.ARITH_PAIR, tile=1 << 8)
    assert L.load().pdfs_solve(C.byref(g), f.ctypes.data, None, C.byref(o), None) == L.PDFS_ERR_INVALID
    assert L.load().pdfs_sweep(C.byref(g), f.ctypes.data, None, 0, None, None) == L.PDFS_ERR_INVALID


def test_release_cached_checks_its_device():
    from conftest import have_gpu
    s = L.load().pdfs_release_cached(-1)
    assert s == (L.PDFS_ERR_INVALID if have_gpu() else L.PDFS_ERR_NO_DEVICE)
    if not have_gpu():
        assert L.load().pdfs_release_cached(0) == L.PDFS_ERR_NO_DEVICE


def test_no_cpu_fallback_without_device():
    from conftest import have_gpu
    if have_gpu():
        pytest.skip("a GPU is present")
    f = np.full((6, 6, 6), 1e10)
    with pytest.raises(api.PdfsError) as ei:
        api.solve(f, (1.0, 1.0, 1.0))
    assert ei.value.status == L.PDFS_ERR_NO_DEVICE
