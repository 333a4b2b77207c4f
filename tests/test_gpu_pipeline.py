"""The drop-in surface on the GPU: the PDFS command line, calc_dist_field and
run_fsm against the reference program's own outputs and the oracle."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from pdfs_gb300 import _lib as L
from pdfs_gb300 import vti as VT

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "vti")
CLI = os.path.join(ROOT, "pdfs_gb300", "PDFS")


@pytest.mark.parametrize("name", ["sphere", "aniso"])
def test_cli_output_byte_identical_to_reference_program(name, tmp_path):
    """`PDFS <in> <prefix>` writes the same file, byte for byte, as the
    reference's own program (reader, pre-pass, one FSM round, post-passes,
    writer) on the same input."""
    prefix = str(tmp_path / name)
    r = subprocess.run([CLI, os.path.join(GOLD, f"{name}_in.vti"), prefix], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "VTI file created" in r.stdout and "Dimensions:" in r.stdout
    got = open(prefix + "_distfield.vti", "rb").read()
    ref = open(os.path.join(GOLD, f"{name}_ref_distfield.vti"), "rb").read()
    assert got == ref


def reference_pipeline(pf_loc, pf_dist, spacing, rounds):
    """calc_dist_field of single_gpu_cuda/src/phi3D.c:107-126 restated on the
    host with the oracle's sweeps."""
    d = pf_dist.copy()
    l = pf_loc
    inner = (l != -1) & (d != np.inf)
    z = inner & ~((d > 0) | (d < 0))
    d[z] = 90000.0
    for _ in range(rounds):
        for sn in range(1, 9):
            O.sweep(d, spacing, sn)
    d[(l != -1) & (d != np.inf) & (l == 1)] = -1.0
    Z, Y, X = d.shape
    out = d.copy()
    for k in range(Z):
        for j in range(Y):
            for i in range(X):
                I = i - 1 if i == X - 1 else (i + 1 if i == 0 else i)
                J = j - 1 if j == Y - 1 else (j + 1 if j == 0 else j)
                K = k - 1 if k == Z - 1 else (k + 1 if k == 0 else k)
                if (I, J, K) != (i, j, k):
                    out[k, j, i] = d[K, J, I]
    return out


@pytest.mark.parametrize("rounds", [1, 3])
def test_calc_dist_field_matches_reference_pipeline(rounds):
    pf = L.Phi()
    assert L.load().pdfs_vti_read(os.path.join(GOLD, "aniso_in.vti").encode(), C.byref(pf)) == L.PDFS_OK
    try:
        n = (pf.x + 2) * (pf.y + 2) * (pf.z + 2)
        shape = (pf.z + 2, pf.y + 2, pf.x + 2)
        loc = np.ctypeslib.as_array(pf.location, shape=(n,)).reshape(shape).copy()
        dist = np.ctypeslib.as_array(pf.distance, shape=(n,)).reshape(shape)
        expect = reference_pipeline(loc, dist.copy(), (pf.dx, pf.dy, pf.dz), rounds)
        st = L.Stats()
        assert L.load().pdfs_calc_dist_field(C.byref(pf), rounds, None, C.byref(st)) == L.PDFS_OK
        assert dist.tobytes() == expect.tobytes()
    finally:
        L.load().pdfs_phi_free(C.byref(pf))


def test_run_fsm_shim_matches_reference_rounds(capfd):
    from pdfs_gb300 import workloads as W
    w = W.random_spheres(40, 33, 27, 1.0, 1.0, 0.5, 4, 2.0, 8.0, seed=3)
    d = w.field.copy()
    pf = L.Phi(w.nx, w.ny, w.nz, w.dx, w.dy, w.dz, None, d.ctypes.data_as(C.POINTER(C.c_double)), 1.0)
    L.load().run_fsm(C.byref(pf), 2)
    assert "Parallel FSM time:" in capfd.readouterr().out
    e = w.field.copy()
    for _ in range(2):
        for sn in range(1, 9):
            O.sweep(e, (w.dx, w.dy, w.dz), sn)
    assert d.tobytes() == e.tobytes()


def test_cli_converge_and_errors(tmp_path):
    r = subprocess.run([CLI, os.path.join(GOLD, "sphere_in.vti"), str(tmp_path / "c"), "--converge"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ext, sp, vals = VT.read_output(str(tmp_path / "c_distfield.vti"))
    assert ext == (20, 18, 16)
    r = subprocess.run([CLI, str(tmp_path / "missing.vti"), str(tmp_path / "x")], capture_output=True, text=True)
    assert r.returncode == 1 and "Unable to read file" in r.stdout
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stdout


def test_cli_fast_polish_and_scheduler_options(tmp_path):
    """--polish --mixed with the learned scheduler: the distance file agrees
    with the converged plain FP64 run to the writer's 6 decimals (plus the
    mixed arithmetic's ~1e-7 relative); an unknown scheduler is a usage error."""
    src = os.path.join(GOLD, "sphere_in.vti")
    r = subprocess.run([CLI, src, str(tmp_path / "c"), "--converge"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([CLI, src, str(tmp_path / "p"), "--polish", "--mixed", "--tol", "1e-6", "--sched", "learned"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, _, a = VT.read_output(str(tmp_path / "c_distfield.vti"))
    _, _, b = VT.read_output(str(tmp_path / "p_distfield.vti"))
    fin = np.isfinite(a)
    assert np.array_equal(fin, np.isfinite(b))
    # tolerance: two units of the writer's last decimal, plus 1e-6 relative
    assert np.all(np.abs(a[fin] - b[fin]) <= 2e-6 + 1e-6 * np.abs(a[fin]))
    r = subprocess.run([CLI, src, str(tmp_path / "q"), "--sched", "sometimes"], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stdout
