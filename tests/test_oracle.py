"""The CPU oracle (oracle/fsm_oracle.c) against the golden fixtures produced
by the reference's own solver (tests/golden/make_golden.py): bit-exact."""
import hashlib
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from pdfs_gb300 import workloads as W

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def same(a, b):
    return a.tobytes() == b.tobytes()


def test_godunov_known_answers():
    z = np.load(os.path.join(GOLD, "godunov_kat.npz"))
    cases, expect = z["cases"], z["expect"]
    got = np.array([O.godunov(*c) for c in cases])
    # bit-exact, NaN included
    assert same(got, expect)


def test_godunov_f32_restatement_close_to_f64():
    rng = np.random.default_rng(3)
    for _ in range(500):
        base = float(rng.choice([0.0, 3.0, 40.0]))
        m = base + rng.uniform(0, 2.0, size=3)
        h = rng.choice([0.5, 1.0, 2.0], size=3)
        ref = O.godunov(*m, *h)
        f = O.lib().orc_godunov_f32(*[float(v) for v in m], *[float(v) for v in h])
        assert abs(f - ref) <= 2e-6 * max(1.0, abs(ref))


@pytest.mark.parametrize("gi", range(7))
def test_single_orderings_match_reference(gi):
    z = np.load(os.path.join(GOLD, "sweeps.npz"))
    f, sp = z[f"g{gi}_in"], tuple(z[f"g{gi}_spacing"])
    for sn in range(1, 9):
        a = f.copy()
        O.sweep(a, sp, sn)
        assert same(a, z[f"g{gi}_sn{sn}"]), f"ordering {sn}"
    a = f.copy()
    for sn in range(1, 9):
        O.sweep(a, sp, sn)
    assert same(a, z[f"g{gi}_round"])


@pytest.mark.parametrize("name", ["sphere16", "sphere32", "multi_aniso", "heightmap"])
@pytest.mark.parametrize("tag,tol", [("tol12", 1e-12), ("exact", 0.0)])
def test_solves_match_reference(name, tag, tol):
    z = np.load(os.path.join(GOLD, "solves.npz"))
    a = z[f"{name}_in"].copy()
    s, _ = O.solve(a, tuple(z[f"{name}_spacing"]), tol=tol)
    assert s == int(z[f"{name}_{tag}_sweeps"])
    assert same(a, z[f"{name}_{tag}"])


def test_openmp_sweep_is_bit_identical():
    w = W.random_spheres(70, 50, 40, 1.0, 1.0, 0.5, 6, 3.0, 10.0, seed=9)
    a, b = w.field.copy(), w.field.copy()
    sp = (w.dx, w.dy, w.dz)
    O.solve(a, sp, tol=0.0, threads=1)
    O.solve(b, sp, tol=0.0, threads=4)
    assert same(a, b)


def test_c1_configuration_pinned():
    meta = json.load(open(os.path.join(GOLD, "c1_sphere64.json")))
    w = W.config("C1")
    assert int(w.frozen.sum()) == meta["frozen_count"]
    # the generator uses only IEEE-exact numpy operations for the sphere
    assert sha(w.field) == meta["input_sha256"]
    for tag in ("tol12", "exact"):
        a = w.field.copy()
        s, c = O.solve(a, (w.dx, w.dy, w.dz), tol=meta[tag]["tol"], threads=4)
        assert s == meta[tag]["sweeps"]
        assert sha(a) == meta[tag]["sha256"]
    a = w.field.copy()
    for sn in range(1, 9):
        O.sweep(a, (w.dx, w.dy, w.dz), sn)
    assert sha(a) == meta["one_round"]["sha256"]


def test_frozen_mask_keeps_interface():
    w = W.unit_sphere(32)
    a = w.field.copy()
    O.solve(a, (w.dx, w.dy, w.dz), tol=0.0, frozen=w.frozen)
    fz = w.frozen.astype(bool)
    assert same(a[fz], w.field[fz])
    # the plain (reference) semantics lowers some interface nodes
    b = w.field.copy()
    O.solve(b, (w.dx, w.dy, w.dz), tol=0.0)
    assert (b[fz] < w.field[fz]).any()


def test_replace_update_fixed_point_equals_min_update():
    """The polish's replace-update u = min(input, G(u)) has the plain FSM's
    fixed point: starting from a perturbed solution it returns to it."""
    w = W.random_spheres(40, 36, 30, 1.0, 1.0, 1.0, 5, 3.0, 9.0, seed=4)
    sp = (w.dx, w.dy, w.dz)
    exact = w.field.copy()
    O.solve(exact, sp, tol=0.0, frozen=w.frozen)
    rng = np.random.default_rng(0)
    start = exact.copy()
    inner = start[1:-1, 1:-1, 1:-1]
    inner *= 1.0 + rng.uniform(-1e-6, 1e-6, size=inner.shape)
    fz = w.frozen.astype(bool)
    start[fz] = w.field[fz]
    s = 0
    while True:
        c = O.sweep_replace(start, sp, s % 8 + 1, w.field, frozen=w.frozen)
        s += 1
        if c <= 1e-13 or s > 200:
            break
    err = np.abs(start[1:-1, 1:-1, 1:-1] - exact[1:-1, 1:-1, 1:-1]).max()
    assert err < 1e-11, err
