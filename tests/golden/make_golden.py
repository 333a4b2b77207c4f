"""Generates the golden fixtures in tests/golden/ by running the reference's
own FSM (mpi_openacc/src/phi3D_fsm.c, compiled unmodified into
oracle/_ref/libref_fsm.so by `make -C oracle ref`).

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden.py

Outputs (all small):
  godunov_kat.npz  -- local-solver known answers: 1x1x1 grids whose six halo
                      neighbours hold the test minima, swept once (ordering 1)
  sweeps.npz       -- single orderings 1..8 and an 8-ordering round on small
                      random fields (odd, prime and anisotropic shapes)
  solves.npz       -- converged solves of small sphere / multi-sphere grids
  c1_sphere64.json -- the 64^3 unit-sphere configuration solved to 1e-12 and to
                      an exact fixed point: sweep counts and SHA-256 of the field
  vti/*.vti        -- input files in the reference reader's layout and the
                      reference program's own output for them (its CLI,
                      single_gpu_cuda/src/main.c, built for the CPU by
                      `make -C oracle ref` with the reference's CPU sweep)
"""
from __future__ import annotations

import hashlib
import subprocess
import json
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from pdfs_gb300 import vti as VT  # noqa: E402
from pdfs_gb300 import workloads as W  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def kat_cases(seed=11):
    rng = np.random.default_rng(seed)
    cases = []
    inf, far = math.inf, 1.0e10
    specials = [
        (0, 0, 0), (1, 1, 1), (0, 1, 2), (2, 1, 0), (1, 0, 1), (0.5, 0.5, inf), (inf, inf, inf),
        (far, far, far), (0, far, far), (far, 0, inf), (1, far, 1), (-1, -1, 0.2), (-1, 3, 3),
        (1000.0, 1000.1, 1000.2), (123456.7, 123456.75, 123456.8), (0.3, 0.3, 0.3001),
    ]
    spacings = [(1, 1, 1), (1, 1, 0.5), (0.5, 1, 2), (1 / 63, 1 / 63, 1 / 63), (0.3, 0.7, 1.1)]
    for sp in spacings:
        for m in specials:
            cases.append((*m, *sp))
    for _ in range(3000):
        sp = spacings[int(rng.integers(0, len(spacings)))]
        base = float(rng.choice([0.0, 1.0, 50.0, 700.0]))
        m = base + rng.uniform(0, 2.5, size=3) * max(sp)
        # ties
        if rng.uniform() < 0.2:
            m[int(rng.integers(0, 3))] = m[int(rng.integers(0, 3))]
        if rng.uniform() < 0.1:
            m[int(rng.integers(0, 3))] = far
        cases.append((*m, *sp))
    return np.array(cases, dtype=np.float64)


def run_kat(cases):
    out = np.empty(len(cases))
    for n, (mx, my, mz, dx, dy, dz) in enumerate(cases):
        f = np.full((3, 3, 3), math.inf)
        # each axis minimum is placed on the minus side, +inf on the plus side
        f[1, 1, 0], f[1, 1, 2] = mx, math.inf
        f[1, 0, 1], f[1, 2, 1] = my, math.inf
        f[0, 1, 1], f[2, 1, 1] = mz, math.inf
        f[1, 1, 1] = math.inf  # old value +inf: the result is the candidate itself
        O.ref(False).ref_sweep(1, 1, 1, dx, dy, dz, f, 1)
        out[n] = f[1, 1, 1]
    return out


SWEEP_GRIDS = [
    ((1, 1, 1), (1.0, 1.0, 1.0), 1),
    ((2, 3, 5), (1.0, 1.0, 1.0), 2),
    ((7, 5, 3), (0.3, 0.7, 1.1), 3),
    ((13, 11, 7), (1.0, 1.0, 0.5), 4),
    ((16, 16, 16), (1.0, 1.0, 1.0), 5),
    ((31, 17, 9), (0.5, 1.0, 2.0), 6),
    ((40, 3, 21), (1.0, 1.0, 1.0), 7),
]


def main():
    O.build(ref=True)
    if not O.have_ref():
        raise SystemExit("reference library missing: run `make -C oracle ref` where the reference exists")

    cases = kat_cases()
    np.savez_compressed(os.path.join(OUT, "godunov_kat.npz"), cases=cases, expect=run_kat(cases))

    sw = {}
    for gi, ((nx, ny, nz), sp, seed) in enumerate(SWEEP_GRIDS):
        f = W.random_field(nx, ny, nz, seed, frac_known=0.08)
        sw[f"g{gi}_in"] = f
        sw[f"g{gi}_spacing"] = np.array(sp)
        for sn in range(1, 9):
            a = f.copy()
            O.ref_sweep(a, sp, sn)
            sw[f"g{gi}_sn{sn}"] = a
        a = f.copy()
        for sn in range(1, 9):
            O.ref_sweep(a, sp, sn)
        sw[f"g{gi}_round"] = a
    np.savez_compressed(os.path.join(OUT, "sweeps.npz"), **sw)

    so = {}
    solve_cases = {
        "sphere16": W.unit_sphere(16),
        "sphere32": W.unit_sphere(32),
        "multi_aniso": W.random_spheres(37, 29, 23, 1.0, 1.0, 0.5, 5, 2.0, 9.0, seed=21),
        "heightmap": W.heightmap(48, 40, 24, 1.0, 1.0, 0.5, seed=22, amp=(2.0, 8.0), width=(4.0, 12.0)),
    }
    for name, w in solve_cases.items():
        sp = (w.dx, w.dy, w.dz)
        so[f"{name}_in"] = w.field
        so[f"{name}_frozen"] = w.frozen
        so[f"{name}_spacing"] = np.array(sp)
        for tag, tol in (("tol12", 1e-12), ("exact", 0.0)):
            a = w.field.copy()
            s, c = O.ref_solve(a, sp, tol=tol)
            so[f"{name}_{tag}"] = a
            so[f"{name}_{tag}_sweeps"] = np.array(s)
    np.savez_compressed(os.path.join(OUT, "solves.npz"), **so)

    w = W.config("C1")
    sp = (w.dx, w.dy, w.dz)
    meta = {"config": "C1 unit sphere 64^3, h=1/63, r=0.25, halo +inf, far 1e10",
            "input_sha256": sha(w.field), "frozen_sha256": sha(w.frozen),
            "frozen_count": int(w.frozen.sum())}
    for tag, tol in (("tol12", 1e-12), ("exact", 0.0)):
        a = w.field.copy()
        s, c = O.ref_solve(a, sp, tol=tol)
        inner = a[1:-1, 1:-1, 1:-1]
        meta[tag] = {"tol": tol, "sweeps": s, "last_change": c, "sha256": sha(a),
                     "max": float(inner.max()), "min": float(inner.min()), "sum": float(inner.sum())}
    # one round only, as the reference product runs it (single_gpu_cuda/src/phi3D.c:118-119)
    a = w.field.copy()
    for sn in range(1, 9):
        O.ref_sweep(a, sp, sn)
    meta["one_round"] = {"sha256": sha(a)}
    with open(os.path.join(OUT, "c1_sphere64.json"), "w") as fh:
        json.dump(meta, fh, indent=1)

    vdir = os.path.join(OUT, "vti")
    os.makedirs(vdir, exist_ok=True)
    cases = {
        "sphere": (18, 16, 14, (1.0, 1.0, 1.0), (8.5, 7.0, 6.5), 4.2),
        "aniso": (15, 13, 20, (0.5, 0.7, 0.4), (3.6, 4.1, 3.9), 2.3),
    }
    for name, (nx, ny, nz, sp, c, r) in cases.items():
        loc, dist = VT.sphere_input(nx, ny, nz, sp, c, r)
        inp = os.path.join(vdir, f"{name}_in.vti")
        VT.write_input(inp, loc, dist, sp)
        prefix = os.path.join(vdir, f"{name}_ref")
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "PDFS_ref"), inp, prefix], check=True,
                       stdout=subprocess.DEVNULL)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
