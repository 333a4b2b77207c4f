"""Trains the learned block scheduler's default weights on the GPU and writes
them as C source (pdfs_gb300/csrc/mlp_default.h), which the next build
compiles into libpdfs so PDFS_SCHED_LEARNED works without a weight blob.

Samples come from plain solves (every block swept) of seeded 256^3
geometries, half random-sphere unions (4..12 spheres, radii log-uniform
4..50 cells, the density of the 768^3 150-sphere workload) and half
Gaussian-bump heightmaps (8 bumps, amplitude 5..40, width 20..120 cells):
each geometry is traced once as FP32 bulk + FP64 polish (tol 1e-5) and
every other one also as a plain FP64 solve to 1e-12.  The network is fitted
by the library's own bf16 forward / backward / Adam kernels; the decision
threshold keeps `recall` of the positive samples.

    python -m pdfs_gb300.train_scheduler [--grids 64] [--size 256] [--out PATH]

`--infer-rows N` instead runs the inference entry point (pdfs_mlp_infer) twice
on N seeded random feature rows and prints the wall time of the second call,
host copies included; it is the workload of the inference kernel's profile.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from pdfs_gb300 import _lib as L  # noqa: E402
from pdfs_gb300 import api  # noqa: E402
from pdfs_gb300 import build as B  # noqa: E402
from pdfs_gb300 import workloads as W  # noqa: E402


def geometry(i, n):
    if i % 2 == 0:
        rng = np.random.default_rng(1000 + i)
        return W.random_spheres(n, n, n, 1.0, 1.0, 1.0, int(rng.integers(4, 13)), 4.0, 50.0, seed=2000 + i)
    return W.heightmap(n, n, n, 1.0, 1.0, 1.0, seed=3000 + i)


def train(grids=64, size=256, epochs=6, recall=0.9999, seed=7, device=0, log=print):
    t0 = time.time()
    tr = api.Trainer(device=device, seed=seed)
    n = 0
    for i in range(grids):
        w = geometry(i, size)
        sp = (w.dx, w.dy, w.dz)
        n = tr.add_solve(w.field, sp, w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64,
                         arith=L.ARITH_FAST, tol=1e-5, device=device)
        if i % 2 == 0:
            n = tr.add_solve(w.field, sp, w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP64,
                             arith=L.ARITH_FAST, tol=1e-12, device=device)
    log(f"traces: {grids} geometries at {size}^3, {n} samples, {time.time() - t0:.1f} s")
    losses = []
    for ep in range(epochs):
        losses.append(tr.fit(epochs=1, batch=8192, lr=2e-3 if ep < epochs - 2 else 5e-4, pos_weight=4.0))
        log(f"epoch {ep}: loss {losses[-1]:.4f}")
    blob, r, a = tr.weights(recall=recall)
    tr.close()
    log(f"threshold {blob[-1]:.4f}: recall {r:.5f}, predicted active {a:.3f} of the nominated blocks")
    return blob, {"grids": grids, "size": size, "samples": n, "epochs": epochs, "loss": losses[-1],
                  "recall": r, "active": a}


def write_header(blob, info, path):
    def lit(v):  # a C float literal ("1" needs a decimal point before the suffix)
        t = f"{float(v):.9g}"
        return (t if any(c in t for c in ".e") else t + ".0") + "f"

    vals = ",\n  ".join(", ".join(lit(v) for v in blob[i:i + 6]) for i in range(0, len(blob), 6))
    with open(path, "w") as f:
        f.write("// mlp_default.h -- the learned scheduler's default weights, written by\n")
        f.write("// pdfs_gb300/train_scheduler.py; regenerate rather than edit.\n")
        f.write(f"// {info['grids']} geometries at {info['size']}^3, {info['samples']} samples, "
                f"{info['epochs']} epochs, final loss {info['loss']:.4f};\n")
        f.write(f"// threshold keeps recall {info['recall']:.5f}, predicts {info['active']:.3f} of the "
                "nominated blocks active.\n")
        f.write("// Layout: PDFS_MLP_PARAMS bf16-exact floats (W1, b1, W2, b2, w3, b3), then the threshold.\n")
        f.write("#pragma once\n")
        f.write(f"static const float kDefaultMlpBlob[PDFS_MLP_BLOB] = {{\n  {vals}}};\n")


def infer_rows(n, seed=0):
    """Two pdfs_mlp_infer calls on n random bf16 feature rows; wall seconds of the second."""
    rng = np.random.default_rng(seed)

    def bits(a):  # bf16 bit patterns by truncation: any bf16 values do for timing
        return (np.ascontiguousarray(a, dtype=np.float32).view(np.uint32) >> 16).astype(np.uint16)

    w = (bits(rng.normal(0.0, 0.25, L.MLP_PARAMS)).astype(np.uint32) << 16).view(np.float32)
    blob = np.concatenate([w, np.zeros(1, np.float32)])
    x = bits(rng.uniform(-2.0, 2.0, (n, L.MLP_IN)))
    api.mlp_infer(blob, x)
    t0 = time.perf_counter()
    api.mlp_infer(blob, x)
    return time.perf_counter() - t0


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--grids", type=int, default=64)
    p.add_argument("--size", type=int, default=256)
    p.add_argument("--epochs", type=int, default=6)
    p.add_argument("--recall", type=float, default=0.9999)
    p.add_argument("--seed", type=int, default=7)
    p.add_argument("--out", default=os.path.join(HERE, "csrc", "mlp_default.h"))
    p.add_argument("--infer-rows", type=int, default=0)
    a = p.parse_args()
    if a.infer_rows:
        dt = infer_rows(a.infer_rows)
        print(f"pdfs_mlp_infer: {a.infer_rows} rows in {dt * 1e3:.2f} ms (host copies included)")
        return
    B.build()
    blob, info = train(a.grids, a.size, a.epochs, a.recall, a.seed)
    assert blob.size == L.MLP_BLOB
    write_header(blob, info, a.out)
    print(f"wrote {a.out}")


if __name__ == "__main__":
    main()
