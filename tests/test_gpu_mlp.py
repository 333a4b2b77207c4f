"""The learned scheduler's GPU kernels against the CPU oracle
(oracle/mlp_oracle.py), through the C ABI: the bf16 forward/backward
gradient, the Adam step and the tensor-core (tcgen05) inference; then the
trainer on real sweep traces and the ablation against the plain sweeps."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from pdfs_gb300 import _lib as L
from pdfs_gb300 import api
from pdfs_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def sample_batch(rng, n):
    """Features in the ranges the scheduler produces (bf16 bits) and labels."""
    x = np.zeros((n, M.NI), np.float32)
    x[:, 0] = rng.uniform(0, 4, n)
    x[:, 1:3] = rng.uniform(-2, 2, (n, 2))
    x[:, 3] = rng.random(n) < 0.5
    x[:, 4] = rng.random(n) < 0.3
    x[:, 5] = rng.uniform(0, 1, n)
    x[np.arange(n), 6 + rng.integers(0, 8, n)] = 1.0
    x[:, 14:16] = rng.uniform(-2, 2, (n, 2))
    y = (rng.random(n) < 0.35).astype(np.uint8)
    return M.bf16_bits(x), y


def params(rng):
    return M.bf16(rng.normal(0.0, 0.25, M.NP).astype(np.float32))


def test_gradient_matches_oracle():
    rng = np.random.default_rng(11)
    p = params(rng)
    xb, y = sample_batch(rng, 1000)   # several CTAs, one partly filled
    g, loss = api.mlp_grad(p, xb, y, pos_weight=3.0)
    lo, go = M.loss_grad(p, M.from_bits(xb), y, 3.0, round_=True)
    # tolerance: FP32 (GPU) vs float64 (oracle) sums can move a bf16
    # activation by one unit in the last place; relative L2 of the gradient
    assert np.linalg.norm(g - go) <= 1e-2 * np.linalg.norm(go)
    assert abs(loss - lo) <= 1e-4 * abs(lo)
    # per-layer check so an error in one block cannot hide in the norm
    o = 0
    for size in (M.NH * M.NI, M.NH, M.NH * M.NH, M.NH, M.NH, 1):
        a, b = g[o:o + size], go[o:o + size]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-7, o
        o += size


def test_adam_matches_oracle():
    rng = np.random.default_rng(12)
    p = rng.normal(size=M.NP).astype(np.float32)
    m = rng.normal(scale=0.1, size=M.NP).astype(np.float32)
    v = rng.uniform(0, 0.01, M.NP).astype(np.float32)
    g = rng.normal(size=M.NP).astype(np.float32)
    p1, m1, v1, pb = api.mlp_adam(p, m, v, g, step=7, lr=1e-3)
    q1, n1, w1 = M.adam(p, m, v, g, step=7, lr=1e-3)
    # tolerance: FP32 on both sides; the GPU fuses b*m + (1-b)*g into one
    # multiply-add and its sqrt/divide may differ by an ulp, which moves a
    # moment that cancels by a few ulps of its inputs
    assert np.allclose(p1, q1, rtol=1e-6, atol=1e-7)
    assert np.allclose(m1, n1, rtol=1e-5, atol=1e-7)
    assert np.allclose(v1, w1, rtol=1e-5, atol=1e-9)
    assert np.array_equal(pb, M.bf16_bits(p1))


def test_inference_matches_oracle():
    rng = np.random.default_rng(13)
    p = params(rng)
    blob = np.concatenate([p, [0.0]]).astype(np.float32)
    xb, _ = sample_batch(rng, 3000)
    z = api.mlp_infer(blob, xb)
    zo, _, _ = M.forward(p, M.from_bits(xb), round_=True)
    # tolerance: FP32 accumulation and rare one-ulp bf16 activation flips
    assert np.max(np.abs(z - zo)) <= 2e-2 * (1.0 + np.max(np.abs(zo)))
    assert np.mean(np.abs(z - zo)) <= 1e-3 * (1.0 + np.mean(np.abs(zo)))


def test_trainer_learns_from_sweep_traces():
    """Samples come from plain solves; a few epochs must lower the loss and
    the threshold must reach the requested recall on the samples."""
    with api.Trainer(seed=1) as tr:
        n = 0
        for seed in (1, 2):
            w = W.random_spheres(96, 80, 72, 1.0, 1.0, 1.0, 6, 3.0, 14.0, seed=seed)
            n = tr.add_solve(w.field, (w.dx, w.dy, w.dz), w.frozen, freeze=L.FREEZE_MASK,
                             precision=L.PREC_FP32_POLISH64, arith=L.ARITH_FAST, tol=1e-9)
        assert n > 0
        l1 = tr.fit(epochs=1, batch=4096, lr=2e-3, pos_weight=4.0)
        l2 = tr.fit(epochs=4, batch=4096, lr=2e-3, pos_weight=4.0)
        assert np.isfinite(l1) and l2 < l1
        blob, recall, active = tr.weights(recall=0.99)
    assert blob.shape == (L.MLP_BLOB,) and np.all(np.isfinite(blob[:-1]))
    assert recall >= 0.99
    assert 0.0 < active <= 1.0


def test_learned_scheduler_gain():
    """Ablation on a geometry the default weights never saw: the plain FP64
    solve to 1e-12 with every block swept, with the history rule alone, and
    with the trained network pruning the rule's candidates.  All three end at
    the same fixed point (a solve only stops on a full sweep).  The network
    must cut the node updates well below the plain method's; against the
    rule alone it prunes candidates at the price of occasional extra sweeps,
    so it must stay within 10% of the rule's updates."""
    w = W.random_spheres(192, 176, 160, 1.0, 1.0, 1.0, 12, 4.0, 24.0, seed=77)
    sp = (w.dx, w.dy, w.dz)
    res = {}
    for name, sched in (("none", L.SCHED_NONE), ("change", L.SCHED_CHANGE), ("learned", L.SCHED_LEARNED)):
        f = w.field.copy()
        st = api.solve(f, sp, frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP64, arith=L.ARITH_FAST,
                       tol=1e-12, scheduler=sched)
        res[name] = (f, st)
        print(f"{name:8s} sweeps {st['sweeps_fp64']:3d} full {st['full_sweeps']:3d} "
              f"updates/node {st['voxel_updates'] / w.interior:6.2f} ms {st['ms_fp64']:8.1f}")
    base = res["none"][0]
    for name in ("change", "learned"):
        # tolerance: a different visiting order reaches the FP64 fixed point to rounding
        got, ref = res[name][0][1:-1, 1:-1, 1:-1], base[1:-1, 1:-1, 1:-1]
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) <= 1e-13
    upd = {k: v[1]["voxel_updates"] for k, v in res.items()}
    assert upd["learned"] <= 0.7 * upd["none"]
    assert upd["learned"] <= 1.10 * upd["change"]
