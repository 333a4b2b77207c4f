"""The learned scheduler's CPU oracle (oracle/mlp_oracle.py) on its own:
its backward pass against central finite differences in float64, its bf16
rounding, and the Adam step against the textbook update.  The GPU kernels
are checked against this oracle in test_gpu_mlp.py."""
import numpy as np

from oracle import mlp_oracle as M


def rand_params(rng, scale=0.3):
    return rng.normal(0.0, scale, M.NP)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159, 0.0, 65504.0], dtype=np.float32)
    r = M.bf16(x)
    # bf16 keeps 8 significant bits; ties go to even
    assert r[0] == 1.0
    assert r[1] == 1.0          # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even is 1
    assert r[2] == 1.0078125    # above the tie: up
    assert r[3] == 1.0078125
    assert abs(r[4] - (-3.140625)) < 1e-7
    assert r[5] == 0.0
    assert np.array_equal(M.from_bits(M.bf16_bits(x)), r)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rand_params(rng)
    x = rng.normal(0.0, 1.0, (40, M.NI))
    y = (rng.random(40) < 0.4).astype(np.uint8)
    _, g = M.loss_grad(p, x, y, pos_weight=3.0, round_=False)
    idx = np.concatenate([rng.choice(M.NP - 1, 60, replace=False), [M.NP - 1]])
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        num = (M.loss_grad(pp, x, y, 3.0, round_=False)[0] - M.loss_grad(pm, x, y, 3.0, round_=False)[0]) / (2 * eps)
        # tolerance: central differences in float64 (ReLU kinks are not hit at these sizes)
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, num, g[i])


def test_adam_step():
    rng = np.random.default_rng(5)
    p, g = rng.normal(size=M.NP), rng.normal(size=M.NP)
    m, v = np.zeros(M.NP), np.zeros(M.NP)
    p1, m1, v1 = M.adam(p, m, v, g, step=1, lr=1e-3)
    # first step from zero moments: the update is lr * g / (|g| + eps)
    exp = p - 1e-3 * g / (np.abs(g) + 1e-8)
    assert np.allclose(p1, exp.astype(np.float32), rtol=1e-5, atol=1e-7)
    # the decay rates are float32: 1 - 0.9f and 1 - 0.999f
    one = np.float32(1)
    assert np.allclose(m1, (one - np.float32(0.9)) * g.astype(np.float32), rtol=1e-6)
    assert np.allclose(v1, (one - np.float32(0.999)) * (g * g).astype(np.float32), rtol=1e-6)
