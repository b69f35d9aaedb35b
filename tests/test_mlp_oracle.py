"""The numpy restatement of the learned order's scorer (oracle/mlp.py), on
the CPU: its gradient against central finite differences, its BF16
rounding against torch's, and the features on hand-worked cases."""
import numpy as np
import pytest

from oracle import mlp


def _weights(seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(mlp.P)
    w[mlp.O_W1:mlp.O_B1] = rng.uniform(-0.7, 0.7, mlp.H * mlp.F)
    w[mlp.O_B1:mlp.O_W2] = rng.uniform(-0.1, 0.1, mlp.H)
    w[mlp.O_W2:mlp.O_B2] = rng.uniform(-0.3, 0.3, mlp.H * mlp.H)
    w[mlp.O_B2:mlp.O_W3] = rng.uniform(-0.1, 0.1, mlp.H)
    w[mlp.O_W3:mlp.O_B3] = rng.uniform(-0.3, 0.3, mlp.H)
    w[mlp.O_B3] = -1.0
    return w


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    w = _weights(1)
    x = rng.random((40, mlp.F))
    y = (rng.random(40) < 0.3).astype(np.float64)
    _, g = mlp.loss_and_grad(w, x, y)
    idx = np.concatenate([rng.choice(mlp.P, 200, replace=False), [mlp.O_B3]])
    eps = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += eps
        wm[i] -= eps
        num = (mlp.loss_and_grad(wp, x, y)[0] - mlp.loss_and_grad(wm, x, y)[0]) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(num), i


def test_adam_moves_against_the_gradient():
    w = _weights(2)
    g = np.linspace(-1, 1, mlp.P)
    w2, m, v = mlp.adam_step(w, g, np.zeros(mlp.P), np.zeros(mlp.P), 1, 1e-3)
    # first Adam step: each weight moves by lr * sign(g) (up to eps)
    assert np.allclose(w - w2, 1e-3 * np.sign(g), atol=1e-6)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    a = (rng.standard_normal(10000) * 10.0 ** rng.integers(-3, 3, 10000)).astype(np.float32)
    a[:4] = [0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -1.0 - 2 ** -8]  # ties
    want = torch.from_numpy(a).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(mlp.bf16(a), want)


def test_features_by_hand():
    x = mlp.features(length=10, lbd=0, age=0, hist_bytes=[0] * 8, total=0, since_last=-1)
    assert np.allclose(x, [10 / 64, 10 / 64, 1, 0, 0, 0, 0, 0, 0, 1, 0, 0])
    x = mlp.features(length=8, lbd=4, age=15, hist_bytes=[3, 0, 9, 0, 0, 0, 0, 200], total=300, since_last=1)
    assert np.allclose(x, [8 / 64, 4 / 64, 0.5, 4 / 16, 3 / 8, 3 / 16, 12 / 32, 64 / 64, 3 / 8, 1 / 16,
                           np.log2(301) / 16, 1.0])


def test_history_rolls_like_the_order():
    h = mlp.History()
    h.born([0, 1], 0)
    h.record(0, {0: 2})
    h.record(1, {})
    h.record(2, {0: 1, 1: 5})
    assert h.hist[0][:3] == [1, 0, 2] and h.total[0] == 3 and h.last[0] == 2
    assert h.hist[1][:3] == [5, 0, 0] and h.last[1] == 2
    x = h.features(0, length=4, lbd=2, now=3)
    assert np.allclose(x[4:9], [1 / 8, 1 / 16, 3 / 32, 3 / 64, 2 / 8])
