"""The MLP oracle itself: its gradients against finite differences, its BF16 rounding, its AUC."""
import numpy as np

from oracle import mlp


def _params(dim, seed, scale=0.3):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(mlp.param_count(dim)) * scale).astype(np.float32)


def test_gradients_match_finite_differences():
    dim = 3
    rng = np.random.default_rng(5)
    params = _params(dim, 1).astype(np.float64)
    x = mlp.features(rng.uniform(-3, 3, (24, dim)), dim).astype(np.float64)
    valid = rng.integers(0, 2, 24)
    _, g = mlp.loss_and_gradients(params, x, valid, dim, bf16_points=False)
    # float64 central differences on a sample of coordinates of every parameter block
    sizes = [256 * mlp.kin_of(dim), 256, 256 * 256, 256, 256, 1]
    starts = np.cumsum([0] + sizes[:-1])
    idx = np.concatenate([s + rng.choice(n, min(n, 12), replace=False) for s, n in zip(starts, sizes)])
    eps = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        l1, _ = mlp.loss_and_gradients(p1, x, valid, dim, bf16_points=False)
        l2, _ = mlp.loss_and_gradients(p2, x, valid, dim, bf16_points=False)
        num = (l1 - l2) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(num), (i, num, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0, 3.0e38], np.float32)
    r = mlp.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                    # tie -> even (mantissa 0)
    assert r[2] == 1.0 + 4 * 2 ** -8      # tie -> even (up)
    assert r[3] == 1.0                    # below half
    assert r[4] == -2.5 and r[5] == 0.0
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)


def test_auc():
    assert mlp.auc([0.1, 0.2, 0.8, 0.9], [0, 0, 1, 1]) == 1.0
    assert mlp.auc([0.9, 0.8, 0.2, 0.1], [0, 0, 1, 1]) == 0.0
    assert mlp.auc([0.5, 0.5, 0.5, 0.5], [0, 1, 0, 1]) == 0.5
