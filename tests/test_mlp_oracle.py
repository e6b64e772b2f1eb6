"""The surrogate network's NumPy oracle checked against itself: its
back-propagated gradients equal central finite differences of its loss
(float64, no BF16 rounding), for the sine first layer, the ReLU layers and
the heads."""
import numpy as np

from oracle import mlp_oracle as MO


def _params(hk, seed):
    rng = np.random.default_rng(seed)
    W = MO.WIDTH
    parts = [rng.uniform(-3, 3, 2 * W), rng.uniform(-np.pi, np.pi, W),
             rng.uniform(-1, 1, W * W) * np.sqrt(6 / W), rng.normal(0, 0.1, W),
             rng.uniform(-1, 1, W * W) * np.sqrt(6 / W), rng.normal(0, 0.1, W),
             rng.uniform(-1, 1, W * hk) / np.sqrt(W), rng.normal(0, 0.1, hk)]
    return np.concatenate(parts)


def test_oracle_gradients_match_finite_differences():
    H, K = 2, 8
    p = _params(H * K, 0)
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (33, 2))
    y = rng.normal(size=(33, K))
    _, g, _ = MO.loss_and_gradients(p, x, y, H, K, exact=True)
    sizes = {n: a.size for n, a in MO.split(p, H * K).items()}
    offsets = np.cumsum([0] + [sizes[n] for n in ("W1", "b1", "W2", "b2", "W3", "b3", "Wh", "bh")])
    probe = np.concatenate([rng.choice(np.arange(a, b), size=6, replace=False)
                            for a, b in zip(offsets[:-1], offsets[1:])])
    h = 1e-6
    for i in probe:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = MO.loss_and_gradients(pp, x, y, H, K, exact=True)[0]
        lm = MO.loss_and_gradients(pm, x, y, H, K, exact=True)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e38], dtype=np.float32)
    r = MO.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                       # tie: rounds to the even mantissa
    assert r[2] == 1.0 + 2 ** -6             # tie: rounds up to the even mantissa
    assert r[3] == -2.5
    assert np.isfinite(r[4])
