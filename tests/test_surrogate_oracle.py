"""The CPU FP64 surrogate network (oracle/surrogate_mlp.py) checked against finite differences, so
that the GPU gradient check rests on a verified backward pass."""
import numpy as np

import surrogate_mlp as sm


def _problem(seed, n=12):
    rng = np.random.default_rng(seed)
    p = np.concatenate([np.concatenate([rng.uniform(-1, 1, fo * fi) * np.sqrt(6.0 / fi), rng.normal(0, 0.1, fo)])
                        for fo, fi in sm.LAYERS])
    B = rng.normal(0, 2.0, (32, 5))
    x = np.stack([rng.uniform(0, 0.998, n), np.deg2rad(rng.uniform(5, 89, n)), rng.uniform(1.3, 3.0, n),
                  rng.uniform(-10, 10, n), rng.uniform(-10, 10, n)], axis=1)
    cls = rng.integers(1, 4, n).astype(np.uint8)
    cls[0] = 0  # an unfinished ray: ignored by the loss
    tgt = rng.normal(0, 0.5, (n, 8))
    return p, B, x, cls, tgt


def test_parameter_count_matches_layers():
    assert sm.num_params() == 64 * 256 + 256 + 3 * (256 * 256 + 256) + 16 * 256 + 16


def test_backward_matches_central_differences():
    p, B, x, cls, tgt = _problem(5)
    g, terms = sm.gradients(p, B, x, cls, tgt)
    assert np.isclose(terms.sum(), sm.loss(p, B, x, cls, tgt), rtol=1e-12)
    rng = np.random.default_rng(11)
    offs = np.cumsum([0] + [fo * fi + fo for fo, fi in sm.LAYERS])
    # a few weights and biases from every layer, including the head's padding rows (gradient 0)
    idx = np.concatenate([rng.integers(offs[l], offs[l + 1], 6) for l in range(5)] + [[offs[5] - 1]])
    for i in idx:
        h = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (sm.loss(pp, B, x, cls, tgt) - sm.loss(pm, B, x, cls, tgt)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1.0 + 2 ** -8 + 2 ** -12], dtype=np.float64)
    r = sm.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 4 * 2 ** -8 and r[3] == -2.5
    assert r[4] == 1.0 + 2 ** -7  # just above the tie: rounds up
