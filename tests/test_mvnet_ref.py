"""The CPU reference of the learned MV proposer's net (oracle/mvnet_ref.py)
checked against central finite differences in float64, so it can check the
GPU backward kernels."""
import numpy as np

import mvnet_ref as R


def _problem(seed=3, h=8, w=12, batch=2):
    rng = np.random.default_rng(seed)
    params = rng.normal(0, 0.15, R.N_PARAMS)
    x0 = rng.normal(0, 1, (batch, R.IN_CH, h, w))
    labels = rng.integers(-16, 17, (batch, (h // 4) * (w // 4), 2))
    return params, x0, labels


def test_parameter_count():
    assert R.N_PARAMS == 28930


def test_backward_matches_finite_differences():
    params, x0, labels = _problem()
    loss, grad = R.loss_and_grads(params, x0, labels, bf16=False)
    rng = np.random.default_rng(11)
    # probe entries of every layer's weights and biases
    offs, off = [], 0
    for co, ci in R.SHAPES:
        offs.append((off, co * ci * 9, co))
        off += co * ci * 9 + co
    idx = []
    for o, nw, nb in offs:
        idx += list(o + rng.integers(0, nw, 6)) + list(o + nw + rng.integers(0, nb, 2))
    eps = 1e-5
    for i in idx:
        p = params.copy()
        p[i] += eps
        lp, _ = R.loss_and_grads(p, x0, labels, bf16=False)
        p[i] -= 2 * eps
        lm, _ = R.loss_and_grads(p, x0, labels, bf16=False)
        num = (lp - lm) / (2 * eps)
        assert abs(num - grad[i]) <= 1e-6 + 1e-4 * abs(num), (i, num, grad[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.3, 0.0], np.float32)
    r = R.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway rounds to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.3) < 0.01 and r[4] == 0.0


def test_bins_cover_the_range():
    assert R.bin_of(-16) == 0 and R.bin_of(16) == 16 and R.bin_of(0) == 8
    assert R.bin_of(-40) == 0 and R.bin_of(40) == 16
