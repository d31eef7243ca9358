"""The CPU oracle of the rank network (oracle/mlp_oracle.py) against finite
differences and against the published Adam update; no GPU."""
import numpy as np

from oracle import mlp_oracle as M


def _problem(nin=7, n=40, seed=0):
    rng = np.random.default_rng(seed)
    theta = rng.standard_normal(M.num_params(nin)) * 0.2
    X = rng.standard_normal((n, nin))
    t = rng.standard_normal(n)
    return theta, X, t


def test_gradient_matches_finite_differences():
    nin = 5
    theta, X, t = _problem(nin)
    loss, g = M.loss_and_grad(theta, X, t, nin, bf16=False)
    rng = np.random.default_rng(1)
    for p in rng.choice(theta.size, 40, replace=False):
        e = np.zeros_like(theta)
        e[p] = 1e-6
        lp, _ = M.loss_and_grad(theta + e, X, t, nin, bf16=False)
        lm, _ = M.loss_and_grad(theta - e, X, t, nin, bf16=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[p]) <= 1e-6 + 1e-5 * abs(fd)


def test_bf16_rounding_is_nearest_even():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 65504.0], np.float32)
    r = M.bf16_round(a)
    # representable values unchanged, others within half a BF16 ulp (2^-8 relative)
    assert r[0] == 1.0 and r[4] == 0.0
    assert r[1] == 1.0  # tie (halfway between 1 and 1 + 2^-7) rounds to even
    assert np.all(np.abs(r - a) <= np.abs(a) * 2.0 ** -8)
    assert np.all(M.bf16_round(r) == r)


def test_adam_descends_on_the_mse():
    nin = 6
    theta, X, t = _problem(nin, n=200, seed=3)
    m = np.zeros_like(theta)
    v = np.zeros_like(theta)
    l0, _ = M.loss_and_grad(theta, X, t, nin, bf16=False)
    for step in range(1, 201):
        _, g = M.loss_and_grad(theta, X, t, nin, bf16=False)
        M.adam_step(theta, m, v, g, step, 1e-2)
    l1, _ = M.loss_and_grad(theta, X, t, nin, bf16=False)
    assert l1 < 0.5 * l0
