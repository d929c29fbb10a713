"""The CPU restatement of the surrogate network (oracle/mlp_ref.py) checked on its own:
its analytic gradient against central finite differences, and its BF16 rounding."""
import numpy as np

from oracle import mlp_ref


def test_reference_gradient_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(mlp_ref, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    rng = np.random.default_rng(0)
    widths = [3, 8, 6, 4]
    n = sum(a * b + b for a, b in zip(widths[:-1], widths[1:]))
    p = rng.normal(0, 0.5, n)
    norm = (rng.normal(0, 1, 3), rng.uniform(0.5, 2, 3), rng.normal(0, 1, 4), rng.uniform(0.5, 2, 4))
    x = rng.normal(0, 1, (5, 3))
    t = rng.normal(0, 1, (5, 4))
    _, g = mlp_ref.loss_grad(p, widths, x, t, norm)
    fd = np.zeros(n)
    e = 1e-6
    for k in range(n):
        pp = p.copy(); pp[k] += e
        pm = p.copy(); pm[k] -= e
        fd[k] = (mlp_ref.loss_grad(pp, widths, x, t, norm)[0] - mlp_ref.loss_grad(pm, widths, x, t, norm)[0]) / (2 * e)
    assert np.abs(fd - g).max() <= 1e-7 * np.abs(g).max()


def test_bf16_rounds_to_nearest_even():
    v = np.array([1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 3.14159, -2.5e-3, 0.0], np.float32)
    r = mlp_ref.bf16(v)
    assert r[0] == 1.0                     # tie -> even mantissa
    assert r[1] == 1.0 + 4 * 2 ** -8       # tie -> even mantissa (upwards)
    assert abs(r[2] - 3.140625) < 1e-7
    assert np.all(np.abs(r - v) <= np.abs(v) * 2 ** -8 + 1e-30)
