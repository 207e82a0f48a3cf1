"""The network oracle's analytic gradient against finite differences (CPU only)."""
import numpy as np

from oracle import mlp as OM


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_par = sum(a * b + b for a, b in OM.LAYERS)
    w = rng.uniform(-0.1, 0.1, n_par)
    X = rng.standard_normal((6, 256))
    T = rng.standard_normal((6, 16))
    M = (rng.uniform(size=(6, 16)) < 0.7).astype(float)
    loss, g = OM.loss_grad(w, X, T, M, round_weights=False, bf16_operands=False)
    for idx in rng.choice(n_par, 12, replace=False):
        e = np.zeros(n_par)
        e[idx] = 1e-6
        lp, _ = OM.loss_grad(w + e, X, T, M, round_weights=False, bf16_operands=False)
        lm, _ = OM.loss_grad(w - e, X, T, M, round_weights=False, bf16_operands=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[idx]) <= 1e-6 + 1e-5 * abs(fd), (idx, fd, g[idx])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159265], np.float32)
    r = OM.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # 1 + 2^-8 rounds to even (down)
    assert r[2] == 1.0078125            # above the half-way point rounds up
    assert abs(r[3] + 3.140625) < 1e-12
