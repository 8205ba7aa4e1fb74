"""The FP64 MLP oracle itself: gradients against finite differences (CPU)."""
import numpy as np
import pytest

from oracle import mlp_ref


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.2, mlp_ref.N_PARAMS)
    X = rng.normal(0, 1, (40, 32))
    T = rng.normal(0, 1, 40)
    _, g = mlp_ref.loss_and_grad(p, X, T)
    eps = 1e-6
    for k in rng.choice(mlp_ref.N_PARAMS, 60, replace=False):
        q = p.copy(); q[k] += eps
        lp, _ = mlp_ref.loss_and_grad(q, X, T)
        q[k] -= 2 * eps
        lm, _ = mlp_ref.loss_and_grad(q, X, T)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(fd)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 0.0], dtype=np.float32)
    r = mlp_ref.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-6 and r[4] == 0.0


def test_mlp_params_save_load_round_trip(tmp_path):
    from horayzon_extpar_gb300 import learned
    p = np.random.default_rng(0).normal(size=learned.N_PARAMS).astype(np.float32)
    path = str(tmp_path / "mlp.npy")
    learned.save_params(path, p)
    np.testing.assert_array_equal(learned.load_params(path), p)
    with pytest.raises(ValueError):
        learned.save_params(path, p[:10])
