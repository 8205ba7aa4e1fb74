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


def test_mixed_precision_oracle_is_close_to_the_exact_network():
    """The BF16 restatement of the GPU arithmetic differs from the exact
    FP64 network only by BF16 rounding (relative 2^-8 per rounded value)."""
    rng = np.random.default_rng(1)
    p = mlp_ref.bf16_round(rng.normal(0, 0.2, mlp_ref.N_PARAMS)).astype(np.float64)
    X = rng.normal(0, 1, (300, 32))
    T = rng.normal(0, 1, 300)
    y, _ = mlp_ref.forward(p, X)
    yb, _ = mlp_ref.forward_bf16(p, X)
    assert np.abs(yb - y).max() <= 0.03 * np.abs(y).max()
    l, g = mlp_ref.loss_and_grad(p, X, T)
    lb, gb = mlp_ref.loss_and_grad_bf16(p, X, T)
    assert abs(lb - l) <= 0.02 * l
    assert np.linalg.norm(gb - g) <= 0.03 * np.linalg.norm(g)
    # Inputs and activations already on the BF16 grid: the restatement's
    # forward pass is the exact one.
    Xq = mlp_ref.bf16_round(X).astype(np.float64)
    _, (Xb, _, _, _, _) = mlp_ref.forward_bf16(p, Xq)
    np.testing.assert_array_equal(Xb, Xq)
