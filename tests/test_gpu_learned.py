"""Learned warm start: the GPU MLP kernels against the FP64 numpy oracle
(forward, loss, gradients), training, and what the trained network changes
in the search (same results within the parity bar, fewer rays than an
untrained network)."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import horizon_svf_comp_py, learned, synthetic
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def _batch(torch, n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 1, (n, 32)).astype(np.float32)
    T = (np.tanh(X[:, :4].sum(1)) + 0.1 * rng.normal(size=n)).astype(np.float32)
    dev = torch.device("cuda:0")
    return X, T, torch.from_numpy(X).to(dev), torch.from_numpy(T).to(dev)


# The tensor-core kernels round X and h1 to BF16 after FP32 sums; the FP64
# oracle rounds the same values after FP64 sums, so a value within FP32
# rounding of a BF16 rounding boundary can round the other way (one BF16
# ulp, 2^-8 relative, of one hidden unit). Forward bar: 97 % of the outputs
# within 1e-4 (relative 1e-4), all within 5e-3.
def _assert_forward_close(y, y_ref):
    d = np.abs(y - y_ref)
    assert np.mean(d <= 1e-4 + 1e-4 * np.abs(y_ref)) >= 0.97, np.sort(d)[-10:]
    assert d.max() <= 5e-3, d.max()


def test_mlp_forward_and_gradients_match_fp64_oracle(torch):
    """Forward pass, loss and gradient of the BF16 tensor-core kernels
    against the FP64 restatement of the same rounding points."""
    p = mlp_ref.bf16_round(learned.init_params(3) + 0.01)
    X, T, Xd, Td = _batch(torch, 700, 1)
    y_ref, _ = mlp_ref.forward_bf16(p, X)
    y = learned.forward(p, Xd).cpu().numpy()
    _assert_forward_close(y, y_ref)
    loss_ref, g_ref = mlp_ref.loss_and_grad_bf16(p, X, T)
    loss, g = learned.gradients(p, Xd, Td)
    assert abs(loss - loss_ref) <= 1e-4 * max(1.0, loss_ref)
    scale = np.abs(g_ref).max()
    np.testing.assert_allclose(g, g_ref, rtol=2e-3, atol=1e-4 * scale)
    # And against the exact FP64 network: within BF16 precision.
    _, g_exact = mlp_ref.loss_and_grad(p, X, T)
    assert np.linalg.norm(g - g_exact) <= 0.03 * np.linalg.norm(g_exact)


def test_mlp_gradients_over_many_chunks(torch):
    """A batch of several thousand samples (many 64-sample chunks per block,
    a ragged last chunk): the per-block accumulators and their reductions."""
    p = mlp_ref.bf16_round(learned.init_params(4) - 0.02)
    X, T, Xd, Td = _batch(torch, 40001, 7)
    loss_ref, g_ref = mlp_ref.loss_and_grad_bf16(p, X, T)
    loss, g = learned.gradients(p, Xd, Td)
    assert abs(loss - loss_ref) <= 1e-4 * max(1.0, loss_ref)
    scale = np.abs(g_ref).max()
    np.testing.assert_allclose(g, g_ref, rtol=2e-3, atol=1e-4 * scale)


def test_mlp_weights_are_rounded_to_bf16(torch):
    p = learned.init_params(5)
    X, _, Xd, _ = _batch(torch, 64, 2)
    y = learned.forward(p, Xd).cpu().numpy()
    y_bf, _ = mlp_ref.forward_bf16(mlp_ref.bf16_round(p), X)
    _assert_forward_close(y, y_bf)


def test_training_reduces_loss(torch):
    _, _, Xd, Td = _batch(torch, 20000, 3)
    p0 = learned.init_params(0)
    l0, _ = learned.gradients(p0, Xd, Td)
    p1, hist = learned.train(Xd, Td, steps=300, batch=4096, lr=3e-3, seed=1)
    l1, _ = learned.gradients(p1, Xd, Td)
    assert l1 < 0.3 * l0


@pytest.fixture(scope="module")
def trained(torch):
    """An MLP trained on the plain method's horizons of two other seeds."""
    kw = dict(edge_km=0.5, box_km=40.0, kind="eroded", hmin=500.0, hmax=4200.0, n_features=0)
    args = (24, 1, 8000.0, 0.2, 1, 2)
    Xs, Ts = [], []
    for seed in (101, 102):
        X, T = learned.training_samples(synthetic.make_domain(seed=seed, **kw), args,
                                        max_samples=400000)
        Xs.append(X)
        Ts.append(T)
    X = torch.cat(Xs)
    T = torch.cat(Ts)
    p, _ = learned.train(X, T, steps=1500, batch=16384, lr=2e-3, seed=0)
    return p, kw, args


def test_learned_start_keeps_results_and_saves_rays(trained):
    """First-azimuth learned start (the reference starts every cell at 0 deg):
    same horizons within the parity bar, fewer rays than the plain chain and
    than an untrained network. Every-azimuth mode: within the parity bar."""
    p, kw, args = trained
    d = synthetic.make_domain(seed=7, **kw)
    # Results can change only where visibility is not monotone in elevation
    # (the bracket's result then depends on where it starts). With the
    # reference's global FP32 frame that happens at ray origins the FP32
    # rounding puts under a steep neighbouring triangle; the local-precision
    # frame removes those, so the comparison runs there.
    loc = dict(precision=1, return_stats=True)
    h0, s0, st0 = horizon_svf_comp_py(*d.inputs(), *args, **loc)
    h1, s1, st1 = horizon_svf_comp_py(*d.inputs(), *args, mlp_params=p, **loc)
    hu, su, stu = horizon_svf_comp_py(*d.inputs(), *args, mlp_params=learned.init_params(0),
                                      **loc)
    he, se, ste = horizon_svf_comp_py(*d.inputs(), *args, mlp_params=p,
                                      mlp_every_azimuth=True, **loc)
    def agree(h, s):
        return (float(np.mean(np.abs(h - h0) <= 0.25)),
                float(np.mean(np.abs(s - s0) <= 1e-3)))

    stats = {"learned": agree(h1, s1), "untrained": agree(hu, su), "every": agree(he, se)}
    print("agreement with the plain search (horizons within 0.25 deg, cells within "
          "SVF 1e-3):", stats)
    for k in ("learned", "untrained"):  # first azimuth from the MLP, then chained
        assert stats[k][0] >= 0.999 and stats[k][1] >= 0.999, stats
    # Every azimuth restarted at its proposal: on this terrain (3.7 km of
    # relief, 8 km search) about 0.6 % of (cell, azimuth) have a hit pattern
    # that is not monotone in elevation (a downward ray ends in mid-air at
    # dist_search above a deep valley while a higher one meets a far
    # ridge), and there a bracket's result depends on where it starts; the
    # bar of the benchmark recipes is tested in test_learned_bars_*.
    assert stats["every"][0] >= 0.995, stats
    # Reference frame: the parity bar on the horizons.
    hr0, _ = horizon_svf_comp_py(*d.inputs(), *args)
    hr1, _ = horizon_svf_comp_py(*d.inputs(), *args, mlp_params=p)
    assert np.mean(np.abs(hr1 - hr0) <= 0.25) >= 0.999
    evals = d.ncell * args[0]
    r = {k: st["num_rays"] / evals for k, st in
         (("plain", st0), ("learned", st1), ("untrained", stu), ("every", ste))}
    print("rays/eval", r)
    assert r["learned"] < r["plain"]
    assert r["learned"] < r["untrained"]
    assert r["every"] >= 2.0 - 1e-9  # a bracket always needs a hit and a miss


def test_learned_start_in_a_batch_equals_single_calls(trained):
    """Each domain of a batch gets its own raster and features: the learned
    start gives every domain the results of its own call."""
    from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch
    p, kw, args = trained
    doms = [synthetic.make_domain(seed=s, **kw) for s in (8, 9)]
    args2 = (16, 1, 6000.0, 0.2, 2, 1)
    outs = horizon_svf_comp_batch([(doms[0].inputs(), args), (doms[1].inputs(), args2)],
                                  mlp_params=p)
    for d, a, (h, s) in zip(doms, (args, args2), outs):
        h1, s1 = horizon_svf_comp_py(*d.inputs(), *a, mlp_params=p)
        np.testing.assert_array_equal(h, h1)
        np.testing.assert_array_equal(s, s1)


def test_split_items_equal_every_azimuth_restarts(trained):
    """One search item per (cell, azimuth) starting at the proposal (groups
    = num_hori) casts exactly the rays of the every-azimuth mode, which
    restarts each azimuth of the chain at its proposal: same results, same
    ray count. The library's own choice (-1) on a small domain is
    num_hori / 2 groups."""
    p, kw, args = trained
    d = synthetic.make_domain(seed=10, **kw)
    loc = dict(mlp_params=p, return_stats=True)
    he, se, ste = horizon_svf_comp_py(*d.inputs(), *args, mlp_every_azimuth=True, **loc)
    hs, ss, sts = horizon_svf_comp_py(*d.inputs(), *args, mlp_azimuth_groups=args[0], **loc)
    np.testing.assert_array_equal(hs, he)
    np.testing.assert_allclose(ss, se, rtol=0, atol=1e-12)
    assert sts["num_rays"] == ste["num_rays"]
    # The library's own choice on a small domain: two azimuths per item.
    ha, sa = horizon_svf_comp_py(*d.inputs(), *args, mlp_params=p, mlp_azimuth_groups=-1)
    h12, s12 = horizon_svf_comp_py(*d.inputs(), *args, mlp_params=p,
                                   mlp_azimuth_groups=args[0] // 2)
    np.testing.assert_array_equal(ha, h12)


def test_split_items_in_a_batch_equal_single_calls(trained):
    from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch
    p, kw, args = trained
    doms = [synthetic.make_domain(seed=s, **kw) for s in (12, 13)]
    args2 = (16, 1, 6000.0, 0.2, 2, 1)
    outs = horizon_svf_comp_batch([(doms[0].inputs(), args), (doms[1].inputs(), args2)],
                                  mlp_params=p, mlp_azimuth_groups=4)
    for d, a, (h, s) in zip(doms, (args, args2), outs):
        h1, s1 = horizon_svf_comp_py(*d.inputs(), *a, mlp_params=p, mlp_azimuth_groups=4)
        np.testing.assert_array_equal(h, h1)
        np.testing.assert_array_equal(s, s1)


def test_split_groups_must_divide_num_hori(trained):
    p, kw, args = trained
    d = synthetic.make_domain(seed=14, **kw)
    with pytest.raises(ValueError, match="does not divide"):
        horizon_svf_comp_py(*d.inputs(), *args, mlp_params=p, mlp_azimuth_groups=5)


@pytest.fixture(scope="module")
def trained_c1(torch):
    """An MLP trained on the plain method's horizons of two other seeds of
    the 2.5 km benchmark recipe (fBm H 0.8 + 20 peaks, 0-3000 m)."""
    Xs, Ts = [], []
    for seed in (201, 202):
        d = synthetic.make_config("c1", seed=seed, box_km=300.0)
        X, T = learned.training_samples(d, (24, 1, 40000.0, 0.2, 1, 2), max_samples=400000)
        Xs.append(X)
        Ts.append(T)
    p, _ = learned.train(torch.cat(Xs), torch.cat(Ts), steps=1500, batch=16384, lr=2e-3, seed=0)
    return p


@pytest.mark.parametrize("mode,bar", [
    (dict(mlp_azimuth_groups=4), 0.999),
    (dict(mlp_azimuth_groups=12), 0.999),
    (dict(mlp_azimuth_groups=-1), 0.999),
    # Every bracket restarted at its proposal (one item per azimuth, or the
    # every-azimuth mode): the start matters on more evaluations.
    (dict(mlp_azimuth_groups=24), 0.998),
    (dict(mlp_every_azimuth=True), 0.998),
])
def test_learned_bars_on_the_2p5km_recipe(trained_c1, mode, bar):
    """Restarted brackets (azimuth groups each starting at its proposal, or
    every azimuth) on a domain of the 2.5 km benchmark recipe (300 x 300 km,
    40 km search) against the CPU oracle: |dhorizon| <= 0.25 deg on >= 99.9 %
    of (cell, azimuth) for the library's own choice of groups (at least two
    azimuths per item) and |dSVF| <= 1e-3. Evaluations whose visibility is
    not monotone in elevation (a ray below the horizon that ends in mid-air
    at dist_search) keep the result of where their bracket starts, so
    restarting every azimuth agrees on 99.8 % here."""
    from oracle import api as oracle
    args = (24, 1, 40000.0, 0.2, 1, 2)
    d = synthetic.make_config("c1", seed=0, box_km=300.0)
    h, s = horizon_svf_comp_py(*d.inputs(), *args, mlp_params=trained_c1, **mode)
    ho, so, _ = oracle.horizon_svf(*d.inputs(), *args)
    within = float(np.mean(np.abs(h - ho) <= 0.25))
    max_svf = float(np.abs(s - so).max())
    print(mode, "within 0.25 deg %.6f, max |dSVF| %.3g" % (within, max_svf))
    assert within >= bar
    assert max_svf <= 1e-3
