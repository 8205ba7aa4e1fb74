"""The downward walk below the clip by doubling and bisection
(hz_options.elev_walk = HZ_WALK_BISECT). Once a downward walk is at or below
+0.25 deg every further step gives a horizon clipped to 0, so the walk only
decides the elevation carried into the next azimuth; the bisection finds the
same stop as the reference's step walk wherever the rays below it hit and
those above it miss.

* Against the oracle's restatement of the same walk (`bisect_walk`): the
  same rays, so identical horizons (1e-9 deg on >= 99.99 %, the same bits
  wherever they agree), SVF to 1e-12 on those cells and the same ray count.
* Against the reference's step walk: identical horizons on >= 99.99 % of
  (cell, azimuth) (the rest are non-monotone walks), within 0.25 deg on
  >= 99.9 %, |dSVF| <= 1e-3, and fewer rays."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import _lib, horizon_svf_comp_py, synthetic
from oracle import api as oracle

pytestmark = pytest.mark.gpu

EXACT_DEG = 1e-9
CASES = [
    ("c1", dict(recipe="c1", box_km=300.0, seed=0), (24, 1, 40000.0, 0.2, 1, 2)),
    ("c3", dict(recipe="c3", box_km=80.0, seed=1), (24, 1, 40000.0, 0.2, 1, 2)),
    ("rough", dict(edge_km=0.5, box_km=40.0, kind="eroded", hmin=500.0, hmax=4200.0,
                   n_features=0, seed=21), (24, 1, 8000.0, 0.2, 1, 2)),
    ("refine_gt0", dict(recipe="c1", box_km=200.0, seed=2), (12, 0, 30000.0, 0.2, 3, 1)),
]


def _domain(kw):
    kw = dict(kw)
    recipe = kw.pop("recipe", None)
    return synthetic.make_config(recipe, **kw) if recipe else synthetic.make_domain(**kw)


@pytest.mark.parametrize("name,kw,args", CASES, ids=[c[0] for c in CASES])
def test_bisect_walk_matches_its_oracle_restatement(name, kw, args):
    d = _domain(kw)
    h, s, st = horizon_svf_comp_py(*d.inputs(), *args, elev_walk=_lib.HZ_WALK_BISECT,
                                   return_stats=True)
    ho, so, sto = oracle.horizon_svf(*d.inputs(), *args, bisect_walk=True)
    dh = np.abs(h - ho)
    same = dh <= EXACT_DEG
    assert same.mean() >= 0.9999, same.mean()
    np.testing.assert_array_equal(h[same], ho[same])
    cells = same.all(axis=0)
    np.testing.assert_allclose(s[cells], so[cells], rtol=0, atol=1e-12)
    assert abs(st["num_rays"] - sto["num_rays"]) <= 1e-4 * sto["num_rays"]


@pytest.mark.parametrize("name,kw,args", CASES, ids=[c[0] for c in CASES])
def test_bisect_walk_keeps_the_reference_results(name, kw, args):
    d = _domain(kw)
    h0, s0, st0 = horizon_svf_comp_py(*d.inputs(), *args, return_stats=True)
    h1, s1, st1 = horizon_svf_comp_py(*d.inputs(), *args, elev_walk=_lib.HZ_WALK_BISECT,
                                      return_stats=True)
    dh = np.abs(h1 - h0)
    evals = d.ncell * args[0] * args[4]
    print(name, "identical %.7f, rays per evaluation %.3f -> %.3f"
          % (np.mean(dh <= EXACT_DEG), st0["num_rays"] / evals, st1["num_rays"] / evals))
    assert np.mean(dh <= EXACT_DEG) >= 0.9999
    assert np.mean(dh <= 0.25) >= 0.999
    assert np.abs(s1 - s0).max() <= 1e-3
    assert st1["num_rays"] <= st0["num_rays"]


def test_bisect_walk_with_azimuth_groups_and_given_starts():
    """The walk inside search items that start at given indices: the same
    rays as the oracle with the same starts and the same walk."""
    torch = pytest.importorskip("torch")
    from horayzon_extpar_gb300 import horizon_svf_comp_device
    dev = torch.device("cuda:0")
    d = _domain(CASES[2][1])
    args = CASES[2][2]
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in d.inputs()]
    m = np.random.default_rng(5).integers(-40, 60, size=(args[0], d.ncell)).astype(np.int16)
    h, s, st = horizon_svf_comp_device(*t, *args, start_index=torch.from_numpy(m).to(dev),
                                       mlp_azimuth_groups=4, elev_walk=_lib.HZ_WALK_BISECT)
    h = h.cpu().numpy()
    ho, so, sto = oracle.horizon_svf(*d.inputs(), *args, start_index=m, groups=4,
                                     bisect_walk=True)
    same = np.abs(h - ho) <= EXACT_DEG
    assert same.mean() >= 0.9999
    assert abs(st["num_rays"] - sto["num_rays"]) <= 1e-4 * sto["num_rays"]


def test_bisect_walk_needs_the_persistent_kernel():
    d = _domain(CASES[2][1])
    with pytest.raises(ValueError, match="persistent"):
        horizon_svf_comp_py(*d.inputs(), *CASES[2][2], kernel=_lib.HZ_KERNEL_PER_CELL,
                            elev_walk=_lib.HZ_WALK_BISECT)


@pytest.mark.parametrize("kernel", [_lib.HZ_KERNEL_PERSISTENT, _lib.HZ_KERNEL_PERSISTENT_BVH2])
def test_bisect_walk_same_on_both_trees(kernel):
    """The 4-wide and the binary tree cast the same rays, so the walk gives
    the same bits on both, in a batch of two domains too."""
    from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch
    name, kw, args = CASES[2]
    d = _domain(kw)
    h, s = horizon_svf_comp_py(*d.inputs(), *args, elev_walk=_lib.HZ_WALK_BISECT,
                               kernel=kernel)
    ho, so, _ = oracle.horizon_svf(*d.inputs(), *args, bisect_walk=True)
    assert np.mean(np.abs(h - ho) <= EXACT_DEG) >= 0.9999
    d2 = _domain(CASES[3][1])
    outs = horizon_svf_comp_batch([(d.inputs(), args), (d2.inputs(), CASES[3][2])],
                                  elev_walk=_lib.HZ_WALK_BISECT, kernel=kernel)
    np.testing.assert_array_equal(outs[0][0], h)
    np.testing.assert_array_equal(outs[0][1], s)
    h2, s2 = horizon_svf_comp_py(*d2.inputs(), *CASES[3][2], elev_walk=_lib.HZ_WALK_BISECT,
                                 kernel=kernel)
    np.testing.assert_array_equal(outs[1][0], h2)
    np.testing.assert_array_equal(outs[1][1], s2)
