"""The oracle's restatement of the walk below the clip by doubling and
bisection (the library's HZ_WALK_BISECT) against its restatement of the
reference's step walk (mo_lradtopo_horayzon.cpp:536-547), on the CPU: the
same horizons wherever visibility is monotone in elevation, fewer rays.
Small domains whose border cells look out over the void exercise the walk
down towards -85 deg."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import synthetic
from oracle import api as oracle

EXACT_DEG = 1e-9
CASES = [
    (dict(edge_km=1.0, box_km=30.0, seed=51), (24, 1, 20000.0, 0.2, 1, 2)),
    (dict(edge_km=0.5, box_km=15.0, kind="eroded", hmin=500.0, hmax=4200.0, n_features=0,
          seed=52), (16, 0, 8000.0, 0.5, 2, 1)),
]


@pytest.mark.parametrize("kw,args", CASES)
def test_oracle_bisect_walk_keeps_the_step_walk_results(kw, args):
    d = synthetic.make_domain(**kw)
    h0, s0, st0 = oracle.horizon_svf(*d.inputs(), *args)
    h1, s1, st1 = oracle.horizon_svf(*d.inputs(), *args, bisect_walk=True)
    same = np.abs(h1 - h0) <= EXACT_DEG
    assert same.mean() >= 0.999, same.mean()
    cells = same.all(axis=0)
    np.testing.assert_allclose(s1[cells], s0[cells], rtol=0, atol=1e-12)
    assert np.abs(s1 - s0).max() <= 1e-3
    assert st1["num_rays"] < st0["num_rays"]
