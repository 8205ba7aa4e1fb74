"""Parity on a mid-size domain of the 500 m benchmark recipe (fBm H 0.7 +
ridged noise, 200-4800 m, 500 m grid) on a 150 x 150 km box (~195k cells,
~585k triangles, nhori 24, dist_search 40 km): the default search (4-wide
tree, reference arithmetic) against the CPU oracle with the reference's
arithmetic, and the local-precision mode against the FP64 oracle, each on a
fixed random cell sample. Bars as the parity tests state them: |dhorizon| <=
0.25 deg on >= 99.9 % of (cell, azimuth), |dSVF| <= 1e-3; the reference
arithmetic is also required to be exact (1e-9 deg) on >= 99.9 %."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import _lib, horizon_svf_comp_py, synthetic
from oracle import api as oracle

pytestmark = pytest.mark.gpu

ARGS = (24, 1, 40000.0, 0.2, 1, 2)  # the benchmark's num_hori ... svf_type
HORIZON_TOL_DEG = 0.25
SVF_TOL = 1e-3
EXACT_DEG = 1e-9


@pytest.fixture(scope="module")
def domain():
    return synthetic.make_config("c3", seed=0, box_km=150.0)


def _sample(d, n, seed):
    return np.sort(np.random.default_rng(seed).choice(d.ncell, n, replace=False))


def _compare(h, s, h_or, s_or, cells):
    dh = np.abs(h[:, cells] - h_or[:, cells])
    ds = np.abs(s[cells] - s_or[cells])
    return float(np.mean(dh <= HORIZON_TOL_DEG)), float(np.mean(dh <= EXACT_DEG)), float(ds.max())


def test_default_search_matches_oracle_on_500m_recipe(domain):
    d = domain
    assert d.ncell > 150000
    h, s, st = horizon_svf_comp_py(*d.inputs(), *ARGS, return_stats=True)
    cells = _sample(d, 30000, 7)
    h_or, s_or, _ = oracle.horizon_svf(*d.inputs(), *ARGS, cells=cells)
    within, exact, max_svf = _compare(h, s, h_or, s_or, cells)
    print("500 m recipe, 150 km box: %d cells, %d triangles; within 0.25 deg %.6f, "
          "identical %.6f, max |dSVF| %.3g" % (d.ncell, st["n_tri"], within, exact, max_svf))
    assert within >= 0.999
    assert exact >= 0.999
    assert max_svf <= SVF_TOL


def test_local_precision_matches_fp64_oracle_on_500m_recipe(domain):
    d = domain
    h, s = horizon_svf_comp_py(*d.inputs(), *ARGS, precision=_lib.HZ_PRECISION_LOCAL)
    cells = _sample(d, 10000, 8)
    h64, s64, _ = oracle.horizon_svf(*d.inputs(), *ARGS, cells=cells, precision=1)
    within, exact, max_svf = _compare(h, s, h64, s64, cells)
    print("local precision vs FP64 oracle: within 0.25 deg %.6f, identical %.6f, "
          "max |dSVF| %.3g" % (within, exact, max_svf))
    assert within >= 0.999
    assert max_svf <= SVF_TOL
