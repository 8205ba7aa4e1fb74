"""The occluder cache of the persistent search (hz_options.occluder_cache):
an upward step of the elevation walk first tests the triangle that hid the
ray one step below. The query is any-hit (mo_lradtopo_horayzon.cpp:446-460),
so a hit there is the traversal's answer: outputs and ray counts are those
of the search without the cache, bit for bit, with fewer node visits."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import _lib, horizon_svf_comp_py, synthetic
from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch

pytestmark = pytest.mark.gpu

CASES = [
    ("c3_recipe", dict(recipe="c3", box_km=80.0, seed=3), (24, 1, 40000.0, 0.2, 1, 2), {}),
    ("rough_bvh2", dict(edge_km=0.5, box_km=40.0, kind="eroded", hmin=500.0, hmax=4200.0,
                        n_features=0, seed=22), (24, 1, 8000.0, 0.2, 1, 2),
     dict(kernel=_lib.HZ_KERNEL_PERSISTENT_BVH2)),
    ("precise", dict(recipe="c1", box_km=200.0, seed=4), (16, 1, 30000.0, 0.2, 1, 1),
     dict(precision=_lib.HZ_PRECISION_LOCAL)),
    ("refine_gt0", dict(recipe="c1", box_km=150.0, seed=5), (12, 0, 20000.0, 0.5, 3, 0), {}),
]


def _domain(kw):
    kw = dict(kw)
    recipe = kw.pop("recipe", None)
    return synthetic.make_config(recipe, **kw) if recipe else synthetic.make_domain(**kw)


@pytest.mark.parametrize("name,kw,args,extra", CASES, ids=[c[0] for c in CASES])
def test_occluder_cache_keeps_results_and_ray_count(name, kw, args, extra):
    d = _domain(kw)
    h0, s0, st0 = horizon_svf_comp_py(*d.inputs(), *args, occluder_cache=False,
                                      count_work=True, return_stats=True, **extra)
    h1, s1, st1 = horizon_svf_comp_py(*d.inputs(), *args, count_work=True,
                                      return_stats=True, **extra)
    np.testing.assert_array_equal(h1, h0)
    np.testing.assert_array_equal(s1, s0)
    assert st1["num_rays"] == st0["num_rays"]
    assert st1["node_visits"] < st0["node_visits"]
    print("%s: node visits per ray %.3f -> %.3f, triangle tests per ray %.3f -> %.3f" % (
        name, st0["node_visits"] / st0["num_rays"], st1["node_visits"] / st1["num_rays"],
        st0["tri_tests"] / st0["num_rays"], st1["tri_tests"] / st1["num_rays"]))


def test_occluder_cache_in_a_batch():
    doms = [(_domain(kw).inputs(), args) for _, kw, args, _ in CASES[:2]]
    off = horizon_svf_comp_batch(doms, occluder_cache=False)
    on = horizon_svf_comp_batch(doms)
    for (h0, s0), (h1, s1) in zip(off, on):
        np.testing.assert_array_equal(h1, h0)
        np.testing.assert_array_equal(s1, s0)
