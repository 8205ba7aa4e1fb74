"""The GPU any-hit query (hz_occluded32: the search's BVH build, traversal
and watertight test on arbitrary rays) against the oracle's BVH and brute
force, hit for hit."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import synthetic
from horayzon_extpar_gb300.horizon_svf import occluded32
from oracle import api as oracle
from test_watertight import grazing_rays, lattice_mesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tree,leaf_size", [(0, 0), (0, 1), (0, 4), (0, 8), (1, 0), (1, 3)])
def test_gpu_random_soup_equals_brute_force(tree, leaf_size):
    rng = np.random.default_rng(4)
    n = 300
    vert = rng.uniform(-100, 100, (n, 3)).astype(np.float32)
    vot = rng.integers(0, n, (400, 3)).astype(np.int32)
    org = rng.uniform(-120, 120, (4000, 3)).astype(np.float32)
    d = rng.normal(size=(4000, 3)).astype(np.float32)
    g = occluded32(vert, vot, org, d, 150.0, tree=tree, leaf_size=leaf_size)
    b = oracle.occluded32(vert, vot, org, d, 150.0, brute_force=True)
    np.testing.assert_array_equal(g, b)
    assert 0 < g.sum() < g.size


@pytest.mark.parametrize("slant", [(0.0, 0.0), (0.25, 0.0), (0.125, 0.375)])
@pytest.mark.parametrize("tree", [0, 1])
def test_gpu_rays_through_vertices_and_edges_hit(slant, tree):
    vert, vot = lattice_mesh()
    org, dirs = grazing_rays(slant=slant)
    assert occluded32(vert, vot, org, dirs, 100.0, tree=tree).all()
    rng = np.random.default_rng(7)
    z = rng.integers(-3, 4, (13, 13)).astype(np.float64)
    vert, vot = lattice_mesh(z=z)
    org, dirs = grazing_rays(height=10.0, slant=slant)
    np.testing.assert_array_equal(occluded32(vert, vot, org, dirs, 100.0, tree=tree),
                                  oracle.occluded32(vert, vot, org, dirs, 100.0,
                                                    brute_force=True))


@pytest.mark.parametrize("tree", [0, 1])
def test_gpu_terrain_rays_equal_oracle(tree):
    """Near-horizontal rays from above the cells of a synthetic domain, as the
    search casts them, against the domain's FP32 ENU mesh."""
    d = synthetic.make_domain(edge_km=2.0, box_km=60.0, seed=12)
    _, e32, vot = oracle.mesh_enu(*d.inputs(), 1)
    rng = np.random.default_rng(3)
    k = rng.integers(0, d.ncell, 20000)
    org = e32[k] + np.float32([0.0, 0.0, 0.2])
    az = rng.uniform(0, 2 * np.pi, k.size)
    el = np.deg2rad(rng.uniform(-10, 20, k.size))
    dirs = np.column_stack([np.cos(el) * np.sin(az), np.cos(el) * np.cos(az),
                            np.sin(el)]).astype(np.float32)
    g = occluded32(e32, vot, org, dirs, 40000.0, tree=tree)
    np.testing.assert_array_equal(g, oracle.occluded32(e32, vot, org, dirs, 40000.0))
    assert 0.05 < g.mean() < 0.95


def test_gpu_occlusion_edge_cases():
    vert, vot = lattice_mesh(n=4)
    org, dirs = grazing_rays(n=4)
    assert occluded32(vert, vot[:0], org, dirs, 100.0).sum() == 0  # no triangles
    assert occluded32(vert, vot, org[:0], dirs[:0], 100.0).size == 0  # no rays
    assert occluded32(vert, vot[:1], org, dirs, 100.0).sum() >= 1  # a single triangle
    bad = vot.copy()
    bad[2, 1] = vert.shape[0]
    with pytest.raises(ValueError, match="out of range"):
        occluded32(vert, bad, org, dirs, 100.0)
