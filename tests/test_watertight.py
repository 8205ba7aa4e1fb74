"""Watertightness of the oracle's ray/triangle test (Woop, Benthin & Wald):
rays through shared vertices and edges of a mesh cannot slip through, and
the BVH gives the brute-force answer on them (the occlusion query of
mo_lradtopo_horayzon.cpp:446-460)."""
import numpy as np
import pytest

from oracle import api as oracle


def lattice_mesh(n=12, z=None):
    """(n+1)^2 integer-lattice vertices (exact in FP32), two triangles per
    square, alternating diagonals; flat (z = 0) or with heights z[i, j]."""
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    h = np.zeros_like(i, dtype=np.float64) if z is None else z
    vert = np.stack([i.ravel(), j.ravel(), h.ravel()], 1).astype(np.float32)
    idx = lambda a, b: a * (n + 1) + b  # noqa: E731
    tris = []
    for a in range(n):
        for b in range(n):
            v00, v10, v01, v11 = idx(a, b), idx(a + 1, b), idx(a, b + 1), idx(a + 1, b + 1)
            if (a + b) % 2 == 0:
                tris += [(v00, v10, v11), (v00, v11, v01)]
            else:
                tris += [(v00, v10, v01), (v10, v11, v01)]
    return vert, np.array(tris, dtype=np.int32)


def grazing_rays(n=12, height=5.0, slant=(0.0, 0.0)):
    """Downward rays aimed exactly at every vertex, edge midpoint and square
    centre of the lattice interior."""
    pts = []
    for a in range(1, n):
        for b in range(1, n):
            pts += [(a, b), (a + 0.5, b), (a, b + 0.5), (a + 0.5, b + 0.5)]
    p = np.array(pts, dtype=np.float64)
    d = np.array([slant[0], slant[1], -1.0])
    org = np.column_stack([p[:, 0] - height * d[0] / -d[2], p[:, 1] - height * d[1] / -d[2],
                           np.full(len(p), height)]).astype(np.float32)
    dirs = np.tile(d, (len(p), 1)).astype(np.float32)
    return org, dirs


@pytest.mark.parametrize("slant", [(0.0, 0.0), (0.25, 0.0), (0.0, -0.5), (0.125, 0.375)])
def test_rays_through_vertices_and_edges_hit(slant):
    vert, vot = lattice_mesh()
    org, dirs = grazing_rays(slant=slant)
    for brute in (False, True):
        hit = oracle.occluded32(vert, vot, org, dirs, 100.0, brute_force=brute)
        assert hit.all(), "%d rays slipped through" % (~hit).sum()


def test_grazing_rays_on_relief_agree_with_brute_force():
    rng = np.random.default_rng(7)
    z = rng.integers(-3, 4, (13, 13)).astype(np.float64)  # integer heights: exact
    vert, vot = lattice_mesh(z=z)
    org, dirs = grazing_rays(height=10.0, slant=(0.25, -0.125))
    a = oracle.occluded32(vert, vot, org, dirs, 100.0)
    b = oracle.occluded32(vert, vot, org, dirs, 100.0, brute_force=True)
    np.testing.assert_array_equal(a, b)
    # A ray that goes from above the highest to below the lowest vertex
    # inside the mesh's footprint crosses the (closed, watertight) surface.
    t_low = (org[:, 2] - (z.min() - 1.0)) / -dirs[:, 2]
    end = org + t_low[:, None] * dirs
    inside = ((org[:, :2] >= 0.5) & (org[:, :2] <= 11.5) & (end[:, :2] >= 0.5)
              & (end[:, :2] <= 11.5)).all(1)
    assert inside.sum() > 300 and a[inside].all()
    # Rays that run inside the plane of a flat face (det == 0) do not hit it.
    vert0, vot0 = lattice_mesh()
    org = np.array([[0.5, 3.0, 0.0], [3.0, 0.5, 0.0]], dtype=np.float32)
    dirs = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], dtype=np.float32)
    np.testing.assert_array_equal(oracle.occluded32(vert0, vot0, org, dirs, 50.0),
                                  oracle.occluded32(vert0, vot0, org, dirs, 50.0, True))


def test_tfar_bound_is_inclusive_and_t_positive():
    vert, vot = lattice_mesh(n=4)
    org = np.array([[2.25, 1.5, 3.0], [2.25, 1.5, 3.0], [2.25, 1.5, 0.0]], dtype=np.float32)
    dirs = np.array([[0, 0, -1], [0, 0, -1], [0, 0, 1]], dtype=np.float32)
    # hit at t = 3 with tfar 3 (inclusive), not with tfar 2.9; an origin on
    # the surface looking up (t = 0 is excluded).
    hit = [oracle.occluded32(vert, vot, org[k:k + 1], dirs[k:k + 1], tf)[0]
           for k, tf in ((0, 3.0), (1, 2.9), (2, 10.0))]
    assert hit == [True, False, False]
