"""GPU border distance (hz_distance_to_border) against the fixture made by
the reference's functions.distance_to_border, and its device variant."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import synthetic
from horayzon_extpar_gb300.border import distance_to_border, distance_to_border_device
from oracle import border_ref
from test_border import cases

pytestmark = pytest.mark.gpu


# The device sin/cos differ from numpy's in the last bit of ~6371 km ECEF
# coordinates (1e-12 km); for chords of a few hundred metres that is a
# relative 2e-12. Tolerance: 1e-12 relative + 1e-9 km (1 micrometre).
RTOL, ATOL = 1e-12, 1e-9


@pytest.mark.parametrize("name,case", cases())
def test_gpu_border_matches_reference_fixture(name, case):
    d = distance_to_border(case["clon"], case["clat"], case["vlon"], case["vlat"],
                           case["cells_of_vertex"])
    np.testing.assert_allclose(d, case["dist"], rtol=RTOL, atol=ATOL)


def test_gpu_border_device_and_large_domain():
    torch = pytest.importorskip("torch")
    d = synthetic.make_domain(edge_km=1.0, box_km=200.0, seed=4)
    ref = border_ref.distance_to_border(d.clon, d.clat, d.vlon, d.vlat, d.cells_of_vertex)
    host = distance_to_border(d.clon, d.clat, d.vlon, d.vlat, d.cells_of_vertex)
    np.testing.assert_allclose(host, ref, rtol=RTOL, atol=ATOL)
    t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in
         (d.clon, d.clat, d.vlon, d.vlat, d.cells_of_vertex)]
    dev = distance_to_border_device(*t).cpu().numpy()
    np.testing.assert_array_equal(dev, host)


def test_gpu_border_without_border_vertices():
    cov = np.zeros((6, 4), dtype=np.int32)
    d = distance_to_border(np.zeros(3), np.zeros(3), np.zeros(4), np.zeros(4), cov)
    assert np.isinf(d).all()
