"""Border-distance oracle against the fixture made by the reference's own
functions.distance_to_border (tests/golden/make_border_golden.py)."""
import os

import numpy as np
import pytest

from oracle import border_ref

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "border_golden.npz")


def cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("_", 1)[0] for k in g.files})
    return [(n, {k.split("_", 1)[1]: g[k] for k in g.files if k.startswith(n + "_")})
            for n in names]


@pytest.mark.parametrize("name,case", cases())
def test_oracle_matches_reference_fixture(name, case):
    d = border_ref.distance_to_border(case["clon"], case["clat"], case["vlon"], case["vlat"],
                                      case["cells_of_vertex"])
    np.testing.assert_allclose(d, case["dist"], rtol=1e-12, atol=0)


def test_oracle_without_border_is_infinite():
    cov = np.zeros((6, 4), dtype=np.int32)
    d = border_ref.distance_to_border(np.zeros(3), np.zeros(3), np.zeros(4), np.zeros(4), cov)
    assert np.isinf(d).all()
