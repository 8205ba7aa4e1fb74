import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    """Horizon/SVF fixtures (make_golden.py); border_golden.npz is separate."""
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "g*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    d = {k: z[k] for k in z.files}
    a = d["args"]
    d["args"] = (int(a[0]), int(a[1]), float(a[2]), float(a[3]), int(a[4]), int(a[5]))
    d["inputs"] = (d["clon"], d["clat"], d["hsurf"], d["vlon"], d["vlat"],
                   d["cells_of_vertex"])
    return d


@pytest.fixture(scope="session")
def small_domain():
    from horayzon_extpar_gb300 import synthetic
    return synthetic.make_domain(edge_km=2.5, box_km=60.0, seed=5)
