"""Generate the border-distance fixture from the reference's own function.

Runs functions.distance_to_border (functions.py:58-97) of the reference tree
(the first argument, or HZ_REFERENCE_SRC) on seeded synthetic domains and
stores inputs and outputs in border_golden.npz. functions.py imports pyproj at
module level for an unrelated function (observer_perspective); pyproj is not
installed here, so an empty stand-in module is registered under that name
before the import (distance_to_border itself uses only numpy and scipy).

    python tests/golden/make_border_golden.py REFERENCE_TREE
"""
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from horayzon_extpar_gb300 import synthetic  # noqa: E402

CASES = {"a": dict(edge_km=2.5, box_km=80.0, seed=21),
         "b": dict(edge_km=1.0, box_km=30.0, seed=22, face_rotation_deg=17.0),
         "c": dict(edge_km=5.0, box_km=400.0, seed=23, lat0_deg=-33.0, lon0_deg=151.0)}


def load_reference_functions():
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HZ_REFERENCE_SRC")
    if not src:
        raise SystemExit("pass the reference tree as the first argument or set "
                         "HZ_REFERENCE_SRC")
    if "pyproj" not in sys.modules:
        stub = types.ModuleType("pyproj")
        stub.Transformer = None
        sys.modules["pyproj"] = stub
    spec = importlib.util.spec_from_file_location("hz_ref_functions",
                                                  os.path.join(src, "functions.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    ref = load_reference_functions()
    out = {}
    for name, kw in CASES.items():
        d = synthetic.make_domain(**kw)
        cov = d.cells_of_vertex.copy()
        if name == "b":  # a vertex with -2 before valid entries, and a hole
            cov[:, 100] = np.roll(cov[:, 100], 2)
        dist = ref.distance_to_border(d.clon, d.clat, d.vlon, d.vlat, cov)
        for k, v in (("clon", d.clon), ("clat", d.clat), ("vlon", d.vlon), ("vlat", d.vlat),
                     ("cells_of_vertex", cov), ("dist", dist)):
            out["%s_%s" % (name, k)] = v
        print(name, d.ncell, "cells", int(np.any(cov == -2, axis=0).sum()), "border vertices",
              "dist range %.3f-%.3f km" % (dist.min(), dist.max()))
    np.savez_compressed(os.path.join(HERE, "border_golden.npz"), **out)


if __name__ == "__main__":
    main()
