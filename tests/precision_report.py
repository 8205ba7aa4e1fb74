"""Error of the GPU search against the FP64 oracle on the benchmark workload
(the report behind the precision figures; run on a GPU machine):

    python tests/precision_report.py [box_km]

Both arithmetic modes of the library (the reference's global FP32 frame and
HZ_PRECISION_LOCAL) run on the 500 m workload; the oracle recomputes a
random sample of 20,000 cells with FP64 vertices, rays and triangle test.
Cells whose 40 km search reaches the domain edge (functions.py:58-97,
verification.py:302-304) are also reported separately. Prints one JSON
object.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

ARGS = (24, 1, 40000.0, 0.2, 1, 2)  # the benchmark's num_hori ... svf_type


def main(box_km=600.0, sample=20000):
    import torch

    from horayzon_extpar_gb300 import _lib, horizon_svf_comp_device, synthetic
    from horayzon_extpar_gb300.border import distance_to_border
    from oracle import api as oracle

    dom = synthetic.make_config("c3", seed=0, box_km=box_km)
    d_in = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in dom.inputs()]
    h_ref, s_ref, _ = horizon_svf_comp_device(*d_in, *ARGS)
    h_loc, s_loc, _ = horizon_svf_comp_device(*d_in, *ARGS, precision=_lib.HZ_PRECISION_LOCAL)
    h_ref, s_ref = h_ref.cpu().numpy(), s_ref.cpu().numpy()
    h_loc, s_loc = h_loc.cpu().numpy(), s_loc.cpu().numpy()
    cells = np.sort(np.random.default_rng(7).choice(dom.ncell, min(sample, dom.ncell),
                                                    replace=False))
    h64, s64, _ = oracle.horizon_svf(*dom.inputs(), *ARGS, precision=1, cells=cells)
    dist = distance_to_border(dom.clon, dom.clat, dom.vlon, dom.vlat, dom.cells_of_vertex)
    inner = dist[cells] >= ARGS[2] * 1e-3

    def stats(h, s):
        dh = np.abs(h[:, cells] - h64[:, cells])
        ds = np.abs(s[cells] - s64[cells])
        return {"frac_evals_differing": float(np.mean(dh > 1e-9)),
                "max_abs_deg": float(dh.max()), "mean_abs_deg": float(dh.mean()),
                "max_abs_svf": float(ds.max()), "mean_abs_svf": float(ds.mean()),
                "border_masked": {"cells": int(inner.sum()),
                                  "frac_evals_differing": float(np.mean(dh[:, inner] > 1e-9)),
                                  "max_abs_deg": float(dh[:, inner].max()),
                                  "max_abs_svf": float(ds[inner].max())}}

    print(json.dumps({"workload": "c3 500 m, %g x %g km, nhori 24" % (box_km, box_km),
                      "oracle": "FP64 vertices, rays and triangle test (oracle/hz_oracle.c)",
                      "sample_cells": int(cells.size),
                      "reference_frame_vs_fp64": stats(h_ref, s_ref),
                      "local_frame_vs_fp64": stats(h_loc, s_loc)}))


if __name__ == "__main__":
    main(float(sys.argv[1]) if len(sys.argv) > 1 else 600.0)
