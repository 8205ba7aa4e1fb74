"""A checked build (-DHZ_CHECKED=1; compute-sanitizer is closed on this
pool): the search validates node references, leaf triangle ranges and
output indices on the device, records the first violation and fails the
call instead of touching memory out of bounds. The parity cases run clean
through it, on both trees, refined azimuths, the local-precision mode and a
batch."""
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

SCRIPT = textwrap.dedent("""
    import numpy as np
    from horayzon_extpar_gb300 import horizon_svf_comp_py, synthetic
    from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch
    from oracle import api as oracle
    cases = [(dict(edge_km=2.5, box_km=60.0, seed=21), (24, 1, 40000.0, 0.2, 1, 2), {}),
             (dict(edge_km=1.0, box_km=25.0, seed=22), (36, 0, 15000.0, 0.2, 3, 0),
              {"kernel": 2}),
             (dict(edge_km=2.0, box_km=40.0, seed=24), (24, 1, 40000.0, 0.2, 1, 1),
              {"leaf_size": 8}),
             (dict(edge_km=2.0, box_km=40.0, seed=23), (16, 1, 30000.0, 0.5, 1, 1),
              {"precision": 1})]
    for dkw, args, kw in cases:
        d = synthetic.make_domain(**dkw)
        h, s = horizon_svf_comp_py(*d.inputs(), *args, **kw)
        assert np.isfinite(h).all() and (s > 0).all() and (s <= 1).all()
        if "precision" not in kw:
            ho, so, _ = oracle.horizon_svf(*d.inputs(), *args)
            assert np.mean(np.abs(h - ho) <= 1e-9) >= 0.999
            assert np.abs(s - so).max() <= 1e-3
    batch = synthetic.make_batch(n_domains=4, seed=3, min_cells=300, max_cells=3000)
    outs = horizon_svf_comp_batch([(d.inputs(), a) for d, a in batch])
    assert all(np.isfinite(h).all() for h, _ in outs)
    print("checked build: clean")
""")


def test_gpu_checked_build_runs_clean(tmp_path):
    from horayzon_extpar_gb300 import _build
    lib = _build.build_checked(str(tmp_path / "checked"))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, HZ_LIBRARY=lib,
               PYTHONPATH=root + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=root, env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "checked build: clean" in r.stdout
