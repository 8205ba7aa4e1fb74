"""Seeded random sweep of the argument space against the oracle: grid
spacing, terrain kind, latitude, grid rotation and every scalar argument of
horizon_svf_comp (num_hori 4-1440, grid_type, dist_search 1-500 km,
ray_org_elev, refine_factor 1-50, svf_type), on small domains."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import horizon_svf_comp_py, synthetic
from oracle import api as oracle
from test_gpu_parity import assert_parity

pytestmark = pytest.mark.gpu

KINDS = ["fbm_peaks", "fbm_ridges", "fbm_ridged", "eroded"]


def case(seed):
    rng = np.random.default_rng(1000 + seed)
    edge = float(rng.choice([0.25, 0.5, 1.0, 2.0, 3.0]))
    cells_side = int(rng.integers(15, 60))
    dkw = dict(edge_km=edge, box_km=edge * cells_side, kind=KINDS[seed % len(KINDS)],
               hmin=float(rng.uniform(0, 1000)), seed=seed,
               lat0_deg=float(rng.uniform(-70, 70)), lon0_deg=float(rng.uniform(-180, 180)),
               face_rotation_deg=float(rng.uniform(0, 60)))
    dkw["hmax"] = dkw["hmin"] + float(rng.uniform(100, 4000))
    num_hori = int(rng.choice([4, 8, 16, 24, 36, 48, 90, 360]))
    refine = int(rng.choice([1, 1, 2, 3, 5, 10])) if num_hori <= 90 else 1
    args = (num_hori, int(rng.integers(0, 2)),
            float(rng.choice([1000.0, 5000.0, 20000.0, 40000.0, 150000.0, 500000.0])),
            float(rng.choice([0.1, 0.2, 1.0, 10.0])), refine, int(rng.integers(0, 3)))
    return dkw, args


@pytest.mark.parametrize("seed", range(24))
def test_gpu_random_configuration_matches_oracle(seed):
    """Host entry, device entry or a two-domain batch (by seed), with the
    4-wide, binary or per-cell search (by seed)."""
    dkw, args = case(seed)
    d = synthetic.make_domain(**dkw)
    kernel = (0, 2, 1)[seed % 3]
    entry = seed % 4
    ho, so, sto = oracle.horizon_svf(*d.inputs(), *args)
    if entry == 1:
        torch = pytest.importorskip("torch")
        from horayzon_extpar_gb300 import horizon_svf_comp_device
        t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in d.inputs()]
        h, s, st = horizon_svf_comp_device(*t, *args, kernel=kernel)
        h, s = h.cpu().numpy(), s.cpu().numpy()
    elif entry == 2:
        from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch
        dkw2, args2 = case(seed + 100)
        d2 = synthetic.make_domain(**dkw2)
        outs, st = horizon_svf_comp_batch([(d2.inputs(), args2), (d.inputs(), args)],
                                          kernel=kernel, return_stats=True)
        h, s = outs[1]
        h2, s2 = outs[0]
        ho2, so2, sto2 = oracle.horizon_svf(*d2.inputs(), *args2)
        assert_parity(h2, s2, ho2, so2)
        sto = dict(sto, num_rays=sto["num_rays"] + sto2["num_rays"])
    else:
        h, s, st = horizon_svf_comp_py(*d.inputs(), *args, kernel=kernel, return_stats=True)
    assert_parity(h, s, ho, so)
    if entry != 2:
        assert st["n_tri"] == sto["n_tri"]
    assert abs(st["num_rays"] - sto["num_rays"]) <= 0.001 * sto["num_rays"]
