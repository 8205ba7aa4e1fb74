"""Given warm-start lattice indices (hz_options.start_index): the bracketing
search restarted at the same indices on the GPU and in the CPU oracle casts
the same rays, for every way the search uses them -- the first azimuth of
the reference's chain, azimuth groups (search items of num_hori / G sectors
each, the split that lets one cell's azimuths run on several lanes) and every
azimuth -- so results agree exactly (horizons to 1e-9 deg on >= 99.99 % of
(cell, azimuth), identical bits wherever they agree, SVF to 1e-12 on cells
whose horizons all agree). The terrain is rough on purpose (3.7 km of relief,
8 km search): where visibility is not monotone in elevation a bracket's
result depends on its start, so agreement here tests the restarts
themselves, not only the chain."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import horizon_svf_comp_device, synthetic
from oracle import api as oracle

pytestmark = pytest.mark.gpu

KW = dict(edge_km=0.5, box_km=40.0, kind="eroded", hmin=500.0, hmax=4200.0, n_features=0)
EXACT_DEG = 1e-9


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def _starts(torch, d, args, dev, seed):
    """Start indices near the plain search's own horizons (rounded to the
    start lattice, +-3 steps of noise)."""
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in d.inputs()]
    L = args[0] * args[4]
    raw = torch.empty((L, d.ncell), dtype=torch.int16, device=dev)
    horizon_svf_comp_device(*t, *args, raw_index=raw)
    j = raw.cpu().numpy().astype(np.int64)
    m = np.rint((j + 1) / 2.0).astype(np.int64)
    m += np.random.default_rng(seed).integers(-3, 4, size=m.shape)
    return t, np.clip(m, -200, 200).astype(np.int16)  # beyond [-170, 180]: clamped


@pytest.mark.parametrize("args,mode", [
    ((24, 1, 8000.0, 0.2, 1, 2), dict(groups=1)),
    ((24, 1, 8000.0, 0.2, 1, 2), dict(groups=4)),
    ((24, 1, 8000.0, 0.2, 1, 0), dict(groups=24)),
    ((24, 1, 8000.0, 0.2, 1, 2), dict(start_all=True)),
    ((12, 1, 6000.0, 0.3, 3, 1), dict(groups=6)),   # refine 3: per-group SVF sums
    ((12, 0, 6000.0, 0.2, 2, 2), dict(groups=12)),  # grid_type 0, refine 2
])
def test_given_starts_match_the_oracle(torch, args, mode):
    dev = torch.device("cuda:0")
    d = synthetic.make_domain(seed=21, **KW)
    t, m = _starts(torch, d, args, dev, seed=3)
    kw = dict(mlp_azimuth_groups=mode.get("groups", 1),
              mlp_every_azimuth=mode.get("start_all", False))
    h, s, st = horizon_svf_comp_device(*t, *args, start_index=torch.from_numpy(m).to(dev),
                                       **kw)
    h, s = h.cpu().numpy(), s.cpu().numpy()
    ho, so, sto = oracle.horizon_svf(*d.inputs(), *args, start_index=m, groups=mode.get("groups", 1),
                                     start_all=mode.get("start_all", False))
    dh = np.abs(h - ho)
    same = dh <= EXACT_DEG
    print(args, mode, "identical %.6f, rays gpu %d oracle %d" % (same.mean(), st["num_rays"],
                                                                  sto["num_rays"]))
    assert same.mean() >= 0.9999
    np.testing.assert_array_equal(h[same], ho[same])
    cells = same.all(axis=0)
    np.testing.assert_allclose(s[cells], so[cells], rtol=0, atol=1e-12)
    assert abs(st["num_rays"] - sto["num_rays"]) <= 1e-4 * sto["num_rays"]


def test_given_starts_change_results_only_where_the_start_matters(torch):
    """The same search from the plain chain and from given starts: results
    differ only on (cell, azimuth) where the oracle's results from the two
    starts differ too (visibility not monotone in elevation)."""
    dev = torch.device("cuda:0")
    args = (24, 1, 8000.0, 0.2, 1, 2)
    d = synthetic.make_domain(seed=22, **KW)
    t, m = _starts(torch, d, args, dev, seed=4)
    h0, _, _ = horizon_svf_comp_device(*t, *args)
    h1, _, _ = horizon_svf_comp_device(*t, *args, start_index=torch.from_numpy(m).to(dev),
                                       mlp_every_azimuth=True)
    ho0, _, _ = oracle.horizon_svf(*d.inputs(), *args)
    ho1, _, _ = oracle.horizon_svf(*d.inputs(), *args, start_index=m, start_all=True)
    gpu_diff = np.abs(h1.cpu().numpy() - h0.cpu().numpy()) > EXACT_DEG
    ora_diff = np.abs(ho1 - ho0) > EXACT_DEG
    print("evaluations whose result depends on the start: gpu %d, oracle %d"
          % (gpu_diff.sum(), ora_diff.sum()))
    assert np.mean(gpu_diff == ora_diff) >= 0.9999


def test_start_index_shape_is_checked(torch):
    dev = torch.device("cuda:0")
    d = synthetic.make_domain(seed=23, **KW)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in d.inputs()]
    bad = torch.zeros((23, d.ncell), dtype=torch.int16, device=dev)
    with pytest.raises(ValueError, match="start_index"):
        horizon_svf_comp_device(*t, 24, 1, 8000.0, 0.2, 1, 2, start_index=bad)
