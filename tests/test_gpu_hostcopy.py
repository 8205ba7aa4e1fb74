"""Host entry points with pageable and page-locked caller buffers: outputs
larger than several staging chunks arrive complete and identical."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import horizon_svf_comp_device, horizon_svf_comp_py, synthetic

pytestmark = pytest.mark.gpu


def test_pageable_and_pinned_buffers_give_identical_outputs():
    torch = pytest.importorskip("torch")
    d = synthetic.make_domain(edge_km=0.5, box_km=70.0, seed=31)
    args = (360, 1, 20000.0, 0.2, 1, 2)  # horizon: 360 x ncell x 8 B, several 16 MB chunks
    assert 360 * d.ncell * 8 > 3 * (16 << 20)
    h, s = horizon_svf_comp_py(*d.inputs(), *args)  # numpy: pageable
    pinned = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
              for a in d.inputs()]
    hp, sp = horizon_svf_comp_py(*pinned, *args)
    np.testing.assert_array_equal(h, hp)
    np.testing.assert_array_equal(s, sp)
    t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in d.inputs()]
    hd, sd, _ = horizon_svf_comp_device(*t, *args)
    np.testing.assert_array_equal(h, hd.cpu().numpy())
    np.testing.assert_array_equal(s, sd.cpu().numpy())
    assert np.isfinite(h).all() and (s > 0).all()
