"""GB300-native (sm_103a) terrain horizon and sky view factor.

A drop-in for the HORAYZON/EXTPAR ``horizon_svf.horizon_svf_comp_py`` call:
ICON cell and vertex coordinates plus cell elevations in, per-cell horizon
angles for ``num_hori`` azimuths and the sky view factor out. Mesh assembly,
LBVH build and the bracketing horizon search run as hand-written CUDA kernels
in ``libhorayzon_gb300.so`` (C ABI: ``include/horayzon_gb300.h``).
"""
from .horizon_svf import (build_mesh, horizon_svf_comp_batch, horizon_svf_comp_device,
                          horizon_svf_comp_py, mesh_enu32)

__all__ = ["horizon_svf_comp_py", "horizon_svf_comp_device", "horizon_svf_comp_batch",
           "build_mesh", "mesh_enu32"]
__version__ = "1.0.0"
