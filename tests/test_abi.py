"""The C ABI library loads without a GPU and exports every function that
include/horayzon_gb300.h declares; the Python layer raises the reference's
exceptions before reaching the library (CPU only, no compute calls)."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from horayzon_extpar_gb300 import _lib, horizon_svf_comp_py, synthetic


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b([a-z_][a-z0-9_]*)\s*\(", src,
                            flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "for", "sizeof")))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    assert set(names) == set(_lib.EXPORTED_SYMBOLS), names


def _struct_fields(name):
    """Member names of `typedef struct { ... } name;` in the public header."""
    src = open(os.path.join(ROOT, "include", "horayzon_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    end = src.index("} %s;" % name)
    body = src[src.rindex("typedef struct", 0, end):end]
    body = body[body.index("{") + 1:]
    names = []
    for decl in body.split(";"):
        parts = [re.sub(r"\[[^\]]*\]", "", p).strip() for p in decl.split(",")]
        if not parts[0]:
            continue
        names += [re.findall(r"\w+", p)[-1] for p in parts]
    return names


def test_python_structs_mirror_the_header():
    """ctypes mirrors of hz_options, hz_stats and hz_domain: the same members
    in the same order as the header."""
    import ctypes as C
    for cls, name in ((_lib.Options, "hz_options"), (_lib.Stats, "hz_stats"),
                      (_lib.Domain, "hz_domain")):
        assert [f for f, _ in cls._fields_] == _struct_fields(name), name
    assert C.sizeof(_lib.Options) > 0


def test_default_options_from_the_library():
    """hz_default_options (no GPU needed) fills the struct the Python layer
    passes: its size field is the ctypes struct's size, and the documented
    defaults hold."""
    import ctypes as C
    o = _lib.Options()
    _lib.load().hz_default_options(C.byref(o))
    assert o.size == C.sizeof(_lib.Options)
    assert o.device == -1 and o.elev_floor_deg == -85.0
    assert o.occluder_cache == 1 and o.elev_walk == _lib.HZ_WALK_REFERENCE
    assert o.advance_min == 0 and o.leaf_min == 0  # 0: the library's defaults


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.hz_version() == 100


@pytest.fixture(scope="module")
def dom():
    return synthetic.make_domain(edge_km=5.0, box_km=40.0, seed=1)


ARGS = (24, 1, 40000.0, 0.2, 1, 2)


@pytest.mark.parametrize("change,exc,msg", [
    (dict(num_hori=3), ValueError, "'num_hori' must be in the range [4, 1440]"),
    (dict(num_hori=1441), ValueError, "'num_hori' must be in the range [4, 1440]"),
    (dict(grid_type=2), ValueError, "'grid_type' must be in the range [0, 1]"),
    (dict(dist_search=999.0), ValueError, "'dist_search' must be in the range [1'000, 500'000] km"),
    (dict(dist_search=500001.0), ValueError, "'dist_search' must be in the range"),
    (dict(ray_org_elev=0.05), TypeError, "Minimal allowed value for 'ray_org_elev' is 0.1 m"),
    (dict(refine_factor=0), ValueError, "'refine_factor' must be in the range [1, 50]"),
    (dict(refine_factor=51), ValueError, "'refine_factor' must be in the range [1, 50]"),
    (dict(svf_type=3), ValueError, "'svf_type' must be in the range [0, 2]"),
])
def test_argument_checks_match_reference(dom, change, exc, msg):
    names = ("num_hori", "grid_type", "dist_search", "ray_org_elev", "refine_factor",
             "svf_type")
    args = dict(zip(names, ARGS))
    args.update(change)
    with pytest.raises(exc, match=re.escape(msg)):
        horizon_svf_comp_py(*dom.inputs(), *[args[n] for n in names])


def test_array_checks_match_reference(dom):
    c = dom.inputs()
    with pytest.raises(ValueError, match="Inconsistent lengths of input arrays 'clon'"):
        horizon_svf_comp_py(c[0][:-1], *c[1:], *ARGS)
    with pytest.raises(ValueError, match="Inconsistent lengths of input arrays 'vlon'"):
        horizon_svf_comp_py(*c[:3], c[3][:-1], *c[4:], *ARGS)
    with pytest.raises(ValueError, match="First dimension of 'cells_of_vertex' must have length 6"):
        horizon_svf_comp_py(*c[:5], c[5][:5], *ARGS)
    # The index check comes before the range checks of the scalar arguments
    # (pyx:88-90 before :91-103); with a valid call the GPU makes it
    # (test_gpu_parity.test_gpu_bad_indices_raise_reference_error).
    bad = c[5].copy()
    bad[0, 0] = dom.ncell
    with pytest.raises(ValueError, match="Indices of 'cells_of_vertex' out of range"):
        horizon_svf_comp_py(*c[:5], bad, 3, *ARGS[1:])
    bad[0, 0] = -1
    with pytest.raises(ValueError, match="Indices of 'cells_of_vertex' out of range"):
        horizon_svf_comp_py(*c[:5], bad, *ARGS[:5], 7)
    with pytest.raises(ValueError, match="Buffer dtype mismatch"):
        horizon_svf_comp_py(c[0].astype(np.float32), *c[1:], *ARGS)
    with pytest.raises(ValueError, match="Buffer dtype mismatch"):
        horizon_svf_comp_py(*c[:5], c[5].astype(np.int64), *ARGS)
    with pytest.raises(ValueError, match="wrong number of dimensions"):
        horizon_svf_comp_py(c[0][None, :], *c[1:], *ARGS)
    with pytest.raises(TypeError, match="incorrect type"):
        horizon_svf_comp_py(list(c[0]), *c[1:], *ARGS)
    with pytest.raises(TypeError):
        horizon_svf_comp_py(*c, 24.5, *ARGS[1:])
    e = np.empty(0)
    with pytest.raises(IndexError):
        horizon_svf_comp_py(e, e, e, *c[3:5], np.full((6, c[3].size), -2, np.int32), *ARGS)
