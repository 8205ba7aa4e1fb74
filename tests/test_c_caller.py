"""The C ABI from C itself (tests/c_caller/horizon_main.c): the header
compiles as strict C99 and the program links against the library (CPU); on
a GPU, the reference prototype, the status variant and the Fortran-buffer
variant give the Python drop-in's results."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from horayzon_extpar_gb300 import _build, horizon_svf_comp_py, synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_caller", "horizon_main.c")


def build_caller(out_dir):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib_dir = os.path.dirname(_build.LIB_PATH)
    if not os.path.exists(_build.LIB_PATH):
        pytest.skip("library not built")
    exe = os.path.join(out_dir, "horizon_main")
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-O1",
           "-I" + os.path.join(ROOT, "include"), SRC, "-o", exe, "-L" + lib_dir,
           "-lhorayzon_gb300", "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_c_caller_compiles_and_links(tmp_path):
    assert os.access(build_caller(str(tmp_path)), os.X_OK)


@pytest.mark.gpu
def test_gpu_c_caller_matches_python(tmp_path):
    exe = build_caller(str(tmp_path))
    d = synthetic.make_domain(edge_km=2.5, box_km=40.0, seed=31)
    for name, a in zip(("clon", "clat", "hsurf", "vlon", "vlat", "cells_of_vertex"),
                       d.inputs()):
        np.ascontiguousarray(a).tofile(str(tmp_path / (name + ".bin")))
    (tmp_path / "sizes.txt").write_text("%d %d\n" % (d.ncell, d.nvertex))
    args = (24, 1, 40000.0, 0.2, 2, 2)
    r = subprocess.run([exe, str(tmp_path)] + [str(a) for a in args], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    h, s = horizon_svf_comp_py(*d.inputs(), *args)
    for k in (1, 2, 3):
        hc = np.fromfile(str(tmp_path / ("horizon%d.bin" % k))).reshape(h.shape)
        sc = np.fromfile(str(tmp_path / ("skyview%d.bin" % k)))
        np.testing.assert_array_equal(hc, h)
        np.testing.assert_array_equal(sc, s)
    log = (tmp_path / "log.txt").read_text()
    assert "horizon" in log.lower() and len(log) > 100
