"""Generate the golden fixtures in this folder from the reference itself.

Run where the reference tree is, naming it with HZ_REFERENCE_SRC or as the
first argument. For every case it builds a seeded synthetic domain and
records the inputs, the outputs of the unmodified reference
(mo_lradtopo_horayzon.cpp compiled against the project's Embree/TBB
stand-ins, oracle/_ref) and the reference's triangle mesh
(build_triangle_mesh). The mesh is also checked against the reference's own
pure-Python builders (development.py:27-179), loaded function by function
because that module imports xarray at the top.

    python tests/golden/make_golden.py REFERENCE_TREE
"""
import ast
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from horayzon_extpar_gb300 import synthetic  # noqa: E402
from oracle import api, build  # noqa: E402

# name: (domain kwargs, (num_hori, grid_type, dist_search, ray_org_elev, refine, svf))
CASES = {
    "g1_n24_r1_svf2": (dict(edge_km=2.5, box_km=80.0, seed=11),
                       (24, 1, 40000.0, 0.2, 1, 2)),
    "g0_n24_r1_svf0": (dict(edge_km=2.5, box_km=80.0, seed=11),
                       (24, 0, 40000.0, 0.2, 1, 0)),
    "g1_n16_r10_svf1": (dict(edge_km=2.0, box_km=50.0, seed=12, kind="fbm_ridged",
                             hmin=200.0, hmax=4800.0, hurst=0.7, n_features=0),
                        (16, 1, 20000.0, 0.5, 10, 1)),
    "g1_n1440_r1_svf2": (dict(edge_km=1.0, box_km=8.0, seed=13, kind="fbm_ridges",
                              hmin=0.0, hmax=4500.0, n_features=3),
                         (1440, 1, 5000.0, 0.2, 1, 2)),
    "g0_n4_r50_svf0_min": (dict(edge_km=1.0, box_km=10.0, seed=14),
                           (4, 0, 1000.0, 0.1, 50, 0)),
    "g1_n24_flat": (dict(edge_km=2.5, box_km=40.0, seed=15, hmin=500.0, hmax=500.0,
                         n_features=0),
                    (24, 1, 40000.0, 0.2, 1, 2)),
    "g1_n48_r1_svf2_rot": (dict(edge_km=1.5, box_km=40.0, seed=16, face_rotation_deg=17.0,
                                kind="eroded", hmin=500.0, hmax=4200.0, n_features=0),
                           (48, 1, 30000.0, 0.2, 1, 2)),
}


def load_development_builders(src):
    """triangle_mesh_circ / triangle_mesh_circ_vert from development.py."""
    path = os.path.join(src, "development.py")
    tree = ast.parse(open(path).read())
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef)
            and n.name in ("triangle_mesh_circ", "triangle_mesh_circ_vert")]
    ns = {"np": np}
    exec(compile(ast.Module(body=keep, type_ignores=[]), path, "exec"), ns)
    return ns["triangle_mesh_circ"], ns["triangle_mesh_circ_vert"]


def main():
    src = build.reference_source(sys.argv[1] if len(sys.argv) > 1 else None)
    if src is None:
        raise SystemExit("reference sources not found: pass the reference tree as the "
                         "first argument or set HZ_REFERENCE_SRC")
    build.build_reference(src)
    tm_circ, tm_circ_vert = load_development_builders(src)
    for name, (dkw, args) in CASES.items():
        dom = synthetic.make_domain(**dkw)
        ref = api.reference_horizon_svf(*dom.inputs(), *args)
        mlon, mlat, mh, vot = api.reference_build_mesh(*dom.inputs(), args[1])
        if args[1] == 0:
            dev_vot = tm_circ(dom.clon, dom.clat, dom.vlon, dom.vlat, dom.cells_of_vertex)
        else:
            dev_vot = tm_circ_vert(dom.clon, dom.clat, dom.hsurf, dom.vlon, dom.vlat,
                                   dom.cells_of_vertex)[0]
        if not np.array_equal(dev_vot.T, vot):
            raise SystemExit("%s: development.py mesh differs from the C++ mesh" % name)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            clon=dom.clon, clat=dom.clat, hsurf=dom.hsurf, vlon=dom.vlon, vlat=dom.vlat,
            cells_of_vertex=dom.cells_of_vertex, args=np.array(args, dtype=np.float64),
            horizon=ref[0], skyview=ref[1], mesh_vot=vot, mesh_lon=mlon, mesh_lat=mlat,
            mesh_h=mh)
        print("%-22s ncell=%6d nvert=%6d ntri=%6d horizon[%g, %g] svf[%.4f, %.4f]"
              % (name, dom.ncell, dom.nvertex, vot.shape[0], ref[0].min(), ref[0].max(),
                 ref[1].min(), ref[1].max()))


if __name__ == "__main__":
    main()
