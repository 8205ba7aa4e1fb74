"""Build recipe for the CPU oracle and for the shim-compiled reference.

TEST INFRASTRUCTURE (see ``oracle/__init__.py``).

* ``build_oracle()`` compiles ``hz_oracle.c`` into
  ``oracle/_build/libhz_oracle.so`` with ``-ffp-contract=off`` so that no
  multiply-add is fused (the CUDA path rounds every operation the same way).
* ``build_reference(src)`` compiles the reference's own
  ``mo_lradtopo_horayzon.cpp`` where it lies (``src``, or the folder named
  by the environment variable ``HZ_REFERENCE_SRC``), unmodified, against
  ``shim/`` plus ``ref_entry.cpp`` into ``oracle/_ref/libhorayzon_ref.so``.
  It is skipped when no reference tree is given or found there.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libhz_oracle.so")
REF_SO = os.path.join(REF_DIR, "libhorayzon_ref.so")

_CFLAGS = ["-O3", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
           "-fno-fast-math"]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout,
                                                        r.stderr))


def build_oracle(force=False):
    """Compile the C oracle; returns the path of the shared library."""
    srcs = [os.path.join(HERE, f) for f in ("hz_oracle.c", "hz_oracle.h",
                                            "hz_occlusion.h")]
    if force or _stale(ORACLE_SO, srcs):
        os.makedirs(BUILD_DIR, exist_ok=True)
        tmp = ORACLE_SO + ".%d.tmp" % os.getpid()
        _run(["gcc", "-std=gnu11"] + _CFLAGS + [srcs[0], "-o", tmp, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_source(src=None):
    """The reference tree: ``src``, else $HZ_REFERENCE_SRC; None when neither
    holds mo_lradtopo_horayzon.cpp."""
    src = src or os.environ.get("HZ_REFERENCE_SRC")
    if not src:
        return None
    cpp = os.path.join(src, "mo_lradtopo_horayzon.cpp")
    return src if os.path.exists(cpp) else None


def build_reference(src=None, force=False):
    """Compile the unmodified reference against the shim; None if absent."""
    src = reference_source(src)
    if src is None:
        return None
    ref_cpp = os.path.join(src, "mo_lradtopo_horayzon.cpp")
    shim = os.path.join(HERE, "shim")
    deps = [ref_cpp, os.path.join(src, "mo_lradtopo_horayzon.h"),
            os.path.join(HERE, "ref_entry.cpp"),
            os.path.join(shim, "rtcore_shim.cpp"),
            os.path.join(shim, "embree4", "rtcore.h"),
            os.path.join(shim, "tbb", "parallel_reduce.h"),
            os.path.join(HERE, "hz_occlusion.h")]
    if force or _stale(REF_SO, deps):
        os.makedirs(REF_DIR, exist_ok=True)
        tmp = REF_SO + ".%d.tmp" % os.getpid()
        _run(["g++", "-std=c++17"] + _CFLAGS +
             ["-I", shim, "-I", src, ref_cpp,
              os.path.join(HERE, "ref_entry.cpp"),
              os.path.join(shim, "rtcore_shim.cpp"), "-o", tmp, "-lm"])
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    # python oracle/build.py [--force] [REFERENCE_TREE]
    tree = [a for a in sys.argv[1:] if not a.startswith("--")]
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(tree[0] if tree else None, force="--force" in sys.argv))
