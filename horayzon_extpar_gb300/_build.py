"""In-tree build of libhorayzon_gb300.so for sm_103a (nvcc, no torch needed).

Each ``csrc/*.cu`` file compiles to an object in parallel; the objects link
into ``horayzon_extpar_gb300/_lib/libhorayzon_gb300.so``. Every unit uses
``-fmad=false`` (device) and ``-ffp-contract=off`` (host): the horizon search
reproduces the reference's FP64 geometry and FP32 intersection arithmetic
operation by operation, so no multiply-add may be fused behind its back.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ_DIR = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libhorayzon_gb300.so")
HEADER = os.path.join(ROOT, "include", "horayzon_gb300.h")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build "
                       "libhorayzon_gb300.so")


def _flags(extra_ptxas: bool = False):
    f = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false",
         "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", CSRC,
         "-I", os.path.join(ROOT, "include")] + ARCH
    if extra_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the CUDA library in-tree; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.h")) +
                     glob.glob(os.path.join(CSRC, "*.cuh"))) + [HEADER]
    objs, procs = [], []
    for src in sources:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, "-c", src, "-o", obj] + _flags(verbose)
            procs.append((src, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                                      stderr=subprocess.STDOUT,
                                                      text=True)))
    errors = []
    for src, cmd, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            print(out)
        if p.returncode != 0:
            errors.append("%s\n%s" % (" ".join(cmd), out))
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if force or procs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".%d.tmp" % os.getpid()
        cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart_static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout,
                                                          r.stderr))
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_checked(out_dir: str) -> str:
    """The library with device-side index checks (-DHZ_CHECKED=1) in out_dir;
    returns its path. Load it through HZ_LIBRARY in a separate process."""
    nvcc = nvcc_path()
    os.makedirs(out_dir, exist_ok=True)
    objs, procs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(out_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        cmd = [nvcc, "-c", src, "-o", obj] + _flags() + ["-DHZ_CHECKED=1"]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT, text=True)))
    errors = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append("%s\n%s" % (" ".join(cmd), out))
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    lib = os.path.join(out_dir, "libhorayzon_gb300.so")
    r = subprocess.run([nvcc, "-shared", "-o", lib] + objs + ARCH + ["-lcudart_static"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return lib


PROBE_SRC = os.path.join(PKG, "probe", "hz_l2_probe.cu")
PROBE_PATH = os.path.join(LIB_DIR, "libhz_probe.so")


def build_probe(force: bool = False) -> str:
    """The benchmark's L2 bandwidth probe (a separate small library)."""
    os.makedirs(LIB_DIR, exist_ok=True)
    if force or _stale(PROBE_PATH, [PROBE_SRC]):
        tmp = PROBE_PATH + ".%d.tmp" % os.getpid()
        cmd = [nvcc_path(), "-shared", "-o", tmp, PROBE_SRC, "-O3", "-std=c++17",
               "-Xcompiler", "-fPIC", "-lcudart_static"] + ARCH
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("probe build failed: %s\n%s%s" % (" ".join(cmd), r.stdout,
                                                                  r.stderr))
        os.replace(tmp, PROBE_PATH)
    return PROBE_PATH


if __name__ == "__main__":
    import sys
    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
