"""Benchmark: horizon evaluations/s of the HORAYZON horizon + SVF path.

One step = one full pass of the hot path over one domain: triangle-mesh
assembly, geodetic frames, LBVH build and the bracketing horizon search with
the SVF epilogue (mo_lradtopo_horayzon.cpp:562-785), on the 500 m / 600 x 600
km / nhori 24 workload (~3.1M cells; grid_type 1, dist_search 40 km,
ray_org_elev 0.2 m, refine_factor 1, svf_type 2). One horizon evaluation is
one (cell, azimuth) of the output.

* ``value``: device-resident inputs (hz_horizon_svf_device), CUDA events
  around each step on the launching stream, L2 flushed (256 MiB write)
  between steps, max over ranks.
* ``e2e``: the public host entry (hz_horizon_svf) on pinned host buffers,
  host->device inputs and device->host outputs inside the timed region.
* ``roofline``: the horizon-search kernel; algorithmic bytes per launch =
  64 B per BVH node visit + 48 B per triangle test, counted on the device
  over the same launch.
* ``cpu_baseline`` (rank 0, N=1): the CPU oracle on all host cores on a
  bounded sample (full mesh + BVH build, ray phase on a random cell subset,
  scaled to the full domain).

``--impl reference`` times the reference's own CPU algorithm on all host
cores on the same workload and prints the same JSON line. It runs the C
restatement of the reference (oracle/hz_oracle.c, bit-identical to the
shim-compiled reference on the golden cases): the reference source is not
present where this benchmark runs, and the reference entry point cannot time
a bounded cell sample.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("horizon evals/s (cells×azimuths) 500 m nhori=24, learned vs plain GPU; "
          "rays/s")
WORKLOAD = "500 m ICON-like grid, 600x600 km, fBm(H=0.7)+ridged noise 200-4800 m, nhori=24"
ARGS = (24, 1, 40000.0, 0.2, 1, 2)  # num_hori, grid_type, dist_search, ray_org_elev, refine, svf
BYTES_PER_NODE = 64
BYTES_PER_TRI = 48
BUILD_BYTES_PER_TRI = 2 * 12 + 36 + 64
EXTRAS = ("learned", "learned_small", "precision", "batch", "drop_in", "configs")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(seed: int, box_km: float):
    """The 500 m workload; box_km < 600 gives a smaller domain of the same recipe."""
    from horayzon_extpar_gb300 import synthetic
    return synthetic.make_config("c3", seed=seed, box_km=box_km)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def l2_read_peak(dev) -> float | None:
    """L2 read bandwidth (GB/s) of this GPU from the project's probe kernel:
    a 32 MiB buffer (L2 resident) streamed 300 times with L1-bypassing loads."""
    import ctypes as C

    import torch

    from horayzon_extpar_gb300 import _build
    path = _build.PROBE_PATH
    if not os.path.exists(path):
        path = _build.build_probe()
    lib = C.CDLL(path)
    lib.hz_probe_l2_read.restype = C.c_int
    lib.hz_probe_l2_read.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_void_p,
                                     C.c_void_p, C.POINTER(C.c_float)]
    nbytes, reps = 32 << 20, 300
    buf = torch.ones(nbytes // 4, dtype=torch.float32, device=dev)
    sink = torch.zeros(4, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    best = None
    for _ in range(3):
        ms = C.c_float(0.0)
        rc = lib.hz_probe_l2_read(buf.data_ptr(), nbytes, reps, sink.data_ptr(),
                                  C.c_void_p(stream.cuda_stream), C.byref(ms))
        if rc != 0 or ms.value <= 0:
            return None
        gbs = nbytes * reps / (ms.value * 1e-3) / 1e9
        best = gbs if best is None else max(best, gbs)
    return best


def traffic_from_profile():
    """DRAM bytes per launch of the search kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_trace_warp_c3_500m.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"],
                    "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample_run(dom, target_ray_s: float, keep_outputs: bool = False):
    """Times the CPU oracle on a bounded sample; returns a dict (and, with
    keep_outputs, the oracle's horizon / skyview with the sampled columns
    filled and the sampled cells, for the parity check of the GPU outputs)."""
    from oracle import api as oracle
    ncell = dom.ncell
    nth = os.cpu_count() or 1
    rng = np.random.default_rng(1234)
    kind = "port"
    # Calibrate the ray phase on 2000 cells, then size the sample.
    cal = rng.choice(ncell, min(2000, ncell), replace=False)
    _, _, st = oracle.horizon_svf(*dom.inputs(), *ARGS, cells=cal, nthreads=nth)
    per_cell = max(st["t_rays"], 1e-6) / cal.size
    n = int(min(ncell, max(2000, target_ray_s / per_cell)))
    cells = np.sort(rng.choice(ncell, n, replace=False))
    t0 = time.perf_counter()
    h_or, s_or, st = oracle.horizon_svf(*dom.inputs(), *ARGS, cells=cells, nthreads=nth)
    wall = time.perf_counter() - t0
    t_full = st["t_mesh"] + st["t_bvh"] + st["t_rays"] * ncell / n
    evals = ncell * ARGS[0]
    rays_full = st["num_rays"] * ncell / n
    out = {"value": evals / t_full, "unit": "evals/s", "cores": nth, "kind": kind,
           "sample": ("full mesh + BVH build (%.2f s) and the ray phase on %d of %d cells "
                      "(%.2f s on %d threads), scaled to the full domain"
                      % (st["t_mesh"] + st["t_bvh"], n, ncell, st["t_rays"], nth)),
           "rays_per_s": rays_full / t_full, "seconds_full_domain": t_full,
           "wall_s": wall}
    if keep_outputs:
        return out, (h_or, s_or, cells)
    return out


PARITY_BAR = "|dhorizon| <= 0.25 deg on >= 99.9 % of (cell, azimuth) and |dSVF| <= 1e-3"


def oracle_sample(dom, args, n_cells: int, seed: int = 7, precision: int = 0):
    """The CPU oracle on a fixed random sample of cells of a domain (all host
    threads): (horizon, skyview, cells) with only the sampled columns filled."""
    from oracle import api as oracle
    rng = np.random.default_rng(seed)
    cells = np.sort(rng.choice(dom.ncell, min(n_cells, dom.ncell), replace=False))
    h, s, _ = oracle.horizon_svf(*dom.inputs(), *args, cells=cells, precision=precision,
                                 nthreads=os.cpu_count() or 1)
    return h, s, cells


def parity_block(h_gpu, s_gpu, sample, oracle_kind="CPU oracle (reference arithmetic: "
                 "FP32 rays in the domain's global ENU frame, FP64 frames)"):
    """Agreement of GPU outputs with the oracle's on the sampled cells."""
    h_or, s_or, cells = sample
    dh = np.abs(np.asarray(h_gpu)[:, cells] - h_or[:, cells])
    ds = np.abs(np.asarray(s_gpu)[cells] - s_or[cells])
    within = float(np.mean(dh <= 0.25))
    max_svf = float(ds.max())
    return {"oracle": oracle_kind, "cells_compared": int(cells.size),
            "evals_compared": int(dh.size), "frac_within_0.25deg": within,
            "frac_identical": float(np.mean(dh <= 1e-9)), "max_abs_deg": float(dh.max()),
            "max_abs_svf": max_svf, "bar": PARITY_BAR,
            "meets_bar": bool(within >= 0.999 and max_svf <= 1e-3)}


def precision_report(d_in, h_ref, stream):
    """The local-frame arithmetic (HZ_PRECISION_LOCAL) on the same workload:
    its search time and its agreement with the reference-frame results. The
    error of both against the FP64 oracle is reported by
    tests/precision_report.py."""
    from horayzon_extpar_gb300 import _lib, horizon_svf_comp_device
    h_loc, _, st = horizon_svf_comp_device(*d_in, *ARGS, stream=stream,
                                           precision=_lib.HZ_PRECISION_LOCAL)
    d = np.abs(h_loc.cpu().numpy() - h_ref)
    return {"local_vs_reference_frame": {"frac_within_0.25deg": float(np.mean(d <= 0.25)),
                                         "frac_identical": float(np.mean(d <= 1e-9))},
            "local_frame_trace_ms": st["ms_trace"]}


def train_mlp(make_dom, args=ARGS, n_seeds=8, samples_per_seed=1_000_000, steps=3000,
              batch=32768):
    """Trains the warm-start MLP (untimed) on the plain method's horizons of
    n_seeds other terrain seeds, on the GPU with the library's own kernels.
    make_dom(i) builds the i-th training domain."""
    import torch

    from horayzon_extpar_gb300 import learned
    t0 = time.perf_counter()
    Xs, Ts = [], []
    for i in range(n_seeds):
        X, T = learned.training_samples(make_dom(i), args, max_samples=samples_per_seed,
                                        seed=i + 1)
        Xs.append(X)
        Ts.append(T)
    X, T = torch.cat(Xs), torch.cat(Ts)
    n = int(X.shape[0])
    params, hist = learned.train(X, T, steps=steps, batch=batch, lr=2e-3, seed=0,
                                 log_every=max(1, steps // 3))
    del X, T, Xs, Ts
    return params, {"samples": n, "steps": steps, "batch": batch,
                    "seconds": time.perf_counter() - t0, "loss_history": hist}


def auto_groups(ncell: int, nhori: int) -> int:
    """The library's choice for mlp_azimuth_groups = -1 (hz_options): the
    smallest divisor G of nhori with ncell x G >= 4 x the GPU's resident
    threads (SMs x 1024), at most nhori / 2."""
    import torch
    target = 4 * torch.cuda.get_device_properties(0).multi_processor_count * 1024
    pick = 1
    for g in range(1, nhori // 2 + 1):
        if nhori % g == 0:
            pick = g
            if ncell * g >= target:
                break
    return pick


# The reference walks down to -85 deg (mo_lradtopo_horayzon.cpp:578) where
# the first ray of a bracket misses; every horizon below -0.25 deg is clipped
# to 0 (cpp:737-741), so a floor of -0.25 deg gives each azimuth the same
# output and changes only the elevation carried into the next azimuth
# (option elev_floor_deg; reported beside the reference's walk).
FAST_FLOOR_DEG = -0.25

# The walk below the clip by doubling and bisection (elev_walk 1): the same
# stop as the step walk wherever visibility is monotone in elevation.
BISECT = dict(elev_walk=1)

LEARNED_MODES = {"first_azimuth": dict(),
                 "every_azimuth": dict(mlp_every_azimuth=True),
                 "azimuth_groups_auto": dict(mlp_azimuth_groups=-1),
                 "first_azimuth_fast_floor": dict(elev_floor_deg=FAST_FLOOR_DEG),
                 "first_azimuth_bisect_walk": dict(BISECT),
                 "every_azimuth_bisect_walk": dict(BISECT, mlp_every_azimuth=True)}


def learned_report(dom, d_in, h_ref, s_ref, stream, plain_ms, args, sample=None):
    """Learned warm start vs the plain chained search on the headline workload
    (timed like the plain steps: CUDA events around each call). The MLP is
    trained on 8 other seeds of the same recipe and domain size (a domain
    whose cells mostly see past its border would teach the model the void).
    Returns the report and the trained parameters."""
    import torch

    from horayzon_extpar_gb300 import horizon_svf_comp_device, synthetic
    params, info = train_mlp(lambda i: synthetic.make_config(
        "c3", seed=1001 + i, box_km=args.box_km))
    info["seeds"] = ("8 other seeds of the same recipe, %g x %g km boxes"
                     % (args.box_km, args.box_km))
    out = {"training": info}
    evals = dom.ncell * ARGS[0]
    modes = dict(LEARNED_MODES)
    modes["plain_fast_floor"] = dict(elev_floor_deg=FAST_FLOOR_DEG)
    modes["plain_bisect_walk"] = dict(BISECT)
    for mode, kw in modes.items():
        if not mode.startswith("plain"):
            kw = dict(kw, mlp_params=params)
        for _ in range(max(1, args.warmup)):
            horizon_svf_comp_device(*d_in, *ARGS, stream=stream, **kw)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        rays = 0
        for k in range(args.steps):
            ev[k][0].record(stream)
            h, s, st = horizon_svf_comp_device(*d_in, *ARGS, stream=stream, **kw)
            ev[k][1].record(stream)
            rays = st["num_rays"]
        torch.cuda.synchronize()
        ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        dh = np.abs(h.cpu().numpy() - h_ref)
        ds = np.abs(s.cpu().numpy() - s_ref)
        out[mode] = {"value": evals / (ms * 1e-3), "unit": "evals/s", "ms_per_step": ms,
                     "speedup_vs_plain": plain_ms / ms, "rays_per_eval": rays / evals,
                     "agreement_with_plain": {
                         "frac_within_0.25deg": float(np.mean(dh <= 0.25)),
                         "frac_identical": float(np.mean(dh <= 1e-9)),
                         "frac_cells_svf_within_1e-3": float(np.mean(ds <= 1e-3)),
                         "max_abs_svf": float(ds.max())}}
        if mode == "azimuth_groups_auto":
            out[mode]["groups"] = auto_groups(dom.ncell, ARGS[0])
        if sample is not None:
            out[mode]["parity"] = parity_block(h.cpu().numpy(), s.cpu().numpy(), sample)
    out["perfect_start_ceiling"] = perfect_start_ceiling(d_in, dom.ncell, stream, plain_ms,
                                                         args)
    return out, params


def perfect_start_ceiling(d_in, ncell, stream, plain_ms, args):
    """The learned start's measured ceiling on this workload: every azimuth
    restarted at the start a perfect model would propose, the lattice index
    of the plain search's own result ((j + 1) / 2 for the unclipped horizon
    j * 0.25 deg, which casts two rays where visibility is monotone), given
    as start indices (no model cost). Timed like the learned modes."""
    import torch

    from horayzon_extpar_gb300 import horizon_svf_comp_device
    L = ARGS[0] * ARGS[4]
    raw = torch.empty((L, ncell), dtype=torch.int16, device=d_in[0].device)
    horizon_svf_comp_device(*d_in, *ARGS, stream=stream, raw_index=raw)
    start = torch.clamp(torch.div(raw.to(torch.int32) + 1, 2, rounding_mode="floor"),
                        -170, 180).to(torch.int16).contiguous()
    out = {"what": "every azimuth started at the plain search's own result (a perfect "
                   "proposal, no model cost); the bound on any learned start here"}
    for name, kw in (("reference_walk", {}), ("bisect_walk", dict(BISECT))):
        kw = dict(kw, start_index=start, mlp_every_azimuth=True)
        for _ in range(max(1, args.warmup)):
            horizon_svf_comp_device(*d_in, *ARGS, stream=stream, **kw)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        rays = 0
        for k in range(args.steps):
            ev[k][0].record(stream)
            _, _, st = horizon_svf_comp_device(*d_in, *ARGS, stream=stream, **kw)
            ev[k][1].record(stream)
            rays = st["num_rays"]
        torch.cuda.synchronize()
        ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
        out[name] = {"ms_per_step": ms, "speedup_vs_plain": plain_ms / ms,
                     "rays_per_eval": rays / (ncell * ARGS[0])}
    return out


def learned_small_report(stream, reps=5, parity_cells=20000):
    """The learned start where the plain chain under-fills the GPU: the
    2.5 km / 400 km domain (57k cells; the chain gives one lane per cell and
    its 24 azimuths run one after another) and the 100 m / 150 km domain of
    the learned configuration, each with an MLP trained on 8 other seeds of
    its own recipe and size. Per mode: best of `reps` calls (search phase, including
    the learned start's raster, features and MLP, and the whole call on
    device-resident inputs), rays per evaluation, and parity against the
    oracle on a cell sample."""
    import torch

    from horayzon_extpar_gb300 import horizon_svf_comp_device, synthetic
    cases = [("c1", "2.5 km grid, 400x400 km, nhori 24",
              lambda i: synthetic.make_config("c1", seed=2001 + i)),
             ("c4", "100 m grid, 150x150 km, nhori 24",
              lambda i: synthetic.make_config("c4", seed=3001 + i))]
    out = {}
    for key, desc, make_train in cases:
        params, info = train_mlp(make_train)
        d = synthetic.make_config(key, seed=0)
        t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in d.inputs()]
        evals = d.ncell * ARGS[0]
        res = {"workload": desc, "ncell": d.ncell, "training": info}
        ff = dict(elev_floor_deg=FAST_FLOOR_DEG)
        modes = {"plain": None, "first_azimuth": {}, "azimuth_groups_auto":
                 {"mlp_azimuth_groups": -1}, "plain_fast_floor": ff,
                 "azimuth_groups_auto_fast_floor": dict(ff, mlp_azimuth_groups=-1),
                 "plain_bisect_walk": dict(BISECT),
                 "azimuth_groups_auto_bisect_walk": dict(BISECT, mlp_azimuth_groups=-1),
                 "every_azimuth": {"mlp_every_azimuth": True},
                 "every_azimuth_bisect_walk": dict(BISECT, mlp_every_azimuth=True)}
        sample = oracle_sample(d, ARGS, parity_cells) if parity_cells > 0 else None
        for mode, kw in modes.items():
            extra = {} if kw is None else (dict(kw) if mode.startswith("plain") else
                                           dict(mlp_params=params, **kw))
            horizon_svf_comp_device(*t, *ARGS, stream=stream, **extra)  # warm-up
            best = None
            for _ in range(reps):
                h, s, st = horizon_svf_comp_device(*t, *ARGS, stream=stream, **extra)
                if best is None or st["ms_trace"] < best["ms_trace"]:
                    best = st
            call_ms = best["ms_mesh"] + best["ms_bvh"] + best["ms_trace"]
            res[mode] = {"search_ms": best["ms_trace"], "call_ms": call_ms,
                         "evals_per_s_search": evals / (best["ms_trace"] * 1e-3),
                         "evals_per_s_call": evals / (call_ms * 1e-3),
                         "rays_per_eval": best["num_rays"] / evals}
            if mode.startswith("azimuth_groups_auto"):
                res[mode]["groups"] = auto_groups(d.ncell, ARGS[0])
            if sample is not None:
                res[mode]["parity"] = parity_block(h.cpu().numpy(), s.cpu().numpy(), sample)
        for mode, base in (("first_azimuth", "plain"), ("azimuth_groups_auto", "plain"),
                           ("every_azimuth", "plain"),
                           ("every_azimuth_bisect_walk", "plain"),
                           ("every_azimuth_bisect_walk", "plain_bisect_walk"),
                           ("plain_fast_floor", "plain"),
                           ("azimuth_groups_auto_fast_floor", "plain"),
                           ("azimuth_groups_auto_fast_floor", "plain_fast_floor"),
                           ("plain_bisect_walk", "plain"),
                           ("azimuth_groups_auto_bisect_walk", "plain"),
                           ("azimuth_groups_auto_bisect_walk", "plain_bisect_walk")):
            tag = base[len("plain"):]
            res[mode]["speedup_vs_plain%s_search" % tag] = (res[base]["search_ms"] /
                                                            res[mode]["search_ms"])
            res[mode]["speedup_vs_plain%s_call" % tag] = (res[base]["call_ms"] /
                                                          res[mode]["call_ms"])
        out[key] = res
        del t
    return out


def drop_in_report(dom, steps):
    """The Python drop-in (horizon_svf_comp_py) on ordinary numpy arrays, as a
    user of the reference calls it: pageable host buffers, wall clock."""
    from horayzon_extpar_gb300 import horizon_svf_comp_py
    inputs = [np.ascontiguousarray(a) for a in dom.inputs()]
    horizon_svf_comp_py(*inputs, *ARGS)  # warm-up
    walls, st = [], None
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        _, _, st = horizon_svf_comp_py(*inputs, *ARGS, return_stats=True)
        walls.append(time.perf_counter() - t0)
    w = float(np.median(walls))
    return {"call": "horizon_svf_comp_py(numpy arrays)", "value": dom.ncell * ARGS[0] / w,
            "unit": "evals/s", "wall_ms": 1e3 * w,
            "phase_ms": {k: st[k] for k in ("ms_h2d", "ms_mesh", "ms_bvh", "ms_trace",
                                              "ms_d2h")}}


def batch_report(args, mlp_params=None):
    """64 uneven independent domains in one call (one persistent search);
    with mlp_params also the same batch with the learned start (the
    library's choice of azimuth groups)."""
    from horayzon_extpar_gb300 import synthetic
    from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch
    batch = synthetic.make_batch(64, seed=0)
    doms = [(d.inputs(), a) for d, a in batch]
    evals = sum(d.ncell * a[0] for d, a in batch)

    def run(**kw):
        horizon_svf_comp_batch(doms, **kw)  # warm-up
        t0 = time.perf_counter()
        _, st = horizon_svf_comp_batch(doms, return_stats=True, **kw)
        wall = time.perf_counter() - t0
        lat = np.array(st["latency_ms"])
        return {"search_ms": st["ms_trace"],
                "evals_per_s_search": evals / (st["ms_trace"] * 1e-3),
                "evals_per_s_e2e_host": evals / wall,
                "rays_per_eval": st["num_rays"] / evals,
                "latency_ms_p50": float(np.percentile(lat, 50)),
                "latency_ms_p99": float(np.percentile(lat, 99)),
                "kernel_launches": st["kernel_launches"]}

    out = {"workload": "64 domains, 10k-500k cells (log-uniform), 0.5-2.5 km, relief "
                       "1000-4500 m, nhori in {16, 24, 36}",
           "cells": int(sum(d.ncell for d, _ in batch)), "evals": int(evals)}
    out.update(run())
    if mlp_params is not None:
        out["learned"] = run(mlp_params=mlp_params, mlp_azimuth_groups=-1)
        out["learned"]["mlp"] = "trained on the 500 m recipe (headline workload's MLP)"
    return out


def configs_report(dom, d_in, stream, reps=2, parity_cells=20000):
    """The other configurations of the workload family, device-resident
    inputs, plain search: the 2.5 km / 400 km, 1 km / 1000 km and 100 m /
    150 km grids at nhori 24, and the 500 m domain at nhori 48, at
    refine_factor 10 and with grid_type 0. One evaluation is one (cell,
    azimuth) of the output (refine_factor 10 traces ten azimuths per
    evaluation). Each configuration's outputs are compared with the CPU
    oracle on a fixed random sample of ``parity_cells`` cells."""
    import torch
    from horayzon_extpar_gb300 import horizon_svf_comp_device, synthetic
    runs = [("c1", "2.5 km grid, 400x400 km, nhori 24", None, ARGS),
            ("c2", "1 km grid, 1000x1000 km, nhori 24", None, ARGS),
            ("c4", "100 m grid, 150x150 km, nhori 24", None, ARGS),
            ("c3_nhori48", "500 m grid, 600x600 km, nhori 48", dom, (48,) + ARGS[1:]),
            ("c3_refine10", "500 m grid, 600x600 km, nhori 24, refine_factor 10", dom,
             ARGS[:4] + (10, ARGS[5])),
            ("c3_grid_type0", "500 m grid, 600x600 km, nhori 24, grid_type 0", dom,
             (ARGS[0], 0) + ARGS[2:])]
    out = {}
    for key, desc, d, args in runs:
        if d is None:
            d = synthetic.make_config(key, seed=0)
            t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in d.inputs()]
        else:
            t = d_in
        horizon_svf_comp_device(*t, *args, stream=stream)  # warm-up
        best = None
        for _ in range(reps):
            h, s, st = horizon_svf_comp_device(*t, *args, stream=stream)
            if best is None or st["ms_trace"] < best["ms_trace"]:
                best = st
        evals = d.ncell * args[0]
        call_ms = best["ms_mesh"] + best["ms_bvh"] + best["ms_trace"]
        out[key] = {"workload": desc, "ncell": d.ncell, "n_tri": best["n_tri"],
                    "evals": evals, "search_ms": best["ms_trace"], "call_ms": call_ms,
                    "evals_per_s_search": evals / (best["ms_trace"] * 1e-3),
                    "evals_per_s_call": evals / (call_ms * 1e-3),
                    "rays_per_eval": best["num_rays"] / evals}
        if parity_cells > 0:
            t0 = time.perf_counter()
            sample = oracle_sample(d, args, parity_cells)
            out[key]["parity"] = parity_block(h.cpu().numpy(), s.cpu().numpy(), sample)
            out[key]["parity"]["oracle_seconds"] = time.perf_counter() - t0
        del h, s
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    dom = make_workload(0, args.box_km)
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_sample_run(dom, args.cpu_seconds)
        if i >= args.warmup:
            vals.append(r)
    v = float(np.mean([r["value"] for r in vals]))
    evals = dom.ncell * ARGS[0]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "evals/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * evals / v, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 rays / f64 frames", "data": "synthetic",
        "config": {"workload": WORKLOAD if args.box_km == 600.0 else
                   WORKLOAD.replace("600x600", "%gx%g" % (args.box_km, args.box_km)),
                   "ncell": dom.ncell, "nvertex": dom.nvertex,
                   "num_hori": ARGS[0], "grid_type": ARGS[1], "dist_search_m": ARGS[2],
                   "ray_org_elev_m": ARGS[3], "refine_factor": ARGS[4], "svf_type": ARGS[5]},
        "cpu_baseline": {"value": v, "unit": "evals/s", "cores": vals[-1]["cores"],
                         "kind": vals[-1]["kind"], "sample": vals[-1]["sample"]},
        "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "rays_per_s": float(np.mean([r["rays_per_s"] for r in vals])),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import ctypes as C

    import torch

    from horayzon_extpar_gb300 import _lib, horizon_svf_comp_device

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    L = _lib.load(build_if_missing=True)

    # Each rank solves its own independent domain (weak scaling).
    dom = make_workload(rank, args.box_km)
    evals = dom.ncell * ARGS[0]
    host = [np.ascontiguousarray(a) for a in dom.inputs()]
    d_in = [torch.from_numpy(a).to(dev) for a in host]
    horizon = torch.empty((ARGS[0], dom.ncell), dtype=torch.float64, device=dev)
    skyview = torch.empty(dom.ncell, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(count=False, kernel=_lib.HZ_KERNEL_PERSISTENT, leaf_size=0):
        return horizon_svf_comp_device(*d_in, *ARGS, horizon=horizon, skyview=skyview,
                                       stream=stream, count_work=count, kernel=kernel,
                                       leaf_size=leaf_size)[2]

    # Untimed: work counters. The algorithmic bytes are defined on the binary
    # LBVH with leaves of <= 4 triangles (64 B per node visit, 48 B per
    # triangle test), so they are counted by the same search on that tree;
    # the counts of the timed kernel (4-wide tree, default leaves) are
    # reported beside them.
    st_count = step(count=True, kernel=_lib.HZ_KERNEL_PERSISTENT_BVH2, leaf_size=4)
    st_wide = step(count=True)
    l2_peak = l2_read_peak(dev)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    stats = []
    with ClockSampler(local) as clk:
        barrier()
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            stats.append(step())
            ev[k][1].record(stream)
        barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = float(np.mean(step_ms))
    trace_ms = float(np.mean([s["ms_trace"] for s in stats]))
    if world > 1:
        t = torch.tensor([ms, trace_ms], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, trace_ms = float(t[0]), float(t[1])
    rays = st_count["num_rays"]

    # End to end through the public host entry with pinned buffers.
    pin = [torch.from_numpy(a).pin_memory() for a in host]
    h_out = torch.empty((ARGS[0], dom.ncell), dtype=torch.float64).pin_memory()
    s_out = torch.empty(dom.ncell, dtype=torch.float64).pin_memory()
    D = C.POINTER(C.c_double)
    I32 = C.POINTER(C.c_int32)
    opt = _lib.default_options(device=local)
    st = _lib.Stats()

    def e2e_step():
        rc = L.hz_horizon_svf(*(C.cast(t.data_ptr(), D) for t in pin[:5]),
                              C.cast(pin[5].data_ptr(), I32), C.cast(h_out.data_ptr(), D),
                              C.cast(s_out.data_ptr(), D), dom.ncell, dom.nvertex, *ARGS,
                              C.byref(opt), C.byref(st))
        _lib.check(rc)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e2e_step()
    barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps
    if world > 1:
        t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t[0])
    h2d = sum(a.nbytes for a in host)
    d2h = h_out.numel() * 8 + s_out.numel() * 8

    # Check once that the timed outputs are sane (lattice, range).
    hz = horizon.cpu().numpy()
    sv = skyview.cpu().numpy()
    if not (np.isfinite(hz).all() and (sv > 0).all() and (sv <= 1).all()):
        raise RuntimeError("invalid outputs")

    # The CPU baseline (rank 0, N = 1): the oracle on all host cores on a
    # random cell sample. Its outputs are kept: the timed GPU outputs are
    # compared with them on the sampled cells (the parity block). Without
    # the CPU leg an untimed sample of parity_cells cells stands in.
    cpu, sample = None, None
    if rank == 0:
        if world == 1 and not args.no_cpu:
            cpu, sample = cpu_sample_run(dom, args.cpu_seconds, keep_outputs=True)
            cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        elif args.parity_cells > 0:
            sample = oracle_sample(dom, ARGS, args.parity_cells)
    parity = parity_block(hz, sv, sample) if sample is not None else None

    # Untimed extras: the learned warm start, the local-precision mode, the
    # batched uneven-domain workload, the numpy drop-in and the other
    # configurations, each compared with the oracle on a cell sample.
    extras = {}
    want = set(EXTRAS if args.extras == "all" else args.extras.split(","))
    if not args.no_extras and rank == 0:
        mlp = None
        if "learned" in want:
            extras["learned"], mlp = learned_report(dom, d_in, hz, sv, stream, ms, args, sample)
        if "learned_small" in want:
            extras["learned_small_domains"] = learned_small_report(
                stream, parity_cells=args.parity_cells)
        if "precision" in want:
            extras["precision"] = precision_report(d_in, hz, stream)
        if "batch" in want:
            extras["batched_domains"] = batch_report(args, mlp)
        if "drop_in" in want:
            extras["drop_in_numpy"] = drop_in_report(dom, min(args.steps, 3))
        if "configs" in want:
            extras["configs"] = configs_report(dom, d_in, stream,
                                               parity_cells=args.parity_cells)
    del sample

    peak, peak_kind = measured_peaks()
    alg_bytes = BYTES_PER_NODE * st_count["node_visits"] + BYTES_PER_TRI * st_count["tri_tests"]
    achieved = alg_bytes / (trace_ms * 1e-3) / 1e9
    # LBVH build phase: 2 sort passes x 12 B + 36 B triangle + 64 B node per
    # triangle, over the phase's CUDA-event time.
    bvh_ms = float(np.mean([s["ms_bvh"] for s in stats]))
    build_bytes = BUILD_BYTES_PER_TRI * st_count["n_tri"]
    build_achieved = build_bytes / (bvh_ms * 1e-3) / 1e9
    traffic = traffic_from_profile()

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0
    launches = stats[0].get("kernel_launches", None)
    line = {
        "metric": METRIC,
        "value": world * evals / (ms * 1e-3),
        "unit": "evals/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 rays / f64 frames",
        "data": "synthetic",
        "config": {"workload": WORKLOAD if args.box_km == 600.0 else
                   WORKLOAD.replace("600x600", "%gx%g" % (args.box_km, args.box_km)),
                   "variant": "plain (chained bracketing search)",
                   "ncell": dom.ncell, "nvertex": dom.nvertex, "n_tri": st_count["n_tri"],
                   "num_hori": ARGS[0], "grid_type": ARGS[1], "dist_search_m": ARGS[2],
                   "ray_org_elev_m": ARGS[3], "refine_factor": ARGS[4], "svf_type": ARGS[5],
                   "evals_per_step": evals, "l2": "256 MiB flush write between steps; "
                   "per-step working set > 2 GB", "parallelism": "replica per GPU" if world > 1
                   else "1 GPU"},
        "rays_per_s": world * rays / (ms * 1e-3),
        "rays_per_eval": rays / evals,
        "phase_ms": {"mesh": float(np.mean([s["ms_mesh"] for s in stats])),
                     "bvh": float(np.mean([s["ms_bvh"] for s in stats])),
                     "trace": trace_ms},
        "e2e": {"value": world * evals / e2e_s, "unit": "evals/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "wall_ms_per_step": 1e3 * e2e_s,
                "phase_ms_last_step": {k: float(getattr(st, k)) for k in (
                    "ms_h2d", "ms_mesh", "ms_bvh", "ms_trace", "ms_d2h")}},
        # The search reads its tree and triangles mostly from L1 / L2 (DRAM
        # traffic is ~2 % of the algorithmic bytes): `frac` is the HBM-
        # equivalent fraction of the measured copy bandwidth, `l2_frac` the
        # fraction of the L2 read bandwidth measured by the project's probe;
        # the measured limiter is L1/L2 latency and instruction issue.
        "roofline": {"kernel": "k_trace_warp", "bound": "l1/l2 latency + issue",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "frac_of": "measured HBM copy bandwidth (MEASURED_PEAKS.json hbm_gbs)",
                     "l2_peak": l2_peak,
                     "l2_frac": achieved / l2_peak if l2_peak else None,
                     "l2_peak_kind": "measured (hz_l2_probe: 32 MiB, 300 passes, ld.global.cg)",
                     "alg_bytes_per_launch": alg_bytes,
                     "node_visits_per_ray": st_count["node_visits"] / rays,
                     "tri_tests_per_ray": st_count["tri_tests"] / rays,
                     "bvh4_node_visits_per_ray": st_wide["node_visits"] / rays,
                     "bvh4_tri_tests_per_ray": st_wide["tri_tests"] / rays,
                     "build_bytes_per_triangle": BUILD_BYTES_PER_TRI,
                     "build_bytes_per_launch": build_bytes, "build_ms": bvh_ms,
                     "build_achieved": build_achieved, "build_frac": build_achieved / peak,
                     "build_bound": "latency (bottom-up refit chains) and issue (Karras "
                                    "splits)"},
        "parity": parity,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": (launches * args.steps) if launches else None,
        **extras,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_sharded(args):
    """One benchmark domain over the N ranks (strong scaling): every rank
    builds the mesh and BVH and traces its contiguous cell range
    (shard.horizon_svf_sharded); a step ends with the all-gather of the
    slices. Timed with CUDA events on each rank (max over ranks), like the
    replica mode."""
    import torch
    import torch.distributed as dist

    from horayzon_extpar_gb300 import _lib, shard

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    else:
        dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % _free_port(),
                                rank=0, world_size=1)
    dev = torch.device("cuda", local)
    _lib.load(build_if_missing=True)
    dom = make_workload(0, args.box_km)
    evals = dom.ncell * ARGS[0]
    host = [np.ascontiguousarray(a) for a in dom.inputs()]
    for _ in range(args.warmup):
        shard.horizon_svf_sharded(*host, *ARGS, device=dev)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        shard.horizon_svf_sharded(*host, *ARGS, device=dev)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    sec = (time.perf_counter() - t0) / args.steps
    t = torch.tensor([sec], dtype=torch.float64, device=dev if world > 1 else "cpu")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    sec = float(t[0])
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": evals / sec, "unit": "evals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32 rays / f64 frames", "data": "synthetic",
            "config": {"workload": WORKLOAD, "ncell": dom.ncell,
                       "parallelism": "cell-range shards of one domain over %d ranks" % world,
                       "timing": "host wall clock per step: H2D of the domain, mesh + BVH, "
                                 "the rank's cell range, all-gather"}}), flush=True)
    dist.destroy_process_group()
    return 0


def _free_port():
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--box-km", type=float, default=600.0,
                    help="domain width (600 = the benchmark workload; smaller for profiling)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip every untimed extra report")
    ap.add_argument("--extras", default="all",
                    help="comma-separated extra reports to run: " + ",".join(EXTRAS))
    ap.add_argument("--cpu-seconds", type=float, default=8.0,
                    help="target seconds of CPU ray work per CPU measurement")
    ap.add_argument("--parity-cells", type=int, default=20000,
                    help="cells of the oracle sample each configuration is compared on "
                         "(the main workload uses the CPU baseline's sample)")
    ap.add_argument("--mode", choices=["replica", "sharded"], default="replica",
                    help="replica: one independent domain per rank (weak scaling, the "
                         "default line); sharded: one domain's cells split over the ranks")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "sharded":
        return run_sharded(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
