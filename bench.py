"""Benchmark: MLUPS of the fused D2Q9 collide+stream step and its HBM roofline.

Workload (one GPU): 4096 x 2048 lattice, channel edges (equilibrium inlet at
ux = 0.08, zero-gradient outflow, periodic top/bottom), tau = 0.55, 200 seeded
solid circles with radii uniform in 4..32 cells, none within 64 cells of the
inlet.  Synthetic geometry from a fixed seed; no dataset is involved.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one fused launch over the whole grid.  `value` times K steps with the
state resident in HBM (CUDA events on the engine's stream): the K-step call is
first made untimed (so the CUDA graph it replays is captured and instantiated
outside the timing), then repeated, each call bracketed by synchronisation and
its own events, until at least --min-seconds have passed; the median call is
reported.  `e2e` runs the same K steps through the public API with host
buffers: populations and mask uploaded from pinned host memory, K steps, rho /
ux / uy read back, all inside the timed region, repeated and reported the same
way.  The grid (570 MB in f32) is larger than L2, so no flush is needed between
steps.  With --gpus N > 1 (torchrun) every rank advances its own replica of the
grid: weak scaling, no collective on the data path.

--impl reference times the reference's own step arithmetic on the host cores:
its WGSL shaders translated to C++ (oracle/_ref) when built, else the oracle
restatement, on a bounded sample of the same grid.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "MLUPS & % of HBM roofline: FP32 vs FP16-store vs learned closure at equal error"
NX, NY, TAU, UX, NCIRC, SEED = 4096, 2048, 0.55, 0.08, 200, 1
BYTES_PER_CELL = {"f32": 72.0, "f16": 36.0, "bf16": 36.0, "f64": 144.0}  # algorithmic, per update
FALLBACK_HBM_GBS = 6800.0


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel_key):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    p = os.path.join(HERE, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(kernel_key)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def repeat_timed(call, stream, min_seconds, world, dist, max_calls=5000, between=None):
    """Median device time (ms) of one `call()`: each call is bracketed by a
    barrier (N > 1) and a device synchronisation on both sides and timed with
    CUDA events on `stream`; calls repeat until `min_seconds` of wall time have
    passed (at least 3).  `between()`, if given, runs before each call,
    outside the timing.  The number of calls is agreed over ranks and each
    call's time is the maximum over ranks.  Returns (median_ms, calls, wall_s)."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def once():
        if between is not None:
            between()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        call()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    t0 = time.perf_counter()
    first = once()
    per = max(time.perf_counter() - t0, 1e-6)
    calls = int(min(max_calls, max(3, -(-min_seconds // per))))
    if world > 1:
        t = torch.tensor([calls], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        calls = int(t.item())
    t0 = time.perf_counter()
    ms = [once() for _ in range(calls)]
    wall = time.perf_counter() - t0
    del first
    if world > 1:
        t = torch.tensor(ms, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = t.tolist()
    return statistics.median(ms), calls, wall


# Plain BGK on the 4096 x 2048 workload (tau 0.55, speeds reaching 0.3 to
# 0.4 around the circles) goes non-finite between steps 28,000 and 34,000 in
# every storage, f32 included.  Timed runs restart from the initial
# equilibrium (untimed) before they would pass this many steps.
RESTART_STEPS = 12000


class restarter:
    """A `between` hook for repeat_timed: before a call of k steps that would
    take the lattice past RESTART_STEPS, re-initialise it to the workload's
    start and take its first (in-place) step, which keeps the buffer parity
    the captured step graphs were made for.  `launches` counts the kernels
    it launched (none of them inside a timed call)."""

    def __init__(self, lat, k):
        self.lat, self.k, self.launches, self.restarts = lat, k, 0, 0

    def __call__(self):
        lat = self.lat
        if lat.get_compute_num() + self.k > RESTART_STEPS:
            l0 = lat.launch_count()
            lat.init_equilibrium(1.0, UX, 0.0, 1e-4, SEED)
            lat.iterate(1)
            lat.synchronize()
            self.launches += lat.launch_count() - l0
            self.restarts += 1


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_mask():
    from lbm_gb300 import geometry
    return geometry.random_circles(NX, NY, NCIRC, 4, 32, seed=SEED, inlet_clearance=64)


def time_storage(lbm, torch, storage, mask, steps, warmup, min_seconds=1.0, store_inlet=False, sr=False):
    """Device-resident MLUPS of one storage format, timed like `value` (the
    K-step call made untimed first, then repeated for `min_seconds`, median
    call); returns (ms_per_step, launches per call).  store_inlet=True keeps
    16-bit words relative to the inlet equilibrium (lbm_set_storage_reference
    1) instead of the rest weights; sr=True rounds them stochastically."""
    lat = lbm.Lattice(NX, NY, 1.0 / TAU, lbm.EDGE_CHANNEL, storage)
    lat.set_storage_reference(store_inlet)
    if sr:
        lat.set_rounding(lbm.ROUND_STOCHASTIC, SR_SEED)
    stream = torch.cuda.Stream()
    lat.set_stream(stream.cuda_stream)
    lat.set_inlet_velocity(UX)
    lat.init_equilibrium(1.0, UX, 0.0, 1e-4, SEED)
    lat.draw_mask(mask)
    lat.iterate(warmup)
    lat.iterate(steps)
    lat.iterate(steps)
    lat.synchronize()
    l0 = lat.launch_count()
    rs = restarter(lat, steps)
    ms, calls, _ = repeat_timed(lambda: lat.iterate(steps), stream, min_seconds, 1, None, between=rs)
    lat.synchronize()
    launches = (lat.launch_count() - l0 - rs.launches) // (calls + 1)
    lat.close()
    return ms / steps, launches


def time_batched_split(lbm, torch, storage, steps, warmup, min_seconds, rank=0, world=1, dist=None, count=512,
                       seed=1):
    """The batched workload's 512 domains dealt whole to `world` ranks by cell
    count (batch.partition), each rank autotuning and stepping its share as
    one batch; strong scaling (the whole workload is fixed).  Returns the
    whole-job MLUPS over all cells and ms per step (median call of `steps`
    steps, max over ranks), each rank's share, and the FP64 conservation
    totals gathered over the ranks (batch.sharded_totals) over the domains
    whose flow stayed finite, with the count of the others."""
    import numpy as np
    from lbm_gb300 import batch as B
    nx, ny, om, u, masks = B.batched_workload(count, seed)
    parts = B.partition(nx, ny, world)
    mine = parts[rank]
    cells = int((nx.astype(np.int64) * ny).sum())
    with B.Batch(nx[mine], ny[mine], om[mine], u[mine], storage) as b:
        for i, d in enumerate(mine):
            b.set_mask(i, masks[d])
        rep = b.autotune(40)
        b.init_equilibrium(1e-3, seed)
        b.step(max(warmup, 3))
        b.step(steps)
        st = torch.cuda.ExternalStream(b.stream())
        ms, calls, _ = repeat_timed(lambda: b.step(steps), st, min_seconds, world, dist)
        try:
            b.synchronize()
        except lbm.LBMError:
            pass  # domains whose flow went non-finite; the timing does not depend on it
        c = b.conservation()
        finite = np.isfinite(c).all(axis=1)
        totals = B.sharded_totals(c[finite], dist)  # over the domains whose flow stayed finite
        bad = B.sharded_totals(np.c_[(~finite).astype(np.float64), np.zeros((len(c), 2))], dist)[0]
    share = (nx[mine].astype(np.int64) * ny[mine]).sum()
    return {"workload": "%d batched domains (widths 128-1024, heights 64-512) dealt whole to %d rank(s) by cell "
                        "count, %s" % (count, world, "f16" if storage == lbm.F16 else "f32"),
            "mlups": round(cells * steps / (ms * 1e-3) / 1e6, 1), "ms_per_step": round(ms / steps, 5),
            "calls": calls, "rank0_domains": int(len(mine)), "rank0_cell_share": round(float(share) / cells, 4),
            "tuned_rank0": rep["chosen"]["schedule"],
            "conservation_totals_finite_domains": [_finite_or_str(float(x), 6) for x in totals],
            "nonfinite_domains": int(bad)}


def time_batched(lbm, torch, storage, steps, warmup, count=512, seed=1):
    """The batched workload: `count` seeded channel domains (width 128-1024,
    height 64-512, multiples of 32; circles and rectangles at 5-15 % solid;
    tau 0.51-0.8; inlet ux 0.02-0.1), autotuned, then `steps` steps timed with
    CUDA events on the batch's stream."""
    import numpy as np
    from lbm_gb300 import batch as B
    nx, ny, om, u, masks = B.batched_workload(count, seed)
    cells = int((nx.astype(np.int64) * ny).sum())
    active = int(sum(int((m[:, 1:] == 0).sum()) for m in masks))
    with B.Batch(nx, ny, om, u, storage) as b:
        for d, m in enumerate(masks):
            b.set_mask(d, m)
        rep = b.autotune(40)
        b.init_equilibrium(1e-3, seed)
        b.step(max(warmup, 3))
        st = torch.cuda.ExternalStream(b.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        b.step(steps)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        try:
            b.synchronize()
        except lbm.LBMError:
            pass  # domains whose flow went non-finite are counted below
        bad = sum(1 for d in range(count) if not np.isfinite(b.field(d, "rho")).all())
    bpc = BYTES_PER_CELL["f32" if storage == lbm.F32 else "f16"]
    return {"mlups": round(cells / (ms * 1e-3) / 1e6, 1), "mflups": round(active / (ms * 1e-3) / 1e6, 1),
            "ms_per_step": round(ms, 4), "steps": steps, "domains": count, "cells": cells,
            "achieved_gbs": round(bpc * active / (ms * 1e-3) / 1e9, 1), "tuned": rep["chosen"],
            "nonfinite_domains": bad}


SLAB = {"nx": 16384, "ny": 8192, "tau": 0.51, "ux": 0.05, "outlet_clearance": 128, "ramp": 3000}


def time_slab(lbm, torch, steps, warmup, min_seconds, rank=0, world=1, dist=None):
    """The large-grid workload (16384 x 8192, circles r 8-64 at 8 % solid kept
    128 cells clear of the outflow, tau 0.51, inlet ux 0.05, f32; the fluid
    starts at rest and the inlet velocity rises over 3000 untimed steps, as
    in lbm_gb300.large_run) split into `world` y-slabs, one per rank, each
    step overlapped with its halo exchange: edge rows, exchange on a side
    stream (NCCL between ranks; a device copy onto itself when alone),
    interior rows, ghost rows.  Strong scaling: the whole grid is fixed.
    Returns the whole-job MLUPS and ms per step (median call of `steps`
    steps, max over ranks)."""
    from lbm_gb300.geometry import random_circles
    from lbm_gb300.slab import DistExchanger, SlabLattice
    c = SLAB
    mask = random_circles(c["nx"], c["ny"], 10 ** 7, 8, 64, 1, inlet_clearance=64, target_fraction=0.08,
                          outlet_clearance=c["outlet_clearance"])
    s = SlabLattice(c["nx"], c["ny"], 1.0 / c["tau"], rank, world, storage=lbm.F32, u_in=0.0)
    stream = torch.cuda.Stream()
    s.lat.set_stream(stream.cuda_stream)
    s.lat.init_equilibrium(1.0, 0.0, 0.0, 1e-4, SEED + rank)
    s.set_mask(mask)
    s.attach(DistExchanger(s, device=True))
    chunk = 100
    for i in range(c["ramp"] // chunk):  # untimed start-up: the inlet rises linearly to ux
        s.step(chunk)
        s.lat.set_inlet_velocity(c["ux"] * (i + 1) * chunk / c["ramp"])
    s.step(max(warmup, 3))
    ms, calls, _ = repeat_timed(lambda: s.step(steps), stream, min_seconds, world, dist)
    try:
        s.lat.synchronize()
        finite = True
    except lbm.LBMError:
        finite = False  # plain BGK at tau 0.51 diverges on this grid; the timing does not depend on it
    s.lat.close()
    n = c["nx"] * c["ny"]
    return {"workload": "%dx%d channel, circles r 8-64 at 8%% solid (outflow clearance %d), tau %.2f, ux %.2f "
                        "(after a %d-step ramp), f32, %d y-slab(s), halo exchange overlapped with the interior rows"
                        % (c["nx"], c["ny"], c["outlet_clearance"], c["tau"], c["ux"], c["ramp"], world),
            "mlups": round(n * steps / (ms * 1e-3) / 1e6, 1), "ms_per_step": round(ms / steps, 5),
            "launches_per_step": 3, "calls": calls, "scaling": "strong", "finite": finite}


def precision_check(lbm, torch, mask, steps, every=500, short=1000):
    """Storage precision on the 4096 x 2048 workload: the same seeded run in
    f64 (the GPU's FP64 run is the reference), f32, f16 and bf16 (words
    relative to the rest weights, f - w), f16_inlet / bf16_inlet (relative
    to the inlet equilibrium), and each 16-bit form again with stochastic
    rounding (the _sr runs) for `steps` steps.  For each: the relative L2 error over fluid
    cells, against f64, of the velocity at step `short` (before the unsteady
    wake amplifies rounding differences into different vortex trajectories),
    of the velocity time-averaged over the second half (samples every `every`
    steps) and of the final velocity; and the FP64 relative drift of the
    fluid mass and x momentum sums from the first step to the last (the
    channel is open at both ends, so the runs are compared with the f64 run's
    drift, not with zero)."""
    import ctypes
    import numpy as np
    L = lbm.load_library()
    dev = torch.device("cuda")
    fl = torch.from_numpy(mask == 0).to(dev)
    fl[:, 0] = False  # the inlet column is set, not computed
    tmp = torch.empty((NY, NX), dtype=torch.float32, device=dev)
    runs = {}
    for name, st, inlet, sr in STORAGE_RUNS:
        stream = torch.cuda.Stream()
        acc = torch.zeros((2, NY, NX), dtype=torch.float64, device=dev)
        fin = torch.empty((2, NY, NX), dtype=torch.float64, device=dev)
        early = torch.empty((2, NY, NX), dtype=torch.float64, device=dev)
        n_avg = 0
        with lbm.Lattice(NX, NY, 1.0 / TAU, lbm.EDGE_CHANNEL, st) as lat:
            lat.set_storage_reference(inlet)
            if sr:
                lat.set_rounding(lbm.ROUND_STOCHASTIC, SR_SEED)
            lat.set_stream(stream.cuda_stream)
            lat.set_inlet_velocity(UX)
            lat.init_equilibrium(1.0, UX, 0.0, 1e-4, SEED)
            lat.draw_mask(mask)
            lat.iterate(1)
            c0 = lat.conservation()
            done = 1
            with torch.cuda.stream(stream):
                while done < steps:
                    k = min(every - done % every, steps - done, short - done if done < short else steps)
                    lat.iterate(k)
                    done += k
                    last = done >= steps
                    if done > steps // 2 or last or done == short:
                        for i, f in enumerate((3, 4)):  # ux, uy
                            lbm._check(L.lbm_read_field_device(lat.handle, f, ctypes.c_void_p(tmp.data_ptr())))
                            if done > steps // 2 and done % every == 0:
                                acc[i] += tmp
                            if last:
                                fin[i] = tmp
                            if done == short:
                                early[i] = tmp
                        n_avg += done > steps // 2 and done % every == 0
            torch.cuda.synchronize()
            try:
                lat.synchronize()
                finite = True
            except lbm.LBMError:
                finite = False
            c1 = lat.conservation()
        runs[name] = {"avg": acc / max(n_avg, 1), "fin": fin, "early": early, "finite": finite,
                      "mass_drift": float((c1[0] - c0[0]) / c0[0]),
                      "momentum_x_drift": float((c1[1] - c0[1]) / c0[1])}
    ref = runs["f64"]

    def rel(a, b):
        d = (a - b)[:, fl]
        return float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(b[:, fl]))

    out = {"workload": "4096x2048 bench workload, %d steps; velocity averaged over the second half" % steps,
           "reference": "f64 storage on the GPU", "short_steps": short}
    for name, r in runs.items():
        e = {"finite": r["finite"], "mass_drift": r["mass_drift"], "momentum_x_drift": r["momentum_x_drift"]}
        if name != "f64":
            e["rel_err_velocity_short"] = _finite_or_str(rel(r["early"], ref["early"]), 7)
            e["rel_err_time_avg_velocity"] = _finite_or_str(rel(r["avg"], ref["avg"]), 7)
            e["rel_err_final_velocity"] = _finite_or_str(rel(r["fin"], ref["fin"]), 7)
        out[name] = e
    return out


# (name, storage, 16-bit words relative to the inlet equilibrium instead of
# the rest weights (the default), stochastic rounding of the stored words)
STORAGE_RUNS = (("f64", 3, False, False), ("f32", 0, False, False), ("f16", 1, False, False), ("bf16", 2, False, False),
                ("f16_inlet", 1, True, False), ("bf16_inlet", 2, True, False), ("f16_sr", 1, False, True),
                ("bf16_sr", 2, False, True), ("f16_inlet_sr", 1, True, True), ("bf16_inlet_sr", 2, True, True))
SR_SEED = 0x5EED

STEADY = {"nx": 1024, "ny": 512, "cx": 256, "cy": 256, "r": 24, "ux": 0.05, "tau": 0.8}


def steady_precision(lbm, steps=20000, every=1000):
    """Storage precision where rounding is not amplified by chaos: flow past
    one cylinder at Reynolds number u D / nu = 0.05 * 48 / 0.1 = 24, below the
    onset of vortex shedding (about 47), so the wake is steady and a rounding
    difference decays instead of growing.  1024 x 512 channel, circle r = 24 at
    (256, 256), tau 0.8, inlet ux 0.05, started from rest at the inlet
    velocity.  Every storage runs `steps` steps; returns, per storage, the
    relative L2 error over fluid cells against the f64 run of the final
    velocity and of the velocity averaged over the second half (samples every
    `every` steps)."""
    import numpy as np
    from lbm_gb300 import geometry
    c = STEADY
    mask = geometry.single_circle(c["nx"], c["ny"], c["cx"], c["cy"], c["r"])
    fl = mask == 0
    fl[:, 0] = False
    res = {}
    for name, st, inlet, sr in STORAGE_RUNS:
        acc, n = 0.0, 0
        with lbm.Lattice(c["nx"], c["ny"], 1.0 / c["tau"], lbm.EDGE_CHANNEL, st) as lat:
            lat.set_storage_reference(inlet)
            if sr:
                lat.set_rounding(lbm.ROUND_STOCHASTIC, SR_SEED)
            lat.set_inlet_velocity(c["ux"])
            lat.init_equilibrium(1.0, c["ux"], 0.0, 0.0, 0)
            lat.draw_mask(mask)
            done = 0
            while done < steps:
                lat.iterate(every)
                done += every
                u = np.stack([lat.field("ux"), lat.field("uy")]).astype(np.float64)
                if done > steps // 2:
                    acc = acc + u
                    n += 1
            res[name] = (u, acc / max(n, 1))

    def rel(a, b):
        return float(np.linalg.norm((a - b)[:, fl]) / np.linalg.norm(b[:, fl]))

    out = {"workload": "steady cylinder wake (Re 24): 1024x512 channel, r 24, tau 0.8, ux 0.05, %d steps" % steps,
           "reference": "f64 storage on the GPU"}
    for name in [r[0] for r in STORAGE_RUNS[1:]]:
        out[name] = {"rel_err_final_velocity": _finite_or_str(rel(res[name][0], res["f64"][0]), 7),
                     "rel_err_time_avg_velocity": _finite_or_str(rel(res[name][1], res["f64"][1]), 7)}
    return out


def _finite_or_str(x, ndigits=4):
    """A float for the JSON line; "non-finite" where the run diverged (strict
    JSON has no Infinity or NaN)."""
    import math
    return round(x, ndigits) if math.isfinite(x) else "non-finite"


def time_closure(lbm, refresh=20, seed=1):
    """The learned-closure workload: one held-out layout of the closure
    training setup (fine 2048x1024, tau 0.52, u 0.06, circles r 6-20 up to
    8 % solid; coarse 4x: 512x256, tau 0.505), the fine f32 run for 8000 steps
    against the coarse f32 run with the trained closure (tensor-core
    inference every `refresh` steps) for the same physical time (2000
    coarse steps).  Both are device-timed with CUDA events, every step and
    inference included; the error is the relative L2 difference of the
    time-averaged velocity (second half) against the block-averaged fine run,
    for the closure and for plain coarse BGK."""
    import numpy as np
    from lbm_gb300 import closure as cl
    path = os.path.join(HERE, "lbm_gb300", "closure_weights", "closure_2048x1024_f4.npz")
    params = np.load(path)["params"]
    nx, ny, F, tau, u, steps = 2048, 1024, 4, 0.52, 0.06, 8000
    tau_c = cl.coarse_tau(tau, F)
    # held-out layout 65 of the training script's seeded set (layouts 0-63 are
    # trained on; 65's fine run stays finite), with that script's run seed
    from lbm_gb300.geometry import random_circles
    mask = random_circles(nx, ny, 10 ** 6, 6.0, 20.0, seed * 1000 + 65, inlet_clearance=64, target_fraction=0.08)
    sc = cl.coarse_solid(mask, F)
    lseed = seed * 7919 + 65
    t_fine = cl.time_run(nx, ny, tau, u, mask, steps, lseed)
    t_cl = cl.time_run(nx // F, ny // F, tau_c, u, sc, steps // F, lseed, params=params, refresh=refresh, drift=1.0)
    uf, _, _ = cl.run_average(nx, ny, tau, u, mask, steps, 20, steps // 2, lseed)
    ufc = cl.block_average(uf, mask, F)
    uc, _, fb = cl.run_average(nx // F, ny // F, tau_c, u, sc, steps // F, 5, steps // F // 2, lseed, params=params,
                               refresh=refresh, drift=1.0)
    up, _, _ = cl.run_average(nx // F, ny // F, tau_c, u, sc, steps // F, 5, steps // F // 2, lseed)
    fine_cells = nx * ny
    return {"workload": "closure: fine 2048x1024 tau 0.52 u 0.06 vs coarse 512x256 + CNN closure (refresh %d)"
                        % refresh,
            "fine_ms": round(t_fine * 1e3, 3), "closure_ms": round(t_cl * 1e3, 3),
            "speedup": round(t_fine / t_cl, 2),
            "fine_mlups": round(fine_cells * steps / t_fine / 1e6, 1),
            "fine_equivalent_mlups": round(fine_cells * steps / t_cl / 1e6, 1),
            "err_closure_vs_fine": _finite_or_str(cl.rel_error(uc, ufc, sc)),
            "err_plain_coarse_vs_fine": _finite_or_str(cl.rel_error(up, ufc, sc)),
            "fallback_fraction": round(fb / max(int((sc == 0)[:, 1:].sum()) * (steps // F), 1), 6)}


def run_ours(args):
    import numpy as np
    import torch
    import lbm_gb300 as lbm
    from lbm_gb300 import build as B

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    if rank == 0 or not os.path.exists(B.LIB):
        B.build()
    if world > 1:
        dist.barrier()
    lbm.load_library()
    if world > 1 and not (args.slab or args.batched_split):
        # the scaling line is the replicated step and its e2e; the single-GPU
        # workloads beside it (slab, storage variants, precision, closure,
        # batched, CPU baseline) run at N = 1 only
        args.no_slab = args.no_variants = args.no_precision = args.no_closure = args.no_batched = True
        args.no_cpu_baseline = True
    mask = workload_mask()
    n = NX * NY
    # cells that move data: in channel mode the inlet column and solid cells are
    # inert (never read or written by the step), so they carry no algorithmic bytes
    active = int((mask[:, 1:] == 0).sum())
    hbm_peak, peak_kind = peaks()
    if args.slab:
        r = time_slab(lbm, torch, args.steps, args.warmup, args.min_seconds, rank, world, dist)
        if rank == 0:
            print(json.dumps({
                "metric": METRIC, "value": r["mlups"], "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded circles)",
                "config": {"workload": r["workload"], "parallelism": "y-slabs x%d" % world},
                "gpu_launches": 3 * args.steps, "slab": r}), flush=True)
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.batched_split:
        st = lbm.F16 if args.batched_split == "f16" else lbm.F32
        r = time_batched_split(lbm, torch, st, args.steps, args.warmup, args.min_seconds, rank, world, dist)
        if rank == 0:
            print(json.dumps({
                "metric": METRIC, "value": r["mlups"], "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": args.batched_split,
                "data": "synthetic (seeded domains)",
                "config": {"workload": r["workload"], "parallelism": "whole domains x%d ranks" % world},
                "gpu_launches": args.steps, "batched_split": r}), flush=True)
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.kernel_only:
        st = {"f32": lbm.F32, "f16": lbm.F16, "bf16": lbm.BF16, "f64": lbm.F64}[args.kernel_only]
        ms, launches = time_storage(lbm, torch, st, mask, args.steps, args.warmup, args.min_seconds,
                                    args.inlet_reference, args.stochastic)
        gbs = BYTES_PER_CELL[args.kernel_only] * active / (ms * 1e-3) / 1e9
        print(json.dumps({"kernel_only": args.kernel_only, "ms_per_step": round(ms, 5),
                          "mlups": round(n / (ms * 1e-3) / 1e6, 1), "achieved_gbs": round(gbs, 1),
                          "frac": round(gbs / hbm_peak, 4), "launches": launches}))
        return

    # --- value: K steps with the state resident, f32 ---------------------------
    lat = lbm.Lattice(NX, NY, 1.0 / TAU, lbm.EDGE_CHANNEL, lbm.F32)
    stream = torch.cuda.Stream()  # the engine's kernels and the timing events share this stream
    lat.set_stream(stream.cuda_stream)
    lat.set_inlet_velocity(UX)
    lat.init_equilibrium(1.0, UX, 0.0, 1e-4, SEED)
    lat.draw_mask(mask)
    lat.iterate(args.warmup)
    # the timed call itself, untimed, at both buffer parities: lbm_step captures
    # and instantiates the CUDA graph it replays for a call of this length here
    lat.iterate(args.steps)
    lat.iterate(args.steps)
    lat.synchronize()
    l0 = lat.launch_count()
    rs = restarter(lat, args.steps)
    with ClockSampler(local) as clocks:
        dev_ms, calls, wall = repeat_timed(lambda: lat.iterate(args.steps), stream, args.min_seconds, world, dist,
                                           between=rs)
    lat.synchronize()
    launches = (lat.launch_count() - l0 - rs.launches) // (calls + 1)
    ms_step = dev_ms / args.steps
    mlups = world * n * args.steps / (dev_ms * 1e-3) / 1e6
    # one launch per step, replayed from a graph: the per-step device time is
    # the launch's duration plus the graph's gap between launches
    kernel_ms = ms_step
    achieved = BYTES_PER_CELL["f32"] * active / (kernel_ms * 1e-3) / 1e9
    lat.close()

    # --- e2e: the public API with pinned host buffers, copies inside the timing --
    pops_h = torch.empty(9 * n, dtype=torch.float32, pin_memory=True)
    mask_h = torch.from_numpy(mask.reshape(-1).copy()).pin_memory()
    outs = [torch.empty(n, dtype=torch.float32, pin_memory=True) for _ in range(3)]
    src = lbm.Lattice(NX, NY, 1.0 / TAU, lbm.EDGE_CHANNEL, lbm.F32)
    src.set_inlet_velocity(UX)
    src.init_equilibrium(1.0, UX, 0.0, 1e-4, SEED)
    pops_h.numpy()[:] = src.populations().reshape(-1)
    src.close()
    lat = lbm.Lattice(NX, NY, 1.0 / TAU, lbm.EDGE_CHANNEL, lbm.F32)
    lat.set_inlet_velocity(UX)
    L = lbm.load_library()
    import ctypes
    lstream = torch.cuda.ExternalStream(lat.get_stream())
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(5)]

    def e2e_once(k):
        marks[0].record(lstream)
        lbm._check(L.lbm_write_populations(lat.handle, ctypes.c_void_p(pops_h.data_ptr())))
        marks[1].record(lstream)
        lbm._check(L.lbm_set_mask(lat.handle, ctypes.c_void_p(mask_h.data_ptr())))
        marks[2].record(lstream)
        lbm._check(L.lbm_step(lat.handle, k))
        marks[3].record(lstream)
        for o, f in zip(outs, (0, 3, 4)):  # rho, ux, uy
            lbm._check(L.lbm_read_field(lat.handle, f, ctypes.c_void_p(o.data_ptr())))
        marks[4].record(lstream)

    # the timed call, untimed first (captures the graph its K steps replay)
    e2e_once(max(args.warmup, 1))
    e2e_once(args.steps)
    e2e_once(args.steps)
    lat.synchronize()
    phases = []

    def e2e_timed():
        e2e_once(args.steps)
        torch.cuda.synchronize()
        phases.append([marks[i].elapsed_time(marks[i + 1]) for i in range(4)])

    e2e_ms, e2e_calls, _ = repeat_timed(e2e_timed, lstream, args.min_seconds, world, dist, max_calls=400)
    lat.close()
    e2e_mlups = world * n * args.steps / (e2e_ms * 1e-3) / 1e6

    # --- the reference's frame loop end to end: the state stays resident; each
    # call uploads the barrier mask (an edit: the engine materialises the
    # state first), steps K times and reads rho / ux / uy back to pinned host
    # memory
    lat = lbm.Lattice(NX, NY, 1.0 / TAU, lbm.EDGE_CHANNEL, lbm.F32)
    lat.set_stream(stream.cuda_stream)
    lat.set_inlet_velocity(UX)
    lat.init_equilibrium(1.0, UX, 0.0, 1e-4, SEED)
    lat.draw_mask(mask)

    def frame_once(k):
        lbm._check(L.lbm_set_mask(lat.handle, ctypes.c_void_p(mask_h.data_ptr())))
        lbm._check(L.lbm_step(lat.handle, k))
        for o, f in zip(outs, (0, 3, 4)):  # rho, ux, uy
            lbm._check(L.lbm_read_field(lat.handle, f, ctypes.c_void_p(o.data_ptr())))

    frame_once(max(args.warmup, 1))
    frame_once(args.steps)
    frame_once(args.steps)
    lat.synchronize()
    rs_frame = restarter(lat, args.steps)
    frame_ms, frame_calls, _ = repeat_timed(lambda: frame_once(args.steps), stream, args.min_seconds, world, dist,
                                            max_calls=400, between=rs_frame)
    lat.close()
    frame_mlups = world * n * args.steps / (frame_ms * 1e-3) / 1e6
    pops_bytes, mask_bytes, out_bytes = 9 * n * 4, n, 3 * n * 4
    h2d = (pops_bytes + mask_bytes) / args.steps
    d2h = out_bytes / args.steps
    ph = [statistics.median(p[i] for p in phases) for i in range(4)]
    link = host_link(torch, pops_bytes)
    e2e_phases = {"write_populations_ms": round(ph[0], 4), "set_mask_ms": round(ph[1], 4),
                  "steps_ms": round(ph[2], 4), "read_fields_ms": round(ph[3], 4),
                  "h2d_gbs": round((pops_bytes + mask_bytes) / ((ph[0] + ph[1]) * 1e-3) / 1e9, 1),
                  "d2h_gbs": round(out_bytes / (ph[3] * 1e-3) / 1e9, 1),
                  "host_link_h2d_gbs": link[0], "host_link_d2h_gbs": link[1], "calls": e2e_calls}

    # --- the large grid split into y-slabs (one here), exchange overlapped ------------
    slab = None
    if not args.no_slab:
        slab = time_slab(lbm, torch, args.steps, args.warmup, min(args.min_seconds, 0.5))

    # --- storage variants (same workload) -----------------------------------------
    variants = {}
    if not args.no_variants:
        for name, st, inlet, sr in STORAGE_RUNS[2:]:
            vms, _ = time_storage(lbm, torch, st, mask, args.steps, args.warmup, args.min_seconds, inlet, sr)
            gbs = BYTES_PER_CELL[name.split("_")[0]] * active / (vms * 1e-3) / 1e9
            variants[name] = {"mlups": round(n / (vms * 1e-3) / 1e6, 1), "ms_per_step": round(vms, 4),
                              "achieved_gbs": round(gbs, 1), "frac": round(gbs / hbm_peak, 4)}

    # --- storage precision against an FP64 run of the same workload ----------------
    precision = None
    if not args.no_precision:
        precision = precision_check(lbm, torch, mask, args.precision_steps)
        precision["steady"] = steady_precision(lbm)

    # --- learned closure: coarse run with the trained network vs the fine run -------
    closure_res = None
    if not args.no_closure:
        closure_res = time_closure(lbm)

    # --- batched: 512 independent domains, one persistent launch per step ----------
    batched = {}
    if not args.no_batched:
        for name, st in (("f32", lbm.F32), ("f16", lbm.F16)):
            batched[name] = time_batched(lbm, torch, st, args.batched_steps, args.warmup)

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    cpu = None if args.no_cpu_baseline else cpu_baseline(mask, budget_s=args.cpu_seconds)
    line = {
        "metric": METRIC, "value": round(mlups, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded circles, equilibrium init +-1e-4 noise)",
        "config": {"workload": "D2Q9 BGK channel 4096x2048, 200 circles r 4-32, tau 0.55, ux 0.08",
                   "nx": NX, "ny": NY, "cells": n, "solid_fraction": round(float(mask.mean()), 4),
                   "storage": "f32", "l2": "state 570 MB > 129 MB L2: no flush",
                   "parallelism": "replicas x%d" % world},
        "e2e_frame": {"value": round(frame_mlups, 1), "unit": "MLUPS", "h2d_bytes_per_step": int(mask_bytes / args.steps),
                      "d2h_bytes_per_step": int(d2h), "ms_per_call": round(frame_ms, 4), "calls": frame_calls,
                      "what": "the reference's frame loop: the state resident, per call the barrier mask uploaded "
                              "(the engine materialises the state for the edit), K steps, rho/ux/uy read to pinned "
                              "host; median of repeated calls"},
        "e2e": {"value": round(e2e_mlups, 1), "unit": "MLUPS", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_call": round(e2e_ms, 4), "phases": e2e_phases,
                "what": "write_populations + set_mask from pinned host, K steps, read rho/ux/uy to pinned host; "
                        "median of repeated calls"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                     "frac": round(achieved / hbm_peak, 4), "traffic": ncu_traffic("k_step_ws_f32_channel"),
                     "peak_source": peak_kind, "bytes_per_cell": BYTES_PER_CELL["f32"],
                     "algorithmic_bytes_per_launch": int(BYTES_PER_CELL["f32"] * active),
                     "active_cells": active,
                     "kernel": "lbm::k_step_ws<StF32, EDGE_CHANNEL, NS=4, CPT=1, closure off>"},
        "mflups": round(world * active * args.steps / (dev_ms * 1e-3) / 1e6, 1),
        "variants": variants,
        "batched": batched,
        "closure": closure_res,
        "precision": precision,
        "slab": slab,
        "gpu_launches": int(launches),
        "timing": {"calls": calls, "per_call": "median", "min_seconds": args.min_seconds,
                   "restarts": rs.restarts, "restart_steps": RESTART_STEPS,
                   "graph": "the K-step call replays a captured graph, instantiated before timing"},
        "clocks": clocks.summary(),
        "wall_s_timed": round(wall, 4),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def host_link(torch, nbytes):
    """Pinned host <-> device copy bandwidth (GB/s) of one `nbytes` buffer,
    the median of 5 copies each way timed with CUDA events: the link the e2e
    copies run over."""
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = []
    for src, dst in ((h, d), (d, h)):
        ms = []
        for _ in range(6):
            torch.cuda.synchronize()
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        out.append(round(nbytes / (statistics.median(ms[1:]) * 1e-3) / 1e9, 1))
    return out


def cpu_baseline(mask, budget_s=12.0, threads=None):
    """The reference's step arithmetic on the host cores, on a bounded number
    of steps of the same grid and barrier layout (its own edge semantics)."""
    import numpy as np
    from oracle import pyoracle as P
    have_ref = P.build(ref=True) or P.ref_available()
    threads = threads or os.cpu_count() or 1
    n = NX * NY
    o = P.Oracle(NX, NY, 1.0 / TAU, P.EDGE_REF, P.P_F32, threads=threads)
    o.init_equilibrium(1.0, UX, 0.0, 1e-4, SEED)
    m = mask.copy()
    m[0] = 1
    m[-1] = 1
    if have_ref:
        pops, _, _, _ = o.state()
        sim = P.RefShaders(NX, NY, np.float32(1.0 / TAU), threads=threads)
        sim.put_state(pops.astype(np.float32))
        sim.set_barrier(m)
        step, kind = sim.iterate, "reference"
    else:
        o.set_mask(m)
        step, kind = o.step, "port"
    step(1)  # warm-up
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s and done < 2000:
        step(1)
        done += 1
    dt = time.perf_counter() - t0
    return {"value": round(n * done / dt / 1e6, 2), "unit": "MLUPS", "cores": threads, "kind": kind,
            "sample": "%d steps of the %dx%d grid (%s, 8 passes per step, f32, OpenMP %d threads)" % (
                done, NX, NY, "reference WGSL translated to C++" if kind == "reference" else "oracle port",
                threads)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    mask = workload_mask()
    from oracle import pyoracle as P
    import numpy as np
    have_ref = P.build(ref=True) or P.ref_available()
    threads = os.cpu_count() or 1
    n = NX * NY
    o = P.Oracle(NX, NY, 1.0 / TAU, P.EDGE_REF, P.P_F32, threads=threads)
    o.init_equilibrium(1.0, UX, 0.0, 1e-4, SEED)
    m = mask.copy()
    m[0] = 1
    m[-1] = 1
    if have_ref:
        pops, _, _, _ = o.state()
        sim = P.RefShaders(NX, NY, np.float32(1.0 / TAU), threads=threads)
        sim.put_state(pops.astype(np.float32))
        sim.set_barrier(m)
        step, kind = sim.iterate, "reference"
    else:
        o.set_mask(m)
        step, kind = o.step, "port"
    tw = time.perf_counter()
    for _ in range(args.warmup):
        step(1)
    per = (time.perf_counter() - tw) / max(args.warmup, 1)
    # each step is one full-grid update; the count is bounded so the run ends in ~2 minutes
    steps = max(3, min(args.steps, int(120.0 / max(per, 1e-6))))
    args.steps = steps
    t0 = time.perf_counter()
    for _ in range(steps):
        step(1)
    dt = time.perf_counter() - t0
    mlups = n * steps / dt / 1e6
    sample = "%d steps of the %dx%d grid, %s, f32, OpenMP %d threads" % (
        args.steps, NX, NY, "reference WGSL shaders translated to C++ (8 passes per step)" if kind == "reference"
        else "oracle port", threads)
    line = {"impl": "reference", "metric": METRIC, "value": round(mlups, 2), "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded circles)",
            "config": {"workload": "D2Q9 BGK channel 4096x2048, 200 circles r 4-32, tau 0.55, ux 0.08",
                       "nx": NX, "ny": NY, "cells": n, "edges": "reference (walls, linear wrap)"},
            "cpu_baseline": {"value": round(mlups, 2), "unit": "MLUPS", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(mlups, 2), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_case(case):
    """Small fixed workloads for ncu captures of the batched and closure kernels."""
    import ctypes
    import numpy as np
    import lbm_gb300 as lbm
    from lbm_gb300 import build as B
    B.build()
    lbm.load_library()
    if case in ("batched64", "batched64_f16"):
        from lbm_gb300 import batch
        nx, ny, om, u, masks = batch.batched_workload(64, 1)
        f16 = case == "batched64_f16"
        with batch.Batch(nx, ny, om, u, lbm.F16 if f16 else lbm.F32) as b:
            for d, m in enumerate(masks):
                b.set_mask(d, m)
            # the autotuner's choices on the full workload: f32 5 stages, 1 cell
            # per thread (variant 0); f16 5 stages, 2 cells per thread (variant 2)
            b.set_schedule(2 if f16 else 0, 1, [32, 32, 32])
            b.init_equilibrium(1e-3, 1)
            b.step(12)
            try:
                b.synchronize()
            except lbm.LBMError:
                pass
        print(json.dumps({"case": case, "cells": int((nx.astype(np.int64) * ny).sum())}))
    else:
        from lbm_gb300 import closure, geometry
        L = lbm.load_library()
        w = closure.init_params(3)
        nx, ny = 2048, 1024
        mask = geometry.random_circles(nx, ny, 10 ** 6, 8, 16, 1, target_fraction=0.08)
        with lbm.Lattice(nx, ny, 1 / 0.51, lbm.EDGE_CHANNEL, lbm.F32) as lat:
            lat.set_inlet_velocity(0.05)
            lat.init_equilibrium(1, 0.05, 0, 1e-3, 1)
            lat.draw_mask(mask)
            lat.iterate(20)
            lbm._check(L.lbm_closure_set_weights(lat.handle, w.ctypes.data_as(ctypes.c_void_p), w.size))
            lbm._check(L.lbm_closure_enable(lat.handle, 1.0))
            for _ in range(4):
                lbm._check(L.lbm_closure_infer(lat.handle))
            lat.synchronize()
        print(json.dumps({"case": case, "cells": nx * ny}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-closure", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-slab", action="store_true")
    ap.add_argument("--slab", action="store_true",
                    help="time only the y-slab decomposition of the 16384x8192 grid across the ranks (strong scaling)")
    ap.add_argument("--batched-split", choices=["f32", "f16"], default=None,
                    help="time only the batched workload's domains dealt whole across the ranks (strong scaling)")
    ap.add_argument("--precision-steps", type=int, default=20000)
    ap.add_argument("--batched-steps", type=int, default=5000)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--min-seconds", type=float, default=1.0,
                    help="repeat the timed K-step call until this much wall time has passed (median reported)")
    ap.add_argument("--inlet-reference", action="store_true",
                    help="with --kernel-only f16 / bf16: words relative to the inlet equilibrium")
    ap.add_argument("--stochastic", action="store_true",
                    help="with --kernel-only f16 / bf16: stochastic rounding of the stored words")
    ap.add_argument("--kernel-only", choices=["f32", "f16", "bf16", "f64"], default=None,
                    help="time only the step kernel of one storage format (profiling runs)")
    ap.add_argument("--case", choices=["batched64", "batched64_f16", "closure2048"], default=None,
                    help="small fixed cases for kernel profiles: 64 batched domains (f32, 12 steps) or the "
                         "closure inference on a 2048x1024 lattice (4 launches)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.case:
        run_case(args.case)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
