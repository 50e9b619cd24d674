"""The large-grid workload: 16384 x 8192 channel, seeded circles (~8 % solid,
radii 8-64), inlet ux 0.05, tau 0.51, run three ways on one GPU:

* f32 plain BGK (the reference's arithmetic),
* f16 storage (words relative to the inlet equilibrium), plain BGK,
* f16 storage with the learned closure (weights from a train_closure .npz),
  refreshed every `--refresh` steps by the tensor-core inference kernel.

By default the circles keep 128 cells clear of the outflow column and the
fluid starts at rest, with the inlet velocity raised linearly over the first
3000 steps.  At tau 0.51 plain BGK does not survive either alternative: a
whole field started at the inlet velocity accelerates the flow through the
narrowest gaps past |u| = 0.3 within 200 steps and the density next to the
walls there goes negative; a circle touching the zero-gradient outflow
column destabilises the cells beside it within the first thousand steps.

    python -m lbm_gb300.large_run --closure closure.npz [--steps 50000] [--every 100]

For each run it reports MLUPS, achieved HBM GB/s on the step kernel
(algorithmic bytes: 72 B per active cell in f32, 36 B in f16, +4 B of
closure records), the relative FP64 drift of the fluid mass and momentum
sums from the first step (with --ramp: the first sample after the ramp) to
the last, and the time-averaged velocity over
the second half, and the first sample by which a step kernel had seen a
non-finite density.  The f16 runs' time-averaged velocities are compared
with the f32 run's (relative L2 over fluid cells).  Velocity averages stay on the
device (lbm_read_field_device); the timed region holds only steps and
inferences.  Prints one JSON line.

With --diagnose, a run that goes non-finite is repeated (the engine is
deterministic) up to the sample before, then stepped one step at a time to
the first step whose density is non-finite; the report gives that step, where
the non-finite cells are (position, distance to the inlet, the outflow and the
nearest solid cell) and the state one step earlier: the largest speed and the
lowest density over the lattice, with their positions.
"""
import argparse
import ctypes
import json
import time

import numpy as np

from . import EDGE_CHANNEL, F16, F32, ROUND_STOCHASTIC, LBMError, Lattice, _check, load_library
from .geometry import random_circles


def run(nx, ny, tau, u, mask, steps, every, storage, params=None, refresh=20, drift=1.0, seed=1, ramp=0,
        stochastic=False):
    """One run (see the module docstring).  ramp > 0 starts the fluid at rest
    and raises the inlet velocity linearly to u over the first `ramp` steps
    (lbm_set_inlet_velocity between samples, outside the timing) instead of
    starting the whole field at u.  stochastic=True rounds the stored words
    of 16-bit storage stochastically (Lattice.set_rounding, seeded by `seed`)."""
    import torch
    lib = load_library()
    stream = torch.cuda.Stream()
    dev = torch.device("cuda")
    acc = torch.zeros((2, ny, nx), dtype=torch.float32, device=dev)
    tmp = torch.empty((ny, nx), dtype=torch.float32, device=dev)
    active = int((mask[:, 1:] == 0).sum())
    sr = stochastic and storage != F32
    out = {"storage": "f32" if storage == F32 else "f16", "closure": params is not None, "ramp": ramp,
           "rounding": "stochastic" if sr else "nearest"}
    with Lattice(nx, ny, 1.0 / tau, EDGE_CHANNEL, storage) as lat:
        lat.set_stream(stream.cuda_stream)
        if sr:
            lat.set_rounding(ROUND_STOCHASTIC, seed)
        u0 = 0.0 if ramp else u
        lat.set_inlet_velocity(u0)
        lat.init_equilibrium(1.0, u0, 0.0, 1e-4, seed)
        lat.draw_mask(mask)
        if params is not None:
            p = np.ascontiguousarray(params, np.float32)
            _check(lib.lbm_closure_set_weights(lat.handle, p.ctypes.data_as(ctypes.c_void_p), p.size))
            _check(lib.lbm_closure_enable(lat.handle, float(drift)))
        lat.iterate(1)
        c0 = None if ramp else lat.conservation()
        done, n_avg, dev_ms, first_bad = 1, 0, 0.0, None
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        while done < steps:
            k = min(every, steps - done)
            torch.cuda.synchronize()
            e0.record(stream)
            left = k
            while left > 0:
                c = min(left, refresh) if params is not None else left
                if params is not None:
                    _check(lib.lbm_closure_infer(lat.handle))
                lat.iterate(c)
                left -= c
            e1.record(stream)
            torch.cuda.synchronize()
            dev_ms += e0.elapsed_time(e1)
            done += k
            if ramp and done - k < ramp:
                lat.set_inlet_velocity(u * min(1.0, done / ramp))
            if c0 is None and done >= ramp:
                c0 = lat.conservation()
            if first_bad is None:  # the step kernels' non-finite flag, outside the timing
                try:
                    lat.synchronize()
                except LBMError:
                    first_bad = done
            if done > steps // 2:
                with torch.cuda.stream(stream):  # ordered after the reads queued on the lattice's stream
                    for i, f in enumerate((3, 4)):  # ux, uy of the last step's moments
                        _check(lib.lbm_read_field_device(lat.handle, f, ctypes.c_void_p(tmp.data_ptr())))
                        acc[i] += tmp
                n_avg += 1
        torch.cuda.synchronize()
        try:
            lat.synchronize()
            out["finite"] = True
        except LBMError:
            out["finite"] = False
        c1 = lat.conservation()
        out["first_nonfinite_by_step"] = first_bad
        if params is not None:
            fb = ctypes.c_uint64(0)
            _check(lib.lbm_closure_fallback_count(lat.handle, ctypes.byref(fb), 1))
            out["fallback_fraction"] = fb.value / max(active * (steps - 1), 1)
    timed = steps - 1
    bpc = (72 if storage == F32 else 36) + (4 if params is not None else 0)
    out.update({"steps": steps, "ms_per_step": dev_ms / timed, "mlups": nx * ny * timed / (dev_ms * 1e-3) / 1e6,
                "achieved_gbs": bpc * active * timed / (dev_ms * 1e-3) / 1e9,
                "mass_drift": float((c1[0] - c0[0]) / c0[0]) if c0 is not None else None,
                "momentum_x_drift": float((c1[1] - c0[1]) / c0[1]) if c0 is not None and c0[1] else None})
    return out, (acc / max(n_avg, 1)).cpu().numpy()


def _field(lat, lib, code, tmp):
    _check(lib.lbm_read_field_device(lat.handle, code, ctypes.c_void_p(tmp.data_ptr())))
    return tmp


def diagnose(nx, ny, tau, u, mask, storage, first_bad, every, params=None, refresh=20, drift=1.0, seed=1, ramp=0,
             stochastic=False):
    """Where and how a run first goes non-finite (see the module docstring).
    `first_bad` is the sample at which the step kernels' flag was first seen
    set; the run is repeated to `first_bad - every` and then stepped singly.
    The repeat follows run()'s schedule exactly (one step, then the closure
    inferred before steps 1, 1 + refresh, ..., and with a ramp the inlet
    raised after steps 1 + every, 1 + 2 every, ...), so it retraces the same
    states bit for bit (with the same rounding: stochastic rounding is a
    function of seed, step and cell)."""
    import torch
    from scipy import ndimage
    lib = load_library()
    stream = torch.cuda.Stream()
    tmp = torch.empty((ny, nx), dtype=torch.float32, device="cuda")
    rep = {}
    with Lattice(nx, ny, 1.0 / tau, EDGE_CHANNEL, storage) as lat:
        lat.set_stream(stream.cuda_stream)
        if stochastic and storage != F32:
            lat.set_rounding(ROUND_STOCHASTIC, seed)
        u0 = 0.0 if ramp else u
        lat.set_inlet_velocity(u0)
        lat.init_equilibrium(1.0, u0, 0.0, 1e-4, seed)
        lat.draw_mask(mask)
        if params is not None:
            p = np.ascontiguousarray(params, np.float32)
            _check(lib.lbm_closure_set_weights(lat.handle, p.ctypes.data_as(ctypes.c_void_p), p.size))
            _check(lib.lbm_closure_enable(lat.handle, float(drift)))
        lat.iterate(1)  # run() takes its first step before any inference
        done = 1
        start = max(first_bad - every, 1)
        fl = torch.from_numpy(mask == 0).cuda()

        def advance(k):
            nonlocal done
            while k > 0:
                c = min(k, refresh - (done - 1) % refresh) if params is not None else k
                if ramp:  # stop at each sample, where run() raises the inlet
                    c = min(c, every - (done - 1) % every)
                if params is not None and (done - 1) % refresh == 0:
                    _check(lib.lbm_closure_infer(lat.handle))
                lat.iterate(c)
                done += c
                k -= c
                if ramp and (done - 1) % every == 0 and done - every < ramp:
                    lat.set_inlet_velocity(u * min(1.0, done / ramp))

        # growth before the failure: the lowest density and the largest speed
        # over the fluid, every `every` / 5 steps from the start
        history = []
        hstep = max(every // 5, 1)
        while done + hstep <= start:
            advance(hstep)
            with torch.cuda.stream(stream):
                rho = _field(lat, lib, 0, tmp).clone()
                spd = _field(lat, lib, 7, tmp).clone()
                rr = torch.where(fl, rho, torch.full_like(rho, float("inf")))
                sp = torch.where(fl & torch.isfinite(spd), spd, torch.zeros_like(spd))
            torch.cuda.synchronize()
            i_sp, i_rho = int(torch.argmax(sp)), int(torch.argmin(rr))
            history.append([done, round(float(rr.view(-1)[i_rho]), 6), [i_rho % nx, i_rho // nx],
                            round(float(sp.view(-1)[i_sp]), 6), [i_sp % nx, i_sp // nx]])
        advance(start - done)
        prev = None
        while done < first_bad + 1:
            with torch.cuda.stream(stream):  # the reads are queued on the lattice's stream
                rho = _field(lat, lib, 0, tmp).clone()
                ux = _field(lat, lib, 3, tmp).clone()
                uy = _field(lat, lib, 4, tmp).clone()
                bad = ~torch.isfinite(rho)
                sp = torch.sqrt(ux * ux + uy * uy)
                sp = torch.where(fl & torch.isfinite(sp), sp, torch.zeros_like(sp))
                rr = torch.where(fl, rho, torch.full_like(rho, float("inf")))
            torch.cuda.synchronize()  # everything above ran on the lattice's stream
            if bool(bad.any()):
                break
            i_sp, i_rho = int(torch.argmax(sp)), int(torch.argmin(rr))
            prev = {"step": done, "max_speed": float(sp.view(-1)[i_sp]), "max_speed_at": [i_sp % nx, i_sp // nx],
                    "min_rho": float(rr.view(-1)[i_rho]), "min_rho_at": [i_rho % nx, i_rho // nx]}
            advance(1)
        if not bool(bad.any()):
            return {"first_nonfinite_step": None}
        ys, xs = np.nonzero(bad.cpu().numpy())
        # distance to the nearest solid cell, within a window around them
        m = 256
        x0, x1 = max(int(xs.min()) - m, 0), min(int(xs.max()) + m + 1, nx)
        y0, y1 = max(int(ys.min()) - m, 0), min(int(ys.max()) + m + 1, ny)
        dist = ndimage.distance_transform_edt(mask[y0:y1, x0:x1] == 0)
        d = dist[ys - y0, xs - x0]
        rep = {"first_nonfinite_step": done, "cells": int(len(xs)),
               "x_range": [int(xs.min()), int(xs.max())], "y_range": [int(ys.min()), int(ys.max())],
               "distance_to_inlet": int(xs.min()), "distance_to_outflow": int(nx - 1 - xs.max()),
               "distance_to_nearest_solid": [float(d.min()), float(np.median(d)), float(d.max())],
               "state_one_step_earlier": prev,
               "history (step, min rho, at, max speed, at)": history}
    return rep


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--size", type=int, nargs=2, default=[16384, 8192])
    ap.add_argument("--steps", type=int, default=50000)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--tau", type=float, default=0.51)
    ap.add_argument("--u", type=float, default=0.05)
    ap.add_argument("--closure", default=None, help="train_closure output (.npz)")
    ap.add_argument("--refresh", type=int, default=20)
    ap.add_argument("--drift", type=float, default=1.0, help="closure drift bound (multiples of the predicted |u|)")
    ap.add_argument("--closure-only", action="store_true", help="skip the plain f32 and f16 runs")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--ramp", type=int, default=3000,
                    help="start at rest and raise the inlet velocity to --u over this many steps (0: start the "
                         "whole field at --u)")
    ap.add_argument("--outlet-clearance", type=int, default=128,
                    help="keep the circles this many cells from the outflow column (-1: they may touch it)")
    ap.add_argument("--stochastic", action="store_true",
                    help="round the f16 runs' stored words stochastically (lbm_set_rounding)")
    ap.add_argument("--diagnose", action="store_true",
                    help="for each run that goes non-finite, locate the first non-finite step and cells")
    a = ap.parse_args(argv)
    nx, ny = a.size
    oc = None if a.outlet_clearance < 0 else a.outlet_clearance
    mask = random_circles(nx, ny, 10 ** 7, 8, 64, a.seed, inlet_clearance=64, target_fraction=0.08,
                          outlet_clearance=oc)
    rep = {"workload": "D2Q9 channel %dx%d, circles r 8-64, %.1f%% solid, tau %.2f, ux %.2f%s%s" %
           (nx, ny, 100 * mask.mean(), a.tau, a.u, "" if oc is None else ", outflow clearance %d" % oc,
            ", inlet ramped over %d steps from rest" % a.ramp if a.ramp else "")}
    t0 = time.time()
    rep["runs"] = []
    u32 = None
    fl = mask == 0
    fl[:, 0] = False

    def err(u):
        if u32 is None:
            return None
        d = (u - u32)[:, fl]
        return float(np.linalg.norm(d) / np.linalg.norm(u32[:, fl])) if np.isfinite(d).all() else float("inf")

    def diag(r, storage, params=None):
        if a.diagnose and r["first_nonfinite_by_step"] is not None:
            r["diagnosis"] = diagnose(nx, ny, a.tau, a.u, mask, storage, r["first_nonfinite_by_step"], a.every,
                                      params=params, refresh=a.refresh, drift=a.drift, seed=a.seed, ramp=a.ramp,
                                      stochastic=a.stochastic)

    if not a.closure_only:
        r32, u32 = run(nx, ny, a.tau, a.u, mask, a.steps, a.every, F32, seed=a.seed, ramp=a.ramp)
        diag(r32, F32)
        r16, u16 = run(nx, ny, a.tau, a.u, mask, a.steps, a.every, F16, seed=a.seed, ramp=a.ramp,
                       stochastic=a.stochastic)
        diag(r16, F16)
        r16["vel_err_vs_f32"] = err(u16)
        rep["runs"] = [r32, r16]
    if a.closure:
        params = np.load(a.closure)["params"]
        rc, uc = run(nx, ny, a.tau, a.u, mask, a.steps, a.every, F16, params=params, refresh=a.refresh, ramp=a.ramp,
                     drift=a.drift, seed=a.seed, stochastic=a.stochastic)
        diag(rc, F16, params)
        rc["vel_err_vs_f32"] = err(uc)
        rc["refresh"], rc["drift"] = a.refresh, a.drift
        rep["runs"].append(rc)
    rep["wall_s"] = time.time() - t0
    print(json.dumps(rep))


if __name__ == "__main__":
    main()
