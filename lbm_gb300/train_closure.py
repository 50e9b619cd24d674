"""Train and evaluate the learned closure on fine-grid runs of this engine.

    python -m lbm_gb300.train_closure [--fine 2048 1024] [--train 64] [--test 16]
        [--steps 8000] [--every 20] [--factor 4] [--tau 0.52] [--u 0.06]
        [--iters 3000] [--batch 4] [--lr 2e-3] [--refresh 20] [--out closure.npz]

Data: `--train` seeded random-circle layouts (radii 8-40 fine cells, ~10 %
solid, none within 64 cells of the inlet) run on the fine grid for `--steps`
steps at tau / u; every `--every` steps a snapshot becomes a coarse training
sample on the device (features and the subgrid-stress fit coefficients).  Training: Adam on minibatches of
`--batch` snapshots with the engine's own forward / backward kernels.
Evaluation on `--test` held-out layouts: time-averaged velocity of the second
half of each run, fine (block-averaged to the coarse grid) against coarse
plain BGK and coarse with the closure, and the wall time of each run.
Prints one JSON report; saves the weights and the report to `--out`.
"""
import argparse
import ctypes
import json
import time

import numpy as np

from . import EDGE_CHANNEL, F32, Lattice, _check, load_library
from . import closure as cl


def _device_velocity(lat, torch, pops):
    _check(load_library().lbm_read_populations_device(lat.handle, ctypes.c_void_p(pops.data_ptr())))
    rho = pops.sum(0)
    jx = pops[2] + pops[5] + pops[8] - pops[0] - pops[3] - pops[6]
    jy = pops[0] + pops[1] + pops[2] - pops[6] - pops[7] - pops[8]
    return torch.stack([jx / rho, jy / rho])


def run_average(torch, nx, ny, tau, u, mask, steps, every, avg_from, seed, params=None, refresh=20, drift=0.5,
                storage=F32):
    """Run a channel lattice; returns (time-averaged velocity [2, ny, nx] over
    steps avg_from..steps as float64 numpy, seconds spent stepping, fallback
    cell-steps).  Averaging reads stay on the device and outside the timing."""
    lib = load_library()
    dev = torch.device("cuda")
    pops = torch.empty((9, ny, nx), dtype=torch.float32, device=dev)
    acc = torch.zeros((2, ny, nx), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    n = 0
    t_step = 0.0
    fb = ctypes.c_uint64(0)
    with Lattice(nx, ny, 1.0 / tau, EDGE_CHANNEL, storage) as lat:
        lat.set_stream(stream.cuda_stream)
        lat.set_inlet_velocity(u)
        lat.init_equilibrium(1.0, u, 0.0, 1e-3, seed)
        lat.draw_mask(mask)
        if params is not None:
            p = np.ascontiguousarray(params, np.float32)
            _check(lib.lbm_closure_set_weights(lat.handle, p.ctypes.data_as(ctypes.c_void_p), p.size))
            _check(lib.lbm_closure_enable(lat.handle, float(drift)))
        done = 0
        chunk = min(every, refresh) if params is not None else every
        while done < steps:
            k = min(chunk, steps - done)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if params is not None and done % refresh == 0:
                _check(lib.lbm_closure_infer(lat.handle))
            lat.iterate(k)
            torch.cuda.synchronize()
            t_step += time.perf_counter() - t0
            done += k
            if done > avg_from and done % every == 0:
                acc += _device_velocity(lat, torch, pops).double()
                n += 1
        if params is not None:
            _check(lib.lbm_closure_fallback_count(lat.handle, ctypes.byref(fb), 1))
        try:
            lat.synchronize()
        except Exception:
            pass  # a run that went non-finite is reported through its error, not raised
    return (acc / max(n, 1)).cpu().numpy(), t_step, fb.value


def block_average(u, mask, F):
    ny, nx = mask.shape
    fl = (mask == 0).astype(np.float64)[:ny // F * F, :nx // F * F].reshape(ny // F, F, nx // F, F)
    uu = np.nan_to_num(u[:, :ny // F * F, :nx // F * F]).reshape(2, ny // F, F, nx // F, F)
    return (uu * fl[None]).sum(axis=(2, 4)) / np.maximum(fl.sum(axis=(1, 3)), 1)


def rel_error(uc, uf, solid_c):
    fl = solid_c == 0
    fl[:, 0] = False
    d = (uc - uf)[:, fl]
    if not np.isfinite(d).all():
        return float("inf")
    return float(np.linalg.norm(d) / np.linalg.norm(uf[:, fl]))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--fine", type=int, nargs=2, default=[2048, 1024])
    ap.add_argument("--train", type=int, default=64)
    ap.add_argument("--test", type=int, default=16)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--start", type=int, default=0, help="first snapshot step")
    ap.add_argument("--factor", type=int, default=4)
    ap.add_argument("--tau", type=float, default=0.52)
    ap.add_argument("--u", type=float, default=0.06)
    ap.add_argument("--rmin", type=float, default=8.0)
    ap.add_argument("--rmax", type=float, default=40.0)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--refresh", type=int, default=20)
    ap.add_argument("--drift", type=float, default=0.5)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default="closure.npz")
    a = ap.parse_args(argv)
    torch = cl._torch()
    nx, ny = a.fine
    F = a.factor
    tau_c = cl.coarse_tau(a.tau, F)
    rep = {"fine": [nx, ny], "factor": F, "tau_fine": a.tau, "tau_coarse": tau_c, "u": a.u, "steps_fine": a.steps,
           "train_layouts": a.train, "test_layouts": a.test}
    layouts = cl.training_layouts(a.train + a.test, a.seed, nx, ny, a.rmin, a.rmax)

    # ---- data ------------------------------------------------------------------
    t0 = time.perf_counter()
    feats, coefs = [], []
    for i in range(a.train):
        f, c, _ = cl.fine_samples(layouts[i], a.tau, a.u, a.steps, a.every, F, seed=a.seed * 7919 + i,
                                  start=a.start)
        feats.append(f)
        coefs.append(c)
    feat = torch.cat(feats)
    coef = torch.cat(coefs)
    del feats, coefs
    norms = coef[:, 2].sum(dim=(1, 2)).double().cpu().numpy()
    torch.cuda.synchronize()
    rep["samples"] = int(feat.shape[0])
    rep["data_seconds"] = time.perf_counter() - t0

    # ---- training --------------------------------------------------------------
    net = cl.ClosureNet(seed=a.seed)
    rng = np.random.default_rng(a.seed)
    S = feat.shape[0]
    t0 = time.perf_counter()
    hist = []
    for it in range(a.iters):
        idx = rng.choice(S, size=min(a.batch, S), replace=False)
        it_t = torch.from_numpy(idx).cuda()
        fb, cb = feat.index_select(0, it_t), coef.index_select(0, it_t)
        lr = a.lr * (0.1 ** (it / max(a.iters, 1)))  # exponential decay to lr / 10
        z = net.forward(fb)
        L, gz = net.loss(z, cb, float(norms[idx].sum()))
        net.backward(gz)
        net.adam(lr)
        if it % max(a.iters // 20, 1) == 0 or it == a.iters - 1:
            hist.append([it, float(L.item())])
    torch.cuda.synchronize()
    rep["train_seconds"] = time.perf_counter() - t0
    rep["loss_history"] = hist
    params = net.numpy()
    # loss with delta_tau = 0 (plain coarse BGK: the whole subgrid stress unexplained) and trained
    k = min(S, 64)
    zero_z = torch.full((k, 1) + tuple(feat.shape[2:]), -30.0, device=feat.device)
    L0, _ = net.loss(zero_z, coef[:k], float(norms[:k].sum()), grad=False)
    rep["loss_plain"] = float(L0.item())
    L1, _ = net.loss(net.forward(feat[:k]), coef[:k], float(norms[:k].sum()), grad=False)
    rep["loss_trained"] = float(L1.item())
    del feat, coef

    # ---- evaluation ------------------------------------------------------------
    steps_c = a.steps // F
    per = []
    for j in range(a.test):
        m = layouts[a.train + j]
        sc = cl.coarse_solid(m, F)
        seed = a.seed * 7919 + a.train + j
        uf, tf, _ = run_average(torch, nx, ny, a.tau, a.u, m, a.steps, a.every, a.steps // 2, seed)
        ufc = block_average(uf, m, F)
        up, tp, _ = run_average(torch, nx // F, ny // F, tau_c, a.u, sc, steps_c, max(a.every // F, 1), steps_c // 2,
                                seed)
        uc, tc, fb = run_average(torch, nx // F, ny // F, tau_c, a.u, sc, steps_c, max(a.every // F, 1),
                                 steps_c // 2, seed, params=params, refresh=a.refresh, drift=a.drift)
        active = int((sc == 0)[:, 1:].sum()) * steps_c
        per.append({"layout": a.train + j, "err_plain": rel_error(up, ufc, sc), "err_closure": rel_error(uc, ufc, sc),
                    "fine_seconds": tf, "plain_seconds": tp, "closure_seconds": tc,
                    "fallback_fraction": fb / max(active, 1)})
    rep["per_layout"] = per
    ep = [p["err_plain"] for p in per]
    ec = [p["err_closure"] for p in per]
    rep["median_err_plain"] = float(np.median(ep))
    rep["median_err_closure"] = float(np.median(ec))
    rep["speedup_vs_fine"] = float(np.median([p["fine_seconds"] / p["closure_seconds"] for p in per]))
    np.savez(a.out, params=params, report=json.dumps(rep))
    print(json.dumps(rep))
    return rep


if __name__ == "__main__":
    main()
