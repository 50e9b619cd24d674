"""Train and evaluate the learned closure on fine-grid runs of this engine.

    python -m lbm_gb300.train_closure [--fine 2048 1024] [--train 64] [--test 16]
        [--steps 8000] [--every 20] [--factor 4] [--tau 0.52] [--u 0.06]
        [--iters 3000] [--batch 4] [--lr 2e-3] [--refresh 20] [--out closure.npz]

Data: `--train` seeded random-circle layouts (radii `--rmin`..`--rmax` fine
cells, default 6-20, up to `--fraction` solid, none within 64 cells of the
inlet) run on the fine grid for `--steps`
steps at tau / u; every `--every` steps a snapshot becomes a coarse sample
on the device (features: rho, u, solid).  Target (`--target rollout`, the
default): per-cell relaxation-time labels from coarse runs at a few uniform
delta_tau offsets, fitted against the fine run's time-averaged velocity
(closure.rollout_labels); `--target sgs` fits an eddy viscosity to the
subgrid stress of each snapshot instead (an a-priori target).  Training: Adam on minibatches of
`--batch` snapshots with the engine's own forward / backward kernels.
Evaluation on `--test` held-out layouts: time-averaged velocity of the second
half of each run, fine (block-averaged to the coarse grid) against coarse
plain BGK and coarse with the closure, and the wall time of each run.
Prints one JSON report; saves the weights and the report to `--out`.
"""
import argparse
import json
import time

import numpy as np

from . import LBMError
from . import closure as cl


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
    ap.add_argument("--rmin", type=float, default=6.0)
    ap.add_argument("--rmax", type=float, default=20.0)
    ap.add_argument("--fraction", type=float, default=0.08)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--refresh", type=int, default=20)
    ap.add_argument("--drift", type=float, default=1.0)
    ap.add_argument("--target", choices=["rollout", "sgs"], default="rollout")
    ap.add_argument("--eval-only", default=None, metavar="NPZ",
                    help="skip data and training; evaluate the weights in this file")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default="closure.npz")
    a = ap.parse_args(argv)
    torch = cl._torch()
    nx, ny = a.fine
    F = a.factor
    tau_c = cl.coarse_tau(a.tau, F)
    rep = {"fine": [nx, ny], "factor": F, "tau_fine": a.tau, "tau_coarse": tau_c, "u": a.u, "steps_fine": a.steps,
           "train_layouts": a.train, "test_layouts": a.test}
    layouts = cl.training_layouts(a.train + a.test, a.seed, nx, ny, a.rmin, a.rmax, fraction=a.fraction)

    steps_c, every_c = a.steps // F, max(a.every // F, 1)
    if a.eval_only:
        saved = np.load(a.eval_only)
        params = saved["params"]
        label_err = []
        rep["weights"] = a.eval_only
        rep["best_uniform_delta_tau"] = json.loads(str(saved["report"])).get("best_uniform_delta_tau", 0.01)
        return evaluate(a, rep, layouts, params, tau_c, steps_c, every_c, nx, ny, F)

    # ---- data ------------------------------------------------------------------
    t0 = time.perf_counter()
    # features per snapshot; coefficients per snapshot (sgs) or per layout
    # (rollout labels, shared by the layout's snapshots): coef_of[sample]
    feats, coefs, coef_of, label_err = [], [], [], []
    skipped = []
    for i in range(a.train):
        seed = a.seed * 7919 + i
        try:
            f, c, _ = cl.fine_samples(layouts[i], a.tau, a.u, a.steps, a.every, F, seed=seed, start=a.start)
        except LBMError:  # the fine BGK run itself went non-finite: no data from this layout
            skipped.append(i)
            continue
        if a.target == "rollout":
            uf, _, _ = cl.run_average(nx, ny, a.tau, a.u, layouts[i], a.steps, a.every, a.steps // 2, seed)
            sc = cl.coarse_solid(layouts[i], F)
            label, w, rels = cl.rollout_labels(sc, tau_c, a.u, steps_c, every_c, cl.block_average(uf, layouts[i], F),
                                               seed)
            label_err.append(rels)
            c = torch.from_numpy(np.stack([w, w * label, w * label * label]).astype(np.float32)).cuda()[None]
            coef_of += [len(coefs)] * f.shape[0]
        else:
            coef_of += list(range(sum(x.shape[0] for x in coefs), sum(x.shape[0] for x in coefs) + f.shape[0]))
        feats.append(f)
        coefs.append(c)
    feat = torch.cat(feats)
    coef = torch.cat(coefs)
    coef_of = np.asarray(coef_of)
    del feats, coefs
    # loss normalisation per sample: the weighted mean squared delta_tau error
    # (rollout labels) or the fraction of the subgrid stress left unexplained
    norms = coef[:, 0 if a.target == "rollout" else 2].sum(dim=(1, 2)).double().cpu().numpy()[coef_of]
    norms = np.where(norms > 0, norms, 1.0)
    torch.cuda.synchronize()
    rep["samples"] = int(feat.shape[0])
    rep["train_layouts_nonfinite_fine"] = skipped
    rep["target"] = a.target
    if label_err:
        rep["candidates"] = list(cl.CANDIDATES)
        rep["candidate_rel_err_median"] = [float(np.median([r[k] for r in label_err])) for k in
                                           range(len(cl.CANDIDATES))]
    rep["data_seconds"] = time.perf_counter() - t0

    # ---- training --------------------------------------------------------------
    # start the output bias at the weighted mean label: the sigmoid then starts
    # in its responsive range instead of saturating toward delta_tau = 0
    init = cl.init_params(a.seed)
    sw = float(coef[:, 0].sum().item())
    mean_label = float(coef[:, 1].sum().item()) / sw if sw > 0 else 0.01  # per layout: equal weight per layout
    frac = min(max(mean_label / cl.DT_MAX, 1e-3), 0.999)
    init[-1] = np.float32(np.log(frac / (1.0 - frac)))
    rep["mean_label"] = mean_label
    net = cl.ClosureNet(params=init)
    rng = np.random.default_rng(a.seed)
    S = feat.shape[0]
    t0 = time.perf_counter()
    hist = []
    for it in range(a.iters):
        idx = rng.choice(S, size=min(a.batch, S), replace=False)
        it_t = torch.from_numpy(idx).cuda()
        fb = feat.index_select(0, it_t)
        cb = coef.index_select(0, torch.from_numpy(coef_of[idx]).cuda())
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
    # loss of delta_tau = 0 (plain coarse BGK) and of the trained network on the first samples
    k = min(S, 64)
    ck = coef.index_select(0, torch.from_numpy(coef_of[:k]).cuda())
    zero_z = torch.full((k, 1) + tuple(feat.shape[2:]), -30.0, device=feat.device)
    L0, _ = net.loss(zero_z, ck, float(norms[:k].sum()), grad=False)
    rep["loss_plain"] = float(L0.item())
    L1, _ = net.loss(net.forward(feat[:k]), ck, float(norms[:k].sum()), grad=False)
    rep["loss_trained"] = float(L1.item())
    del feat, coef

    if label_err:
        med = rep["candidate_rel_err_median"]
        rep["best_uniform_delta_tau"] = float(cl.CANDIDATES[int(np.argmin(med))])
    return evaluate(a, rep, layouts, params, tau_c, steps_c, every_c, nx, ny, F)


def evaluate(a, rep, layouts, params, tau_c, steps_c, every_c, nx, ny, F):
    # ---- evaluation ------------------------------------------------------------
    # baselines: plain coarse BGK (delta_tau = 0) and the uniform candidate
    # with the lowest median error over the training layouts
    best_dt = rep.get("best_uniform_delta_tau", 0.0)
    per = []
    for j in range(a.test):
        m = layouts[a.train + j]
        sc = cl.coarse_solid(m, F)
        seed = a.seed * 7919 + a.train + j
        uf, _, _ = cl.run_average(nx, ny, a.tau, a.u, m, a.steps, a.every, a.steps // 2, seed)
        if not np.isfinite(uf).all():  # the fine run went non-finite: no reference for this layout
            per.append({"layout": a.train + j, "fine_nonfinite": True})
            continue
        ufc = cl.block_average(uf, m, F)
        up, _, _ = cl.run_average(nx // F, ny // F, tau_c, a.u, sc, steps_c, every_c, steps_c // 2, seed)
        ub, _, _ = cl.run_average(nx // F, ny // F, tau_c + best_dt, a.u, sc, steps_c, every_c, steps_c // 2, seed)
        uc, _, fb = cl.run_average(nx // F, ny // F, tau_c, a.u, sc, steps_c, every_c, steps_c // 2, seed,
                                   params=params, refresh=a.refresh, drift=a.drift)
        tf = cl.time_run(nx, ny, a.tau, a.u, m, a.steps, seed)
        tc = cl.time_run(nx // F, ny // F, tau_c, a.u, sc, steps_c, seed, params=params, refresh=a.refresh,
                         drift=a.drift)
        tp = cl.time_run(nx // F, ny // F, tau_c + best_dt, a.u, sc, steps_c, seed)
        active = int((sc == 0)[:, 1:].sum()) * steps_c
        per.append({"layout": a.train + j, "err_plain": cl.rel_error(up, ufc, sc),
                    "err_best_uniform": cl.rel_error(ub, ufc, sc), "err_closure": cl.rel_error(uc, ufc, sc),
                    "fine_seconds": tf, "uniform_seconds": tp, "closure_seconds": tc,
                    "fallback_fraction": fb / max(active, 1)})
    rep["per_layout"] = per
    per = [p for p in per if "err_plain" in p]
    ep = [p["err_plain"] for p in per]
    ec = [p["err_closure"] for p in per]
    rep["median_err_plain"] = float(np.median(ep))
    rep["median_err_closure"] = float(np.median(ec))
    rep["median_err_best_uniform"] = float(np.median([p["err_best_uniform"] for p in per]))
    rep["speedup_vs_fine"] = float(np.median([p["fine_seconds"] / p["closure_seconds"] for p in per]))
    rep["closure_better_than_plain"] = int(sum(p["err_closure"] < p["err_plain"] for p in per))
    rep["closure_better_than_best_uniform"] = int(sum(p["err_closure"] < p["err_best_uniform"] for p in per))
    rep["refresh"] = a.refresh
    np.savez(a.out, params=params, report=json.dumps(rep))
    print(json.dumps(rep))
    return rep


if __name__ == "__main__":
    main()
