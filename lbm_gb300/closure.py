"""Learned closure: training data from fine-grid runs of this engine, training
of the relaxation-time network with the engine's own CUDA kernels, and
coarse runs that apply it (include/lbm_cnn.h).

The reference has no closure; this module adds one around the engine:

* `fine_samples` runs a fine channel lattice and turns snapshots into coarse
  training samples on the device (lbm_cnn_closure_sample): features (rho, u,
  solid) and the coefficients of an eddy-viscosity fit of the subgrid stress
  that block averaging removes (an a-priori target);
* `ClosureNet` holds the parameters, gradients and Adam state in device
  memory (torch tensors serve only as allocations and a stream) and runs
  forward / backward / loss / update through the C ABI kernels;
* `rollout_labels` turns coarse runs at a few uniform relaxation-time
  offsets into per-cell labels: which offset brings the coarse time-averaged
  velocity closest to the fine run's;
* `run_average` advances a lattice, refreshing the closure every `refresh`
  steps, and time-averages its velocity on the device.

Acoustic scaling links the grids: a coarse cell is F x F fine cells, a coarse
step is F fine steps, the lattice velocity is unchanged and the viscosity in
coarse units is nu_fine / F, i.e. tau_coarse = 0.5 + (tau_fine - 0.5) / F.
"""
import ctypes

import numpy as np

from . import EDGE_CHANNEL, F32, LBMError, Lattice, _check, load_library
from .geometry import random_circles

LAYERS = [(4, 32, True), (32, 32, True), (32, 32, True), (32, 1, False)]  # (cin, cout, relu)
N_PARAMS = sum(co * ci * 9 + co for ci, co, _ in LAYERS)
S_RHO, S_U, DT_MAX = 50.0, 10.0, 0.25


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise LBMError(2, "the closure needs a CUDA device")
    return torch


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def coarse_tau(tau_fine, factor):
    return 0.5 + (tau_fine - 0.5) / factor


def unpack(flat):
    """Packed parameters -> [[w (cout, cin, 3, 3), b (cout)], ...]."""
    out, o = [], 0
    for ci, co, _ in LAYERS:
        w = flat[o:o + co * ci * 9].reshape(co, ci, 3, 3)
        o += co * ci * 9
        out.append([w, flat[o:o + co]])
        o += co
    return out


def pack(params):
    return np.concatenate([np.concatenate([np.asarray(w).reshape(-1), np.asarray(b).reshape(-1)])
                           for w, b in params]).astype(np.float32)


def round_bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(np.shape(a))


def init_params(seed):
    """He-uniform weights from a seeded generator, zero biases; the last
    layer scaled by 0.1."""
    rng = np.random.default_rng(seed)
    params = []
    for i, (ci, co, _) in enumerate(LAYERS):
        lim = np.sqrt(6.0 / (ci * 9)) * (0.1 if i == len(LAYERS) - 1 else 1.0)
        params.append([rng.uniform(-lim, lim, (co, ci, 3, 3)), np.zeros(co)])
    return pack(params)


class ClosureNet:
    """Network parameters and work buffers on the current CUDA device."""

    def __init__(self, params=None, seed=0):
        self.torch = torch = _torch()
        self.lib = load_library()
        flat = init_params(seed) if params is None else np.asarray(params, np.float32)
        if flat.size != N_PARAMS:
            raise ValueError("need %d parameters" % N_PARAMS)
        dev = torch.device("cuda")
        self.params = torch.from_numpy(flat.copy()).to(dev)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.t = 0
        self.scratch = torch.empty(max(self.lib.lbm_cnn_weight_scratch_bytes(ci, co) for ci, co, _ in LAYERS) // 4,
                                   dtype=torch.float32, device=dev)
        self.loss_scratch = torch.empty(608, dtype=torch.float64, device=dev)
        self.loss_out = torch.empty(1, dtype=torch.float64, device=dev)
        self._acts = None

    def _views(self, buf):
        out, o = [], 0
        for ci, co, _ in LAYERS:
            w = buf[o:o + co * ci * 9]
            o += co * ci * 9
            out.append((w, buf[o:o + co]))
            o += co
        return out

    @property
    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def numpy(self):
        return self.params.cpu().numpy()

    def forward(self, feat):
        """feat: [N, 4, H, W] float32 CUDA tensor -> z [N, 1, H, W]."""
        torch = self.torch
        N, _, H, W = feat.shape
        acts = [feat.contiguous()]
        for (w, b), (ci, co, relu) in zip(self._views(self.params), LAYERS):
            y = torch.empty((N, co, H, W), dtype=torch.float32, device=feat.device)
            _check(self.lib.lbm_cnn_conv_forward(_p(acts[-1]), N, ci, H, W, _p(w), _p(b), co, 1 if relu else 0, _p(y),
                                                 self.stream))
            acts.append(y)
        self._acts = acts
        return acts[-1]

    def backward(self, gz):
        """Gradients of the last forward w.r.t. the parameters, into self.grads."""
        torch = self.torch
        acts = self._acts
        N, _, H, W = acts[0].shape
        g = gz.contiguous()
        views = self._views(self.params)
        gviews = self._views(self.grads)
        for l in range(len(LAYERS) - 1, -1, -1):
            ci, co, relu = LAYERS[l]
            out = acts[l + 1] if relu else None
            outp = _p(out) if out is not None else None
            _check(self.lib.lbm_cnn_conv_backward_weight(_p(acts[l]), _p(g), outp, N, ci, H, W, co, _p(gviews[l][0]),
                                                         _p(gviews[l][1]), _p(self.scratch),
                                                         self.scratch.numel() * 4, self.stream))
            if l > 0:
                gx = torch.empty((N, ci, H, W), dtype=torch.float32, device=g.device)
                _check(self.lib.lbm_cnn_conv_backward_data(_p(g), outp, N, ci, H, W, _p(views[l][0]), co, _p(gx),
                                                           self.stream))
                g = gx

    def loss(self, z, coef, norm, grad=True):
        """Closure loss (a device scalar, float64) and, with grad, dL/dz."""
        N, _, H, W = z.shape
        gz = self.torch.empty_like(z) if grad else None
        _check(self.lib.lbm_cnn_closure_loss(_p(z), _p(coef), N, H, W, float(norm), _p(gz) if grad else None,
                                             _p(self.loss_scratch), _p(self.loss_out), self.stream))
        return self.loss_out, gz

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.t += 1
        _check(self.lib.lbm_cnn_adam(_p(self.params), _p(self.grads), _p(self.m), _p(self.v), N_PARAMS, self.t,
                                     float(lr), b1, b2, eps, self.stream))


def sample(lib, stream, pops, solid_f, factor, feat, coef, scratch, solid_c):
    hf, wf = solid_f.shape
    _check(lib.lbm_cnn_closure_sample(_p(pops), _p(solid_f), hf, wf, factor, _p(feat), _p(coef), _p(scratch),
                                      _p(solid_c), stream))


def fine_samples(mask, tau, u, steps, every, factor, seed=0, noise=1e-3, start=0, storage=F32):
    """Run a fine channel lattice with `mask` for `steps` steps and return the
    coarse samples of the snapshots taken every `every` steps from step
    `start` on: (feat [S, 4, H, W], coef [S, 3, H, W], coarse solid [H, W]) as
    CUDA tensors."""
    torch = _torch()
    lib = load_library()
    ny, nx = mask.shape
    H, W = ny // factor, nx // factor
    dev = torch.device("cuda")
    times = list(range(max(start, every), steps + 1, every))
    feat = torch.empty((len(times), 4, H, W), dtype=torch.float32, device=dev)
    coef = torch.empty((len(times), 3, H, W), dtype=torch.float32, device=dev)
    solid_c = torch.empty((H, W), dtype=torch.uint8, device=dev)
    solid_f = torch.from_numpy(np.ascontiguousarray(mask, dtype=np.uint8)).to(dev)
    pops = torch.empty((9, ny, nx), dtype=torch.float32, device=dev)
    scratch = torch.empty(6 * H * W, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    with Lattice(nx, ny, 1.0 / tau, EDGE_CHANNEL, storage) as lat:
        lat.set_stream(stream.cuda_stream)
        lat.set_inlet_velocity(u)
        lat.init_equilibrium(1.0, u, 0.0, noise, seed)
        lat.draw_mask(mask)
        done = 0
        for k, t in enumerate(times):
            lat.iterate(t - done)
            done = t
            _check(lib.lbm_read_populations_device(lat.handle, _p(pops)))
            sample(lib, ctypes.c_void_p(stream.cuda_stream), pops, solid_f, factor, feat[k], coef[k], scratch,
                   solid_c)
        lat.synchronize()
    return feat, coef, solid_c


def _device_velocity(lat, torch, pops):
    _check(load_library().lbm_read_populations_device(lat.handle, _p(pops)))
    rho = pops.sum(0)
    jx = pops[2] + pops[5] + pops[8] - pops[0] - pops[3] - pops[6]
    jy = pops[0] + pops[1] + pops[2] - pops[6] - pops[7] - pops[8]
    return torch.stack([jx / rho, jy / rho])


def run_average(nx, ny, tau, u, mask, steps, every, avg_from, seed, params=None, refresh=20, drift=0.5,
                storage=F32, noise=1e-3):
    """Run a channel lattice; returns (time-averaged velocity [2, ny, nx] over
    steps avg_from..steps as float64 numpy, seconds spent stepping, fallback
    cell-steps).  With params the closure is refreshed every `refresh` steps.
    Averaging reads stay on the device and outside the timing."""
    import time
    torch = _torch()
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
        lat.init_equilibrium(1.0, u, 0.0, noise, seed)
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
        except LBMError:
            pass  # a run that went non-finite shows up as non-finite averages
    return (acc / max(n, 1)).cpu().numpy(), t_step, fb.value


def time_run(nx, ny, tau, u, mask, steps, seed, params=None, refresh=20, drift=0.5, storage=F32, noise=1e-3,
             warmup=40):
    """Seconds of device time for `steps` steps (plus the closure's
    inferences every `refresh` steps), timed with CUDA events on the
    lattice's stream after a warm-up, with no readback in between."""
    torch = _torch()
    lib = load_library()
    stream = torch.cuda.Stream()
    with Lattice(nx, ny, 1.0 / tau, EDGE_CHANNEL, storage) as lat:
        lat.set_stream(stream.cuda_stream)
        lat.set_inlet_velocity(u)
        lat.init_equilibrium(1.0, u, 0.0, noise, seed)
        lat.draw_mask(mask)
        if params is not None:
            p = np.ascontiguousarray(params, np.float32)
            _check(lib.lbm_closure_set_weights(lat.handle, p.ctypes.data_as(ctypes.c_void_p), p.size))
            _check(lib.lbm_closure_enable(lat.handle, float(drift)))

        def run(n):
            done = 0
            while done < n:
                k = min(refresh, n - done) if params is not None else n - done
                if params is not None:
                    _check(lib.lbm_closure_infer(lat.handle))
                lat.iterate(k)
                done += k

        run(warmup)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        run(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        try:
            lat.synchronize()
        except LBMError:
            pass
        return e0.elapsed_time(e1) * 1e-3


def block_average(u, mask, F):
    """Average [2, ny, nx] over the fluid cells of F x F blocks."""
    ny, nx = mask.shape
    fl = (mask == 0).astype(np.float64)[:ny // F * F, :nx // F * F].reshape(ny // F, F, nx // F, F)
    uu = u[:, :ny // F * F, :nx // F * F].reshape(2, ny // F, F, nx // F, F)
    with np.errstate(invalid="ignore"):
        return (uu * fl[None]).sum(axis=(2, 4)) / np.maximum(fl.sum(axis=(1, 3)), 1)


def rel_error(uc, uf, solid_c):
    """Relative L2 error of a coarse time-averaged velocity over the fluid
    cells off the inlet column (inf when the run went non-finite)."""
    fl = solid_c == 0
    fl[:, 0] = False
    d = (uc - uf)[:, fl]
    if not np.isfinite(d).all():
        return float("inf")
    return float(np.linalg.norm(d) / np.linalg.norm(uf[:, fl]))


def coarse_solid(mask, factor):
    ny, nx = mask.shape
    fl = (mask[:ny // factor * factor, :nx // factor * factor] == 0).reshape(ny // factor, factor, nx // factor,
                                                                             factor)
    return (2 * fl.sum(axis=(1, 3)) < factor * factor).astype(np.uint8)


CANDIDATES = (0.0, 0.005, 0.01, 0.02, 0.04, 0.08)


def _box(a, r):
    """Mean over a (2r+1)^2 window (edges replicated)."""
    p = np.pad(a, r, mode="edge")
    c = np.cumsum(np.cumsum(p, 0), 1)
    c = np.pad(c, ((1, 0), (1, 0)))
    k = 2 * r + 1
    return (c[k:, k:] - c[:-k, k:] - c[k:, :-k] + c[:-k, :-k]) / (k * k)


def rollout_labels(mask_c, tau_c, u, steps_c, every_c, uf_c, seed, candidates=CANDIDATES, smooth=2):
    """Per-cell relaxation-time labels from candidate rollouts: the coarse
    lattice is run at each uniform delta_tau candidate, its time-averaged
    velocity compared with the block-averaged fine one, the squared error
    smoothed over a (2 smooth + 1)^2 window and fitted per cell by a parabola
    in delta_tau (least squares over the candidates that stayed finite).  The
    label is the parabola's minimum clipped to the range of those candidates
    (the best candidate where the fit is not convex) and the weight is how much the error varies
    across the candidates.  Returns (label [H, W], weight [H, W], errors
    per candidate as relative L2)."""
    H, W = mask_c.shape
    errs, rels = [], []
    for dt in candidates:
        uc, _, _ = run_average(W, H, tau_c + dt, u, mask_c, steps_c, every_c, steps_c // 2, seed)
        e = ((uc - uf_c) ** 2).sum(0)
        errs.append(_box(e, smooth) if np.isfinite(e).all() else np.full((H, W), np.inf))
        rels.append(rel_error(uc, uf_c, mask_c))
    E = np.stack(errs)  # [K, H, W]
    x = np.asarray(candidates, np.float64)
    ok = np.isfinite(E).all(axis=(1, 2))
    label = np.zeros((H, W))
    weight = np.zeros((H, W))
    if ok.sum() >= 1:
        Ek, xk = E[ok], x[ok]
        best = xk[np.argmin(Ek, axis=0)]
        label = best.copy()
        if ok.sum() >= 3:
            V = np.stack([xk * xk, xk, np.ones_like(xk)], 1)  # e ~ a x^2 + b x + c
            coef, *_ = np.linalg.lstsq(V, Ek.reshape(len(xk), -1), rcond=None)
            a, b = coef[0].reshape(H, W), coef[1].reshape(H, W)
            with np.errstate(divide="ignore", invalid="ignore"):
                vert = np.clip(-b / (2 * a), xk.min(), xk.max())  # never below a candidate that diverged
            label = np.where(a > 0, vert, best)
        weight = Ek.max(0) - Ek.min(0)
        if not ok.all():  # diverged candidates: low delta_tau is unsafe, weigh the choice fully
            weight = np.maximum(weight, np.nanmax(weight))
    fl = mask_c == 0
    fl[:, 0] = False
    weight = np.where(fl, weight, 0.0)
    s = weight[fl].mean() if fl.any() and weight[fl].mean() > 0 else 1.0
    return label, weight / s, rels


def training_layouts(count, seed, nx, ny, rmin, rmax, fraction=0.1, clearance=64):
    """Seeded random-circle layouts for the fine runs."""
    return [random_circles(nx, ny, 10 ** 6, rmin, rmax, seed * 1000 + i, inlet_clearance=clearance,
                           target_fraction=fraction) for i in range(count)]
