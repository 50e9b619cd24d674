"""Learned-closure kernels on the GPU against the float64 CPU oracle
(oracle/cnn_oracle.py).

Tolerances (f32 kernels against f64 maths): layer outputs and gradients
within 1e-5 relative to the largest magnitude of the compared array; the
closure records within binary16 rounding (2e-3 relative); the per-cell
relaxation path bit-exact against a plain run at the same omega."""
import ctypes

import numpy as np
import pytest

from oracle import cnn_oracle as C

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(cuda_ok):
    import torch
    return torch


def close(got, want, tol=1e-5, atol=0.0):
    got = np.asarray(got, np.float64)
    scale = max(np.abs(want).max(), 1e-30)
    err = np.abs(got - want).max()
    assert err <= tol * scale + atol, "max error %.3e of scale %.3e" % (err, scale)


def params_for(seed):
    from lbm_gb300 import closure
    return closure.unpack(closure.init_params(seed).astype(np.float64))


def test_gpu_conv_layers_forward_and_backward(lbm, torch_cuda, oracle_mod):
    torch = torch_cuda
    from lbm_gb300 import closure
    net = closure.ClosureNet(seed=5)
    ps = closure.unpack(net.numpy().astype(np.float64))
    rng = np.random.default_rng(1)
    N, H, W = 2, 13, 150
    feat = rng.normal(size=(N, 4, H, W)) * np.array([0.3, 0.6, 0.2, 1.0])[None, :, None, None]
    ft = torch.from_numpy(feat.astype(np.float32)).cuda()
    z = net.forward(ft)
    acts = C.forward(ps, feat.astype(np.float32).astype(np.float64))
    for l in range(1, 5):
        close(net._acts[l].cpu().numpy(), acts[l])
    gz = rng.normal(size=(N, 1, H, W))
    net.backward(torch.from_numpy(gz.astype(np.float32)).cuda())
    grads = C.backward(ps, acts, gz.astype(np.float32).astype(np.float64))
    got = closure.unpack(net.grads.cpu().numpy().astype(np.float64))
    for l in range(4):
        close(got[l][0], grads[l][0], 2e-5)
        close(got[l][1], grads[l][1], 2e-5)
    torch.cuda.synchronize()


def test_gpu_closure_loss_and_full_gradient(lbm, torch_cuda):
    torch = torch_cuda
    from lbm_gb300 import closure
    net = closure.ClosureNet(seed=7)
    ps = closure.unpack(net.numpy().astype(np.float64))
    rng = np.random.default_rng(2)
    N, H, W = 3, 17, 40
    feat = (rng.normal(size=(N, 4, H, W)) * 0.5).astype(np.float32)
    sxx, sxy = rng.normal(size=(2, N, H, W)) * 1e-2
    dxx = -0.02 * sxx + 1e-4 * rng.normal(size=sxx.shape)
    txy = -0.02 * sxy + 1e-4 * rng.normal(size=sxy.shape)
    coef = np.stack([(8 / 9) * (sxx ** 2 + sxy ** 2), -(4 / 3) * (dxx * sxx + txy * sxy),
                     2 * (dxx ** 2 + txy ** 2)], axis=1).astype(np.float32)
    norm = float(coef[:, 2].sum())
    z = net.forward(torch.from_numpy(feat).cuda())
    L, gz = net.loss(z, torch.from_numpy(coef).cuda(), norm)
    acts = C.forward(ps, feat.astype(np.float64))
    L64, gz64 = C.loss(acts[-1], coef.astype(np.float64), norm)
    assert float(L.item()) == pytest.approx(L64, rel=1e-5)
    close(gz.cpu().numpy(), gz64, 1e-4)
    net.backward(gz)
    g64 = C.backward(ps, acts, gz64)
    got = closure.unpack(net.grads.cpu().numpy().astype(np.float64))
    for l in range(4):
        close(got[l][0], g64[l][0], 2e-4)
        close(got[l][1], g64[l][1], 2e-4)


def test_gpu_adam_matches_oracle(lbm, torch_cuda):
    torch = torch_cuda
    from lbm_gb300 import closure
    net = closure.ClosureNet(seed=3)
    p = net.numpy().astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    rng = np.random.default_rng(3)
    for t in range(1, 4):
        g = rng.normal(size=p.size).astype(np.float32)
        net.grads.copy_(torch.from_numpy(g))
        net.adam(1e-3)
        C.adam(p, g.astype(np.float64), m, v, t, 1e-3)
    close(net.numpy(), p, 1e-6)


def test_gpu_closure_samples_match_oracle(lbm, torch_cuda):
    """Samples of a real fine run (96 x 64 channel, circle) at three snapshots."""
    from lbm_gb300 import closure, geometry
    mask = geometry.single_circle(96, 64, 30, 31.5, 7)
    feat, coef, solid_c = closure.fine_samples(mask, 0.55, 0.06, 60, 20, 4, seed=1)
    with lbm.Lattice(96, 64, 1.0 / 0.55, lbm.EDGE_CHANNEL, lbm.F32) as lat:
        lat.set_inlet_velocity(0.06)
        lat.init_equilibrium(1.0, 0.06, 0.0, 1e-3, 1)
        lat.draw_mask(mask)
        for k in range(3):
            lat.iterate(20)
            pops = lat.populations().astype(np.float64)
            f64, c64 = C.sample(pops, mask, 4)
            close(feat[k].cpu().numpy(), f64, 1e-5)
            # the stresses are differences of O(u^2) f32 products (subgrid
            # variances ~1e-6 of u^2 ~ 4e-3): f32 leaves ~1e-3 relative on them
            for j in range(3):
                close(coef[k, j].cpu().numpy(), c64[j], 5e-3, atol=1e-16)
    np.testing.assert_array_equal(solid_c.cpu().numpy(), C.coarsen(pops, mask, 4)[-1])


@pytest.mark.parametrize("kernel", [0, 1])
def test_gpu_fused_inference_matches_oracle(lbm, torch_cuda, kernel):
    """The tile-fused network on a lattice's moments (kernel 0: tcgen05 tensor
    cores with BF16 activations; 1: CUDA cores with f32 activations) against
    the whole-image oracle network with the same BF16-rounded weights.  The
    tensor-core kernel rounds each layer's activations to BF16 (8-bit
    mantissa): its delta_tau is held to 2 % of the largest value."""
    from lbm_gb300 import closure, geometry
    nx, ny = 150, 70  # ragged tiles on both axes
    mask = geometry.single_circle(nx, ny, 40, 35, 8)
    flat = closure.init_params(11)
    flat[-1] = 0.3  # output bias
    L = lbm.load_library()
    with lbm.Lattice(nx, ny, 1.0 / 0.51, lbm.EDGE_CHANNEL, lbm.F32) as lat:
        lat.set_inlet_velocity(0.08)
        lat.init_equilibrium(1.0, 0.08, 0.0, 1e-2, 4)
        lat.draw_mask(mask)
        lat.iterate(30)
        p = flat.copy()
        lbm._check(L.lbm_closure_set_weights(lat.handle, p.ctypes.data_as(ctypes.c_void_p), p.size))
        lbm._check(L.lbm_closure_enable(lat.handle, 0.5))
        lbm._check(L.lbm_closure_set_inference(lat.handle, kernel))
        lbm._check(L.lbm_closure_infer(lat.handle))
        lat.synchronize()
        dt = np.zeros(nx * ny, np.float32)
        sp = np.zeros(nx * ny, np.float32)
        lbm._check(L.lbm_closure_read(lat.handle, dt.ctypes.data_as(ctypes.c_void_p),
                                      sp.ctypes.data_as(ctypes.c_void_p)))
        rho, jx, jy = lat.field("rho"), lat.field("jx"), lat.field("jy")
    fl = mask == 0
    r = np.where(fl, rho, 1.0).astype(np.float64)
    feat = np.stack([np.where(fl, (r - 1) * C.S_RHO, 0), np.where(fl, jx / r * C.S_U, 0),
                     np.where(fl, jy / r * C.S_U, 0), (~fl).astype(np.float64)])[None]
    ps = closure.unpack(closure.round_bf16(flat).astype(np.float64))
    z = C.forward(ps, feat)[-1][0, 0]
    want = C.delta_tau(z)
    got = dt.reshape(ny, nx)
    tol = 2e-3 if kernel == 1 else 2e-2
    err = np.abs(got - want)[fl].max() / want.max()
    print("kernel %d: max delta_tau error %.3e of %.3e" % (kernel, err, want.max()))
    assert err <= tol
    speed = np.hypot(jx, jy) / r
    assert np.abs(sp.reshape(ny, nx) - speed)[fl].max() <= 2e-3 * speed[fl].max()


@pytest.mark.parametrize("storage,sr", [(0, False), (1, False), (2, False), (1, True), (2, True)])
@pytest.mark.parametrize("kernel", [0, 1, 3, 8, 9, 11])
def test_gpu_closure_step_equals_plain_step_at_the_same_omega(lbm, torch_cuda, storage, sr, kernel):
    """All-zero weights give z = bias = 0, delta_tau = DT_MAX / 2 = 0.125
    exactly, so every fluid cell relaxes with 1 / (1 / omega + 0.125): that
    must reproduce a plain run at that omega bit for bit.  A NaN bias gives
    no valid prediction: every cell takes the plain omega and is counted.
    With stochastic rounding the closure kernels store cell by cell and the
    plain 16-bit kernels two cells per word, from the same random bits: the
    runs still agree bit for bit."""
    if storage == 0 and kernel == 8:
        kernel = 6
    from lbm_gb300 import closure, geometry
    nx, ny, steps = 300, 90, 25
    mask = geometry.random_layout(nx, ny, 0.08, 3, rmin=2.0, inlet_clearance=8)
    L = lbm.load_library()
    om0 = np.float32(1.0 / 0.52)
    om_eff = np.float32(1.0) / (np.float32(1.0) / om0 + np.float32(0.125))

    def run(omega, weights=None):
        with lbm.Lattice(nx, ny, float(omega), lbm.EDGE_CHANNEL, storage) as lat:
            lat.set_tuning(8, kernel)
            lat.set_inlet_velocity(0.07)
            lat.init_equilibrium(1.0, 0.07, 0.0, 1e-2, 2)
            lat.draw_mask(mask)
            if sr:
                lat.set_rounding(lbm.ROUND_STOCHASTIC, 31)
            fb = ctypes.c_uint64(0)
            if weights is not None:
                lbm._check(L.lbm_closure_set_weights(lat.handle, weights.ctypes.data_as(ctypes.c_void_p),
                                                     weights.size))
                lbm._check(L.lbm_closure_enable(lat.handle, 1e9))
                lbm._check(L.lbm_closure_infer(lat.handle))
            lat.iterate(steps)
            if weights is not None:
                lbm._check(L.lbm_closure_fallback_count(lat.handle, ctypes.byref(fb), 1))
            return lat.populations(), fb.value

    zero = np.zeros(closure.N_PARAMS, np.float32)
    nan = zero.copy()
    nan[-1] = np.nan
    ref_eff, _ = run(om_eff)
    ref_0, _ = run(om0)
    got, fb = run(om0, zero)
    np.testing.assert_array_equal(got, ref_eff)
    assert fb == 0
    got, fb = run(om0, nan)
    np.testing.assert_array_equal(got, ref_0)
    assert fb == int(((mask == 0)[:, 1:]).sum()) * steps
