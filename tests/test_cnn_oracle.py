"""The closure's CPU oracle pinned by finite differences, plus host-side
helpers of lbm_gb300.closure (no GPU)."""
import numpy as np
import pytest

from oracle import cnn_oracle as C


def small_net(seed):
    rng = np.random.default_rng(seed)
    layers = [(3, 5, True), (5, 4, True), (4, 1, False)]
    params = [[rng.normal(0, 0.4, (co, ci, 3, 3)), rng.normal(0, 0.1, co)] for ci, co, _ in layers]
    return layers, params


def run(layers, params, x):
    acts = [x]
    for (w, b), (_, _, relu) in zip(params, layers):
        acts.append(C.conv_forward(acts[-1], w, b, relu))
    return acts


def test_conv_forward_matches_direct_sum():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(2, 3, 5, 6))
    w = rng.normal(size=(4, 3, 3, 3))
    b = rng.normal(size=4)
    y = C.conv_forward(x, w, b, False)
    n, co, yy, xx = 1, 2, 0, 5
    s = b[co]
    for ci in range(3):
        for ky in range(3):
            for kx in range(3):
                r, c = yy + ky - 1, xx + kx - 1
                if 0 <= r < 5 and 0 <= c < 6:
                    s += w[co, ci, ky, kx] * x[n, ci, r, c]
    assert y[n, co, yy, xx] == pytest.approx(s, rel=1e-12)


def test_backward_matches_finite_differences():
    layers, params = small_net(2)
    rng = np.random.default_rng(3)
    x = rng.normal(size=(2, 3, 6, 7))
    r = rng.normal(size=(2, 1, 6, 7))

    def loss_of(ps, xx):
        return 0.5 * ((run(layers, ps, xx)[-1] - r) ** 2).sum()

    acts = run(layers, params, x)
    g = acts[-1] - r
    grads = [None] * 3
    for l in range(2, -1, -1):
        gx, gw, gb = C.conv_backward(acts[l], params[l][0], acts[l + 1], g, layers[l][2])
        grads[l] = (gw, gb)
        g = gx
    eps = 1e-6
    for l, idx in [(0, (1, 2, 0, 1)), (1, (3, 4, 2, 2)), (2, (0, 1, 1, 0))]:
        p2 = [[w.copy(), b.copy()] for w, b in params]
        p2[l][0][idx] += eps
        lp = loss_of(p2, x)
        p2[l][0][idx] -= 2 * eps
        lm = loss_of(p2, x)
        assert grads[l][0][idx] == pytest.approx((lp - lm) / (2 * eps), rel=1e-5, abs=1e-8)
        p2 = [[w.copy(), b.copy()] for w, b in params]
        p2[l][1][0] += eps
        lp = loss_of(p2, x)
        p2[l][1][0] -= 2 * eps
        assert grads[l][1][0] == pytest.approx((lp - loss_of(p2, x)) / (2 * eps), rel=1e-5, abs=1e-8)
    xi = (1, 2, 3, 4)
    x2 = x.copy()
    x2[xi] += eps
    lp = loss_of(params, x2)
    x2[xi] -= 2 * eps
    assert g[xi] == pytest.approx((lp - loss_of(params, x2)) / (2 * eps), rel=1e-5, abs=1e-8)


def test_closure_loss_gradient_and_minimum():
    """Stresses generated by an eddy viscosity dt / 3 plus noise: the loss is the
    squared residual, its gradient matches finite differences, and its
    minimum over delta tau is the generating value."""
    rng = np.random.default_rng(4)
    z = rng.normal(size=(2, 1, 4, 5))
    sxx, sxy = rng.normal(size=(2, 2, 4, 5)) * 1e-2
    dt_true = 0.05
    dxx = -(2 / 3) * dt_true * sxx + 1e-6 * rng.normal(size=sxx.shape)
    txy = -(2 / 3) * dt_true * sxy + 1e-6 * rng.normal(size=sxy.shape)
    coef = np.stack([(8 / 9) * (sxx ** 2 + sxy ** 2), -(4 / 3) * (dxx * sxx + txy * sxy),
                     2 * (dxx ** 2 + txy ** 2)], axis=1)
    L, gz = C.loss(z, coef, 7.0)
    dt = C.delta_tau(z[:, 0])
    direct = 2 * (((dxx + (2 / 3) * dt * sxx) ** 2) + ((txy + (2 / 3) * dt * sxy) ** 2)).sum() / 7.0
    assert L == pytest.approx(direct, rel=1e-9)
    eps = 1e-6
    i = (1, 0, 2, 3)
    z2 = z.copy()
    z2[i] += eps
    lp = C.loss(z2, coef, 7.0)[0]
    z2[i] -= 2 * eps
    assert gz[i] == pytest.approx((lp - C.loss(z2, coef, 7.0)[0]) / (2 * eps), rel=1e-6)
    zs = np.linspace(-6, 3, 9001)
    one = coef[:1, :, :1, :1]
    losses = [C.loss(np.full((1, 1, 1, 1), v), one, 1.0)[0] for v in zs]
    assert C.delta_tau(zs[int(np.argmin(losses))]) == pytest.approx(dt_true, abs=1e-3)


def test_sample_of_a_uniform_flow_and_of_a_shear_flow():
    H, W, F = 8, 12, 4
    rng = np.random.default_rng(5)
    rho = 1 + 0.01 * rng.random((H * F, W * F))
    solid = np.zeros((H * F, W * F), np.uint8)
    solid[8:16, 20:28] = 1  # coarse blocks (2..3, 5..6)
    solid[17, 3] = 1  # one cell of sixteen: the block stays fluid
    # uniform flow: no strain, no subgrid stress
    f = C.equilibrium(rho, 0.05 + 0 * rho, 0 * rho)
    feat, coef = C.sample(f, solid, F)
    sc = C.coarsen(f, solid, F)[-1]
    assert sc[2:4, 5:7].all() and sc.sum() == 4
    assert np.abs(coef).max() < 1e-14
    assert feat[1][sc == 0] == pytest.approx(0.05 * C.S_U, rel=1e-12)
    assert (coef[:, :, 0] == 0).all() and (coef[:, :, -1] == 0).all()
    # linear shear ux = g * row: Favre averages of a linear profile carry a
    # subgrid variance g^2 (F^2 - 1) / 12 in xx only, the strain is (g F) / 2 in xy
    g = 1e-3
    rows = np.arange(H * F)[:, None] + 0 * rho
    f = C.equilibrium(1.0 + 0 * rho, g * rows, 0 * rho)
    _, Ux, _, txx, txy, tyy, _ = C.coarsen(f, np.zeros_like(solid), F)
    assert txx == pytest.approx(g * g * (F * F - 1) / 12, rel=1e-9)
    assert np.abs(txy).max() < 1e-15 and np.abs(tyy).max() < 1e-15
    feat, coef = C.sample(f, np.zeros_like(solid), F)
    inner = coef[:, 2:-2, 2:-2]
    sxy = -g * F / 2  # dUx/dy with y pointing north (rows southwards)
    assert inner[0] == pytest.approx((8 / 9) * sxy * sxy, rel=1e-9)
    assert inner[1] == pytest.approx(0.0, abs=1e-18)  # a normal stress against a shear: no projection


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    from lbm_gb300 import closure
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.normal(size=1000).astype(np.float32),
                        np.array([1.0, 1.00390625, 1.01171875, -2.5, 0.0, 3.0e-3], np.float32)])
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(closure.round_bf16(x), ref)


def test_pack_unpack_and_param_count():
    from lbm_gb300 import closure
    flat = closure.init_params(3)
    assert flat.size == closure.N_PARAMS == 19969
    ps = closure.unpack(flat)
    assert [w.shape for w, _ in ps] == [(32, 4, 3, 3), (32, 32, 3, 3), (32, 32, 3, 3), (1, 32, 3, 3)]
    np.testing.assert_array_equal(closure.pack(ps), flat)
    assert closure.coarse_tau(0.52, 4) == pytest.approx(0.505)
