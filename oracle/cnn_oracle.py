"""CPU oracle (test infrastructure) for the learned closure: the coarse-grained
training samples, the 3x3 convolution network, its loss and backward pass,
and the Adam update, in float64 numpy.

The reference has no learned closure (lbm-wgpu runs plain BGK only), so this
file restates the maths the engine's closure kernels implement; it is pinned
by finite differences (tests/test_cnn_oracle.py), not by reference vectors.
Only tests and the CPU baseline may use it.

Conventions shared with the CUDA kernels (lbm_gb300/csrc/lbm_cnn.cu):

* activations are [N, C, H, W]; 3x3 convolution with zero padding outside
  the image; weights [Cout, Cin, 3, 3], tap (ky, kx) reads input row
  y + ky - 1, column x + kx - 1; bias per output channel;
* network 4 -> 32 -> 32 -> 32 -> 1, ReLU after the first three layers;
* input features of a cell: (rho - 1) * S_RHO, ux * S_U, uy * S_U, solid
  (1 / 0); output z -> delta tau = DT_MAX * sigmoid(z);
* a training sample is a coarse cell of a fine run block-averaged by a
  factor F: a_i = f_i - feq_i(rho, u) of the coarse populations at t,
  b_i = f_i(x, t) - f_i(x + c_i, t + F fine steps); with
  omega = 1 / (tau0 + delta tau) the cell's loss is sum_i (omega a_i - b_i)^2
  = omega^2 A - 2 omega B + C (A = sum a^2, B = sum a b, C = sum b^2): how
  far one coarse BGK collision at that omega is from the fine run's own
  evolution.  Cells next to a solid, on the inlet column or whose
  downstream neighbour leaves the grid carry no sample (A = B = C = 0).
"""
import numpy as np

S_RHO, S_U, DT_MAX = 50.0, 10.0, 0.25
LAYERS = [(4, 32, True), (32, 32, True), (32, 32, True), (32, 1, False)]  # (cin, cout, relu)

# D2Q9 in the engine's direction order: q = 3 * (dy + 1) + (dx + 1), row-major
# offsets (dy = -1 is the previous row); weights 1/36, 1/9, 4/9.
CX = np.array([q % 3 - 1 for q in range(9)])
CY = np.array([q // 3 - 1 for q in range(9)])
W9 = np.array([1 / 36, 1 / 9, 1 / 36, 1 / 9, 4 / 9, 1 / 9, 1 / 36, 1 / 9, 1 / 36])


def _shift(x, dy, dx):
    """out[..., y, x] = x[..., y + dy, x + dx], zero outside."""
    H, W = x.shape[-2:]
    out = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if ys < ye and xs < xe:
        out[..., ys:ye, xs:xe] = x[..., ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv_forward(x, w, b, relu):
    """y[n, co] = act(b[co] + sum_ci sum_k w[co, ci, ky, kx] x[n, ci, y+ky-1, x+kx-1])."""
    N, Ci, H, W = x.shape
    Co = w.shape[0]
    y = np.broadcast_to(b[None, :, None, None], (N, Co, H, W)).astype(np.float64).copy()
    for ky in range(3):
        for kx in range(3):
            xs = _shift(x, ky - 1, kx - 1)
            y += np.einsum("oc,nchw->nohw", w[:, :, ky, kx], xs)
    return np.maximum(y, 0.0) if relu else y


def conv_backward(x, w, a, ga, relu):
    """Gradients of a layer given its input x, output a (post-activation) and
    the gradient ga w.r.t. a.  Returns (gx, gw, gb)."""
    g = ga * (a > 0) if relu else ga
    gw = np.zeros_like(w)
    gx = np.zeros_like(x)
    for ky in range(3):
        for kx in range(3):
            xs = _shift(x, ky - 1, kx - 1)
            gw[:, :, ky, kx] = np.einsum("nohw,nchw->oc", g, xs)
            gx += _shift(np.einsum("oc,nohw->nchw", w[:, :, ky, kx], g), 1 - ky, 1 - kx)
    return gx, gw, g.sum(axis=(0, 2, 3))


def init_params(seed):
    """He-uniform weights from a seeded generator, zero biases; the last layer
    scaled down so that the untrained network predicts delta tau ~ DT_MAX / 2."""
    rng = np.random.default_rng(seed)
    params = []
    for i, (ci, co, _) in enumerate(LAYERS):
        lim = np.sqrt(6.0 / (ci * 9))
        if i == len(LAYERS) - 1:
            lim *= 0.1
        params.append([rng.uniform(-lim, lim, (co, ci, 3, 3)), np.zeros(co)])
    return params


def forward(params, feat):
    acts = [feat]
    for (w, b), (_, _, relu) in zip(params, LAYERS):
        acts.append(conv_forward(acts[-1], w, b, relu))
    return acts  # acts[-1] is z [N, 1, H, W]


def backward(params, acts, gz):
    grads = [None] * len(params)
    g = gz
    for l in range(len(params) - 1, -1, -1):
        gx, gw, gb = conv_backward(acts[l], params[l][0], acts[l + 1], g, LAYERS[l][2])
        grads[l] = [gw, gb]
        g = gx
    return grads


def delta_tau(z):
    return DT_MAX / (1.0 + np.exp(-z))


def loss(z, coef, tau0, norm):
    """Sum over cells of omega^2 A - 2 omega B + C, divided by norm; and its
    gradient w.r.t. z.  coef is [N, 3, H, W]."""
    s = 1.0 / (1.0 + np.exp(-z[:, 0]))
    om = 1.0 / (tau0 + DT_MAX * s)
    A, B, C = coef[:, 0], coef[:, 1], coef[:, 2]
    L = (om * om * A - 2.0 * om * B + C).sum() / norm
    dl_dom = (2.0 * om * A - 2.0 * B) / norm
    gz = dl_dom * (-om * om) * DT_MAX * s * (1.0 - s)
    return L, gz[:, None]


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) with bias correction; updates in place."""
    m *= b1
    m += (1 - b1) * g
    v *= b2
    v += (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    p -= lr * mh / (np.sqrt(vh) + eps)


def equilibrium(rho, ux, uy):
    """BGK equilibrium in the engine's direction order; uy along the row axis
    with the sign of the engine's jy (sum of f_q * cy(q) with cy = -1 north,
    negated: north is +y)."""
    out = np.empty((9,) + np.shape(rho))
    usq = ux * ux + uy * uy
    for q in range(9):
        cu = CX[q] * ux - CY[q] * uy
        out[q] = W9[q] * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * usq)
    return out


def moments(f):
    rho = f.sum(0)
    jx = np.tensordot(CX.astype(np.float64), f, 1)
    jy = -np.tensordot(CY.astype(np.float64), f, 1)
    return rho, jx, jy


def coarsen(pops, solid, F):
    """Block-average fine populations [9, Hf, Wf] over the fluid cells of each
    F x F block; a coarse cell is solid when fewer than half its fine cells
    are fluid.  Returns (coarse pops [9, H, W], coarse solid [H, W])."""
    Hf, Wf = solid.shape
    H, W = Hf // F, Wf // F
    fl = (solid[:H * F, :W * F] == 0).astype(np.float64).reshape(H, F, W, F)
    n = fl.sum(axis=(1, 3))
    p = pops[:, :H * F, :W * F].reshape(9, H, F, W, F)
    s = (p * fl[None]).sum(axis=(2, 4))
    out = np.where(n > 0, s / np.maximum(n, 1), 0.0)
    return out, (2 * n < F * F).astype(np.uint8)


def sample(pops_t, pops_t1, solid_f, F):
    """Features [4, H, W] and loss coefficients [3, H, W] of one snapshot pair."""
    f, sc = coarsen(pops_t, solid_f, F)
    g, _ = coarsen(pops_t1, solid_f, F)
    H, W = sc.shape
    rho, jx, jy = moments(f)
    fluid = sc == 0
    rs = np.where(fluid, rho, 1.0)
    ux, uy = jx / rs, jy / rs
    feq = equilibrium(rs, ux, uy)
    a = f - feq
    b = np.empty_like(f)
    valid = fluid.copy()
    valid[:, 0] = False
    yy, xx = np.mgrid[0:H, 0:W]
    for q in range(9):
        X = xx + CX[q]
        Y = (yy + CY[q]) % H
        inside = (X >= 0) & (X < W)
        Xc = np.clip(X, 0, W - 1)
        b[q] = f[q] - g[q][Y, Xc]
        valid &= inside & (sc[Y, Xc] == 0)
    feat = np.stack([np.where(fluid, (rho - 1.0) * S_RHO, 0.0), np.where(fluid, ux * S_U, 0.0),
                     np.where(fluid, uy * S_U, 0.0), sc.astype(np.float64)])
    v = valid.astype(np.float64)
    coef = np.stack([v * (a * a).sum(0), v * (a * b).sum(0), v * (b * b).sum(0)])
    return feat, coef
