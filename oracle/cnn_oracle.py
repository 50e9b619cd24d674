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
  factor F (Favre averages over the block's fluid cells): the subgrid stress
  tau_ij = <rho u_i u_j> / <rho> - U_i U_j of the fine velocity around the
  coarse velocity U, against the coarse strain rate S_ij of U (central
  differences, per coarse cell).  An eddy viscosity nu_t = delta_tau / 3 (the
  BGK viscosity (tau - 1/2) / 3) models the deviatoric stress as
  -2 nu_t S^d; the cell's loss is the squared Frobenius residual
  |tau^d + (2/3) delta_tau S^d|^2 = A dt^2 - 2 B dt + C with
  A = (4/9)|S^d|^2, B = -(2/3) <tau^d, S^d>, C = |tau^d|^2.  Cells that are
  solid, on the first or last column or next to a solid carry no sample
  (A = B = C = 0).
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


def loss(z, coef, norm):
    """Sum over cells of A dt^2 - 2 B dt + C (dt = delta_tau(z)), divided by
    norm; and its gradient w.r.t. z.  coef is [N, 3, H, W]."""
    s = 1.0 / (1.0 + np.exp(-z[:, 0]))
    dt = DT_MAX * s
    A, B, C = coef[:, 0], coef[:, 1], coef[:, 2]
    L = (dt * dt * A - 2.0 * dt * B + C).sum() / norm
    gz = (2.0 * (dt * A - B) / norm) * DT_MAX * s * (1.0 - s)
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
    """Favre block averages of a fine state [9, Hf, Wf] over the fluid cells
    of each F x F block: (rho, Ux, Uy, tau_xx, tau_xy, tau_yy, coarse solid),
    a block being solid when fewer than half its cells are fluid."""
    Hf, Wf = solid.shape
    H, W = Hf // F, Wf // F
    rho, jx, jy = moments(pops[:, :H * F, :W * F])
    fl = (solid[:H * F, :W * F] == 0).astype(np.float64)
    r = np.where(fl > 0, rho, 1.0)
    ux, uy = jx / r, jy / r

    def bsum(a):
        return (a * fl).reshape(H, F, W, F).sum(axis=(1, 3))

    n = bsum(np.ones_like(rho))
    R = bsum(rho)
    Rs = np.where(n > 0, R, 1.0)
    Ux, Uy = bsum(jx) / Rs, bsum(jy) / Rs
    txx = bsum(rho * ux * ux) / Rs - Ux * Ux
    txy = bsum(rho * ux * uy) / Rs - Ux * Uy
    tyy = bsum(rho * uy * uy) / Rs - Uy * Uy
    return R / np.maximum(n, 1), Ux, Uy, txx, txy, tyy, (2 * n < F * F).astype(np.uint8)


def sample(pops, solid_f, F):
    """Features [4, H, W] and loss coefficients [3, H, W] of one fine snapshot."""
    rho, Ux, Uy, txx, txy, tyy, sc = coarsen(pops, solid_f, F)
    H, W = sc.shape
    fluid = sc == 0
    up = np.roll(np.arange(H), 1)   # row - 1 (north), periodic
    dn = np.roll(np.arange(H), -1)  # row + 1 (south)
    xl = np.clip(np.arange(W) - 1, 0, W - 1)
    xr = np.clip(np.arange(W) + 1, 0, W - 1)
    dUx_dx = (Ux[:, xr] - Ux[:, xl]) / 2
    dUy_dx = (Uy[:, xr] - Uy[:, xl]) / 2
    dUx_dy = (Ux[up] - Ux[dn]) / 2  # y points north: rows count southwards
    dUy_dy = (Uy[up] - Uy[dn]) / 2
    sxx = (dUx_dx - dUy_dy) / 2  # deviatoric parts
    sxy = (dUx_dy + dUy_dx) / 2
    dxx = (txx - tyy) / 2
    valid = fluid & fluid[:, xl] & fluid[:, xr] & fluid[up] & fluid[dn]
    valid[:, 0] = False
    valid[:, -1] = False
    v = valid.astype(np.float64)
    A = v * (4.0 / 9.0) * 2 * (sxx * sxx + sxy * sxy)
    B = v * -(2.0 / 3.0) * 2 * (dxx * sxx + txy * sxy)
    C = v * 2 * (dxx * dxx + txy * txy)
    feat = np.stack([np.where(fluid, (rho - 1.0) * S_RHO, 0.0), np.where(fluid, Ux * S_U, 0.0),
                     np.where(fluid, Uy * S_U, 0.0), sc.astype(np.float64)])
    return feat, np.stack([A, B, C])
