"""FP64 numpy oracle of the preconditioner network (test infrastructure only).

The network is the 4-layer 3x3 convolutional net that the learned preconditioner applies on the
nodal grid (NHWC layout, zero padding, dilation per layer): forward, losses (masked mean-squared
error; energy norm with the crop's assembled stiffness) and backward (input and weight
gradients) written out with explicit shifts, used to check the GPU training kernels.
"""

import numpy as np

TAPS = [(dy, dx) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]  # tap t = (dy+1)*3 + (dx+1)


def shift(x, dy, dx):
    """out[:, y, x, :] = x[:, y+dy, x+dx, :] with zeros outside."""
    B, H, W, C = x.shape
    out = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if ys < ye and xs < xe:
        out[:, ys:ye, xs:xe, :] = x[:, ys + dy:ye + dy, xs + dx:xe + dx, :]
    return out


def conv(x, W, b, dil):
    """y[p, co] = b[co] + sum_t sum_ci x[p + dil*off_t, ci] W[t, ci, co]."""
    y = np.zeros(x.shape[:3] + (W.shape[2],))
    for t, (dy, dx) in enumerate(TAPS):
        y += np.einsum("bhwc,cd->bhwd", shift(x, dil * dy, dil * dx), W[t])
    return y + b


def conv_bwd(x, W, dil, dy_):
    """Gradients of sum(dy_ * conv(x, W, b, dil)) w.r.t. x, W and b."""
    dx = np.zeros_like(x)
    dW = np.zeros_like(W)
    for t, (sy, sx) in enumerate(TAPS):
        xs = shift(x, dil * sy, dil * sx)
        dW[t] = np.einsum("bhwc,bhwd->cd", xs, dy_)
        dx += shift(np.einsum("bhwd,cd->bhwc", dy_, W[t]), -dil * sy, -dil * sx)
    db = dy_.sum(axis=(0, 1, 2))
    return dx, dW, db


def forward(x, params, dils):
    """params: list of (W [9,cin,cout], b [cout]); ReLU after every layer but the last.
    Returns the output and the activations (inputs of each layer)."""
    acts = [x]
    h = x
    for k, ((W, b), d) in enumerate(zip(params, dils)):
        h = conv(h, W, b, d)
        if k + 1 < len(params):
            h = np.maximum(h, 0.0)
        acts.append(h)
    return h, acts


def backward(acts, params, dils, g):
    """Gradients w.r.t. every W and b for the output gradient g."""
    grads = [None] * len(params)
    for k in reversed(range(len(params))):
        W, b = params[k]
        dx, dW, db = conv_bwd(acts[k], W, dils[k], g)
        grads[k] = (dW, db)
        if k > 0:
            g = dx * (acts[k] > 0.0)
    return grads


def loss_and_grads(x, target, mask, params, dils):
    """Masked mean-squared error and its gradients w.r.t. every W and b."""
    y, acts = forward(x, params, dils)
    n = mask.sum() * y.shape[-1]
    diff = (y - target) * mask[..., None]
    loss = float((diff ** 2).sum() / n)
    g = 2.0 * diff / n
    return loss, backward(acts, params, dils, g)


def crop_stiffness(E):
    """Assembled stiffness of one S x S node crop (scipy CSR, dof = node * 2 + component, node =
    y * S + x) of unit square Quad4 elements with moduli E [S-1, S-1, 2] (K, G), through the
    oracle's element integrals (oracle.statics.stiffness)."""
    from . import gfref as R
    from . import statics as ST

    S = E.shape[0] + 1
    coor, conn = R.quad4_regular(S - 1, S - 1)
    return ST.stiffness(coor, conn, E[..., 0].ravel().astype(np.float64),
                        E[..., 1].ravel().astype(np.float64))


def energy_loss_and_grads(x, target, E, F, margin, params, dils):
    """Energy-norm loss sum_b e_b^T A_b e_b / sum_b t_b^T A_b t_b (e = M F (y - T), t = M F T,
    M the crop interior [margin, S - margin)^2, A_b the crop stiffness) and its gradients."""
    y, acts = forward(x, params, dils)
    B, S = y.shape[0], y.shape[1]
    M = np.zeros((S, S, 1))
    M[margin:S - margin, margin:S - margin] = 1.0
    num, den = 0.0, 0.0
    Ae_all = np.zeros_like(y)
    for b in range(B):
        A = crop_stiffness(E[b])
        w = (M * F[b]).ravel()
        e = w * (y[b] - target[b]).ravel()
        t = w * target[b].ravel()
        Ae = A @ e
        num += float(e @ Ae)
        den += float(t @ (A @ t))
        Ae_all[b] = (w * Ae).reshape(S, S, 2)
    return num / den, backward(acts, params, dils, 2.0 * Ae_all / den)
