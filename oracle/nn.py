"""FP64 numpy oracle of the preconditioner network (test infrastructure only).

The network is the 4-layer 3x3 convolutional net that the learned preconditioner applies on the
nodal grid (NHWC layout, zero padding, dilation per layer): forward, loss and backward (input and
weight gradients) written out with explicit shifts, used to check the GPU training kernels.
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


def loss_and_grads(x, target, mask, params, dils):
    """Masked mean-squared error and its gradients w.r.t. every W and b."""
    y, acts = forward(x, params, dils)
    n = mask.sum() * y.shape[-1]
    diff = (y - target) * mask[..., None]
    loss = float((diff ** 2).sum() / n)
    g = 2.0 * diff / n
    grads = [None] * len(params)
    for k in reversed(range(len(params))):
        W, b = params[k]
        dx, dW, db = conv_bwd(acts[k], W, dils[k], g)
        grads[k] = (dW, db)
        if k > 0:
            g = dx * (acts[k] > 0.0)
    return loss, grads
