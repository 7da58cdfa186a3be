"""FP64 CPU oracle for the U-Net denoiser's operators (TEST INFRASTRUCTURE ONLY).

RenderToy has no learned part (its demos call Intel OIDN, a closed binary),
so there is no reference to pin against: these are the textbook definitions,
written for clarity in float64 numpy, used to check the GPU kernels' forward
values and gradients on small shapes.  Layout NHWC; a 3x3 convolution weight
is [Cout, 3, 3, Cin]; "same" zero padding, stride 1.
"""
from __future__ import annotations

import numpy as np


def conv3x3(x, w, b=None):
    """y[n,y,x,o] = b[o] + sum_{i,j,c} x[n, y+i-1, x+j-1, c] * w[o,i,j,c]."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    n, h, wd, c = x.shape
    xp = np.zeros((n, h + 2, wd + 2, c))
    xp[:, 1:-1, 1:-1] = x
    y = np.zeros((n, h, wd, w.shape[0]))
    for i in range(3):
        for j in range(3):
            y += np.einsum("nhwc,oc->nhwo", xp[:, i:i + h, j:j + wd], w[:, i, j, :])
    if b is not None:
        y += np.asarray(b, np.float64)
    return y


def conv3x3_dgrad(dy, w):
    """d x = conv of dy with the spatially flipped, channel-transposed weight."""
    dy = np.asarray(dy, np.float64)
    w = np.asarray(w, np.float64)
    n, h, wd, o = dy.shape
    dyp = np.zeros((n, h + 2, wd + 2, o))
    dyp[:, 1:-1, 1:-1] = dy
    dx = np.zeros((n, h, wd, w.shape[3]))
    for i in range(3):
        for j in range(3):
            # x[y+i-1] contributed to dy[y] with w[i]; so dx[y] gets dy[y-i+1] w[i]
            dx += np.einsum("nhwo,oc->nhwc", dyp[:, 2 - i:2 - i + h, 2 - j:2 - j + wd], w[:, i, j, :])
    return dx


def conv3x3_wgrad(x, dy):
    """dw[o,i,j,c] = sum_{n,y,x} dy[n,y,x,o] x[n, y+i-1, x+j-1, c]; db = sum dy."""
    x = np.asarray(x, np.float64)
    dy = np.asarray(dy, np.float64)
    n, h, wd, c = x.shape
    xp = np.zeros((n, h + 2, wd + 2, c))
    xp[:, 1:-1, 1:-1] = x
    dw = np.zeros((dy.shape[3], 3, 3, c))
    for i in range(3):
        for j in range(3):
            dw[:, i, j, :] = np.einsum("nhwo,nhwc->oc", dy, xp[:, i:i + h, j:j + wd])
    return dw, dy.sum(axis=(0, 1, 2))


def relu(x):
    return np.maximum(x, 0.0)


def relu_grad(x, dy):
    return np.where(x > 0.0, dy, 0.0)


def avgpool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def avgpool2_grad(dy):
    return np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2) * 0.25


def upsample2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample2_grad(dy):
    n, h, w, c = dy.shape
    return dy.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def l1_log_loss(pred, target):
    """mean |pred - log(1 + target)|; pred is in log space."""
    t = np.log1p(np.maximum(np.asarray(target, np.float64), 0.0))
    d = np.asarray(pred, np.float64) - t
    return np.abs(d).mean(), np.sign(d) / d.size


def adam(p, g, m, v, step, lr=3e-4, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
