"""CPU oracle of the warm-start surrogate's network operations (test infrastructure).

HemeLB has no learned component, so nothing here restates reference code: these
are the textbook definitions of a channels-last 3-D convolution with zero padding,
its input and weight gradients, 2x average pooling, nearest 2x upsampling and a
masked mean squared error, in FP64 numpy.  They check the BF16 tensor-core
kernels of the product (which must agree within BF16 input rounding, since both
sides see the same BF16-rounded operands and accumulate in at least FP32), and
the gradients here are pinned against finite differences of the forward pass.
Only tests import this module.
"""
from __future__ import annotations

import numpy as np


def tap_offset(tap: int, taps: int = 27):
    """(dz, dy, dx) of tap `tap` in a 3x3x3 stencil, x fastest; (0, 0, 0) for 1x1x1."""
    if taps == 1:
        return 0, 0, 0
    return tap // 9 - 1, (tap // 3) % 3 - 1, tap % 3 - 1


def shift(x, dz, dy, dx):
    """out[n, z, y, x, :] = x[n, z + dz, y + dy, x + dx, :], zero outside."""
    out = np.zeros_like(x)
    _, D, H, W, _ = x.shape
    zs, ze = max(0, -dz), min(D, D - dz)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if zs < ze and ys < ye and xs < xe:
        out[:, zs:ze, ys:ye, xs:xe] = x[:, zs + dz:ze + dz, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv3d(x, w, b=None, relu=False):
    """x (N, D, H, W, Cin), w (taps, Cout, Cin) -> (N, D, H, W, Cout)."""
    taps = w.shape[0]
    out = np.zeros(x.shape[:4] + (w.shape[1],))
    for t in range(taps):
        out += shift(x, *tap_offset(t, taps)) @ w[t].T
    if b is not None:
        out = out + b
    return np.maximum(out, 0.0) if relu else out


def conv3d_data_grad(dy, w):
    """d(sum dy * conv3d(x, w)) / dx."""
    taps = w.shape[0]
    dx = np.zeros(dy.shape[:4] + (w.shape[2],))
    for t in range(taps):
        dz, dyy, dxx = tap_offset(t, taps)
        dx += shift(dy, -dz, -dyy, -dxx) @ w[t]
    return dx


def conv3d_weight_grad(x, dy, taps=27):
    """d(sum dy * conv3d(x, w)) / dw, shape (taps, Cout, Cin)."""
    cin, cout = x.shape[-1], dy.shape[-1]
    dw = np.zeros((taps, cout, cin))
    dyf = dy.reshape(-1, cout)
    for t in range(taps):
        dw[t] = dyf.T @ shift(x, *tap_offset(t, taps)).reshape(-1, cin)
    return dw


def pool2(x):
    n, d, h, w, c = x.shape
    return x.reshape(n, d // 2, 2, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4, 6))


def pool2_backward(dy):
    return dy.repeat(2, 1).repeat(2, 2).repeat(2, 3) / 8.0


def up2(x):
    return x.repeat(2, 1).repeat(2, 2).repeat(2, 3)


def up2_backward(dy):
    n, d, h, w, c = dy.shape
    return dy.reshape(n, d // 2, 2, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4, 6))


def masked_mse(pred, target, mask):
    """Mean over masked voxels and channels of (pred - target)^2, and d/dpred."""
    c = pred.shape[-1]
    d = (pred - target) * mask[..., None]
    cnt = max(float(mask.sum()) * c, 1.0)
    return float((d * d).sum()) / cnt, 2.0 * d / cnt


def adam_step(w, g, m, v, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v
