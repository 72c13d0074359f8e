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


# ---------------------------------------------------------------------------
# the surrogate's U-Net (hemelb_gb300.surrogate.UNet), forward and backward,
# with the BF16 roundings of the GPU path at the same points when rnd=True
# ---------------------------------------------------------------------------
def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as FP64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


UNET_LAYERS = ("e0a", "e0b", "e1a", "e1b", "e2a", "e2b", "ba", "bb",
               "d2a", "d2b", "d1a", "d1b", "d0a", "d0b", "head")


def unet_forward(P, x, rnd=True):
    """P: name -> (w (taps, cout, cin), b); x (n, B, B, B, cin).  Returns (out, cache)."""
    R = bf16 if rnd else (lambda a: a)
    cache = {}

    def conv(name, a, relu=True, last=False):
        w, b = P[name]
        y = conv3d(a, w, b, relu=relu)
        cache[name] = (a, y if last else R(y))
        return y if last else R(y)

    def pool(a):
        return R(pool2(a))

    e0 = conv("e0b", conv("e0a", x))
    e1 = conv("e1b", conv("e1a", pool(e0)))
    e2 = conv("e2b", conv("e2a", pool(e1)))
    b = conv("bb", conv("ba", pool(e2)))
    d2 = conv("d2b", conv("d2a", np.concatenate([up2(b), e2], axis=-1)))
    d1 = conv("d1b", conv("d1a", np.concatenate([up2(d2), e1], axis=-1)))
    d0 = conv("d0b", conv("d0a", np.concatenate([up2(d1), e0], axis=-1)))
    out = conv("head", d0, relu=False, last=True)
    cache["shapes"] = (e0.shape, e1.shape, e2.shape, b.shape, d2.shape, d1.shape)
    return out, cache


def unet_backward(P, cache, dout, rnd=True):
    """Weight and bias gradients (name -> (dw, db)) for the output gradient dout."""
    R = bf16 if rnd else (lambda a: a)
    G = {}

    def back(name, dy, relu=True, need_dx=True):
        a, y = cache[name]
        w, _ = P[name]
        if relu:
            dy = dy * (y > 0)
        G[name] = (conv3d_weight_grad(a, dy, taps=w.shape[0]), dy.reshape(-1, dy.shape[-1]).sum(axis=0))
        return R(conv3d_data_grad(dy, w)) if need_dx else None

    s0, s1, s2, sb, sd2, sd1 = cache["shapes"]

    def split_up(g, c_up):
        return R(up2_backward(g[..., :c_up])), g[..., c_up:]

    g = back("d0a", back("d0b", back("head", dout, relu=False)))
    g, ge0 = split_up(g, sd1[-1])
    g = back("d1a", back("d1b", g))
    g, ge1 = split_up(g, sd2[-1])
    g = back("d2a", back("d2b", g))
    g, ge2 = split_up(g, sb[-1])
    g = back("ba", back("bb", g))
    ge2 = R(ge2 + R(pool2_backward(g)))
    g = back("e2a", back("e2b", ge2))
    ge1 = R(ge1 + R(pool2_backward(g)))
    g = back("e1a", back("e1b", ge1))
    ge0 = R(ge0 + R(pool2_backward(g)))
    back("e0a", back("e0b", ge0), need_dx=False)
    return G
