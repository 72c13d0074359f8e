"""The network oracle's gradients are the derivatives of its forward pass
(central finite differences in FP64), so the GPU kernels checked against it are
checked against the true gradients."""
import numpy as np

from oracle import nn_oracle as O


def _fd(f, x, idx, h=1e-6):
    xp = x.copy()
    xm = x.copy()
    xp[idx] += h
    xm[idx] -= h
    return (f(xp) - f(xm)) / (2 * h)


def test_conv3d_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, 4, 3, 5, 3))
    w = rng.standard_normal((27, 2, 3))
    dy = rng.standard_normal((1, 4, 3, 5, 2))
    loss_x = lambda xx: float((dy * O.conv3d(xx, w)).sum())
    loss_w = lambda ww: float((dy * O.conv3d(x, ww)).sum())
    gx = O.conv3d_data_grad(dy, w)
    gw = O.conv3d_weight_grad(x, dy)
    for idx in [(0, 0, 0, 0, 0), (0, 3, 2, 4, 2), (0, 1, 1, 2, 1), (0, 2, 0, 3, 0)]:
        assert abs(gx[idx] - _fd(loss_x, x, idx)) < 1e-7
    for idx in [(0, 0, 0), (13, 1, 2), (26, 1, 1), (5, 0, 2)]:
        assert abs(gw[idx] - _fd(loss_w, w, idx)) < 1e-7


def test_pool_upsample_and_mse_gradients():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((1, 4, 4, 2, 2))
    dyc = rng.standard_normal((1, 2, 2, 1, 2))
    dyf = rng.standard_normal((1, 8, 8, 4, 2))
    gp = O.pool2_backward(dyc)
    gu = O.up2_backward(dyf)
    for idx in [(0, 0, 0, 0, 0), (0, 3, 1, 1, 1)]:
        assert abs(gp[idx] - _fd(lambda xx: float((dyc * O.pool2(xx)).sum()), x, idx)) < 1e-8
    xc = rng.standard_normal((1, 4, 4, 2, 2))
    for idx in [(0, 0, 0, 0, 0), (0, 3, 2, 1, 1)]:
        assert abs(gu[idx] - _fd(lambda xx: float((dyf * O.up2(xx)).sum()), xc, idx)) < 1e-8
    pred = rng.standard_normal((10, 4))
    tgt = rng.standard_normal((10, 4))
    mask = (rng.random(10) > 0.4).astype(np.float64)
    _, g = O.masked_mse(pred, tgt, mask)
    for idx in [(0, 0), (3, 2), (9, 3)]:
        assert abs(g[idx] - _fd(lambda p: O.masked_mse(p, tgt, mask)[0], pred, idx)) < 1e-8


def _tiny_unet(rng, cin=2, ch=(2, 3, 3, 4), cout=2):
    c0, c1, c2, c3 = ch
    spec = {"e0a": (cin, c0), "e0b": (c0, c0), "e1a": (c0, c1), "e1b": (c1, c1), "e2a": (c1, c2),
            "e2b": (c2, c2), "ba": (c2, c3), "bb": (c3, c3), "d2a": (c3 + c2, c2), "d2b": (c2, c2),
            "d1a": (c2 + c1, c1), "d1b": (c1, c1), "d0a": (c1 + c0, c0), "d0b": (c0, c0)}
    P = {k: (rng.standard_normal((27, co, ci)) * 0.5, rng.standard_normal(co) * 0.1 + 0.3)
         for k, (ci, co) in spec.items()}
    P["head"] = (rng.standard_normal((1, cout, c0)), rng.standard_normal(cout) * 0.1)
    return P


def test_unet_gradients_match_finite_differences():
    """The oracle's U-Net backward (FP64, no rounding) against central differences
    of its forward on a tiny network (box 8, a few channels)."""
    rng = np.random.default_rng(2)
    P = _tiny_unet(rng)
    x = rng.standard_normal((1, 8, 8, 8, 2))
    dout = rng.standard_normal((1, 8, 8, 8, 2))
    out, cache = O.unet_forward(P, x, rnd=False)
    G = O.unet_backward(P, cache, dout, rnd=False)
    for name, idx in [("head", (0, 1, 0)), ("d0b", (13, 0, 1)), ("d1a", (4, 2, 5)), ("bb", (26, 3, 2)),
                      ("ba", (0, 1, 1)), ("e2b", (7, 2, 0)), ("e1a", (20, 0, 1)), ("e0a", (13, 1, 0))]:
        w, b = P[name]

        def loss(ww):
            Q = dict(P)
            Q[name] = (ww, b)
            return float((dout * O.unet_forward(Q, x, rnd=False)[0]).sum())
        fd = _fd(loss, w, idx, h=1e-5)
        assert abs(G[name][0][idx] - fd) <= 1e-6 * max(1.0, abs(fd)), (name, G[name][0][idx], fd)
    # a bias too
    w, b = P["d2a"]

    def loss_b(bb):
        Q = dict(P)
        Q["d2a"] = (w, bb)
        return float((dout * O.unet_forward(Q, x, rnd=False)[0]).sum())
    assert abs(G["d2a"][1][1] - _fd(loss_b, b, (1,), h=1e-5)) <= 1e-6 * max(1.0, abs(G["d2a"][1][1]))


def test_bf16_rounding_is_nearest_even():
    # BF16 keeps 7 fraction bits: spacing 2^-7 just above 1
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -8 + 2 ** -12, -2.5], dtype=np.float32)
    r = O.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # a tie rounds to the even mantissa (down)
    assert r[2] == 1.0 + 2 ** -6            # a tie between odd and even rounds to even (up)
    assert r[3] == 1.0 + 2 ** -7            # above the tie rounds up
    assert r[4] == -2.5
