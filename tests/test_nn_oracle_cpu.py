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
