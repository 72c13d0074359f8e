"""The surrogate's BF16 tensor-core kernels against the CPU network oracle (FP64
numpy on the same BF16-rounded operands): forward, input and weight gradients of
the 3-D convolution, pooling, upsampling, concatenation, masked MSE and Adam."""
import numpy as np
import pytest

from oracle import nn_oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from hemelb_gb300 import nn  # noqa: E402


def bf16(a):
    t = torch.tensor(np.asarray(a, np.float32)).to(torch.bfloat16)
    return t.float().numpy().astype(np.float64), t.cuda()


def close(got, ref, rel):
    return np.abs(got - ref).max() <= rel * np.abs(ref).max() + 1e-6


@pytest.mark.parametrize("cin,cout,taps,relu,shape", [
    (16, 32, 27, False, (2, 6, 5, 7)), (32, 48, 27, True, (2, 6, 5, 7)), (16, 4, 1, False, (2, 6, 5, 7)),
    (48, 16, 27, False, (2, 6, 5, 7)), (16, 8, 27, True, (2, 6, 5, 7)), (16, 64, 27, True, (2, 6, 5, 7)),
    (32, 64, 27, False, (1, 13, 20, 24)), (48, 96, 27, True, (1, 9, 12, 17))])
def test_conv_forward(cin, cout, taps, relu, shape):
    """Shapes with partial 4x4x8 bricks at the volume edges, and volumes of many bricks."""
    rng = np.random.default_rng(cin + cout)
    x, xt = bf16(rng.standard_normal(shape + (cin,)))
    w, wt = bf16(rng.standard_normal((taps, cout, cin)) / np.sqrt(27 * cin))
    b = rng.standard_normal(cout).astype(np.float32)
    y = torch.empty(shape + (cout,), dtype=torch.bfloat16, device="cuda")
    y32 = torch.empty(shape + (cout,), dtype=torch.float32, device="cuda")
    nn.conv3d(xt, wt, torch.tensor(b, device="cuda"), y, y32, taps=taps, relu=relu, engine="mma")
    torch.cuda.synchronize()
    ref = O.conv3d(x, w, b.astype(np.float64), relu=relu)
    # FP32 accumulation of exact BF16 products: tolerance 1e-4 of the output scale
    assert close(y32.cpu().numpy(), ref, 1e-4)
    # the BF16 output is the FP32 value rounded once (relative 2^-8)
    assert np.all(np.abs(y.float().cpu().numpy() - y32.cpu().numpy()) <= 2.0 ** -8 * np.abs(y32.cpu().numpy()) + 1e-30)


@pytest.mark.parametrize("cin,cout,taps,relu,shape", [
    (16, 16, 27, False, (2, 6, 5, 7)), (16, 32, 27, True, (2, 6, 5, 7)), (32, 48, 27, False, (1, 9, 12, 17)),
    (48, 96, 27, True, (1, 13, 20, 24)), (96, 192, 27, False, (1, 8, 8, 16)), (288, 96, 27, True, (1, 8, 12, 12)),
    (16, 64, 1, False, (2, 6, 5, 7)), (192, 256, 27, False, (1, 4, 4, 8))])
def test_conv_forward_tcgen05(cin, cout, taps, relu, shape):
    """The tcgen05 / TMEM / TMA convolution against the oracle and against the
    mma.sync kernel: partial 8x4x4 bricks at every volume edge (TMA zero fill is the
    padding), 1 to 18 channel slices per tap, N = 16 to 256."""
    rng = np.random.default_rng(3 * cin + cout)
    x, xt = bf16(rng.standard_normal(shape + (cin,)))
    w, wt = bf16(rng.standard_normal((taps, cout, cin)) / np.sqrt(27 * cin))
    b = rng.standard_normal(cout).astype(np.float32)
    bt = torch.tensor(b, device="cuda")
    y = torch.empty(shape + (cout,), dtype=torch.bfloat16, device="cuda")
    y32 = torch.empty(shape + (cout,), dtype=torch.float32, device="cuda")
    nn.tc_error(reset=True)
    nn.conv3d_tc(xt, wt, bt, y, y32, taps=taps, relu=relu)
    torch.cuda.synchronize()
    assert nn.tc_error() == 0
    ref = O.conv3d(x, w, b.astype(np.float64), relu=relu)
    assert close(y32.cpu().numpy(), ref, 1e-4)
    assert np.all(np.abs(y.float().cpu().numpy() - y32.cpu().numpy()) <= 2.0 ** -8 * np.abs(y32.cpu().numpy()) + 1e-30)
    z32 = torch.empty_like(y32)
    nn.conv3d(xt, wt, bt, torch.empty_like(y), z32, taps=taps, relu=relu, engine="mma")
    torch.cuda.synchronize()
    assert close(y32.cpu().numpy(), z32.cpu().numpy(), 1e-5)


@pytest.mark.parametrize("cin,cout,shape", [(16, 32, (2, 6, 5, 4)), (32, 16, (2, 6, 5, 4)), (48, 48, (2, 6, 5, 4)),
                                             (32, 32, (2, 13, 20, 24)), (16, 48, (1, 9, 12, 17))])
@pytest.mark.parametrize("engine", ["mma", "auto"])
def test_conv_gradients(cin, cout, shape, engine):
    rng = np.random.default_rng(7 + cin)
    x, xt = bf16(rng.standard_normal(shape + (cin,)))
    w, wt = bf16(rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin))
    dy, dyt = bf16(rng.standard_normal(shape + (cout,)))
    dx = torch.empty(shape + (cin,), dtype=torch.bfloat16, device="cuda")
    dx32 = torch.empty(shape + (cin,), dtype=torch.float32, device="cuda")
    nn.conv3d_data_grad(dyt, wt, dx, dx32, engine=engine)
    dw = torch.zeros((27, cout, cin), dtype=torch.float32, device="cuda")
    nn.conv3d_weight_grad(xt, dyt, dw)
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    nn.bias_grad(dyt, db)
    torch.cuda.synchronize()
    assert close(dx32.cpu().numpy(), O.conv3d_data_grad(dy, w), 1e-4)
    assert close(dw.cpu().numpy(), O.conv3d_weight_grad(x, dy), 1e-4)
    assert close(db.cpu().numpy(), dy.reshape(-1, cout).sum(axis=0), 1e-5)


def test_weight_gradient_accumulates():
    rng = np.random.default_rng(9)
    x, xt = bf16(rng.standard_normal((1, 4, 4, 4, 16)))
    dy, dyt = bf16(rng.standard_normal((1, 4, 4, 4, 16)))
    dw = torch.zeros((1, 16, 16), dtype=torch.float32, device="cuda")
    nn.conv3d_weight_grad(xt, dyt, dw)
    nn.conv3d_weight_grad(xt, dyt, dw)
    torch.cuda.synchronize()
    assert close(dw.cpu().numpy(), 2 * O.conv3d_weight_grad(x, dy, taps=1), 1e-5)


def test_relu_backward():
    rng = np.random.default_rng(4)
    y, yt = bf16(rng.standard_normal(1000))
    g, gt = bf16(rng.standard_normal(1000))
    nn.relu_backward(gt, yt)
    assert np.array_equal(gt.float().cpu().numpy(), np.where(y > 0, g, 0.0))


def test_pool_upsample_concat_and_their_gradients():
    rng = np.random.default_rng(3)
    x, xd = bf16(rng.standard_normal((2, 4, 6, 8, 16)))
    p = torch.empty((2, 2, 3, 4, 16), dtype=torch.bfloat16, device="cuda")
    nn.pool2(xd, p)
    assert close(p.float().cpu().numpy(), O.pool2(x), 2.0 ** -8)
    pc = p.float().cpu().numpy().astype(np.float64)
    u = torch.empty_like(xd)
    nn.up2(p, u)
    assert np.array_equal(u.float().cpu().numpy(), O.up2(pc))
    g = torch.empty_like(xd)
    nn.pool2_backward(p, g)
    assert np.array_equal(g.float().cpu().numpy(), O.pool2_backward(pc))  # division by 8 is exact
    s = torch.empty_like(p)
    nn.up2_backward(xd, s)
    assert close(s.float().cpu().numpy(), O.up2_backward(x), 2.0 ** -7)
    a = torch.randn((2, 4, 6, 8, 16), device="cuda").to(torch.bfloat16)
    cat = torch.empty((2, 4, 6, 8, 32), dtype=torch.bfloat16, device="cuda")
    nn.concat(a, xd, cat)
    assert torch.equal(cat[..., :16], a) and torch.equal(cat[..., 16:], xd)
    da = torch.empty_like(a)
    db = torch.empty_like(xd)
    nn.split(cat, da, db)
    assert torch.equal(da, a) and torch.equal(db, xd)


def test_masked_mse_and_adam():
    rng = np.random.default_rng(5)
    pred = rng.standard_normal((100, 4))
    tgt = rng.standard_normal((100, 4))
    mask = (rng.random(100) > 0.3).astype(np.float64)
    tp = torch.tensor(pred, dtype=torch.float32, device="cuda")
    tt = torch.tensor(tgt, dtype=torch.float32, device="cuda")
    tm = torch.tensor(mask, dtype=torch.float32, device="cuda")
    dpred = torch.empty((100, 4), dtype=torch.bfloat16, device="cuda")
    loss = nn.mse(tp, tt, tm, dpred)
    ref_loss, ref_g = O.masked_mse(tp.double().cpu().numpy(), tt.double().cpu().numpy(), mask)
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss
    assert close(dpred.float().cpu().numpy(), ref_g, 2.0 ** -8)
    w = rng.standard_normal(50)
    g = rng.standard_normal(50)
    tw = torch.tensor(w, dtype=torch.float32, device="cuda")
    wb = torch.empty(50, dtype=torch.bfloat16, device="cuda")
    tg = torch.tensor(g, dtype=torch.float32, device="cuda")
    m = torch.zeros_like(tw)
    v = torch.zeros_like(tw)
    mr, vr, wr = np.zeros(50), np.zeros(50), tw.double().cpu().numpy()
    for step in (1, 2, 3):
        nn.adam(tw, wb, tg, m, v, lr=1e-2, step=step)
        wr, mr, vr = O.adam_step(wr, tg.double().cpu().numpy(), mr, vr, 1e-2, step)
    torch.cuda.synchronize()
    assert np.allclose(tw.double().cpu().numpy(), wr, rtol=1e-6, atol=1e-6)
    assert torch.equal(wb, tw.to(torch.bfloat16))


def test_unet_forward_and_gradients_match_oracle():
    """The whole U-Net (BF16 kernels, FP32 accumulation) against the oracle's U-Net.
    Forward: every layer's BF16 output against the oracle convolution of the same
    layer input, within one BF16 rounding.  Backward: the oracle's backward pass on
    the GPU's own activations (so both see the same ReLU masks; a mask flip near
    zero would change a gradient by O(1) and is a property of BF16, not of the
    kernels), against every weight and bias gradient."""
    from hemelb_gb300.surrogate import N_IN, UNet
    net = UNet(ch=(16, 16, 32, 16), seed=1)
    rng = np.random.default_rng(0)
    x, xt = bf16(rng.standard_normal((1, 16, 16, 16, N_IN)))
    out = net.forward(xt)
    torch.cuda.synchronize()
    acts = {k: (c.x.float().cpu().numpy().astype(np.float64), c.y.float().cpu().numpy().astype(np.float64))
            for k, c in net.L.items()}
    P = {k: (c.wb.float().cpu().numpy().astype(np.float64), c.b.cpu().numpy().astype(np.float64))
         for k, c in net.L.items()}
    for k, (a, y) in acts.items():
        w, b = P[k]
        ref = O.conv3d(a, w, b, relu=net.L[k].relu)
        assert np.all(np.abs(y - ref) <= 2.0 ** -8 * np.abs(ref) + 1e-6 * np.abs(ref).max()), k
    assert close(out.cpu().numpy(), O.conv3d(*acts["head"][:1], *P["head"]), 1e-5)
    dout, doutt = bf16(rng.standard_normal(tuple(out.shape)))
    net.zero_grad()
    net.backward(doutt)
    torch.cuda.synchronize()
    cache = dict(acts)
    cache["shapes"] = tuple(acts[k][1].shape for k in ("e0b", "e1b", "e2b", "bb", "d2b", "d1b"))
    G = O.unet_backward(P, cache, dout)
    for k, c in net.L.items():
        assert close(c.gw.cpu().numpy(), G[k][0], 1e-2), k
        assert close(c.gb.cpu().numpy(), G[k][1], 1e-2), k
