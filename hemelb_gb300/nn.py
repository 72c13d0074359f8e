"""Python side of the surrogate's kernels (include/hemelb_gb300_nn.h).

Each function takes torch CUDA tensors as plain device memory (channels-last
BF16 activations, [taps][C_out][C_in] BF16 weights, FP32 gradients and master
weights), checks shapes and dtypes, and enqueues the library's kernel on torch's
current stream.  There is no fallback: the kernels are the implementation.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import capi

_BF16 = torch.bfloat16
_F32 = torch.float32


def _lib():
    return capi.load()


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _need(t, dtype, what):
    if t.dtype != dtype or not t.is_cuda or not t.is_contiguous():
        raise ValueError(f"{what}: need a contiguous CUDA {dtype} tensor, got {t.dtype} "
                         f"{'cuda' if t.is_cuda else 'cpu'} contiguous={t.is_contiguous()}")


def _ok(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


def tc_eligible(cin: int, cout: int, *tensors) -> bool:
    """Shapes the tcgen05 convolution takes: C_in a multiple of 16, C_out a multiple
    of 16 up to 256, 16-byte aligned buffers."""
    return (cin % 16 == 0 and cout % 16 == 0 and 16 <= cout <= 256
            and all(t is None or t.data_ptr() % 16 == 0 for t in tensors))


def tc_tiles(n: int, d: int, h: int, w: int) -> int:
    """CTAs of the tcgen05 convolution: one per 8 x 16 x 2 output tile."""
    return n * -(-d // 2) * -(-h // 16) * -(-w // 8)


# Below one tile per SM the mma.sync kernel is faster (measured on the 12^3 layers).
_TC_MIN_TILES = 152


def conv3d(x, w, bias, out, out_f32=None, taps=27, relu=False, engine="auto"):
    """out[n,z,y,x,co] = act(sum_{tap,ci} x[n,(z,y,x)+off(tap),ci] w[tap,co,ci] + bias[co]).

    engine "tc": the tcgen05 / TMEM / TMA kernel (hlbg_nn_conv3d_tc); "mma": the
    mma.sync kernel (hlbg_nn_conv3d, every shape); "auto": tcgen05 where it takes
    the shape, else mma.sync."""
    _need(x, _BF16, "conv3d input")
    _need(w, _BF16, "conv3d weights")
    _need(out, _BF16, "conv3d output")
    n, d, h, wd, cin = x.shape
    t, cout, cin_w = w.shape
    if t != taps or cin_w != cin or out.shape != (n, d, h, wd, cout):
        raise ValueError(f"conv3d shapes: x {tuple(x.shape)} w {tuple(w.shape)} out {tuple(out.shape)}")
    if bias is not None:
        _need(bias, _F32, "conv3d bias")
    if out_f32 is not None:
        _need(out_f32, _F32, "conv3d FP32 output")
    if engine == "auto":
        engine = ("tc" if tc_eligible(cin, cout, x, w, out, out_f32) and tc_tiles(n, d, h, wd) >= _TC_MIN_TILES
                  else "mma")
    fn = _lib().hlbg_nn_conv3d_tc if engine == "tc" else _lib().hlbg_nn_conv3d
    _ok(fn(_p(x), cin, _p(w), _p(bias), _p(out), _p(out_f32), cout, n, d, h, wd, taps, int(relu), _stream()),
        "hlbg_nn_conv3d_tc" if engine == "tc" else "hlbg_nn_conv3d")


def conv3d_tc(x, w, bias, out, out_f32=None, taps=27, relu=False):
    """conv3d on the tcgen05 tensor cores (cin and cout multiples of 16, cout <= 256)."""
    conv3d(x, w, bias, out, out_f32, taps, relu, engine="tc")


def tc_error(reset: bool = True) -> int:
    """Nonzero when a bounded wait of a tcgen05 convolution gave up."""
    return int(_lib().hlbg_nn_tc_error(int(reset)))


def flip_transpose(w, wt):
    _need(w, _BF16, "weights")
    _need(wt, _BF16, "flipped weights")
    taps, cout, cin = w.shape
    if wt.shape != (taps, cin, cout):
        raise ValueError("flip_transpose shapes")
    _ok(_lib().hlbg_nn_flip_transpose(_p(w), _p(wt), cout, cin, taps, _stream()), "hlbg_nn_flip_transpose")


def conv3d_data_grad(dy, w, dx, dx_f32=None, wt=None, engine="auto"):
    """dx = conv(dy, flipped transposed w): the input gradient of conv3d."""
    taps, cout, cin = w.shape
    if wt is None:
        wt = torch.empty((taps, cin, cout), dtype=_BF16, device=w.device)
    flip_transpose(w, wt)
    conv3d(dy, wt, None, dx, dx_f32, taps=taps, relu=False, engine=engine)


def conv3d_weight_grad(x, dy, dw):
    """dw[tap,co,ci] += sum over voxels of dy[m,co] x[m+off(tap),ci] (FP32 accumulate)."""
    _need(x, _BF16, "wgrad input")
    _need(dy, _BF16, "wgrad output gradient")
    _need(dw, _F32, "wgrad weight gradient")
    n, d, h, wd, cin = x.shape
    taps, cout, cin_w = dw.shape
    if cin_w != cin or dy.shape != (n, d, h, wd, cout):
        raise ValueError("conv3d_weight_grad shapes")
    _ok(_lib().hlbg_nn_conv3d_wgrad(_p(x), cin, _p(dy), cout, _p(dw), n, d, h, wd, taps, _stream()),
        "hlbg_nn_conv3d_wgrad")


def relu_backward(dy, y):
    _need(dy, _BF16, "relu dy")
    _need(y, _BF16, "relu y")
    _ok(_lib().hlbg_nn_relu_bwd(_p(dy), _p(y), dy.numel(), _stream()), "hlbg_nn_relu_bwd")


def bias_grad(dy, db):
    _need(dy, _BF16, "bias dy")
    _need(db, _F32, "bias gradient")
    c = dy.shape[-1]
    _ok(_lib().hlbg_nn_bias_grad(_p(dy), _p(db), dy.numel() // c, c, _stream()), "hlbg_nn_bias_grad")


def pool2(x, y):
    _need(x, _BF16, "pool input")
    _need(y, _BF16, "pool output")
    n, d, h, w, c = x.shape
    _ok(_lib().hlbg_nn_pool2(_p(x), _p(y), n, d, h, w, c, 0, _stream()), "hlbg_nn_pool2")


def pool2_backward(dy, dx):
    n, d, h, w, c = dx.shape
    _need(dy, _BF16, "pool dy")
    _need(dx, _BF16, "pool dx")
    _ok(_lib().hlbg_nn_pool2(_p(dy), _p(dx), n, d, h, w, c, 1, _stream()), "hlbg_nn_pool2")


def up2(x, y):
    _need(x, _BF16, "upsample input")
    _need(y, _BF16, "upsample output")
    n, d, h, w, c = y.shape
    _ok(_lib().hlbg_nn_up2(_p(x), _p(y), n, d, h, w, c, 0, _stream()), "hlbg_nn_up2")


def up2_backward(dy, dx):
    n, d, h, w, c = dx.shape
    _need(dy, _BF16, "upsample dy")
    _need(dx, _BF16, "upsample dx")
    _ok(_lib().hlbg_nn_up2(_p(dy), _p(dx), n, d, h, w, c, 1, _stream()), "hlbg_nn_up2")


def concat(a, b, y):
    ca, cb = a.shape[-1], b.shape[-1]
    m = a.numel() // ca
    for t, w in ((a, "concat a"), (b, "concat b"), (y, "concat y")):
        _need(t, _BF16, w)
    _ok(_lib().hlbg_nn_concat(_p(a), ca, _p(b), cb, _p(y), m, _stream()), "hlbg_nn_concat")


def split(y, da, db, accumulate_b=False):
    ca, cb = da.shape[-1], db.shape[-1]
    m = da.numel() // ca
    for t, w in ((y, "split y"), (da, "split da"), (db, "split db")):
        _need(t, _BF16, w)
    _ok(_lib().hlbg_nn_split(_p(y), _p(da), ca, _p(db), cb, m, int(accumulate_b), _stream()),
        "hlbg_nn_split")


def add_(a, b):
    _need(a, _BF16, "add a")
    _need(b, _BF16, "add b")
    _ok(_lib().hlbg_nn_add(_p(a), _p(b), a.numel(), _stream()), "hlbg_nn_add")


def mse(pred, target, mask, dpred, loss=None):
    """Masked mean squared error over voxels with mask 1; writes dpred and returns the
    loss (a host float when `loss` is None, else accumulated into the FP32 device scalar)."""
    _need(pred, _F32, "mse pred")
    _need(target, _F32, "mse target")
    _need(mask, _F32, "mse mask")
    _need(dpred, _BF16, "mse dpred")
    c = pred.shape[-1]
    m = pred.numel() // c
    cnt = float(mask.sum()) * c
    own = loss is None
    if own:
        loss = torch.zeros(1, dtype=_F32, device=pred.device)
    _ok(_lib().hlbg_nn_mse(_p(pred), _p(target), _p(mask), _p(dpred), _p(loss), m, c,
                           1.0 / max(cnt, 1.0), _stream()), "hlbg_nn_mse")
    return float(loss) / max(cnt, 1.0) if own else None


def adam(w, wb, g, m, v, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    for t, n in ((w, "adam w"), (g, "adam g"), (m, "adam m"), (v, "adam v")):
        _need(t, _F32, n)
    if wb is not None:
        _need(wb, _BF16, "adam bf16 copy")
    _ok(_lib().hlbg_nn_adam(_p(w), _p(wb), _p(g), _p(m), _p(v), w.numel(), lr, b1, b2, eps, step,
                            _stream()), "hlbg_nn_adam")


def to_bf16(x, y):
    _need(x, _F32, "to_bf16 input")
    _need(y, _BF16, "to_bf16 output")
    _ok(_lib().hlbg_nn_to_bf16(_p(x), _p(y), x.numel(), _stream()), "hlbg_nn_to_bf16")
