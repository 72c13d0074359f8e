"""Learned warm start for steady vessel flow.

A 3-D convolutional U-Net predicts the steady velocity and pressure of a vessel
from its geometry (fluid mask, signed distance to the wall, inlet pressure and
relaxation time on a cubic voxel box).  The solver then starts from the
equilibrium on that prediction (``hlbg_init_equilibrium_field``, the
reference's EquilibriumInitialCondition applied per site,
Code/lb/InitialCondition.hpp:40-52), instead of from rest, and steps until the
StabilityTester convergence test holds (``hlbg_run_to_steady``).

The network is trained and run on the GPU by the library's own BF16 tensor-core
kernels (include/hemelb_gb300_nn.h: implicit-GEMM 3-D convolutions and their
input and weight gradients, pooling, upsampling, masked MSE, Adam); torch only
provides device memory and the stream.  Activations and weights are BF16, every
product accumulates in FP32, and the master weights and the network output are
FP32.

Targets come from the plain FP64 D3Q19 LBGK solver itself: bounce-back walls,
Nash pressure iolets (inlet density 1 + drho, outlets 1), run from rest to
max |du| / U_ref <= 1e-6.  Training samples are solved with a one-off average of
the first two time levels (``hlbg_average_time_levels``), which removes the
lattice's slowly decaying staggered-momentum mode and shortens data generation
about sixfold; held-out samples are solved exactly as the reference would, from
rest, and that plain solve is the yardstick for the error of every warm-started run.

U_ref, the StabilityTester reference speed, is the Poiseuille centreline speed
of the inlet tube under the mean pressure gradient: (drho c_s^2 / box) R_in^2 / (4 nu).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import capi, nn
from .lbm import Case, InOutLetCosine, LbmParameters, SyntheticGeometry

CS2 = 1.0 / 3.0
N_IN = 16   # input channels (7 used, the rest zero: the convolution wants multiples of 16)
N_OUT = 16  # output channels (u_x, u_y, u_z, p used; the rest are trained towards zero)


# ---------------------------------------------------------------------------
# samples and the plain solver
# ---------------------------------------------------------------------------
@dataclass
class Sample:
    """One seeded vessel in a box with its flow parameters."""

    seed: int
    kind: int      # 0 stenosis, 1 bifurcation
    tau: float     # U[0.7, 1.0]
    drho: float    # inlet density excess, U[5e-4, 3e-3]
    box: int = 96

    @staticmethod
    def draw(index: int, base_seed: int = 20240607, box: int = 96) -> "Sample":
        rng = np.random.default_rng([base_seed, index])
        return Sample(seed=int(rng.integers(1 << 62)), kind=int(rng.integers(2)),
                      tau=float(rng.uniform(0.7, 1.0)), drho=float(rng.uniform(5e-4, 3e-3)),
                      box=box)

    def geometry(self) -> SyntheticGeometry:
        return SyntheticGeometry.vessel_box(self.seed, self.box, self.kind, 19)

    def case(self, g: SyntheticGeometry | None = None) -> Case:
        g = g or self.geometry()
        inl, outl = [], []
        for k in range(g.n_inlets):
            pos, nrm, _ = g.iolet(False, k)
            inl.append(InOutLetCosine(pos, nrm, density_mean=1.0 + self.drho))
        for k in range(g.n_outlets):
            pos, nrm, _ = g.iolet(True, k)
            outl.append(InOutLetCosine(pos, nrm, density_mean=1.0))
        p = LbmParameters(tau=self.tau, kernel=capi.KERNEL_LBGK, wall=capi.WALL_SBB,
                          inlet=capi.IOLET_NASH, outlet=capi.IOLET_NASH, precision=capi.FP64)
        return Case("vessel_box_%d" % self.seed, g, p, inl, outl, 0)

    def u_ref(self, g: SyntheticGeometry) -> float:
        r_in = g.iolet(False, 0)[2]
        nu = (self.tau - 0.5) * CS2
        return (self.drho * CS2 / self.box) * r_in * r_in / (4.0 * nu)


class SteadyRunner:
    """One solver context for a sample, reused by every start.  Its CUDA graphs (one
    per array parity) are captured before any timed run, so a timed run covers the
    initial condition, the optional averaging step and the steps to steady state."""

    def __init__(self, case: Case, u_ref: float, tol: float = 1e-6, check_batch: int = 25):
        self.s = case.solver()
        self.u_ref, self.tol, self.check_batch = u_ref, tol, check_batch
        self.coords = self.s.site_coords()
        for pre in (0, 1):  # capture the graphs of both parities, untimed
            self.s.SetInitialConditions()
            if pre:
                self.s.DoTimeStep(1)
            self.s.RunToSteady(tol, u_ref, check_batch, check_batch)

    def run(self, start=None, average: bool = False, max_steps: int = 400_000, timed: bool = True):
        """From rest (start None) or from the equilibrium on start(coords) -> (rho, u)
        in contiguous site order.  Returns (record, rho, u) of the final state.  A
        timed run first waits for all device work, so its clock covers only itself."""
        s = self.s
        if timed:
            torch.cuda.synchronize()
        t0 = time.perf_counter()
        if start is None:
            s.SetInitialConditions()
        else:
            rho0, u0 = start(self.coords)
            s.SetInitialField(rho0, u0)
        t_init = time.perf_counter() - t0
        pre = 0
        if average:
            s.DoTimeStep(1, sync=False)
            s.AverageTimeLevels()
            pre = 1
        steps, run, du, rc = s.RunToSteady(self.tol, self.u_ref, max_steps, self.check_batch)
        seconds = time.perf_counter() - t0
        rec = {"steps": steps + pre if rc == 0 else -1, "steps_run": run + pre, "seconds": seconds,
               "init_seconds": t_init, "final_rel_du": du, "status": rc}
        rho, u = s.macro()
        return rec, rho, u

    def close(self):
        self.s.close()


# ---------------------------------------------------------------------------
# network inputs and targets on the box grid
# ---------------------------------------------------------------------------
class Grids:
    """Compact per-sample grids on the device: fluid mask (uint8), signed distance
    (FP16), scalar parameters, and normalised targets (FP32 u/U_ref, (rho-1)/drho)."""

    def __init__(self, n: int, box: int, device="cuda", with_targets=True):
        shp = (n, box, box, box)
        self.box = box
        self.mask = torch.zeros(shp, dtype=torch.uint8, device=device)
        self.sdf = torch.zeros(shp, dtype=torch.float16, device=device)
        self.scal = torch.zeros((n, 2), dtype=torch.float32, device=device)
        self.target = torch.zeros(shp + (4,), dtype=torch.float32, device=device) if with_targets else None
        c = (torch.arange(box, dtype=torch.float32, device=device) + 0.5) / box - 0.5
        self.coord = torch.stack(torch.meshgrid(c, c, c, indexing="ij"), dim=-1)  # (B, B, B, 3)

    @staticmethod
    def host_inputs(g: SyntheticGeometry):
        """(fluid mask uint8, scaled signed distance FP16) on the box grid."""
        sd = np.clip(g.signed_distance() / 8.0, -2.0, 2.0).astype(np.float16)
        return g.fluid_grid().astype(np.uint8), sd

    def put(self, i: int, g: SyntheticGeometry | None, smp: Sample, coords=None, rho=None, u=None,
            u_ref=None, inputs=None):
        fl, sd = inputs if inputs is not None else self.host_inputs(g)
        self.mask[i] = torch.from_numpy(fl).to(self.mask.device)
        self.sdf[i] = torch.from_numpy(sd).to(self.sdf.device)
        self.scal[i, 0] = (smp.drho - 1.75e-3) / 1.25e-3
        self.scal[i, 1] = (smp.tau - 0.85) / 0.15
        if coords is not None and self.target is not None:
            t = np.zeros((self.box,) * 3 + (4,), dtype=np.float32)
            x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
            t[x, y, z, 0:3] = u / u_ref
            t[x, y, z, 3] = (rho - 1.0) / smp.drho
            self.target[i] = torch.from_numpy(t).to(self.target.device)

    @staticmethod
    def _space(t, code: int):
        """Exact symmetries of the problem in the x-y plane (inlet plane z fixed):
        bit 0 mirrors x, bit 1 mirrors y, bit 2 swaps x and y (dims 1 and 2)."""
        if code & 1:
            t = t.flip(1)
        if code & 2:
            t = t.flip(2)
        if code & 4:
            t = t.transpose(1, 2)
        return t

    def features(self, idx, code: int = 0) -> torch.Tensor:
        """BF16 input tensor (n, B, B, B, 16) for the samples idx, transformed by `code`."""
        idx = torch.as_tensor(idx, device=self.mask.device)
        n = idx.numel()
        f = torch.zeros((n,) + (self.box,) * 3 + (N_IN,), dtype=torch.float32, device=self.mask.device)
        f[..., 0] = self._space(self.mask[idx].float(), code)
        f[..., 1] = self._space(self.sdf[idx].float(), code)
        f[..., 2] = self.scal[idx, 0].view(n, 1, 1, 1)
        f[..., 3] = self.scal[idx, 1].view(n, 1, 1, 1)
        f[..., 4:7] = self.coord  # position in the box, not transformed
        return f.to(torch.bfloat16).contiguous()

    def targets(self, idx, code: int = 0):
        """(FP32 targets padded to 16 channels, FP32 fluid mask) for the samples idx,
        transformed by `code` (mirrored velocity components change sign; the swap
        exchanges u_x and u_y)."""
        idx = torch.as_tensor(idx, device=self.mask.device)
        src = self._space(self.target[idx], code)
        t = torch.zeros(src.shape[:-1] + (N_OUT,), dtype=torch.float32, device=self.mask.device)
        t[..., :4] = src
        if code & 1:
            t[..., 0] = -t[..., 0]
        if code & 2:
            t[..., 1] = -t[..., 1]
        if code & 4:
            t[..., [0, 1]] = t[..., [1, 0]]
        return t.contiguous(), self._space(self.mask[idx].float(), code).contiguous()


# ---------------------------------------------------------------------------
# the U-Net, forward and backward by hand on the library's kernels
# ---------------------------------------------------------------------------
class Conv:
    """3x3x3 (or 1x1x1) convolution, bias and optional ReLU, with FP32 master
    weights, their BF16 copy, FP32 gradients and Adam moments."""

    def __init__(self, cin, cout, rng, taps=27, relu=True, device="cuda", scale=1.0):
        self.cin, self.cout, self.taps, self.relu = cin, cout, taps, relu
        w = rng.standard_normal((taps, cout, cin)) * math.sqrt(2.0 / (taps * cin)) * scale
        self.w = torch.tensor(w, dtype=torch.float32, device=device)
        self.wb = self.w.to(torch.bfloat16)
        self.b = torch.zeros(cout, dtype=torch.float32, device=device)
        self.gw = torch.zeros_like(self.w)
        self.gb = torch.zeros_like(self.b)
        self.mw, self.vw = torch.zeros_like(self.w), torch.zeros_like(self.w)
        self.mb, self.vb = torch.zeros_like(self.b), torch.zeros_like(self.b)
        self.wt = torch.empty((taps, cout, cin), dtype=torch.bfloat16, device=device).transpose(1, 2).contiguous()
        self.x = self.y = None

    def n_params(self):
        return self.w.numel() + self.b.numel()

    def forward(self, x, out_f32=False):
        shp = tuple(x.shape[:4]) + (self.cout,)
        y = torch.empty(shp, dtype=torch.bfloat16, device=x.device)
        y32 = torch.empty(shp, dtype=torch.float32, device=x.device) if out_f32 else None
        nn.conv3d(x, self.wb, self.b, y, y32, taps=self.taps, relu=self.relu)
        self.x, self.y = x, y
        return y32 if out_f32 else y

    def backward(self, dy, need_dx=True):
        if self.relu:
            nn.relu_backward(dy, self.y)
        nn.bias_grad(dy, self.gb)
        nn.conv3d_weight_grad(self.x, dy, self.gw)
        dx = None
        if need_dx:
            dx = torch.empty(self.x.shape, dtype=torch.bfloat16, device=dy.device)
            nn.conv3d_data_grad(dy, self.wb, dx, wt=self.wt)
        self.x = self.y = None
        return dx

    def zero_grad(self):
        self.gw.zero_()
        self.gb.zero_()

    def step(self, lr, t):
        nn.adam(self.w, self.wb, self.gw, self.mw, self.vw, lr, t)
        nn.adam(self.b, None, self.gb, self.mb, self.vb, lr, t)

    def state(self):
        return {"w": self.w.cpu().numpy(), "b": self.b.cpu().numpy()}

    def load(self, st):
        self.w.copy_(torch.from_numpy(st["w"]))
        self.b.copy_(torch.from_numpy(st["b"]))
        self.wb.copy_(self.w.to(torch.bfloat16))


class UNet:
    """Four-level 3-D U-Net: two 3x3x3 convolutions + ReLU per level, 2x average
    pooling down, nearest 2x upsampling and skip concatenation up, a 1x1x1 FP32
    head.  Channels (16, 48, 96, 192) give about 3.2M parameters."""

    NAMES = ("e0a", "e0b", "e1a", "e1b", "e2a", "e2b", "ba", "bb",
             "d2a", "d2b", "d1a", "d1b", "d0a", "d0b", "head")

    def __init__(self, ch=(16, 48, 96, 192), seed=0, device="cuda"):
        c0, c1, c2, c3 = ch
        for c in ch:
            if c % 16:
                raise ValueError("channel counts must be multiples of 16")
        rng = np.random.default_rng(seed)
        spec = {"e0a": (N_IN, c0), "e0b": (c0, c0), "e1a": (c0, c1), "e1b": (c1, c1),
                "e2a": (c1, c2), "e2b": (c2, c2), "ba": (c2, c3), "bb": (c3, c3),
                "d2a": (c3 + c2, c2), "d2b": (c2, c2), "d1a": (c2 + c1, c1), "d1b": (c1, c1),
                "d0a": (c1 + c0, c0), "d0b": (c0, c0)}
        self.L = {k: Conv(ci, co, rng, device=device) for k, (ci, co) in spec.items()}
        self.L["head"] = Conv(c0, N_OUT, rng, taps=1, relu=False, device=device, scale=0.1)
        self.ch = ch
        self.t = 0
        self._saved = None

    def n_params(self):
        return sum(c.n_params() for c in self.L.values())

    @staticmethod
    def _pool(x):
        n, d, h, w, c = x.shape
        y = torch.empty((n, d // 2, h // 2, w // 2, c), dtype=torch.bfloat16, device=x.device)
        nn.pool2(x, y)
        return y

    @staticmethod
    def _up_cat(x, skip):
        n, d, h, w, c = skip.shape
        u = torch.empty((n, d, h, w, x.shape[-1]), dtype=torch.bfloat16, device=x.device)
        nn.up2(x, u)
        y = torch.empty((n, d, h, w, x.shape[-1] + c), dtype=torch.bfloat16, device=x.device)
        nn.concat(u, skip, y)
        return y

    def forward(self, x):
        """x: BF16 (n, B, B, B, 16), B a multiple of 8.  Returns FP32 (n, B, B, B, 16)."""
        L = self.L
        e0 = L["e0b"].forward(L["e0a"].forward(x))
        e1 = L["e1b"].forward(L["e1a"].forward(self._pool(e0)))
        e2 = L["e2b"].forward(L["e2a"].forward(self._pool(e1)))
        b = L["bb"].forward(L["ba"].forward(self._pool(e2)))
        d2 = L["d2b"].forward(L["d2a"].forward(self._up_cat(b, e2)))
        d1 = L["d1b"].forward(L["d1a"].forward(self._up_cat(d2, e1)))
        d0 = L["d0b"].forward(L["d0a"].forward(self._up_cat(d1, e0)))
        self._saved = (e0, e1, e2, b, d2, d1)
        return L["head"].forward(d0, out_f32=True)

    @staticmethod
    def _split_up(g, x_shape, skip_grad):
        """Gradient of concat(up2(x), skip): returns dx and writes the skip part."""
        n, d, h, w, _ = skip_grad.shape
        gu = torch.empty((n, d, h, w, x_shape[-1]), dtype=torch.bfloat16, device=g.device)
        nn.split(g, gu, skip_grad)
        gx = torch.empty(x_shape, dtype=torch.bfloat16, device=g.device)
        nn.up2_backward(gu, gx)
        return gx

    @staticmethod
    def _pool_back_add(g, acc):
        tmp = torch.empty(acc.shape, dtype=torch.bfloat16, device=g.device)
        nn.pool2_backward(g, tmp)
        nn.add_(acc, tmp)

    def backward(self, dout):
        """dout: BF16 gradient of the loss w.r.t. the FP32 output; accumulates the
        weight gradients of every layer."""
        L = self.L
        e0, e1, e2, b, d2, d1 = self._saved
        g = L["d0a"].backward(L["d0b"].backward(L["head"].backward(dout)))
        ge0 = torch.empty_like(e0)
        g = self._split_up(g, d1.shape, ge0)
        g = L["d1a"].backward(L["d1b"].backward(g))
        ge1 = torch.empty_like(e1)
        g = self._split_up(g, d2.shape, ge1)
        g = L["d2a"].backward(L["d2b"].backward(g))
        ge2 = torch.empty_like(e2)
        g = self._split_up(g, b.shape, ge2)
        g = L["ba"].backward(L["bb"].backward(g))
        self._pool_back_add(g, ge2)
        g = L["e2a"].backward(L["e2b"].backward(ge2))
        self._pool_back_add(g, ge1)
        g = L["e1a"].backward(L["e1b"].backward(ge1))
        self._pool_back_add(g, ge0)
        L["e0a"].backward(L["e0b"].backward(ge0), need_dx=False)
        self._saved = None

    def zero_grad(self):
        for c in self.L.values():
            c.zero_grad()

    def step(self, lr):
        self.t += 1
        for c in self.L.values():
            c.step(lr, self.t)

    def state(self):
        return {k: c.state() for k, c in self.L.items()}

    def load(self, st):
        for k, c in self.L.items():
            c.load(st[k])


# ---------------------------------------------------------------------------
# dataset, training, prediction
# ---------------------------------------------------------------------------
def _solve_sample(smp: Sample, average: bool):
    g = smp.geometry()
    ur = smp.u_ref(g)
    runner = SteadyRunner(smp.case(g), ur)
    try:
        rec, rho, u = runner.run(average=average, timed=False)
    finally:
        runner.close()
    rec.update({"sites": int(g.n_fluid), "u_ref": ur, "kind": smp.kind, "tau": smp.tau, "drho": smp.drho})
    return rec, runner.coords, rho, u, Grids.host_inputs(g)


def generate(samples, box: int, average: bool = True, workers: int = 8, log=None):
    """Solve every sample with the plain FP64 solver, `workers` contexts at a time
    (one host thread and CUDA stream each: a single small geometry leaves most of
    the GPU idle).  Returns (Grids, records)."""
    from concurrent.futures import ThreadPoolExecutor
    grids = Grids(len(samples), box)
    recs = [None] * len(samples)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=workers) as ex:
        futs = [ex.submit(_solve_sample, smp, average) for smp in samples]
        for i, (smp, f) in enumerate(zip(samples, futs)):
            rec, co, rho, u, inputs = f.result()
            grids.put(i, None, smp, co, rho, u, rec["u_ref"], inputs=inputs)
            recs[i] = rec
            if log and (i + 1) % 250 == 0:
                log("generated %d/%d samples in %.1f s" % (i + 1, len(samples), time.perf_counter() - t0))
    return grids, recs


def train(net: UNet, grids: Grids, n: int, batch: int = 4, seconds: float = 600.0,
          max_epochs: int = 1000, lr_max: float = 1e-3, lr_min: float = 2e-5, seed: int = 0,
          augment: bool = True, log=None, epochs: int | None = None):
    """Adam on the masked MSE of the normalised targets, cosine learning-rate decay
    over the time budget (or, with `epochs`, over that many epochs regardless of
    time, so that the result does not depend on the machine's speed), each batch
    under a random symmetry of the x-y plane when `augment`.  Returns the loss
    history (per epoch mean)."""
    rng = np.random.default_rng(seed)
    hist = []
    t0 = time.perf_counter()
    epoch = 0
    done = False
    per_epoch = max(1, (n - batch) // batch + 1)
    if epochs is not None:
        max_epochs = epochs
    while not done and epoch < max_epochs:
        order = rng.permutation(n)
        tot, cnt = 0.0, 0
        for k in range(0, n - batch + 1, batch):
            if epochs is not None:
                frac = (epoch * per_epoch + cnt) / float(epochs * per_epoch)
            else:
                frac = min(1.0, (time.perf_counter() - t0) / seconds)
            lr = lr_min + 0.5 * (lr_max - lr_min) * (1.0 + math.cos(math.pi * frac))
            idx = order[k:k + batch]
            code = int(rng.integers(8)) if augment else 0
            x = grids.features(idx, code)
            tgt, mask = grids.targets(idx, code)
            out = net.forward(x)
            dout = torch.empty(out.shape, dtype=torch.bfloat16, device=out.device)
            loss = nn.mse(out, tgt, mask, dout)
            net.zero_grad()
            net.backward(dout)
            net.step(lr)
            tot += loss
            cnt += 1
            if epochs is None and time.perf_counter() - t0 > seconds:
                done = True
                break
        epoch += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log("epoch %d loss %.3e (%.0f s)" % (epoch, hist[-1], time.perf_counter() - t0))
    return hist


def predict(net: UNet, grids: Grids, i: int, smp: Sample, coords, u_ref: float):
    """Prediction for sample i at the fluid sites `coords` (contiguous order):
    (rho, u) in lattice units."""
    out = net.forward(grids.features([i]))[0]
    x = torch.as_tensor(coords[:, 0], device=out.device, dtype=torch.long)
    y = torch.as_tensor(coords[:, 1], device=out.device, dtype=torch.long)
    z = torch.as_tensor(coords[:, 2], device=out.device, dtype=torch.long)
    v = out[x, y, z, :4].double().cpu().numpy()
    return 1.0 + v[:, 3] * smp.drho, v[:, :3] * u_ref


def rel_l2(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


def evaluate(net: UNet, samples, box: int, plain_warm: int = 0, log=None):
    """Held-out evaluation.  Per sample, on one context: the plain solve from rest
    (the reference's start; the others are measured against its field), rest with the one-off
    averaging, and the warm start (prediction, averaging); for the first
    `plain_warm` samples also the warm start without averaging.  Wall times include
    the prediction and the field upload."""
    grids = Grids(len(samples), box, with_targets=False)
    out = []
    t0 = time.perf_counter()
    for i, smp in enumerate(samples):
        g = smp.geometry()
        grids.put(i, g, smp)
        ur = smp.u_ref(g)
        runner = SteadyRunner(smp.case(g), ur)
        try:
            rest, rho_p, u_p = runner.run()
            rest_avg, rho_a, u_a = runner.run(average=True)
            pred = lambda co: predict(net, grids, i, smp, co, ur)
            warm, rho_w, u_w = runner.run(start=pred, average=True)
            warm_plain = None
            if i < plain_warm:
                warm_plain, _, u_wp = runner.run(start=pred, average=False)
            rho0, u0 = pred(runner.coords)
        finally:
            runner.close()
        dp = lambda r: (r - 1.0) / smp.drho
        rec = {"sample": i, "kind": smp.kind, "tau": smp.tau, "drho": smp.drho, "sites": int(g.n_fluid),
               "u_ref": ur, "rest": rest, "rest_avg": rest_avg, "warm": warm,
               "prediction_u_rel_l2": rel_l2(u0, u_p), "prediction_p_rel_l2": rel_l2(dp(rho0), dp(rho_p)),
               "warm_u_rel_l2": rel_l2(u_w, u_p), "warm_p_rel_l2": rel_l2(dp(rho_w), dp(rho_p)),
               "rest_avg_u_rel_l2": rel_l2(u_a, u_p)}
        if warm_plain is not None:
            rec["warm_plain"] = warm_plain
            rec["warm_plain_u_rel_l2"] = rel_l2(u_wp, u_p)
        out.append(rec)
        if log and (i + 1) % 25 == 0:
            log("evaluated %d/%d (%.1f s)" % (i + 1, len(samples), time.perf_counter() - t0))
    return out


def summarise(evals) -> dict:
    """Medians and totals over held-out samples."""
    res = {"n": len(evals)}
    for arm in ("rest", "rest_avg", "warm", "warm_plain"):
        sub = [e for e in evals if arm in e]
        if not sub:
            continue
        st = np.array([e[arm]["steps"] for e in sub], dtype=np.float64)
        secs = np.array([e[arm]["seconds"] for e in sub], dtype=np.float64)
        ok = st > 0
        res[arm] = {"n": len(sub), "converged": int(ok.sum()),
                    "median_steps": float(np.median(st[ok])) if ok.any() else None,
                    "total_steps": float(st[ok].sum()), "total_seconds": float(secs.sum()),
                    "median_seconds": float(np.median(secs))}
    both = np.array([e["rest"]["steps"] > 0 and e["warm"]["steps"] > 0 for e in evals])
    if both.any():
        r = np.array([e["rest"]["steps"] for e in evals])[both]
        w = np.array([e["warm"]["steps"] for e in evals])[both]
        rs = np.array([e["rest"]["seconds"] for e in evals])[both]
        ws = np.array([e["warm"]["seconds"] for e in evals])[both]
        ra = np.array([e["rest_avg"]["steps"] for e in evals])[both]
        res["speedup_steps_vs_rest"] = float(r.sum() / w.sum())
        res["speedup_seconds_vs_rest"] = float(rs.sum() / ws.sum())
        res["median_speedup_steps_vs_rest"] = float(np.median(r / w))
        res["speedup_steps_vs_rest_avg"] = float(ra.sum() / w.sum())
    for k in ("prediction_u_rel_l2", "prediction_p_rel_l2", "warm_u_rel_l2", "warm_p_rel_l2",
              "rest_avg_u_rel_l2", "warm_plain_u_rel_l2"):
        v = np.array([e[k] for e in evals if k in e])
        if not v.size:
            continue
        res[k] = {"median": float(np.median(v)), "p90": float(np.percentile(v, 90)), "max": float(v.max())}
    return res


def _field_at(grid, coords, smp: Sample, u_ref: float):
    """(rho, u) in lattice units at the fluid sites `coords` from a predicted box
    grid (B, B, B, 4) of normalised (u, p)."""
    v = grid[coords[:, 0], coords[:, 1], coords[:, 2]].astype(np.float64)
    return 1.0 + v[:, 3] * smp.drho, v[:, :3] * u_ref


def _accuracy_one(i: int, smp: Sample, grid, check_every: int) -> dict:
    g = smp.geometry()
    ur = smp.u_ref(g)
    runner = SteadyRunner(smp.case(g), ur)
    s = runner.s
    try:
        rest, _, u_p = runner.run(timed=False)
        steps_rest = rest["steps_run"]
        s.RunToSteady(1e-9, ur, max(3 * steps_rest, 20000), runner.check_batch)
        u_ref_field = s.macro()[1]
        e_plain = rel_l2(u_p, u_ref_field)
        rec = {"sample": i, "kind": smp.kind, "tau": smp.tau, "rest_steps": steps_rest,
               "rest_error": e_plain}
        for arm in ("rest_avg", "warm"):
            if arm == "rest_avg":
                s.SetInitialConditions()
            else:
                s.SetInitialField(*_field_at(grid, runner.coords, smp, ur))
            s.DoTimeStep(1)
            s.AverageTimeLevels()
            steps, err = 1, float("inf")
            while steps < 4 * steps_rest:
                s.DoTimeStepGraph(check_every)
                steps += check_every
                err = rel_l2(s.macro()[1], u_ref_field)
                if err <= e_plain:
                    break
            rec[arm + "_steps_to_match"] = steps if err <= e_plain else -1
            rec[arm + "_error"] = err
    finally:
        runner.close()
    return rec


def accuracy_study(net: UNet, samples, box: int, check_every: int = 50, workers: int = 8, log=None):
    """Steps to the plain solve's own accuracy.  A reference field comes from the
    plain solve continued to max |du| / U_ref <= 1e-9 (or three times its steps);
    the plain solve's error against it is the accuracy to match.  The rest start
    with averaging and the warm start are then stepped, checked every
    `check_every` steps, until their error against the reference is no larger.
    The predictions are made first; the samples then run `workers` contexts at a
    time (steps are counted, not timed)."""
    from concurrent.futures import ThreadPoolExecutor
    grids = Grids(1, box, with_targets=False)
    preds = []
    for smp in samples:
        grids.put(0, smp.geometry(), smp)
        preds.append(net.forward(grids.features([0]))[0][..., :4].float().cpu().numpy())
    del grids
    out = [None] * len(samples)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        futs = [ex.submit(_accuracy_one, i, smp, preds[i], check_every) for i, smp in enumerate(samples)]
        for i, f in enumerate(futs):
            out[i] = f.result()
            preds[i] = None
            if log and (i + 1) % 25 == 0:
                log("accuracy study %d/%d" % (i + 1, len(samples)))
    ok = [r for r in out if r["warm_steps_to_match"] > 0]
    both = [r for r in ok if r["rest_avg_steps_to_match"] > 0]
    summ = {"n": len(out), "matched": len(ok), "rest_avg_matched": len(both),
            "median_rest_error": float(np.median([r["rest_error"] for r in out])),
            "rest_steps_total": float(sum(r["rest_steps"] for r in ok)),
            "warm_steps_to_match_total": float(sum(r["warm_steps_to_match"] for r in ok)),
            "rest_avg_steps_to_match_total": float(sum(max(r["rest_avg_steps_to_match"], 0) for r in ok))}
    if ok:
        summ["speedup_at_same_accuracy_vs_rest"] = summ["rest_steps_total"] / summ["warm_steps_to_match_total"]
        summ["median_speedup_at_same_accuracy"] = float(np.median(
            [r["rest_steps"] / r["warm_steps_to_match"] for r in ok]))
    if both:
        # what the trained network adds over the same start without it (rest +
        # one average), on the samples where both reach the plain solve's accuracy
        summ["network_gain_at_same_accuracy"] = (sum(r["rest_avg_steps_to_match"] for r in both)
                                                 / sum(r["warm_steps_to_match"] for r in both))
        summ["median_network_gain_at_same_accuracy"] = float(np.median(
            [r["rest_avg_steps_to_match"] / r["warm_steps_to_match"] for r in both]))
    return out, summ


def bench_kernels(reps: int = 10, batch: int = 4):
    """CUDA-event time of the convolution kernels at the U-Net's layer shapes on a
    batch of 96^3 boxes (inputs far larger than L2): TFLOP/s of forward, input
    gradient and weight gradient, 2 * 27 * C_in * C_out FLOP per voxel each."""
    shapes = [(96, N_IN, 16), (96, 16, 16), (48, 16, 48), (48, 48, 48), (24, 48, 96), (24, 96, 96),
              (12, 96, 192), (12, 192, 192), (24, 288, 96), (48, 144, 48), (96, 64, 16)]
    out = []
    for dim, cin, cout in shapes:
        x = torch.randn((batch, dim, dim, dim, cin), device="cuda").to(torch.bfloat16)
        w = (torch.randn((27, cout, cin), device="cuda") * 0.05).to(torch.bfloat16)
        b = torch.zeros(cout, device="cuda")
        y = torch.empty((batch, dim, dim, dim, cout), dtype=torch.bfloat16, device="cuda")
        dx = torch.empty_like(x)
        wt = torch.empty((27, cin, cout), dtype=torch.bfloat16, device="cuda")
        dw = torch.zeros((27, cout, cin), device="cuda")
        flop = 2.0 * 27 * cin * cout * batch * dim ** 3
        rec = {"voxels": batch * dim ** 3, "c_in": cin, "c_out": cout,
               "tc_forward": nn.tc_eligible(cin, cout), "tc_input_grad": nn.tc_eligible(cout, cin),
               "tc_tiles": nn.tc_tiles(batch, dim, dim, dim)}
        for name, fn in (("forward", lambda: nn.conv3d(x, w, b, y, None, 27, True, engine="mma")),
                         ("forward_tc", lambda: nn.conv3d(x, w, b, y, None, 27, True, engine="auto")),
                         ("input_grad", lambda: nn.conv3d_data_grad(y, w, dx, None, wt, engine="mma")),
                         ("input_grad_tc", lambda: nn.conv3d_data_grad(y, w, dx, None, wt, engine="auto")),
                         ("weight_grad", lambda: nn.conv3d_weight_grad(x, y, dw))):
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            rec[name] = {"ms": ms, "tflops": flop / ms / 1e9}
        out.append(rec)
    return out


def main(argv=None):
    """Generate, train, evaluate: the warm-start report as one JSON document."""
    import argparse
    import json
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--train", type=int, default=3000)
    ap.add_argument("--test", type=int, default=300)
    ap.add_argument("--box", type=int, default=96)
    ap.add_argument("--train-seconds", type=float, default=900.0)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--plain-warm", type=int, default=16)
    ap.add_argument("--accuracy-study", type=int, default=300)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--out", default="")
    ap.add_argument("--save-weights", default="")
    ap.add_argument("--bench-kernels", action="store_true",
                    help="only time the convolution kernels at the network's layer shapes")
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)
    if a.bench_kernels:
        res = bench_kernels()
        log(json.dumps(res, indent=1))
        return res
    train_s = [Sample.draw(i, box=a.box) for i in range(a.train)]
    test_s = [Sample.draw(1_000_000 + i, box=a.box) for i in range(a.test)]
    t0 = time.perf_counter()
    grids, recs = generate(train_s, a.box, average=True, workers=a.workers, log=log)
    t_gen = time.perf_counter() - t0
    st = np.array([r["steps"] for r in recs])
    net = UNet(seed=0)
    t0 = time.perf_counter()
    hist = train(net, grids, a.train, batch=a.batch, seconds=a.train_seconds, log=log)
    t_train = time.perf_counter() - t0
    del grids
    torch.cuda.empty_cache()
    evals = evaluate(net, test_s, a.box, plain_warm=a.plain_warm, log=log)
    summ = summarise(evals)
    acc, acc_summ = accuracy_study(net, test_s[:a.accuracy_study], a.box, workers=a.workers, log=log)
    doc = {"workload": "%d training + %d held-out seeded stenoses/bifurcations in a %d^3 box, D3Q19 LBGK "
                       "FP64, bounce-back walls, Nash pressure iolets" % (a.train, a.test, a.box),
           "criterion": "max |u_new - u_old| / U_ref <= 1e-6 after every step",
           "network": {"params": net.n_params(), "channels": list(net.ch), "dtype": "bf16, fp32 accumulate"},
           "datagen": {"seconds": t_gen, "median_steps": float(np.median(st)), "failed": int((st < 0).sum())},
           "training": {"seconds": t_train, "epochs": len(hist), "loss_first": hist[0], "loss_last": hist[-1]},
           "heldout": summ, "accuracy_study": acc_summ,
           "samples": evals, "accuracy_samples": acc}
    if a.out:
        with open(a.out, "w") as f:
            json.dump(doc, f, indent=1, default=float)
    if a.save_weights:
        np.savez_compressed(a.save_weights, **{k + "_" + n: v for k, c in net.state().items()
                                               for n, v in c.items()})
    log(json.dumps({k: doc[k] for k in ("network", "datagen", "training", "heldout", "accuracy_study")},
                   indent=1, default=float))
    return doc


if __name__ == "__main__":
    main()
