"""The multi-rank exchange on the device, with ranks emulated as contexts on one GPU.

Each emulated rank holds a context created on its halo's local geometry (owned +
ghost blocks).  A step is StreamAndCollide on every rank; a device pack of each
send list (hlbg_halo_pack_device) into a buffer, and, once every pack has
completed, a device unpack of the matching buffer into the receiving rank's new
distributions (hlbg_halo_unpack_device); then PostStep and the swap on every
rank.  The host orders the phases (every wait is a stream synchronisation on the
host; no kernel waits on another).  The owned sites then equal the single-context
update bit for bit in FP64, FP32-deviation and FP16 storage: the exchange moves
stored values, so it is exact in every form.  The same holds with the library's
exchange (halo.HaloExchange) run by two processes over gloo.
"""
import ctypes as C

import numpy as np
import pytest

from hemelb_gb300 import capi, cases, halo
from hemelb_gb300.lbm import LBM

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

I32, I8, I16, I64 = C.POINTER(C.c_int32), C.POINTER(C.c_int8), C.POINTER(C.c_int16), C.POINTER(C.c_int64)


def _bifurcation():
    c = cases.bifurcation(seed=11, parent_radius=8.0, parent_length=40.0, daughter_length_factor=1.2,
                          period=200.0)
    c.params.kernel = capi.KERNEL_TRT
    return c


def _offsets(lib, s, triples):
    b = np.ascontiguousarray(triples[:, 0], dtype=np.int32)
    d = np.ascontiguousarray(triples[:, 1], dtype=np.int8)
    t = np.ascontiguousarray(triples[:, 2], dtype=np.int16)
    out = np.empty(len(triples), dtype=np.int64)
    capi.check(lib.hlbg_halo_offsets(s.ctx, b.ctypes.data_as(I32), d.ctypes.data_as(I8), t.ctypes.data_as(I16),
                                     len(triples), out.ctypes.data_as(I64)), s.ctx)
    return torch.from_numpy(out).cuda()


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class Rank:
    def __init__(self, lib, c, ranks, world, r, precision):
        self.h = halo.Halo(c.geometry.view, ranks, world, r)
        params = c.params
        self.s = LBM(self.h.view, type(params)(**{**params.__dict__, "precision": precision}), c.inlets,
                     c.outlets)
        self.elem = lib.hlbg_storage_bytes(self.s.ctx)
        self.plans = []
        for ex in self.h.exchanges:
            so, ro = _offsets(lib, self.s, ex.send), _offsets(lib, self.s, ex.recv)
            buf = torch.empty(len(ex.send) * self.elem, dtype=torch.uint8, device="cuda")
            self.plans.append((ex.peer, so, ro, buf))


def _partitioned_run(c, world, precision, steps):
    lib = capi.load()
    ranks = halo.partition(c.geometry.view, world)
    rs = [Rank(lib, c, ranks, world, r, precision) for r in range(world)]
    for r in rs:
        r.s.SetInitialConditions()
    torch.cuda.synchronize()
    for _ in range(steps):
        for r in rs:
            r.s.StreamAndCollide(0, r.s.n_sites)
        for r in rs:
            for peer, so, ro, buf in r.plans:
                capi.check(lib.hlbg_halo_pack_device(r.s.ctx, _ptr(so), so.numel(), _ptr(buf)), r.s.ctx)
        for r in rs:
            capi.check(lib.hlbg_halo_check(r.s.ctx), r.s.ctx)
        for r in rs:
            for peer, so, ro, buf in r.plans:
                dst = rs[peer]
                back = [p for p in dst.plans if p[0] == r.h.rank][0]
                ro_dst = back[2]
                assert ro_dst.numel() == so.numel()
                capi.check(lib.hlbg_halo_unpack_device(dst.s.ctx, _ptr(ro_dst), ro_dst.numel(), _ptr(buf)),
                           dst.s.ctx)
        for r in rs:
            capi.check(lib.hlbg_halo_check(r.s.ctx), r.s.ctx)
            r.s.PostStep(0, r.s.n_sites)
            r.s.SwapOldAndNew()
    return rs


def _owned_state(r):
    coords = r.s.site_coords()
    owned = {tuple(x) for x in r.h.block_coords[: r.h.n_owned].tolist()}
    mine = np.array([tuple(x) in owned for x in (coords // 8).tolist()])
    return coords[mine], r.s.GetFOld()[mine], r.s.GetFNew()[mine]


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32DEV, capi.FP16])
@pytest.mark.parametrize("world", [2, 4])
def test_emulated_ranks_equal_single_context(world, precision):
    c = _bifurcation()
    steps = 40
    rs = _partitioned_run(c, world, precision, steps)
    one = c.solver(precision)
    one.SetInitialConditions()
    one.DoTimeStep(steps)
    coords1 = one.site_coords()
    index = {tuple(x): i for i, x in enumerate(coords1.tolist())}
    f1_old, f1_new = one.GetFOld(), one.GetFNew()
    seen = np.zeros(one.n_sites, dtype=int)
    sent = 0
    for r in rs:
        coords, fo, fn = _owned_state(r)
        idx = np.array([index[tuple(x)] for x in coords.tolist()])
        seen[idx] += 1
        assert np.array_equal(fo, f1_old[idx])
        assert np.array_equal(fn, f1_new[idx])
        sent += sum(p[1].numel() for p in r.plans)
    assert np.all(seen == 1) and sent > 0


def test_halo_offsets_outside_the_arrays_are_reported():
    lib = capi.load()
    c = _bifurcation()
    ranks = halo.partition(c.geometry.view, 2)
    r = Rank(lib, c, ranks, 2, 0, capi.FP64)
    r.s.SetInitialConditions()
    before = r.s.GetFNew()
    limit = 19 * r.s.n_slots
    off = torch.tensor([-1, limit, limit + 7], dtype=torch.int64, device="cuda")
    buf = torch.zeros(3 * r.elem, dtype=torch.uint8, device="cuda")
    assert lib.hlbg_halo_unpack_device(r.s.ctx, _ptr(off), 3, _ptr(buf)) == capi.HLBG_OK
    assert lib.hlbg_halo_check(r.s.ctx) == capi.HLBG_ERR_INVAL
    assert b"offset outside" in lib.hlbg_last_error(r.s.ctx)
    assert lib.hlbg_halo_check(r.s.ctx) == capi.HLBG_OK  # the flag is cleared
    assert np.array_equal(r.s.GetFNew(), before)


# ---- the exchange between processes --------------------------------------------

def _free_port():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _process_rank(rank, world, port, precision, steps, out):
    import os
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _process_rank_body(rank, world, precision, steps, out)
    except Exception:
        import traceback
        out.put((rank, "error", traceback.format_exc()))
        raise
    finally:
        dist.destroy_process_group()


def _process_rank_body(rank, world, precision, steps, out):
    import torch.distributed as dist
    c = _bifurcation()
    ranks = halo.partition(c.geometry.view, world)
    h = halo.Halo(c.geometry.view, ranks, world, rank)
    params = c.params
    s = LBM(h.view, type(params)(**{**params.__dict__, "precision": precision}), c.inlets, c.outlets)
    s.SetInitialConditions()
    ex = halo.HaloExchange(s, h)
    ex.step(steps)
    coords = s.site_coords()
    owned = {tuple(x) for x in h.block_coords[: h.n_owned].tolist()}
    mine = np.array([tuple(x) in owned for x in (coords // 8).tolist()])
    out.put((rank, coords[mine].copy(), s.GetFOld()[mine].copy(), s.GetFNew()[mine].copy(),
             sum(len(e.send) for e in h.exchanges)))
    dist.barrier()
    s.close()


@pytest.mark.parametrize("precision", [capi.FP64, capi.FP32DEV])
def test_processes_exchanging_over_gloo_equal_single_context(precision):
    """halo.HaloExchange in two processes that share this GPU, one context each: the
    device pack, the transport (gloo, staged through host memory; every wait is on
    the host, between kernels), the device unpack.  The owned sites equal the
    single-context update bit for bit after 30 steps."""
    import torch.multiprocessing as mp
    world, steps = 2, 30
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_process_rank, args=(r, world, port, precision, steps, q)) for r in range(world)]
    for p in procs:
        p.start()
    parts = []
    for _ in range(world):
        x = q.get(timeout=300)
        if isinstance(x[1], str):  # a rank failed: the other one may wait for it forever
            for p in procs:
                p.terminate()
            pytest.fail(x[2])
        parts.append(x)
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    c = _bifurcation()
    one = c.solver(precision)
    one.SetInitialConditions()
    one.DoTimeStep(steps)
    index = {tuple(x): i for i, x in enumerate(one.site_coords().tolist())}
    f_old, f_new = one.GetFOld(), one.GetFNew()
    seen = np.zeros(one.n_sites, dtype=int)
    for _, coords, fo, fn, sent in parts:
        idx = np.array([index[tuple(x)] for x in coords.tolist()])
        seen[idx] += 1
        assert np.array_equal(fo, f_old[idx]) and np.array_equal(fn, f_new[idx])
        assert sent > 0
    assert np.all(seen == 1)
