"""Multi-rank halo index maps (the C ABI's hlbg_halo_*), for splitting one geometry
over ranks with one exchange per step.

The reference decomposes its domain and exchanges, after StreamAndCollide, the
distributions each rank streamed into sites another rank owns
(geometry::FieldData::SendAndReceive / CopyReceived, Code/geometry/FieldData.cc:
27-49), updating the sites with off-rank neighbours first (Code/lb/lb.hpp:176-309).
`Halo` exposes one rank's share: its local geometry (owned blocks, then ghost
blocks), the edge blocks, and per peer the send and receive lists as
(local block, direction, in-block site) triples in the order both sides agree on.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from hemelb_gb300 import capi


def _check(lib, rc, h=None, what=""):
    if rc != capi.HLBG_OK:
        msg = lib.hlbg_halo_last_error(h).decode() if h else what
        raise capi.HlbgError(rc, msg or what)


def partition(geometry_view: capi.Geometry, n_ranks: int) -> np.ndarray:
    """Rank of every input block: contiguous z-column ranges of equal fluid-site count."""
    lib = capi.load()
    out = np.empty(geometry_view.n_blocks, dtype=np.int32)
    _check(lib, lib.hlbg_halo_partition(C.byref(geometry_view), n_ranks,
                                         out.ctypes.data_as(C.POINTER(C.c_int32))), what="hlbg_halo_partition")
    return out


@dataclass
class Exchange:
    """One peer's lists: each an (n, 3) int array of (local block, direction, site)."""

    peer: int
    send: np.ndarray
    recv: np.ndarray


class Halo:
    def __init__(self, geometry_view: capi.Geometry, block_rank: np.ndarray, n_ranks: int, rank: int):
        self._lib = lib = capi.load()
        self._keep = np.ascontiguousarray(block_rank, dtype=np.int32)
        h = C.c_void_p()
        rc = lib.hlbg_halo_create(C.byref(geometry_view), self._keep.ctypes.data_as(C.POINTER(C.c_int32)),
                                  n_ranks, rank, C.byref(h))
        self._h = h
        if rc != capi.HLBG_OK:
            msg = lib.hlbg_halo_last_error(h).decode() if h else ""
            self.close()
            raise capi.HlbgError(rc, msg)
        self.rank, self.n_ranks = rank, n_ranks
        self.view = capi.Geometry()
        n_owned = C.c_int64()
        _check(lib, lib.hlbg_halo_local_geometry(h, C.byref(self.view), C.byref(n_owned)), h)
        self.n_owned = n_owned.value
        self.n_local = self.view.n_blocks
        self.block_source = np.empty(self.n_local, dtype=np.int64)
        _check(lib, lib.hlbg_halo_block_source(h, self.block_source.ctypes.data_as(C.POINTER(C.c_int64))), h)
        self.edge = np.empty(self.n_owned, dtype=np.uint8)
        if self.n_owned:
            _check(lib, lib.hlbg_halo_edge_blocks(h, self.edge.ctypes.data_as(C.POINTER(C.c_uint8))), h)
        self.block_coords = np.ctypeslib.as_array(self.view.block_coords, (self.n_local * 3,)).reshape(-1, 3).copy()
        self.exchanges = []
        for k in range(lib.hlbg_halo_peer_count(h)):
            pr, ns, nr = C.c_int32(), C.c_int64(), C.c_int64()
            _check(lib, lib.hlbg_halo_peer(h, k, C.byref(pr), C.byref(ns), C.byref(nr)), h)
            lists = []
            for is_recv, n in ((0, ns.value), (1, nr.value)):
                b = np.empty(n, dtype=np.int32)
                d = np.empty(n, dtype=np.int8)
                s = np.empty(n, dtype=np.int16)
                if n:
                    _check(lib, lib.hlbg_halo_list(h, k, is_recv, b.ctypes.data_as(C.POINTER(C.c_int32)),
                                                   d.ctypes.data_as(C.POINTER(C.c_int8)),
                                                   s.ctypes.data_as(C.POINTER(C.c_int16))), h)
                lists.append(np.stack([b.astype(np.int64), d.astype(np.int64), s.astype(np.int64)], axis=1))
            self.exchanges.append(Exchange(pr.value, lists[0], lists[1]))

    def site_coords(self, triples: np.ndarray) -> np.ndarray:
        """Lattice coordinates (n, 3) of the sites named by (local block, *, site) triples."""
        b, s = triples[:, 0], triples[:, 2]
        local = np.stack([s >> 6, (s >> 3) & 7, s & 7], axis=1)
        return self.block_coords[b].astype(np.int64) * 8 + local

    def global_keys(self, triples: np.ndarray) -> np.ndarray:
        """(input block, site, direction) of each triple: the order both sides share."""
        return np.stack([self.block_source[triples[:, 0]], triples[:, 2], triples[:, 1]], axis=1)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.hlbg_halo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- transport ------------------------------------------------------------------

def exchange_buffers(send: dict, recv: dict, group=None) -> None:
    """One exchange over torch.distributed: post every send and every receive (peer
    -> 1-D tensor; a send list and the matching receive list on the peer have the
    same length and order), then wait for all of them, as FieldData::SendAndReceive
    posts its requests before waiting (Code/geometry/FieldData.cc:27-49).  With a
    backend that moves host memory only (gloo), device tensors travel through host
    copies; NCCL moves them directly."""
    import torch
    import torch.distributed as dist
    staged = dist.get_backend(group) != "nccl"
    reqs, keep, landing = [], [], []
    for peer in sorted(send):
        t = send[peer]
        src = t.cpu() if staged and t.is_cuda else t
        keep.append(src)
        reqs.append(dist.isend(src, peer, group=group))
    for peer in sorted(recv):
        t = recv[peer]
        dst = torch.empty(t.shape, dtype=t.dtype) if staged and t.is_cuda else t
        if dst is not t:
            landing.append((t, dst))
        reqs.append(dist.irecv(dst, peer, group=group))
    for r in reqs:
        r.wait()
    for t, dst in landing:
        t.copy_(dst)
    if any(t.is_cuda for t in recv.values()):
        torch.cuda.synchronize()  # the receives are complete before the context's stream reads them


class HaloExchange:
    """One rank's update of a partitioned geometry on its own device: the context
    (an `LBM` on the halo's local geometry) steps every local site; after
    StreamAndCollide the values its sites streamed into ghost sites are packed on
    the device in their storage type (hlbg_halo_pack_device), exchanged with the
    peers (`exchange_buffers`), unpacked into the owned sites they target
    (hlbg_halo_unpack_device), and then PostStep and the swap run -- the order of
    lb::LBM around FieldData's exchange (Code/lb/lb.hpp:176-309).  The owned sites
    then evolve exactly as in one context over the whole geometry."""

    def __init__(self, solver, halo: Halo, group=None):
        import torch
        self._lib = lib = capi.load()
        self.s, self.h, self.group = solver, halo, group
        self.elem = lib.hlbg_storage_bytes(solver.ctx)
        self.plans = []
        for ex in halo.exchanges:
            so, ro = self._offsets(ex.send), self._offsets(ex.recv)
            sbuf = torch.empty(len(ex.send) * self.elem, dtype=torch.uint8, device="cuda")
            rbuf = torch.empty(len(ex.recv) * self.elem, dtype=torch.uint8, device="cuda")
            self.plans.append((ex.peer, so, ro, sbuf, rbuf))

    def _offsets(self, triples: np.ndarray):
        import torch
        b = np.ascontiguousarray(triples[:, 0], dtype=np.int32)
        d = np.ascontiguousarray(triples[:, 1], dtype=np.int8)
        t = np.ascontiguousarray(triples[:, 2], dtype=np.int16)
        out = np.empty(len(triples), dtype=np.int64)
        capi.check(self._lib.hlbg_halo_offsets(self.s.ctx, b.ctypes.data_as(C.POINTER(C.c_int32)),
                                               d.ctypes.data_as(C.POINTER(C.c_int8)),
                                               t.ctypes.data_as(C.POINTER(C.c_int16)), len(triples),
                                               out.ctypes.data_as(C.POINTER(C.c_int64))), self.s.ctx)
        return torch.from_numpy(out).cuda()

    def exchange(self) -> None:
        lib, ctx = self._lib, self.s.ctx
        for _, so, _, sbuf, _ in self.plans:
            capi.check(lib.hlbg_halo_pack_device(ctx, C.c_void_p(so.data_ptr()), so.numel(),
                                                 C.c_void_p(sbuf.data_ptr())), ctx)
        capi.check(lib.hlbg_sync(ctx), ctx)
        capi.check(lib.hlbg_halo_check(ctx), ctx)
        exchange_buffers({p[0]: p[3] for p in self.plans}, {p[0]: p[4] for p in self.plans}, self.group)
        for _, _, ro, _, rbuf in self.plans:
            capi.check(lib.hlbg_halo_unpack_device(ctx, C.c_void_p(ro.data_ptr()), ro.numel(),
                                                   C.c_void_p(rbuf.data_ptr())), ctx)
        capi.check(lib.hlbg_halo_check(ctx), ctx)

    def step(self, n: int = 1) -> None:
        s = self.s
        for _ in range(n):
            s.StreamAndCollide(0, s.n_sites)
            self.exchange()
            s.PostStep(0, s.n_sites)
            s.SwapOldAndNew()
