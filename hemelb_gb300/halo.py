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
