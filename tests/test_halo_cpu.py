"""Multi-rank halo index maps (hlbg_halo_*), on CPU.

1. The partition: contiguous ranges of the device block order with balanced
   fluid-site counts.
2. The lists: rank r's send list to p and p's receive list from r name the same
   distributions in the same order; every received target is an owned fluid
   site; edge blocks are exactly the owned blocks that stream into ghost blocks.
3. The exchange, on gloo ranks (world size 2 and 4): each rank runs the oracle on
   its local geometry (owned + ghost blocks), sends the distributions its sites
   streamed into ghost sites (the library's transport, halo.exchange_buffers),
   scatters what it receives, then runs PostStep and swaps -- the order of lb::LBM (Code/lb/lb.hpp:176-309) around
   FieldData::SendAndReceive / CopyReceived (Code/geometry/FieldData.cc:27-49).
   After every step the owned sites equal the single-rank run bit for bit.
This is the host logic of a multi-GPU update; no GPU takes part.
"""
import os
import socket

import numpy as np
import pytest

from hemelb_gb300 import capi, cases, halo

Q = 19
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1])


def _case(kind):
    """Geometries with every link type: BFL walls, Ladd inlet, Nash outlets (TRT),
    and a pipe with SBB walls and Nash iolets (LBGK)."""
    if kind == "bifurcation":
        c = cases.bifurcation(seed=11, parent_radius=8.0, parent_length=40.0, daughter_length_factor=1.2,
                              period=200.0)
        c.params.kernel = capi.KERNEL_TRT
        return c
    return cases.pipe(radius=6.0, length=48)


def _fluid_counts(view):
    m = np.ctypeslib.as_array(view.fluid_mask, (view.n_blocks * 8,)).reshape(-1, 8)
    return np.array([sum(bin(int(w)).count("1") for w in row) for row in m])


def _zcol_order(view):
    bc = np.ctypeslib.as_array(view.block_coords, (view.n_blocks * 3,)).reshape(-1, 3)

    def key(c):
        m = 0
        for k in range(16):
            m |= ((int(c[0]) >> k) & 1) << (3 * k + 2)
            m |= ((int(c[1]) >> k) & 1) << (3 * k + 1)
        return (m << 16) | int(c[2])

    return np.array(sorted(range(len(bc)), key=lambda b: key(bc[b])))


@pytest.mark.parametrize("n_ranks", [1, 2, 3, 4, 7])
def test_partition_is_contiguous_and_balanced(n_ranks):
    c = _case("bifurcation")
    v = c.geometry.view
    ranks = halo.partition(v, n_ranks)
    order = _zcol_order(v)
    along = ranks[order]
    assert np.all(np.diff(along) >= 0) and along[0] == 0 and along[-1] == n_ranks - 1
    counts = _fluid_counts(v)
    per = np.bincount(ranks, weights=counts, minlength=n_ranks)
    assert per.sum() == counts.sum()
    assert np.abs(per - counts.sum() / n_ranks).max() <= counts.max()


def _all_halos(c, n_ranks):
    v = c.geometry.view
    ranks = halo.partition(v, n_ranks)
    return ranks, [halo.Halo(v, ranks, n_ranks, r) for r in range(n_ranks)]


@pytest.mark.parametrize("kind", ["bifurcation", "pipe"])
@pytest.mark.parametrize("n_ranks", [2, 4])
def test_send_and_receive_lists_pair_up(kind, n_ranks):
    c = _case(kind)
    ranks, hs = _all_halos(c, n_ranks)
    v = c.geometry.view
    fluid = np.ctypeslib.as_array(v.fluid_mask, (v.n_blocks * 8,)).reshape(-1, 8)
    total = 0
    for h in hs:
        owned = set(h.block_source[: h.n_owned].tolist())
        assert owned == set(np.nonzero(ranks == h.rank)[0].tolist())
        assert all(ranks[b] != h.rank for b in h.block_source[h.n_owned:])
        for ex in h.exchanges:
            peer = hs[ex.peer]
            back = [e for e in peer.exchanges if e.peer == h.rank]
            assert len(back) == 1
            # same distributions, same order, in the input geometry's terms
            assert np.array_equal(h.global_keys(ex.send), peer.global_keys(back[0].recv))
            assert np.array_equal(h.global_keys(ex.recv), peer.global_keys(back[0].send))
            # sends target ghost blocks owned by the peer; receives own fluid sites
            assert np.all(ex.send[:, 0] >= h.n_owned)
            assert np.all(ranks[h.block_source[ex.send[:, 0]]] == ex.peer)
            assert np.all(ex.recv[:, 0] < h.n_owned)
            for b, s in zip(h.block_source[ex.recv[:, 0]], ex.recv[:, 2]):
                assert (int(fluid[b, s >> 6]) >> int(s & 63)) & 1
            total += len(ex.send)
            # the upstream site of every sent distribution is an owned site of an
            # edge block; no mid block streams into a ghost block
            up = h.site_coords(ex.send) - np.stack([CX, CY, CZ], axis=1)[ex.send[:, 1]]
            up_block = {tuple(x) for x in (up // 8).tolist()}
            edge_blocks = {tuple(x) for x in h.block_coords[: h.n_owned][h.edge.astype(bool)].tolist()}
            assert up_block <= edge_blocks
    assert total > 0


def test_rejects_bad_arguments():
    c = _case("pipe")
    v = c.geometry.view
    ranks = halo.partition(v, 2)
    with pytest.raises(capi.HlbgError):
        halo.Halo(v, ranks, 2, 2)
    bad = ranks.copy()
    bad[0] = 5
    with pytest.raises(capi.HlbgError, match="rank out of range"):
        halo.Halo(v, bad, 2, 0)


# ---- the exchange on gloo ranks ---------------------------------------------------

def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _site_index(o):
    coords = o.arrays()["coords"]
    return {tuple(x): i for i, x in enumerate(coords.tolist())}


def _flat(h, triples, index):
    keys = h.site_coords(triples)
    return np.array([index[tuple(k)] * Q + d for k, d in zip(keys.tolist(), triples[:, 1])], dtype=np.int64)


def _rank_worker(rank, world, port, kind, steps, out):
    import torch
    import torch.distributed as dist
    from oracle.oracle import OracleLBM
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        c = _case(kind)
        ranks = halo.partition(c.geometry.view, world)
        h = halo.Halo(c.geometry.view, ranks, world, rank)
        o = OracleLBM(h.view, c.params, c.inlets, c.outlets)
        o.set_equilibrium()
        index = _site_index(o)
        plans = [(ex.peer, _flat(h, ex.send, index), _flat(h, ex.recv, index)) for ex in h.exchanges]
        for _ in range(steps):
            o.stream_and_collide(0, o.n)
            send = {peer: torch.from_numpy(o.f_new[si].copy()) for peer, si, _ in plans}
            recv = {peer: torch.empty(len(ri), dtype=torch.float64) for peer, _, ri in plans}
            halo.exchange_buffers(send, recv)  # the library's transport
            for peer, _, ri in plans:
                o.f_new[ri] = recv[peer].numpy()
            o.post_step(0, o.n)
            o.swap()
        # owned sites, keyed by coordinates
        coords = o.arrays()["coords"]
        owned_blocks = {tuple(x) for x in h.block_coords[: h.n_owned].tolist()}
        mine = np.array([tuple(x) in owned_blocks for x in (coords // 8).tolist()])
        out.put((rank, coords[mine].copy(), o.fold()[mine].copy(), o.fnew()[mine].copy()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind,world", [("bifurcation", 2), ("bifurcation", 4), ("pipe", 4)])
def test_partitioned_steps_equal_single_rank_bit_for_bit(kind, world):
    import torch.multiprocessing as mp
    from oracle.oracle import OracleLBM
    steps = 12
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_worker, args=(r, world, port, kind, steps, q)) for r in range(world)]
    for p in procs:
        p.start()
    parts = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    c = _case(kind)
    o = OracleLBM(c.geometry.view, c.params, c.inlets, c.outlets)
    o.set_equilibrium()
    o.step(steps)
    index = _site_index(o)
    seen = np.zeros(o.n, dtype=int)
    for _, coords, fold, fnew in parts:
        idx = np.array([index[tuple(x)] for x in coords.tolist()])
        seen[idx] += 1
        assert np.array_equal(fold, o.fold()[idx])
        assert np.array_equal(fnew, o.fnew()[idx])
    assert np.all(seen == 1)  # every site owned by exactly one rank
