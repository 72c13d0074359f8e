"""Multi-rank host logic on CPU (gloo, world size 2): the benchmark's replica
timing (barrier, max over ranks, whole-job aggregate) and a two-rank run of the
oracle over halves of one geometry whose union equals the single-rank result
(sites are independent within a step once the push targets are known)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(dist)
    v = bench.max_over_ranks(dist, float(10 + rank))
    # each rank advances its own half of the sites of the same oracle domain
    from hemelb_gb300 import cases
    from oracle.oracle import OracleLBM
    c = cases.pipe(radius=4.0, length=12)
    o = OracleLBM(c.geometry.view, c.params, c.inlets, c.outlets)
    o.set_equilibrium()
    half = o.n // 2
    first, count = (0, half) if rank == 0 else (half, o.n - half)
    o.stream_and_collide(first, count)
    part = np.zeros_like(o.f_new[:-1])
    touched = np.zeros(part.shape, dtype=bool)
    # record which fNew slots this rank wrote by diffing against a marker fill
    marker = o.f_new.copy()
    o.f_new[:] = np.nan
    o.stream_and_collide(first, count)
    touched = ~np.isnan(o.f_new[:-1])
    part[touched] = o.f_new[:-1][touched]
    t = torch.from_numpy(np.where(touched, part, 0.0))
    dist.all_reduce(t)
    cnt = torch.from_numpy(touched.astype(np.int64))
    dist.all_reduce(cnt)
    if rank == 0:
        out.put((v, t.numpy().copy(), cnt.numpy().copy(), marker))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_timing_and_site_partition():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    v, summed, cnt, _ = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert v == 11.0  # max over ranks
    # no fNew slot is written by both ranks, and the union equals one full sweep
    assert cnt.max() <= 1
    from hemelb_gb300 import cases
    from oracle.oracle import OracleLBM
    c = cases.pipe(radius=4.0, length=12)
    o = OracleLBM(c.geometry.view, c.params, c.inlets, c.outlets)
    o.set_equilibrium()
    o.f_new[:] = np.nan
    o.stream_and_collide(0, o.n)
    full = o.f_new[:-1]
    written = ~np.isnan(full)
    assert np.array_equal(written, cnt.astype(bool))
    assert np.array_equal(full[written], summed[written])
