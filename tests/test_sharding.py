"""A stream split across ranks (sharding.py): work-balanced release ranges,
and on world_size 2 (gloo, CPU) each rank integrating its range as a
sub-range run and the gather, against one run of the whole stream — on the
oracle, so no GPU is needed."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from .conftest import PROG_WF


def test_balanced_ranges():
    from streamsculptor_gb300.sharding import balanced_ranges, stream_work
    n_rel, ppr, spr = 4000, 250, 2
    n_steps = n_rel * spr
    for world in (1, 2, 3, 4, 8):
        r = balanced_ranges(n_rel * ppr, ppr, spr, n_steps, world)
        assert r[0][0] == 0 and r[-1][1] == n_rel * ppr
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        assert all(p0 % ppr == 0 for p0, _ in r)
        w = np.array([stream_work(p1, ppr, spr, n_steps) - stream_work(p0, ppr, spr, n_steps) for p0, p1 in r])
        one_release = ppr * n_steps
        assert w.max() - w.min() <= 2 * one_release, world
    # the closed form is the sum of the per-particle step counts
    p = np.arange(0, 2000, 7)
    brute = [sum(n_steps - (q // ppr) * spr for q in range(pp)) for pp in p[:20]]
    assert np.array_equal(stream_work(p[:20], ppr, spr, n_steps), brute)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, ics, ppr, spr, n_steps, ranges, q):
    import torch
    import torch.distributed as dist

    from oracle import oracle
    from streamsculptor_gb300.sharding import gather_ranges
    os.environ["OMP_NUM_THREADS"] = "2"
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        p0, p1 = ranges[rank]
        model = oracle.HostModel(oracle.mw3())
        part, _, _ = oracle.stream(model, 0.0, 1.0, n_steps, ics[p0:p1], ppr, spr, first_particle=p0)
        full = gather_ranges(torch.from_numpy(part), ranges)
        q.put((rank, full.numpy()))
    finally:
        dist.destroy_process_group()


def test_sharded_stream_gloo_world_2(oracle):
    from streamsculptor_gb300.sharding import balanced_ranges
    n_rel, ppr, spr = 60, 4, 1
    n_steps = n_rel * spr
    rng = np.random.default_rng(9)
    ics = PROG_WF + rng.normal(0, 0.3, (n_rel * ppr, 6)) * np.array([1, 1, 1, 0.01, 0.01, 0.01])
    whole, _, _ = oracle.stream(oracle.HostModel(oracle.mw3()), 0.0, 1.0, n_steps, ics, ppr, spr)
    world = 2
    ranges = balanced_ranges(n_rel * ppr, ppr, spr, n_steps, world)
    assert ranges[0][1] < n_rel * ppr // 2  # the early releases carry more steps
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, ics, ppr, spr, n_steps, ranges, q))
             for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        assert np.array_equal(got[r], whole)
