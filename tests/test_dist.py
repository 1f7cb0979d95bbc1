"""Multi-GPU host logic on CPU: the cost split of a batch's views across ranks
and the whole-job aggregation, with two gloo processes (127.0.0.1)."""

from __future__ import annotations

import socket

import numpy as np
import pytest


def test_split_by_cost_covers_and_balances():
    from singularity_gb300 import dist as D
    rng = np.random.default_rng(0)
    # the 64 batched views' shapes: side in {128..1024}, spp in [1, 64]
    sides = rng.integers(2, 17, 64) * 64
    spp = rng.integers(1, 65, 64)
    costs = [D.view_cost(s, s, p) for s, p in zip(sides, spp)]
    for world in (1, 2, 4, 8):
        parts = D.split_by_cost(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        assert all(p == sorted(p) for p in parts)
        assert D.imbalance(costs, parts) < (1.0001 if world == 1 else 1.25)
    assert D.split_by_cost(costs, 4) == D.split_by_cost(costs, 4)  # deterministic
    assert D.split_by_cost([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        D.split_by_cost(costs, 0)


def test_view_azimuth():
    from singularity_gb300 import dist as D
    assert D.view_azimuth(0, 1) == 0.0
    assert abs(D.view_azimuth(1, 4) - np.pi / 2) < 1e-12


def _worker(rank, world, port, q):
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    from singularity_gb300 import dist as D
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r traced (r + 1) * 1e6 rays in (r + 1) * 0.5 s
        rate = D.whole_job_rate((rank + 1) * 1e6, (rank + 1) * 0.5)
        mx = D.max_over_ranks(float(rank))
        sm = D.sum_over_ranks(1.0)
        q.put((rank, rate, mx, sm, D.env_rank()))
    finally:
        dist.destroy_process_group()


def test_whole_job_aggregation_two_gloo_ranks():
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, mx, sm, env in out:
        assert rate == pytest.approx(3e6 / 1.0)  # (1e6 + 2e6) rays / the slower rank's 1.0 s
        assert mx == 1.0 and sm == 2.0
        assert env[0] == rank and env[1] == 2


def test_single_process_fallbacks():
    from singularity_gb300 import dist as D
    assert D.max_over_ranks(3.5) == 3.5 and D.sum_over_ranks(2.0) == 2.0
    assert D.whole_job_rate(10.0, 2.0) == 5.0
