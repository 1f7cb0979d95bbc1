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


def test_slice_geometry_matches_the_c_abi_and_partitions_the_rows(sgx):
    """Frame slices: bands of `band` rows dealt round-robin; the Python
    restatement equals sgx_slice_rows / sgx_slice_row, and the slices of a
    frame cover every row exactly once."""
    from singularity_gb300 import _native as N
    from singularity_gb300 import dist as D
    lib = N.load()
    for H in (1, 7, 8, 9, 31, 100, 1081, 2160):
        for band in (0, 1, 3, 8, 16):
            for count in (1, 2, 3, 5, 8):
                rows = []
                for i in range(count + 1):
                    n = lib.sgx_slice_rows(H, band, count, i)
                    assert n == D.slice_rows(H, band, count, i)
                    idx = D.slice_row_indices(H, band, count, i)
                    assert len(idx) == n
                    assert [lib.sgx_slice_row(H, band, count, i, k) for k in range(n)] == list(idx)
                    assert lib.sgx_slice_row(H, band, count, i, n) == 2**32 - 1
                    rows += list(idx)
                assert sorted(rows) == list(range(H))
    # balance of the 4K frame over 8 GPUs: 270 bands of 8 rows, 33-34 per rank
    assert {D.slice_rows(2160, 8, 8, i) for i in range(8)} == {264, 272}


def _slice_worker(rank, world, port, q, u_bytes):
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import numpy as np
    import torch
    import torch.distributed as dist
    from oracle import pyoracle as O
    from singularity_gb300 import _native as N
    from singularity_gb300 import dist as D
    u = N.Uniforms.from_buffer_copy(u_bytes)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        band = 5
        rows = D.slice_row_indices(u.height, band, world, rank)
        pix = (rows[:, None] * u.width + np.arange(u.width)[None, :]).reshape(-1).astype(np.uint32)
        rgba, _ = O.render(u, pixels=pix, threads=2)  # this rank's rows, as the oracle computes them
        local = torch.from_numpy(rgba.reshape(len(rows), u.width, 4).copy())
        frame = D.gather_frame(local, u.height, band)
        q.put((rank, None if frame is None else frame.numpy()))
    finally:
        dist.destroy_process_group()


def test_split_frame_gathers_to_the_whole_frame_two_gloo_ranks(sgx, oracle):
    """One frame split by interleaved row bands over two gloo ranks: each
    renders its rows with the oracle, rank 0 gathers them, and the assembled
    frame equals the oracle's whole frame."""
    import torch.multiprocessing as mp
    scene = sgx.Scene(spin_a_over_M=0.94, disc_inner_M=2.0, disc_outer_M=30.0, render_supersample=2)
    u = sgx.pack_uniforms(scene, sgx.build_orbital_camera(30.0, 0.2, 0.0, 45.0), 40, 37)
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_slice_worker, args=(r, 2, port, q, u.to_bytes())) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[1] is None
    whole, _ = oracle.render(u)
    np.testing.assert_array_equal(out[0], whole)


def test_assemble_slices_with_torch_tensors():
    """dist.assemble_slices puts the rows of torch slices (the gathered NCCL
    buffers) back in frame order, as it does for numpy arrays."""
    import torch
    from singularity_gb300 import dist as D
    H, W, band, count = 37, 5, 4, 3
    frame = torch.arange(H * W * 4, dtype=torch.int32).reshape(H, W, 4)
    parts = [frame[torch.as_tensor(D.slice_row_indices(H, band, count, i))] for i in range(count)]
    assert torch.equal(D.assemble_slices(parts, H, band), frame)
    assert np.array_equal(D.assemble_slices([p.numpy() for p in parts], H, band), frame.numpy())
