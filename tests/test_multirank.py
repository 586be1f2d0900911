"""The N > 1 host path on CPU: world_size-2 gloo ranks score their shard with
the oracle and gather on rank 0; the result equals the single-rank batch."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist

    from mmo_gb300 import shard, synth
    from oracle import oracle as O

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s = synth.pose_batch(n_poses=10, seed=4, n_atoms=14, n_rot=3, n_pocket=150, radius=8.0)
        a, b = shard.pose_range(10, world, rank)
        E, G, st = O.score_batch(s.pocket, s.ligand, s.poses[a:b], mode=1)
        t = shard.max_over_ranks(float(rank + 1))
        out = shard.gather_to_rank0({"E": E, "G": G, "st": st}, 10, world, rank)
        if rank == 0:
            q.put((out["E"], out["G"], out["st"], t))
    finally:
        dist.destroy_process_group()


def test_pose_range_partition():
    from mmo_gb300.shard import pose_range

    for n in (0, 1, 7, 4096):
        for w in (1, 2, 3, 8):
            spans = [pose_range(n, w, r) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(w - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        pose_range(4, 2, 2)


def test_two_gloo_ranks_gather_equals_single(oracle):
    import multiprocessing as mp

    from mmo_gb300 import synth

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    E, G, st, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    s = synth.pose_batch(n_poses=10, seed=4, n_atoms=14, n_rot=3, n_pocket=150, radius=8.0)
    E1, G1, st1 = oracle.score_batch(s.pocket, s.ligand, s.poses, mode=1)
    assert np.array_equal(E, E1) and np.array_equal(G, G1) and np.array_equal(st, st1)
    assert tmax == 2.0
