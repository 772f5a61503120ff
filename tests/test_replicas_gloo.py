"""World-size-2 gloo tests (CPU) of the replicas path: event sharding, the cross-rank kernel
sum and bench.py's max-over-ranks timing. Per-rank work runs on the CPU oracle."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), OMP_NUM_THREADS="2")
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from ses3d_gb300 import replicas, synth
        p = synth.make_problem("tiny", nt=20, n_events=3, seed=77)
        mine = replicas.shard_events(3, rank, world)
        # per-event "result": the final assembled vz of each event, summed over my events
        acc = np.zeros(p.n_nodes, np.float64)
        for k in mine:
            o = oracle.Oracle(p, event=k)
            o.run(20)
            acc = acc + o.get("vz").astype(np.float64)
        total = replicas.sum_over_ranks([acc])[0]
        t = replicas.max_over_ranks(1.0 + rank)
        import bench
        t2 = bench.max_over_ranks(10.0 * (rank + 1), world)
        bench.barrier(world)
        q.put((rank, mine, total, t, t2))
    finally:
        dist.destroy_process_group()


def test_shard_events_covers_all():
    from ses3d_gb300 import replicas
    for n in (1, 5, 16):
        for w in (1, 2, 3, 8):
            got = [e for r in range(w) for e in replicas.shard_events(n, r, w)]
            assert got == list(range(n))


def test_two_rank_gloo_kernel_sum_and_timing(oracle_mod):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = [q.get(timeout=600) for _ in range(2)]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    res.sort()
    assert res[0][1] == [0, 1] and res[1][1] == [2]
    # both ranks hold the same sum, equal to the single-process sum over all events
    assert np.array_equal(res[0][2], res[1][2])
    from ses3d_gb300 import synth
    p = synth.make_problem("tiny", nt=20, n_events=3, seed=77)
    ref = np.zeros(p.n_nodes)
    for k in range(3):
        o = oracle_mod.Oracle(p, event=k)
        o.run(20)
        ref += o.get("vz").astype(np.float64)
    assert np.allclose(res[0][2], ref, rtol=1e-12, atol=0)
    assert res[0][3] == res[1][3] == 2.0
    assert res[0][4] == res[1][4] == 20.0
