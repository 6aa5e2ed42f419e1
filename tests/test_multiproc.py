"""The N > 1 host path on CPU: two gloo ranks (127.0.0.1) shard independent
systems without overlap or loss, agree on the assignment, and reduce the
step time to its maximum over ranks; the reference arm's non-zero ranks do
no work.  No GPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from blockstructuredsolvers_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, costs, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = replicas.rank_env()
    mine = replicas.my_systems(costs, r, w)
    gathered = [None] * w
    dist.all_gather_object(gathered, mine)
    t = replicas.reduce_max(1.5 + rank)
    out.put((rank, mine, gathered, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    rng_costs = [replicas.system_cost(N, n, k) for N, n, k in
                 [(100, 16, 1), (1000, 64, 2), (17, 128, 8), (512, 32, 1), (900, 96, 4), (50, 8, 1), (2, 16, 3)]]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, rng_costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, mine0, g0, t0), (r1, mine1, g1, t1) = res
    assert g0 == g1 == [mine0, mine1]
    assert sorted(mine0 + mine1) == list(range(len(rng_costs)))
    assert t0 == t1 == 2.5
    loads = [sum(rng_costs[i] for i in m) for m in (mine0, mine1)]
    assert max(loads) <= 4.0 / 3.0 * max(sum(rng_costs) / 2, max(rng_costs)) + 1e-6


def test_shard_systems_properties():
    costs = [replicas.system_cost(N, n) for N, n in [(16 + 37 * i % 1000, [16, 32, 48, 64, 96, 128][i % 6])
                                                      for i in range(2048)]]
    for world in (1, 2, 3, 8):
        sh = replicas.shard_systems(costs, world)
        assert sorted(i for s in sh for i in s) == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in sh]
        assert max(loads) <= 4.0 / 3.0 * max(sum(costs) / world, max(costs))
        assert sh == replicas.shard_systems(costs, world)  # deterministic


def test_reference_arm_nonzero_rank_does_nothing(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        warmup, steps, gpus = 1, 1, 2
    bench.run_reference(A())
    assert capsys.readouterr().out == ""
