"""The N>1 path of the sampler on the CPU: world_size-2 gloo ranks, as torchrun
starts them, agree on the slowest rank's time and the whole-job throughput,
and get disjoint chain seeds."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from bmagwa_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = replicas.rank_info()
        secs = 1.5 + r  # rank 1 is the slowest
        smax = replicas.max_over_ranks(secs)
        v = replicas.job_throughput(smax, steps=10, chains_per_rank=4, world=w)
        q.put((r, w, lr, smax, v, replicas.replica_seeds(r, 4)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_and_throughput():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == pytest.approx(2.5) for o in out)
    assert all(o[4] == pytest.approx(10 * 4 * 2 / 2.5) for o in out)
    seeds = out[0][5] + out[1][5]
    assert len(set(seeds)) == len(seeds)


def test_single_process_needs_no_group():
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.job_throughput(2.0, 10, 8, 1) == 40.0
    with pytest.raises(ValueError):
        replicas.job_throughput(0.0, 10, 8, 1)
