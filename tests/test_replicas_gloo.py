"""Replica sharding of the benchmark on CPU: two gloo ranks get distinct batches
and agree on the slowest rank's time (max over ranks), as the torchrun launch of
``bench.py --gpus N`` does over NCCL."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, repo)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, _ = bench._env_rank()
    seed = bench._batch_seed(r)
    specs = bench._config3_specs(seed, n=8)
    t = bench.max_over_ranks(10.0 + r, w, "cpu")
    q.put((r, seed, specs[0], t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_distinct_batches_and_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, p0, t0), (r1, s1, p1, t1) = out
    assert (r0, r1) == (0, 1)
    assert s0 == 3 and s1 != s0 and p0 != p1      # rank 0 runs the config-3 batch itself
    assert t0 == t1 == 11.0                        # both see the slowest rank
