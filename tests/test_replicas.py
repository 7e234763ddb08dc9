"""The multi-GPU logic (replicas only) on CPU: world_size-2 gloo ranks take
the max of their times and count the units of both ranks; body slices cover
every body exactly once."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from stonefish_gb300.replicas import max_over_ranks, shard_range, whole_job_rate  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = max_over_ranks(1.5 + rank, dist, "cpu")       # rank 1 is the slow one
    lo, hi = shard_range(10, rank, world)
    dist.barrier()
    out[rank] = (t, whole_job_rate(hi - lo, world, t), lo, hi)
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_time_and_whole_job_rate():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.5
    assert res[0][1] == pytest.approx(2 * 5 / 2.5)
    assert (res[0][2], res[0][3], res[1][2], res[1][3]) == (0, 5, 5, 10)


@pytest.mark.parametrize("n,world", [(0, 3), (1, 4), (7, 2), (4096, 8), (13, 5)])
def test_shard_range_partitions(n, world):
    seen = []
    sizes = []
    for r in range(world):
        lo, hi = shard_range(n, r, world)
        seen.extend(range(lo, hi))
        sizes.append(hi - lo)
    assert seen == list(range(n))
    assert max(sizes) - min(sizes) <= 1


def test_single_rank_is_identity():
    assert max_over_ranks(3.25) == 3.25
    assert whole_job_rate(100, 1, 2.0) == 50.0
