"""Multi-process host logic of `bench.py --gpus N` ("replicas only": independent replicas,
no collective on the data path): the whole-job rate is every rank's interactions over the
slowest rank's step time.  Two gloo ranks on CPU, rendezvous on 127.0.0.1."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, world, rank)
        value, step_max = bench.whole_job(10.0 + 5.0 * rank, 1000.0, world, dist, "cpu")
        dist.barrier()
        q.put((rank, value, step_max))
    finally:
        dist.destroy_process_group()


def test_whole_job_rate_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, step_max in got:
        assert step_max == 15.0                       # the slower rank's time
        assert value == pytest.approx(2 * 1000.0 / 15e-3)


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.whole_job(20.0, 500.0, 1) == (500.0 / 20e-3, 20.0)
