"""The N-GPU bench path on CPU: two gloo ranks run bench._job_value as the
torchrun ranks do (max time over ranks, units of all ranks), with rank and
world read from the environment by bench._dist."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, local = bench._dist()
    ms, value = bench._job_value(10.0 + 5.0 * rank, 1e9, 5, w, dist, device="cpu")
    q.put((rank, r, w, local, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_all_units():
    import torch.multiprocessing as mp
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
    for rank, r, w, local, ms, value in out:
        assert (r, w, local) == (rank, 2, rank)
        assert ms == 15.0                              # the slower rank
        assert value == pytest.approx(2 * 1e9 * 5 / 15e-3)


def test_one_process_needs_no_group():
    import bench
    ms, value = bench._job_value(20.0, 1e9, 4, 1, None)
    assert ms == 20.0 and value == pytest.approx(1e9 * 4 / 20e-3)
