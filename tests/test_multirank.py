"""The N-GPU path of bench.py on CPU: ranks are replicas (probes are
independent, no data-path collective); the job's time is the slowest rank's
(an all-reduce MAX over gloo here, NCCL on GPUs) and its rate counts every
rank's probes; under torchrun only rank 0 runs the reference arm."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    times = [10.0, 25.0, 17.5, 3.0]
    mx = bench.max_over_ranks(times[rank], dist, "cpu")
    rate = bench.whole_job_rate(4096 * 20, world, mx)
    ref = bench.run_reference(type("A", (), {"ref_probes": 8, "warmup": 0, "steps": 1, "gpus": world})(), rank)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, mx, rate, ref is None))


@pytest.mark.parametrize("world", [2, 4])
def test_replicas_time_is_the_slowest_rank(world):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = max([10.0, 25.0, 17.5, 3.0][:world])
    for rank, mx, rate, ref_none in res:
        assert mx == slowest
        assert rate == pytest.approx(world * 4096 * 20 / (slowest / 1e3))
        assert ref_none == (rank != 0)  # the reference arm runs on rank 0 only
