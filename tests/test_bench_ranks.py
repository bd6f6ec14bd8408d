"""The multi-rank host logic of bench.py on CPU: two gloo ranks (one process each, as
torchrun starts them) agree on the slowest rank's time, the whole-job value counts every
rank's replica, and the reference arm runs on rank 0 only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        slow = bench.max_over_ranks(10.0 + 5.0 * rank, w, device="cpu")
        value = bench.aggregate_value(1000, 20, w, slow)
        # The reference arm: ranks other than 0 return at once and print nothing.
        printed = ""
        if rank != 0:
            buf = io.StringIO()
            with redirect_stdout(buf):
                bench.run_reference(type("A", (), {"workload": "grid1025", "steps": 1, "warmup": 3, "gpus": w})())
            printed = buf.getvalue()
        dist.barrier()
        out.put((rank, r, w, local, slow, value, printed))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    torch_mp = pytest.importorskip("torch.multiprocessing")
    ctx = torch_mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, w, local, slow, value, printed in got:
        assert (r, w, local) == (rank, 2, rank)
        assert slow == 15.0  # the slowest rank's time, on every rank
        assert value == pytest.approx(1000 * 20 * 2 / 0.015)  # both replicas over the slowest time
        assert printed == ""
