"""bench.py's N > 1 path (independent replicas, one per rank) on CPU with the
gloo backend, world size 2: the timing is the slowest rank's, the job value
adds up the replicas, and --impl reference runs on rank 0 only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(WORLD),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    import bench
    ws, r, _ = bench.dist_info()
    ms = bench.max_over_ranks(10.0 + 5.0 * r, ws, "cpu")
    out.put((r, ms, bench.job_value(1000, ws, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_add_up():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(WORLD)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(WORLD))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, ms, v in res:
        assert ms == 15.0
        assert v == pytest.approx(2 * 1000 / 0.015)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = type("A", (), dict(config="config2", steps=1, warmup=0, gpus=2))()
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args)
    assert buf.getvalue() == ""
