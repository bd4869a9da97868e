"""The multi-process host logic of bench.py on CPU: world_size 2 with the gloo backend.

Every rank runs its own replica (the path has no exchange step), the ranks meet at barriers
around the timed region, and rank 0 reports the slowest rank's time."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        slowest = d.max(float(rank + 1) * 0.5)  # rank r pretends to take (r + 1)/2 s
        d.barrier()
        q.put((rank, d.world, slowest))
    finally:
        d.close()


@pytest.mark.timeout(120)
def test_two_rank_max_and_barrier():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=90) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert out == [(0, 2, 1.0), (1, 2, 1.0)]


def test_reference_arm_other_ranks_exit_quietly(monkeypatch, capsys):
    """Under torchrun the reference arm runs on rank 0 only; other ranks print nothing."""
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1",
                                      "--warmup", "3"])
    bench.main()
    assert capsys.readouterr().out == ""
