"""The multi-rank logic of bench.py on CPU with gloo, world size 2 (no GPU): the job
time is the slowest rank's, and the reference arm runs and prints on rank 0 only."""
import io
import os
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(1.0 + rank, world, "cpu")
        args = bench.argparse.Namespace(n=16, steps=1, warmup=1)
        buf = io.StringIO()
        with redirect_stdout(buf):
            bench.run_reference(args)
        dist.barrier()
        q.put((rank, slowest, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    pytest.importorskip("torch.distributed")
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict((r, (s, out)) for r, s, out in (q.get(timeout=300) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][0] == 2.0 and res[1][0] == 2.0  # both ranks see the slowest rank's time
    assert '"impl": "reference"' in res[0][1]       # rank 0 prints the reference line
    assert res[1][1] == ""                          # the other rank exits without work
