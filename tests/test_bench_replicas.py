"""The bench's multi-GPU path is replicas only: one process per GPU, no data exchange, the
job's time is the slowest replica's and the throughput is the sum over ranks.  Covered here
with two gloo ranks on the CPU (no GPU): the max-over-ranks reduction, the aggregate rate and
the reference arm, which only rank 0 runs and prints."""

import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world_size, port, q, workload="polymer128"):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world_size),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    r, ws, _ = bench.dist_setup(world_size)
    slowest = bench.max_over_ranks(10.0 * (rank + 1), ws)
    rate = bench.aggregate_rate(1000.0, slowest, ws)
    args = bench.argparse.Namespace(gpus=world_size, steps=2, warmup=3, ref_side=6,
                                    workload=workload)
    out = io.StringIO()
    with redirect_stdout(out):
        bench.run_reference_arm(args)
    dist.destroy_process_group()
    q.put((rank, r, ws, slowest, rate, out.getvalue()))


@pytest.mark.timeout(300)
@pytest.mark.parametrize("workload", ["polymer128", "batched512"])
def test_replicas_two_gloo_ranks(workload):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q, workload)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for rank, r, ws, slowest, rate, out in res:
        assert r == rank and ws == 2
        assert slowest == 20.0                       # the slowest replica's time
        assert rate == pytest.approx(2 * 1000.0 / 0.020)  # units of both ranks / that time
    assert res[1][5] == ""                           # rank 1 prints nothing
    line = json.loads(res[0][5].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
