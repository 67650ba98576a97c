"""Multi-process host logic on CPU (gloo, world size 2): the benchmark's
max-over-ranks timing reduction and per-rank forest replicas, and the
`--impl reference` leg under torchrun, where only rank 0 runs and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, queue):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slowest = bench.reduce_max(10.0 + rank, dist)
    forest = bench.Forest(6, 4, bench.rank_seed(0, rank))
    queue.put((rank, slowest, forest.total_nodes))
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_max_and_replicas_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    context = mp.get_context("spawn")
    queue = context.Queue()
    port = _free_port()
    processes = [context.Process(target=_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in processes:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in processes)
    for p in processes:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in results] == [11.0, 11.0]
    assert results[0][2] != results[1][2]  # distinct replicas


def test_reference_leg_under_torchrun_prints_one_line():
    port = _free_port()
    command = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
               "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
               str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--trees", "12",
               "--steps", "1", "--warmup", "0", "--cpu-sample-nodes", "20000"]
    result = subprocess.run(command, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert result.returncode == 0, result.stderr[-2000:]
    lines = [line for line in result.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    record = json.loads(lines[0])
    assert record["impl"] == "reference" and record["value"] > 0
    assert record["e2e"]["h2d_bytes_per_step"] == 0
