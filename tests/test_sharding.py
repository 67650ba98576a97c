"""Forests across ranks (host logic, CPU): trees partitioned by node count,
and the total log partition summed over two gloo ranks equals the
single-process sum over the whole forest."""
import os
import socket
import sys

import numpy as np

from parallel_tree_hmm_gb300 import sharding

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_partition_covers_every_tree_once_and_balances_nodes():
    rng = np.random.default_rng(3)
    counts = np.round(np.exp(rng.uniform(np.log(200), np.log(20000), 4096))).astype(int)
    for world in (1, 2, 3, 8):
        shares = sharding.partition_trees(counts, world)
        assert len(shares) == world
        flat = sorted(t for share in shares for t in share)
        assert flat == list(range(len(counts)))
        assert all(share == sorted(share) for share in shares)
        loads = [int(counts[share].sum()) for share in shares]
        # Greedy largest-first: no rank above the mean plus the largest tree.
        assert max(loads) <= counts.sum() / world + counts.max()
        assert max(loads) - min(loads) <= counts.max()


def test_partition_edge_cases():
    assert sharding.partition_trees([], 3) == [[], [], []]
    assert sharding.partition_trees([5], 2) == [[0], []]
    # Ties: equal trees alternate ranks deterministically.
    assert sharding.partition_trees([7, 7, 7, 7], 2) == [[0, 2], [1, 3]]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _forest_log_z(parents_list, K, seed):
    from oracle import bridge
    from parallel_tree_hmm_gb300 import synthetic

    values = []
    for t, parents in enumerate(parents_list):
        rng = np.random.default_rng(seed + t)
        plan = bridge.CpuPlan(parents)
        nodes = rng.random(plan.num_nodes * K) + 0.1
        edges = synthetic.stochastic_edges(rng, plan.num_edges, K, 1.0)
        values.append(bridge.log_partition(plan, K, nodes, edges))
    return values


def _worker(rank, world, port, queue):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    from parallel_tree_hmm_gb300 import synthetic

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(11)
    parents = [synthetic.random_recursive(rng, int(n)) for n in rng.integers(2, 300, 9)]
    share = sharding.partition_trees([len(p) for p in parents], world)[rank]
    # Tree t keeps its own seed whichever rank contracts it.
    local = [_forest_log_z([parents[t]], 4, 100 + t)[0] for t in share]
    total = sharding.sum_log_partitions(local, dist)
    queue.put((rank, total, share))
    dist.barrier()
    dist.destroy_process_group()


def test_sum_log_partition_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    from parallel_tree_hmm_gb300 import synthetic

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
    rng = np.random.default_rng(11)
    parents = [synthetic.random_recursive(rng, int(n)) for n in rng.integers(2, 300, 9)]
    expected = sum(_forest_log_z([parents[t]], 4, 100 + t)[0] for t in range(len(parents)))
    assert abs(results[0][1] - expected) <= 1e-9 * abs(expected)
    assert results[0][1] == results[1][1]
    assert sorted(results[0][2] + results[1][2]) == list(range(len(parents)))
