"""Benchmark: batched posterior marginals (log Z + node/edge marginals, the
gradient of log Z) over an uneven forest, on GB300.

Workloads (--workload): `forest` (default, below); `gw`: Galton-Watson
forest, K = 8, MAP + posterior sampling; `dense`: dense lognormal factors,
spine-heavy trees at K = 64/128 on the tensor-core engine, or with --shape
recursive --states 20 --tree-nodes 5000 the differentiation workload;
`sites`: the reference's batch API on one binary tree with many sites
(phylogenetic-style, the shared-topology layout). The forest and gw
workloads autotune the launch (thmm_autotune) before timing; the timed device
steps replay a CUDA graph (thmm_enqueue); prepared calls overlap copies and
kernels in stripes.

Workload (one step = one categorical kFactors call over the whole forest):
4096 trees with node counts log-uniform in [200, 20000], half random recursive
trees, half caterpillars; K = 4 states (--states 20 for the larger variant);
row-stochastic Dirichlet(0.5) edge factors, every leaf observed with a byte
uniform over K categories, Dirichlet(1) root factor and emission rows. Inputs
are seeded synthetic data. The edge factors of one step (1.1 GB at K = 4)
exceed the 129 MB L2, so no flush is needed between timed steps.

Reported:
  value       device-resident throughput, tree nodes/s: the persistent kernel
              re-run on inputs already in HBM, CUDA events on the workspace
              stream.
  e2e         the same metric through the C ABI prepared call with pinned host
              buffers: upload of the step's edge/root/emission factors, kernel,
              download of log Z and all node and edge marginals.
  roofline    algorithmic bytes per launch / launch time against the measured
              HBM copy bandwidth.
  cpu_baseline  the oracle port of the reference FP64 CPU path on a bounded
              sample of the same forest, all host cores.
  config.plain_fp64_*  the same kernel with FP64 arithmetic (the plain FP64
              form) on the same inputs.

`--impl reference` times the reference CPU algorithm (oracle port, FP64, all
host cores) on the same workload instead.
"""
from __future__ import annotations

import argparse
import concurrent.futures
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "tree-nodes/s for logZ+marginals+grad"
UNIT = "nodes/s"


def parse_args():
    parser = argparse.ArgumentParser()
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=100)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=["ours", "reference"], default="ours")
    parser.add_argument("--states", type=int, default=4)
    parser.add_argument("--trees", type=int, default=4096)
    parser.add_argument("--seed", type=int, default=0)
    parser.add_argument("--e2e-steps", type=int, default=None)
    parser.add_argument("--cpu-sample-nodes", type=int, default=20_000_000)
    parser.add_argument("--windows", type=int, default=1,
                        help="dense workload: stream the trees through the device in this "
                             "many windows, inputs drawn on the GPU (full-size runs)")
    parser.add_argument("--precision", choices=["tf32x3", "bf16"], default="tf32x3",
                        help="dense workload above 32 states: tensor-core product tier")
    parser.add_argument("--schedule", choices=["phases", "teams"], default="phases",
                        help="dense workload above 32 states: every round of every tree "
                             "grid-wide (phases) or one CTA per tree (teams)")
    parser.add_argument("--phase-rounds", type=int, default=None,
                        help="forest workload with --no-autotune: grid-wide rounds of the "
                             "phase schedule (0 automatic)")
    parser.add_argument("--partition", action="store_true",
                        help="forest workload under torchrun: the ranks share ONE forest, "
                             "trees partitioned by node count (strong scaling), instead of "
                             "one replica per rank (weak scaling)")
    parser.add_argument("--no-autotune", action="store_true",
                        help="forest and gw workloads: keep the default launch tuning "
                             "(a short run, e.g. under a profiler)")
    parser.add_argument("--check-trees", type=int, default=16,
                        help="gw workload: trees checked against the oracle")
    parser.add_argument("--sites", type=int, default=4096,
                        help="sites workload: batch items (sites) sharing the tree")
    parser.add_argument("--workload", choices=["forest", "gw", "dense", "sites"],
                        default="forest",
                        help="forest: uneven forest, marginals (default); gw: "
                             "Galton-Watson forest, MAP + posterior sampling; dense: "
                             "spine-heavy trees, K = 64 or 128, tensor-core marginals; "
                             "sites: the batch API on one binary tree with many sites")
    parser.add_argument("--tree-nodes", type=int, default=None,
                        help="dense workload: nodes per tree; sites workload: nodes of "
                             "the tree (default 2001)")
    parser.add_argument("--shape", choices=["spine-heavy", "recursive"], default="spine-heavy",
                        help="dense workload: tree shape")
    parser.add_argument("--edge-sigma", type=float, default=2.0,
                        help="dense workload: edge factors lognormal(0, sigma)")
    parser.add_argument("--zero-fraction", type=float, default=0.05,
                        help="dense workload: fraction of exactly zero edge entries")
    args = parser.parse_args()
    if args.workload == "gw":
        if args.trees == 4096:
            args.trees = 1024
        if args.states == 4:
            args.states = 8
    if args.workload == "dense":
        if args.trees == 4096:
            args.trees = 256
        if args.states == 4:
            args.states = 64
        if args.tree_nodes is None:
            args.tree_nodes = 2000 if args.states <= 64 else 500
    return args


# ------------------------------------------------------------------ workload
class Forest:
    def __init__(self, trees: int, states: int, seed: int):
        from parallel_tree_hmm_gb300 import synthetic

        rng = np.random.default_rng(seed)
        sizes = np.exp(rng.uniform(math.log(200), math.log(20000), size=trees))
        sizes = np.maximum(2, np.round(sizes).astype(np.int64))
        self.parents = []
        for index, n in enumerate(sizes):
            if index % 2 == 0:
                self.parents.append(synthetic.random_recursive(rng, int(n)))
            else:
                self.parents.append(synthetic.caterpillar(int(n)))
        self.states = states
        self.observed = [synthetic.leaves(p) for p in self.parents]
        self.num_nodes = np.array([len(p) for p in self.parents], dtype=np.int64)
        self.total_nodes = int(self.num_nodes.sum())
        self.total_edges = int((self.num_nodes - 1).sum())
        self.total_observed = int(sum(len(o) for o in self.observed))
        self.rng = rng
        self.cpu_plans = {}  # tree -> oracle planner plan (CPU legs)

    def take(self, trees):
        """The forest restricted to `trees` (indices, in order)."""
        self.parents = [self.parents[t] for t in trees]
        self.observed = [self.observed[t] for t in trees]
        self.num_nodes = np.array([len(p) for p in self.parents], dtype=np.int64)
        self.total_nodes = int(self.num_nodes.sum())
        self.total_edges = int((self.num_nodes - 1).sum())
        self.total_observed = int(sum(len(o) for o in self.observed))
        self.cpu_plans = {}
        return self

    def factors(self, seed: int):
        """One kFactors draw: root, emission and edge factors (float32)."""
        from parallel_tree_hmm_gb300 import synthetic

        rng = np.random.default_rng(seed)
        K = self.states
        root = synthetic.dirichlet_rows(rng, 1, K, 1.0, np.float32).ravel()
        emission = synthetic.dirichlet_rows(rng, K, K, 1.0, np.float32).ravel()
        g = rng.standard_gamma(0.5, size=(self.total_edges * K, K), dtype=np.float32)
        g /= g.sum(axis=1, keepdims=True)
        np.nan_to_num(g, copy=False, nan=1.0 / K)
        return root, emission, g.ravel()

    def observations(self):
        return self.rng.integers(0, self.states, size=self.total_observed,
                                 dtype=np.uint8)

    def algorithmic_bytes(self, scalar_bytes: int = 4) -> int:
        """Compulsory bytes of one marginal launch: edge factors in, one byte
        per observation in, node marginals, edge marginals and log Z out."""
        K = self.states
        return (self.total_edges * K * K * scalar_bytes * 2
                + self.total_observed
                + self.total_nodes * K * scalar_bytes
                + len(self.parents) * scalar_bytes
                + (K + K * K) * scalar_bytes)


# -------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.process = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.process = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.process = None
        return self

    def _read(self):
        for line in self.process.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.process is not None:
            self.process.terminate()
            try:
                self.process.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.process.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)

    def summary(self):
        sm, max_sm, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                max_sm = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"],
                    "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max_sm,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU leg
def cpu_baseline(forest: Forest, root, emission, edges, observations, sample_nodes):
    """Reference FP64 CPU marginals (oracle port) on the first trees of the
    forest whose node count reaches `sample_nodes`, over all host cores. Plans
    come from the oracle's own planner library, so this leg loads no product
    code."""
    from oracle import bridge

    K = forest.states
    edge_offsets = np.concatenate([[0], np.cumsum(forest.num_nodes - 1)])
    obs_offsets = np.concatenate([[0], np.cumsum([len(o) for o in forest.observed])])
    chosen, nodes_total = [], 0
    for t in range(len(forest.parents)):
        chosen.append(t)
        nodes_total += int(forest.num_nodes[t])
        if nodes_total >= sample_nodes:
            break
    emission64 = emission.astype(np.float64).reshape(K, K)
    root64 = root.astype(np.float64)
    jobs = []
    for t in chosen:
        parents = forest.parents[t]
        dense = np.ones((len(parents), K))
        dense[0] = root64
        obs = observations[obs_offsets[t]:obs_offsets[t + 1]]
        dense[forest.observed[t]] *= emission64[obs]
        tree_edges = edges[edge_offsets[t] * K * K:edge_offsets[t + 1] * K * K]
        if t not in forest.cpu_plans:
            forest.cpu_plans[t] = bridge.CpuPlan(parents)
        jobs.append((forest.cpu_plans[t], dense.ravel(), tree_edges.astype(np.float64)))
    cores = os.cpu_count() or 1

    def run(job):
        plan, dense, tree_edges = job
        return bridge.marginals(plan, K, dense, tree_edges)[0]

    start = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(max_workers=cores) as pool:
        list(pool.map(run, jobs))
    elapsed = time.perf_counter() - start
    return {"value": nodes_total / elapsed, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"first {len(chosen)} trees ({nodes_total} nodes) of the forest, "
                      f"FP64 log-domain marginals, {elapsed:.2f} s"}


# ------------------------------------------------------------------- main
def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist  # noqa: F811

        if args.impl == "ours":
            torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")

    if args.workload == "gw":
        run_gw(args, rank, world, local_rank, dist)
    elif args.workload == "dense":
        run_dense(args, rank, world, local_rank, dist)
    elif args.workload == "sites":
        run_sites(args, rank, world, local_rank, dist)
    elif args.impl == "reference":
        run_reference(args, rank, world, dist)
    else:
        run_ours(args, rank, world, local_rank, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def reduce_max(value, dist):
    """Maximum of `value` over all ranks (the slowest rank's time)."""
    if dist is None:
        return value
    import torch

    on_gpu = dist.get_backend() == "nccl"
    tensor = torch.tensor([value], dtype=torch.float64, device="cuda" if on_gpu else "cpu")
    dist.all_reduce(tensor, op=dist.ReduceOp.MAX)
    return float(tensor.item())


def reduce_sum(value, dist):
    """Sum of `value` over all ranks."""
    if dist is None:
        return value
    import torch

    on_gpu = dist.get_backend() == "nccl"
    tensor = torch.tensor([float(value)], dtype=torch.float64,
                          device="cuda" if on_gpu else "cpu")
    dist.all_reduce(tensor, op=dist.ReduceOp.SUM)
    return float(tensor.item())


def rank_seed(seed: int, rank: int) -> int:
    """Each rank contracts its own forest replica (weak scaling, no
    collective on the data path); replicas differ only by seed."""
    return seed + 1000 * rank


def run_reference(args, rank, world, dist):
    if rank != 0:
        return
    forest = Forest(args.trees, args.states, args.seed)
    root, emission, edges = forest.factors(args.seed + 1)
    observations = forest.observations()
    # Every step contracts the whole forest (the same workload as the GPU
    # arm), about a second on the GPU host's cores.
    sample = forest.total_nodes
    for _ in range(args.warmup):
        cpu_baseline(forest, root, emission, edges, observations, sample // 8)
    values = []
    for _ in range(args.steps):
        values.append(cpu_baseline(forest, root, emission, edges, observations, sample))
    value = statistics.median(v["value"] for v in values)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, forest),
        "cpu_baseline": {**values[-1], "value": value},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args, forest):
    return {
        "workload": (f"uneven forest: {len(forest.parents)} trees, nodes log-uniform "
                     f"[200, 20000], half random recursive / half caterpillar, "
                     f"K={forest.states}, categorical leaves, kFactors posterior marginals"),
        "trees": len(forest.parents), "nodes_per_rank": forest.total_nodes,
        "edges_per_rank": forest.total_edges, "states": forest.states,
        "seed": args.seed, "parallelism": f"replicas of the forest per GPU x{args.gpus}",
        "l2": "inputs larger than L2 (edge factors of one step > 129 MB)",
    }


def run_ours(args, rank, world, local_rank, dist):
    import torch

    import parallel_tree_hmm_gb300 as thmm

    device = local_rank
    torch.cuda.set_device(device)
    if args.partition:
        from parallel_tree_hmm_gb300 import sharding

        forest = Forest(args.trees, args.states, args.seed)
        forest.take(sharding.partition_trees(forest.num_nodes, world)[rank])
    else:
        forest = Forest(args.trees, args.states, rank_seed(args.seed, rank))
    K = forest.states
    setup_start = time.perf_counter()
    plans = thmm.Plan.many(forest.parents)
    plan_s = time.perf_counter() - setup_start
    factor_sets = [forest.factors(rank_seed(args.seed, rank) + 1 + i) for i in range(2)]
    observations = forest.observations()

    def reserve(compute):
        ws = thmm.Workspace()
        ws.reserve_forest_categorical(plans, K, K, forest.observed, device, kind="marginals",
                                      scalar=np.float32, compute=compute)
        return ws

    def stage(ws, factors):
        staged = ws.categorical_inputs()
        root, emission, edges = factors
        staged.root_potential[:] = root
        staged.emission_potentials[:] = emission
        staged.edge_potentials[:] = edges
        return staged

    reserve_start = time.perf_counter()
    ws = reserve(np.float32)
    reserve_s = time.perf_counter() - reserve_start
    staged = stage(ws, factor_sets[0])
    staged.observations[:] = observations
    first = ws.posterior_marginals_prepared(staged, thmm.CategoricalInputUpdate.kAll)
    if not np.all(np.isfinite(first.log_partitions)):
        raise RuntimeError("non-finite log partition in the benchmark workload")
    log_z_reference = first.log_partitions.copy()
    node_sum = first.nodes.reshape(-1, K).sum(axis=1)
    normalisation_error = float(np.max(np.abs(node_sum - 1.0)))

    if args.no_autotune and args.phase_rounds is not None:
        ws.set_tuning(ws.tuning["team_threshold"], phase_rounds=args.phase_rounds)
    tuning = ws.tuning if args.no_autotune else ws.autotune(4, repeats=3)

    def device_time(workspace, steps, warmup, sampler=None):
        ext = torch.cuda.ExternalStream(workspace.stream, device=device)
        for _ in range(warmup):
            workspace.enqueue(4)
        torch.cuda.synchronize(device)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(device)
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record(ext)
        nodes = 0
        for _ in range(steps):
            nodes += workspace.enqueue(4)
        stop.record(ext)
        stop.synchronize()
        torch.cuda.synchronize(device)
        if dist is not None:
            dist.barrier()
        return start.elapsed_time(stop), nodes

    sampler = ClockSampler(device)
    with sampler:
        elapsed_ms, nodes_done = device_time(ws, args.steps, args.warmup)
    launches_per_step = ws.launches
    elapsed_ms = reduce_max(elapsed_ms, dist)
    launch_ms = elapsed_ms / args.steps
    # Replicas: every rank contracts its own forest of the same size; a
    # partitioned forest: the ranks' shares add up to one forest.
    all_nodes = (int(reduce_sum(forest.total_nodes, dist)) if args.partition
                 else forest.total_nodes * world)
    value = (reduce_sum(nodes_done, dist) if args.partition else nodes_done * world) / (
        elapsed_ms / 1e3)

    # Plain FP64 arithmetic on the same inputs.
    ws64 = reserve(np.float64)
    staged64 = stage(ws64, factor_sets[0])
    staged64.observations[:] = observations
    plain = ws64.posterior_marginals_prepared(staged64, thmm.CategoricalInputUpdate.kAll)
    plain_tuning = ws64.tuning if args.no_autotune else ws64.autotune(4, repeats=2)
    plain_logz_diff = float(np.max(np.abs(plain.log_partitions.astype(np.float64)
                                          - log_z_reference.astype(np.float64))
                                   / np.maximum(1.0, np.abs(plain.log_partitions))))
    plain_steps = max(2, args.steps // 4)
    plain_ms, plain_nodes = device_time(ws64, plain_steps, 1)
    plain_value = (reduce_sum(plain_nodes, dist) if args.partition else plain_nodes * world) / (
        reduce_max(plain_ms, dist) / 1e3)
    del ws64, staged64, plain

    # End to end through the prepared call: pinned staging -> H2D -> kernel -> D2H.
    e2e_steps = args.e2e_steps or max(3, min(args.steps, 10))
    for i in range(args.warmup):
        stage(ws, factor_sets[i % 2])
        ws.posterior_marginals_prepared(staged, thmm.CategoricalInputUpdate.kFactors)
    e2e_total = 0.0
    api_kernel_ms, api_upload_ms, api_download_ms, api_wall_ms = [], [], [], []
    call_ms = []
    for i in range(e2e_steps):
        stage(ws, factor_sets[i % 2])
        torch.cuda.synchronize(device)
        if dist is not None:
            dist.barrier()
        begin = time.perf_counter()
        result = ws.posterior_marginals_prepared(staged, thmm.CategoricalInputUpdate.kFactors)
        call_ms.append(1e3 * (time.perf_counter() - begin))
        e2e_total += call_ms[-1] / 1e3
        api_kernel_ms.append(result.timings.kernel_ms)
        api_upload_ms.append(result.timings.upload_ms)
        api_download_ms.append(result.timings.download_ms)
        api_wall_ms.append(result.timings.wall_ms)
    e2e_total = reduce_max(e2e_total, dist)
    e2e_value = all_nodes * e2e_steps / e2e_total
    S = 4
    h2d = forest.total_edges * K * K * S + (K + K * K) * S
    d2h = len(plans) * S + forest.total_nodes * K * S + forest.total_edges * K * K * S + 16

    algorithmic = forest.algorithmic_bytes()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = algorithmic / (launch_ms / 1e3) / 1e9
    traffic = None
    traffic_file = ROOT / "profiles" / "engine_traffic.json"
    if traffic_file.exists():
        info = json.loads(traffic_file.read_text())
        key = f"K{K}"
        if key in info:
            traffic = info[key]["bytes_per_node"] * forest.total_nodes

    partition = {}
    if args.partition:
        from parallel_tree_hmm_gb300 import sharding

        partition = {"parallelism": f"one forest partitioned by node count over {world} GPUs",
                     "trees": args.trees, "nodes_all_ranks": all_nodes,
                     "nodes_this_rank": forest.total_nodes,
                     "sum_log_partition_all_ranks": sharding.sum_log_partitions(
                         log_z_reference, dist)}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": launch_ms,
        "higher_is_better": True, "scaling": "strong" if args.partition else "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {**workload_config(args, forest), **partition,
                   "plain_fp64_nodes_per_s": plain_value,
                   "chosen_over_plain_fp64": value / plain_value,
                   "plain_fp64_log_z_rel_diff": plain_logz_diff,
                   "tuning": tuning, "plain_fp64_tuning": plain_tuning,
                   "host_plan_s": plan_s, "reserve_s": reserve_s,
                   "node_marginal_normalisation_error": normalisation_error},
        "roofline": {"bound": "hbm", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": "measured" if peaks else "fallback",
                     "traffic": traffic,
                     "algorithmic_bytes_per_launch": algorithmic},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "api_kernel_ms_median": statistics.median(api_kernel_ms),
                "api_upload_ms_median": statistics.median(api_upload_ms),
                "api_download_ms_median": statistics.median(api_download_ms),
                "api_wall_ms_median": statistics.median(api_wall_ms),
                "call_ms_median": statistics.median(call_ms),
                "call_ms": [round(v, 3) for v in call_ms],
                "api_wall_ms": [round(v, 3) for v in api_wall_ms],
                "api_upload_ms": [round(v, 3) for v in api_upload_ms],
                "api_kernel_ms": [round(v, 3) for v in api_kernel_ms],
                "api_download_ms": [round(v, 3) for v in api_download_ms],
                "launches_per_call": ws.launches},
        "gpu_launches": args.steps * launches_per_step,
        "clocks": sampler.summary(),
    }
    if rank == 0 and world == 1 and args.cpu_sample_nodes > 0:
        root, emission, edges = factor_sets[0]
        line["cpu_baseline"] = cpu_baseline(forest, root, emission, edges, observations,
                                            args.cpu_sample_nodes)
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------- MAP + sampling workload
class GaltonWatsonForest:
    """Poisson(2) Galton-Watson trees of 1,000-50,000 nodes (grown breadth
    first to a uniform size cap), K states, byte observations on the leaves
    with a Dirichlet(2) emission table, Dirichlet(0.3) edge rows, Dirichlet(1)
    root factor and one U[0,1) variate per node."""

    # Above this many edge rows the Dirichlet rows are drawn on the GPU
    # (torch) straight into the caller's buffer instead of by numpy on the
    # host: 16,384 trees hold about 27 G gamma variates.
    DEVICE_ROWS = 1 << 28

    def __init__(self, trees: int, states: int, seed: int, edges_on_device: bool = False):
        from parallel_tree_hmm_gb300 import synthetic

        rng = np.random.default_rng(seed)
        self.seed = seed
        self.parents = [synthetic.galton_watson(rng) for _ in range(trees)]
        self.states = states
        self.observed = [synthetic.leaves(p) for p in self.parents]
        self.num_nodes = np.array([len(p) for p in self.parents], dtype=np.int64)
        self.total_nodes = int(self.num_nodes.sum())
        self.total_edges = int((self.num_nodes - 1).sum())
        self.total_observed = int(sum(len(o) for o in self.observed))
        K = states
        self.root = synthetic.dirichlet_rows(rng, 1, K, 1.0, np.float32).ravel()
        self.emission = synthetic.dirichlet_rows(rng, K, K, 2.0, np.float32).ravel()
        self.edges_on_device = edges_on_device and self.total_edges * K > self.DEVICE_ROWS
        if self.edges_on_device:
            self.edges = None  # fill_edges() writes them into the caller's buffer
        else:
            g = rng.standard_gamma(0.3, size=(self.total_edges * K, K), dtype=np.float32)
            g /= g.sum(axis=1, keepdims=True)
            np.nan_to_num(g, copy=False, nan=1.0 / K)
            self.edges = g.ravel()
        self.observations = rng.integers(0, K, size=self.total_observed, dtype=np.uint8)
        self.uniforms = rng.random(self.total_nodes, dtype=np.float32)

    def fill_edges(self, out: np.ndarray, device: int) -> None:
        """Dirichlet(0.3) edge rows drawn on the GPU in chunks and copied into
        `out` (float32, every edge's K x K matrix); afterwards self.edges is
        `out`."""
        import torch

        K = self.states
        rows = self.total_edges * K
        generator = torch.Generator(device=f"cuda:{device}")
        generator.manual_seed(self.seed)
        target = torch.from_numpy(out)
        chunk = 1 << 24
        alpha = torch.full((chunk, K), 0.3, dtype=torch.float32, device=f"cuda:{device}")
        for start in range(0, rows, chunk):
            n = min(chunk, rows - start)
            g = torch._standard_gamma(alpha[:n], generator=generator)
            g /= g.sum(dim=1, keepdim=True)
            torch.nan_to_num_(g, nan=1.0 / K)
            target[start * K:(start + n) * K].copy_(g.reshape(-1))
        torch.cuda.synchronize(device)
        self.edges = out

    def tree_inputs(self, t, dtype):
        """Dense node factors, edge factors and uniforms of tree t."""
        K = self.states
        node0 = int(self.num_nodes[:t].sum())
        edge0 = node0 - t
        obs0 = int(sum(len(o) for o in self.observed[:t]))
        n = int(self.num_nodes[t])
        dense = np.ones((n, K), dtype=np.float64)
        dense[0] = self.root
        obs = self.observations[obs0:obs0 + len(self.observed[t])]
        dense[self.observed[t]] *= self.emission.astype(np.float64).reshape(K, K)[obs]
        if dtype == np.float32:
            # (root ? root : 1) * emission[obs] in FP32, as the kernel forms it.
            dense32 = np.ones((n, K), dtype=np.float32)
            dense32[0] = self.root
            dense32[self.observed[t]] = (dense32[self.observed[t]] *
                                         self.emission.reshape(K, K)[obs])
            dense = dense32
        if self.edges is None:
            # Edges drawn on the device were never made on this host (the CPU
            # reference arm of a large forest): the tree's own Dirichlet(0.3)
            # rows from a per-tree seed, same law.
            rng = np.random.default_rng([self.seed, t])
            g = rng.standard_gamma(0.3, size=((n - 1) * K, K))
            g /= g.sum(axis=1, keepdims=True)
            np.nan_to_num(g, copy=False, nan=1.0 / K)
            edges = g.ravel().astype(dtype)
        else:
            edges = self.edges[edge0 * K * K:(edge0 + n - 1) * K * K].astype(dtype)
        return dense.ravel().astype(dtype), edges, self.uniforms[node0:node0 + n]


def run_gw(args, rank, world, local_rank, dist):
    import parallel_tree_hmm_gb300 as thmm
    from oracle import bridge

    forest = GaltonWatsonForest(args.trees, args.states, rank_seed(args.seed, rank),
                                edges_on_device=True)
    K = forest.states
    config = {
        "workload": (f"Galton-Watson forest: {args.trees} Poisson(2) trees of "
                     f"1,000-50,000 nodes, K={K}, byte leaf observations, "
                     f"Dirichlet(0.3) edges, MAP + posterior sampling"),
        "trees": args.trees, "nodes_per_rank": forest.total_nodes, "states": K,
        "seed": args.seed, "parallelism": f"replicas of the forest per GPU x{args.gpus}",
        "l2": "inputs larger than L2 (edge factors of one step > 129 MB)",
    }
    metric = "tree-nodes/s for MAP+posterior sampling"
    if args.impl == "reference":
        if rank != 0:
            return
        sample_trees = max(1, min(args.trees, 64))
        per_step = []
        for _ in range(args.warmup + args.steps):
            start = time.perf_counter()
            nodes = 0
            jobs = [(t, bridge.CpuPlan(forest.parents[t])) for t in range(sample_trees)]

            def run(job):
                t, plan = job
                dense, edges, uniforms = forest.tree_inputs(t, np.float64)
                bridge.maximum(plan, K, dense, edges)
                bridge.sample(plan, K, dense, edges, uniforms.astype(np.float64))
                return plan.num_nodes

            with concurrent.futures.ThreadPoolExecutor(os.cpu_count() or 1) as pool:
                nodes = sum(pool.map(run, jobs))
            per_step.append(nodes / (time.perf_counter() - start))
        value = statistics.median(per_step[args.warmup:])
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count() or 1,
                             "kind": "port",
                             "sample": f"first {sample_trees} trees, FP64 MAP + sample"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return

    import torch

    device = local_rank
    torch.cuda.set_device(device)
    plans = thmm.Plan.many(forest.parents)
    ws = thmm.Workspace()
    ws.reserve_forest_categorical(plans, K, K, forest.observed, device,
                                  kind="maximum,sampling", scalar=np.float32)
    staged = ws.categorical_inputs()
    staged.root_potential[:] = forest.root
    staged.emission_potentials[:] = forest.emission
    if forest.edges_on_device:
        forest.fill_edges(staged.edge_potentials, device)
    else:
        staged.edge_potentials[:] = forest.edges
    staged.observations[:] = forest.observations
    uniforms = ws.uniforms()
    uniforms[:] = forest.uniforms
    map_view = ws.maximum_a_posteriori_prepared(staged, thmm.CategoricalInputUpdate.kAll)
    map_states = np.array(map_view.states)
    map_weights = np.array(map_view.log_weights)
    sample_states = np.array(ws.posterior_sample_prepared(
        staged, uniforms, thmm.CategoricalInputUpdate.kNone).states)

    # Checks on the first trees (the oracle as checker):
    #  * bit-exactness against the oracle with the device's reproducible
    #    exp/log (FP32);
    #  * agreement of MAP states and samples with the reference FP32 build
    #    (libm-mode oracle) and with FP64, every disagreement classified by the
    #    margin of the comparison that decided it (oracle/agreement.py).
    from oracle import agreement

    check_trees = min(args.check_trees, args.trees)
    exact = 0
    parts = {"map_fp32_reference": [], "sample_fp32_reference": [], "map_fp64": [],
             "sample_fp64": []}
    node0 = 0
    for t in range(check_trees):
        n = int(forest.num_nodes[t])
        got_map, got_sample = map_states[node0:node0 + n], sample_states[node0:node0 + n]
        dense, edges, u = forest.tree_inputs(t, np.float32)
        if t < 8:
            w32, s32 = bridge.maximum(plans[t], K, dense, edges, np.float32,
                                      bridge.MATH_PORTABLE)
            draw = bridge.sample(plans[t], K, dense, edges, u, np.float32,
                                 bridge.MATH_PORTABLE)
            exact += int(np.array_equal(s32, got_map) and w32 == map_weights[t] and
                         np.array_equal(draw, got_sample))
        _, s, m = bridge.maximum_margins(plans[t], K, dense, edges, np.float32)
        parts["map_fp32_reference"].append(
            agreement.classify(plans[t], got_map, s, m, agreement.MAP_TIE_MARGIN))
        s, m = bridge.sample_margins(plans[t], K, dense, edges, u, np.float32)
        parts["sample_fp32_reference"].append(
            agreement.classify(plans[t], got_sample, s, m, agreement.SAMPLE_TIE_MARGIN))
        dense64, edges64, _ = forest.tree_inputs(t, np.float64)
        _, s, m = bridge.maximum_margins(plans[t], K, dense64, edges64)
        parts["map_fp64"].append(
            agreement.classify(plans[t], got_map, s, m, agreement.MAP_TIE_MARGIN))
        s, m = bridge.sample_margins(plans[t], K, dense64, edges64, u.astype(np.float64))
        parts["sample_fp64"].append(
            agreement.classify(plans[t], got_sample, s, m, agreement.SAMPLE_TIE_MARGIN))
        node0 += n
    agreements = {key: agreement.merge(value) for key, value in parts.items()}

    tuning_map = ws.tuning if args.no_autotune else ws.autotune(2, repeats=2)
    tuning_sample = ws.tuning if args.no_autotune else ws.autotune(3, repeats=2)

    def step():
        ws.enqueue(2)
        ws.enqueue(3)

    ext = torch.cuda.ExternalStream(ws.stream, device=device)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(device)
    if dist is not None:
        dist.barrier()
    sampler = ClockSampler(device)
    with sampler:
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record(ext)
        for _ in range(args.steps):
            step()
        stop.record(ext)
        stop.synchronize()
    elapsed_ms = reduce_max(start.elapsed_time(stop), dist)
    step_ms = elapsed_ms / args.steps
    value = forest.total_nodes * world / (step_ms / 1e3)

    e2e_steps = args.e2e_steps or max(3, min(args.steps, 10))
    e2e_total = 0.0
    for _ in range(e2e_steps):
        torch.cuda.synchronize(device)
        begin = time.perf_counter()
        ws.maximum_a_posteriori_prepared(staged, thmm.CategoricalInputUpdate.kFactors)
        ws.posterior_sample_prepared(staged, uniforms, thmm.CategoricalInputUpdate.kNone)
        e2e_total += time.perf_counter() - begin
    e2e_total = reduce_max(e2e_total, dist)
    S = 4
    h2d = forest.total_edges * K * K * S + (K + K * K) * S + forest.total_nodes * S
    d2h = 2 * forest.total_nodes * 4 + len(plans) * S + 32

    algorithmic = (2 * forest.total_edges * K * K * S + 2 * forest.total_observed
                   + forest.total_nodes * (S + 4 + 4) + len(plans) * S)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = algorithmic / (step_ms / 1e3) / 1e9
    line = {
        "metric": metric, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {**config, "tuning_map": tuning_map, "tuning_sample": tuning_sample,
                   "bit_exact_trees": f"{exact}/{min(8, check_trees)}",
                   "agreement_trees": check_trees,
                   "map_fp32_reference_agreement": agreements["map_fp32_reference"]["rate"],
                   "sample_fp32_reference_agreement":
                       agreements["sample_fp32_reference"]["rate"],
                   "map_fp64_agreement": agreements["map_fp64"]["rate"],
                   "sample_fp64_agreement": agreements["sample_fp64"]["rate"],
                   "agreement_detail": agreements},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "peak_source": "measured" if peaks else "fallback",
                     "traffic": None, "algorithmic_bytes_per_launch": algorithmic},
        "e2e": {"value": forest.total_nodes * world * e2e_steps / e2e_total, "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": 2 * args.steps,
        "clocks": sampler.summary(),
    }
    if rank == 0 and world == 1 and args.cpu_sample_nodes > 0:
        # Reference FP64 CPU MAP + sample (oracle port) on the first trees,
        # over all host cores; plans from the oracle's planner library.
        sample_trees = max(1, min(args.trees, 64))
        jobs = [(t, bridge.CpuPlan(forest.parents[t])) for t in range(sample_trees)]

        def run_cpu(job):
            t, plan = job
            dense, edges, u = forest.tree_inputs(t, np.float64)
            bridge.maximum(plan, K, dense, edges)
            bridge.sample(plan, K, dense, edges, u.astype(np.float64))
            return plan.num_nodes

        start = time.perf_counter()
        with concurrent.futures.ThreadPoolExecutor(os.cpu_count() or 1) as pool:
            done = sum(pool.map(run_cpu, jobs))
        elapsed = time.perf_counter() - start
        line["cpu_baseline"] = {"value": done / elapsed, "unit": UNIT,
                                "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"first {sample_trees} trees ({done} nodes), "
                                          f"FP64 MAP + sample, {elapsed:.2f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)


# -------------------------------------------- dense-contraction workload
def run_dense(args, rank, world, local_rank, dist):
    """Dense-factor marginals. Default: spine-heavy random recursive trees
    (node i attaches to i - 1 with probability 0.95, else to a uniform earlier
    node), K = 64 or 128, node factors lognormal(0, 1), edge factors
    lognormal(0, 2) with 5% exact zeros, on the tensor-core engine; the trees
    are scaled down from 100,000 nodes so that the edge factors fit in HBM and
    host memory (--tree-nodes). With --shape recursive --states 20
    --tree-nodes 5000 --trees 1024 --edge-sigma 1.5 --zero-fraction 0.02 it is
    the differentiation workload (gradient = marginals) at full size."""
    import parallel_tree_hmm_gb300 as thmm
    from oracle import bridge
    from parallel_tree_hmm_gb300 import synthetic

    K = args.states
    rng = np.random.default_rng(rank_seed(args.seed, rank))
    grow = synthetic.spine_heavy if args.shape == "spine-heavy" else synthetic.random_recursive
    parents = [grow(rng, args.tree_nodes) for _ in range(args.trees)]
    if args.windows > 1 and args.impl == "ours":
        run_dense_streamed(args, rank, world, local_rank, dist, parents)
        return
    # The reference arm plans with the oracle's planner library (no product
    # code loaded); the same planner source gives the same plans.
    plans = ([bridge.CpuPlan(p) for p in parents] if args.impl == "reference"
             else thmm.Plan.many(parents))
    total_nodes = sum(p.num_nodes for p in plans)
    total_edges = sum(p.num_edges for p in plans)
    compressions = sum(int(p.num_compressions) for p in plans)
    config = {
        "workload": (f"dense factors: {args.trees} {args.shape} trees of {args.tree_nodes} "
                     f"nodes, K={K}, lognormal(0,1) node and lognormal(0,{args.edge_sigma:g}) "
                     f"edge factors with {100 * args.zero_fraction:g}% zeros, marginals"),
        "trees": args.trees, "nodes_per_rank": total_nodes, "states": K,
        "compressions_per_rank": compressions, "seed": args.seed,
        "parallelism": f"replicas per GPU x{args.gpus}",
        "l2": "inputs larger than L2 (edge factors of one step > 129 MB)",
        "scaled_from": ("256 trees x 100,000 nodes (1.7 TB of edge factors at K=128)"
                        if args.shape == "spine-heavy" else None),
    }
    metric = "tree-nodes/s for logZ+marginals+grad (dense factors)"

    def edge_chunks(fill):
        chunk = 1 << 24
        values = total_edges * K * K
        for start in range(0, values, chunk):
            n = min(chunk, values - start)
            block = np.exp(np.float32(args.edge_sigma) * rng.standard_normal(n, dtype=np.float32))
            block[rng.random(n, dtype=np.float32) < args.zero_fraction] = 0.0
            fill(start, block)

    node_factors = np.exp(rng.standard_normal(total_nodes * K, dtype=np.float32))

    if args.impl == "reference" or (rank == 0 and world == 1 and args.cpu_sample_nodes > 0):
        sample = min(16, args.trees)
        edge0 = np.cumsum([0] + [p.num_edges for p in plans])
        node0 = np.cumsum([0] + [p.num_nodes for p in plans])
        sample_edges = np.empty(int(edge0[sample]) * K * K, dtype=np.float32)

        def keep(start, block):
            stop = min(start + len(block), sample_edges.size)
            if start < stop:
                sample_edges[start:stop] = block[:stop - start]

        state = rng.bit_generator.state
        edge_chunks(keep)
        rng.bit_generator.state = state

        oracle_results = {}

        def job(t):
            log_z, _, node_m, _ = bridge.marginals(
                plans[t], K, node_factors[node0[t] * K:node0[t + 1] * K].astype(np.float64),
                sample_edges[edge0[t] * K * K:edge0[t + 1] * K * K].astype(np.float64))
            oracle_results[t] = (log_z, node_m)
            return plans[t].num_nodes

        start = time.perf_counter()
        with concurrent.futures.ThreadPoolExecutor(os.cpu_count() or 1) as pool:
            done = sum(pool.map(job, range(sample)))
        cpu = {"value": done / (time.perf_counter() - start), "unit": UNIT,
               "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"first {sample} trees, FP64 log-domain marginals"}
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({
                    "impl": "reference", "metric": metric, "value": cpu["value"],
                    "unit": UNIT, "n_gpus": args.gpus, "steps": 1, "warmup": 0,
                    "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                    "config": config, "cpu_baseline": cpu,
                    "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                            "d2h_bytes_per_step": 0}}), flush=True)
            return
    else:
        cpu = None
        oracle_results = {}

    import torch

    device = local_rank
    torch.cuda.set_device(device)
    ws = thmm.Workspace()
    ws.reserve_forest(plans, K, device, kind="marginals", scalar=np.float32,
                      compute="bf16" if args.precision == "bf16" else None)
    select_schedule(ws, args)
    staged = ws.inputs()
    staged.node_potentials[:] = node_factors

    def fill(start, block):
        staged.edge_potentials[start:start + len(block)] = block

    edge_chunks(fill)
    first = ws.posterior_marginals_prepared(staged)
    finite = bool(np.all(np.isfinite(first.log_partitions)))
    node_sum_error = float(np.max(np.abs(
        np.array(first.nodes).reshape(-1, K).sum(axis=1) - 1.0)))
    # Errors against the FP64 oracle on the CPU leg's sample trees.
    accuracy = {}
    if oracle_results:
        got_nodes = np.array(first.nodes)
        rel, worst = 0.0, 0.0
        for t, (log_z, node_m) in oracle_results.items():
            rel = max(rel, abs(float(first.log_partitions[t]) - log_z) / max(1.0, abs(log_z)))
            worst = max(worst, float(np.max(np.abs(
                got_nodes[node0[t] * K:node0[t + 1] * K] - node_m))))
        accuracy = {"checked_trees": len(oracle_results), "log_z_max_rel_error": rel,
                    "node_marginal_max_abs_error": worst}

    ext = torch.cuda.ExternalStream(ws.stream, device=device)
    for _ in range(args.warmup):
        ws.enqueue(4)
    torch.cuda.synchronize(device)
    if dist is not None:
        dist.barrier()
    sampler = ClockSampler(device)
    with sampler:
        begin = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        begin.record(ext)
        for _ in range(args.steps):
            ws.enqueue(4)
        end.record(ext)
        end.synchronize()
    launches = ws.launches
    step_ms = reduce_max(begin.elapsed_time(end), dist) / args.steps
    value = total_nodes * world / (step_ms / 1e3)

    e2e_steps = args.e2e_steps or 3
    e2e_total = 0.0
    for _ in range(e2e_steps):
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        ws.posterior_marginals_prepared(staged)
        e2e_total += time.perf_counter() - t0
    e2e_total = reduce_max(e2e_total, dist)

    S = 4
    algorithmic = (2 * total_edges * K * K * S + 2 * total_nodes * K * S + len(plans) * S)
    # Useful tensor-core work: 2 K^3 per product, one product per compression
    # forward and two in the adjoint.
    useful_flops = 3 * 2 * compressions * K ** 3
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = algorithmic / (step_ms / 1e3) / 1e9
    line = {
        "metric": metric, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("f32" if K <= 32 else "f32 (BF16 tensor-core products)"
                  if args.precision == "bf16" else "f32 (3xTF32 tensor-core products)"),
        "data": "synthetic",
        "config": {**config, "all_log_z_finite": finite, "precision_tier": args.precision,
                   "schedule": args.schedule if K > 32 else None,
                   "accuracy_vs_fp64_oracle": accuracy,
                   "node_marginal_normalisation_error": node_sum_error,
                   ("useful_tensor_tflops" if K > 32 else "useful_product_tflops"):
                       useful_flops / (step_ms / 1e3) / 1e12},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "peak_source": "measured" if peaks else "fallback",
                     "traffic": None, "algorithmic_bytes_per_launch": algorithmic},
        "e2e": {"value": total_nodes * world * e2e_steps / e2e_total, "unit": UNIT,
                "h2d_bytes_per_step": (total_edges * K * K + total_nodes * K) * S,
                "d2h_bytes_per_step": (total_edges * K * K + total_nodes * K) * S
                + len(plans) * S + 16},
        "gpu_launches": launches * args.steps,
        "clocks": sampler.summary(),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_sites(args, rank, world, local_rank, dist):
    """Phylogenetic-style batch through the reference's batch API: ONE random
    binary tree (leaf splitting, --tree-nodes, default 2001 nodes) and
    --sites node-factor sets (sites) sharing its edge factors; K=4, leaf
    observations uniform over 4 categories, a Dirichlet(5) emission table,
    Dirichlet(1) root and edge rows; log Z and node/edge marginals per site.
    The shared-topology layout reads each edge row once per warp of 32 sites,
    so the step reads the edge factors from DRAM once (edge_bytes_read) where
    a per-site layout would read them once per site (edge_bytes_per_site)."""
    import torch

    import parallel_tree_hmm_gb300 as thmm
    from oracle import bridge
    from parallel_tree_hmm_gb300 import synthetic

    K, B = 4, args.sites
    rng = np.random.default_rng(rank_seed(args.seed, rank))
    parents = synthetic.leaf_splitting(rng, args.tree_nodes or 2001)
    cpu_plan = bridge.CpuPlan(parents)
    observed = synthetic.leaves(parents)
    n, e, leaves = cpu_plan.num_nodes, cpu_plan.num_edges, len(observed)
    root = synthetic.dirichlet_rows(rng, 1, K, 1.0, np.float32).ravel()
    emission = synthetic.dirichlet_rows(rng, K, K, 5.0, np.float32).ravel()
    edges = synthetic.stochastic_edges(rng, e, K, 1.0, np.float32)
    observations = rng.integers(0, K, B * leaves).astype(np.uint8)

    # FP64 oracle on a sample of sites (the CPU baseline, and the reference arm).
    sample = min(B, 256)
    obs = observations.reshape(B, leaves)
    emit = emission.reshape(K, K).astype(np.float64)
    root_node = int(np.flatnonzero(np.asarray(parents) < 0)[0])

    def site(b):
        dense = np.ones((n, K))
        dense[root_node] = root
        dense[observed] = dense[observed] * emit[obs[b]]
        z, _, _, _ = bridge.marginals(cpu_plan, K, dense.ravel(), edges.astype(np.float64))
        return z

    if rank != 0 and args.impl == "reference":
        return
    start = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(os.cpu_count() or 1) as pool:
        oracle_z = list(pool.map(site, range(sample)))
    cpu_s = time.perf_counter() - start
    cpu = {"value": sample * n / cpu_s, "unit": UNIT, "cores": os.cpu_count() or 1,
           "kind": "port", "sample": f"{sample} sites, FP64 log-domain marginals, {cpu_s:.2f} s"}
    metric = "tree-nodes/s for logZ+marginals+grad (batch API, one tree, many sites)"
    config = {"workload": (f"phylogenetic-style batch: one random binary tree of {n} "
                           f"nodes ({leaves} observed leaves), {B} sites, K={K}, "
                           f"kAll marginals through the batch API"),
              "sites": B, "tree_nodes": n, "states": K}
    if args.impl == "reference":
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": cpu["value"], "unit": UNIT,
            "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config, "cpu_baseline": cpu,
            "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return

    plan = thmm.Plan(parents)
    device = local_rank
    torch.cuda.set_device(device)
    ws = thmm.Workspace()
    ws.reserve_categorical_marginals(plan, K, B, K, observed, device, scalar=np.float32)
    staged = ws.categorical_inputs(B)
    staged.root_potential[:] = root
    staged.emission_potentials[:] = emission
    staged.edge_potentials[:] = edges
    staged.observations[:] = observations
    first = ws.posterior_marginals_prepared(staged, thmm.CategoricalInputUpdate.kAll)
    log_z = np.array(first.log_partitions, dtype=np.float64)
    rel = max(abs(log_z[b] - oracle_z[b]) / max(1.0, abs(oracle_z[b])) for b in range(sample))

    ext = torch.cuda.ExternalStream(ws.stream, device=device)
    for _ in range(args.warmup):
        ws.enqueue(4)
    torch.cuda.synchronize(device)
    if dist is not None:
        dist.barrier()
    sampler = ClockSampler(device)
    with sampler:
        begin = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        begin.record(ext)
        for _ in range(args.steps):
            ws.enqueue(4)
        end.record(ext)
        end.synchronize()
    launches = ws.launches
    step_ms = reduce_max(begin.elapsed_time(end), dist) / args.steps
    value = B * n * world / (step_ms / 1e3)

    e2e_steps = args.e2e_steps or 5
    calls = []
    for _ in range(e2e_steps):
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        ws.posterior_marginals_prepared(staged, thmm.CategoricalInputUpdate.kAll)
        calls.append(time.perf_counter() - t0)
    e2e_total = reduce_max(sum(calls), dist)

    S = 4
    edge_bytes = e * K * K * S
    algorithmic = (edge_bytes + B * leaves + B * (n * K + e * K * K) * S + B * S)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = algorithmic / (step_ms / 1e3) / 1e9
    line = {
        "metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {**config, "tuning": ws.tuning,
                   "edge_bytes_read": edge_bytes,
                   "edge_bytes_per_site_layout": B * edge_bytes,
                   "log_z_max_rel_error_vs_fp64_oracle": rel, "checked_sites": sample,
                   "l2": "outputs larger than L2 (node and edge marginals of every site)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": "measured" if peaks else "fallback",
                     "traffic": None, "algorithmic_bytes_per_launch": algorithmic},
        "e2e": {"value": B * n * world * e2e_steps / e2e_total, "unit": UNIT,
                "h2d_bytes_per_step": B * leaves + (K + K * K) * S + edge_bytes,
                "d2h_bytes_per_step": B * S + B * (n * K + e * K * K) * S + 16,
                "call_ms": [round(1e3 * c, 3) for c in calls]},
        "gpu_launches": launches * args.steps,
        "clocks": sampler.summary(),
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def select_schedule(ws, args):
    """Applies --schedule to a workspace above 32 states (the forest default
    is the phase schedule)."""
    from parallel_tree_hmm_gb300 import _lib

    if args.states > 32:
        wanted = (_lib.THMM_SCHEDULE_PHASES if args.schedule == "phases"
                  else _lib.THMM_SCHEDULE_TEAMS)
        ws.set_tuning(ws.tuning["team_threshold"], schedule=wanted)


def run_dense_streamed(args, rank, world, local_rank, dist, parents):
    """The dense workload at a size beyond HBM: the trees pass through one
    workspace in `args.windows` windows. Each window's node and edge factors
    are drawn on the GPU straight into the workspace's device buffers
    (device_buffers, device_inputs_ready) and contracted by the device-only
    step; the value is all nodes over the summed device time of the windows'
    steps. Accuracy is covered by the scaled runs of the same laws and by the
    streamed-window parity tests; the CPU baseline is the FP64 oracle on one
    2,000-node tree of the same laws (K <= 64)."""
    import torch

    import parallel_tree_hmm_gb300 as thmm
    from oracle import bridge

    K = args.states
    device = local_rank
    torch.cuda.set_device(device)
    generator = torch.Generator(device=f"cuda:{device}")
    generator.manual_seed(rank_seed(args.seed, rank))
    bounds = np.linspace(0, len(parents), args.windows + 1).astype(int)
    ws = thmm.Workspace()
    window_ms, nodes_done, compressions = [], 0, 0
    finite, node_sum_error, cpu, launches = True, 0.0, None, 0
    sampler = ClockSampler(device)

    def fill(view, sigma, zero_fraction):
        chunk = 1 << 26
        for start in range(0, view.numel(), chunk):
            n = min(chunk, view.numel() - start)
            x = torch.randn(n, generator=generator, device=view.device)
            x.mul_(sigma).exp_()
            if zero_fraction > 0:
                x[torch.rand(n, generator=generator, device=view.device) < zero_fraction] = 0
            view[start:start + n].copy_(x)

    with sampler:
        for w in range(args.windows):
            plans = thmm.Plan.many(parents[bounds[w]:bounds[w + 1]])
            ws.reserve_forest(plans, K, device, kind="marginals,device", scalar=np.float32,
                              compute="bf16" if args.precision == "bf16" else None)
            select_schedule(ws, args)
            buffers = ws.device_buffers()
            fill(buffers["node_potentials"], 1.0, 0.0)
            fill(buffers["edge_potentials"], args.edge_sigma, args.zero_fraction)
            torch.cuda.synchronize(device)
            ws.device_inputs_ready()
            ext = torch.cuda.ExternalStream(ws.stream, device=device)
            ws.enqueue(4)  # untimed: captures the step's CUDA graph
            begin = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            begin.record(ext)
            nodes_done += ws.enqueue(4)
            end.record(ext)
            end.synchronize()
            launches += ws.launches
            window_ms.append(begin.elapsed_time(end))
            compressions += sum(int(p.num_compressions) for p in plans)
            log_z = buffers["values"].cpu().numpy()
            finite = finite and bool(np.all(np.isfinite(log_z)))
            node_sum_error = max(node_sum_error, float(
                (buffers["node_marginals"].view(-1, K).sum(dim=1) - 1).abs().max()))
            if w == 0 and rank == 0 and K <= 64 and args.cpu_sample_nodes > 0:
                # A 100,000-node tree takes the FP64 oracle minutes, so the CPU
                # sample is one 2,000-node tree of the same shape and factor laws.
                from parallel_tree_hmm_gb300 import synthetic

                sample_rng = np.random.default_rng(rank_seed(args.seed, rank) + 7)
                grow = (synthetic.spine_heavy if args.shape == "spine-heavy"
                        else synthetic.random_recursive)
                plan = bridge.CpuPlan(grow(sample_rng, 2000))
                n, e = plan.num_nodes, plan.num_edges
                nodes = np.exp(sample_rng.standard_normal(n * K))
                edges = np.exp(args.edge_sigma * sample_rng.standard_normal(e * K * K))
                edges[sample_rng.random(e * K * K) < args.zero_fraction] = 0.0
                start = time.perf_counter()
                bridge.marginals(plan, K, nodes, edges)
                elapsed = time.perf_counter() - start
                cpu = {"value": n / elapsed, "unit": UNIT, "cores": 1, "kind": "port",
                       "sample": f"one {n}-node tree of the same laws, FP64 log-domain "
                                 f"marginals, {elapsed:.1f} s on one core"}
            del buffers
    total_ms = reduce_max(sum(window_ms), dist)
    total_nodes = sum(len(p) for p in parents)
    total_edges = total_nodes - len(parents)
    value = nodes_done * world / (total_ms / 1e3)
    S = 4
    algorithmic = 2 * total_edges * K * K * S + 2 * total_nodes * K * S + len(parents) * S
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    line = {
        "metric": "tree-nodes/s for logZ+marginals+grad (dense factors)", "value": value,
        "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": total_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("f32 (BF16 tensor-core products)" if args.precision == "bf16"
                  else "f32 (3xTF32 tensor-core products)") if K > 32 else "f32",
        "data": "synthetic, drawn on the GPU",
        "config": {"workload": (f"dense factors at full size: {len(parents)} {args.shape} trees "
                                f"of {args.tree_nodes} nodes, K={K}, lognormal(0,1) node and "
                                f"lognormal(0,{args.edge_sigma:g}) edge factors with "
                                f"{100 * args.zero_fraction:g}% zeros, marginals"),
                   "trees": len(parents), "nodes_per_rank": total_nodes, "states": K,
                   "windows": args.windows, "window_ms": [round(v, 2) for v in window_ms],
                   "edge_factor_bytes": total_edges * K * K * S,
                   "compressions_per_rank": compressions, "precision_tier": args.precision,
                   "all_log_z_finite": finite,
                   "node_marginal_normalisation_error": node_sum_error,
                   ("useful_tensor_tflops" if K > 32 else "useful_product_tflops"):
                       3 * 2 * compressions * K ** 3 / (total_ms / 1e3) / 1e12,
                   "schedule": args.schedule if K > 32 else None,
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": algorithmic / (total_ms / 1e3) / 1e9,
                     "peak": peak, "unit": "GB/s",
                     "frac": algorithmic / (total_ms / 1e3) / 1e9 / peak,
                     "peak_source": "measured" if peaks else "fallback", "traffic": None,
                     "algorithmic_bytes_per_launch": algorithmic},
        "e2e": {"value": None, "unit": UNIT,
                "reason": "inputs exceed host memory; drawn on the device, no host copies",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": launches,
        "clocks": sampler.summary(),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
