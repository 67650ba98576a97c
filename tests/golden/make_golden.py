"""Generates the golden fixtures in tests/golden/ from the reference's own CPU
library (src/inference.cc compiled from the reference tree into oracle/_ref by
`make -C oracle ref`, against this project's planner).

Each case is a seeded tree, state count and factor set. The fixture stores the
reference build's outputs: scaled log Z, raw Z, log-domain marginals, MAP
weight and states, and a posterior sample for seeded uniforms, in FP64 and
FP32 builds. Run from the repository root:

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import bridge  # noqa: E402
from parallel_tree_hmm_gb300 import synthetic  # noqa: E402

OUT = pathlib.Path(__file__).resolve().parent


def cases():
    rng = np.random.default_rng(20261203)
    trees = [
        ("pair", np.array([-1, 0])),
        ("five", np.array([-1, 0, 0, 1, 3])),
        ("seven_binary", np.array([-1, 0, 0, 1, 1, 2, 2])),
        ("chain64", np.arange(-1, 63)),
        ("star17", np.array([-1] + [0] * 17)),
        ("binary31", synthetic.leaf_splitting(rng, 31)),
        ("recursive200", synthetic.random_recursive(rng, 200)),
        ("caterpillar100", synthetic.caterpillar(100)),
        ("spine_heavy150", synthetic.spine_heavy(rng, 150)),
    ]
    for name, parents in trees:
        for states in (1, 2, 3, 4, 5, 8):
            if len(parents) > 64 and states not in (2, 4):
                continue
            if len(parents) > 20 and states > 4:
                continue
            for zeros in (0.0, 0.08):
                n = len(parents)
                nodes = rng.random(n * states) * 0.9 + 0.1
                edges = rng.random((n - 1) * states * states) * 0.9 + 0.1
                if zeros:
                    nodes[rng.random(nodes.size) < zeros] = 0.0
                    edges[rng.random(edges.size) < zeros] = 0.0
                uniforms = rng.random(n)
                yield f"{name}_k{states}_z{int(zeros * 100)}", parents, states, nodes, edges, uniforms


def run(reference, parents, states, nodes, edges, uniforms, dtype):
    handle = reference.model(parents, states)
    n = len(parents)
    record = {}
    try:
        for key, call in (
                ("log_partition", lambda: reference.log_partition(handle, nodes, edges)),
                ("partition", lambda: reference.partition(handle, nodes, edges))):
            record[key] = np.asarray(call(), dtype=dtype)
        try:
            log_z, z, node_m, edge_m = reference.marginals(handle, nodes, edges, n, n - 1,
                                                           states)
            record.update(marginal_log_partition=np.asarray(log_z, dtype=dtype),
                          marginal_partition=np.asarray(z, dtype=dtype),
                          node_marginals=node_m, edge_marginals=edge_m)
        except bridge.OracleError as error:
            record["marginal_status"] = np.asarray(error.status)
        try:
            weight, states_map = reference.maximum(handle, nodes, edges, n)
            record.update(map_log_weight=np.asarray(weight, dtype=dtype), map_states=states_map)
        except bridge.OracleError as error:
            record["map_status"] = np.asarray(error.status)
        try:
            record["sample_states"] = reference.sample(handle, nodes, edges, uniforms, n)
        except bridge.OracleError as error:
            record["sample_status"] = np.asarray(error.status)
    finally:
        reference.destroy(handle)
    return record


def main():
    references = {np.float64: bridge.Reference(np.float64),
                  np.float32: bridge.Reference(np.float32)}
    payload = {}
    for name, parents, states, nodes, edges, uniforms in cases():
        payload[f"{name}/parents"] = parents.astype(np.int64)
        payload[f"{name}/states"] = np.asarray(states)
        for dtype, tag in ((np.float64, "f64"), (np.float32, "f32")):
            n_ = nodes.astype(dtype)
            e_ = edges.astype(dtype)
            u_ = uniforms.astype(dtype)
            payload[f"{name}/{tag}/nodes"] = n_
            payload[f"{name}/{tag}/edges"] = e_
            payload[f"{name}/{tag}/uniforms"] = u_
            for key, value in run(references[dtype], parents, states, n_, e_, u_,
                                  dtype).items():
                payload[f"{name}/{tag}/{key}"] = value
    np.savez_compressed(OUT / "reference_cpu.npz", **payload)
    print(f"wrote {len(payload)} arrays to {OUT / 'reference_cpu.npz'}")


if __name__ == "__main__":
    main()
