"""Differentiation: d(sum log Z)/d(log node and edge factors) from the
adjoint kernel, through the torch.autograd wrapper, on trees shaped like the
differentiation workload (random recursive trees of 5000 nodes, K = 20, dense
node factors lognormal(0, 1), edge factors lognormal(0, 1.5) with 2% exact
zeros; FP32 arithmetic with exact power-of-two scaling).

Checked against
  * the oracle's FP64 marginals (max abs error <= 1e-5), and
  * FP64 central finite differences of the oracle's log Z on 200 random
    coordinates with nonzero factors, h = 1e-4 in log space (abs error <=
    2e-5: truncation O(h^2) and rounding O(eps |log Z| / h) are both below
    1e-7 here, the rest is the FP32 kernel).
"""
import concurrent.futures

import numpy as np
import pytest

from oracle import bridge
from parallel_tree_hmm_gb300 import synthetic

pytestmark = pytest.mark.gpu


def test_gradient_matches_marginals_and_finite_differences(gpu):
    torch = pytest.importorskip("torch")
    from parallel_tree_hmm_gb300 import autograd

    rng = np.random.default_rng(3)
    trees, nodes_per_tree, K = 6, 5000, 20
    plans = [gpu.Plan(synthetic.random_recursive(rng, nodes_per_tree)) for _ in range(trees)]
    N = sum(p.num_nodes for p in plans)
    E = sum(p.num_edges for p in plans)
    log_nodes = torch.from_numpy(rng.normal(0.0, 1.0, size=(N, K)))
    edge_values = synthetic.lognormal(rng, E * K * K, 1.5, zero_fraction=0.02)
    with np.errstate(divide="ignore"):
        log_edges = torch.from_numpy(np.log(edge_values).reshape(E, K, K))
    log_nodes.requires_grad_(True)
    log_edges.requires_grad_(True)

    ws = autograd.forest_workspace(plans, K)
    log_z = autograd.forest_log_partition(ws, log_nodes, log_edges)
    log_z.sum().backward()
    grad_nodes = log_nodes.grad.numpy()
    grad_edges = log_edges.grad.numpy()

    node_offsets = np.cumsum([0] + [p.num_nodes for p in plans])
    edge_offsets = np.cumsum([0] + [p.num_edges for p in plans])
    nodes64 = np.exp(log_nodes.detach().numpy()).astype(np.float32).astype(np.float64)
    edges64 = edge_values.astype(np.float32).astype(np.float64).reshape(E, K, K)

    def tree_inputs(t):
        return (nodes64[node_offsets[t]:node_offsets[t + 1]].ravel(),
                edges64[edge_offsets[t]:edge_offsets[t + 1]].ravel())

    # Marginals = gradient, against the FP64 oracle.
    for t in range(2):
        nodes_t, edges_t = tree_inputs(t)
        expected_log_z, _, node_m, edge_m = bridge.marginals(plans[t], K, nodes_t, edges_t)
        assert abs(log_z[t].item() - expected_log_z) <= 1e-6 * abs(expected_log_z)
        got_n = grad_nodes[node_offsets[t]:node_offsets[t + 1]].ravel()
        got_e = grad_edges[edge_offsets[t]:edge_offsets[t + 1]].ravel()
        assert np.max(np.abs(got_n - node_m)) <= 1e-5
        assert np.max(np.abs(got_e - edge_m)) <= 1e-5

    # Central finite differences in FP64 on 200 coordinates with nonzero factors.
    h = 1e-4
    picks = []
    while len(picks) < 200:
        t = int(rng.integers(trees))
        if rng.random() < 0.5:
            n = int(rng.integers(plans[t].num_nodes))
            k = int(rng.integers(K))
            picks.append((t, "node", n, k))
        else:
            e = int(rng.integers(plans[t].num_edges))
            i, j = int(rng.integers(K)), int(rng.integers(K))
            if edges64[edge_offsets[t] + e, i, j] > 0:
                picks.append((t, "edge", e, i * K + j))

    def difference(pick):
        t, kind, index, entry = pick
        nodes_t, edges_t = tree_inputs(t)
        values = []
        for sign in (1.0, -1.0):
            n_, e_ = nodes_t.copy(), edges_t.copy()
            if kind == "node":
                n_[index * K + entry] *= np.exp(sign * h)
            else:
                e_[index * K * K + entry] *= np.exp(sign * h)
            values.append(bridge.log_partition(plans[t], K, n_, e_))
        return (values[0] - values[1]) / (2 * h)

    with concurrent.futures.ThreadPoolExecutor(max_workers=16) as pool:
        finite = list(pool.map(difference, picks))
    worst = 0.0
    for (t, kind, index, entry), fd in zip(picks, finite):
        if kind == "node":
            analytic = grad_nodes[node_offsets[t] + index, entry]
        else:
            analytic = grad_edges[edge_offsets[t] + index].ravel()[entry]
        worst = max(worst, abs(analytic - fd))
    assert worst <= 2e-5, worst
