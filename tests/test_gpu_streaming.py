"""Sub-batch streaming through a bounded device window, with inputs written
on the device.

A forest too large for HBM (the dense-contraction workload at its stated size
holds 0.42-1.7 TB of edge factors) is contracted window by window: one
workspace is reserved for the trees of a window, the window's factors are
written straight into the workspace's device buffers (device_buffers(), here
from host arrays, in the bench drawn on the GPU), declared resident
(device_inputs_ready()), contracted by the device-only step (enqueue()) and
its results read from the device buffers. Every window must match the FP64
oracle tree by tree: K = 4 (the phase schedule, dense and categorical) and
K = 40 (the tensor-core engine), three windows each.
"""
import numpy as np
import pytest

from oracle import bridge
from parallel_tree_hmm_gb300 import synthetic

pytestmark = pytest.mark.gpu


def windows(items, count):
    bounds = np.linspace(0, len(items), count + 1).astype(int)
    return [items[a:b] for a, b in zip(bounds[:-1], bounds[1:])]


@pytest.mark.parametrize("K", [4, 40])
def test_dense_forest_streamed_in_windows(gpu, K):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4000 + K)
    parents = [synthetic.spine_heavy(rng, int(n)) for n in (90, 300, 45, 160, 220, 70)]
    ws = gpu.Workspace()
    checked = 0
    for number, window in enumerate(windows(parents, 3)):
        plans = [gpu.Plan(p) for p in window]
        # Alternate staged and device-only reservations (no pinned staging).
        kind = "marginals,device" if number % 2 else "marginals"
        ws.reserve_forest(plans, K, kind=kind, scalar=np.float32)
        n_total = sum(p.num_nodes for p in plans)
        e_total = sum(p.num_edges for p in plans)
        nodes = (rng.random(n_total * K) * 0.9 + 0.1).astype(np.float32)
        edges = synthetic.stochastic_edges(rng, e_total, K, 0.5, np.float32)
        buffers = ws.device_buffers()
        buffers["node_potentials"].copy_(torch.from_numpy(nodes))
        buffers["edge_potentials"].copy_(torch.from_numpy(edges))
        torch.cuda.synchronize()
        ws.device_inputs_ready()
        assert ws.enqueue(4) == n_total
        ws.synchronize()
        log_z = buffers["values"].cpu().numpy()
        node_m = buffers["node_marginals"].cpu().numpy()
        edge_m = buffers["edge_marginals"].cpu().numpy()
        n0 = e0 = 0
        for t, plan in enumerate(plans):
            n, e = plan.num_nodes, plan.num_edges
            z, _, nm, em = bridge.marginals(plan, K,
                                            nodes[n0 * K:(n0 + n) * K].astype(np.float64),
                                            edges[e0 * K * K:(e0 + e) * K * K].astype(np.float64))
            assert abs(log_z[t] - z) <= 1e-6 * max(1.0, abs(z))
            assert np.max(np.abs(node_m[n0 * K:(n0 + n) * K] - nm)) <= 1e-5
            assert np.max(np.abs(edge_m[e0 * K * K:(e0 + e) * K * K] - em)) <= 1e-5
            n0, e0 = n0 + n, e0 + e
            checked += 1
    assert checked == len(parents)


def test_categorical_forest_streamed_in_windows(gpu):
    """Observations written on the device: device_inputs_ready() rebuilds the
    phase schedule's phase-ordered copy of them."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    K = 4
    parents = [synthetic.random_recursive(rng, int(n)) for n in (400, 120, 900, 60)]
    root = (rng.random(K) + 0.1).astype(np.float32)
    emission = (rng.random(K * K) + 0.1).astype(np.float32)
    ws = gpu.Workspace()
    for window in windows(parents, 2):
        plans = [gpu.Plan(p) for p in window]
        observed = [synthetic.leaves(p) for p in window]
        ws.reserve_forest_categorical(plans, K, K, observed, kind="marginals,device",
                                      scalar=np.float32)
        assert ws.tuning["schedule"] == 1
        with pytest.raises(gpu.LogicError):  # device-only: no host staging
            ws.categorical_inputs()
        e_total = sum(p.num_edges for p in plans)
        edges = synthetic.stochastic_edges(rng, e_total, K, 0.5, np.float32)
        obs = rng.integers(0, K, sum(len(o) for o in observed)).astype(np.uint8)
        buffers = ws.device_buffers()
        buffers["edge_potentials"].copy_(torch.from_numpy(edges))
        buffers["observations"].copy_(torch.from_numpy(obs))
        buffers["root_potential"].copy_(torch.from_numpy(root))
        buffers["emission_potentials"].copy_(torch.from_numpy(emission))
        torch.cuda.synchronize()
        ws.device_inputs_ready()
        ws.enqueue(1)  # log partition
        ws.synchronize()
        log_z = buffers["values"].cpu().numpy()
        e0 = o0 = 0
        for t, plan in enumerate(plans):
            e, o = plan.num_edges, len(observed[t])
            dense = np.ones((plan.num_nodes, K), dtype=np.float32)
            dense[plan.root] = root
            dense[observed[t]] = dense[observed[t]] * emission.reshape(K, K)[obs[o0:o0 + o]]
            z = bridge.log_partition(plan, K, dense.astype(np.float64).ravel(),
                                     edges[e0 * K * K:(e0 + e) * K * K].astype(np.float64))
            assert abs(log_z[t] - z) <= 1e-6 * max(1.0, abs(z))
            e0, o0 = e0 + e, o0 + o
