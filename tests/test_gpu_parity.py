"""GPU parity: the accelerator (through the C ABI) against the oracle.

Tolerances:
  * log Z: relative error <= 1e-6 against the FP64 oracle (FP32 arithmetic
    with exact power-of-two scaling); 1e-12 with FP64 arithmetic.
  * marginals (node and edge posteriors, = d log Z / d log factors): absolute
    error <= 1e-5 against the FP64 oracle; 1e-11 with FP64 arithmetic.
  * MAP states and weights, posterior samples: bit-exact against the oracle run
    with the same reproducible exp/log (oracle MATH_PORTABLE) in the same
    precision.
"""
import numpy as np
import pytest

from oracle import bridge
from parallel_tree_hmm_gb300 import synthetic

pytestmark = pytest.mark.gpu

LOG_Z_RTOL = {np.float32: 1e-6, np.float64: 1e-12}
MARGINAL_ATOL = {np.float32: 1e-5, np.float64: 1e-11}


def trees(rng):
    return {
        "root_only": np.array([-1]),
        "pair": np.array([-1, 0]),
        "reference_fixture": np.array([-1, 0, 0, 1, 3]),
        "chain": np.arange(-1, 63),
        "star": np.array([-1] + [0] * 17),
        "binary": synthetic.leaf_splitting(rng, 201),
        "recursive": synthetic.random_recursive(rng, 700),
        "caterpillar": synthetic.caterpillar(300),
        "spine_heavy": synthetic.spine_heavy(rng, 500),
    }


def dense_inputs(rng, plan, states, batch, zeros=0.0, dtype=np.float64):
    nodes = rng.random((batch, plan.num_nodes, states)) * 0.9 + 0.1
    edges = rng.random((plan.num_edges, states, states)) * 0.9 + 0.1
    if zeros:
        nodes[rng.random(nodes.shape) < zeros] = 0.0
        edges[rng.random(edges.shape) < zeros] = 0.0
    return nodes.astype(dtype), edges.astype(dtype).ravel()


@pytest.mark.parametrize("compute", [np.float32, np.float64])
@pytest.mark.parametrize("scalar", [np.float32, np.float64])
@pytest.mark.parametrize("states", [1, 2, 3, 4, 5, 8, 9, 16, 20, 32])
def test_marginals_against_fp64_oracle(gpu, states, scalar, compute):
    rng = np.random.default_rng(states * 7 + (scalar == np.float32))
    for name, parents in trees(rng).items():
        if states >= 16 and name in ("recursive", "spine_heavy"):
            parents = parents[:120]
        plan = gpu.Plan(parents)
        batch = 3
        nodes, edges = dense_inputs(rng, plan, states, batch, dtype=scalar)
        ws = gpu.Workspace()
        ws.reserve_marginals(plan, states, batch, scalar=scalar, compute=compute)
        view = ws.posterior_marginals_prepared(
            gpu.BatchedModelView(plan, states, batch, nodes.ravel(), edges))
        got_nodes = view.nodes.reshape(batch, -1)
        got_edges = view.edges.reshape(batch, -1)
        rtol = max(LOG_Z_RTOL[compute], LOG_Z_RTOL[scalar])
        atol = max(MARGINAL_ATOL[compute], MARGINAL_ATOL[scalar] * 10)
        for b in range(batch):
            log_z, _, node_m, edge_m = bridge.marginals(
                plan, states, nodes[b].astype(np.float64).ravel(), edges.astype(np.float64))
            assert abs(view.log_partitions[b] - log_z) <= rtol * max(1, abs(log_z)), name
            assert np.max(np.abs(got_nodes[b] - node_m), initial=0) <= atol, name
            assert np.max(np.abs(got_edges[b] - edge_m), initial=0) <= atol, name


@pytest.mark.parametrize("scalar", [np.float32, np.float64])
def test_log_partition_and_partition(gpu, scalar):
    rng = np.random.default_rng(11)
    for name, parents in trees(rng).items():
        plan = gpu.Plan(parents)
        states, batch = 4, 5
        nodes, edges = dense_inputs(rng, plan, states, batch, dtype=scalar)
        ws = gpu.Workspace()
        ws.reserve(plan, states, batch, scalar=scalar)
        model = gpu.BatchedModelView(plan, states, batch, nodes.ravel(), edges)
        log_view = ws.log_partition_function_prepared(model)
        expected = [bridge.log_partition(plan, states, nodes[b].astype(np.float64).ravel(),
                                         edges.astype(np.float64)) for b in range(batch)]
        np.testing.assert_allclose(log_view.values, expected, rtol=1e-6, atol=1e-6,
                                   err_msg=name)
        raw_view = ws.partition_function_prepared(model)
        # Raw Z leaves the float32 range on large trees; inf is then correct.
        with np.errstate(over="ignore"):
            expected_raw = np.exp(np.asarray(expected)).astype(scalar)
        np.testing.assert_allclose(raw_view.values, expected_raw, rtol=2e-5,
                                   err_msg=name)
        assert raw_view.timings.kernel_ms >= 0


@pytest.mark.parametrize("scalar", [np.float32, np.float64])
@pytest.mark.parametrize("states", [1, 2, 3, 4, 8, 9, 20])
def test_map_bit_exact(gpu, states, scalar):
    rng = np.random.default_rng(100 + states)
    for name, parents in trees(rng).items():
        plan = gpu.Plan(parents)
        batch = 4
        nodes, edges = dense_inputs(rng, plan, states, batch, zeros=0.05, dtype=scalar)
        ws = gpu.Workspace()
        ws.reserve_maximum(plan, states, batch, scalar=scalar)
        expected = []
        for b in range(batch):
            try:
                expected.append(bridge.maximum(plan, states, nodes[b].ravel(), edges,
                                               scalar, bridge.MATH_PORTABLE))
            except bridge.OracleError:
                expected.append(None)
        model = gpu.BatchedModelView(plan, states, batch, nodes.ravel(), edges)
        if any(e is None for e in expected):
            with pytest.raises(gpu.DomainError):
                ws.maximum_a_posteriori_prepared(model)
            continue
        view = ws.maximum_a_posteriori_prepared(model)
        got_states = view.states.reshape(batch, -1)
        for b in range(batch):
            assert view.log_weights[b] == expected[b][0], name
            assert np.array_equal(got_states[b], expected[b][1]), name


@pytest.mark.parametrize("scalar", [np.float32, np.float64])
@pytest.mark.parametrize("states", [1, 2, 3, 4, 8, 9, 20])
def test_sampling_bit_exact(gpu, states, scalar):
    rng = np.random.default_rng(200 + states)
    for name, parents in trees(rng).items():
        plan = gpu.Plan(parents)
        batch = 4
        nodes, edges = dense_inputs(rng, plan, states, batch, dtype=scalar)
        uniforms = rng.random((batch, plan.num_nodes)).astype(scalar)
        ws = gpu.Workspace()
        ws.reserve_sampling(plan, states, batch, scalar=scalar)
        view = ws.posterior_sample_prepared(
            gpu.BatchedModelView(plan, states, batch, nodes.ravel(), edges),
            uniforms.ravel())
        got = view.states.reshape(batch, -1)
        for b in range(batch):
            expected = bridge.sample(plan, states, nodes[b].ravel(), edges, uniforms[b],
                                     scalar, bridge.MATH_PORTABLE)
            assert np.array_equal(got[b], expected), name


def test_sampling_rejects_invalid_uniform(gpu):
    plan = gpu.Plan([-1, 0, 1, 1, 0, 4, 5, 5])
    states, batch = 4, 5
    rng = np.random.default_rng(3)
    nodes, edges = dense_inputs(rng, plan, states, batch)
    ws = gpu.Workspace()
    ws.reserve_sampling(plan, states, batch)
    staged = ws.inputs(batch)
    staged.node_potentials[:] = nodes.ravel()
    staged.edge_potentials[:] = edges
    uniforms = ws.uniforms(batch)
    uniforms[:] = rng.random(uniforms.size)
    ws.posterior_sample_prepared(staged, uniforms)
    uniforms[0] = 1.0
    with pytest.raises(gpu.InvalidArgument):
        ws.posterior_sample_prepared(staged, uniforms)


@pytest.mark.parametrize("scalar", [np.float32, np.float64])
def test_categorical_marginals_and_residency(gpu, scalar):
    rng = np.random.default_rng(5)
    parents = synthetic.random_recursive(rng, 400)
    plan = gpu.Plan(parents)
    observed = synthetic.leaves(parents)
    states, batch, categories = 4, 6, 5
    ws = gpu.Workspace()
    ws.reserve_categorical_marginals(plan, states, batch, categories, observed,
                                     scalar=scalar)
    staged = ws.categorical_inputs(batch)
    staged.observations[:] = rng.integers(0, categories, staged.observations.size)
    staged.root_potential[:] = rng.random(states) + 0.1
    staged.emission_potentials[:] = rng.random(categories * states) + 0.05
    staged.edge_potentials[:] = synthetic.stochastic_edges(rng, plan.num_edges, states, 0.5)
    view = ws.posterior_marginals_prepared(staged, gpu.CategoricalInputUpdate.kAll)
    obs = staged.observations.reshape(batch, -1)
    for b in range(batch):
        dense = np.ones((plan.num_nodes, states))
        dense[plan.root] = staged.root_potential
        for slot, node in enumerate(observed):
            category = obs[b, slot]
            emission = (staged.emission_potentials.reshape(categories, states)[category]
                        if category < categories else np.zeros(states))
            dense[node] = dense[node] * emission
        dense = dense.astype(scalar).astype(np.float64)
        try:
            log_z, _, node_m, edge_m = bridge.marginals(
                plan, states, dense.ravel(), staged.edge_potentials.astype(np.float64))
        except bridge.OracleError:
            continue
        assert abs(view.log_partitions[b] - log_z) <= 1e-6 * max(1, abs(log_z))
        assert np.max(np.abs(view.nodes.reshape(batch, -1)[b] - node_m)) <= 1e-5
        assert np.max(np.abs(view.edges.reshape(batch, -1)[b] - edge_m)) <= 1e-5


def test_out_of_range_category_has_zero_emission(gpu):
    # A category >= categories contributes an all-zero emission
    # (src/gpu_backend_impl.inc:366-378): Z = 0, log Z = -inf, and the
    # marginal call reports a domain error like the reference.
    plan = gpu.Plan([-1, 0, 0])
    ws = gpu.Workspace()
    ws.reserve_categorical_marginals(plan, 2, 2, 2, np.array([1, 2], dtype=np.uint32))
    model = gpu.BatchedCategoricalModelView(
        plan, 2, 2, 2, np.array([1, 2], dtype=np.uint32),
        np.array([0, 1, 1, 2], dtype=np.uint8), np.array([0.4, 0.6]),
        np.array([0.9, 0.1, 0.2, 0.8]), np.full(2 * 4, 0.5))
    with pytest.raises(gpu.DomainError):
        ws.posterior_marginals_prepared(model, gpu.CategoricalInputUpdate.kAll)
    log_z = ws.log_partition_function_prepared(model, gpu.CategoricalInputUpdate.kAll)
    assert np.isfinite(log_z.values[0]) and log_z.values[1] == -np.inf


def test_categorical_residency_rules(gpu):
    plan = gpu.Plan([-1, 0, 0, 1, 1, 2, 2])
    states, batch, categories = 4, 5, 4
    observed = np.array([3, 4, 5, 6], dtype=np.uint32)
    ws = gpu.Workspace()
    ws.reserve_categorical(plan, states, batch, categories, observed)
    rng = np.random.default_rng(1)
    observations = (np.arange(batch * 4) % categories).astype(np.uint8)
    root = 0.1 * np.arange(1, states + 1)
    emission = np.eye(states)
    edges = 0.02 + 0.003 * rng.random(plan.num_edges * states * states)
    model = gpu.BatchedCategoricalModelView(plan, states, batch, categories, observed,
                                            observations, root, emission, edges)
    for update in (gpu.CategoricalInputUpdate.kFactors, gpu.CategoricalInputUpdate.kNone):
        with pytest.raises(gpu.LogicError):
            ws.log_partition_function_prepared(model, update)
    baseline = ws.log_partition_function_prepared(model, gpu.CategoricalInputUpdate.kAll).values.copy()
    observations[0] = (observations[0] + 1) % categories
    reused = ws.log_partition_function_prepared(model, gpu.CategoricalInputUpdate.kFactors).values.copy()
    assert np.array_equal(reused, baseline)
    updated = ws.log_partition_function_prepared(model, gpu.CategoricalInputUpdate.kAll).values.copy()
    assert not np.array_equal(updated, baseline)
    edges *= 0.9
    kept = ws.log_partition_function_prepared(model, gpu.CategoricalInputUpdate.kNone).values.copy()
    assert np.array_equal(kept, updated)
    changed = ws.log_partition_function_prepared(model, gpu.CategoricalInputUpdate.kFactors).values.copy()
    assert not np.array_equal(changed, updated)
    tail = gpu.BatchedCategoricalModelView(plan, states, 3, categories, observed,
                                           observations[:12], root, emission, edges)
    with pytest.raises(gpu.LogicError):
        ws.log_partition_function_prepared(tail, gpu.CategoricalInputUpdate.kFactors)
    ws.reserve_categorical(plan, states, batch, categories, observed)
    with pytest.raises(gpu.LogicError):
        ws.log_partition_function_prepared(model, gpu.CategoricalInputUpdate.kNone)


@pytest.mark.parametrize("states", [4, 8, 20])
def test_forest_marginals(gpu, states):
    rng = np.random.default_rng(states)
    shapes = [synthetic.random_recursive(rng, int(n)) for n in (1, 2, 50, 900, 3000, 5000)]
    shapes += [synthetic.caterpillar(int(n)) for n in (7, 400, 4100)]
    plans = [gpu.Plan(p) for p in shapes]
    node_total = sum(p.num_nodes for p in plans)
    edge_total = sum(p.num_edges for p in plans)
    nodes = rng.random(node_total * states) + 0.05
    edges = synthetic.stochastic_edges(rng, edge_total, states, 0.5)
    ws = gpu.Workspace()
    ws.reserve_forest(plans, states, kind="marginals", scalar=np.float32)
    view = ws.posterior_marginals_prepared(
        gpu.BatchedModelView(None, states, len(plans), nodes.astype(np.float32),
                             edges.astype(np.float32)))
    n0 = e0 = 0
    for t, plan in enumerate(plans):
        n1, e1 = n0 + plan.num_nodes, e0 + plan.num_edges
        tree_nodes = nodes[n0 * states:n1 * states].astype(np.float32).astype(np.float64)
        tree_edges = edges[e0 * states**2:e1 * states**2].astype(np.float32).astype(np.float64)
        log_z, _, node_m, edge_m = bridge.marginals(plan, states, tree_nodes, tree_edges)
        assert abs(view.log_partitions[t] - log_z) <= 1e-6 * max(1, abs(log_z))
        assert np.max(np.abs(view.nodes[n0 * states:n1 * states] - node_m)) <= 1e-5
        assert np.max(np.abs(view.edges[e0 * states**2:e1 * states**2] - edge_m),
                      initial=0) <= 1e-5
        n0, e0 = n1, e1


def test_long_chain_does_not_underflow(gpu):
    n = 4096
    plan = gpu.Plan(np.arange(-1, n - 1))
    ws = gpu.Workspace()
    ws.reserve(plan, 1, 1)
    view = ws.log_partition_function_prepared(
        gpu.BatchedModelView(plan, 1, 1, np.full(n, 0.5), np.ones(n - 1)))
    assert abs(view.values[0] - n * np.log(0.5)) <= 2e-3
    raw = ws.partition_function_prepared(
        gpu.BatchedModelView(plan, 1, 1, np.full(n, 0.5), np.ones(n - 1)))
    assert raw.values[0] == 0.0


def test_enqueue_matches_prepared_call(gpu):
    rng = np.random.default_rng(9)
    plan = gpu.Plan(synthetic.random_recursive(rng, 1000))
    states, batch = 4, 16
    nodes, edges = dense_inputs(rng, plan, states, batch, dtype=np.float32)
    ws = gpu.Workspace()
    ws.reserve_marginals(plan, states, batch, scalar=np.float32)
    first = ws.posterior_marginals_prepared(
        gpu.BatchedModelView(plan, states, batch, nodes.ravel(), edges))
    values = first.log_partitions.copy()
    # Phase schedule (the default at K <= 4) in the batch API's shared-topology
    # layout: every round grid-wide (all items have every round, so there is
    # no per-tree tail whatever phase_rounds asks): gather and compress
    # launches per round, the finish launch, two adjoint launches per round.
    assert ws.tuning["phase_rounds"] == plan.num_rounds
    assert plan.num_rounds * 2 + 1 <= ws.launches <= plan.num_rounds * 4 + 1
    ws.set_tuning(1024, schedule=1, phase_rounds=2)
    assert ws.tuning["phase_rounds"] == plan.num_rounds
    ws.set_tuning(1024, schedule=0)
    ws.posterior_marginals_prepared(
        gpu.BatchedModelView(plan, states, batch, nodes.ravel(), edges))
    assert ws.launches == 2  # per-tree teams: forward sweep, then adjoint sweep
    assert ws.enqueue(4) == batch * plan.num_nodes
    ws.synchronize()
    again = ws.posterior_marginals_prepared(
        gpu.BatchedModelView(plan, states, batch, nodes.ravel(), edges))
    assert np.array_equal(again.log_partitions, values)


def test_galton_watson_categorical_map_and_sampling_bit_exact(gpu):
    """MAP and sampling on the MAP+sampling workload's tree and factor shapes
    (Poisson(2) Galton-Watson trees, K = 8, byte leaf observations with a
    Dirichlet(2) emission table, Dirichlet(0.3) edge rows), categorical
    forest, FP32: states, weights and draws bit-exact against the oracle."""
    rng = np.random.default_rng(2024)
    K = 8
    parents = [synthetic.galton_watson(rng, 1000, 4000) for _ in range(3)]
    plans = [gpu.Plan(p) for p in parents]
    observed = [synthetic.leaves(p) for p in parents]
    root = synthetic.dirichlet_rows(rng, 1, K, 1.0, np.float32).ravel()
    emission = synthetic.dirichlet_rows(rng, K, K, 2.0, np.float32)
    edges = [synthetic.dirichlet_rows(rng, (len(p) - 1) * K, K, 0.3, np.float32).ravel()
             for p in parents]
    obs = [rng.integers(0, K, len(o), dtype=np.uint8) for o in observed]
    uniforms = [rng.random(len(p)).astype(np.float32) for p in parents]
    ws = gpu.Workspace()
    ws.reserve_forest_categorical(plans, K, K, observed, kind="maximum,sampling",
                                  scalar=np.float32)
    staged = ws.categorical_inputs()
    staged.root_potential[:] = root
    staged.emission_potentials[:] = emission.ravel()
    staged.edge_potentials[:] = np.concatenate(edges)
    staged.observations[:] = np.concatenate(obs)
    u = ws.uniforms()
    u[:] = np.concatenate(uniforms)
    map_view = ws.maximum_a_posteriori_prepared(staged, 0)
    # Result spans live in workspace memory until the next call: copy them.
    map_weights, map_states = np.array(map_view.log_weights), np.array(map_view.states)
    sample_states = np.array(ws.posterior_sample_prepared(staged, u, 2).states)
    node0 = 0
    for t, plan in enumerate(plans):
        n = plan.num_nodes
        dense = np.ones((n, K), dtype=np.float32)
        dense[0] = root
        dense[observed[t]] = dense[observed[t]] * emission[obs[t]]
        weight, states = bridge.maximum(plan, K, dense.ravel(), edges[t], np.float32,
                                        bridge.MATH_PORTABLE)
        assert map_weights[t] == weight
        assert np.array_equal(map_states[node0:node0 + n], states)
        draw = bridge.sample(plan, K, dense.ravel(), edges[t], uniforms[t], np.float32,
                             bridge.MATH_PORTABLE)
        assert np.array_equal(sample_states[node0:node0 + n], draw)
        node0 += n


def test_plain_method_configuration(gpu):
    """The reference's CPU-runnable case: 64 binary trees of 999 nodes grown by
    uniform leaf splitting, K = 4, Dirichlet(1) root factor and edge rows,
    byte observations on the leaves with a Dirichlet(5) emission table,
    all-ones internal factors; log Z and marginals for every tree against the
    FP64 oracle (FP32 arithmetic)."""
    rng = np.random.default_rng(1999)
    K, trees = 4, 64
    parents = [synthetic.leaf_splitting(rng, 999) for _ in range(trees)]
    plans = gpu.Plan.many(parents)
    observed = [synthetic.leaves(p) for p in parents]
    root = synthetic.dirichlet_rows(rng, 1, K, 1.0, np.float32).ravel()
    emission = synthetic.dirichlet_rows(rng, K, K, 5.0, np.float32)
    edges = [synthetic.dirichlet_rows(rng, (len(p) - 1) * K, K, 1.0, np.float32).ravel()
             for p in parents]
    obs = [rng.integers(0, K, len(o), dtype=np.uint8) for o in observed]
    ws = gpu.Workspace()
    ws.reserve_forest_categorical(plans, K, K, observed, kind="marginals", scalar=np.float32)
    staged = ws.categorical_inputs()
    staged.root_potential[:] = root
    staged.emission_potentials[:] = emission.ravel()
    staged.edge_potentials[:] = np.concatenate(edges)
    staged.observations[:] = np.concatenate(obs)
    view = ws.posterior_marginals_prepared(staged, gpu.CategoricalInputUpdate.kAll)
    n0 = e0 = 0
    for t, plan in enumerate(plans):
        n, e = plan.num_nodes, plan.num_edges
        dense = np.ones((n, K), dtype=np.float32)
        dense[plan.root] = root
        dense[observed[t]] = dense[observed[t]] * emission[obs[t]]
        log_z, _, node_m, edge_m = bridge.marginals(
            plan, K, dense.astype(np.float64).ravel(), edges[t].astype(np.float64))
        assert abs(view.log_partitions[t] - log_z) <= 1e-6 * max(1, abs(log_z))
        assert np.max(np.abs(view.nodes[n0 * K:(n0 + n) * K] - node_m)) <= 1e-5
        assert np.max(np.abs(view.edges[e0 * K * K:(e0 + e) * K * K] - edge_m)) <= 1e-5
        n0, e0 = n0 + n, e0 + e


@pytest.mark.parametrize("categorical", [False, True])
def test_shared_topology_batch_of_257(gpu, categorical):
    """The reference's batch API (one plan, B node-factor sets, one shared
    edge input) at B = 257, more than one block of batch items
    (tests/accelerator_test.h:24 of the reference): the shared-topology phase
    layout, where every item reads the one tree's records and the shared
    edge rows together, against the FP64 oracle, and bit-identical to the
    per-tree schedule. Dense and categorical inputs, log Z and marginals,
    and a call on the first 100 items only."""
    rng = np.random.default_rng(257)
    K, B = 4, 257
    parents = synthetic.random_recursive(rng, 400)
    plan = gpu.Plan(parents)
    edges = synthetic.stochastic_edges(rng, plan.num_edges, K, 0.7, np.float32)
    ws = gpu.Workspace()
    if categorical:
        observed = synthetic.leaves(parents)
        ws.reserve_categorical_marginals(plan, K, B, K, observed, scalar=np.float32)
        staged = ws.categorical_inputs(B)
        staged.root_potential[:] = rng.random(K) + 0.1
        staged.emission_potentials[:] = rng.random(K * K) + 0.1
        staged.edge_potentials[:] = edges
        staged.observations[:] = rng.integers(0, K, staged.observations.size)
        model = staged
        dense = np.ones((B, plan.num_nodes, K), dtype=np.float32)
        dense[:, plan.root] = staged.root_potential
        obs = np.array(staged.observations).reshape(B, -1)
        emission = np.array(staged.emission_potentials).reshape(K, K)
        dense[:, observed] = dense[:, observed] * emission[obs]
        dense = dense.astype(np.float64)
    else:
        ws.reserve_marginals(plan, K, B, scalar=np.float32)
        nodes = (rng.random((B, plan.num_nodes, K)) * 0.9 + 0.1).astype(np.float32)
        model = gpu.BatchedModelView(plan, K, B, nodes.ravel(), edges)
        dense = nodes.astype(np.float64)
    assert ws.tuning["schedule"] == 1
    view = ws.posterior_marginals_prepared(model)
    got = [np.array(view.log_partitions), np.array(view.nodes), np.array(view.edges)]
    nodes_out = got[1].reshape(B, -1)
    edges_out = got[2].reshape(B, -1)
    for b in range(0, B, 16):
        log_z, _, node_m, edge_m = bridge.marginals(plan, K, dense[b].ravel(),
                                                    edges.astype(np.float64))
        assert abs(got[0][b] - log_z) <= 1e-6 * max(1.0, abs(log_z))
        assert np.max(np.abs(nodes_out[b] - node_m)) <= 1e-5
        assert np.max(np.abs(edges_out[b] - edge_m)) <= 1e-5
    ws.set_tuning(1024, schedule=0)
    teams = ws.posterior_marginals_prepared(model)
    assert np.array_equal(np.array(teams.log_partitions), got[0])
    assert np.array_equal(np.array(teams.nodes), got[1])
    assert np.array_equal(np.array(teams.edges), got[2])
    if not categorical:
        ws.set_tuning(1024, schedule=1)
        part = ws.log_partition_function_prepared(
            gpu.BatchedModelView(plan, K, 100, nodes[:100].ravel(), edges))
        assert np.array_equal(np.array(part.values), got[0][:100])
