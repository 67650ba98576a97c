"""Launch tuning, schedules and graph replay change no result bit.

The team threshold (which trees a whole CTA contracts instead of one warp),
the CTAs per SM of each kernel and CUDA-graph replay of the device-only step
only move work between SMs, CTAs and warps; the phase schedule (every round
of every tree in one grid-wide launch, K <= 4) performs each operation's
arithmetic in the same order and carries the power-of-two exponents with the
stored values instead of per team, whichever rounds run grid-wide and which
run in one warp per tree. Every operation's floating-point result
and the integer exponent sums are the same, so every output must be
bit-identical across all of them.
"""
import numpy as np
import pytest

from parallel_tree_hmm_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu

TEAMS = _lib.THMM_SCHEDULE_TEAMS
PHASES = _lib.THMM_SCHEDULE_PHASES


def forest(gpu, rng, states):
    shapes = [synthetic.random_recursive(rng, int(n)) for n in (1, 60, 700, 1500, 5000)]
    shapes += [synthetic.caterpillar(int(n)) for n in (9, 300, 2600)]
    plans = [gpu.Plan(p) for p in shapes]
    node_total = sum(p.num_nodes for p in plans)
    edge_total = sum(p.num_edges for p in plans)
    nodes = (rng.random(node_total * states) + 0.05).astype(np.float32)
    edges = synthetic.stochastic_edges(rng, edge_total, states, 0.5).astype(np.float32)
    return plans, nodes, edges


def outputs(view):
    return [np.array(view.log_partitions), np.array(view.nodes), np.array(view.edges)]


@pytest.mark.parametrize("states", [4, 8, 13, 20, 22, 27, 32])
def test_tunings_give_identical_marginals(gpu, states):
    rng = np.random.default_rng(40 + states)
    plans, nodes, edges = forest(gpu, rng, states)
    ws = gpu.Workspace()
    ws.reserve_forest(plans, states, kind="marginals", scalar=np.float32)
    model = gpu.BatchedModelView(None, states, len(plans), nodes, edges)
    # The phase schedule is the forest default; above 4 states it has no
    # tail, so every phase_rounds setting runs all rounds grid-wide.
    assert ws.tuning["schedule"] == PHASES
    reference = outputs(ws.posterior_marginals_prepared(model))
    settings = [(1, (0, 0, 0, 0)),          # every tree to a CTA team
                (1 << 31, (0, 0, 0, 0)),    # every tree to a warp team
                (1000, (1, 0, 0, 1)),       # one CTA per SM for both sweeps
                (300, (2, 0, 0, 3))]
    for schedule, phase_rounds in ((TEAMS, 0), (PHASES, 0), (PHASES, 1), (PHASES, 3),
                                   (PHASES, 99)):
        for threshold, caps in settings:
            ws.set_tuning(threshold, caps, schedule=schedule, phase_rounds=phase_rounds)
            assert ws.tuning["team_threshold"] == threshold
            assert ws.tuning["ctas_per_sm"] == list(caps)
            assert ws.tuning["schedule"] == schedule
            got = outputs(ws.posterior_marginals_prepared(model))
            for a, b in zip(got, reference):
                assert np.array_equal(a, b)
            log_z = np.array(ws.log_partition_function_prepared(model).values)
            assert np.array_equal(log_z, reference[0])
    chosen = ws.autotune(4, repeats=1)
    assert chosen["candidates"] >= 2 and chosen["kernel_ms"] > 0
    assert ws.tuning["team_threshold"] == chosen["team_threshold"]
    got = outputs(ws.posterior_marginals_prepared(model))
    for a, b in zip(got, reference):
        assert np.array_equal(a, b)


def test_lane_group_phases_replay(gpu):
    """4 < K <= 32 on the phase schedule (one lane group per operation, no
    tail): graph replay gives the prepared call's bits, with one launch per
    kind and round."""
    rng = np.random.default_rng(78)
    plans, nodes, edges = forest(gpu, rng, 20)
    ws = gpu.Workspace()
    ws.reserve_forest(plans, 20, kind="marginals", scalar=np.float32)
    rounds = max(p.num_rounds for p in plans)
    assert ws.tuning["schedule"] == PHASES and ws.tuning["phase_rounds"] == rounds
    ws.set_tuning(1024, schedule=PHASES, phase_rounds=2)
    assert ws.tuning["phase_rounds"] == rounds
    model = gpu.BatchedModelView(None, 20, len(plans), nodes, edges)
    reference = outputs(ws.posterior_marginals_prepared(model))
    total = sum(p.num_nodes for p in plans)
    for _ in range(3):
        assert ws.enqueue(4) == total
    ws.synchronize()
    assert 2 * rounds + 1 <= ws.launches <= 4 * rounds + 1
    ws.set_tuning(1024, schedule=TEAMS)
    for a, b in zip(outputs(ws.posterior_marginals_prepared(model)), reference):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("schedule", [TEAMS, PHASES])
def test_graph_replay_matches_prepared_call(gpu, schedule):
    rng = np.random.default_rng(77)
    plans, nodes, edges = forest(gpu, rng, 4)
    ws = gpu.Workspace()
    ws.reserve_forest(plans, 4, kind="marginals", scalar=np.float32)
    rounds = max(p.num_rounds for p in plans)
    ws.set_tuning(1024, schedule=schedule, phase_rounds=rounds)
    model = gpu.BatchedModelView(None, 4, len(plans), nodes, edges)
    reference = outputs(ws.posterior_marginals_prepared(model))
    staged = ws.inputs()
    total = sum(p.num_nodes for p in plans)
    for _ in range(3):  # capture, then two replays
        assert ws.enqueue(4) == total
    ws.synchronize()
    if schedule == TEAMS:
        assert ws.launches == 2
    else:  # gather + compress per round, finish, two adjoint phases per round
        assert 2 * rounds + 1 <= ws.launches <= 4 * rounds + 1
        # Two grid-wide rounds, then one warp per tree: two tail launches.
        ws.set_tuning(1024, schedule=schedule, phase_rounds=2)
        assert ws.tuning["phase_rounds"] == 2
        ws.enqueue(4)
        ws.synchronize()
        assert 2 * 2 + 3 <= ws.launches <= 2 * 4 + 3
        ws.set_tuning(1024, schedule=schedule, phase_rounds=rounds)
    # Outputs of the replays are in device memory; a kNone-style rerun through
    # the prepared call downloads the same values.
    got = outputs(ws.posterior_marginals_prepared(
        gpu.BatchedModelView(None, 4, len(plans), staged.node_potentials,
                             staged.edge_potentials)))
    for a, b in zip(got, reference):
        assert np.array_equal(a, b)
    ws.set_tuning(1, (0, 0, 0, 0))  # drops the graph; the next enqueue recaptures
    ws.enqueue(4)
    ws.enqueue(1)
    ws.synchronize()


def test_map_and_sampling_tuning_identical(gpu):
    rng = np.random.default_rng(5)
    plans, nodes, edges = forest(gpu, rng, 4)
    ws = gpu.Workspace()
    ws.reserve_forest(plans, 4, kind="maximum,sampling", scalar=np.float32)
    model = gpu.BatchedModelView(None, 4, len(plans), nodes, edges)
    uniforms = rng.random(sum(p.num_nodes for p in plans)).astype(np.float32)
    map_ref = ws.maximum_a_posteriori_prepared(model)
    map_states = np.array(map_ref.states)
    map_weights = np.array(map_ref.log_weights)
    sample_ref = np.array(ws.posterior_sample_prepared(model, uniforms).states)
    for threshold in (1, 1 << 31):
        ws.set_tuning(threshold, (0, 1, 1, 0))
        again = ws.maximum_a_posteriori_prepared(model)
        assert np.array_equal(again.states, map_states)
        assert np.array_equal(again.log_weights, map_weights)
        assert np.array_equal(ws.posterior_sample_prepared(model, uniforms).states,
                              sample_ref)
    ws.autotune(3, repeats=1)
    assert np.array_equal(ws.posterior_sample_prepared(model, uniforms).states, sample_ref)


@pytest.mark.parametrize("states", [4, 20])
def test_striped_calls_match_single_stripe(gpu, states):
    """Prepared calls cut into stripes (overlapped copies and kernels) return
    the same bits as one stripe: dense and categorical forests, the batch API
    with shared edges, every operation."""
    rng = np.random.default_rng(11)
    plans, nodes, edges = forest(gpu, rng, states)
    total = sum(p.num_nodes for p in plans)
    uniforms = rng.random(total).astype(np.float32)
    ws = gpu.Workspace()
    ws.reserve_forest(plans, states, kind="marginals", scalar=np.float32)
    model = gpu.BatchedModelView(None, states, len(plans), nodes, edges)
    ws.set_tuning(1024, stripes=1, schedule=TEAMS)
    single = outputs(ws.posterior_marginals_prepared(model))
    single_log_z = np.array(ws.log_partition_function_prepared(model).values)
    for schedule in (TEAMS, PHASES):
        for stripes in (2, 3, 8):
            ws.set_tuning(1024, stripes=stripes, schedule=schedule)
            assert ws.tuning["stripes"] == stripes
            for a, b in zip(outputs(ws.posterior_marginals_prepared(model)), single):
                assert np.array_equal(a, b)
            # Stripes balance nodes, so a dominant tree can merge stripes.
            if schedule == TEAMS:
                assert ws.launches % 2 == 0 and 2 <= ws.launches <= 2 * stripes
            assert np.array_equal(ws.log_partition_function_prepared(model).values,
                                  single_log_z)

    ws2 = gpu.Workspace()
    ws2.reserve_forest(plans, states, kind="maximum,sampling", scalar=np.float32)
    ws2.set_tuning(1024, stripes=1)
    map1 = ws2.maximum_a_posteriori_prepared(model)
    map_states, map_weights = np.array(map1.states), np.array(map1.log_weights)
    sample1 = np.array(ws2.posterior_sample_prepared(model, uniforms).states)
    ws2.set_tuning(1024, stripes=5)
    map5 = ws2.maximum_a_posteriori_prepared(model)
    assert np.array_equal(map5.states, map_states)
    assert np.array_equal(map5.log_weights, map_weights)
    assert np.array_equal(ws2.posterior_sample_prepared(model, uniforms).states, sample1)


def test_striped_categorical_and_batch_api(gpu):
    rng = np.random.default_rng(12)
    K = 4
    plans = [gpu.Plan(synthetic.random_recursive(rng, int(n))) for n in (40, 900, 2000, 3100)]
    observed = [np.arange(1, p.num_nodes, 2, dtype=np.uint32) for p in plans]
    ws = gpu.Workspace()
    ws.reserve_forest_categorical(plans, K, K, observed, kind="marginals",
                                  scalar=np.float32)
    staged = ws.categorical_inputs()
    staged.root_potential[:] = rng.random(K) + 0.1
    staged.emission_potentials[:] = rng.random(K * K) + 0.1
    staged.edge_potentials[:] = rng.random(staged.edge_potentials.size) + 0.1
    staged.observations[:] = rng.integers(0, K, staged.observations.size)
    ws.set_tuning(1024, stripes=1, schedule=TEAMS)
    single = outputs(ws.posterior_marginals_prepared(staged, 0))  # kAll
    for schedule in (TEAMS, PHASES):
        ws.set_tuning(1024, stripes=3, schedule=schedule)
        for update in (0, 1, 2):  # kAll, kFactors, kNone
            for a, b in zip(outputs(ws.posterior_marginals_prepared(staged, update)),
                            single):
                assert np.array_equal(a, b)

    plan = gpu.Plan(synthetic.random_recursive(rng, 600))
    batch = 7
    dense_nodes = (rng.random(batch * plan.num_nodes * K) + 0.1).astype(np.float32)
    dense_edges = (rng.random(plan.num_edges * K * K) + 0.1).astype(np.float32)
    wb = gpu.Workspace()
    wb.reserve_marginals(plan, K, batch, scalar=np.float32)
    view = gpu.BatchedModelView(plan, K, batch, dense_nodes, dense_edges)
    wb.set_tuning(1024, stripes=1, schedule=TEAMS)
    single = outputs(wb.posterior_marginals_prepared(view))
    for schedule in (TEAMS, PHASES):
        wb.set_tuning(1024, stripes=4, schedule=schedule)
        for a, b in zip(outputs(wb.posterior_marginals_prepared(view)), single):
            assert np.array_equal(a, b)
    small = gpu.BatchedModelView(plan, K, 3, dense_nodes[:3 * plan.num_nodes * K],
                                 dense_edges)
    wb.set_tuning(1024, stripes=1, schedule=TEAMS)
    single = outputs(wb.posterior_marginals_prepared(small))
    for schedule in (TEAMS, PHASES):
        for stripes in (1, 4):
            wb.set_tuning(1024, stripes=stripes, schedule=schedule)
            for a, b in zip(outputs(wb.posterior_marginals_prepared(small)), single):
                assert np.array_equal(a, b)
