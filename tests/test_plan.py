"""Planner (restated btrc) invariants, checked on many tree shapes:
every non-root node is eliminated exactly once (raked as a leaf or spliced
out as a compressed middle), the operations of one batch are independent,
branches and tapes are numbered in creation order, edge e sits above the e-th
non-root node, and the number of rounds grows logarithmically."""
import math

import numpy as np
import pytest

from parallel_tree_hmm_gb300 import synthetic


def shapes(rng):
    yield "root", np.array([-1])
    yield "pair", np.array([-1, 0])
    yield "chain", np.arange(-1, 1000)
    yield "star", np.array([-1] + [0] * 300)
    yield "binary", synthetic.leaf_splitting(rng, 1001)
    yield "recursive", synthetic.random_recursive(rng, 3000)
    yield "caterpillar", synthetic.caterpillar(2000)
    yield "spine", synthetic.spine_heavy(rng, 3000)
    yield "galton_watson", synthetic.galton_watson(rng, 1000, 3000)
    # Parents need not precede children.
    perm = rng.permutation(500)
    base = synthetic.random_recursive(rng, 500)
    shuffled = np.empty(500, dtype=np.int64)
    for node in range(500):
        shuffled[perm[node]] = -1 if base[node] < 0 else perm[base[node]]
    yield "shuffled", shuffled


@pytest.mark.parametrize("index", range(10))
def test_plan_invariants(index, thmm):
    rng = np.random.default_rng(index)
    name, parents = list(shapes(rng))[index]
    plan = thmm.Plan(parents)
    n = len(parents)
    assert plan.num_nodes == n and plan.num_edges == n - 1
    root = int(np.flatnonzero(parents < 0)[0])
    assert plan.root == root
    non_root = [v for v in range(n) if v != root]
    assert list(plan.edge_children) == non_root
    assert list(plan.edge_parents) == [int(parents[v]) for v in non_root]

    eliminated = np.zeros(n, dtype=int)
    eliminated[plan.rakes[:, 1]] += 1
    eliminated[plan.compressions[:, 1]] += 1
    assert eliminated[root] == 0
    assert np.all(eliminated[non_root] == 1), name
    assert list(plan.rakes[:, 2]) == list(range(plan.num_branches))
    assert list(plan.compressions[:, 3]) == list(range(plan.num_compressions))

    for primitive, offset, count in plan.batches:
        assert count > 0
        if primitive == 0:
            ops = plan.rakes[offset:offset + count]
            assert len(set(ops[:, 1])) == count  # distinct leaves
        elif primitive == 1:
            ops = plan.combinations[offset:offset + count]
            touched = np.concatenate([ops[:, 0], ops[:, 1]])
            assert len(set(touched)) == 2 * count  # disjoint pairs
        elif primitive == 2:
            ops = plan.absorptions[offset:offset + count]
            assert len(set(ops[:, 0])) == count
        else:
            ops = plan.compressions[offset:offset + count]
            middles = set(ops[:, 1])
            # No compressed node is an endpoint of another compression.
            assert not (middles & set(ops[:, 4])) and not (middles & set(ops[:, 5]))
            assert len(set(ops[:, 0]) | set(ops[:, 2])) == 2 * count
    if n > 1:
        assert plan.num_rounds <= 4 * math.log2(n) + 4, (name, plan.num_rounds)


def test_wide_star_has_multistage_reduction(thmm):
    plan = thmm.Plan([-1] + [0] * 17)
    stages = sum(1 for p, _, _ in plan.batches if p == 1)
    assert stages >= 4


def test_compression_happens_on_the_five_node_tree(thmm):
    assert thmm.Plan([-1, 0, 0, 1, 3]).num_compressions != 0


@pytest.mark.parametrize("parents", [[], [0], [-1, -1], [-1, 5], [-1, 2, 1], [1, 0, -1, 2, 2, 9]])
def test_invalid_trees_are_rejected(parents, thmm):
    with pytest.raises(thmm.InvalidArgument):
        thmm.Plan(np.array(parents, dtype=np.int64))


def test_plans_built_in_parallel_match_single_builds(thmm):
    rng = np.random.default_rng(31)
    parents = [synthetic.random_recursive(rng, int(n)) for n in (1, 2, 50, 700, 3000)]
    parents += [synthetic.caterpillar(400), synthetic.spine_heavy(rng, 900)]
    for threads in (0, 1, 3):
        many = thmm.Plan.many(parents, threads=threads)
        assert len(many) == len(parents)
        for p, plan in zip(parents, many):
            single = thmm.Plan(p)
            assert plan.num_nodes == single.num_nodes
            assert plan.root == single.root
            for name in ("rakes", "compressions", "batches", "edge_children"):
                assert np.array_equal(getattr(plan, name), getattr(single, name))
    assert thmm.Plan.many([]) == []


def test_parallel_plan_errors_name_the_first_bad_tree(thmm):
    good = np.array([-1, 0, 0])
    with pytest.raises(thmm.InvalidArgument):
        thmm.Plan.many([good, np.array([-1, 5]), good, np.array([0, 0])], threads=2)
