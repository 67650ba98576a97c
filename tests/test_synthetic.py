"""Workload generators: valid trees with the requested shapes and sizes, and
factor distributions with the requested structure."""
import numpy as np

from parallel_tree_hmm_gb300 import synthetic


def is_tree(parents):
    n = len(parents)
    if (parents < 0).sum() != 1:
        return False
    return all(parents[i] < i for i in range(1, n)) and parents[0] == -1


def test_generators_build_trees():
    rng = np.random.default_rng(0)
    assert is_tree(synthetic.random_recursive(rng, 1000))
    assert is_tree(synthetic.caterpillar(1000)) and len(synthetic.caterpillar(999)) == 999
    assert is_tree(synthetic.spine_heavy(rng, 1000))
    binary = synthetic.leaf_splitting(rng, 1000)
    assert len(binary) == 999 and is_tree(binary)
    counts = np.bincount(binary[1:], minlength=len(binary))
    assert set(np.unique(counts)) <= {0, 2}  # full binary tree
    gw = synthetic.galton_watson(rng, 1000, 2000)
    assert 1000 <= len(gw) <= 2000 and is_tree(gw)


def test_caterpillar_shape():
    parents = synthetic.caterpillar(10)
    leaves = synthetic.leaves(parents)
    spine = [v for v in range(10) if v not in set(leaves)]
    assert spine == [0, 1, 2, 3, 4]
    assert list(leaves) == [5, 6, 7, 8, 9]


def test_factor_structure():
    rng = np.random.default_rng(1)
    edges = synthetic.stochastic_edges(rng, 500, 4, 0.5).reshape(500, 4, 4)
    assert np.allclose(edges.sum(axis=2), 1.0)
    values = synthetic.lognormal(rng, 10000, 1.5, zero_fraction=0.02)
    zeros = np.mean(values == 0)
    assert 0.01 < zeros < 0.03 and np.all(values >= 0)
