"""Seeded synthetic workloads with the shapes and distributions of the
benchmark configurations (no public dataset is involved).

Tree generators return parent arrays (int64, -1 at the root, parents precede
children). Factor generators return float arrays in the layouts of the
accelerator API: node factors [node, state], edge factors [edge, parent,
child] in the plan's edge order (edge e sits above the e-th non-root node).
"""
from __future__ import annotations

import numpy as np


def random_recursive(rng: np.random.Generator, n: int) -> np.ndarray:
    """Node i attaches to a uniform earlier node."""
    parents = np.empty(n, dtype=np.int64)
    parents[0] = -1
    if n > 1:
        i = np.arange(1, n)
        parents[1:] = np.floor(rng.random(n - 1) * i).astype(np.int64)
    return parents


def caterpillar(n: int) -> np.ndarray:
    """A spine of ceil(n/2) nodes with one leaf hanging from each of the
    first floor(n/2) spine nodes."""
    spine = (n + 1) // 2
    parents = np.empty(n, dtype=np.int64)
    parents[0] = -1
    parents[1:spine] = np.arange(0, spine - 1)
    parents[spine:] = np.arange(0, n - spine)
    return parents


def spine_heavy(rng: np.random.Generator, n: int, spine_probability: float = 0.95):
    """Node i attaches to i-1 with the given probability, else to a uniform
    earlier node."""
    parents = random_recursive(rng, n)
    if n > 1:
        keep = rng.random(n - 1) < spine_probability
        parents[1:][keep] = np.arange(0, n - 1)[keep]
    return parents


def leaf_splitting(rng: np.random.Generator, n: int) -> np.ndarray:
    """Random full binary tree: repeatedly give a uniform current leaf two
    children. Full binary trees have an odd node count, so n is rounded down to
    the nearest odd count (1000 -> 999)."""
    n = n if n % 2 == 1 else n - 1
    parents = [-1]
    leaves = [0]
    while len(parents) < n:
        index = int(rng.integers(len(leaves)))
        leaf = leaves[index]
        leaves[index] = len(parents)
        parents.append(leaf)
        leaves.append(len(parents))
        parents.append(leaf)
    return np.asarray(parents, dtype=np.int64)


def galton_watson(rng: np.random.Generator, minimum: int = 1000,
                  maximum: int = 50000, mean: float = 2.0) -> np.ndarray:
    """Poisson(mean) Galton-Watson tree grown breadth first until a size cap
    drawn uniformly from [minimum, maximum] is reached; a tree that dies out
    below `minimum` nodes is discarded and regrown.

    Breadth-first growth appends the children of node 0, then of node 1, and
    so on, so with offspring counts c_k the parent array is node k repeated
    c_k times, in order; the tree dies out at the first node k that does not
    exist (1 + c_0 + ... + c_{k-1} <= k)."""
    cap = int(rng.integers(minimum, maximum + 1))
    while True:
        counts = rng.poisson(mean, size=cap)
        born = 1 + np.cumsum(counts)  # nodes present after processing node k
        alive = born[:-1] > np.arange(1, cap)  # node k + 1 exists
        dead = np.flatnonzero(~alive)
        processed = cap if dead.size == 0 else int(dead[0]) + 1
        children = np.repeat(np.arange(processed, dtype=np.int64), counts[:processed])
        parents = np.concatenate([[-1], children])[:cap]
        if len(parents) >= minimum:
            return parents


def dirichlet_rows(rng: np.random.Generator, rows: int, states: int,
                   alpha: float, dtype=np.float64) -> np.ndarray:
    g = rng.standard_gamma(alpha, size=(rows, states))
    total = g.sum(axis=1, keepdims=True)
    # A row of all-underflowed gammas (tiny alpha) falls back to uniform.
    bad = total[:, 0] <= 0
    g[bad] = 1.0
    total[bad] = states
    return (g / total).astype(dtype)


def stochastic_edges(rng: np.random.Generator, edges: int, states: int,
                     alpha: float, dtype=np.float64) -> np.ndarray:
    """[edge, parent, child] with every parent row ~ Dirichlet(alpha)."""
    return dirichlet_rows(rng, edges * states, states, alpha, dtype).reshape(-1)


def lognormal(rng: np.random.Generator, count: int, sigma: float,
              zero_fraction: float = 0.0, dtype=np.float64) -> np.ndarray:
    values = np.exp(rng.normal(0.0, sigma, size=count))
    if zero_fraction > 0:
        values[rng.random(count) < zero_fraction] = 0.0
    return values.astype(dtype)


def leaves(parents: np.ndarray) -> np.ndarray:
    """Sorted indices of the nodes without children."""
    has_child = np.zeros(len(parents), dtype=bool)
    has_child[parents[parents >= 0]] = True
    return np.flatnonzero(~has_child).astype(np.uint32)
