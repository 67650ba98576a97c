"""ORACLE - test infrastructure only: agreement of discrete outputs (MAP
states, posterior samples) between the device and the reference-pinned CPU
oracle, with every disagreement classified by the margin of the comparison
that decided it.

A node's state is decided given the states of the nodes its choice depends
on: a raked leaf given its parent, a compressed middle node given both ends
of the compression, the root given nothing. A disagreement is

  - "inherited" when one of those states already differs (the decision was
    made on different inputs), otherwise
  - an independent disagreement, binned by the oracle's decision margin:
    for MAP the gap between the chosen maximum and the runner-up relative to
    max(1, |maximum|); for sampling the distance from the node's uniform to
    the nearer end of the chosen state's cumulative interval.

Independent disagreements with a margin at the level of float32 rounding
are ties: two correct implementations whose exp/log differ in the last bit
can legitimately break them differently. For MAP the compared values are
sums of logs, so a last-bit difference in one log moves them by a few ulps
(tie margin 2**-20). For sampling the compared cumulative weights come from
log-sum-exp messages whose rounding accumulates along the tree, so the tie
margin allows more (2**-14, about depth x a few ulps).
"""
from __future__ import annotations

import numpy as np

MAP_TIE_MARGIN = 2.0 ** -20
SAMPLE_TIE_MARGIN = 2.0 ** -14
BINS = (0.0, 2.0 ** -23, 2.0 ** -20, 1e-5, 1e-4, 1e-3, np.inf)
BIN_NAMES = ("<=2^-23", "<=2^-20", "<=1e-5", "<=1e-4", "<=1e-3", ">1e-3")


def dependencies(plan) -> list[np.ndarray]:
    """(node, parent, other) arrays: the decision inputs of every non-root
    node (other = parent for rakes, the child end for compressions)."""
    rakes = np.asarray(plan.rakes).reshape(-1, 4)
    comps = np.asarray(plan.compressions).reshape(-1, 6)
    node = np.concatenate([rakes[:, 1], comps[:, 1]])
    parent = np.concatenate([rakes[:, 3], comps[:, 4]])
    other = np.concatenate([rakes[:, 3], comps[:, 5]])
    return [node, parent, other]


def classify(plan, device: np.ndarray, oracle: np.ndarray, margins: np.ndarray,
             tie_margin: float) -> dict:
    """Counts of agreements and classified disagreements for one tree."""
    device = np.asarray(device)
    oracle = np.asarray(oracle)
    differ = device != oracle
    node, parent, other = dependencies(plan)
    inherited_mask = np.zeros(len(device), dtype=bool)
    inherited_mask[node] = differ[parent] | differ[other]
    independent = differ & ~inherited_mask
    result = {"nodes": int(len(device)), "agree": int(np.sum(~differ)),
              "inherited": int(np.sum(differ & inherited_mask)),
              "independent": int(np.sum(independent))}
    gaps = np.abs(np.asarray(margins, dtype=np.float64)[independent])
    hist = np.histogram(gaps, bins=BINS)[0]
    result["margins"] = {name: int(c) for name, c in zip(BIN_NAMES, hist)}
    result["independent_ties"] = int(np.sum(gaps <= tie_margin))
    return result


def merge(parts: list[dict]) -> dict:
    total = {"nodes": 0, "agree": 0, "inherited": 0, "independent": 0,
             "independent_ties": 0, "margins": {name: 0 for name in BIN_NAMES}}
    for part in parts:
        for key in ("nodes", "agree", "inherited", "independent", "independent_ties"):
            total[key] += part[key]
        for name in BIN_NAMES:
            total["margins"][name] += part["margins"][name]
    total["rate"] = total["agree"] / max(1, total["nodes"])
    return total
