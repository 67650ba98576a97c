"""torch.autograd wrapper around the marginal kernel (test-facing, thin).

`forest_log_partition(plans, log_nodes, log_edges)` returns log Z for every
tree of a forest as a differentiable function of the log node factors
[sum of nodes, K] and log edge factors [sum of edges, K, K] (per-tree edges,
concatenated in tree order). The forward pass is one C-ABI prepared marginal
call; the backward pass needs no further kernel because the marginals it
returns are exactly the gradient:

    d log Z_t / d log nodes[n, k]     = P(x_n = k)            (node marginal)
    d log Z_t / d log edges[e, i, j]  = P(x_parent = i, x_child = j)

The gradient of an exactly-zero factor's log (-inf) is its marginal, 0.
"""
from __future__ import annotations

import numpy as np
import torch

from .api import BatchedModelView, Workspace


class _ForestLogPartition(torch.autograd.Function):
    @staticmethod
    def forward(ctx, log_nodes, log_edges, workspace, tree_count, states):
        nodes = torch.exp(log_nodes.detach()).cpu().numpy().astype(workspace.dtype).ravel()
        edges = torch.exp(log_edges.detach()).cpu().numpy().astype(workspace.dtype).ravel()
        view = workspace.posterior_marginals_prepared(
            BatchedModelView(None, states, tree_count, nodes, edges))
        node_m = torch.from_numpy(np.array(view.nodes, dtype=np.float64))
        edge_m = torch.from_numpy(np.array(view.edges, dtype=np.float64))
        ctx.save_for_backward(node_m.reshape(log_nodes.shape).to(log_nodes.device),
                              edge_m.reshape(log_edges.shape).to(log_edges.device))
        ctx.node_tree = workspace_node_tree(workspace, log_nodes.device)
        ctx.edge_tree = workspace_edge_tree(workspace, log_edges.device)
        log_z = torch.from_numpy(np.array(view.log_partitions, dtype=np.float64))
        return log_z.to(dtype=log_nodes.dtype, device=log_nodes.device)

    @staticmethod
    def backward(ctx, grad_log_z):
        node_m, edge_m = ctx.saved_tensors
        grad = grad_log_z.to(torch.float64)
        grad_nodes = node_m * grad[ctx.node_tree].reshape(-1, *([1] * (node_m.dim() - 1)))
        grad_edges = edge_m * grad[ctx.edge_tree].reshape(-1, *([1] * (edge_m.dim() - 1)))
        return (grad_nodes.to(grad_log_z.dtype), grad_edges.to(grad_log_z.dtype), None, None,
                None)


def workspace_node_tree(workspace: Workspace, device) -> torch.Tensor:
    counts = [plan.num_nodes for plan in workspace._plans]
    return torch.repeat_interleave(torch.arange(len(counts)),
                                   torch.tensor(counts)).to(device)


def workspace_edge_tree(workspace: Workspace, device) -> torch.Tensor:
    counts = [plan.num_edges for plan in workspace._plans]
    return torch.repeat_interleave(torch.arange(len(counts)),
                                   torch.tensor(counts)).to(device)


def forest_workspace(plans, states, scalar=np.float32, compute=np.float32,
                     device: int = 0) -> Workspace:
    workspace = Workspace()
    workspace.reserve_forest(plans, states, device, kind="marginals", scalar=scalar,
                             compute=compute)
    return workspace


def forest_log_partition(workspace: Workspace, log_nodes: torch.Tensor,
                         log_edges: torch.Tensor) -> torch.Tensor:
    """log Z per tree; differentiable in `log_nodes` and `log_edges`."""
    states = log_nodes.shape[-1]
    return _ForestLogPartition.apply(log_nodes, log_edges, workspace,
                                     len(workspace._plans), states)
