"""The allocation-free entry point thmm_log_partition_static.

Some callers cannot call cudaMalloc: their device memory is owned by another
allocator, or they run where new allocations are not permitted. For them the
library offers one entry point that allocates nothing and keeps every
intermediate in a static device array. This test calls it through the C ABI on
caller-owned device buffers and checks it against the workspace entry point
(thmm_log_partition_function) on two calls in a row, with the log Z tolerance
the other GPU tests use (1e-6 relative), and checks that an oversized request
is rejected. The file name sorts last so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from parallel_tree_hmm_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu

LOG_Z_RTOL = 1e-6


def _static_log_partition(plan, states, batch, nodes, edges, out, stream):
    lib = _lib.library()
    return lib.thmm_log_partition_static(plan.handle, states, batch, nodes.data_ptr(),
                                         edges.data_ptr(), out.data_ptr(), stream)


def _case(gpu, rng, parents, states, batch):
    torch = pytest.importorskip("torch")
    plan = gpu.Plan(parents)
    nodes = (rng.random((batch, plan.num_nodes, states)) + 0.05).astype(np.float32)
    edges = synthetic.stochastic_edges(rng, plan.num_edges, states, 0.5, np.float32)
    ws = gpu.Workspace()
    ws.reserve(plan, states, batch, scalar=np.float32)
    expected = ws.log_partition_function_prepared(
        gpu.BatchedModelView(plan, states, batch, nodes.ravel(), edges)).values.copy()
    nodes_d = torch.from_numpy(nodes.ravel()).cuda()
    edges_d = torch.from_numpy(edges).cuda()
    out_d = torch.full((batch,), float("nan"), dtype=torch.float32, device="cuda")
    return plan, states, batch, nodes_d, edges_d, out_d, expected


def _close(got, expected):
    return np.all(np.abs(got - expected) <= LOG_Z_RTOL * np.maximum(1, np.abs(expected)))


def test_static_log_partition_matches_workspace_on_two_calls(gpu):
    """Each case is run twice in a row; the cases cover one thread per
    operation (K <= 4) and the lane-group paths (K = 8 and 20)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    shapes = [(synthetic.random_recursive(rng, 3000), 4, 6),
              (synthetic.caterpillar(801), 3, 5),
              (synthetic.random_recursive(rng, 1500), 8, 4),
              (synthetic.spine_heavy(rng, 600), 20, 3)]
    stream = torch.cuda.current_stream().cuda_stream
    for parents, states, batch in shapes:
        plan, states, batch, nodes_d, edges_d, out_d, expected = _case(
            gpu, rng, parents, states, batch)
        for _ in range(2):
            out_d.fill_(float("nan"))
            status = _static_log_partition(plan, states, batch, nodes_d, edges_d, out_d,
                                           stream)
            assert status == _lib.THMM_OK, _lib.library().thmm_last_error().decode()
            torch.cuda.synchronize()
            assert _close(out_d.cpu().numpy(), expected), (states, batch)


def test_static_log_partition_back_to_back_calls_share_the_array(gpu):
    """Two calls with different plans and state counts, issued on one stream
    with no synchronisation between them: a large program and scratch
    followed by a small one, then the reverse. Each output must match the
    workspace result, so neither call sees the other's leftovers."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(99)
    large = _case(gpu, rng, synthetic.random_recursive(rng, 4000), 20, 4)
    small = _case(gpu, rng, synthetic.caterpillar(257), 4, 7)
    stream = torch.cuda.current_stream().cuda_stream
    for first, second in ((large, small), (small, large)):
        for case in (first, second):
            case[5].fill_(float("nan"))
        for case in (first, second):
            plan, states, batch, nodes_d, edges_d, out_d, _ = case
            status = _static_log_partition(plan, states, batch, nodes_d, edges_d, out_d,
                                           stream)
            assert status == _lib.THMM_OK, _lib.library().thmm_last_error().decode()
        torch.cuda.synchronize()
        for case in (first, second):
            assert _close(case[5].cpu().numpy(), case[6]), case[1]
    assert _lib.library().thmm_last_error().decode() == ""


def test_static_log_partition_rejects_oversized_requests(gpu):
    torch = pytest.importorskip("torch")
    plan = gpu.Plan(synthetic.caterpillar(20000))
    states, batch = 4, 400  # far beyond the static scratch
    nodes_d = torch.ones(1, dtype=torch.float32, device="cuda")
    edges_d = torch.ones(1, dtype=torch.float32, device="cuda")
    out_d = torch.empty(1, dtype=torch.float32, device="cuda")
    status = _static_log_partition(plan, states, batch, nodes_d, edges_d, out_d,
                                   torch.cuda.current_stream().cuda_stream)
    assert status == _lib.THMM_INVALID_ARGUMENT
    assert "static scratch" in _lib.library().thmm_last_error().decode()
