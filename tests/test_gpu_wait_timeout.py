"""The bounded device waits give up and report an error instead of hanging.

Every mbarrier wait of the tensor-core engine has a cycle budget; a wait
that runs out sets an error bit, the kernel still releases its tensor
memory, and the host turns the bit into THMM_RUNTIME_ERROR
(std::runtime_error in the C++ layer). thmm_wait_timeout_check runs that
path in one warp whose wait cannot complete (bytes announced on the barrier,
no copy issued) with a small budget. No fault or hang is involved: the wait
ends by itself after about a millisecond, and the device stays usable, as
the tensor-core engine call afterwards shows (it needs every tensor-memory
column of an SM, so leaked columns would make it wait).
"""
import numpy as np
import pytest

from oracle import bridge
from parallel_tree_hmm_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_becomes_runtime_error(gpu):
    lib = _lib.library()
    status = lib.thmm_wait_timeout_check(0, 1 << 21)
    assert status == _lib.THMM_RUNTIME_ERROR
    assert "tensor-core wait timed out" in lib.thmm_last_error().decode()
    with pytest.raises(RuntimeError, match="wait timed out"):
        gpu.api._check(lib.thmm_wait_timeout_check(0, 1 << 20))
    assert lib.thmm_wait_timeout_check(0, 0) == _lib.THMM_INVALID_ARGUMENT

    # The device and its tensor memory are still fully usable.
    rng = np.random.default_rng(3)
    K = 40
    plan = gpu.Plan(synthetic.spine_heavy(rng, 60))
    nodes = (rng.random(plan.num_nodes * K) + 0.05).astype(np.float32)
    edges = synthetic.stochastic_edges(rng, plan.num_edges, K, 1.0, np.float32)
    ws = gpu.Workspace()
    ws.reserve(plan, K, 1, scalar=np.float32)
    got = ws.log_partition_function_prepared(
        gpu.BatchedModelView(plan, K, 1, nodes, edges)).values[0]
    expected = bridge.log_partition(plan, K, nodes.astype(np.float64),
                                    edges.astype(np.float64))
    assert abs(got - expected) <= 1e-6 * max(1.0, abs(expected))
