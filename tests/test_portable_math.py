"""Error bounds of the reproducible exp/log used by the MAP and sampling
kernels (parallel_tree_hmm_gb300/csrc/portable_math.h), against float64/longer
references: within 1 ulp for float, 2 ulps for double, with exact special
values."""
import math

import numpy as np

from oracle import bridge


def ulp_error_f32(values, function, reference):
    worst = 0.0
    for x in values:
        got = np.float32(function(np.float32(x)))
        want = reference(float(np.float32(x)))
        if math.isinf(want) or math.isnan(want) or want == 0.0:
            continue
        ulp = float(np.spacing(np.float32(abs(want))))
        worst = max(worst, abs(float(got) - want) / ulp)
    return worst


def test_float_exp_log_within_one_ulp():
    lib = bridge.library()
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-100, 88, 20000), rng.uniform(-1, 1, 20000)])
    assert ulp_error_f32(xs, lib.oracle_portable_expf, math.exp) <= 1.0
    ys = np.concatenate([np.exp(rng.uniform(-80, 80, 20000)), rng.uniform(0.5, 2, 20000),
                         rng.uniform(1e-44, 1e-38, 2000)])
    assert ulp_error_f32(ys, lib.oracle_portable_logf, math.log) <= 1.0


def test_double_exp_log_within_two_ulps():
    lib = bridge.library()
    rng = np.random.default_rng(1)
    worst = 0.0
    for x in np.concatenate([rng.uniform(-700, 700, 20000), rng.uniform(-1, 1, 5000)]):
        got = lib.oracle_portable_exp(float(x))
        want = math.exp(float(x))
        worst = max(worst, abs(got - want) / float(np.spacing(want)))
    assert worst <= 2.0
    worst = 0.0
    for x in np.concatenate([np.exp(rng.uniform(-700, 700, 20000)), rng.uniform(0.5, 2, 5000),
                             [5e-324, 1e-310]]):
        got = lib.oracle_portable_log(float(x))
        want = math.log(float(x))
        worst = max(worst, abs(got - want) / float(np.spacing(abs(want))))
    assert worst <= 2.0


def test_special_values():
    lib = bridge.library()
    assert lib.oracle_portable_logf(0.0) == -math.inf
    assert math.isnan(lib.oracle_portable_logf(-1.0))
    assert lib.oracle_portable_logf(math.inf) == math.inf
    assert lib.oracle_portable_expf(-math.inf) == 0.0
    assert lib.oracle_portable_expf(200.0) == math.inf
    assert lib.oracle_portable_expf(0.0) == 1.0 and lib.oracle_portable_logf(1.0) == 0.0
    assert lib.oracle_portable_log(0.0) == -math.inf
    assert lib.oracle_portable_exp(-math.inf) == 0.0
    assert lib.oracle_portable_exp(0.0) == 1.0 and lib.oracle_portable_log(1.0) == 0.0
