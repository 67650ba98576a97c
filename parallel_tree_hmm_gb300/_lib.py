"""ctypes binding of libthmm_gb300.so (declarations in include/thmm_gb300.h).

The library is the only implementation: if it is missing or fails to load,
`library()` raises, there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes
import pathlib

PACKAGE = pathlib.Path(__file__).resolve().parent
LIBRARY_PATH = PACKAGE / "libthmm_gb300.so"

c_size = ctypes.c_size_t
c_u32 = ctypes.c_uint32
c_u64 = ctypes.c_uint64
c_int = ctypes.c_int
c_void_p = ctypes.c_void_p
u32_p = ctypes.POINTER(ctypes.c_uint32)
u8_p = ctypes.POINTER(ctypes.c_uint8)

THMM_OK = 0
THMM_INVALID_ARGUMENT = 1
THMM_LOGIC_ERROR = 2
THMM_DOMAIN_ERROR = 3
THMM_LENGTH_ERROR = 4
THMM_RUNTIME_ERROR = 5

THMM_SCALAR_F32 = 4
THMM_SCALAR_F64 = 8
THMM_RESERVE_MAXIMUM = 1
THMM_RESERVE_SAMPLING = 2
THMM_RESERVE_MARGINALS = 4
THMM_RESERVE_DEVICE_ONLY = 8
THMM_COMPUTE_F64 = 0x100
THMM_COMPUTE_BF16 = 0x200
THMM_UPDATE_ALL = 0
THMM_UPDATE_FACTORS = 1
THMM_UPDATE_NONE = 2
THMM_OP_PARTITION = 0
THMM_OP_LOG_PARTITION = 1
THMM_OP_MAXIMUM = 2
THMM_OP_SAMPLE = 3
THMM_OP_MARGINALS = 4
THMM_SCHEDULE_TEAMS = 0
THMM_SCHEDULE_PHASES = 1


class PlanInfo(ctypes.Structure):
    _fields_ = [("num_nodes", c_size), ("num_edges", c_size), ("num_branches", c_size),
                ("num_compressions", c_size), ("num_combinations", c_size),
                ("num_absorptions", c_size), ("num_batches", c_size),
                ("num_rounds", c_size), ("root", c_u32)]


class PlanArrays(ctypes.Structure):
    _fields_ = [("edge_parents", u32_p), ("edge_children", u32_p), ("rakes", u32_p),
                ("combinations", u32_p), ("absorptions", u32_p),
                ("compressions", u32_p), ("batches", u32_p)]


class DenseInputView(ctypes.Structure):
    _fields_ = [("states", c_size), ("batch", c_size), ("node_potentials", c_void_p),
                ("node_count", c_size), ("edge_potentials", c_void_p),
                ("edge_count", c_size)]


class CategoricalInputView(ctypes.Structure):
    _fields_ = [("states", c_size), ("batch", c_size), ("categories", c_size),
                ("observation_nodes", u32_p), ("observation_node_count", c_size),
                ("observations", u8_p), ("observation_count", c_size),
                ("root_potential", c_void_p), ("root_count", c_size),
                ("emission_potentials", c_void_p), ("emission_count", c_size),
                ("edge_potentials", c_void_p), ("edge_count", c_size)]


class DenseModel(ctypes.Structure):
    _fields_ = [("plan", c_void_p), ("states", c_size), ("batch", c_size),
                ("node_potentials", c_void_p), ("node_count", c_size),
                ("edge_potentials", c_void_p), ("edge_count", c_size)]


class CategoricalModel(ctypes.Structure):
    _fields_ = [("plan", c_void_p), ("states", c_size), ("batch", c_size),
                ("categories", c_size), ("observation_nodes", c_void_p),
                ("observation_node_count", c_size), ("observations", c_void_p),
                ("observation_count", c_size), ("root_potential", c_void_p),
                ("root_count", c_size), ("emission_potentials", c_void_p),
                ("emission_count", c_size), ("edge_potentials", c_void_p),
                ("edge_count", c_size)]


class Timings(ctypes.Structure):
    _fields_ = [("upload_ms", ctypes.c_double), ("kernel_ms", ctypes.c_double),
                ("download_ms", ctypes.c_double), ("wall_ms", ctypes.c_double)]


class PartitionResult(ctypes.Structure):
    _fields_ = [("values", c_void_p), ("count", c_size), ("timings", Timings)]


class MaximumResult(ctypes.Structure):
    _fields_ = [("log_weights", c_void_p), ("count", c_size), ("states", u32_p),
                ("state_count", c_size), ("timings", Timings)]


class SampleResult(ctypes.Structure):
    _fields_ = [("states", u32_p), ("count", c_size), ("timings", Timings)]


class MarginalResult(ctypes.Structure):
    _fields_ = [("log_partitions", c_void_p), ("count", c_size), ("nodes", c_void_p),
                ("node_count", c_size), ("edges", c_void_p), ("edge_count", c_size),
                ("timings", Timings)]


class DeviceBuffers(ctypes.Structure):
    _fields_ = [(name, c_void_p) for name in (
        "node_potentials", "edge_potentials", "observations", "root_potential",
        "emission_potentials", "uniforms", "values", "node_marginals", "edge_marginals",
        "states")]


class Tuning(ctypes.Structure):
    _fields_ = [("team_threshold", c_u32), ("ctas_per_sm", c_u32 * 4),
                ("stripes", c_u32), ("kernel_ms", ctypes.c_float), ("candidates", c_u32),
                ("schedule", c_u32), ("phase_rounds", c_u32)]


# name -> (restype, argtypes)
PROTOTYPES = {
    "thmm_last_error": (ctypes.c_char_p, []),
    "thmm_plan_create": (c_int, [ctypes.POINTER(ctypes.c_int64), c_size,
                                 ctypes.POINTER(c_void_p)]),
    "thmm_plan_create_many": (c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(c_size),
                                      c_size, ctypes.c_uint, ctypes.POINTER(c_void_p)]),
    "thmm_plan_destroy": (None, [c_void_p]),
    "thmm_plan_get_info": (c_int, [c_void_p, ctypes.POINTER(PlanInfo)]),
    "thmm_plan_get_arrays": (c_int, [c_void_p, ctypes.POINTER(PlanArrays)]),
    "thmm_available": (c_int, []),
    "thmm_device_description": (c_int, [c_int, ctypes.c_char_p, c_size]),
    "thmm_workspace_create": (c_int, [ctypes.POINTER(c_void_p)]),
    "thmm_workspace_destroy": (None, [c_void_p]),
    "thmm_reserve": (c_int, [c_void_p, c_void_p, c_size, c_size, c_int, c_u32, c_u32]),
    "thmm_reserve_categorical": (c_int, [c_void_p, c_void_p, c_size, c_size, c_size,
                                         c_void_p, c_size, c_int, c_u32, c_u32]),
    "thmm_reserve_forest": (c_int, [c_void_p, c_void_p, c_size, c_size, c_int, c_u32,
                                    c_u32]),
    "thmm_reserve_forest_categorical": (c_int, [c_void_p, c_void_p, c_size, c_size,
                                                c_size, c_void_p, c_void_p, c_int,
                                                c_u32, c_u32]),
    "thmm_inputs": (c_int, [c_void_p, c_size, ctypes.POINTER(DenseInputView)]),
    "thmm_categorical_inputs": (c_int, [c_void_p, c_size,
                                        ctypes.POINTER(CategoricalInputView)]),
    "thmm_uniforms": (c_int, [c_void_p, c_size, ctypes.POINTER(c_void_p),
                              ctypes.POINTER(c_size)]),
    "thmm_partition_function": (c_int, [c_void_p, ctypes.POINTER(DenseModel),
                                        ctypes.POINTER(PartitionResult)]),
    "thmm_log_partition_function": (c_int, [c_void_p, ctypes.POINTER(DenseModel),
                                            ctypes.POINTER(PartitionResult)]),
    "thmm_maximum_a_posteriori": (c_int, [c_void_p, ctypes.POINTER(DenseModel),
                                          ctypes.POINTER(MaximumResult)]),
    "thmm_posterior_sample": (c_int, [c_void_p, ctypes.POINTER(DenseModel), c_void_p,
                                      c_size, ctypes.POINTER(SampleResult)]),
    "thmm_posterior_marginals": (c_int, [c_void_p, ctypes.POINTER(DenseModel),
                                         ctypes.POINTER(MarginalResult)]),
    "thmm_categorical_partition_function": (
        c_int, [c_void_p, ctypes.POINTER(CategoricalModel), c_int,
                ctypes.POINTER(PartitionResult)]),
    "thmm_categorical_log_partition_function": (
        c_int, [c_void_p, ctypes.POINTER(CategoricalModel), c_int,
                ctypes.POINTER(PartitionResult)]),
    "thmm_categorical_maximum_a_posteriori": (
        c_int, [c_void_p, ctypes.POINTER(CategoricalModel), c_int,
                ctypes.POINTER(MaximumResult)]),
    "thmm_categorical_posterior_sample": (
        c_int, [c_void_p, ctypes.POINTER(CategoricalModel), c_void_p, c_size, c_int,
                ctypes.POINTER(SampleResult)]),
    "thmm_categorical_posterior_marginals": (
        c_int, [c_void_p, ctypes.POINTER(CategoricalModel), c_int,
                ctypes.POINTER(MarginalResult)]),
    "thmm_enqueue": (c_int, [c_void_p, c_int, ctypes.POINTER(c_u64)]),
    "thmm_autotune": (c_int, [c_void_p, c_int, c_int, ctypes.POINTER(Tuning)]),
    "thmm_get_tuning": (c_int, [c_void_p, ctypes.POINTER(Tuning)]),
    "thmm_set_tuning": (c_int, [c_void_p, ctypes.POINTER(Tuning)]),
    "thmm_workspace_stream": (c_void_p, [c_void_p]),
    "thmm_workspace_synchronize": (c_int, [c_void_p]),
    "thmm_workspace_launches": (c_u64, [c_void_p]),
    "thmm_wait_timeout_check": (c_int, [c_int, c_u64]),
    "thmm_device_buffers_get": (c_int, [c_void_p, ctypes.POINTER(DeviceBuffers)]),
    "thmm_device_inputs_ready": (c_int, [c_void_p, c_size]),
    "thmm_log_partition_static": (c_int, [c_void_p, c_size, c_size, c_void_p, c_void_p,
                                          c_void_p, c_void_p]),
}

_LIB = None


def library() -> ctypes.CDLL:
    """Loads libthmm_gb300.so (built in-tree by parallel_tree_hmm_gb300.build)."""
    global _LIB
    if _LIB is None:
        if not LIBRARY_PATH.exists():
            raise RuntimeError(
                f"{LIBRARY_PATH} is missing; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(str(LIBRARY_PATH))
        for name, (restype, argtypes) in PROTOTYPES.items():
            function = getattr(lib, name)
            function.restype = restype
            function.argtypes = argtypes
        _LIB = lib
    return _LIB
