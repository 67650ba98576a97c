"""ORACLE - test infrastructure only.

ctypes access to
  * liboracle.so: the C restatement of the reference CPU algebras
    (oracle/oracle.h), built everywhere, and
  * oracle/_ref/libref_{f64,f32}.so: the reference's own src/inference.cc
    compiled from the reference tree (only where that tree exists).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the product never does.
"""
from __future__ import annotations

import ctypes
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

MATH_LIBM = 0
MATH_PORTABLE = 1

ORACLE_OK = 0
ORACLE_INVALID_ARGUMENT = 1
ORACLE_DOMAIN_ERROR = 3


class OracleError(RuntimeError):
    def __init__(self, status: int):
        super().__init__(f"oracle status {status}")
        self.status = status


class OraclePlan(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint32) for name in (
        "num_nodes", "num_edges", "root", "num_rakes", "num_combinations",
        "num_absorptions", "num_compressions", "num_batches")] + [
        (name, ctypes.POINTER(ctypes.c_uint32)) for name in (
            "edge_parents", "edge_children", "rakes", "combinations", "absorptions",
            "compressions", "batches")]


def _u32(array) -> ctypes.POINTER(ctypes.c_uint32):
    return array.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


PLAN_LIB = HERE / "liboracle_plan.so"
_PLANNER = None


def planner() -> ctypes.CDLL:
    """liboracle_plan.so: the restated planner for the CPU baselines."""
    global _PLANNER
    if _PLANNER is None:
        if not PLAN_LIB.exists():
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        lib = ctypes.CDLL(str(PLAN_LIB))
        lib.oracle_plan_create.argtypes = [ctypes.POINTER(ctypes.c_int64), ctypes.c_size_t]
        lib.oracle_plan_create.restype = ctypes.c_void_p
        lib.oracle_plan_destroy.argtypes = [ctypes.c_void_p]
        lib.oracle_plan_destroy.restype = None
        lib.oracle_plan_view.argtypes = [ctypes.c_void_p, ctypes.POINTER(OraclePlan)]
        lib.oracle_plan_view.restype = None
        _PLANNER = lib
    return _PLANNER


class CpuPlan:
    """A tree's rake/compress plan built by liboracle_plan.so, with the
    attributes the oracle functions read (those of
    parallel_tree_hmm_gb300.Plan), so CPU baselines need no product library."""

    def __init__(self, parents):
        parents = np.ascontiguousarray(parents, dtype=np.int64)
        self._lib = planner()
        self._handle = self._lib.oracle_plan_create(
            parents.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), parents.size)
        if not self._handle:
            raise ValueError("not a tree")
        view = OraclePlan()
        self._lib.oracle_plan_view(self._handle, ctypes.byref(view))
        self._view = view
        self.num_nodes = view.num_nodes
        self.num_edges = view.num_edges
        self.root = view.root
        self.num_branches = view.num_rakes
        self.num_combinations = view.num_combinations
        self.num_absorptions = view.num_absorptions
        self.num_compressions = view.num_compressions
        self.num_batches = view.num_batches

    def _array(self, pointer, rows, width):
        if rows == 0:
            return np.zeros((0, width), dtype=np.uint32)
        return np.ctypeslib.as_array(pointer, shape=(rows * width,)).reshape(rows, width).copy()

    @property
    def rakes(self):
        return self._array(self._view.rakes, self.num_branches, 4)

    @property
    def compressions(self):
        return self._array(self._view.compressions, self.num_compressions, 6)

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle:
            self._lib.oracle_plan_destroy(handle)
            self._handle = None


def oracle_plan(plan):
    """OraclePlan struct for a parallel_tree_hmm_gb300.Plan or a CpuPlan
    (keeps the arrays alive)."""
    if isinstance(plan, CpuPlan):
        struct = OraclePlan()
        ctypes.pointer(struct)[0] = plan._view
        struct._keep = plan
        return struct
    keep = [np.ascontiguousarray(a, dtype=np.uint32) for a in (
        plan.edge_parents, plan.edge_children, plan.rakes, plan.combinations,
        plan.absorptions, plan.compressions, plan.batches)]
    struct = OraclePlan(plan.num_nodes, plan.num_edges, plan.root, plan.num_branches,
                        plan.num_combinations, plan.num_absorptions,
                        plan.num_compressions, plan.num_batches, *[_u32(a) for a in keep])
    struct._keep = keep
    return struct


_ORACLE = None


def library() -> ctypes.CDLL:
    global _ORACLE
    if _ORACLE is None:
        if not ORACLE_LIB.exists():
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        _ORACLE = ctypes.CDLL(str(ORACLE_LIB))
        for name, scalar in (("f64", ctypes.c_double), ("f32", ctypes.c_float)):
            p = ctypes.POINTER(scalar)
            u = ctypes.POINTER(ctypes.c_uint32)
            plan = ctypes.POINTER(OraclePlan)
            size = ctypes.c_size_t
            sig = {
                f"oracle_partition_{name}": [plan, size, p, p, p],
                f"oracle_log_partition_{name}": [plan, size, p, p, p],
                f"oracle_marginals_{name}": [plan, size, p, p, p, p, p, p],
                f"oracle_map_{name}": [plan, size, p, p, ctypes.c_int, p, u],
                f"oracle_sample_{name}": [plan, size, p, p, p, ctypes.c_int, u],
                f"oracle_map_margins_{name}": [plan, size, p, p, ctypes.c_int, p, u, p],
                f"oracle_sample_margins_{name}": [plan, size, p, p, p, ctypes.c_int, u, p],
            }
            for fn, args in sig.items():
                getattr(_ORACLE, fn).argtypes = args
                getattr(_ORACLE, fn).restype = ctypes.c_int
        for fn, scalar in (("oracle_portable_expf", ctypes.c_float),
                           ("oracle_portable_logf", ctypes.c_float),
                           ("oracle_portable_exp", ctypes.c_double),
                           ("oracle_portable_log", ctypes.c_double)):
            getattr(_ORACLE, fn).argtypes = [scalar]
            getattr(_ORACLE, fn).restype = scalar
    return _ORACLE


def _suffix(dtype) -> str:
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def _ptr(array):
    ctype = ctypes.c_double if array.dtype == np.float64 else ctypes.c_float
    return array.ctypes.data_as(ctypes.POINTER(ctype))


def _check(status):
    if status != ORACLE_OK:
        raise OracleError(status)


def partition(plan, states, nodes, edges, dtype=np.float64):
    nodes = np.ascontiguousarray(nodes, dtype=dtype)
    edges = np.ascontiguousarray(edges, dtype=dtype)
    out = np.zeros(1, dtype=dtype)
    _check(getattr(library(), f"oracle_partition_{_suffix(dtype)}")(
        ctypes.byref(oracle_plan(plan)), states, _ptr(nodes), _ptr(edges), _ptr(out)))
    return out[0]


def log_partition(plan, states, nodes, edges, dtype=np.float64):
    nodes = np.ascontiguousarray(nodes, dtype=dtype)
    edges = np.ascontiguousarray(edges, dtype=dtype)
    out = np.zeros(1, dtype=dtype)
    _check(getattr(library(), f"oracle_log_partition_{_suffix(dtype)}")(
        ctypes.byref(oracle_plan(plan)), states, _ptr(nodes), _ptr(edges), _ptr(out)))
    return out[0]


def marginals(plan, states, nodes, edges, dtype=np.float64):
    """(log Z, Z, node marginals [N*K], edge marginals [E*K*K])."""
    nodes = np.ascontiguousarray(nodes, dtype=dtype)
    edges = np.ascontiguousarray(edges, dtype=dtype)
    log_z = np.zeros(1, dtype=dtype)
    z = np.zeros(1, dtype=dtype)
    node_m = np.zeros(plan.num_nodes * states, dtype=dtype)
    edge_m = np.zeros(plan.num_edges * states * states, dtype=dtype)
    _check(getattr(library(), f"oracle_marginals_{_suffix(dtype)}")(
        ctypes.byref(oracle_plan(plan)), states, _ptr(nodes), _ptr(edges), _ptr(log_z),
        _ptr(z), _ptr(node_m), _ptr(edge_m)))
    return log_z[0], z[0], node_m, edge_m


def maximum(plan, states, nodes, edges, dtype=np.float64, math=MATH_LIBM):
    """(log weight, states [N] uint32)."""
    nodes = np.ascontiguousarray(nodes, dtype=dtype)
    edges = np.ascontiguousarray(edges, dtype=dtype)
    weight = np.zeros(1, dtype=dtype)
    assignment = np.zeros(plan.num_nodes, dtype=np.uint32)
    _check(getattr(library(), f"oracle_map_{_suffix(dtype)}")(
        ctypes.byref(oracle_plan(plan)), states, _ptr(nodes), _ptr(edges), math,
        _ptr(weight), _u32(assignment)))
    return weight[0], assignment


def maximum_margins(plan, states, nodes, edges, dtype=np.float64, math=MATH_LIBM):
    """(log weight, states [N] uint32, margins [N]): MAP with, per node, the
    gap between the chosen maximum and the best other candidate of the
    comparison that decided its state."""
    nodes = np.ascontiguousarray(nodes, dtype=dtype)
    edges = np.ascontiguousarray(edges, dtype=dtype)
    weight = np.zeros(1, dtype=dtype)
    assignment = np.zeros(plan.num_nodes, dtype=np.uint32)
    margins = np.zeros(plan.num_nodes, dtype=dtype)
    _check(getattr(library(), f"oracle_map_margins_{_suffix(dtype)}")(
        ctypes.byref(oracle_plan(plan)), states, _ptr(nodes), _ptr(edges), math,
        _ptr(weight), _u32(assignment), _ptr(margins)))
    return weight[0], assignment, margins


def sample_margins(plan, states, nodes, edges, uniforms, dtype=np.float64,
                   math=MATH_LIBM):
    """(states [N] uint32, margins [N]): a posterior sample with, per node,
    the distance from its uniform to the nearer end of the chosen state's
    cumulative interval."""
    nodes = np.ascontiguousarray(nodes, dtype=dtype)
    edges = np.ascontiguousarray(edges, dtype=dtype)
    uniforms = np.ascontiguousarray(uniforms, dtype=dtype)
    assignment = np.zeros(plan.num_nodes, dtype=np.uint32)
    margins = np.zeros(plan.num_nodes, dtype=dtype)
    _check(getattr(library(), f"oracle_sample_margins_{_suffix(dtype)}")(
        ctypes.byref(oracle_plan(plan)), states, _ptr(nodes), _ptr(edges),
        _ptr(uniforms), math, _u32(assignment), _ptr(margins)))
    return assignment, margins


def sample(plan, states, nodes, edges, uniforms, dtype=np.float64, math=MATH_LIBM):
    nodes = np.ascontiguousarray(nodes, dtype=dtype)
    edges = np.ascontiguousarray(edges, dtype=dtype)
    uniforms = np.ascontiguousarray(uniforms, dtype=dtype)
    assignment = np.zeros(plan.num_nodes, dtype=np.uint32)
    _check(getattr(library(), f"oracle_sample_{_suffix(dtype)}")(
        ctypes.byref(oracle_plan(plan)), states, _ptr(nodes), _ptr(edges),
        _ptr(uniforms), math, _u32(assignment)))
    return assignment


# ------------------------------------------------------------ reference build
class Reference:
    """The reference's own CPU library (oracle/_ref), one tree per model."""

    def __init__(self, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        path = REF_DIR / f"libref_{_suffix(dtype)}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(str(path))
        scalar = ctypes.c_double if self.dtype == np.float64 else ctypes.c_float
        p = ctypes.POINTER(scalar)
        u = ctypes.POINTER(ctypes.c_uint32)
        v = ctypes.c_void_p
        lib.ref_model_create.argtypes = [ctypes.POINTER(ctypes.c_int64), ctypes.c_size_t,
                                         ctypes.c_size_t]
        lib.ref_model_create.restype = v
        lib.ref_model_destroy.argtypes = [v]
        lib.ref_model_destroy.restype = None
        for fn, args in (("ref_partition", [v, p, p, p]),
                         ("ref_log_partition", [v, p, p, p]),
                         ("ref_marginals", [v, p, p, p, p, p, p]),
                         ("ref_map", [v, p, p, p, u]),
                         ("ref_sample", [v, p, p, p, u])):
            getattr(lib, fn).argtypes = args
            getattr(lib, fn).restype = ctypes.c_int
        lib.ref_last_error.restype = ctypes.c_char_p
        self.lib = lib

    @staticmethod
    def available(dtype=np.float64) -> bool:
        return (REF_DIR / f"libref_{_suffix(dtype)}.so").exists()

    def model(self, parents, states):
        parents = np.ascontiguousarray(parents, dtype=np.int64)
        handle = self.lib.ref_model_create(
            parents.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), parents.size, states)
        if not handle:
            raise ValueError(self.lib.ref_last_error().decode())
        return handle

    def destroy(self, handle):
        self.lib.ref_model_destroy(handle)

    def _call(self, status):
        if status != 0:
            raise OracleError(status)

    def marginals(self, handle, nodes, edges, num_nodes, num_edges, states):
        nodes = np.ascontiguousarray(nodes, dtype=self.dtype)
        edges = np.ascontiguousarray(edges, dtype=self.dtype)
        log_z = np.zeros(1, dtype=self.dtype)
        z = np.zeros(1, dtype=self.dtype)
        node_m = np.zeros(num_nodes * states, dtype=self.dtype)
        edge_m = np.zeros(num_edges * states * states, dtype=self.dtype)
        self._call(self.lib.ref_marginals(handle, _ptr(nodes), _ptr(edges), _ptr(log_z),
                                          _ptr(z), _ptr(node_m), _ptr(edge_m)))
        return log_z[0], z[0], node_m, edge_m

    def log_partition(self, handle, nodes, edges):
        nodes = np.ascontiguousarray(nodes, dtype=self.dtype)
        edges = np.ascontiguousarray(edges, dtype=self.dtype)
        out = np.zeros(1, dtype=self.dtype)
        self._call(self.lib.ref_log_partition(handle, _ptr(nodes), _ptr(edges), _ptr(out)))
        return out[0]

    def partition(self, handle, nodes, edges):
        nodes = np.ascontiguousarray(nodes, dtype=self.dtype)
        edges = np.ascontiguousarray(edges, dtype=self.dtype)
        out = np.zeros(1, dtype=self.dtype)
        self._call(self.lib.ref_partition(handle, _ptr(nodes), _ptr(edges), _ptr(out)))
        return out[0]

    def maximum(self, handle, nodes, edges, num_nodes):
        nodes = np.ascontiguousarray(nodes, dtype=self.dtype)
        edges = np.ascontiguousarray(edges, dtype=self.dtype)
        weight = np.zeros(1, dtype=self.dtype)
        assignment = np.zeros(num_nodes, dtype=np.uint32)
        self._call(self.lib.ref_map(handle, _ptr(nodes), _ptr(edges), _ptr(weight),
                                    _u32(assignment)))
        return weight[0], assignment

    def sample(self, handle, nodes, edges, uniforms, num_nodes):
        nodes = np.ascontiguousarray(nodes, dtype=self.dtype)
        edges = np.ascontiguousarray(edges, dtype=self.dtype)
        uniforms = np.ascontiguousarray(uniforms, dtype=self.dtype)
        assignment = np.zeros(num_nodes, dtype=np.uint32)
        self._call(self.lib.ref_sample(handle, _ptr(nodes), _ptr(edges), _ptr(uniforms),
                                       _u32(assignment)))
        return assignment
