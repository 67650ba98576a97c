"""Python mirror of the reference accelerator API, over the C ABI.

Names follow include/tree_hmm/accelerator.h and
include/tree_hmm/detail/gpu_backend_api.inc of the reference (snake_case):
Workspace.reserve*, inputs(), categorical_inputs(), uniforms(), and the
prepared calls. C++ exception classes map to the Python exceptions below.
Returned arrays are views of workspace-owned pinned memory, valid until the
workspace is reserved again or destroyed (accelerator.h:113-114).
"""
from __future__ import annotations

import ctypes
import dataclasses
import enum
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import library


class InvalidArgument(ValueError):
    """std::invalid_argument."""


class LogicError(RuntimeError):
    """std::logic_error."""


class DomainError(ArithmeticError):
    """std::domain_error."""


class LengthError(OverflowError):
    """std::length_error."""


class AcceleratorError(RuntimeError):
    """std::runtime_error raised by a failing CUDA runtime call."""


_ERRORS = {
    _lib.THMM_INVALID_ARGUMENT: InvalidArgument,
    _lib.THMM_LOGIC_ERROR: LogicError,
    _lib.THMM_DOMAIN_ERROR: DomainError,
    _lib.THMM_LENGTH_ERROR: LengthError,
    _lib.THMM_RUNTIME_ERROR: AcceleratorError,
}


def _check(status: int) -> None:
    if status != _lib.THMM_OK:
        message = library().thmm_last_error().decode()
        raise _ERRORS.get(status, AcceleratorError)(message)


def _ptr(array: np.ndarray | None) -> int | None:
    return None if array is None else array.ctypes.data


def _view(address: int | None, count: int, dtype) -> np.ndarray:
    dtype = np.dtype(dtype)
    if count == 0 or not address:
        return np.zeros(0, dtype=dtype)
    buffer = (ctypes.c_char * (count * dtype.itemsize)).from_address(address)
    return np.frombuffer(buffer, dtype=dtype, count=count)


class CategoricalInputUpdate(enum.IntEnum):
    """tree_hmm::CategoricalInputUpdate (accelerator.h:89-93)."""

    kAll = _lib.THMM_UPDATE_ALL
    kFactors = _lib.THMM_UPDATE_FACTORS
    kNone = _lib.THMM_UPDATE_NONE


class Plan:
    """btrc::MakePlan(parents): the rake/compress plan of one tree."""

    def __init__(self, parents: Sequence[int] | None = None, *, _handle: int | None = None):
        lib = library()
        if _handle is None:
            parents = np.ascontiguousarray(parents, dtype=np.int64)
            handle = ctypes.c_void_p()
            _check(lib.thmm_plan_create(
                parents.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), parents.size,
                ctypes.byref(handle)))
            _handle = handle.value
        self._handle = _handle
        self._lib = lib
        info = _lib.PlanInfo()
        _check(lib.thmm_plan_get_info(self._handle, ctypes.byref(info)))
        self.num_nodes = info.num_nodes
        self.num_edges = info.num_edges
        self.num_branches = info.num_branches
        self.num_compressions = info.num_compressions
        self.num_combinations = info.num_combinations
        self.num_absorptions = info.num_absorptions
        self.num_batches = info.num_batches
        self.num_rounds = info.num_rounds
        self.root = info.root
        self._arrays = None

    @classmethod
    def many(cls, parent_arrays: Sequence[Sequence[int]], threads: int = 0) -> list["Plan"]:
        """Plans of many trees built on `threads` host threads (0: all)."""
        lib = library()
        arrays = [np.ascontiguousarray(p, dtype=np.int64) for p in parent_arrays]
        offsets = np.zeros(len(arrays) + 1, dtype=np.uintp)
        offsets[1:] = np.cumsum([a.size for a in arrays])
        flat = (np.concatenate(arrays) if arrays else np.zeros(0, dtype=np.int64))
        flat = np.ascontiguousarray(flat, dtype=np.int64)
        handles = (ctypes.c_void_p * max(1, len(arrays)))()
        _check(lib.thmm_plan_create_many(
            flat.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)), len(arrays), threads,
            handles))
        return [cls(_handle=handles[t]) for t in range(len(arrays))]

    _WIDTHS = {"edge_parents": ("num_edges", 1), "edge_children": ("num_edges", 1),
               "rakes": ("num_branches", 4), "combinations": ("num_combinations", 3),
               "absorptions": ("num_absorptions", 3),
               "compressions": ("num_compressions", 6), "batches": ("num_batches", 3)}

    def __getattr__(self, name):
        # Operation arrays are copied out of the C++ plan on first use only.
        if name not in Plan._WIDTHS:
            raise AttributeError(name)
        if self.__dict__.get("_arrays") is None:
            arrays = _lib.PlanArrays()
            _check(self._lib.thmm_plan_get_arrays(self._handle, ctypes.byref(arrays)))
            self.__dict__["_arrays"] = arrays
        rows_attr, width = Plan._WIDTHS[name]
        rows = getattr(self, rows_attr)
        address = ctypes.cast(getattr(self._arrays, name), ctypes.c_void_p).value
        values = _view(address, rows * width, np.uint32).copy()
        values = values if width == 1 else values.reshape(rows, width)
        self.__dict__[name] = values
        return values

    @property
    def handle(self) -> int:
        return self._handle

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle:
            self._lib.thmm_plan_destroy(handle)
            self._handle = None


@dataclasses.dataclass
class AcceleratorTimings:
    upload_ms: float
    kernel_ms: float
    download_ms: float
    wall_ms: float

    @classmethod
    def from_c(cls, timings: _lib.Timings) -> "AcceleratorTimings":
        return cls(timings.upload_ms, timings.kernel_ms, timings.download_ms,
                   timings.wall_ms)


@dataclasses.dataclass
class PartitionView:
    values: np.ndarray
    timings: AcceleratorTimings


@dataclasses.dataclass
class BatchedMaximumAssignmentView:
    log_weights: np.ndarray
    states: np.ndarray
    timings: AcceleratorTimings


@dataclasses.dataclass
class BatchedPosteriorSampleView:
    states: np.ndarray
    timings: AcceleratorTimings


@dataclasses.dataclass
class BatchedMarginalView:
    log_partitions: np.ndarray
    nodes: np.ndarray
    edges: np.ndarray
    timings: AcceleratorTimings


@dataclasses.dataclass
class BatchedModelView:
    """BatchedModelView (accelerator.h:13-23). For a forest workspace `plan`
    may be None and `batch` is the tree count."""

    plan: Plan | None
    states: int
    batch: int
    node_potentials: np.ndarray
    edge_potentials: np.ndarray


@dataclasses.dataclass
class BatchedCategoricalModelView:
    """BatchedCategoricalModelView (accelerator.h:41-58)."""

    plan: Plan | None
    states: int
    batch: int
    categories: int
    observation_nodes: np.ndarray
    observations: np.ndarray
    root_potential: np.ndarray
    emission_potentials: np.ndarray
    edge_potentials: np.ndarray


MutableBatchedModelView = BatchedModelView
MutableBatchedCategoricalModelView = BatchedCategoricalModelView


class Workspace:
    """tree_hmm::cuda::Workspace (gpu_backend_api.inc:4-95)."""

    def __init__(self):
        self._lib = library()
        handle = ctypes.c_void_p()
        _check(self._lib.thmm_workspace_create(ctypes.byref(handle)))
        self._handle = handle.value
        self._dtype = np.dtype(np.float64)
        self._plans: list[Plan] = []
        self._observation_nodes = np.zeros(0, dtype=np.uint32)
        self._capacity = 0
        self._forest = False
        self._states = 0
        self._categories = 0

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle:
            self._lib.thmm_workspace_destroy(handle)
            self._handle = None

    @property
    def handle(self) -> int:
        return self._handle

    @property
    def dtype(self) -> np.dtype:
        return self._dtype

    @staticmethod
    def _flags(kind: str, compute) -> int:
        table = {"": 0, "maximum": _lib.THMM_RESERVE_MAXIMUM,
                 "sampling": _lib.THMM_RESERVE_SAMPLING,
                 "marginals": _lib.THMM_RESERVE_MARGINALS,
                 "device": _lib.THMM_RESERVE_DEVICE_ONLY}
        flags = 0
        for part in kind.split(","):  # e.g. "maximum,sampling"
            flags |= table[part.strip()]
        if isinstance(compute, str) and compute == "bf16":
            flags |= _lib.THMM_COMPUTE_BF16  # BF16 tier of the tensor-core engine
        elif compute is not None and np.dtype(compute) == np.float64:
            flags |= _lib.THMM_COMPUTE_F64
        return flags

    def _scalar(self, scalar) -> int:
        self._dtype = np.dtype(scalar)
        if self._dtype not in (np.float32, np.float64):
            raise InvalidArgument("scalar must be float32 or float64")
        return self._dtype.itemsize

    # ------------------------------------------------------------- reserve
    def _reserve(self, kind, plan, states, batch_capacity, device, scalar, compute):
        self._forest, self._states = False, states
        self._plans = [plan]
        self._capacity = batch_capacity
        self._observation_nodes = np.zeros(0, dtype=np.uint32)
        _check(self._lib.thmm_reserve(self._handle, plan.handle, states, batch_capacity,
                                      device, self._flags(kind, compute),
                                      self._scalar(scalar)))

    def reserve(self, plan, states, batch_capacity, device=0, *, scalar=np.float64,
                compute=None):
        self._reserve("", plan, states, batch_capacity, device, scalar, compute)

    def reserve_maximum(self, plan, states, batch_capacity, device=0, *,
                        scalar=np.float64, compute=None):
        self._reserve("maximum", plan, states, batch_capacity, device, scalar, compute)

    def reserve_sampling(self, plan, states, batch_capacity, device=0, *,
                         scalar=np.float64, compute=None):
        self._reserve("sampling", plan, states, batch_capacity, device, scalar, compute)

    def reserve_marginals(self, plan, states, batch_capacity, device=0, *,
                          scalar=np.float64, compute=None):
        self._reserve("marginals", plan, states, batch_capacity, device, scalar, compute)

    def _reserve_categorical(self, kind, plan, states, batch_capacity, categories,
                             observation_nodes, device, scalar, compute):
        nodes = np.ascontiguousarray(observation_nodes, dtype=np.uint32)
        self._forest, self._states, self._categories = False, states, categories
        self._plans = [plan]
        self._capacity = batch_capacity
        self._observation_nodes = nodes
        _check(self._lib.thmm_reserve_categorical(
            self._handle, plan.handle, states, batch_capacity, categories,
            _ptr(nodes), nodes.size, device, self._flags(kind, compute),
            self._scalar(scalar)))

    def reserve_categorical(self, plan, states, batch_capacity, categories,
                            observation_nodes, device=0, *, scalar=np.float64,
                            compute=None):
        self._reserve_categorical("", plan, states, batch_capacity, categories,
                                  observation_nodes, device, scalar, compute)

    def reserve_categorical_maximum(self, plan, states, batch_capacity, categories,
                                    observation_nodes, device=0, *, scalar=np.float64,
                                    compute=None):
        self._reserve_categorical("maximum", plan, states, batch_capacity, categories,
                                  observation_nodes, device, scalar, compute)

    def reserve_categorical_sampling(self, plan, states, batch_capacity, categories,
                                     observation_nodes, device=0, *, scalar=np.float64,
                                     compute=None):
        self._reserve_categorical("sampling", plan, states, batch_capacity, categories,
                                  observation_nodes, device, scalar, compute)

    def reserve_categorical_marginals(self, plan, states, batch_capacity, categories,
                                      observation_nodes, device=0, *,
                                      scalar=np.float64, compute=None):
        self._reserve_categorical("marginals", plan, states, batch_capacity, categories,
                                  observation_nodes, device, scalar, compute)

    def reserve_forest(self, plans, states, device=0, *, kind="", scalar=np.float64,
                       compute=None):
        """Extension: one independent tree per plan, each with its own edges."""
        self._forest, self._states = True, states
        self._plans = list(plans)
        self._capacity = len(self._plans)
        self._observation_nodes = np.zeros(0, dtype=np.uint32)
        handles = (ctypes.c_void_p * len(self._plans))(*[p.handle for p in self._plans])
        _check(self._lib.thmm_reserve_forest(
            self._handle, handles, len(self._plans), states, device,
            self._flags(kind, compute), self._scalar(scalar)))

    def reserve_forest_categorical(self, plans, states, categories, observation_nodes,
                                   device=0, *, kind="", scalar=np.float64,
                                   compute=None):
        """Extension: categorical forest; `observation_nodes[t]` lists tree t's
        observed nodes (strictly increasing)."""
        self._forest, self._states, self._categories = True, states, categories
        self._plans = list(plans)
        self._capacity = len(self._plans)
        counts = np.array([len(o) for o in observation_nodes], dtype=np.uint64)
        flat = (np.concatenate([np.asarray(o, dtype=np.uint32) for o in observation_nodes])
                if len(observation_nodes) else np.zeros(0, dtype=np.uint32))
        flat = np.ascontiguousarray(flat, dtype=np.uint32)
        self._observation_nodes = flat
        handles = (ctypes.c_void_p * len(self._plans))(*[p.handle for p in self._plans])
        _check(self._lib.thmm_reserve_forest_categorical(
            self._handle, handles, len(self._plans), states, categories, _ptr(flat),
            _ptr(counts), device, self._flags(kind, compute), self._scalar(scalar)))

    # ------------------------------------------------------------- staging
    def inputs(self, batch=None) -> BatchedModelView:
        view = _lib.DenseInputView()
        _check(self._lib.thmm_inputs(self._handle, self._batch(batch), ctypes.byref(view)))
        return BatchedModelView(self._plan_or_none(), view.states, view.batch,
                                _view(view.node_potentials, view.node_count, self._dtype),
                                _view(view.edge_potentials, view.edge_count, self._dtype))

    def categorical_inputs(self, batch=None) -> BatchedCategoricalModelView:
        view = _lib.CategoricalInputView()
        _check(self._lib.thmm_categorical_inputs(self._handle, self._batch(batch),
                                                 ctypes.byref(view)))
        obs_nodes = _view(ctypes.cast(view.observation_nodes, ctypes.c_void_p).value,
                          view.observation_node_count, np.uint32)
        return BatchedCategoricalModelView(
            self._plan_or_none(), view.states, view.batch, view.categories, obs_nodes,
            _view(ctypes.cast(view.observations, ctypes.c_void_p).value,
                  view.observation_count, np.uint8),
            _view(view.root_potential, view.root_count, self._dtype),
            _view(view.emission_potentials, view.emission_count, self._dtype),
            _view(view.edge_potentials, view.edge_count, self._dtype))

    def uniforms(self, batch=None) -> np.ndarray:
        address = ctypes.c_void_p()
        count = ctypes.c_size_t()
        _check(self._lib.thmm_uniforms(self._handle, self._batch(batch),
                                       ctypes.byref(address), ctypes.byref(count)))
        return _view(address.value, count.value, self._dtype)

    def device_buffers(self) -> dict:
        """Extension: zero-copy torch CUDA views of the workspace's device
        input and result buffers (thmm_device_buffers_get), keyed by name;
        absent where the workspace has no such buffer. Write inputs produced
        on the GPU into them, then call device_inputs_ready(); read the
        results of enqueue() from them. Valid until the next reserve."""
        import torch

        buffers = _lib.DeviceBuffers()
        _check(self._lib.thmm_device_buffers_get(self._handle, ctypes.byref(buffers)))
        K = self._states
        if self._forest:
            nodes = sum(p.num_nodes for p in self._plans)
            edges_in = edges_out = sum(p.num_edges for p in self._plans)
        else:
            nodes = self._capacity * self._plans[0].num_nodes
            edges_in = self._plans[0].num_edges
            edges_out = self._capacity * edges_in
        scalar = "<f8" if self._dtype == np.float64 else "<f4"
        shapes = {"node_potentials": (nodes * K, scalar),
                  "edge_potentials": (edges_in * K * K, scalar),
                  "observations": (len(self._observation_nodes) *
                                   (1 if self._forest else self._capacity), "|u1"),
                  "root_potential": (K, scalar),
                  "emission_potentials": (None, scalar),
                  "uniforms": (nodes, scalar), "values": (self._capacity, scalar),
                  "node_marginals": (nodes * K, scalar),
                  "edge_marginals": (edges_out * K * K, scalar), "states": (nodes, "<u4")}
        out = {}
        for name, (count, typestr) in shapes.items():
            address = getattr(buffers, name)
            if not address:
                continue
            if count is None:  # emission table: categories x K
                count = self._categories * K
            out[name] = torch.as_tensor(_DeviceArray(address, count, typestr), device="cuda")
        return out

    def device_inputs_ready(self, batch=None) -> None:
        """Extension: the device inputs written through device_buffers() are
        resident for `batch` items (thmm_device_inputs_ready)."""
        _check(self._lib.thmm_device_inputs_ready(self._handle, self._batch(batch)))

    def _plan_or_none(self):
        return self._plans[0] if len(self._plans) == 1 else None

    def _batch(self, batch):
        return self._capacity if batch is None else batch

    # ------------------------------------------------------- model structs
    def _array(self, values, dtype=None):
        return np.ascontiguousarray(values, dtype=dtype or self._dtype)

    def _dense(self, model: BatchedModelView):
        nodes = self._array(model.node_potentials)
        edges = self._array(model.edge_potentials)
        plan = model.plan.handle if model.plan is not None else None
        struct = _lib.DenseModel(plan, model.states, model.batch, _ptr(nodes), nodes.size,
                                 _ptr(edges), edges.size)
        return struct, (nodes, edges)

    def _categorical(self, model: BatchedCategoricalModelView):
        obs_nodes = self._array(model.observation_nodes, np.uint32)
        obs = self._array(model.observations, np.uint8)
        root = self._array(model.root_potential)
        emission = self._array(model.emission_potentials)
        edges = self._array(model.edge_potentials)
        plan = model.plan.handle if model.plan is not None else None
        struct = _lib.CategoricalModel(
            plan, model.states, model.batch, model.categories, _ptr(obs_nodes),
            obs_nodes.size, _ptr(obs), obs.size, _ptr(root), root.size, _ptr(emission),
            emission.size, _ptr(edges), edges.size)
        return struct, (obs_nodes, obs, root, emission, edges)

    # -------------------------------------------------------- prepared calls
    def _partition(self, model, update, dense_fn, categorical_fn) -> PartitionView:
        result = _lib.PartitionResult()
        if isinstance(model, BatchedCategoricalModelView):
            struct, keep = self._categorical(model)
            _check(categorical_fn(self._handle, ctypes.byref(struct),
                                  int(update if update is not None else 0),
                                  ctypes.byref(result)))
        else:
            struct, keep = self._dense(model)
            _check(dense_fn(self._handle, ctypes.byref(struct), ctypes.byref(result)))
        del keep
        return PartitionView(_view(result.values, result.count, self._dtype),
                             AcceleratorTimings.from_c(result.timings))

    def partition_function_prepared(self, model, update=None) -> PartitionView:
        return self._partition(model, update, self._lib.thmm_partition_function,
                               self._lib.thmm_categorical_partition_function)

    def log_partition_function_prepared(self, model, update=None) -> PartitionView:
        return self._partition(model, update, self._lib.thmm_log_partition_function,
                               self._lib.thmm_categorical_log_partition_function)

    def maximum_a_posteriori_prepared(self, model, update=None):
        result = _lib.MaximumResult()
        if isinstance(model, BatchedCategoricalModelView):
            struct, keep = self._categorical(model)
            _check(self._lib.thmm_categorical_maximum_a_posteriori(
                self._handle, ctypes.byref(struct), int(update or 0),
                ctypes.byref(result)))
        else:
            struct, keep = self._dense(model)
            _check(self._lib.thmm_maximum_a_posteriori(self._handle, ctypes.byref(struct),
                                                       ctypes.byref(result)))
        del keep
        states = _view(ctypes.cast(result.states, ctypes.c_void_p).value,
                       result.state_count, np.uint32)
        return BatchedMaximumAssignmentView(
            _view(result.log_weights, result.count, self._dtype), states,
            AcceleratorTimings.from_c(result.timings))

    def posterior_sample_prepared(self, model, uniforms, update=None):
        result = _lib.SampleResult()
        uniforms = self._array(uniforms)
        if isinstance(model, BatchedCategoricalModelView):
            struct, keep = self._categorical(model)
            _check(self._lib.thmm_categorical_posterior_sample(
                self._handle, ctypes.byref(struct), _ptr(uniforms), uniforms.size,
                int(update or 0), ctypes.byref(result)))
        else:
            struct, keep = self._dense(model)
            _check(self._lib.thmm_posterior_sample(self._handle, ctypes.byref(struct),
                                                   _ptr(uniforms), uniforms.size,
                                                   ctypes.byref(result)))
        del keep
        states = _view(ctypes.cast(result.states, ctypes.c_void_p).value, result.count,
                       np.uint32)
        return BatchedPosteriorSampleView(states, AcceleratorTimings.from_c(result.timings))

    def posterior_marginals_prepared(self, model, update=None) -> BatchedMarginalView:
        result = _lib.MarginalResult()
        if isinstance(model, BatchedCategoricalModelView):
            struct, keep = self._categorical(model)
            _check(self._lib.thmm_categorical_posterior_marginals(
                self._handle, ctypes.byref(struct), int(update or 0),
                ctypes.byref(result)))
        else:
            struct, keep = self._dense(model)
            _check(self._lib.thmm_posterior_marginals(self._handle, ctypes.byref(struct),
                                                      ctypes.byref(result)))
        del keep
        return BatchedMarginalView(
            _view(result.log_partitions, result.count, self._dtype),
            _view(result.nodes, result.node_count, self._dtype),
            _view(result.edges, result.edge_count, self._dtype),
            AcceleratorTimings.from_c(result.timings))

    # ------------------------------------------------------- device-only
    def enqueue(self, operation: int) -> int:
        nodes = ctypes.c_uint64()
        _check(self._lib.thmm_enqueue(self._handle, operation, ctypes.byref(nodes)))
        return nodes.value

    def autotune(self, operation: int = 4, repeats: int = 3) -> dict:
        """Times candidate team thresholds and CTAs per SM for `operation`
        (thmm_enqueue codes) on the resident inputs and keeps the fastest."""
        tuning = _lib.Tuning()
        _check(self._lib.thmm_autotune(self._handle, operation, repeats,
                                       ctypes.byref(tuning)))
        return _tuning_dict(tuning)

    @property
    def tuning(self) -> dict:
        tuning = _lib.Tuning()
        _check(self._lib.thmm_get_tuning(self._handle, ctypes.byref(tuning)))
        return _tuning_dict(tuning)

    def set_tuning(self, team_threshold: int, ctas_per_sm=(0, 0, 0, 0),
                   stripes: int = 0, schedule: int | None = None,
                   phase_rounds: int | None = None) -> None:
        """Applies a launch tuning. `schedule` (THMM_SCHEDULE_TEAMS or
        THMM_SCHEDULE_PHASES) and `phase_rounds` (grid-wide rounds of the
        phase schedule, 0 automatic) default to the workspace's current
        ones."""
        current = self.tuning
        if schedule is None:
            schedule = current["schedule"]
        if phase_rounds is None:
            phase_rounds = current["phase_rounds"]
        tuning = _lib.Tuning()
        tuning.team_threshold = team_threshold
        for i, value in enumerate(ctas_per_sm):
            tuning.ctas_per_sm[i] = value
        tuning.stripes = stripes
        tuning.schedule = schedule
        tuning.phase_rounds = phase_rounds
        _check(self._lib.thmm_set_tuning(self._handle, ctypes.byref(tuning)))

    @property
    def stream(self) -> int:
        return self._lib.thmm_workspace_stream(self._handle)

    def synchronize(self) -> None:
        _check(self._lib.thmm_workspace_synchronize(self._handle))

    @property
    def launches(self) -> int:
        return self._lib.thmm_workspace_launches(self._handle)


class _DeviceArray:
    """A device buffer described by the CUDA array interface (for
    torch.as_tensor without a copy)."""

    def __init__(self, address: int, count: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": typestr,
                                         "data": (address, False), "version": 3,
                                         "strides": None}


def _tuning_dict(tuning) -> dict:
    return {"team_threshold": int(tuning.team_threshold),
            "ctas_per_sm": [int(v) for v in tuning.ctas_per_sm],
            "stripes": int(tuning.stripes),
            "kernel_ms": float(tuning.kernel_ms), "candidates": int(tuning.candidates),
            "schedule": int(tuning.schedule), "phase_rounds": int(tuning.phase_rounds)}


def available() -> bool:
    """tree_hmm::cuda::Available()."""
    return bool(library().thmm_available())


def device_description(device: int = 0) -> str:
    """tree_hmm::cuda::DeviceDescription(device)."""
    buffer = ctypes.create_string_buffer(256)
    _check(library().thmm_device_description(device, buffer, len(buffer)))
    return buffer.value.decode()
