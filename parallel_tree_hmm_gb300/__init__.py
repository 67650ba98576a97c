"""GB300-native batched tree-HMM inference (sum-product log Z, posterior
marginals = d log Z / d log factors, MAP, posterior sampling) over rake/compress
plans, behind the accelerator API of parallel_tree_hmm.

The compute path is libthmm_gb300.so (hand-written sm_103a kernels + C++ host
runtime); this package is its ctypes front end.
"""
from .api import (AcceleratorError, AcceleratorTimings, BatchedCategoricalModelView,
                  BatchedMarginalView, BatchedMaximumAssignmentView, BatchedModelView,
                  BatchedPosteriorSampleView, CategoricalInputUpdate, DomainError,
                  InvalidArgument, LengthError, LogicError, MutableBatchedCategoricalModelView,
                  MutableBatchedModelView, PartitionView, Plan, Workspace, available,
                  device_description)

__all__ = [
    "AcceleratorError", "AcceleratorTimings", "BatchedCategoricalModelView",
    "BatchedMarginalView", "BatchedMaximumAssignmentView", "BatchedModelView",
    "BatchedPosteriorSampleView", "CategoricalInputUpdate", "DomainError",
    "InvalidArgument", "LengthError", "LogicError", "MutableBatchedCategoricalModelView",
    "MutableBatchedModelView", "PartitionView", "Plan", "Workspace", "available",
    "device_description",
]
