// C++ accelerator API on GB300: the reference's tree_hmm::cuda interface
// (include/tree_hmm/detail/gpu_backend_api.inc:1-142) as a header-only layer
// over the C ABI of libthmm_gb300.so (include/thmm_gb300.h).
//
// Names, overloads, argument meaning, returned views, their lifetime and the
// exception classes are the reference's; code written against tree_hmm::cuda
// switches by including this header and using tree_hmm::gb300 (or
// tree_hmm/gb300_as_cuda.h, which makes tree_hmm::cuda an alias). Two
// additions: Workspace::SetCompute selects FP32 (default) or FP64 arithmetic
// for the sum-product paths, and Workspace::native_handle exposes the C
// handle (for the forest and device-only entry points of the C ABI).
#ifndef TREE_HMM_GB300_H_
#define TREE_HMM_GB300_H_

#include <cstddef>
#include <cstdint>
#include <span>
#include <stdexcept>
#include <string>
#include <utility>

#include "thmm_gb300.h"
#include "tree_hmm/accelerator.h"

namespace tree_hmm::gb300 {

enum class Compute { kFloat32, kFloat64 };

namespace detail {

// Rethrows a C-ABI status as the reference's exception class.
inline void Throw(thmm_status status) {
  if (status == THMM_OK)
    return;
  const std::string message = thmm_last_error();
  switch (status) {
  case THMM_INVALID_ARGUMENT:
    throw std::invalid_argument(message);
  case THMM_LOGIC_ERROR:
    throw std::logic_error(message);
  case THMM_DOMAIN_ERROR:
    throw std::domain_error(message);
  case THMM_LENGTH_ERROR:
    throw std::length_error(message);
  default:
    throw std::runtime_error(message);
  }
}

inline const thmm_plan *Handle(const btrc::Plan &plan) {
  return reinterpret_cast<const thmm_plan *>(&plan);
}

inline constexpr std::uint32_t kScalarBytes = sizeof(Scalar);

inline AcceleratorTimings Timings(const thmm_timings &t) {
  return {t.upload_ms, t.kernel_ms, t.download_ms, t.wall_ms};
}

inline thmm_dense_model Dense(const BatchedModelView &m) {
  return {Handle(m.plan),          m.states,
          m.batch,                 m.node_potentials.data(),
          m.node_potentials.size(), m.edge_potentials.data(),
          m.edge_potentials.size()};
}

inline thmm_categorical_model Categorical(const BatchedCategoricalModelView &m) {
  return {Handle(m.plan),
          m.states,
          m.batch,
          m.categories,
          m.observation_nodes.data(),
          m.observation_nodes.size(),
          m.observations.data(),
          m.observations.size(),
          m.root_potential.data(),
          m.root_potential.size(),
          m.emission_potentials.data(),
          m.emission_potentials.size(),
          m.edge_potentials.data(),
          m.edge_potentials.size()};
}

inline int Update(CategoricalInputUpdate update) {
  switch (update) {
  case CategoricalInputUpdate::kAll:
    return THMM_UPDATE_ALL;
  case CategoricalInputUpdate::kFactors:
    return THMM_UPDATE_FACTORS;
  case CategoricalInputUpdate::kNone:
    return THMM_UPDATE_NONE;
  }
  return THMM_UPDATE_ALL;
}

inline std::span<const Scalar> Values(const void *data, std::size_t count) {
  return {static_cast<const Scalar *>(data), count};
}

} // namespace detail

inline bool Available() { return thmm_available() != 0; }

inline std::string DeviceDescription(int device = 0) {
  char buffer[256];
  detail::Throw(thmm_device_description(device, buffer, sizeof buffer));
  return buffer;
}

class Workspace {
public:
  Workspace() { detail::Throw(thmm_workspace_create(&handle_)); }
  ~Workspace() {
    if (handle_ != nullptr)
      thmm_workspace_destroy(handle_);
  }
  Workspace(Workspace &&other) noexcept
      : handle_(std::exchange(other.handle_, nullptr)),
        plan_(std::exchange(other.plan_, nullptr)),
        capacity_(std::exchange(other.capacity_, 0)), compute_(other.compute_) {}
  Workspace &operator=(Workspace &&other) noexcept {
    if (this != &other) {
      if (handle_ != nullptr)
        thmm_workspace_destroy(handle_);
      handle_ = std::exchange(other.handle_, nullptr);
      plan_ = std::exchange(other.plan_, nullptr);
      capacity_ = std::exchange(other.capacity_, 0);
      compute_ = other.compute_;
    }
    return *this;
  }
  Workspace(const Workspace &) = delete;
  Workspace &operator=(const Workspace &) = delete;

  // Arithmetic of the sum-product paths; applies from the next Reserve*.
  void SetCompute(Compute compute) { compute_ = compute; }

  void Reserve(const btrc::Plan &plan, std::size_t states,
               std::size_t batch_capacity, int device = 0) {
    ReserveDense(plan, states, batch_capacity, device, 0);
  }
  void ReserveCategorical(const btrc::Plan &plan, std::size_t states,
                          std::size_t batch_capacity, std::size_t categories,
                          std::span<const btrc::Index> observation_nodes,
                          int device = 0) {
    ReserveCategoricalWith(plan, states, batch_capacity, categories,
                           observation_nodes, device, 0);
  }
  void ReserveMaximum(const btrc::Plan &plan, std::size_t states,
                      std::size_t batch_capacity, int device = 0) {
    ReserveDense(plan, states, batch_capacity, device, THMM_RESERVE_MAXIMUM);
  }
  void ReserveCategoricalMaximum(const btrc::Plan &plan, std::size_t states,
                                 std::size_t batch_capacity, std::size_t categories,
                                 std::span<const btrc::Index> observation_nodes,
                                 int device = 0) {
    ReserveCategoricalWith(plan, states, batch_capacity, categories,
                           observation_nodes, device, THMM_RESERVE_MAXIMUM);
  }
  void ReserveSampling(const btrc::Plan &plan, std::size_t states,
                       std::size_t batch_capacity, int device = 0) {
    ReserveDense(plan, states, batch_capacity, device, THMM_RESERVE_SAMPLING);
  }
  void ReserveCategoricalSampling(const btrc::Plan &plan, std::size_t states,
                                  std::size_t batch_capacity, std::size_t categories,
                                  std::span<const btrc::Index> observation_nodes,
                                  int device = 0) {
    ReserveCategoricalWith(plan, states, batch_capacity, categories,
                           observation_nodes, device, THMM_RESERVE_SAMPLING);
  }
  void ReserveMarginals(const btrc::Plan &plan, std::size_t states,
                        std::size_t batch_capacity, int device = 0) {
    ReserveDense(plan, states, batch_capacity, device, THMM_RESERVE_MARGINALS);
  }
  void ReserveCategoricalMarginals(const btrc::Plan &plan, std::size_t states,
                                   std::size_t batch_capacity, std::size_t categories,
                                   std::span<const btrc::Index> observation_nodes,
                                   int device = 0) {
    ReserveCategoricalWith(plan, states, batch_capacity, categories,
                           observation_nodes, device, THMM_RESERVE_MARGINALS);
  }

  MutableBatchedModelView Inputs() { return Inputs(capacity_); }
  MutableBatchedModelView Inputs(std::size_t batch) {
    thmm_dense_input_view view{};
    detail::Throw(thmm_inputs(handle_, batch, &view));
    return {*plan_, view.states, view.batch,
            {static_cast<Scalar *>(view.node_potentials), view.node_count},
            {static_cast<Scalar *>(view.edge_potentials), view.edge_count}};
  }
  MutableBatchedCategoricalModelView CategoricalInputs() {
    return CategoricalInputs(capacity_);
  }
  MutableBatchedCategoricalModelView CategoricalInputs(std::size_t batch) {
    thmm_categorical_input_view view{};
    detail::Throw(thmm_categorical_inputs(handle_, batch, &view));
    return {*plan_,
            view.states,
            view.batch,
            view.categories,
            {view.observation_nodes, view.observation_node_count},
            {view.observations, view.observation_count},
            {static_cast<Scalar *>(view.root_potential), view.root_count},
            {static_cast<Scalar *>(view.emission_potentials), view.emission_count},
            {static_cast<Scalar *>(view.edge_potentials), view.edge_count}};
  }
  std::span<Scalar> Uniforms() { return Uniforms(capacity_); }
  std::span<Scalar> Uniforms(std::size_t batch) {
    void *data = nullptr;
    std::size_t count = 0;
    detail::Throw(thmm_uniforms(handle_, batch, &data, &count));
    return {static_cast<Scalar *>(data), count};
  }

  thmm_workspace *native_handle() const { return handle_; }

private:
  std::uint32_t ComputeFlags() const {
    return compute_ == Compute::kFloat64 ? THMM_COMPUTE_F64 : 0u;
  }
  void ReserveDense(const btrc::Plan &plan, std::size_t states, std::size_t batch,
                    int device, std::uint32_t flags) {
    detail::Throw(thmm_reserve(handle_, detail::Handle(plan), states, batch, device,
                               flags | ComputeFlags(), detail::kScalarBytes));
    plan_ = &plan;
    capacity_ = batch;
  }
  void ReserveCategoricalWith(const btrc::Plan &plan, std::size_t states,
                              std::size_t batch, std::size_t categories,
                              std::span<const btrc::Index> observation_nodes,
                              int device, std::uint32_t flags) {
    detail::Throw(thmm_reserve_categorical(
        handle_, detail::Handle(plan), states, batch, categories,
        observation_nodes.data(), observation_nodes.size(), device,
        flags | ComputeFlags(), detail::kScalarBytes));
    plan_ = &plan;
    capacity_ = batch;
  }

  thmm_workspace *handle_ = nullptr;
  const btrc::Plan *plan_ = nullptr;
  std::size_t capacity_ = 0;
  Compute compute_ = Compute::kFloat32;
};

// ----------------------------------------------------------- prepared calls
inline PartitionView PartitionFunctionPrepared(BatchedModelView model,
                                               Workspace &workspace) {
  const thmm_dense_model m = detail::Dense(model);
  thmm_partition_result r{};
  detail::Throw(thmm_partition_function(workspace.native_handle(), &m, &r));
  return {detail::Values(r.values, r.count), detail::Timings(r.timings)};
}

inline PartitionView LogPartitionFunctionPrepared(BatchedModelView model,
                                                  Workspace &workspace) {
  const thmm_dense_model m = detail::Dense(model);
  thmm_partition_result r{};
  detail::Throw(thmm_log_partition_function(workspace.native_handle(), &m, &r));
  return {detail::Values(r.values, r.count), detail::Timings(r.timings)};
}

inline PartitionView
PartitionFunctionPrepared(BatchedCategoricalModelView model, Workspace &workspace,
                          CategoricalInputUpdate update) {
  const thmm_categorical_model m = detail::Categorical(model);
  thmm_partition_result r{};
  detail::Throw(thmm_categorical_partition_function(workspace.native_handle(), &m,
                                                    detail::Update(update), &r));
  return {detail::Values(r.values, r.count), detail::Timings(r.timings)};
}

inline PartitionView PartitionFunctionPrepared(BatchedCategoricalModelView model,
                                               Workspace &workspace) {
  return PartitionFunctionPrepared(model, workspace, CategoricalInputUpdate::kAll);
}

inline PartitionView
LogPartitionFunctionPrepared(BatchedCategoricalModelView model, Workspace &workspace,
                             CategoricalInputUpdate update) {
  const thmm_categorical_model m = detail::Categorical(model);
  thmm_partition_result r{};
  detail::Throw(thmm_categorical_log_partition_function(
      workspace.native_handle(), &m, detail::Update(update), &r));
  return {detail::Values(r.values, r.count), detail::Timings(r.timings)};
}

inline PartitionView LogPartitionFunctionPrepared(BatchedCategoricalModelView model,
                                                  Workspace &workspace) {
  return LogPartitionFunctionPrepared(model, workspace, CategoricalInputUpdate::kAll);
}

inline BatchedMaximumAssignmentView
MaximumAPosterioriPrepared(BatchedModelView model, Workspace &workspace) {
  const thmm_dense_model m = detail::Dense(model);
  thmm_maximum_result r{};
  detail::Throw(thmm_maximum_a_posteriori(workspace.native_handle(), &m, &r));
  return {detail::Values(r.log_weights, r.count), {r.states, r.state_count},
          detail::Timings(r.timings)};
}

inline BatchedMaximumAssignmentView
MaximumAPosterioriPrepared(BatchedCategoricalModelView model, Workspace &workspace,
                           CategoricalInputUpdate update) {
  const thmm_categorical_model m = detail::Categorical(model);
  thmm_maximum_result r{};
  detail::Throw(thmm_categorical_maximum_a_posteriori(
      workspace.native_handle(), &m, detail::Update(update), &r));
  return {detail::Values(r.log_weights, r.count), {r.states, r.state_count},
          detail::Timings(r.timings)};
}

inline BatchedMaximumAssignmentView
MaximumAPosterioriPrepared(BatchedCategoricalModelView model, Workspace &workspace) {
  return MaximumAPosterioriPrepared(model, workspace, CategoricalInputUpdate::kAll);
}

inline BatchedPosteriorSampleView
PosteriorSamplePrepared(BatchedModelView model, std::span<const Scalar> uniforms,
                        Workspace &workspace) {
  const thmm_dense_model m = detail::Dense(model);
  thmm_sample_result r{};
  detail::Throw(thmm_posterior_sample(workspace.native_handle(), &m, uniforms.data(),
                                      uniforms.size(), &r));
  return {{r.states, r.count}, detail::Timings(r.timings)};
}

inline BatchedPosteriorSampleView
PosteriorSamplePrepared(BatchedCategoricalModelView model,
                        std::span<const Scalar> uniforms, Workspace &workspace,
                        CategoricalInputUpdate update) {
  const thmm_categorical_model m = detail::Categorical(model);
  thmm_sample_result r{};
  detail::Throw(thmm_categorical_posterior_sample(workspace.native_handle(), &m,
                                                  uniforms.data(), uniforms.size(),
                                                  detail::Update(update), &r));
  return {{r.states, r.count}, detail::Timings(r.timings)};
}

inline BatchedPosteriorSampleView
PosteriorSamplePrepared(BatchedCategoricalModelView model,
                        std::span<const Scalar> uniforms, Workspace &workspace) {
  return PosteriorSamplePrepared(model, uniforms, workspace,
                                 CategoricalInputUpdate::kAll);
}

inline BatchedMarginalView PosteriorMarginalsPrepared(BatchedModelView model,
                                                      Workspace &workspace) {
  const thmm_dense_model m = detail::Dense(model);
  thmm_marginal_result r{};
  detail::Throw(thmm_posterior_marginals(workspace.native_handle(), &m, &r));
  return {detail::Values(r.log_partitions, r.count), detail::Values(r.nodes, r.node_count),
          detail::Values(r.edges, r.edge_count), detail::Timings(r.timings)};
}

inline BatchedMarginalView
PosteriorMarginalsPrepared(BatchedCategoricalModelView model, Workspace &workspace,
                           CategoricalInputUpdate update) {
  const thmm_categorical_model m = detail::Categorical(model);
  thmm_marginal_result r{};
  detail::Throw(thmm_categorical_posterior_marginals(workspace.native_handle(), &m,
                                                     detail::Update(update), &r));
  return {detail::Values(r.log_partitions, r.count), detail::Values(r.nodes, r.node_count),
          detail::Values(r.edges, r.edge_count), detail::Timings(r.timings)};
}

inline BatchedMarginalView
PosteriorMarginalsPrepared(BatchedCategoricalModelView model, Workspace &workspace) {
  return PosteriorMarginalsPrepared(model, workspace, CategoricalInputUpdate::kAll);
}

} // namespace tree_hmm::gb300

#endif // TREE_HMM_GB300_H_
