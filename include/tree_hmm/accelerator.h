// Accelerator API types (views, update policy, timings). Field names, order
// and meaning are those of the reference's include/tree_hmm/accelerator.h:
// 13-147 so that code written against the reference compiles unchanged; the
// include guard is shared so the two headers never conflict.
#ifndef TREE_HMM_ACCELERATOR_H_
#define TREE_HMM_ACCELERATOR_H_

#include <cstddef>
#include <cstdint>
#include <span>

#include "btrc/plan.h"
#include "tree_hmm/scalar.h"

namespace tree_hmm {

// One topology and one set of edge factors for the whole batch; node factors
// [batch, node, state], edge factors [edge, parent state, child state].
struct BatchedModelView {
  const btrc::Plan &plan;
  std::size_t states;
  std::size_t batch;
  std::span<const Scalar> node_potentials;
  std::span<const Scalar> edge_potentials;
};

// Writable view of the same layout (workspace-owned pinned storage).
struct MutableBatchedModelView {
  const btrc::Plan &plan;
  std::size_t states;
  std::size_t batch;
  std::span<Scalar> node_potentials;
  std::span<Scalar> edge_potentials;

  operator BatchedModelView() const {
    return {plan, states, batch, node_potentials, edge_potentials};
  }
};

// Byte observations on selected nodes, combined with a shared emission table.
struct BatchedCategoricalModelView {
  const btrc::Plan &plan;
  std::size_t states;
  std::size_t batch;
  std::size_t categories;
  std::span<const btrc::Index> observation_nodes; // strictly increasing
  std::span<const std::uint8_t> observations;     // [batch, observation node]
  std::span<const Scalar> root_potential;         // [state]
  std::span<const Scalar> emission_potentials;    // [category, state]
  std::span<const Scalar> edge_potentials;        // [edge, parent, child]
};

struct MutableBatchedCategoricalModelView {
  const btrc::Plan &plan;
  std::size_t states;
  std::size_t batch;
  std::size_t categories;
  std::span<const btrc::Index> observation_nodes;
  std::span<std::uint8_t> observations;
  std::span<Scalar> root_potential;
  std::span<Scalar> emission_potentials;
  std::span<Scalar> edge_potentials;

  operator BatchedCategoricalModelView() const {
    return {plan,           states,        batch,
            categories,     observation_nodes, observations,
            root_potential, emission_potentials, edge_potentials};
  }
};

// Which categorical inputs a prepared call stages: kAll everything, kFactors
// the root/emission/edge factors (observations stay resident), kNone nothing.
enum class CategoricalInputUpdate {
  kAll,
  kFactors,
  kNone,
};

struct AcceleratorTimings {
  double upload_ms = 0.0;   // requested host-to-device transfers
  double kernel_ms = 0.0;   // device execution
  double download_ms = 0.0; // device-to-host result transfers
  double wall_ms = 0.0;     // whole prepared call
};

// Results are views of workspace-owned storage, valid until the workspace is
// reserved again, reused, moved or destroyed.
struct PartitionView {
  std::span<const Scalar> values;
  AcceleratorTimings timings;
};

struct BatchedMaximumAssignmentView {
  std::span<const Scalar> log_weights;   // [batch]
  std::span<const std::uint32_t> states; // [batch, node]
  AcceleratorTimings timings;
};

struct BatchedPosteriorSampleView {
  std::span<const std::uint32_t> states; // [batch, node]
  AcceleratorTimings timings;
};

struct BatchedMarginalView {
  std::span<const Scalar> log_partitions; // [batch]
  std::span<const Scalar> nodes;          // [batch, node, state]
  std::span<const Scalar> edges;          // [batch, edge, parent, child]
  AcceleratorTimings timings;
};

} // namespace tree_hmm

#endif // TREE_HMM_ACCELERATOR_H_
