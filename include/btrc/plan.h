// Rake/compress topology plan for one rooted tree.
//
// This header restates the public interface of the third-party planner
// `bidirectional_tree_rake_compress` v0.1.0 (git commit
// 36cfd7592a653011ac36ffd8e3d918acc59a2e05, pinned in the reference's
// MODULE.bazel:12,15-19). That module is not vendored by the reference, so the
// interface below is reconstructed from its call sites:
//   - struct sizes 16/12/12/24 bytes: src/gpu_backend_impl.inc:39-42
//   - Index = uint32_t, sentinel max(): src/accelerator_path_storage.h:13-14
//   - operation fields read by the algebras: src/inference.cc:155-518 and
//     src/gpu_backend_impl.inc:411-1235
//   - plan accessors: src/gpu_backend_impl.inc:1803-1863,2245-2250;
//     tests/accelerator_test.h:241,391-396; tests/inference_test.cc:75-78
//   - MakePlan(std::vector<int64_t> parents): tests/inference_test.cc:159-160
//
// Semantics shared with the reference algebras:
//   * Rake: a current leaf `leaf`, attached to `parent` through the path stored
//     in slot `edge`, is eliminated into a fresh branch slot `branch`.
//   * BranchCombination: branch `source` is multiplied into `destination`
//     (sibling branches of `parent`, reduced pairwise in stages).
//   * BranchAbsorption: branch `branch` is multiplied into node `parent`.
//   * Compression: unary node `middle` between `parent` and `child` is spliced
//     out; the path `left_edge` (parent->middle) becomes
//     left_edge * diag(middle) * right_edge (parent->child). `tape` is unique.
// Operations within one PrimitiveBatch are mutually independent. Edge e is the
// edge above the e-th non-root node in increasing node order.
#ifndef BTRC_PLAN_H_
#define BTRC_PLAN_H_

#include <cstddef>
#include <cstdint>
#include <limits>
#include <span>
#include <vector>

namespace btrc {

using Index = std::uint32_t;
inline constexpr Index kNoIndex = std::numeric_limits<Index>::max();

struct Rake {
  Index edge;
  Index leaf;
  Index branch;
  Index parent;
};

struct BranchCombination {
  Index destination;
  Index source;
  // Node whose sibling branches are being reduced.
  Index parent;
};

struct BranchAbsorption {
  Index parent;
  Index branch;
  // Round in which the absorption happens.
  Index round;
};

struct Compression {
  Index left_edge;
  Index middle;
  Index right_edge;
  Index tape;
  Index parent;
  Index child;
};

static_assert(sizeof(Rake) == 16);
static_assert(sizeof(BranchCombination) == 12);
static_assert(sizeof(BranchAbsorption) == 12);
static_assert(sizeof(Compression) == 24);

enum class Primitive : std::uint32_t {
  kRake = 0,
  kBranchCombination = 1,
  kBranchAbsorption = 2,
  kCompression = 3,
};

// `offset` and `count` index the operation array of `primitive`.
struct PrimitiveBatch {
  Primitive primitive;
  Index offset;
  Index count;
};

// One pairwise stage of sibling-branch reduction; indexes
// branch_combinations().
struct BranchReductionStage {
  Index offset;
  Index count;
};

struct Round {
  // Range of primitive_batches() executed by this round.
  Index first_batch = 0;
  Index batch_count = 0;
  Index rakes = 0;
  Index compressions = 0;
  std::vector<BranchReductionStage> branch_reduction_stages;
};

class Plan {
public:
  Plan() = default;

  std::size_t num_nodes() const { return num_nodes_; }
  std::size_t num_edges() const { return edge_children_.size(); }
  std::size_t num_branches() const { return rakes_.size(); }
  std::size_t num_compressions() const { return compressions_.size(); }
  Index root() const { return root_; }

  std::span<const Index> edge_parents() const { return edge_parents_; }
  std::span<const Index> edge_children() const { return edge_children_; }
  std::span<const Rake> rakes() const { return rakes_; }
  std::span<const BranchCombination> branch_combinations() const {
    return combinations_;
  }
  std::span<const BranchAbsorption> branch_absorptions() const {
    return absorptions_;
  }
  std::span<const Compression> compressions() const { return compressions_; }
  std::span<const PrimitiveBatch> primitive_batches() const { return batches_; }
  std::span<const Round> rounds() const { return rounds_; }

private:
  friend Plan MakePlan(std::span<const std::int64_t> parents);

  std::size_t num_nodes_ = 0;
  Index root_ = 0;
  std::vector<Index> edge_parents_;
  std::vector<Index> edge_children_;
  std::vector<Rake> rakes_;
  std::vector<BranchCombination> combinations_;
  std::vector<BranchAbsorption> absorptions_;
  std::vector<Compression> compressions_;
  std::vector<PrimitiveBatch> batches_;
  std::vector<Round> rounds_;
};

// Builds the plan of the tree given by `parents` (-1 marks the single root).
// Throws std::invalid_argument for an empty array, several or no roots, an
// out-of-range parent or a cycle, and std::length_error when the tree has more
// nodes than Index can address.
Plan MakePlan(std::span<const std::int64_t> parents);

inline Plan MakePlan(const std::vector<std::int64_t> &parents) {
  return MakePlan(std::span<const std::int64_t>(parents));
}

} // namespace btrc

#endif // BTRC_PLAN_H_
