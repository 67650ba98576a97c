// ORACLE - test infrastructure only: the restated rake/compress planner
// (parallel_tree_hmm_gb300/csrc/btrc_plan.cc, compiled again here) behind a C
// ABI, so that the CPU baselines and checkers can plan trees without loading
// the product library. Plans are the same as the product's (same source).
#include <cstddef>
#include <cstdint>
#include <exception>
#include <new>
#include <span>

#include "btrc/plan.h"
#include "oracle.h"

extern "C" {

// Plan of one tree (parents[i] = parent of node i, -1 for the root); NULL if
// the parent array is not a tree.
void *oracle_plan_create(const std::int64_t *parents, std::size_t count) {
  try {
    return new btrc::Plan(btrc::MakePlan(std::span<const std::int64_t>(parents, count)));
  } catch (const std::exception &) {
    return nullptr;
  }
}

void oracle_plan_destroy(void *plan) { delete static_cast<btrc::Plan *>(plan); }

// Fills `out` with the plan's sizes and raw operation arrays (valid while
// the plan lives), the layout oracle.h documents.
void oracle_plan_view(const void *handle, oracle_plan *out) {
  const btrc::Plan &p = *static_cast<const btrc::Plan *>(handle);
  static_assert(sizeof(btrc::Rake) == 16 && sizeof(btrc::BranchCombination) == 12 &&
                sizeof(btrc::BranchAbsorption) == 12 && sizeof(btrc::Compression) == 24 &&
                sizeof(btrc::PrimitiveBatch) == 12);
  out->num_nodes = static_cast<std::uint32_t>(p.num_nodes());
  out->num_edges = static_cast<std::uint32_t>(p.num_edges());
  out->root = p.root();
  out->num_rakes = static_cast<std::uint32_t>(p.rakes().size());
  out->num_combinations = static_cast<std::uint32_t>(p.branch_combinations().size());
  out->num_absorptions = static_cast<std::uint32_t>(p.branch_absorptions().size());
  out->num_compressions = static_cast<std::uint32_t>(p.compressions().size());
  out->num_batches = static_cast<std::uint32_t>(p.primitive_batches().size());
  out->edge_parents = p.edge_parents().data();
  out->edge_children = p.edge_children().data();
  out->rakes = reinterpret_cast<const std::uint32_t *>(p.rakes().data());
  out->combinations = reinterpret_cast<const std::uint32_t *>(p.branch_combinations().data());
  out->absorptions = reinterpret_cast<const std::uint32_t *>(p.branch_absorptions().data());
  out->compressions = reinterpret_cast<const std::uint32_t *>(p.compressions().data());
  out->batches = reinterpret_cast<const std::uint32_t *>(p.primitive_batches().data());
}

} // extern "C"
