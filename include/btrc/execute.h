// Drivers that walk a btrc::Plan and hand each primitive batch to a
// dispatcher, restating the traversal interface of the third-party module
// `bidirectional_tree_rake_compress` v0.1.0 (commit 36cfd759..., see plan.h).
//
// Dispatcher interface, from the reference's call sites:
//   Contract: Rake / CombineBranches / AbsorbBranches / Compress, once per
//             primitive batch in plan order (src/inference.cc:888,901,912,923,
//             934; dispatchers at src/inference.cc:155-214,259-324,576-639).
//   Reverse:  ReverseCompressions / ReverseAbsorbBranches /
//             ReverseCombineBranches / ReverseRakes in reverse batch order
//             (src/inference.cc:915,416-518).
//   Expand:   ExpandRakes / ExpandCompressions in reverse batch order; the
//             other primitives carry no state to restore
//             (src/inference.cc:925,937,363-412,651-667; same order as the
//             reference accelerator at src/gpu_backend_impl.inc:2330,2535).
#ifndef BTRC_EXECUTE_H_
#define BTRC_EXECUTE_H_

#include <cstddef>
#include <span>

#include "btrc/plan.h"

namespace btrc {

template <class Dispatcher>
void Contract(const Plan &plan, Dispatcher &dispatcher) {
  for (const PrimitiveBatch &batch : plan.primitive_batches()) {
    switch (batch.primitive) {
    case Primitive::kRake:
      dispatcher.Rake(plan.rakes().subspan(batch.offset, batch.count));
      break;
    case Primitive::kBranchCombination:
      dispatcher.CombineBranches(
          plan.branch_combinations().subspan(batch.offset, batch.count));
      break;
    case Primitive::kBranchAbsorption:
      dispatcher.AbsorbBranches(
          plan.branch_absorptions().subspan(batch.offset, batch.count));
      break;
    case Primitive::kCompression:
      dispatcher.Compress(plan.compressions().subspan(batch.offset, batch.count));
      break;
    }
  }
}

template <class Dispatcher>
void Reverse(const Plan &plan, Dispatcher &dispatcher) {
  const std::span<const PrimitiveBatch> batches = plan.primitive_batches();
  for (std::size_t index = batches.size(); index-- > 0;) {
    const PrimitiveBatch &batch = batches[index];
    switch (batch.primitive) {
    case Primitive::kRake:
      dispatcher.ReverseRakes(plan.rakes().subspan(batch.offset, batch.count));
      break;
    case Primitive::kBranchCombination:
      dispatcher.ReverseCombineBranches(
          plan.branch_combinations().subspan(batch.offset, batch.count));
      break;
    case Primitive::kBranchAbsorption:
      dispatcher.ReverseAbsorbBranches(
          plan.branch_absorptions().subspan(batch.offset, batch.count));
      break;
    case Primitive::kCompression:
      dispatcher.ReverseCompressions(
          plan.compressions().subspan(batch.offset, batch.count));
      break;
    }
  }
}

template <class Dispatcher>
void Expand(const Plan &plan, Dispatcher &dispatcher) {
  const std::span<const PrimitiveBatch> batches = plan.primitive_batches();
  for (std::size_t index = batches.size(); index-- > 0;) {
    const PrimitiveBatch &batch = batches[index];
    switch (batch.primitive) {
    case Primitive::kRake:
      dispatcher.ExpandRakes(plan.rakes().subspan(batch.offset, batch.count));
      break;
    case Primitive::kCompression:
      dispatcher.ExpandCompressions(
          plan.compressions().subspan(batch.offset, batch.count));
      break;
    case Primitive::kBranchCombination:
    case Primitive::kBranchAbsorption:
      break;
    }
  }
}

} // namespace btrc

#endif // BTRC_EXECUTE_H_
