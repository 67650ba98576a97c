// Compilation of one btrc::Plan into the device program format (engine.h),
// written once over a storage policy so that the workspace path (std::vector)
// and the allocation-free path (fixed host arenas) emit identical programs.
//
// Storage must provide the output sequences programs, steps, rakes, combines,
// absorbs, compress, compress_ends and gathers (push_back / size / back) and
// `Temp<T>(count, value)`, a zero-based scratch array valid for one Build.
#ifndef THMM_PROGRAM_BUILDER_H_
#define THMM_PROGRAM_BUILDER_H_

#include <cstddef>
#include <cstdint>
#include <span>
#include <stdexcept>

#include "btrc/plan.h"
#include "engine.h"

namespace thmm {

struct Uint2 {
  std::uint32_t x, y;
};
struct Uint4 {
  std::uint32_t x, y, z, w;
};

// Stable bottom-up merge sort of data[0, n) using temp[0, n); no allocation.
template <class T, class Less>
void StableSort(T *data, std::size_t n, T *temp, Less less) {
  for (std::size_t width = 1; width < n; width *= 2) {
    for (std::size_t lo = 0; lo < n; lo += 2 * width) {
      const std::size_t mid = lo + width < n ? lo + width : n;
      const std::size_t hi = lo + 2 * width < n ? lo + 2 * width : n;
      std::size_t a = lo, b = mid, out = lo;
      while (a < mid && b < hi)
        temp[out++] = less(data[b], data[a]) ? data[b++] : data[a++];
      while (a < mid)
        temp[out++] = data[a++];
      while (b < hi)
        temp[out++] = data[b++];
    }
    for (std::size_t i = 0; i < n; ++i)
      data[i] = temp[i];
  }
}

struct PendingGather {
  std::uint32_t parent;
  std::uint32_t first;
  std::uint32_t count;
};

template <class Storage>
std::uint32_t BuildProgram(const btrc::Plan &plan,
                           std::span<const std::uint32_t> observation_nodes,
                           bool categorical, Storage &out) {
  const std::size_t nodes = plan.num_nodes();
  const std::size_t edges = plan.num_edges();
  if (nodes >= kFlag || plan.num_compressions() >= kFlag)
    throw std::length_error("tree is too large for the accelerator program");

  DevProgram program{};
  program.step_begin = static_cast<std::uint32_t>(out.steps.size());
  program.num_nodes = static_cast<std::uint32_t>(nodes);
  program.num_edges = static_cast<std::uint32_t>(edges);
  program.num_rakes = static_cast<std::uint32_t>(plan.num_branches());
  program.num_compressions = static_cast<std::uint32_t>(plan.num_compressions());
  program.rake_base = static_cast<std::uint32_t>(out.rakes.size());
  program.compress_base = static_cast<std::uint32_t>(out.compress.size());

  auto slot = out.template Temp<std::uint32_t>(nodes, kNone);
  if (categorical)
    for (std::size_t index = 0; index < observation_nodes.size(); ++index)
      slot[observation_nodes[index]] = static_cast<std::uint32_t>(index);

  // Current version of every path slot (see engine.h) and whether a node has
  // an absorbed value stored in scratch.
  auto version = out.template Temp<std::uint32_t>(edges, 0u);
  for (std::size_t e = 0; e < edges; ++e)
    version[e] = static_cast<std::uint32_t>(e);
  auto stored = out.template Temp<std::uint8_t>(nodes, 0);
  // Rakes are stored grouped by parent within each batch; branch ids are
  // renumbered to the stored order so that rake i still fills branch i.
  auto branch_of = out.template Temp<std::uint32_t>(plan.num_branches(), kNone);
  std::size_t widest = 1;
  for (const btrc::PrimitiveBatch &batch : plan.primitive_batches())
    widest = batch.count > widest ? batch.count : widest;
  auto order = out.template Temp<std::uint32_t>(widest, 0u);
  auto order_temp = out.template Temp<std::uint32_t>(widest, 0u);
  auto pending = out.template Temp<PendingGather>(widest, PendingGather{});
  auto pending_temp = out.template Temp<PendingGather>(widest, PendingGather{});
  std::size_t pending_count = 0;
  // Fused forward steps, emitted after the plan's own steps.
  auto fused = out.template Temp<DevStep>(plan.primitive_batches().size() + 1, DevStep{});
  std::size_t fused_count = 0;
  DevStep round_rakes{}; // rake step of the current round

  for (const btrc::PrimitiveBatch &batch : plan.primitive_batches()) {
    DevStep step{};
    step.count = batch.count;
    switch (batch.primitive) {
    case btrc::Primitive::kRake: {
      step.kind = kStepRake;
      step.offset = static_cast<std::uint32_t>(out.rakes.size());
      const auto ops = plan.rakes().subspan(batch.offset, batch.count);
      for (std::uint32_t i = 0; i < ops.size(); ++i)
        order[i] = i;
      StableSort(&order[0], ops.size(), &order_temp[0],
                 [&](std::uint32_t a, std::uint32_t b) {
                   return ops[a].parent < ops[b].parent;
                 });
      pending_count = 0;
      round_rakes = step;
      for (std::size_t k = 0; k < ops.size(); ++k) {
        const btrc::Rake &op = ops[order[k]];
        branch_of[op.branch] =
            static_cast<std::uint32_t>(out.rakes.size()) - program.rake_base;
        if (pending_count == 0 || pending[pending_count - 1].parent != op.parent)
          pending[pending_count++] = {op.parent,
                                      static_cast<std::uint32_t>(out.rakes.size()), 0};
        ++pending[pending_count - 1].count;
        out.rakes.push_back({version[op.edge], op.leaf | (stored[op.leaf] ? kFlag : 0u),
                             op.parent, slot[op.leaf]});
      }
      break;
    }
    case btrc::Primitive::kBranchCombination:
      step.kind = kStepCombine;
      step.offset = static_cast<std::uint32_t>(out.combines.size());
      for (const btrc::BranchCombination &op :
           plan.branch_combinations().subspan(batch.offset, batch.count))
        out.combines.push_back({branch_of[op.destination], branch_of[op.source]});
      break;
    case btrc::Primitive::kBranchAbsorption: {
      step.kind = kStepAbsorb;
      step.offset = static_cast<std::uint32_t>(out.absorbs.size());
      // Fused forward: one gather per absorbing parent, largest fan-in first
      // so the threads of a warp do similar amounts of work.
      StableSort(&pending[0], pending_count, &pending_temp[0],
                 [](const PendingGather &a, const PendingGather &b) {
                   return a.count > b.count;
                 });
      DevStep gather_step{};
      gather_step.kind = kStepGather;
      gather_step.offset = static_cast<std::uint32_t>(out.gathers.size());
      gather_step.count = static_cast<std::uint32_t>(pending_count);
      gather_step.aux_offset = round_rakes.offset;
      gather_step.aux_count = round_rakes.count;
      for (std::size_t k = 0; k < pending_count; ++k) {
        const PendingGather &g = pending[k];
        out.gathers.push_back({g.parent | (stored[g.parent] ? 0u : kFlag),
                               slot[g.parent], g.first, g.count});
      }
      // Each rake of the round is absorbed by exactly one gather: a second
      // absorption batch after the same rake batch emits none, so a program
      // never holds more gathers than rakes.
      pending_count = 0;
      fused[fused_count++] = gather_step;
      for (const btrc::BranchAbsorption &op :
           plan.branch_absorptions().subspan(batch.offset, batch.count)) {
        out.absorbs.push_back({op.parent | (stored[op.parent] ? 0u : kFlag),
                               branch_of[op.branch], slot[op.parent], 0u});
        stored[op.parent] = 1;
      }
      break;
    }
    case btrc::Primitive::kCompression: {
      step.kind = kStepCompress;
      step.offset = static_cast<std::uint32_t>(out.compress.size());
      const auto ops = plan.compressions().subspan(batch.offset, batch.count);
      for (const btrc::Compression &op : ops) {
        if (op.tape != out.compress.size() - program.compress_base)
          throw std::logic_error("plan tapes are not numbered in compression order");
        out.compress.push_back({version[op.left_edge],
                                op.middle | (stored[op.middle] ? kFlag : 0u),
                                version[op.right_edge], slot[op.middle]});
        out.compress_ends.push_back({op.parent, op.child});
      }
      for (const btrc::Compression &op : ops)
        version[op.left_edge] = kFlag | op.tape;
      fused[fused_count++] = step;
      break;
    }
    }
    out.steps.push_back(step);
  }
  program.step_count =
      static_cast<std::uint32_t>(out.steps.size()) - program.step_begin;
  program.fused_begin = static_cast<std::uint32_t>(out.steps.size());
  program.fused_count = static_cast<std::uint32_t>(fused_count);
  for (std::size_t k = 0; k < fused_count; ++k)
    out.steps.push_back(fused[k]);
  program.root = plan.root() | (stored[plan.root()] ? kFlag : 0u);
  program.root_obs = slot[plan.root()];
  out.programs.push_back(program);
  return static_cast<std::uint32_t>(out.programs.size() - 1);
}

} // namespace thmm

#endif // THMM_PROGRAM_BUILDER_H_
