#include "program.h"

#include <algorithm>
#include <numeric>
#include <stdexcept>

namespace thmm {

std::uint32_t ProgramSet::Add(const btrc::Plan &plan,
                              std::span<const std::uint32_t> observation_nodes,
                              bool categorical) {
  const std::size_t nodes = plan.num_nodes();
  const std::size_t edges = plan.num_edges();
  if (nodes >= kFlag || plan.num_compressions() >= kFlag)
    throw std::length_error("tree is too large for the accelerator program");

  DevProgram program{};
  program.step_begin = static_cast<std::uint32_t>(steps.size());
  program.num_nodes = static_cast<std::uint32_t>(nodes);
  program.num_edges = static_cast<std::uint32_t>(edges);
  program.num_rakes = static_cast<std::uint32_t>(plan.num_branches());
  program.num_compressions = static_cast<std::uint32_t>(plan.num_compressions());
  program.rake_base = static_cast<std::uint32_t>(rakes.size());
  program.compress_base = static_cast<std::uint32_t>(compress.size());

  std::vector<std::uint32_t> slot(nodes, kNone);
  if (categorical)
    for (std::size_t index = 0; index < observation_nodes.size(); ++index)
      slot[observation_nodes[index]] = static_cast<std::uint32_t>(index);

  // Current version of every path slot (see engine.h) and whether a node has
  // an absorbed value stored in scratch.
  std::vector<std::uint32_t> version(edges);
  std::iota(version.begin(), version.end(), 0u);
  std::vector<char> stored(nodes, 0);
  // Rakes are stored grouped by parent within each batch; branch ids are
  // renumbered to the stored order so that rake i still fills branch i.
  std::vector<std::uint32_t> branch_of(plan.num_branches(), kNone);
  // Fused forward steps, emitted after the plan's own steps.
  std::vector<DevStep> fused;
  struct PendingGather {
    std::uint32_t parent;
    std::uint32_t first;
    std::uint32_t count;
  };
  std::vector<PendingGather> pending; // gathers of the current round
  DevStep round_rakes{};               // rake step of the current round

  for (const btrc::PrimitiveBatch &batch : plan.primitive_batches()) {
    DevStep step{};
    step.count = batch.count;
    switch (batch.primitive) {
    case btrc::Primitive::kRake: {
      step.kind = kStepRake;
      step.offset = static_cast<std::uint32_t>(rakes.size());
      const auto ops = plan.rakes().subspan(batch.offset, batch.count);
      std::vector<std::uint32_t> order(ops.size());
      std::iota(order.begin(), order.end(), 0u);
      std::stable_sort(order.begin(), order.end(), [&](std::uint32_t a, std::uint32_t b) {
        return ops[a].parent < ops[b].parent;
      });
      pending.clear();
      round_rakes = step;
      for (const std::uint32_t index : order) {
        const btrc::Rake &op = ops[index];
        const std::uint32_t stored_index =
            static_cast<std::uint32_t>(rakes.size()) - program.rake_base;
        branch_of[op.branch] = stored_index;
        if (pending.empty() || pending.back().parent != op.parent)
          pending.push_back({op.parent, static_cast<std::uint32_t>(rakes.size()), 0});
        ++pending.back().count;
        rakes.push_back({version[op.edge], op.leaf | (stored[op.leaf] ? kFlag : 0u),
                         op.parent, slot[op.leaf]});
      }
      break;
    }
    case btrc::Primitive::kBranchCombination:
      step.kind = kStepCombine;
      step.offset = static_cast<std::uint32_t>(combines.size());
      for (const btrc::BranchCombination &op :
           plan.branch_combinations().subspan(batch.offset, batch.count))
        combines.push_back({branch_of[op.destination], branch_of[op.source]});
      break;
    case btrc::Primitive::kBranchAbsorption: {
      step.kind = kStepAbsorb;
      step.offset = static_cast<std::uint32_t>(absorbs.size());
      // Fused forward: one gather per absorbing parent, largest fan-in first
      // so the threads of a warp do similar amounts of work.
      std::vector<PendingGather> ordered = pending;
      std::stable_sort(ordered.begin(), ordered.end(),
                       [](const PendingGather &a, const PendingGather &b) {
                         return a.count > b.count;
                       });
      DevStep gather_step{};
      gather_step.kind = kStepGather;
      gather_step.offset = static_cast<std::uint32_t>(gathers.size());
      gather_step.count = static_cast<std::uint32_t>(ordered.size());
      gather_step.aux_offset = round_rakes.offset;
      gather_step.aux_count = round_rakes.count;
      for (const PendingGather &g : ordered)
        gathers.push_back({g.parent | (stored[g.parent] ? 0u : kFlag), slot[g.parent],
                           g.first, g.count});
      fused.push_back(gather_step);
      for (const btrc::BranchAbsorption &op :
           plan.branch_absorptions().subspan(batch.offset, batch.count)) {
        absorbs.push_back({op.parent | (stored[op.parent] ? 0u : kFlag),
                           branch_of[op.branch], slot[op.parent], 0u});
        stored[op.parent] = 1;
      }
      break;
    }
    case btrc::Primitive::kCompression: {
      step.kind = kStepCompress;
      step.offset = static_cast<std::uint32_t>(compress.size());
      const auto ops = plan.compressions().subspan(batch.offset, batch.count);
      for (const btrc::Compression &op : ops) {
        if (op.tape != compress.size() - program.compress_base)
          throw std::logic_error("plan tapes are not numbered in compression order");
        compress.push_back({version[op.left_edge],
                            op.middle | (stored[op.middle] ? kFlag : 0u),
                            version[op.right_edge], slot[op.middle]});
        compress_ends.push_back({op.parent, op.child});
      }
      for (const btrc::Compression &op : ops)
        version[op.left_edge] = kFlag | op.tape;
      fused.push_back(step);
      break;
    }
    }
    steps.push_back(step);
  }
  program.step_count =
      static_cast<std::uint32_t>(steps.size()) - program.step_begin;
  program.fused_begin = static_cast<std::uint32_t>(steps.size());
  program.fused_count = static_cast<std::uint32_t>(fused.size());
  steps.insert(steps.end(), fused.begin(), fused.end());
  program.root = plan.root() | (stored[plan.root()] ? kFlag : 0u);
  program.root_obs = slot[plan.root()];
  programs.push_back(program);
  return static_cast<std::uint32_t>(programs.size() - 1);
}

} // namespace thmm
