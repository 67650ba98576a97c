#include "program.h"

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

  // Current version of every path slot (see engine.h) and whether a node has
  // an absorbed value stored in scratch.
  std::vector<std::uint32_t> version(edges);
  for (std::size_t e = 0; e < edges; ++e)
    version[e] = static_cast<std::uint32_t>(e);
  std::vector<char> stored(nodes, 0);

  for (const btrc::PrimitiveBatch &batch : plan.primitive_batches()) {
    DevStep step{};
    step.count = batch.count;
    switch (batch.primitive) {
    case btrc::Primitive::kRake:
      step.kind = kStepRake;
      step.offset = static_cast<std::uint32_t>(rakes.size());
      for (const btrc::Rake &op : plan.rakes().subspan(batch.offset, batch.count))
        rakes.push_back({version[op.edge], op.leaf | (stored[op.leaf] ? kFlag : 0u),
                         op.branch, op.parent});
      break;
    case btrc::Primitive::kBranchCombination:
      step.kind = kStepCombine;
      step.offset = static_cast<std::uint32_t>(combines.size());
      for (const btrc::BranchCombination &op :
           plan.branch_combinations().subspan(batch.offset, batch.count))
        combines.push_back({op.destination, op.source});
      break;
    case btrc::Primitive::kBranchAbsorption:
      step.kind = kStepAbsorb;
      step.offset = static_cast<std::uint32_t>(absorbs.size());
      for (const btrc::BranchAbsorption &op :
           plan.branch_absorptions().subspan(batch.offset, batch.count)) {
        absorbs.push_back({op.parent | (stored[op.parent] ? 0u : kFlag), op.branch});
        stored[op.parent] = 1;
      }
      break;
    case btrc::Primitive::kCompression: {
      step.kind = kStepCompress;
      step.offset = static_cast<std::uint32_t>(compress.size() / 2);
      const auto ops = plan.compressions().subspan(batch.offset, batch.count);
      for (const btrc::Compression &op : ops) {
        compress.push_back({version[op.left_edge],
                            op.middle | (stored[op.middle] ? kFlag : 0u),
                            version[op.right_edge], op.tape});
        compress.push_back({op.parent, op.child, 0u, 0u});
      }
      for (const btrc::Compression &op : ops)
        version[op.left_edge] = kFlag | op.tape;
      break;
    }
    }
    steps.push_back(step);
  }
  program.step_count =
      static_cast<std::uint32_t>(steps.size()) - program.step_begin;
  program.root = plan.root() | (stored[plan.root()] ? kFlag : 0u);
  program.obs_map = 0;
  if (categorical) {
    program.obs_map = static_cast<std::uint32_t>(obs_map.size());
    obs_map.resize(obs_map.size() + nodes, -1);
    for (std::size_t slot = 0; slot < observation_nodes.size(); ++slot)
      obs_map[program.obs_map + observation_nodes[slot]] =
          static_cast<std::int32_t>(slot);
  }
  programs.push_back(program);
  return static_cast<std::uint32_t>(programs.size() - 1);
}

} // namespace thmm
