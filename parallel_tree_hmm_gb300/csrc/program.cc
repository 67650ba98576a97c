#include "program.h"

namespace thmm {

std::uint32_t ProgramSet::Add(const btrc::Plan &plan,
                              std::span<const std::uint32_t> observation_nodes,
                              bool categorical) {
  return BuildProgram(plan, observation_nodes, categorical, *this);
}

} // namespace thmm
