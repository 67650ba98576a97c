#include "program.h"

#include <algorithm>
#include <exception>
#include <thread>

namespace thmm {

std::uint32_t ProgramSet::Add(const btrc::Plan &plan,
                              std::span<const std::uint32_t> observation_nodes,
                              bool categorical) {
  return BuildProgram(plan, observation_nodes, categorical, *this);
}

namespace {

// Appends `part` to `all`, shifting every offset that points into one of the
// concatenated arrays (program and step offsets, the first rake of gathers).
void Append(ProgramSet &all, const ProgramSet &part) {
  const auto steps = static_cast<std::uint32_t>(all.steps.size());
  const auto rakes = static_cast<std::uint32_t>(all.rakes.size());
  const auto combines = static_cast<std::uint32_t>(all.combines.size());
  const auto absorbs = static_cast<std::uint32_t>(all.absorbs.size());
  const auto compress = static_cast<std::uint32_t>(all.compress.size());
  const auto gathers = static_cast<std::uint32_t>(all.gathers.size());
  for (DevProgram program : part.programs) {
    program.step_begin += steps;
    program.fused_begin += steps;
    program.rake_base += rakes;
    program.compress_base += compress;
    all.programs.push_back(program);
  }
  for (DevStep step : part.steps) {
    switch (step.kind) {
    case kStepRake:
      step.offset += rakes;
      break;
    case kStepCombine:
      step.offset += combines;
      break;
    case kStepAbsorb:
      step.offset += absorbs;
      break;
    case kStepCompress:
      step.offset += compress;
      break;
    case kStepGather:
      step.offset += gathers;
      step.aux_offset += rakes;
      break;
    }
    all.steps.push_back(step);
  }
  all.rakes.insert(all.rakes.end(), part.rakes.begin(), part.rakes.end());
  all.combines.insert(all.combines.end(), part.combines.begin(), part.combines.end());
  all.absorbs.insert(all.absorbs.end(), part.absorbs.begin(), part.absorbs.end());
  all.compress.insert(all.compress.end(), part.compress.begin(), part.compress.end());
  all.compress_ends.insert(all.compress_ends.end(), part.compress_ends.begin(),
                           part.compress_ends.end());
  for (Uint4 gather : part.gathers) {
    gather.z += rakes; // first rake of the gather
    all.gathers.push_back(gather);
  }
}

} // namespace

ProgramSet BuildPrograms(std::span<const ProgramRequest> requests, bool categorical,
                         unsigned threads) {
  std::uint64_t total_nodes = 0;
  for (const ProgramRequest &request : requests)
    total_nodes += request.plan->num_nodes();
  unsigned workers = threads != 0 ? threads : std::thread::hardware_concurrency();
  workers = std::max(1u, workers);
  // Small sets are not worth the threads.
  workers = static_cast<unsigned>(std::min<std::uint64_t>(
      {workers, requests.size(), std::max<std::uint64_t>(1, total_nodes / 65536)}));
  if (workers <= 1) {
    ProgramSet set;
    for (const ProgramRequest &request : requests)
      set.Add(*request.plan, request.observation_nodes, categorical);
    return set;
  }
  // Contiguous runs of about equal node count.
  std::vector<std::size_t> bounds{0};
  std::uint64_t seen = 0;
  for (std::size_t r = 0; r < requests.size(); ++r) {
    seen += requests[r].plan->num_nodes();
    if (bounds.size() < workers && seen * workers >= total_nodes * bounds.size())
      bounds.push_back(r + 1);
  }
  if (bounds.back() != requests.size())
    bounds.push_back(requests.size());
  const std::size_t parts = bounds.size() - 1;
  std::vector<ProgramSet> sets(parts);
  std::vector<std::exception_ptr> errors(parts);
  const auto work = [&](std::size_t c) {
    try {
      for (std::size_t r = bounds[c]; r < bounds[c + 1]; ++r)
        sets[c].Add(*requests[r].plan, requests[r].observation_nodes, categorical);
    } catch (...) {
      errors[c] = std::current_exception();
    }
  };
  std::vector<std::thread> pool;
  for (std::size_t c = 1; c < parts; ++c)
    pool.emplace_back(work, c);
  work(0);
  for (std::thread &thread : pool)
    thread.join();
  for (const std::exception_ptr &error : errors)
    if (error)
      std::rethrow_exception(error);
  ProgramSet all;
  for (const ProgramSet &part : sets)
    Append(all, part);
  return all;
}

} // namespace thmm
