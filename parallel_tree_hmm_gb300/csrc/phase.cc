// Host construction of the phase schedule (phase.h) from compiled programs.
#include "phase.h"

#include <algorithm>
#include <exception>
#include <thread>

#include "program.h"

namespace thmm {
namespace {

// Where each round's operations of one program sit in the ProgramSet arrays.
struct ProgramLayout {
  ProgramRounds counts;
  std::vector<std::uint32_t> gather_at, rake_at, compress_at; // [round], set indices
  // Rounds that compress, with the program-local index (tape) of their first
  // compression; tapes are numbered in compression order, so these starts
  // increase.
  std::vector<std::uint32_t> tape_round, tape_start;
};

ProgramLayout Layout(const ProgramSet &set, const DevProgram &program) {
  ProgramLayout layout;
  ProgramRounds &c = layout.counts;
  for (std::uint32_t s = 0; s < program.fused_count; ++s) {
    const DevStep &step = set.steps[program.fused_begin + s];
    if (step.kind == kStepGather) {
      ++c.rounds;
      c.gathers.push_back(step.count);
      c.rakes.push_back(step.aux_count);
      c.compressions.push_back(0);
      layout.gather_at.push_back(step.offset);
      layout.rake_at.push_back(step.aux_offset);
      layout.compress_at.push_back(0);
    } else if (step.kind == kStepCompress) {
      if (c.rounds == 0)
        throw std::logic_error("compression step before the first gather step");
      c.compressions.back() = step.count;
      layout.compress_at.back() = step.offset;
      layout.tape_round.push_back(c.rounds - 1);
      layout.tape_start.push_back(step.offset - program.compress_base);
    }
  }
  return layout;
}

} // namespace

std::pair<std::uint64_t, std::uint64_t>
PhasePlan::OpRange(int kind, std::uint32_t round, std::uint32_t a, std::uint32_t b) const {
  const auto count_of = [&](std::uint32_t instance) -> std::uint64_t {
    const ProgramRounds &c = program_rounds[instance_program[instance]];
    if (round >= c.rounds)
      return 0;
    return kind == kPhaseGather  ? c.gathers[round]
           : kind == kPhaseCompress ? c.compressions[round]
                                    : c.rakes[round];
  };
  const std::vector<std::uint64_t> &base =
      kind == kPhaseGather ? gather_base : kind == kPhaseCompress ? compress_base : rake_base;
  std::uint64_t first = base[round];
  if (program_rounds.size() == 1) {
    const std::uint64_t each = count_of(0);
    return {first + a * each, first + b * each};
  }
  for (std::uint32_t i = 0; i < a; ++i)
    first += count_of(i);
  std::uint64_t last = first;
  for (std::uint32_t i = a; i < b; ++i)
    last += count_of(i);
  return {first, last};
}

PhasePlan::Tail PhasePlan::BuildTail(std::uint32_t tail_round) const {
  Tail tail;
  const std::size_t n = instance_program.size();
  std::vector<std::uint64_t> gather_at(rounds, 0), rake_at(rounds, 0),
      compress_at(rounds, 0);
  for (std::uint32_t r = 0; r < rounds; ++r) {
    gather_at[r] = gather_base[r];
    rake_at[r] = rake_base[r];
    compress_at[r] = compress_base[r];
  }
  for (std::size_t i = 0; i < n; ++i) {
    const ProgramRounds &c = program_rounds[instance_program[i]];
    if (c.rounds > tail_round) {
      tail.items.push_back({static_cast<std::uint32_t>(i),
                            static_cast<std::uint32_t>(tail.rounds.size()),
                            c.rounds - tail_round, 0u});
      for (std::uint32_t r = tail_round; r < c.rounds; ++r) {
        tail.rounds.push_back({static_cast<std::uint32_t>(gather_at[r]), c.gathers[r],
                               static_cast<std::uint32_t>(compress_at[r]),
                               c.compressions[r]});
        tail.rakes.push_back({static_cast<std::uint32_t>(rake_at[r]), c.rakes[r]});
      }
    }
    for (std::uint32_t r = 0; r < c.rounds; ++r) {
      gather_at[r] += c.gathers[r];
      rake_at[r] += c.rakes[r];
      compress_at[r] += c.compressions[r];
    }
  }
  return tail;
}

std::uint32_t PhasePlan::AutoTailRound(std::uint64_t ops) const {
  for (std::uint32_t r = 0; r < rounds; ++r)
    if ((gather_base[r + 1] - gather_base[r]) + (compress_base[r + 1] - compress_base[r]) <
        ops)
      return r;
  return rounds;
}

PhasePlan BuildPhasePlan(const ProgramSet &set, std::span<const PhaseInstance> instances,
                         std::uint64_t total_nodes, std::uint64_t total_edges_out,
                         unsigned threads) {
  PhasePlan plan;
  const std::size_t n = instances.size();
  // Record fields carry 31-bit node, edge and compression indices; every
  // tree's exponent sum must stay inside int32 (at most 2 exponents of
  // magnitude < 3400 per eliminated node).
  constexpr std::uint64_t kIndexLimit = kFlag;
  constexpr std::uint64_t kTreeLimit = (1ull << 31) / (2 * 3400);
  if (n == 0 || total_nodes >= kIndexLimit || total_edges_out >= kIndexLimit)
    return plan;
  for (const DevProgram &program : set.programs)
    if (program.num_nodes > kTreeLimit)
      return plan;

  std::vector<ProgramLayout> layouts;
  layouts.reserve(set.programs.size());
  for (const DevProgram &program : set.programs)
    layouts.push_back(Layout(set, program));
  std::uint32_t rounds = 0;
  for (const ProgramLayout &layout : layouts)
    rounds = std::max(rounds, layout.counts.rounds);

  // Per round and instance: first gather, rake and compression of the
  // instance relative to the round's base.
  const auto count = [&](const ProgramLayout &l, const std::vector<std::uint32_t> &v,
                         std::uint32_t r) -> std::uint64_t {
    return r < l.counts.rounds ? v[r] : 0;
  };
  std::vector<std::vector<std::uint64_t>> gather_at(rounds), rake_at(rounds),
      compress_at(rounds);
  plan.gather_base.assign(rounds + 1, 0);
  plan.rake_base.assign(rounds + 1, 0);
  plan.compress_base.assign(rounds + 1, 0);
  for (std::uint32_t r = 0; r < rounds; ++r) {
    gather_at[r].resize(n);
    rake_at[r].resize(n);
    compress_at[r].resize(n);
    std::uint64_t g = 0, k = 0, c = 0;
    for (std::size_t i = 0; i < n; ++i) {
      const ProgramLayout &l = layouts[instances[i].program];
      gather_at[r][i] = g;
      rake_at[r][i] = k;
      compress_at[r][i] = c;
      g += count(l, l.counts.gathers, r);
      k += count(l, l.counts.rakes, r);
      c += count(l, l.counts.compressions, r);
    }
    plan.gather_base[r + 1] = plan.gather_base[r] + g;
    plan.rake_base[r + 1] = plan.rake_base[r] + k;
    plan.compress_base[r + 1] = plan.compress_base[r] + c;
  }
  if (plan.compress_base[rounds] >= kIndexLimit || plan.rake_base[rounds] >= (1ull << 32) ||
      plan.gather_base[rounds] >= (1ull << 32))
    return plan;

  plan.rakes.resize(plan.rake_base[rounds]);
  plan.gathers.resize(plan.gather_base[rounds]);
  plan.compress.resize(plan.compress_base[rounds]);
  plan.roots.resize(n);

  const auto fill = [&](std::size_t first, std::size_t last) {
    for (std::size_t i = first; i < last; ++i) {
      const PhaseInstance &inst = instances[i];
      const DevProgram &program = set.programs[inst.program];
      const ProgramLayout &l = layouts[inst.program];
      const auto node = [&](std::uint32_t ref) {
        return static_cast<std::uint32_t>(inst.node_base + (ref & kMask)) | (ref & kFlag);
      };
      const auto obs = [&](std::uint32_t slot) {
        return slot == kNone ? kNone : static_cast<std::uint32_t>(inst.obs_base + slot);
      };
      // Global index of the instance's compression `tape`.
      const auto path = [&](std::uint32_t ref) -> std::uint32_t {
        if (!(ref & kFlag))
          return static_cast<std::uint32_t>(inst.edge_out_base + ref);
        const std::uint32_t tape = ref & kMask;
        const auto at = std::upper_bound(l.tape_start.begin(), l.tape_start.end(), tape) -
                        l.tape_start.begin() - 1;
        const std::uint32_t r = l.tape_round[at];
        return kFlag | static_cast<std::uint32_t>(plan.compress_base[r] + compress_at[r][i] +
                                                  (tape - l.tape_start[at]));
      };
      const std::uint32_t root = program.root & kMask;
      for (std::uint32_t r = 0; r < l.counts.rounds; ++r) {
        const std::uint64_t rake0 = plan.rake_base[r] + rake_at[r][i];
        for (std::uint32_t k = 0; k < l.counts.rakes[r]; ++k) {
          const Uint4 &src = set.rakes[l.rake_at[r] + k];
          plan.rakes[rake0 + k] = {path(src.x), node(src.y), obs(src.w),
                                   static_cast<std::uint32_t>(inst.node_base + src.z)};
        }
        const std::uint64_t gather0 = plan.gather_base[r] + gather_at[r][i];
        for (std::uint32_t g = 0; g < l.counts.gathers[r]; ++g) {
          const Uint4 &src = set.gathers[l.gather_at[r] + g];
          if (src.w > kCountMask)
            throw std::length_error("gather fan-in exceeds the phase record field");
          const std::uint32_t first_rake =
              static_cast<std::uint32_t>(rake0 + (src.z - l.rake_at[r]));
          plan.gathers[gather0 + g] = {node(src.x), obs(src.y), first_rake,
                                       src.w | ((src.x & kMask) == root ? kRootBit : 0u)};
        }
        const std::uint64_t comp0 = plan.compress_base[r] + compress_at[r][i];
        for (std::uint32_t c = 0; c < l.counts.compressions[r]; ++c) {
          const Uint4 &src = set.compress[l.compress_at[r] + c];
          plan.compress[comp0 + c] = {path(src.x), node(src.y), path(src.z), obs(src.w)};
        }
      }
      plan.roots[i] = {static_cast<std::uint32_t>(inst.node_base + root) |
                           (program.root & kFlag),
                       obs(program.root_obs)};
    }
  };
  unsigned workers = threads != 0 ? threads : std::thread::hardware_concurrency();
  workers = static_cast<unsigned>(std::clamp<std::uint64_t>(
      std::min<std::uint64_t>(workers, plan.rakes.size() / 65536), 1, n));
  if (workers <= 1) {
    fill(0, n);
  } else {
    std::vector<std::exception_ptr> errors(workers);
    std::vector<std::thread> pool;
    for (unsigned w = 0; w < workers; ++w)
      pool.emplace_back([&, w] {
        try {
          fill(n * w / workers, n * (w + 1) / workers);
        } catch (...) {
          errors[w] = std::current_exception();
        }
      });
    for (std::thread &thread : pool)
      thread.join();
    for (const std::exception_ptr &error : errors)
      if (error)
        std::rethrow_exception(error);
  }

  // Observation reads in the order the phases make them. Each observed node's
  // input factor is read by exactly one record: the first-absorption gather
  // of the node, the rake of a leaf with nothing absorbed, the compression of
  // a middle node with nothing absorbed, or the root record. Those records
  // get consecutive slots of a phase-ordered copy of the observations (the
  // runtime gathers it from the caller's array whenever observations are
  // uploaded), so the phases read their observation bytes sequentially
  // instead of one scattered byte per 32-byte sector; every other record's
  // observation field becomes kNone.
  const auto take = [&](std::uint32_t &field, bool reads) {
    if (reads && field != kNone) {
      plan.observation_order.push_back(field);
      field = static_cast<std::uint32_t>(plan.observation_order.size() - 1);
    } else {
      field = kNone;
    }
  };
  for (std::uint32_t r = 0; r < rounds; ++r) {
    for (std::uint64_t g = plan.gather_base[r]; g < plan.gather_base[r + 1]; ++g) {
      Uint4 &gather = plan.gathers[g];
      take(gather.y, (gather.x & kFlag) != 0);
      for (std::uint32_t k = 0; k < (gather.w & kCountMask); ++k) {
        Uint4 &rake = plan.rakes[gather.z + k];
        take(rake.z, (rake.y & kFlag) == 0);
      }
    }
    for (std::uint64_t c = plan.compress_base[r]; c < plan.compress_base[r + 1]; ++c)
      take(plan.compress[c].w, (plan.compress[c].y & kFlag) == 0);
  }
  for (Uint2 &root : plan.roots)
    take(root.y, (root.x & kFlag) == 0);
  if (plan.observation_order.size() >= kIndexLimit)
    return PhasePlan{};

  plan.rounds = rounds;
  plan.total_compressions = plan.compress_base[rounds];
  plan.program_rounds.reserve(layouts.size());
  for (ProgramLayout &layout : layouts)
    plan.program_rounds.push_back(std::move(layout.counts));
  plan.instance_program.resize(n);
  for (std::size_t i = 0; i < n; ++i)
    plan.instance_program[i] = instances[i].program;
  plan.enabled = true;
  return plan;
}

} // namespace thmm
