// Parallel program compilation (BuildPrograms with several threads) must give
// exactly the arrays of a one-thread build, for dense and categorical forests
// of mixed shapes. Runs without a GPU.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "btrc/plan.h"
#include "program.h"

namespace {

template <class T> bool Same(const std::vector<T> &a, const std::vector<T> &b) {
  return a.size() == b.size() &&
         (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}

bool SameSet(const thmm::ProgramSet &a, const thmm::ProgramSet &b) {
  return Same(a.programs, b.programs) && Same(a.steps, b.steps) && Same(a.rakes, b.rakes) &&
         Same(a.combines, b.combines) && Same(a.absorbs, b.absorbs) &&
         Same(a.compress, b.compress) && Same(a.compress_ends, b.compress_ends) &&
         Same(a.gathers, b.gathers);
}

std::vector<std::int64_t> Tree(std::mt19937_64 &rng, std::size_t n, int shape) {
  std::vector<std::int64_t> parents(n);
  parents[0] = -1;
  for (std::size_t i = 1; i < n; ++i) {
    if (shape == 0)
      parents[i] = static_cast<std::int64_t>(rng() % i);             // random recursive
    else if (shape == 1)                                               // caterpillar
      parents[i] = (i % 2 == 1 || i < 2) ? static_cast<std::int64_t>(i - 1)
                                         : static_cast<std::int64_t>(i - 2);
    else
      parents[i] = rng() % 20 ? static_cast<std::int64_t>(i - 1)     // spine heavy
                              : static_cast<std::int64_t>(rng() % i);
  }
  return parents;
}

} // namespace

int main() {
  std::mt19937_64 rng(7);
  std::vector<btrc::Plan> plans;
  std::vector<std::vector<std::uint32_t>> observed;
  for (int t = 0; t < 300; ++t) {
    const std::size_t n = 1 + rng() % (t % 7 == 0 ? 20000 : 3000);
    const auto parents = Tree(rng, n, t % 3);
    plans.push_back(btrc::MakePlan(std::span<const std::int64_t>(parents)));
    std::vector<bool> has_child(n, false);
    for (std::size_t i = 1; i < n; ++i)
      has_child[static_cast<std::size_t>(parents[i])] = true;
    std::vector<std::uint32_t> leaves;
    for (std::size_t i = 0; i < n; ++i)
      if (!has_child[i] || rng() % 5 == 0)
        leaves.push_back(static_cast<std::uint32_t>(i));
    observed.push_back(leaves);
  }
  int failures = 0;
  for (int categorical = 0; categorical < 2; ++categorical) {
    std::vector<thmm::ProgramRequest> requests;
    for (std::size_t t = 0; t < plans.size(); ++t)
      requests.push_back({&plans[t], categorical ? std::span<const std::uint32_t>(observed[t])
                                                 : std::span<const std::uint32_t>()});
    const thmm::ProgramSet serial = thmm::BuildPrograms(requests, categorical != 0, 1);
    for (unsigned threads : {2u, 3u, 8u, 0u}) {
      const thmm::ProgramSet parallel = thmm::BuildPrograms(requests, categorical != 0, threads);
      if (!SameSet(serial, parallel)) {
        std::printf("FAIL categorical=%d threads=%u\n", categorical, threads);
        ++failures;
      }
    }
  }
  std::printf(failures ? "program build test FAILED\n" : "program build test passed\n");
  return failures ? 1 : 0;
}
