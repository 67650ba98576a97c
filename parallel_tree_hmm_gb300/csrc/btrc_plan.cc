// Rake/compress planner: a restatement of the published contraction scheme
// consumed by the reference (bidirectional_tree_rake_compress v0.1.0, see
// include/btrc/plan.h for the interface and its provenance).
//
// Each round
//   1. rakes every current leaf into a fresh branch slot (one rake batch),
//   2. reduces the raked siblings of each parent pairwise, stage s pairing
//      branches 2^s apart (one combination batch per stage),
//   3. absorbs each parent's reduced branch into the parent (one batch),
//   4. compresses every other node of each maximal chain of unary nodes,
//      starting at the top of the chain, so that no two compressed nodes are
//      adjacent (one compression batch).
// Rounds repeat until only the root remains. Every non-root node is eliminated
// exactly once, either as a raked leaf or as a compressed middle node, and each
// round removes a constant fraction of the remaining nodes, so a tree of n
// nodes takes O(log n) rounds and O(n log n) host time.
#include "btrc/plan.h"

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace btrc {

Plan MakePlan(std::span<const std::int64_t> parents) {
  const std::size_t n = parents.size();
  if (n == 0)
    throw std::invalid_argument("a tree plan needs at least one node");
  if (n >= static_cast<std::size_t>(kNoIndex))
    throw std::length_error("tree node count exceeds btrc::Index");

  Plan plan;
  plan.num_nodes_ = n;

  // Validate the parent array and find the root.
  std::size_t roots = 0;
  Index root = 0;
  for (std::size_t node = 0; node < n; ++node) {
    const std::int64_t parent = parents[node];
    if (parent == -1) {
      ++roots;
      root = static_cast<Index>(node);
    } else if (parent < 0 || static_cast<std::uint64_t>(parent) >= n ||
               static_cast<std::size_t>(parent) == node) {
      throw std::invalid_argument("tree parent index " + std::to_string(parent) +
                                  " of node " + std::to_string(node) +
                                  " is out of range");
    }
  }
  if (roots != 1)
    throw std::invalid_argument("a tree plan needs exactly one root (parent -1)");
  plan.root_ = root;

  // Children in CSR form, used for the reachability check.
  std::vector<Index> child_offsets(n + 1, 0);
  for (std::size_t node = 0; node < n; ++node)
    if (node != root)
      ++child_offsets[static_cast<std::size_t>(parents[node]) + 1];
  for (std::size_t node = 0; node < n; ++node)
    child_offsets[node + 1] += child_offsets[node];
  std::vector<Index> children(n == 0 ? 0 : n - 1);
  {
    std::vector<Index> fill(child_offsets.begin(), child_offsets.end() - 1);
    for (std::size_t node = 0; node < n; ++node)
      if (node != root)
        children[fill[static_cast<std::size_t>(parents[node])]++] =
            static_cast<Index>(node);
  }
  {
    std::vector<Index> queue;
    queue.reserve(n);
    queue.push_back(root);
    for (std::size_t head = 0; head < queue.size(); ++head) {
      const Index node = queue[head];
      for (Index index = child_offsets[node]; index < child_offsets[node + 1];
           ++index)
        queue.push_back(children[index]);
    }
    if (queue.size() != n)
      throw std::invalid_argument("tree parent array contains a cycle");
  }

  // Edge e sits above the e-th non-root node.
  std::vector<Index> slot(n, kNoIndex);
  plan.edge_parents_.reserve(n - 1);
  plan.edge_children_.reserve(n - 1);
  for (std::size_t node = 0; node < n; ++node) {
    if (node == root)
      continue;
    slot[node] = static_cast<Index>(plan.edge_children_.size());
    plan.edge_parents_.push_back(static_cast<Index>(parents[node]));
    plan.edge_children_.push_back(static_cast<Index>(node));
  }

  // Current (contracted) tree.
  std::vector<Index> current_parent(n, kNoIndex);
  std::vector<Index> child_count(n, 0);
  std::vector<std::uint64_t> child_sum(n, 0);
  for (std::size_t node = 0; node < n; ++node) {
    if (node == root)
      continue;
    const Index parent = static_cast<Index>(parents[node]);
    current_parent[node] = parent;
    ++child_count[parent];
    child_sum[parent] += node;
  }
  std::vector<Index> alive(n);
  for (std::size_t node = 0; node < n; ++node)
    alive[node] = static_cast<Index>(node);
  std::vector<char> removed(n, 0);
  const auto is_unary = [&](Index node) {
    return node != root && child_count[node] == 1;
  };

  std::vector<std::pair<Index, Index>> groups;  // (parent, branch)
  std::vector<Index> compress;
  while (alive.size() > 1) {
    Round round;
    round.first_batch = static_cast<Index>(plan.batches_.size());
    const Index round_index = static_cast<Index>(plan.rounds_.size());

    // 1. Rake every current leaf, in increasing node order.
    const Index rake_offset = static_cast<Index>(plan.rakes_.size());
    groups.clear();
    for (const Index node : alive) {
      if (node == root || child_count[node] != 0)
        continue;
      const Index branch = static_cast<Index>(plan.rakes_.size());
      plan.rakes_.push_back({slot[node], node, branch, current_parent[node]});
      groups.emplace_back(current_parent[node], branch);
    }
    const Index rake_count =
        static_cast<Index>(plan.rakes_.size()) - rake_offset;
    if (rake_count != 0) {
      plan.batches_.push_back({Primitive::kRake, rake_offset, rake_count});
      round.rakes = rake_count;

      // 2. Pairwise sibling reduction. Branches were created in increasing
      // leaf order, so a stable sort by parent keeps each group ordered.
      std::stable_sort(groups.begin(), groups.end(),
                       [](const auto &left, const auto &right) {
                         return left.first < right.first;
                       });
      std::size_t largest = 0;
      for (std::size_t begin = 0; begin < groups.size();) {
        std::size_t end = begin;
        while (end < groups.size() && groups[end].first == groups[begin].first)
          ++end;
        largest = std::max(largest, end - begin);
        begin = end;
      }
      for (std::size_t stride = 1; stride < largest; stride *= 2) {
        const Index offset = static_cast<Index>(plan.combinations_.size());
        for (std::size_t begin = 0; begin < groups.size();) {
          std::size_t end = begin;
          while (end < groups.size() &&
                 groups[end].first == groups[begin].first)
            ++end;
          const std::size_t size = end - begin;
          for (std::size_t index = 0; index + stride < size;
               index += 2 * stride) {
            plan.combinations_.push_back({groups[begin + index].second,
                                          groups[begin + index + stride].second,
                                          groups[begin].first});
          }
          begin = end;
        }
        const Index count =
            static_cast<Index>(plan.combinations_.size()) - offset;
        plan.batches_.push_back({Primitive::kBranchCombination, offset, count});
        round.branch_reduction_stages.push_back({offset, count});
      }

      // 3. Absorb each reduced branch into its parent.
      const Index absorb_offset = static_cast<Index>(plan.absorptions_.size());
      for (std::size_t begin = 0; begin < groups.size();) {
        std::size_t end = begin;
        while (end < groups.size() && groups[end].first == groups[begin].first)
          ++end;
        plan.absorptions_.push_back(
            {groups[begin].first, groups[begin].second, round_index});
        begin = end;
      }
      plan.batches_.push_back(
          {Primitive::kBranchAbsorption, absorb_offset,
           static_cast<Index>(plan.absorptions_.size()) - absorb_offset});

      // Remove the raked leaves from the current tree.
      for (Index rake = rake_offset; rake < rake_offset + rake_count; ++rake) {
        const Index leaf = plan.rakes_[rake].leaf;
        const Index parent = current_parent[leaf];
        --child_count[parent];
        child_sum[parent] -= leaf;
        removed[leaf] = 1;
      }
    }

    // 4. Compress alternate nodes of each maximal unary chain, top first.
    compress.clear();
    for (const Index node : alive) {
      if (removed[node] || !is_unary(node))
        continue;
      const Index parent = current_parent[node];
      if (parent != root && is_unary(parent))
        continue;  // not the top of its chain
      bool take = true;
      for (Index walk = node; is_unary(walk);
           walk = static_cast<Index>(child_sum[walk])) {
        if (take)
          compress.push_back(walk);
        take = !take;
      }
    }
    if (!compress.empty()) {
      std::sort(compress.begin(), compress.end());
      const Index offset = static_cast<Index>(plan.compressions_.size());
      for (const Index middle : compress) {
        const Index child = static_cast<Index>(child_sum[middle]);
        const Index parent = current_parent[middle];
        const Index tape = static_cast<Index>(plan.compressions_.size());
        plan.compressions_.push_back(
            {slot[middle], middle, slot[child], tape, parent, child});
        // Splice: the left slot now carries parent -> child.
        slot[child] = slot[middle];
        current_parent[child] = parent;
        child_sum[parent] += static_cast<std::uint64_t>(child);
        child_sum[parent] -= static_cast<std::uint64_t>(middle);
        removed[middle] = 1;
      }
      const Index count = static_cast<Index>(plan.compressions_.size()) - offset;
      plan.batches_.push_back({Primitive::kCompression, offset, count});
      round.compressions = count;
    }

    std::size_t kept = 0;
    for (const Index node : alive)
      if (!removed[node])
        alive[kept++] = node;
    if (kept == alive.size())
      throw std::logic_error("tree contraction made no progress");
    alive.resize(kept);
    round.batch_count =
        static_cast<Index>(plan.batches_.size()) - round.first_batch;
    plan.rounds_.push_back(std::move(round));
  }
  return plan;
}

} // namespace btrc
