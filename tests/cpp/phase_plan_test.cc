// The phase schedule (phase.h) of forests and of shared-edge batches, checked
// on the host without a GPU:
//   1. every record field indexes inside its array, and every input edge,
//      compressed path and node value is produced before it is consumed and
//      consumed exactly once;
//   2. a double-precision host run of the phase records, launch range by
//      launch range (whole batch, cut into instance stripes through
//      PhasePlan::OpRange, and with the last rounds taken from the per-tree
//      tail records), reproduces the oracle's log Z and marginals, both with
//      the adjoint of a compression recomputing its product (the K <= 32
//      kernels) and with it reading the stored compressed path and its own
//      scale, comp_scale minus its inputs' scales (the tensor-core phase
//      kernels, wide_phase.cuh).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <span>
#include <vector>

#include "btrc/plan.h"
#include "oracle.h"
#include "phase.h"
#include "program.h"

namespace {

using thmm::kFlag;
using thmm::kMask;
using thmm::kNone;

int failures = 0;
#define EXPECT(cond)                                                                     \
  do {                                                                                   \
    if (!(cond)) {                                                                       \
      if (++failures < 20)                                                               \
        std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);                    \
    }                                                                                    \
  } while (0)

std::vector<std::int64_t> Tree(std::mt19937_64 &rng, std::size_t n, int shape) {
  std::vector<std::int64_t> parents(n);
  parents[0] = -1;
  for (std::size_t i = 1; i < n; ++i) {
    if (shape == 0)
      parents[i] = static_cast<std::int64_t>(rng() % i);
    else if (shape == 1)
      parents[i] = (i % 2 == 1 || i < 2) ? static_cast<std::int64_t>(i - 1)
                                         : static_cast<std::int64_t>(i - 2);
    else
      parents[i] = rng() % 20 ? static_cast<std::int64_t>(i - 1)
                              : static_cast<std::int64_t>(rng() % i);
  }
  return parents;
}

oracle_plan OraclePlan(const btrc::Plan &p, std::vector<std::uint32_t> &storage) {
  // Flatten the plan arrays the way the oracle reads them.
  storage.clear();
  auto push = [&](std::uint32_t v) { storage.push_back(v); };
  const std::size_t e0 = storage.size();
  for (auto v : p.edge_parents()) push(v);
  const std::size_t e1 = storage.size();
  for (auto v : p.edge_children()) push(v);
  const std::size_t r0 = storage.size();
  for (const auto &r : p.rakes()) { push(r.edge); push(r.leaf); push(r.branch); push(r.parent); }
  const std::size_t c0 = storage.size();
  for (const auto &c : p.branch_combinations()) { push(c.destination); push(c.source); push(c.parent); }
  const std::size_t a0 = storage.size();
  for (const auto &a : p.branch_absorptions()) { push(a.parent); push(a.branch); push(a.round); }
  const std::size_t m0 = storage.size();
  for (const auto &c : p.compressions()) {
    push(c.left_edge); push(c.middle); push(c.right_edge); push(c.tape); push(c.parent); push(c.child);
  }
  const std::size_t b0 = storage.size();
  for (const auto &b : p.primitive_batches()) {
    push(static_cast<std::uint32_t>(b.primitive)); push(b.offset); push(b.count);
  }
  push(0);
  oracle_plan o{};
  o.num_nodes = static_cast<std::uint32_t>(p.num_nodes());
  o.num_edges = static_cast<std::uint32_t>(p.num_edges());
  o.root = p.root();
  o.num_rakes = static_cast<std::uint32_t>(p.rakes().size());
  o.num_combinations = static_cast<std::uint32_t>(p.branch_combinations().size());
  o.num_absorptions = static_cast<std::uint32_t>(p.branch_absorptions().size());
  o.num_compressions = static_cast<std::uint32_t>(p.compressions().size());
  o.num_batches = static_cast<std::uint32_t>(p.primitive_batches().size());
  o.edge_parents = storage.data() + e0;
  o.edge_children = storage.data() + e1;
  o.rakes = storage.data() + r0;
  o.combinations = storage.data() + c0;
  o.absorptions = storage.data() + a0;
  o.compressions = storage.data() + m0;
  o.batches = storage.data() + b0;
  return o;
}

// Host run of the phase records in double precision with a natural-log
// scale per stored object (the device carries a power-of-two exponent; the
// algebra is the same).
struct HostRun {
  const thmm::PhasePlan &plan;
  const std::vector<thmm::Uint4> &rakes, &gathers, &compress;
  const std::vector<thmm::Uint2> &roots;
  std::size_t K;
  const std::vector<double> &node_in, &edge_in;
  std::uint32_t modulus;
  std::vector<double> nodes, node_scale, comps, comp_scale, comp_mu;
  std::vector<double> values, node_out, edge_out;
  std::vector<int> edge_uses, comp_writes, comp_reads;
  bool stored_ratio = false; // adjoint ratio from the stored compressed path

  void Input(std::uint32_t node, double *out) const {
    for (std::size_t j = 0; j < K; ++j)
      out[j] = node_in[node * K + j];
  }
  const double *Path(std::uint32_t ref) const {
    if (ref & kFlag)
      return &comps[(ref & kMask) * K * K];
    const std::uint32_t row = modulus ? ref % modulus : ref;
    return &edge_in[static_cast<std::size_t>(row) * K * K];
  }
  double Scale(std::uint32_t ref) const { return (ref & kFlag) ? comp_scale[ref & kMask] : 0.0; }
  void Node(std::uint32_t ref, double *out, double &scale) const {
    if (ref & kFlag) {
      for (std::size_t j = 0; j < K; ++j)
        out[j] = nodes[(ref & kMask) * K + j];
      scale += node_scale[ref & kMask];
    } else {
      Input(ref, out);
    }
  }
  static double Normalise(double *v, std::size_t n) {
    double m = 0;
    for (std::size_t j = 0; j < n; ++j)
      m = std::max(m, v[j]);
    if (!(m > 0))
      return 0;
    for (std::size_t j = 0; j < n; ++j)
      v[j] /= m;
    return std::log(m);
  }

  void Gather(std::uint32_t i) {
    const thmm::Uint4 op = gathers[i];
    const std::uint32_t node = op.x & kMask;
    std::vector<double> v(K), leaf(K), message(K);
    double scale = 0;
    if (op.x & kFlag) {
      Input(node, v.data());
    } else {
      for (std::size_t j = 0; j < K; ++j)
        v[j] = nodes[node * K + j];
      scale = node_scale[node];
    }
    for (std::uint32_t k = 0; k < (op.w & thmm::kCountMask); ++k) {
      const thmm::Uint4 rake = rakes[op.z + k];
      EXPECT((rake.w & kMask) == node);
      Node(rake.y, leaf.data(), scale);
      scale += Scale(rake.x);
      if (rake.x & kFlag)
        ++comp_reads[rake.x & kMask];
      const double *path = Path(rake.x);
      for (std::size_t p = 0; p < K; ++p) {
        double dot = 0;
        for (std::size_t c = 0; c < K; ++c)
          dot += path[p * K + c] * leaf[c];
        message[p] = dot;
      }
      for (std::size_t p = 0; p < K; ++p)
        v[p] *= message[p];
      scale += Normalise(v.data(), K);
    }
    for (std::size_t j = 0; j < K; ++j)
      nodes[node * K + j] = v[j];
    node_scale[node] = scale;
  }

  void Compress(std::uint32_t i) {
    const thmm::Uint4 op = compress[i];
    std::vector<double> middle(K), out(K * K, 0.0);
    double scale = Scale(op.x) + Scale(op.z);
    Node(op.y, middle.data(), scale);
    for (const std::uint32_t ref : {op.x, op.z})
      if (ref & kFlag)
        ++comp_reads[ref & kMask];
    const double *left = Path(op.x), *right = Path(op.z);
    for (std::size_t p = 0; p < K; ++p)
      for (std::size_t m = 0; m < K; ++m)
        for (std::size_t c = 0; c < K; ++c)
          out[p * K + c] += left[p * K + m] * middle[m] * right[m * K + c];
    scale += Normalise(out.data(), K * K);
    for (std::size_t j = 0; j < K * K; ++j)
      comps[i * K * K + j] = out[j];
    comp_scale[i] = scale;
    ++comp_writes[i];
  }

  void Finish(std::uint32_t i) {
    const thmm::Uint2 rec = roots[i];
    const std::uint32_t node = rec.x & kMask;
    std::vector<double> root(K);
    double scale = 0;
    if (rec.x & kFlag) {
      for (std::size_t j = 0; j < K; ++j)
        root[j] = nodes[node * K + j];
      scale = node_scale[node];
    } else {
      Input(node, root.data());
    }
    double sum = 0;
    for (double r : root)
      sum += r;
    values[i] = sum > 0 ? scale + std::log(sum) : -INFINITY;
    for (std::size_t j = 0; j < K; ++j)
      node_out[node * K + j] = sum > 0 ? root[j] / sum : 0;
  }

  void StoreAdjoint(std::uint32_t ref, std::size_t r, const double *row) {
    double *dst = (ref & kFlag) ? &comp_mu[(ref & kMask) * K * K + r * K]
                                : &edge_out[static_cast<std::size_t>(ref) * K * K + r * K];
    for (std::size_t j = 0; j < K; ++j)
      dst[j] = row[j];
    if (!(ref & kFlag) && r == 0)
      ++edge_uses[ref];
  }

  void RakeReverse(std::uint32_t i) {
    const thmm::Uint4 op = rakes[i];
    std::vector<double> leaf(K), ratio(K), w(K), adjoint(K, 0.0);
    double unused = 0;
    Node(op.y, leaf.data(), unused);
    const double *path = Path(op.x);
    for (std::size_t p = 0; p < K; ++p) {
      double unnormalised = 0;
      for (std::size_t c = 0; c < K; ++c)
        unnormalised += path[p * K + c] * leaf[c];
      ratio[p] = unnormalised > 0 ? node_out[op.w * K + p] / unnormalised : 0;
      for (std::size_t c = 0; c < K; ++c)
        w[c] = ratio[p] * path[p * K + c] * leaf[c];
      StoreAdjoint(op.x, p, w.data());
    }
    for (std::size_t c = 0; c < K; ++c) {
      for (std::size_t p = 0; p < K; ++p)
        adjoint[c] += ratio[p] * path[p * K + c];
      node_out[(op.y & kMask) * K + c] = leaf[c] * adjoint[c];
    }
  }

  void CompressReverse(std::uint32_t i) {
    const thmm::Uint4 op = compress[i];
    std::vector<double> middle(K), ratio(K * K, 0.0), row(K), mid_adj(K, 0.0);
    double inputs = Scale(op.x) + Scale(op.z);
    Node(op.y, middle.data(), inputs);
    const double *left = Path(op.x), *right = Path(op.z);
    if (stored_ratio) {
      // product = stored path * exp(own scale); ratio = mu / product.
      const double own = comp_scale[i] - inputs;
      for (std::size_t j = 0; j < K * K; ++j) {
        const double stored = comps[i * K * K + j];
        ratio[j] = stored > 0 ? comp_mu[i * K * K + j] / stored * std::exp(-own) : 0;
      }
    } else {
      for (std::size_t p = 0; p < K; ++p)
        for (std::size_t m = 0; m < K; ++m)
          for (std::size_t c = 0; c < K; ++c)
            ratio[p * K + c] += left[p * K + m] * middle[m] * right[m * K + c];
      for (std::size_t j = 0; j < K * K; ++j)
        ratio[j] = ratio[j] > 0 ? comp_mu[i * K * K + j] / ratio[j] : 0;
    }
    for (std::size_t p = 0; p < K; ++p) {
      for (std::size_t m = 0; m < K; ++m) {
        double dot = 0;
        for (std::size_t c = 0; c < K; ++c)
          dot += right[m * K + c] * ratio[p * K + c];
        row[m] = left[p * K + m] * middle[m] * dot;
      }
      StoreAdjoint(op.x, p, row.data());
    }
    for (std::size_t m = 0; m < K; ++m) {
      double total = 0;
      for (std::size_t c = 0; c < K; ++c) {
        double acc = 0;
        for (std::size_t p = 0; p < K; ++p)
          acc += left[p * K + m] * ratio[p * K + c];
        row[c] = right[m * K + c] * middle[m] * acc;
        total += row[c];
      }
      mid_adj[m] = total;
      StoreAdjoint(op.z, m, row.data());
    }
    for (std::size_t m = 0; m < K; ++m)
      node_out[(op.y & kMask) * K + m] = mid_adj[m];
  }

  // Runs instances [a, b) the way the runtime launches them: the first
  // `grid_rounds` rounds as grid-wide phases, the rest from the tail records.
  void Run(std::uint32_t a, std::uint32_t b, std::uint32_t grid_rounds,
           const thmm::PhasePlan::Tail &tail) {
    grid_rounds = std::min(grid_rounds, plan.rounds);
    for (std::uint32_t r = 0; r < grid_rounds; ++r) {
      const auto g = plan.OpRange(thmm::kPhaseGather, r, a, b);
      for (std::uint64_t i = g.first; i < g.second; ++i)
        Gather(static_cast<std::uint32_t>(i));
      const auto c = plan.OpRange(thmm::kPhaseCompress, r, a, b);
      for (std::uint64_t i = c.first; i < c.second; ++i)
        Compress(static_cast<std::uint32_t>(i));
    }
    for (const thmm::Uint4 &item : tail.items) {
      if (item.x < a || item.x >= b)
        continue;
      for (std::uint32_t e = 0; e < item.z; ++e) {
        const thmm::Uint4 &round = tail.rounds[item.y + e];
        for (std::uint32_t i = 0; i < round.y; ++i)
          Gather(round.x + i);
        for (std::uint32_t i = 0; i < round.w; ++i)
          Compress(round.z + i);
      }
    }
    for (std::uint32_t i = a; i < b; ++i)
      Finish(i);
    for (const thmm::Uint4 &item : tail.items) {
      if (item.x < a || item.x >= b)
        continue;
      for (std::uint32_t e = item.z; e-- > 0;) {
        const thmm::Uint4 &round = tail.rounds[item.y + e];
        for (std::uint32_t i = 0; i < round.w; ++i)
          CompressReverse(round.z + i);
        const thmm::Uint2 &rakes_of = tail.rakes[item.y + e];
        for (std::uint32_t i = 0; i < rakes_of.y; ++i)
          RakeReverse(rakes_of.x + i);
      }
    }
    for (std::uint32_t r = grid_rounds; r-- > 0;) {
      const auto c = plan.OpRange(thmm::kPhaseCompress, r, a, b);
      for (std::uint64_t i = c.first; i < c.second; ++i)
        CompressReverse(static_cast<std::uint32_t>(i));
      const auto k = plan.OpRange(thmm::kPhaseRakeReverse, r, a, b);
      for (std::uint64_t i = k.first; i < k.second; ++i)
        RakeReverse(static_cast<std::uint32_t>(i));
    }
  }
};

void CheckForest(std::mt19937_64 &rng, bool shared_edges, std::size_t K, int stripes) {
  std::vector<btrc::Plan> plans;
  const std::size_t trees = shared_edges ? 1 : 40;
  const std::size_t batch = shared_edges ? 9 : trees;
  for (std::size_t t = 0; t < trees; ++t) {
    const std::size_t n = 1 + rng() % (t % 5 == 0 ? 3000 : 400);
    const auto parents = Tree(rng, shared_edges ? 700 : n, static_cast<int>(t % 3));
    plans.push_back(btrc::MakePlan(std::span<const std::int64_t>(parents)));
  }
  std::vector<thmm::ProgramRequest> requests;
  for (const btrc::Plan &p : plans)
    requests.push_back({&p, {}});
  const thmm::ProgramSet set = thmm::BuildPrograms(requests, false, 1);
  std::vector<thmm::PhaseInstance> instances;
  std::uint64_t nodes = 0, edges = 0;
  std::vector<const btrc::Plan *> of;
  for (std::size_t i = 0; i < batch; ++i) {
    const btrc::Plan &p = plans[shared_edges ? 0 : i];
    instances.push_back({static_cast<std::uint32_t>(shared_edges ? 0 : i), nodes, edges, 0});
    of.push_back(&p);
    nodes += p.num_nodes();
    edges += p.num_edges();
  }
  const thmm::PhasePlan plan = thmm::BuildPhasePlan(set, instances, nodes, edges, 2);
  EXPECT(plan.enabled);
  if (!plan.enabled)
    return;

  // 1. Record bounds.
  const std::uint64_t comps = plan.total_compressions;
  const auto path_ok = [&](std::uint32_t ref) {
    return (ref & kFlag) ? (ref & kMask) < comps : ref < edges;
  };
  for (const thmm::Uint4 &r : plan.rakes) {
    EXPECT(path_ok(r.x));
    EXPECT((r.y & kMask) < nodes);
    EXPECT(r.z == kNone);
    EXPECT(r.w < nodes);
  }
  for (const thmm::Uint4 &g : plan.gathers) {
    EXPECT((g.x & kMask) < nodes);
    EXPECT(g.z + (g.w & thmm::kCountMask) <= plan.rakes.size());
    EXPECT((g.w & thmm::kCountMask) >= 1);
  }
  for (const thmm::Uint4 &c : plan.compress) {
    EXPECT(path_ok(c.x) && path_ok(c.z));
    EXPECT((c.y & kMask) < nodes);
  }
  EXPECT(plan.roots.size() == batch);

  std::vector<double> node_in(nodes * K), edge_in((shared_edges ? plans[0].num_edges() : edges) * K * K);
  std::uniform_real_distribution<double> u(0.05, 1.0);
  for (double &v : node_in)
    v = u(rng);
  for (double &v : edge_in)
    v = rng() % 17 == 0 ? 0.0 : u(rng);

  // 2. Host run: whole batch, striped, with tails from rounds 1 and 2, and
  //    (pass 4) striped with the stored-path adjoint ratio.
  for (int pass = 0; pass < 5; ++pass) {
    const std::uint32_t grid_rounds =
        pass < 2 || pass == 4 ? plan.rounds : static_cast<std::uint32_t>(pass - 1);
    const thmm::PhasePlan::Tail tail =
        grid_rounds < plan.rounds ? plan.BuildTail(grid_rounds) : thmm::PhasePlan::Tail{};
    HostRun run{plan, plan.rakes, plan.gathers, plan.compress, plan.roots, K, node_in, edge_in,
                shared_edges ? static_cast<std::uint32_t>(plans[0].num_edges()) : 0u};
    run.nodes.assign(nodes * K, 0);
    run.node_scale.assign(nodes, 0);
    run.comps.assign(comps * K * K, 0);
    run.comp_scale.assign(comps, 0);
    run.comp_mu.assign(comps * K * K, 0);
    run.values.assign(batch, 0);
    run.node_out.assign(nodes * K, -1);
    run.edge_out.assign(edges * K * K, -1);
    run.edge_uses.assign(edges, 0);
    run.comp_writes.assign(comps, 0);
    run.comp_reads.assign(comps, 0);
    run.stored_ratio = pass == 4;
    const int parts = pass == 0 ? 1 : stripes;
    for (int s = 0; s < parts; ++s)
      run.Run(static_cast<std::uint32_t>(batch * s / parts),
              static_cast<std::uint32_t>(batch * (s + 1) / parts), grid_rounds, tail);
    for (std::size_t e = 0; e < edges; ++e)
      EXPECT(run.edge_uses[e] == 1);
    for (std::size_t c = 0; c < comps; ++c)
      EXPECT(run.comp_writes[c] == 1 && run.comp_reads[c] == 1);
    for (std::size_t i = 0; i < batch; ++i) {
      const btrc::Plan &p = *of[i];
      std::vector<std::uint32_t> storage;
      const oracle_plan op = OraclePlan(p, storage);
      const std::size_t n = p.num_nodes(), m = p.num_edges();
      std::vector<double> node_m(n * K), edge_m(m * K * K);
      double log_z = 0, z = 0;
      const std::size_t node0 = instances[i].node_base, edge0 = instances[i].edge_out_base;
      const double *edges_of = shared_edges ? edge_in.data() : edge_in.data() + edge0 * K * K;
      const int status = oracle_marginals_f64(&op, K, node_in.data() + node0 * K, edges_of,
                                              &log_z, &z, node_m.data(), edge_m.data());
      if (status != ORACLE_OK) {
        EXPECT(run.values[i] == -INFINITY);
        continue;
      }
      EXPECT(std::fabs(run.values[i] - log_z) <= 1e-9 * std::max(1.0, std::fabs(log_z)));
      double worst = 0;
      for (std::size_t j = 0; j < n * K; ++j)
        worst = std::max(worst, std::fabs(run.node_out[node0 * K + j] - node_m[j]));
      for (std::size_t j = 0; j < m * K * K; ++j)
        worst = std::max(worst, std::fabs(run.edge_out[edge0 * K * K + j] - edge_m[j]));
      EXPECT(worst <= 1e-9);
    }
  }
}

} // namespace

int main() {
  std::mt19937_64 rng(11);
  for (std::size_t K : {1, 3, 4, 7}) {
    CheckForest(rng, false, K, 3);
    CheckForest(rng, true, K, 4);
  }
  if (failures != 0) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("passed\n");
  return 0;
}
