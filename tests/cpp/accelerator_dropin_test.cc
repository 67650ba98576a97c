// Drop-in check of the C++ accelerator API: code written against the
// reference's tree_hmm::cuda namespace (gpu_backend_api.inc), compiled against
// include/tree_hmm/gb300_as_cuda.h and linked with libthmm_gb300.so, run on a
// GB300. Covers the scenarios of the reference's accelerator suite
// (tests/accelerator_test.h) with this project's own data, checked against the
// oracle (oracle/oracle.h, linked as test infrastructure):
//   dense batch of 257 > one thread block, staged Inputs(), capacity-backed
//   tail batch, per-edge unary chain, 4096-node chain without underflow,
//   9 states, a 17-leaf star, categorical likelihood == dense likelihood,
//   categorical MAP / samples / marginals, residency rules and their
//   exceptions, dense MAP and samples bit-exact, invalid uniforms, marginals
//   with exact zeros, root-only plan and wide-star reverse.
// Built twice by __graft_entry__.build(): FP64 (default Scalar) and FP32
// (TREE_HMM_USE_FLOAT). Exit status 0 means every check passed.
#include "tree_hmm/gb300_as_cuda.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "oracle.h"

namespace {

using tree_hmm::Scalar;
using Vec = std::vector<Scalar>;
// Against the FP64 oracle: FP32 arithmetic with exact power-of-two scaling.
constexpr double kLogZ = 1e-6;
constexpr double kMarginal = 1e-5;

int g_checks = 0;

void Check(bool condition, const std::string &what) {
  ++g_checks;
  if (!condition)
    throw std::runtime_error("check failed: " + what);
}

bool NearRel(double a, double b, double tol) {
  return std::abs(a - b) <= tol * std::max({1.0, std::abs(a), std::abs(b)});
}

struct Oracle {
  oracle_plan plan{};
  explicit Oracle(const btrc::Plan &p) {
    plan.num_nodes = static_cast<uint32_t>(p.num_nodes());
    plan.num_edges = static_cast<uint32_t>(p.num_edges());
    plan.root = p.root();
    plan.num_rakes = static_cast<uint32_t>(p.rakes().size());
    plan.num_combinations = static_cast<uint32_t>(p.branch_combinations().size());
    plan.num_absorptions = static_cast<uint32_t>(p.branch_absorptions().size());
    plan.num_compressions = static_cast<uint32_t>(p.compressions().size());
    plan.num_batches = static_cast<uint32_t>(p.primitive_batches().size());
    plan.edge_parents = p.edge_parents().data();
    plan.edge_children = p.edge_children().data();
    plan.rakes = reinterpret_cast<const uint32_t *>(p.rakes().data());
    plan.combinations = reinterpret_cast<const uint32_t *>(p.branch_combinations().data());
    plan.absorptions = reinterpret_cast<const uint32_t *>(p.branch_absorptions().data());
    plan.compressions = reinterpret_cast<const uint32_t *>(p.compressions().data());
    plan.batches = reinterpret_cast<const uint32_t *>(p.primitive_batches().data());
  }
  // FP64 log-domain marginals.
  int Marginals(std::size_t K, const Vec &nodes, const Vec &edges, double &log_z,
                std::vector<double> &node_m, std::vector<double> &edge_m) const {
    std::vector<double> n(nodes.begin(), nodes.end()), e(edges.begin(), edges.end());
    node_m.assign(plan.num_nodes * K, 0.0);
    edge_m.assign(plan.num_edges * K * K, 0.0);
    double z = 0;
    return oracle_marginals_f64(&plan, K, n.data(), e.data(), &log_z, &z, node_m.data(),
                                edge_m.data());
  }
  double LogZ(std::size_t K, const Vec &nodes, const Vec &edges) const {
    std::vector<double> n(nodes.begin(), nodes.end()), e(edges.begin(), edges.end());
    double out = 0;
    if (oracle_log_partition_f64(&plan, K, n.data(), e.data(), &out) != ORACLE_OK)
      throw std::runtime_error("oracle log partition failed");
    return out;
  }
  // MAP and samples in the Scalar precision with the reproducible exp/log.
  int Map(std::size_t K, const Vec &nodes, const Vec &edges, Scalar &weight,
          std::vector<uint32_t> &states) const {
    states.assign(plan.num_nodes, 0);
#ifdef TREE_HMM_USE_FLOAT
    return oracle_map_f32(&plan, K, nodes.data(), edges.data(), ORACLE_MATH_PORTABLE,
                          &weight, states.data());
#else
    return oracle_map_f64(&plan, K, nodes.data(), edges.data(), ORACLE_MATH_PORTABLE,
                          &weight, states.data());
#endif
  }
  int Sample(std::size_t K, const Vec &nodes, const Vec &edges, const Vec &uniforms,
             std::vector<uint32_t> &states) const {
    states.assign(plan.num_nodes, 0);
#ifdef TREE_HMM_USE_FLOAT
    return oracle_sample_f32(&plan, K, nodes.data(), edges.data(), uniforms.data(),
                             ORACLE_MATH_PORTABLE, states.data());
#else
    return oracle_sample_f64(&plan, K, nodes.data(), edges.data(), uniforms.data(),
                             ORACLE_MATH_PORTABLE, states.data());
#endif
  }
};

Vec Slice(const Vec &v, std::size_t item, std::size_t width) {
  return Vec(v.begin() + item * width, v.begin() + (item + 1) * width);
}

template <class Exception, class Body> bool Throws(Body body) {
  try {
    body();
  } catch (const Exception &) {
    return true;
  }
  return false;
}

// Simple deterministic generator (no dependence on <random> distributions).
struct Lcg {
  uint64_t state;
  double Next() {
    state = state * 6364136223846793005ULL + 1442695040888963407ULL;
    return static_cast<double>(state >> 11) * 0x1.0p-53;
  }
};

void DenseLikelihood() {
  const btrc::Plan plan = btrc::MakePlan(std::vector<int64_t>{-1, 0, 0, 1, 1, 2, 2});
  const std::size_t K = 4, B = 257, N = plan.num_nodes(), E = plan.num_edges();
  Lcg rng{1};
  Vec nodes(B * N * K), edges(E * K * K);
  for (Scalar &v : nodes)
    v = static_cast<Scalar>(0.1 + rng.Next());
  for (Scalar &v : edges)
    v = static_cast<Scalar>(0.05 + rng.Next());
  tree_hmm::cuda::Workspace ws;
  ws.Reserve(plan, K, B);
  const Oracle oracle(plan);
  const tree_hmm::PartitionView raw =
      tree_hmm::cuda::PartitionFunctionPrepared({plan, K, B, nodes, edges}, ws);
  Check(raw.values.size() == B && raw.timings.kernel_ms >= 0, "raw Z shape");
  for (std::size_t b = 0; b < B; ++b)
    Check(NearRel(std::log(raw.values[b]), oracle.LogZ(K, Slice(nodes, b, N * K), edges),
                  2e-6),
          "raw partition");
  // Staged inputs skip the host copy.
  tree_hmm::MutableBatchedModelView staged = ws.Inputs(B);
  std::copy(nodes.begin(), nodes.end(), staged.node_potentials.begin());
  std::copy(edges.begin(), edges.end(), staged.edge_potentials.begin());
  const tree_hmm::PartitionView log_view = tree_hmm::cuda::LogPartitionFunctionPrepared(
      static_cast<tree_hmm::BatchedModelView>(staged), ws);
  for (std::size_t b = 0; b < B; ++b)
    Check(NearRel(log_view.values[b], oracle.LogZ(K, Slice(nodes, b, N * K), edges), kLogZ),
          "staged log partition");
  // Capacity-backed tail batch.
  tree_hmm::MutableBatchedModelView tail = ws.Inputs(3);
  Check(tail.node_potentials.size() == 3 * N * K, "tail staging shape");
  std::copy(nodes.begin(), nodes.begin() + 3 * N * K, tail.node_potentials.begin());
  std::copy(edges.begin(), edges.end(), tail.edge_potentials.begin());
  const auto tail_view = tree_hmm::cuda::LogPartitionFunctionPrepared(
      static_cast<tree_hmm::BatchedModelView>(tail), ws);
  Check(tail_view.values.size() == 3, "tail output shape");
}

void ChainsStatesAndStars() {
  // Per-edge unary chain: paths are composed, so broadcasting mistakes show.
  const btrc::Plan chain = btrc::MakePlan(std::vector<int64_t>{-1, 0, 1, 2, 3, 4, 5});
  const std::size_t K = 4, B = 5;
  Lcg rng{2};
  Vec nodes(B * chain.num_nodes() * K), edges(chain.num_edges() * K * K);
  for (Scalar &v : nodes)
    v = static_cast<Scalar>(0.1 + rng.Next());
  for (std::size_t e = 0; e < chain.num_edges(); ++e)
    for (std::size_t i = 0; i < K * K; ++i)
      edges[e * K * K + i] = static_cast<Scalar>(0.02 + 0.01 * (1 + e + 2 * (i / K) + 3 * (i % K)));
  tree_hmm::cuda::Workspace ws;
  ws.Reserve(chain, K, B);
  const auto chain_view =
      tree_hmm::cuda::LogPartitionFunctionPrepared({chain, K, B, nodes, edges}, ws);
  for (std::size_t b = 0; b < B; ++b)
    Check(NearRel(chain_view.values[b],
                  Oracle(chain).LogZ(K, Slice(nodes, b, chain.num_nodes() * K), edges), kLogZ),
          "unary chain");
  // Long chain: scaled likelihood does not underflow.
  std::vector<int64_t> parents(4096);
  for (std::size_t i = 0; i < parents.size(); ++i)
    parents[i] = static_cast<int64_t>(i) - 1;
  const btrc::Plan long_plan = btrc::MakePlan(parents);
  ws.Reserve(long_plan, 1, 1);
  const Vec long_nodes(4096, Scalar(0.5)), long_edges(4095, Scalar(1));
  const auto long_view =
      tree_hmm::cuda::LogPartitionFunctionPrepared({long_plan, 1, 1, long_nodes, long_edges}, ws);
  Check(std::abs(long_view.values[0] - 4096 * std::log(0.5)) <= 2e-3, "long chain");
  // Nine states (the generic-state path) and a 17-leaf star (multi-stage
  // sibling reduction).
  const btrc::Plan five = btrc::MakePlan(std::vector<int64_t>{-1, 0, 1, 2, 3});
  Vec n9(2 * 5 * 9), e9(4 * 81);
  for (Scalar &v : n9)
    v = static_cast<Scalar>(0.1 + rng.Next());
  for (Scalar &v : e9)
    v = static_cast<Scalar>(0.02 + rng.Next());
  ws.Reserve(five, 9, 2);
  const auto v9 = tree_hmm::cuda::LogPartitionFunctionPrepared({five, 9, 2, n9, e9}, ws);
  for (std::size_t b = 0; b < 2; ++b)
    Check(NearRel(v9.values[b], Oracle(five).LogZ(9, Slice(n9, b, 45), e9), kLogZ), "K=9");
  std::vector<int64_t> star(18, 0);
  star[0] = -1;
  const btrc::Plan star_plan = btrc::MakePlan(star);
  Check(star_plan.rounds().front().branch_reduction_stages.size() >= 4, "star stages");
  Vec ns(3 * 18 * 3), es(17 * 9);
  for (Scalar &v : ns)
    v = static_cast<Scalar>(0.14 + 0.5 * rng.Next());
  for (Scalar &v : es)
    v = static_cast<Scalar>(0.03 + rng.Next());
  ws.Reserve(star_plan, 3, 3);
  const auto vs = tree_hmm::cuda::LogPartitionFunctionPrepared({star_plan, 3, 3, ns, es}, ws);
  for (std::size_t b = 0; b < 3; ++b)
    Check(NearRel(vs.values[b], Oracle(star_plan).LogZ(3, Slice(ns, b, 54), es), kLogZ),
          "wide star");
}

struct CategoricalCase {
  btrc::Plan plan = btrc::MakePlan(std::vector<int64_t>{-1, 0, 1, 1, 0, 4, 5, 5});
  std::size_t K = 4, B = 7, C = 6;
  std::vector<btrc::Index> observed{2, 3, 6, 7};
  std::vector<uint8_t> observations;
  Vec root{0.1f, 0.2f, 0.3f, 0.4f};
  Vec emission{1, 1, 1, 1, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 1, 0, 1, 0};
  Vec edges;
  CategoricalCase() {
    observations.resize(B * observed.size());
    for (std::size_t b = 0; b < B; ++b)
      for (std::size_t o = 0; o < observed.size(); ++o)
        observations[b * observed.size() + o] = static_cast<uint8_t>((b + 2 * o) % C);
    edges.resize(plan.num_edges() * K * K);
    for (std::size_t i = 0; i < edges.size(); ++i)
      edges[i] = (i % (K * K)) / K == (i % K) ? Scalar(0.79) : Scalar(0.07);
  }
  // Dense node factors equivalent to item b (the product in Scalar precision).
  Vec Dense(std::size_t b) const {
    Vec nodes(plan.num_nodes() * K, Scalar(1));
    std::copy(root.begin(), root.end(), nodes.begin());
    for (std::size_t o = 0; o < observed.size(); ++o)
      for (std::size_t k = 0; k < K; ++k)
        nodes[observed[o] * K + k] *= emission[observations[b * observed.size() + o] * K + k];
    return nodes;
  }
  void Stage(tree_hmm::MutableBatchedCategoricalModelView staged) const {
    std::copy(observations.begin(), observations.end(), staged.observations.begin());
    std::copy(root.begin(), root.end(), staged.root_potential.begin());
    std::copy(emission.begin(), emission.end(), staged.emission_potentials.begin());
    std::copy(edges.begin(), edges.end(), staged.edge_potentials.begin());
  }
};

void Categorical() {
  const CategoricalCase c;
  const Oracle oracle(c.plan);
  const std::size_t N = c.plan.num_nodes();
  tree_hmm::cuda::Workspace ws;
  tree_hmm::cuda::Workspace dense_ws;
  ws.ReserveCategoricalMaximum(c.plan, c.K, c.B, c.C, c.observed);
  c.Stage(ws.CategoricalInputs(c.B));
  const auto staged = static_cast<tree_hmm::BatchedCategoricalModelView>(ws.CategoricalInputs(c.B));
  const auto log_view = tree_hmm::cuda::LogPartitionFunctionPrepared(staged, ws);
  const Vec log_values(log_view.values.begin(), log_view.values.end());
  const auto map = tree_hmm::cuda::MaximumAPosterioriPrepared(staged, ws);
  Vec dense;
  for (std::size_t b = 0; b < c.B; ++b) {
    const Vec item = c.Dense(b);
    dense.insert(dense.end(), item.begin(), item.end());
  }
  dense_ws.Reserve(c.plan, c.K, c.B);
  const auto dense_view =
      tree_hmm::cuda::LogPartitionFunctionPrepared({c.plan, c.K, c.B, dense, c.edges}, dense_ws);
  for (std::size_t b = 0; b < c.B; ++b) {
    const Vec item = c.Dense(b);
    Check(NearRel(log_values[b], oracle.LogZ(c.K, item, c.edges), kLogZ), "categorical log Z");
    Check(dense_view.values[b] == log_values[b], "categorical == dense bit for bit");
    Scalar weight = 0;
    std::vector<uint32_t> states;
    Check(oracle.Map(c.K, item, c.edges, weight, states) == ORACLE_OK, "oracle MAP");
    Check(map.log_weights[b] == weight, "categorical MAP weight");
    for (std::size_t n = 0; n < N; ++n)
      Check(map.states[b * N + n] == states[n], "categorical MAP states");
  }
  Check(ws.CategoricalInputs(3).observations.size() == 3 * c.observed.size(), "tail shape");

  ws.ReserveCategoricalSampling(c.plan, c.K, c.B, c.C, c.observed);
  c.Stage(ws.CategoricalInputs(c.B));
  std::span<Scalar> uniforms = ws.Uniforms(c.B);
  for (std::size_t i = 0; i < uniforms.size(); ++i)
    uniforms[i] = static_cast<Scalar>(0.13 + 0.12 * (i % 7));
  const auto samples = tree_hmm::cuda::PosteriorSamplePrepared(
      static_cast<tree_hmm::BatchedCategoricalModelView>(ws.CategoricalInputs(c.B)),
      uniforms, ws);
  for (std::size_t b = 0; b < c.B; ++b) {
    std::vector<uint32_t> expected;
    const Vec u(uniforms.begin() + b * N, uniforms.begin() + (b + 1) * N);
    Check(oracle.Sample(c.K, c.Dense(b), c.edges, u, expected) == ORACLE_OK, "oracle sample");
    for (std::size_t n = 0; n < N; ++n)
      Check(samples.states[b * N + n] == expected[n], "categorical sample");
  }

  ws.ReserveCategoricalMarginals(c.plan, c.K, c.B, c.C, c.observed);
  c.Stage(ws.CategoricalInputs(c.B));
  const auto marginals = tree_hmm::cuda::PosteriorMarginalsPrepared(
      static_cast<tree_hmm::BatchedCategoricalModelView>(ws.CategoricalInputs(c.B)), ws);
  Check(marginals.nodes.size() == c.B * N * c.K, "marginal shape");
  for (std::size_t b = 0; b < c.B; ++b) {
    double log_z = 0;
    std::vector<double> node_m, edge_m;
    Check(oracle.Marginals(c.K, c.Dense(b), c.edges, log_z, node_m, edge_m) == ORACLE_OK,
          "oracle marginals");
    Check(NearRel(marginals.log_partitions[b], log_z, kLogZ), "categorical marginal log Z");
    for (std::size_t i = 0; i < node_m.size(); ++i)
      Check(std::abs(marginals.nodes[b * node_m.size() + i] - node_m[i]) <= kMarginal,
            "categorical node marginal");
    for (std::size_t i = 0; i < edge_m.size(); ++i)
      Check(std::abs(marginals.edges[b * edge_m.size() + i] - edge_m[i]) <= kMarginal,
            "categorical edge marginal");
  }
}

void Residency() {
  const btrc::Plan plan = btrc::MakePlan(std::vector<int64_t>{-1, 0, 0, 1, 1, 2, 2});
  const std::size_t K = 4, B = 5, C = 4;
  const std::vector<btrc::Index> observed{3, 4, 5, 6};
  tree_hmm::cuda::Workspace ws;
  ws.ReserveCategorical(plan, K, B, C, observed);
  std::vector<uint8_t> observations(B * 4);
  for (std::size_t i = 0; i < observations.size(); ++i)
    observations[i] = static_cast<uint8_t>(i % C);
  Vec root{0.1f, 0.2f, 0.3f, 0.4f}, emission(C * K, Scalar(0));
  for (std::size_t k = 0; k < K; ++k)
    emission[k * K + k] = 1;
  Vec edges(plan.num_edges() * K * K);
  for (std::size_t i = 0; i < edges.size(); ++i)
    edges[i] = static_cast<Scalar>(0.02 + 0.003 * (1 + i % 29));
  const tree_hmm::BatchedCategoricalModelView model{plan, K, B, C, observed, observations,
                                                    root, emission, edges};
  using Update = tree_hmm::CategoricalInputUpdate;
  for (const Update update : {Update::kFactors, Update::kNone})
    Check(Throws<std::logic_error>([&] {
            tree_hmm::cuda::LogPartitionFunctionPrepared(model, ws, update);
          }),
          "reuse before staging is rejected");
  const auto first = tree_hmm::cuda::LogPartitionFunctionPrepared(model, ws, Update::kAll);
  const Vec baseline(first.values.begin(), first.values.end());
  observations.front() = static_cast<uint8_t>((observations.front() + 1) % C);
  const auto reused = tree_hmm::cuda::LogPartitionFunctionPrepared(model, ws, Update::kFactors);
  Check(std::equal(reused.values.begin(), reused.values.end(), baseline.begin()),
        "kFactors keeps resident observations");
  const auto updated = tree_hmm::cuda::LogPartitionFunctionPrepared(model, ws, Update::kAll);
  const Vec after(updated.values.begin(), updated.values.end());
  Check(!std::equal(after.begin(), after.end(), baseline.begin()), "kAll stages observations");
  for (Scalar &v : edges)
    v *= Scalar(0.9);
  const auto kept = tree_hmm::cuda::LogPartitionFunctionPrepared(model, ws, Update::kNone);
  Check(std::equal(kept.values.begin(), kept.values.end(), after.begin()),
        "kNone keeps resident factors");
  const auto changed = tree_hmm::cuda::LogPartitionFunctionPrepared(model, ws, Update::kFactors);
  Check(!std::equal(changed.values.begin(), changed.values.end(), after.begin()),
        "kFactors stages factors");
  const tree_hmm::BatchedCategoricalModelView tail{
      plan, K, 3, C, observed, std::span<const uint8_t>(observations).first(12), root,
      emission, edges};
  Check(Throws<std::logic_error>([&] {
          tree_hmm::cuda::LogPartitionFunctionPrepared(tail, ws, Update::kFactors);
        }),
        "observations of another batch size are not reused");
  ws.ReserveCategorical(plan, K, B, C, observed);
  Check(Throws<std::logic_error>([&] {
          tree_hmm::cuda::LogPartitionFunctionPrepared(model, ws, Update::kNone);
        }),
        "Reserve invalidates residency");
  tree_hmm::cuda::Workspace fresh;
  Check(Throws<std::logic_error>([&] { fresh.Inputs(1); }), "Inputs before Reserve");
  fresh.Reserve(plan, K, 2);
  Check(Throws<std::logic_error>([&] { fresh.CategoricalInputs(1); }),
        "CategoricalInputs on a dense workspace");
  Check(Throws<std::invalid_argument>([&] { fresh.Reserve(plan, 129, 2); }),
        "more than 128 states");
}

void DenseRecovery() {
  const btrc::Plan plan = btrc::MakePlan(std::vector<int64_t>{-1, 0, 1, 1, 0, 4, 5, 5});
  const Oracle oracle(plan);
  const std::size_t K = 4, B = 5, N = plan.num_nodes(), E = plan.num_edges();
  Vec nodes(B * N * K), edges(E * K * K);
  for (std::size_t i = 0; i < nodes.size(); ++i)
    nodes[i] = static_cast<Scalar>(0.11 + 0.013 * (1 + 3 * (i / (N * K)) + 5 * ((i / K) % N) + i % K));
  for (std::size_t i = 0; i < edges.size(); ++i)
    edges[i] = static_cast<Scalar>(0.03 + 0.007 * (1 + i / (K * K) + 2 * ((i / K) % K) + 3 * (i % K)));
  tree_hmm::cuda::Workspace ws;
  ws.ReserveMaximum(plan, K, B);
  tree_hmm::MutableBatchedModelView staged = ws.Inputs(B);
  std::copy(nodes.begin(), nodes.end(), staged.node_potentials.begin());
  std::copy(edges.begin(), edges.end(), staged.edge_potentials.begin());
  const auto map = tree_hmm::cuda::MaximumAPosterioriPrepared(
      static_cast<tree_hmm::BatchedModelView>(staged), ws);
  for (std::size_t b = 0; b < B; ++b) {
    Scalar weight = 0;
    std::vector<uint32_t> states;
    Check(oracle.Map(K, Slice(nodes, b, N * K), edges, weight, states) == ORACLE_OK, "oracle MAP");
    Check(map.log_weights[b] == weight, "MAP weight");
    for (std::size_t n = 0; n < N; ++n)
      Check(map.states[b * N + n] == states[n], "MAP states");
  }
  ws.ReserveSampling(plan, K, B);
  tree_hmm::MutableBatchedModelView sampling = ws.Inputs(B);
  std::copy(nodes.begin(), nodes.end(), sampling.node_potentials.begin());
  std::copy(edges.begin(), edges.end(), sampling.edge_potentials.begin());
  std::span<Scalar> uniforms = ws.Uniforms(B);
  for (std::size_t i = 0; i < uniforms.size(); ++i)
    uniforms[i] = static_cast<Scalar>(0.07 + 0.11 * (i % 8));
  const auto samples = tree_hmm::cuda::PosteriorSamplePrepared(
      static_cast<tree_hmm::BatchedModelView>(sampling), uniforms, ws);
  for (std::size_t b = 0; b < B; ++b) {
    std::vector<uint32_t> expected;
    const Vec u(uniforms.begin() + b * N, uniforms.begin() + (b + 1) * N);
    Check(oracle.Sample(K, Slice(nodes, b, N * K), edges, u, expected) == ORACLE_OK,
          "oracle sample");
    for (std::size_t n = 0; n < N; ++n)
      Check(samples.states[b * N + n] == expected[n], "posterior sample");
  }
  uniforms[0] = 1;
  Check(Throws<std::invalid_argument>([&] {
          tree_hmm::cuda::PosteriorSamplePrepared(
              static_cast<tree_hmm::BatchedModelView>(sampling), uniforms, ws);
        }),
        "uniform 1.0 is rejected");
}

void Marginals() {
  const btrc::Plan plan = btrc::MakePlan(std::vector<int64_t>{-1, 0, 1, 1, 0, 4, 5, 5});
  const Oracle oracle(plan);
  const std::size_t K = 4, B = 5, N = plan.num_nodes(), E = plan.num_edges();
  Vec nodes(B * N * K), edges(E * K * K);
  for (std::size_t i = 0; i < nodes.size(); ++i)
    nodes[i] = i % 13 == 0 ? Scalar(0) : static_cast<Scalar>(0.17 + 0.011 * (1 + i % 19));
  for (std::size_t i = 0; i < edges.size(); ++i)
    edges[i] = i % 17 == 0 ? Scalar(0) : static_cast<Scalar>(0.09 + 0.008 * (1 + i % 23));
  tree_hmm::cuda::Workspace ws;
  ws.ReserveMarginals(plan, K, B);
  const auto view = tree_hmm::cuda::PosteriorMarginalsPrepared({plan, K, B, nodes, edges}, ws);
  Check(view.log_partitions.size() == B && view.edges.size() == B * E * K * K, "shape");
  for (std::size_t b = 0; b < B; ++b) {
    double log_z = 0;
    std::vector<double> node_m, edge_m;
    Check(oracle.Marginals(K, Slice(nodes, b, N * K), edges, log_z, node_m, edge_m) == ORACLE_OK,
          "oracle marginals");
    Check(NearRel(view.log_partitions[b], log_z, kLogZ), "marginal log Z");
    for (std::size_t i = 0; i < node_m.size(); ++i)
      Check(std::abs(view.nodes[b * N * K + i] - node_m[i]) <= kMarginal, "node marginal");
    for (std::size_t i = 0; i < edge_m.size(); ++i)
      Check(std::abs(view.edges[b * E * K * K + i] - edge_m[i]) <= kMarginal, "edge marginal");
    for (std::size_t n = 0; n < N; ++n) {
      double total = 0;
      for (std::size_t k = 0; k < K; ++k)
        total += view.nodes[(b * N + n) * K + k];
      Check(std::abs(total - 1) <= 1e-5, "normalised node marginal");
    }
  }
  const btrc::Plan root_plan = btrc::MakePlan(std::vector<int64_t>{-1});
  const Vec root_nodes{0.2f, 0.3f, 0.5f, 0.1f, 0.0f, 0.9f, 0.4f, 0.4f, 0.2f};
  ws.ReserveMarginals(root_plan, 3, 3);
  const auto root_view =
      tree_hmm::cuda::PosteriorMarginalsPrepared({root_plan, 3, 3, root_nodes, Vec{}}, ws);
  for (std::size_t b = 0; b < 3; ++b) {
    double total = 0;
    for (std::size_t k = 0; k < 3; ++k)
      total += root_nodes[b * 3 + k];
    for (std::size_t k = 0; k < 3; ++k)
      Check(std::abs(root_view.nodes[b * 3 + k] - root_nodes[b * 3 + k] / total) <= 5e-6,
            "root-only marginal");
  }
  std::vector<int64_t> star(18, 0);
  star[0] = -1;
  const btrc::Plan star_plan = btrc::MakePlan(star);
  Vec ns(2 * 18 * 3), es(17 * 9);
  for (std::size_t i = 0; i < ns.size(); ++i)
    ns[i] = i % 29 == 0 ? Scalar(0) : static_cast<Scalar>(0.16 + 0.005 * (i % 17));
  for (std::size_t i = 0; i < es.size(); ++i)
    es[i] = static_cast<Scalar>(0.04 + 0.003 * (i % 31));
  ws.ReserveMarginals(star_plan, 3, 2);
  const auto star_view = tree_hmm::cuda::PosteriorMarginalsPrepared({star_plan, 3, 2, ns, es}, ws);
  for (std::size_t b = 0; b < 2; ++b) {
    double log_z = 0;
    std::vector<double> node_m, edge_m;
    Check(Oracle(star_plan).Marginals(3, Slice(ns, b, 54), es, log_z, node_m, edge_m) ==
              ORACLE_OK,
          "oracle star marginals");
    for (std::size_t i = 0; i < edge_m.size(); ++i)
      Check(std::abs(star_view.edges[b * edge_m.size() + i] - edge_m[i]) <= kMarginal,
            "wide-star edge marginal");
  }
}

} // namespace

int main() {
  try {
    if (!tree_hmm::cuda::Available()) {
      std::puts("no accelerator available");
      return 2;
    }
    std::printf("%s on %s\n", tree_hmm::kPrecisionName,
                tree_hmm::cuda::DeviceDescription(0).c_str());
    DenseLikelihood();
    ChainsStatesAndStars();
    Categorical();
    Residency();
    DenseRecovery();
    Marginals();
    std::printf("accelerator drop-in checks passed: %d\n", g_checks);
    return 0;
  } catch (const std::exception &error) {
    std::fprintf(stderr, "%s (after %d checks)\n", error.what(), g_checks);
    return 1;
  }
}
