// ORACLE - test infrastructure only.
//
// extern "C" wrapper over the reference's own CPU library
// (include/tree_hmm/inference.h, src/inference.cc), so tests can call the
// unmodified reference build from Python. Built by `make -C oracle ref` into
// oracle/_ref/ together with the reference sources it wraps; nothing here is
// part of the product.
#include "tree_hmm/inference.h"

#include <cstdint>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string g_error;

struct Model {
  btrc::Plan plan;
  std::size_t states;
  tree_hmm::Workspace workspace;
};

template <class Body> int Guard(Body body) {
  try {
    body();
    return 0;
  } catch (const std::invalid_argument &error) {
    g_error = error.what();
    return 1;
  } catch (const std::domain_error &error) {
    g_error = error.what();
    return 3;
  } catch (const std::length_error &error) {
    g_error = error.what();
    return 4;
  } catch (const std::logic_error &error) {
    g_error = error.what();
    return 2;
  } catch (const std::exception &error) {
    g_error = error.what();
    return 5;
  }
}

tree_hmm::ModelView View(Model *model, const tree_hmm::Scalar *nodes,
                         const tree_hmm::Scalar *edges) {
  const std::size_t k = model->states;
  return {model->plan, k,
          std::span<const tree_hmm::Scalar>(nodes, model->plan.num_nodes() * k),
          std::span<const tree_hmm::Scalar>(edges,
                                            model->plan.num_edges() * k * k)};
}

} // namespace

extern "C" {

int ref_scalar_bytes() { return static_cast<int>(sizeof(tree_hmm::Scalar)); }

const char *ref_last_error() { return g_error.c_str(); }

void *ref_model_create(const std::int64_t *parents, std::size_t count,
                       std::size_t states) {
  Model *result = nullptr;
  const int status = Guard([&] {
    result = new Model{btrc::MakePlan(std::vector<std::int64_t>(
                           parents, parents + count)),
                       states, tree_hmm::Workspace()};
    result->workspace.Reserve(result->plan, states);
  });
  if (status != 0) {
    delete result;
    return nullptr;
  }
  return result;
}

void ref_model_destroy(void *model) { delete static_cast<Model *>(model); }

int ref_partition(void *handle, const tree_hmm::Scalar *nodes,
                  const tree_hmm::Scalar *edges, tree_hmm::Scalar *out) {
  Model *model = static_cast<Model *>(handle);
  return Guard([&] {
    *out = tree_hmm::PartitionFunctionPrepared(View(model, nodes, edges),
                                               model->workspace);
  });
}

int ref_log_partition(void *handle, const tree_hmm::Scalar *nodes,
                      const tree_hmm::Scalar *edges, tree_hmm::Scalar *out) {
  Model *model = static_cast<Model *>(handle);
  return Guard([&] {
    *out = tree_hmm::LogPartitionFunctionPrepared(View(model, nodes, edges),
                                                  model->workspace);
  });
}

int ref_marginals(void *handle, const tree_hmm::Scalar *nodes,
                  const tree_hmm::Scalar *edges,
                  tree_hmm::Scalar *log_partition, tree_hmm::Scalar *partition,
                  tree_hmm::Scalar *node_marginals,
                  tree_hmm::Scalar *edge_marginals) {
  Model *model = static_cast<Model *>(handle);
  return Guard([&] {
    const tree_hmm::MarginalView view = tree_hmm::PosteriorMarginalsPrepared(
        View(model, nodes, edges), model->workspace);
    *log_partition = view.log_partition;
    *partition = view.partition;
    std::memcpy(node_marginals, view.nodes.data(), view.nodes.size_bytes());
    std::memcpy(edge_marginals, view.edges.data(), view.edges.size_bytes());
  });
}

int ref_map(void *handle, const tree_hmm::Scalar *nodes,
            const tree_hmm::Scalar *edges, tree_hmm::Scalar *log_weight,
            std::uint32_t *states) {
  Model *model = static_cast<Model *>(handle);
  return Guard([&] {
    const tree_hmm::MaximumAssignmentView view =
        tree_hmm::MaximumAPosterioriPrepared(View(model, nodes, edges),
                                             model->workspace);
    *log_weight = view.log_weight;
    for (std::size_t node = 0; node < view.states.size(); ++node)
      states[node] = static_cast<std::uint32_t>(view.states[node]);
  });
}

int ref_sample(void *handle, const tree_hmm::Scalar *nodes,
               const tree_hmm::Scalar *edges, const tree_hmm::Scalar *uniforms,
               std::uint32_t *states) {
  Model *model = static_cast<Model *>(handle);
  return Guard([&] {
    const std::span<const std::size_t> sample =
        tree_hmm::PosteriorSamplePrepared(
            View(model, nodes, edges),
            std::span<const tree_hmm::Scalar>(uniforms,
                                              model->plan.num_nodes()),
            model->workspace);
    for (std::size_t node = 0; node < sample.size(); ++node)
      states[node] = static_cast<std::uint32_t>(sample[node]);
  });
}

} // extern "C"
