// Host runtime of the accelerator: workspaces, staging, launch sequencing and
// the C ABI declared in include/thmm_gb300.h.
//
// Behaviour follows the reference host driver (src/gpu_backend_impl.inc:
// 1636-3130): one non-blocking stream and one device per workspace, pinned
// staging buffers exposed through Inputs()/CategoricalInputs()/Uniforms(),
// the kAll/kFactors/kNone residency rules for categorical inputs, six CUDA
// events for the upload/kernel/download split plus a wall clock, and the same
// exception classes (reported here as status codes). Where the reference
// launches one kernel per primitive batch and phase, a prepared call here
// launches one persistent kernel (engine.cuh) after a small memset, two for
// marginals (forward sweep, then adjoint sweep).
#include "thmm_gb300.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <exception>
#include <limits>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "btrc/plan.h"
#include "engine.h"
#include "phase.h"
#include "program.h"

struct thmm_plan; // a btrc::Plan in disguise

namespace thmm {
namespace {

thread_local std::string g_last_error;
using Clock = std::chrono::steady_clock;

void Check(cudaError_t status, const char *what) {
  if (status != cudaSuccess)
    throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(status));
}

std::size_t CheckedProduct(std::initializer_list<std::size_t> values,
                           const char *what) {
  std::size_t result = 1;
  for (const std::size_t value : values) {
    if (value != 0 && result > std::numeric_limits<std::size_t>::max() / value)
      throw std::length_error(std::string(what) + " overflows size_t");
    result *= value;
  }
  return result;
}

const btrc::Plan &AsPlan(const thmm_plan *plan) {
  if (plan == nullptr)
    throw std::invalid_argument("plan must not be null");
  return *reinterpret_cast<const btrc::Plan *>(plan);
}

// Raw device allocation owned by a workspace.
struct DeviceBuffer {
  void *ptr = nullptr;
  std::size_t bytes = 0;
  void Allocate(std::size_t size) {
    Free();
    Check(cudaMalloc(&ptr, std::max<std::size_t>(size, 16)), "cudaMalloc");
    bytes = size;
  }
  void Free() noexcept {
    if (ptr != nullptr)
      static_cast<void>(cudaFree(ptr));
    ptr = nullptr;
    bytes = 0;
  }
  template <class T> T *as() const { return static_cast<T *>(ptr); }
  template <class T> void Upload(const std::vector<T> &values, cudaStream_t stream) {
    Allocate(values.size() * sizeof(T));
    if (!values.empty())
      Check(cudaMemcpyAsync(ptr, values.data(), values.size() * sizeof(T),
                            cudaMemcpyHostToDevice, stream),
            "cudaMemcpyAsync program upload");
  }
  ~DeviceBuffer() { Free(); }
};

struct HostBuffer {
  void *ptr = nullptr;
  std::size_t bytes = 0;
  void Allocate(std::size_t size) {
    Free();
    Check(cudaMallocHost(&ptr, std::max<std::size_t>(size, 16)), "cudaMallocHost");
    bytes = size;
  }
  void Free() noexcept {
    if (ptr != nullptr)
      static_cast<void>(cudaFreeHost(ptr));
    ptr = nullptr;
    bytes = 0;
  }
  template <class T> T *as() const { return static_cast<T *>(ptr); }
  ~HostBuffer() { Free(); }
};

// Trees with at least this many nodes get a whole CTA; smaller ones a warp.
int TeamThreshold() {
  if (const char *value = std::getenv("THMM_TEAM_THRESHOLD"))
    return std::max(1, std::atoi(value));
  return 1024;
}

} // namespace

struct Workspace {
  // Reservation.
  bool reserved = false;
  bool forest = false;
  const btrc::Plan *plan = nullptr;
  std::size_t states = 0;
  std::size_t capacity = 0; // batch capacity, or tree count for a forest
  int device = 0;
  int scalar = THMM_SCALAR_F64;
  bool compute_f64 = false;
  bool bf16 = false; // BF16 tier of the tensor-core engine
  bool device_only = false; // no host staging (THMM_RESERVE_DEVICE_ONLY)
  bool maximum = false;
  bool sampling = false;
  bool marginals = false;
  bool categorical = false;
  std::size_t categories = 0;
  std::vector<std::uint32_t> observation_nodes;
  std::size_t resident_observation_batch = 0;
  bool resident_factors = false;
  std::size_t last_batch = 0;
  bool has_run = false;
  std::uint64_t launches = 0;

  // Sizes for the full capacity.
  std::size_t nodes_per_item = 0;     // batch API
  std::size_t edges_per_item = 0;     // batch API
  std::size_t observations_per_item = 0;
  std::uint64_t total_nodes = 0;      // all instances
  std::uint64_t total_edges_out = 0;  // all instances
  std::uint64_t edge_inputs = 0;      // matrices in the edge input
  std::uint64_t total_observations = 0;
  std::vector<std::uint64_t> tree_nodes; // forest: per tree

  // Device program.
  DeviceBuffer programs, steps, rakes, combines, absorbs, compress, instances;
  DeviceBuffer compress_ends, gathers, team_order, control;
  std::uint32_t big_count = 0;
  std::uint32_t small_count = 0;
  bool items_big = false;

  // Team assignment and grid. `team_order` lists the instances largest
  // first; the first `big_count` (instances with at least `team_threshold`
  // nodes) are contracted by whole CTAs, the rest by single warps.
  // `cta_cap[slot]` (0 = none) caps the resident CTAs per SM of one kernel
  // below its occupancy limit. Both are tunable (Autotune) and leave every
  // result bit-identical.
  std::vector<std::uint64_t> sorted_nodes;
  std::uint32_t team_threshold = 0;
  int cta_cap[4] = {0, 0, 0, 0};
  float tuned_ms = 0.0f;

  // Instantiated CUDA graphs of the device-only step, per operation and batch.
  struct Graph {
    int operation;
    std::size_t batch;
    cudaGraphExec_t exec;
  };
  std::vector<Graph> graphs;

  // Striped prepared calls. The instances of a call are cut into up to
  // kMaxStripes contiguous stripes of about equal node count; stripe c's
  // inputs are copied on `copy_in`, its kernels run on `stream` once they
  // have arrived, and its outputs are copied back on `copy_out` while later
  // stripes still compute, so the host<->device copies of one call overlap
  // each other and the kernels. `stripe_order` holds each stripe's instances
  // largest first at the stripe's own position.
  static constexpr std::uint32_t kMaxStripes = 8;
  static constexpr std::uint64_t kNodesPerStripe = 2u << 20;
  struct Stripe {
    std::uint32_t first, last; // instance range
    std::uint32_t big, small;  // CTA and warp team counts
  };
  std::vector<Stripe> stripe_plan;
  std::size_t stripe_batch = 0;
  std::uint32_t stripe_threshold = 0;
  std::uint32_t stripes_setting = 0; // 0: automatic
  std::uint32_t stripe_wanted = 0;
  DeviceBuffer stripe_order;
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t arrived[kMaxStripes] = {}, computed[kMaxStripes] = {};
  cudaEvent_t stripe_timing[8] = {};
  // Prefix offsets of each instance's slice (count + 1 entries).
  std::vector<std::uint64_t> off_nodes, off_edges, off_obs;
  bool shared_edge_input = false;

  // Level-synchronous phase schedule (phase.h) of the sum-product calls for
  // up to 4 states; its node values and compressed paths live in `scratch`.
  PhasePlan phase;
  DeviceBuffer phase_rakes, phase_gathers, phase_compress, phase_roots;
  DeviceBuffer node_exp, comp_exp;
  std::uint32_t schedule = THMM_SCHEDULE_TEAMS;
  // Rounds run as grid-wide phases; later rounds run in one warp per tree
  // (the tail, phase.h). `tail_instances` lists the tail trees in order.
  std::uint32_t phase_rounds = 0;
  DeviceBuffer tail_items, tail_rounds, tail_rakes;
  std::vector<std::uint32_t> tail_instances;
  // Phase-ordered copy of the observations (PhasePlan::observation_order),
  // rebuilt on the device whenever observations are uploaded.
  DeviceBuffer phase_observations, observation_order;
  std::uint64_t observation_reads = 0;
  // The batch API's phase layout: one tree's records for every item.
  bool phase_batch = false;
  // Operation ranges of each round for an instance range (cached).
  struct PhaseRanges {
    std::uint32_t a, b;
    std::vector<std::pair<std::uint64_t, std::uint64_t>> gather, rake, compress;
  };
  std::vector<PhaseRanges> phase_ranges;

  // Device data.
  DeviceBuffer node_in, edge_in, observations, root_potential, emission;
  DeviceBuffer uniforms, values, node_out, edge_out, states_out, scratch, bytes;

  // Pinned staging.
  HostBuffer h_node_in, h_edge_in, h_observations, h_root, h_emission;
  HostBuffer h_uniforms, h_values, h_node_out, h_edge_out, h_states, h_control;

  cudaStream_t stream = nullptr;
  cudaEvent_t events[6] = {};
  int sms = 1;
  // Resident CTAs per SM: linear forward, maximum, sample, linear adjoint.
  int occupancy[4] = {1, 1, 1, 1};

  ~Workspace() { Clear(); }

  void DropGraphs() noexcept {
    for (Graph &graph : graphs)
      static_cast<void>(cudaGraphExecDestroy(graph.exec));
    graphs.clear();
  }

  void Clear() noexcept {
    if (stream != nullptr) {
      static_cast<void>(cudaSetDevice(device));
      static_cast<void>(cudaStreamSynchronize(stream));
    }
    DropGraphs();
    sorted_nodes.clear();
    team_threshold = 0;
    std::fill(std::begin(cta_cap), std::end(cta_cap), 0);
    tuned_ms = 0.0f;
    phase = PhasePlan{};
    phase_ranges.clear();
    schedule = THMM_SCHEDULE_TEAMS;
    phase_rounds = 0;
    tail_instances.clear();
    observation_reads = 0;
    phase_batch = false;
    for (DeviceBuffer *buffer :
         {&programs, &steps, &rakes, &combines, &absorbs, &compress, &instances,
          &compress_ends, &gathers, &team_order, &stripe_order, &control, &node_in,
          &phase_rakes, &phase_gathers, &phase_compress, &phase_roots, &node_exp,
          &comp_exp, &tail_items, &tail_rounds, &tail_rakes, &phase_observations,
          &observation_order, &edge_in,
          &observations, &root_potential, &emission, &uniforms, &values,
          &node_out, &edge_out, &states_out, &scratch, &bytes})
      buffer->Free();
    for (HostBuffer *buffer :
         {&h_node_in, &h_edge_in, &h_observations, &h_root, &h_emission,
          &h_uniforms, &h_values, &h_node_out, &h_edge_out, &h_states,
          &h_control})
      buffer->Free();
    for (cudaEvent_t *group : {events, arrived, computed, stripe_timing}) {
      const std::size_t n = group == events ? 6 : group == stripe_timing ? 8 : kMaxStripes;
      for (std::size_t i = 0; i < n; ++i) {
        if (group[i] != nullptr)
          static_cast<void>(cudaEventDestroy(group[i]));
        group[i] = nullptr;
      }
    }
    for (cudaStream_t *s : {&stream, &copy_in, &copy_out}) {
      if (*s != nullptr)
        static_cast<void>(cudaStreamDestroy(*s));
      *s = nullptr;
    }
    stripe_plan.clear();
    stripe_batch = 0;
    stripe_threshold = 0;
    stripes_setting = 0;
    stripe_wanted = 0;
    off_nodes.clear();
    off_edges.clear();
    off_obs.clear();
    shared_edge_input = false;
    reserved = forest = false;
    plan = nullptr;
    states = capacity = 0;
    maximum = sampling = marginals = categorical = false;
    categories = 0;
    observation_nodes.clear();
    tree_nodes.clear();
    resident_observation_batch = 0;
    resident_factors = false;
    last_batch = 0;
    has_run = false;
  }

  std::size_t ScalarBytes() const { return static_cast<std::size_t>(scalar); }

  // ---------------------------------------------------------------- reserve
  // Common part of every Reserve* (src/gpu_backend_impl.inc:1803-1870).
  void Begin(std::size_t state_count, int device_index, std::uint32_t flags,
             std::uint32_t scalar_bytes) {
    if (scalar_bytes != THMM_SCALAR_F32 && scalar_bytes != THMM_SCALAR_F64)
      throw std::invalid_argument("scalar width must be 4 or 8 bytes");
    if (state_count == 0)
      throw std::invalid_argument(
          "accelerator state and batch counts must be nonzero");
    if (state_count > 128)
      throw std::invalid_argument(
          "state count exceeds the accelerator compression block limit");
    // 32 < K <= 128 runs on the tensor-core sum-product engine, which takes
    // FP32 factors and FP32 arithmetic and has no MAP or sampling kernel.
    if (state_count > 32 &&
        (scalar_bytes != THMM_SCALAR_F32 || (flags & THMM_COMPUTE_F64) != 0 ||
         (flags & (THMM_RESERVE_MAXIMUM | THMM_RESERVE_SAMPLING)) != 0))
      throw std::invalid_argument(
          "state counts above 32 support FP32 log partitions and marginals only");
    if ((flags & THMM_COMPUTE_BF16) != 0 && state_count <= 32)
      throw std::invalid_argument(
          "BF16 tensor products are a tier of the tensor-core engine (more than 32 states)");
    Clear();
    device = device_index;
    Check(cudaSetDevice(device), "cudaSetDevice");
    Check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device),
          "cudaDeviceGetAttribute");
    Check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking),
          "cudaStreamCreateWithFlags");
    for (cudaEvent_t &event : events)
      Check(cudaEventCreate(&event), "cudaEventCreate");
    Check(cudaStreamCreateWithFlags(&copy_in, cudaStreamNonBlocking),
          "cudaStreamCreateWithFlags");
    Check(cudaStreamCreateWithFlags(&copy_out, cudaStreamNonBlocking),
          "cudaStreamCreateWithFlags");
    for (std::uint32_t c = 0; c < kMaxStripes; ++c) {
      Check(cudaEventCreateWithFlags(&arrived[c], cudaEventDisableTiming),
            "cudaEventCreate");
      Check(cudaEventCreateWithFlags(&computed[c], cudaEventDisableTiming),
            "cudaEventCreate");
    }
    for (cudaEvent_t &event : stripe_timing)
      Check(cudaEventCreate(&event), "cudaEventCreate");
    states = state_count;
    scalar = static_cast<int>(scalar_bytes);
    compute_f64 = (flags & THMM_COMPUTE_F64) != 0;
    bf16 = (flags & THMM_COMPUTE_BF16) != 0;
    device_only = (flags & THMM_RESERVE_DEVICE_ONLY) != 0;
    maximum = (flags & THMM_RESERVE_MAXIMUM) != 0;
    sampling = (flags & THMM_RESERVE_SAMPLING) != 0;
    marginals = (flags & THMM_RESERVE_MARGINALS) != 0;
  }

  // Builds programs, instances, work queues and buffers for `plans[i]`
  // applied to instance i.
  void Build(const std::vector<const btrc::Plan *> &instance_plans,
             const std::vector<std::vector<std::uint32_t>> &instance_observations,
             bool shared_edges) {
    std::unordered_map<const btrc::Plan *, std::uint32_t> program_of;
    const std::size_t count = instance_plans.size();
    // Which instances need a program of their own (a distinct plan, or a
    // categorical forest tree with its own observation set), then all
    // programs compiled on the host's threads.
    std::vector<std::uint32_t> program_index(count);
    std::vector<ProgramRequest> requests;
    for (std::size_t i = 0; i < count; ++i) {
      const btrc::Plan *p = instance_plans[i];
      const auto found = program_of.find(p);
      if (found != program_of.end() && (!categorical || shared_edges)) {
        program_index[i] = found->second;
        continue;
      }
      program_index[i] = static_cast<std::uint32_t>(requests.size());
      program_of[p] = program_index[i];
      requests.push_back({p, instance_observations.empty()
                                 ? std::span<const std::uint32_t>()
                                 : std::span<const std::uint32_t>(instance_observations[i])});
    }
    const ProgramSet set = BuildPrograms(requests, categorical, 0);
    std::vector<DevInstance> table(count);
    const std::uint64_t K = states;
    const std::uint64_t KK = K * K;
    std::uint64_t node_base = 0, edge_base = 0, obs_base = 0;
    std::uint64_t scratch_base = 0, byte_base = 0;
    const std::size_t compute_bytes =
        std::max<std::size_t>(ScalarBytes(), compute_f64 ? 8 : 4);
    for (std::size_t i = 0; i < count; ++i) {
      const btrc::Plan &p = *instance_plans[i];
      DevInstance &instance = table[i];
      instance.program = program_index[i];
      instance.node_base = node_base;
      instance.edge_in_base = shared_edges ? 0 : edge_base;
      instance.edge_out_base = edge_base;
      instance.obs_base = obs_base;
      // Scratch: the largest layout among the reserved operations.
      ScratchSize size = InstanceScratch(p.num_nodes(), p.num_branches(),
                                         p.num_compressions(), K, kModeLinear,
                                         marginals);
      if (maximum) {
        const ScratchSize m = InstanceScratch(p.num_nodes(), p.num_branches(),
                                              p.num_compressions(), K,
                                              kModeMaximum, false);
        size.elements = std::max(size.elements, m.elements);
        size.bytes = std::max(size.bytes, m.bytes);
      }
      instance.scratch_base = scratch_base;
      instance.byte_base = byte_base;
      scratch_base += size.elements;
      byte_base += size.bytes;
      node_base += p.num_nodes();
      edge_base += p.num_edges();
      obs_base += instance_observations.empty() ? 0
                  : instance_observations[i].size();
      tree_nodes.push_back(p.num_nodes());
    }
    total_nodes = node_base;
    total_edges_out = edge_base;
    edge_inputs = shared_edges ? instance_plans.front()->num_edges() : edge_base;
    total_observations = obs_base;
    shared_edge_input = shared_edges;
    off_nodes.resize(count + 1);
    off_edges.resize(count + 1);
    off_obs.resize(count + 1);
    for (std::size_t i = 0; i < count; ++i) {
      off_nodes[i] = table[i].node_base;
      off_edges[i] = table[i].edge_out_base;
      off_obs[i] = table[i].obs_base;
    }
    off_nodes[count] = total_nodes;
    off_edges[count] = total_edges_out;
    off_obs[count] = total_observations;

    // Work queue: instances largest first; a prefix goes to whole-CTA teams,
    // the rest to single-warp teams (ApplyThreshold).
    std::vector<std::uint32_t> order(count);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](std::uint32_t a, std::uint32_t b) {
      return tree_nodes[a] > tree_nodes[b];
    });
    sorted_nodes.resize(count);
    for (std::size_t i = 0; i < count; ++i)
      sorted_nodes[i] = tree_nodes[order[i]];
    ApplyThreshold(static_cast<std::uint32_t>(TeamThreshold()));

    programs.Upload(set.programs, stream);
    steps.Upload(set.steps, stream);
    rakes.Upload(set.rakes, stream);
    combines.Upload(set.combines, stream);
    absorbs.Upload(set.absorbs, stream);
    compress.Upload(set.compress, stream);
    compress_ends.Upload(set.compress_ends, stream);
    gathers.Upload(set.gathers, stream);
    instances.Upload(table, stream);
    team_order.Upload(order, stream);
    // Phase schedule of the sum-product calls. A forest gets records for
    // every tree; the batch API (one plan shared by every item, shared edge
    // input) gets, for up to 4 states, the records of one tree, which every
    // item reads (the shared-topology layout of phase_engine.cuh); above 4
    // states the batch API keeps the per-tree engine.
    if (PaddedStates(states) == 4 || !shared_edges) {
      phase_batch = shared_edges;
      std::vector<PhaseInstance> phase_instances(phase_batch ? 1 : count);
      for (std::size_t i = 0; i < phase_instances.size(); ++i)
        phase_instances[i] = {table[i].program, table[i].node_base, table[i].edge_out_base,
                              table[i].obs_base};
      phase = phase_batch
                  ? BuildPhasePlan(set, phase_instances, nodes_per_item, edges_per_item, 0)
                  : BuildPhasePlan(set, phase_instances, total_nodes, total_edges_out, 0);
      // Stored objects of the batch layout are item-minor over the capacity.
      const std::uint64_t copies = phase_batch ? count : 1;
      if (phase.enabled && phase_batch &&
          (total_nodes >= kFlag || phase.total_compressions * copies >= kFlag))
        phase = PhasePlan{};
      if (phase.enabled) {
        phase_rakes.Upload(phase.rakes, stream);
        phase_gathers.Upload(phase.gathers, stream);
        phase_compress.Upload(phase.compress, stream);
        phase_roots.Upload(phase.roots, stream);
        node_exp.Allocate(total_nodes * sizeof(int));
        comp_exp.Allocate(phase.total_compressions * copies * sizeof(int));
        observation_reads = categorical ? phase.observation_order.size() : 0;
        observation_order.Upload(phase.observation_order, stream);
        phase_observations.Allocate(observation_reads * copies);
        phase.observation_order = {};
        // The records now live on the device; the host keeps the counts.
        phase.rakes = {};
        phase.gathers = {};
        phase.compress = {};
        phase.roots = {};
        schedule = THMM_SCHEDULE_PHASES;
        SetPhaseRounds(0);
      }
    }
    // Work counters of the forward [0..1] and adjoint [4..5] launches; [2] is
    // the error word; words 8 + 8c .. 15 + 8c hold the counters of stripe c.
    control.Allocate((8 + 8 * kMaxStripes) * sizeof(std::uint32_t));

    // Inputs, outputs and scratch.
    const std::size_t S = ScalarBytes();
    const std::uint64_t edge_values = edge_inputs * KK;
    // Pinned host staging, unless the workspace is reserved for device
    // inputs only (THMM_RESERVE_DEVICE_ONLY).
    const auto host = [&](HostBuffer &buffer, std::size_t size) {
      if (!device_only)
        buffer.Allocate(size);
    };
    if (!categorical) {
      node_in.Allocate(total_nodes * K * S);
      host(h_node_in, total_nodes * K * S);
    } else {
      observations.Allocate(total_observations);
      host(h_observations, total_observations);
      root_potential.Allocate(K * S);
      host(h_root, K * S);
      emission.Allocate(categories * K * S);
      host(h_emission, categories * K * S);
    }
    edge_in.Allocate(edge_values * S);
    host(h_edge_in, edge_values * S);
    values.Allocate(count * S);
    host(h_values, count * S);
    h_control.Allocate(16);
    if (marginals) {
      node_out.Allocate(total_nodes * K * S);
      host(h_node_out, total_nodes * K * S);
      edge_out.Allocate(total_edges_out * KK * S);
      host(h_edge_out, total_edges_out * KK * S);
    }
    if (maximum || sampling) {
      states_out.Allocate(total_nodes * sizeof(std::uint32_t));
      host(h_states, total_nodes * sizeof(std::uint32_t));
    }
    if (sampling) {
      uniforms.Allocate(total_nodes * S);
      host(h_uniforms, total_nodes * S);
    }
    scratch.Allocate(scratch_base * compute_bytes);
    bytes.Allocate(byte_base);

    // Occupancy of each kernel this workspace may launch.
    const unsigned kmax = PaddedStates(states);
    EngineArgs probe{};
    occupancy[0] = occupancy[1] = occupancy[2] = occupancy[3] = 1;
    for (int part = 0; part < (marginals ? 2 : 1); ++part) {
      int *slot = &occupancy[part == 0 ? 0 : 3];
      Check(scalar == 8 ? LaunchLinearF64(compute_f64, kmax, part, probe, 0, nullptr, slot)
                        : LaunchLinearF32(compute_f64, kmax, part, probe, 0, nullptr, slot),
            "occupancy query");
    }
    if (maximum)
      Check(LaunchMaximum(scalar, kmax, probe, 0, nullptr, &occupancy[1]),
            "occupancy query");
    if (sampling)
      Check(LaunchSample(scalar, kmax, probe, 0, nullptr, &occupancy[2]),
            "occupancy query");
    Check(cudaStreamSynchronize(stream), "topology upload");
    reserved = true;
  }

  void ReserveBatch(const btrc::Plan &p, std::size_t state_count,
                    std::size_t batch, int device_index, std::uint32_t flags,
                    std::uint32_t scalar_bytes, bool is_categorical,
                    std::size_t category_count,
                    std::span<const std::uint32_t> observed) {
    if (is_categorical) {
      if (category_count == 0 || category_count > 256)
        throw std::invalid_argument("accelerator categorical model must have "
                                    "between 1 and 256 categories");
      ValidateObservationNodes(p, observed);
    }
    if (batch == 0)
      throw std::invalid_argument(
          "accelerator state and batch counts must be nonzero");
    Begin(state_count, device_index, flags, scalar_bytes);
    plan = &p;
    capacity = batch;
    categorical = is_categorical;
    categories = category_count;
    observation_nodes.assign(observed.begin(), observed.end());
    nodes_per_item = p.num_nodes();
    edges_per_item = p.num_edges();
    observations_per_item = observed.size();
    CheckedProduct({batch, p.num_nodes(), state_count}, "node workspace");
    CheckedProduct({batch, p.num_edges(), state_count, state_count},
                   "edge workspace");
    std::vector<const btrc::Plan *> instance_plans(batch, &p);
    std::vector<std::vector<std::uint32_t>> instance_observations;
    if (categorical)
      instance_observations.assign(batch, observation_nodes);
    Build(instance_plans, instance_observations, true);
  }

  void ReserveForest(std::span<const btrc::Plan *const> plans,
                     std::size_t state_count, int device_index,
                     std::uint32_t flags, std::uint32_t scalar_bytes,
                     bool is_categorical, std::size_t category_count,
                     const std::uint32_t *observed, const std::size_t *counts) {
    if (plans.empty())
      throw std::invalid_argument("a forest needs at least one tree");
    for (const btrc::Plan *p : plans)
      if (p == nullptr)
        throw std::invalid_argument("forest plan must not be null");
    std::vector<std::vector<std::uint32_t>> instance_observations;
    if (is_categorical) {
      if (category_count == 0 || category_count > 256)
        throw std::invalid_argument("accelerator categorical model must have "
                                    "between 1 and 256 categories");
      std::size_t offset = 0;
      for (std::size_t t = 0; t < plans.size(); ++t) {
        const std::size_t n = counts == nullptr ? 0 : counts[t];
        const std::span<const std::uint32_t> tree_observed(
            observed == nullptr ? nullptr : observed + offset, n);
        ValidateObservationNodes(*plans[t], tree_observed);
        instance_observations.emplace_back(tree_observed.begin(),
                                           tree_observed.end());
        offset += n;
      }
    }
    Begin(state_count, device_index, flags, scalar_bytes);
    forest = true;
    capacity = plans.size();
    categorical = is_categorical;
    categories = category_count;
    for (const auto &tree : instance_observations)
      observation_nodes.insert(observation_nodes.end(), tree.begin(), tree.end());
    Build(std::vector<const btrc::Plan *>(plans.begin(), plans.end()),
          instance_observations, false);
  }

  static void ValidateObservationNodes(const btrc::Plan &p,
                                       std::span<const std::uint32_t> observed) {
    for (std::size_t i = 0; i < observed.size(); ++i) {
      if (observed[i] >= p.num_nodes() || (i > 0 && observed[i] <= observed[i - 1]))
        throw std::invalid_argument(
            "accelerator categorical observation nodes must be valid and "
            "strictly increasing");
    }
  }

  // ----------------------------------------------------------- staging views
  void RequireReserved() const {
    if (!reserved)
      throw std::logic_error("accelerator Workspace::Reserve must precede Inputs");
  }
  void RequireStaging() const {
    if (device_only)
      throw std::logic_error(
          "workspace reserved for device inputs only has no host staging: write the inputs "
          "through thmm_device_buffers_get and run thmm_enqueue");
  }

  std::size_t NodesFor(std::size_t batch) const {
    return forest ? total_nodes : batch * nodes_per_item;
  }
  std::size_t EdgeOutFor(std::size_t batch) const {
    return forest ? total_edges_out : batch * edges_per_item;
  }
  std::size_t ObservationsFor(std::size_t batch) const {
    return forest ? total_observations : batch * observations_per_item;
  }
  void CheckBatch(std::size_t batch, const char *what) const {
    if (forest ? batch != capacity : (batch == 0 || batch > capacity))
      throw std::invalid_argument(std::string("accelerator ") + what +
                                  " batch exceeds the reserved capacity");
  }

  // ------------------------------------------------------------------- run
  // Which per-instance slice of a buffer a stripe owns.
  enum Slice : int { kWhole, kNodes, kEdges, kObservations };
  struct Upload {
    const void *source;
    HostBuffer *staging;
    DeviceBuffer *device;
    std::size_t bytes;
    Slice slice = kWhole; // kWhole: copied with the first stripe
    std::size_t unit = 0; // bytes per node, edge or observation
  };

  // Kernel arguments of `operation`, without the work queue.
  EngineArgs MakeArgs(int operation) const {
    EngineArgs args{};
    args.programs = programs.as<DevProgram>();
    args.steps = steps.as<DevStep>();
    args.rakes = rakes.ptr;
    args.combines = combines.ptr;
    args.absorbs = absorbs.ptr;
    args.compress = compress.ptr;
    args.compress_ends = compress_ends.ptr;
    args.gathers = gathers.ptr;
    args.instances = instances.as<DevInstance>();
    args.error = control.as<std::uint32_t>() + 2;
    args.node_in = node_in.ptr;
    args.observations = observations.as<std::uint8_t>();
    args.root_potential = root_potential.ptr;
    args.emission = emission.ptr;
    args.categories = static_cast<std::uint32_t>(categories);
    args.categorical = categorical ? 1u : 0u;
    args.edge_in = edge_in.ptr;
    args.states = static_cast<std::uint32_t>(states);
    args.reverse = operation == THMM_OP_MARGINALS ? 1u : 0u;
    args.raw = operation == THMM_OP_PARTITION ? 1u : 0u;
    args.scratch = scratch.ptr;
    args.bytes = bytes.as<std::uint8_t>();
    args.values = values.ptr;
    args.node_out = node_out.ptr;
    args.edge_out = edge_out.ptr;
    args.states_out = states_out.as<std::uint32_t>();
    args.uniforms = uniforms.ptr;
    args.bf16 = bf16 ? 1u : 0u;
    return args;
  }

  // Launches the kernels of `operation` over the queue set in `args`, with
  // work counters at counters[0..1] (forward) and counters[4..5] (adjoint);
  // the counters must be zero. Returns the number of kernel launches.
  int LaunchTeams(int operation, EngineArgs args, std::uint32_t *counters) {
    const unsigned kmax = PaddedStates(states);
    args.queue = counters;
    const int kind = operation == THMM_OP_MAXIMUM ? 1
                     : operation == THMM_OP_SAMPLE ? 2
                                                   : 0;
    const std::uint64_t teams_needed =
        std::max<std::uint64_t>(args.big_count, (args.small_count + kWarpsPerCta - 1) /
                                                    kWarpsPerCta);
    const auto grid_for = [&](int slot) {
      int per_sm = std::max(occupancy[slot], 1);
      if (cta_cap[slot] > 0)
        per_sm = std::min(per_sm, cta_cap[slot]);
      return static_cast<int>(std::max<std::uint64_t>(
          1, std::min<std::uint64_t>(teams_needed,
                                     static_cast<std::uint64_t>(sms) * per_sm)));
    };
    cudaError_t status;
    int count = 1;
    if (kind == 1) {
      status = LaunchMaximum(scalar, kmax, args, grid_for(1), stream, nullptr);
    } else if (kind == 2) {
      status = LaunchSample(scalar, kmax, args, grid_for(2), stream, nullptr);
    } else {
      const auto linear = [&](int part, int grid) {
        return scalar == 8
                   ? LaunchLinearF64(compute_f64, kmax, part, args, grid, stream, nullptr)
                   : LaunchLinearF32(compute_f64, kmax, part, args, grid, stream, nullptr);
      };
      status = linear(0, grid_for(0));
      if (status == cudaSuccess && args.reverse) {
        args.queue = counters + 4;
        status = linear(1, grid_for(3));
        count = 2;
      }
    }
    Check(status, "tree-HMM accelerator kernel launch");
    return count;
  }

  // Rounds of the phase schedule run grid-wide (0: the first round with
  // fewer than 2^17 gathers and compressions); uploads the tail records of
  // the rest. A tail of more than 2^20 trees stays grid-wide, and so do the
  // batch layout (every item has every round) and every state count above 4.
  void SetPhaseRounds(std::uint32_t rounds) {
    if (!phase.enabled)
      return;
    std::uint32_t wanted = rounds != 0 ? rounds : phase.AutoTailRound(1u << 17);
    wanted = std::max<std::uint32_t>(wanted, 1);
    if (phase_batch || states > 4)
      wanted = phase.rounds; // no tail kinds above 4 states
    PhasePlan::Tail tail;
    if (wanted < phase.rounds) {
      tail = phase.BuildTail(wanted);
      if (tail.items.size() > (1u << 20)) {
        wanted = phase.rounds;
        tail = PhasePlan::Tail{};
      }
    }
    phase_rounds = std::min(wanted, phase.rounds);
    tail_instances.clear();
    for (const Uint4 &item : tail.items)
      tail_instances.push_back(item.x);
    tail_items.Upload(tail.items, stream);
    tail_rounds.Upload(tail.rounds, stream);
    tail_rakes.Upload(tail.rakes, stream);
    Check(cudaStreamSynchronize(stream), "tail record upload");
    DropGraphs();
  }

  // Rebuilds the phase-ordered observation copy on stream `s` (after the
  // observations themselves arrived on it).
  void OrderObservations(cudaStream_t s) {
    if (phase.enabled && observation_reads != 0)
      Check(LaunchObservationGather(observations.as<std::uint8_t>(),
                                    observation_order.as<std::uint32_t>(),
                                    phase_observations.as<std::uint8_t>(), observation_reads,
                                    phase_batch ? capacity : 1,
                                    phase_batch ? observations_per_item : 0, s),
            "observation ordering launch");
  }
  bool UploadsObservations(const std::vector<Upload> &uploads) const {
    for (const Upload &upload : uploads)
      if (upload.device == &observations && upload.bytes != 0)
        return true;
    return false;
  }

  bool UsePhases(int operation) const {
    return schedule == THMM_SCHEDULE_PHASES && phase.enabled &&
           (operation == THMM_OP_PARTITION || operation == THMM_OP_LOG_PARTITION ||
            operation == THMM_OP_MARGINALS);
  }

  const PhaseRanges &PhaseRangesFor(std::uint32_t a, std::uint32_t b) {
    for (const PhaseRanges &ranges : phase_ranges)
      if (ranges.a == a && ranges.b == b)
        return ranges;
    PhaseRanges ranges{a, b, {}, {}, {}};
    for (std::uint32_t r = 0; r < phase.rounds; ++r) {
      ranges.gather.push_back(phase.OpRange(kPhaseGather, r, a, b));
      ranges.rake.push_back(phase.OpRange(kPhaseRakeReverse, r, a, b));
      ranges.compress.push_back(phase.OpRange(kPhaseCompress, r, a, b));
    }
    if (phase_ranges.size() >= 32)
      phase_ranges.erase(phase_ranges.begin());
    phase_ranges.push_back(std::move(ranges));
    return phase_ranges.back();
  }

  // Launches the phase schedule of `operation` over instances [a, b):
  // gather and compress phases round by round, the finish phase, then (for
  // marginals) the adjoint phases in reverse round order. Returns the number
  // of kernel launches.
  int LaunchPhases(int operation, std::uint32_t a, std::uint32_t b) {
    // Batch layout: every item runs the one tree's operations; items [a, b).
    const PhaseRanges &ranges = phase_batch ? PhaseRangesFor(0, 1) : PhaseRangesFor(a, b);
    const std::size_t K = states;
    const std::size_t compute_bytes = compute_f64 ? 8 : 4;
    unsigned char *work = scratch.as<unsigned char>();
    PhaseArgs args{};
    args.rakes = phase_rakes.as<uint4>();
    args.gathers = phase_gathers.as<uint4>();
    args.compress = phase_compress.as<uint4>();
    args.roots = phase_roots.as<uint2>();
    args.node_in = node_in.ptr;
    args.observations = phase_observations.as<std::uint8_t>();
    args.root_potential = root_potential.ptr;
    args.emission = emission.ptr;
    args.categories = static_cast<std::uint32_t>(categories);
    args.categorical = categorical ? 1u : 0u;
    args.edge_in = edge_in.ptr;
    args.edge_modulus = shared_edge_input ? static_cast<std::uint32_t>(edges_per_item) : 0u;
    args.states = static_cast<std::uint32_t>(states);
    args.nodes = work;
    args.comps = work + total_nodes * K * compute_bytes;
    const std::uint64_t copies = phase_batch ? capacity : 1;
    args.comp_mu =
        work + (total_nodes * K + phase.total_compressions * copies * K * K) * compute_bytes;
    if (phase_batch) {
      args.batch = 1;
      args.first_item = a;
      args.items = b - a;
      args.item_stride = capacity;
      args.item_nodes = nodes_per_item;
      args.item_edges = edges_per_item;
      args.edge_modulus = 0;
    }
    args.node_exp = node_exp.as<int>();
    args.comp_exp = comp_exp.as<int>();
    args.values = values.ptr;
    args.node_out = node_out.ptr;
    args.edge_out = edge_out.ptr;
    args.raw = operation == THMM_OP_PARTITION ? 1u : 0u;
    args.reverse = operation == THMM_OP_MARGINALS ? 1u : 0u;
    args.tail_items = tail_items.as<uint4>();
    args.tail_rounds = tail_rounds.as<uint4>();
    args.tail_rakes = tail_rakes.as<uint2>();
    args.error = control.as<std::uint32_t>() + 2;
    args.bf16 = bf16 ? 1u : 0u;
    int count = 0;
    const auto launch = [&](int kind, std::pair<std::uint64_t, std::uint64_t> range) {
      if (range.second <= range.first)
        return;
      args.offset = static_cast<std::uint32_t>(range.first);
      args.count = static_cast<std::uint32_t>(range.second - range.first);
      Check(LaunchPhase(scalar, compute_f64, kind, args, stream, nullptr),
            "tree-HMM accelerator kernel launch");
      ++count;
    };
    // Tail trees of instances [a, b).
    const std::pair<std::uint64_t, std::uint64_t> tail{
        std::lower_bound(tail_instances.begin(), tail_instances.end(), a) -
            tail_instances.begin(),
        std::lower_bound(tail_instances.begin(), tail_instances.end(), b) -
            tail_instances.begin()};
    const std::uint32_t grid_rounds = std::min(phase_rounds, phase.rounds);
    for (std::uint32_t r = 0; r < grid_rounds; ++r) {
      launch(kPhaseGather, ranges.gather[r]);
      launch(kPhaseCompress, ranges.compress[r]);
    }
    launch(kPhaseTailForward, tail);
    launch(kPhaseFinish, phase_batch ? std::pair<std::uint64_t, std::uint64_t>{0, 1}
                                     : std::pair<std::uint64_t, std::uint64_t>{a, b});
    if (operation == THMM_OP_MARGINALS) {
      launch(kPhaseTailReverse, tail);
      for (std::uint32_t r = grid_rounds; r-- > 0;) {
        launch(kPhaseCompressReverse, ranges.compress[r]);
        launch(kPhaseRakeReverse, ranges.rake[r]);
      }
    }
    return count;
  }

  // One device step over all instances of the batch, on the workspace stream.
  void EnqueueDevice(int operation, std::size_t batch) {
    EngineArgs args = MakeArgs(operation);
    args.big_items = team_order.as<std::uint32_t>();
    args.small_items = team_order.as<std::uint32_t>() + big_count;
    if (forest) {
      args.big_count = big_count;
      args.small_count = small_count;
    } else {
      args.big_count = items_big ? static_cast<std::uint32_t>(batch) : 0u;
      args.small_count = items_big ? 0u : static_cast<std::uint32_t>(batch);
    }
    Check(cudaMemsetAsync(control.ptr, 0, 32, stream), "cudaMemsetAsync");
    const auto items = static_cast<std::uint32_t>(forest ? capacity : batch);
    launches = static_cast<std::uint64_t>(
        UsePhases(operation) ? LaunchPhases(operation, 0, items)
                             : LaunchTeams(operation, args, control.as<std::uint32_t>()));
  }

  // Splits the largest-first queue at `threshold` nodes (CTA teams above).
  void ApplyThreshold(std::uint32_t threshold) {
    team_threshold = std::max<std::uint32_t>(threshold, 1);
    if (states > 32)
      team_threshold = 1; // the wide-state engine contracts every tree with a CTA
    const auto split = std::partition_point(
        sorted_nodes.begin(), sorted_nodes.end(),
        [&](std::uint64_t n) { return n >= team_threshold; });
    big_count = static_cast<std::uint32_t>(split - sorted_nodes.begin());
    small_count = static_cast<std::uint32_t>(sorted_nodes.end() - split);
    items_big = big_count != 0;
    DropGraphs();
  }

  // Device-only step replayed from a CUDA graph captured on first use (the
  // memset of the work counters plus the kernel launches of EnqueueDevice).
  void EnqueueGraph(int operation, std::size_t batch) {
    for (const Graph &graph : graphs)
      if (graph.operation == operation && graph.batch == batch) {
        Check(cudaGraphLaunch(graph.exec, stream), "cudaGraphLaunch");
        return;
      }
    cudaGraph_t graph = nullptr;
    Check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed),
          "cudaStreamBeginCapture");
    try {
      EnqueueDevice(operation, batch);
    } catch (...) {
      static_cast<void>(cudaStreamEndCapture(stream, &graph));
      if (graph != nullptr)
        static_cast<void>(cudaGraphDestroy(graph));
      throw;
    }
    Check(cudaStreamEndCapture(stream, &graph), "cudaStreamEndCapture");
    cudaGraphExec_t exec = nullptr;
    const cudaError_t status = cudaGraphInstantiate(&exec, graph, 0);
    static_cast<void>(cudaGraphDestroy(graph));
    Check(status, "cudaGraphInstantiate");
    graphs.push_back({operation, batch, exec});
    Check(cudaGraphLaunch(exec, stream), "cudaGraphLaunch");
  }

  static int KernelSlot(int operation) {
    return operation == THMM_OP_MAXIMUM ? 1 : operation == THMM_OP_SAMPLE ? 2 : 0;
  }

  // Mean device time of `repeats` steps of `operation` on the resident
  // inputs, after one untimed step.
  float TimeSteps(int operation, int repeats) {
    EnqueueDevice(operation, last_batch);
    Check(cudaEventRecord(events[0], stream), "cudaEventRecord");
    for (int r = 0; r < repeats; ++r)
      EnqueueDevice(operation, last_batch);
    Check(cudaEventRecord(events[1], stream), "cudaEventRecord");
    Check(cudaEventSynchronize(events[1]), "autotune step");
    float ms = 0.0f;
    Check(cudaEventElapsedTime(&ms, events[0], events[1]), "cudaEventElapsedTime");
    return ms / static_cast<float>(repeats);
  }

  // Searches the team threshold and the CTAs per SM of the kernels that
  // `operation` launches, timing each candidate on the resident inputs, and
  // keeps the fastest. Candidates that give the same team split are timed
  // once.
  thmm_tuning Autotune(int operation, int repeats) {
    const int slot = KernelSlot(operation);
    const bool adjoint = operation == THMM_OP_MARGINALS;
    std::vector<std::uint32_t> thresholds;
    std::vector<std::uint32_t> splits;
    for (std::uint32_t t : {256u, 512u, 1024u, 2048u, 4096u, 8192u, 16384u, 1u << 31}) {
      const auto split = static_cast<std::uint32_t>(
          std::partition_point(sorted_nodes.begin(), sorted_nodes.end(),
                               [&](std::uint64_t n) { return n >= t; }) -
          sorted_nodes.begin());
      if (std::find(splits.begin(), splits.end(), split) == splits.end()) {
        splits.push_back(split);
        thresholds.push_back(t);
      }
    }
    const auto caps_for = [&](int s) {
      std::vector<int> caps;
      for (int c = std::max(occupancy[s], 1); c >= 1 && caps.size() < 3; --c)
        caps.push_back(c);
      return caps;
    };
    const std::vector<int> forward_caps = caps_for(slot);
    const std::vector<int> reverse_caps = adjoint ? caps_for(3) : std::vector<int>{0};
    schedule = THMM_SCHEDULE_TEAMS; // team candidates first
    thmm_tuning best{};
    best.kernel_ms = std::numeric_limits<float>::infinity();
    std::uint32_t tried = 0;
    for (const std::uint32_t threshold : thresholds) {
      ApplyThreshold(threshold);
      for (const int forward : forward_caps) {
        for (const int reverse : reverse_caps) {
          cta_cap[slot] = forward;
          cta_cap[3] = reverse;
          const float ms = TimeSteps(operation, repeats);
          ++tried;
          if (ms < best.kernel_ms) {
            best.kernel_ms = ms;
            best.team_threshold = threshold;
            std::fill(std::begin(best.ctas_per_sm), std::end(best.ctas_per_sm), 0u);
            best.ctas_per_sm[slot] = static_cast<std::uint32_t>(forward);
            best.ctas_per_sm[3] = static_cast<std::uint32_t>(reverse);
          }
        }
      }
    }
    // The phase schedule's one setting: how many rounds run grid-wide.
    if (phase.enabled && operation != THMM_OP_MAXIMUM && operation != THMM_OP_SAMPLE) {
      schedule = THMM_SCHEDULE_PHASES;
      std::vector<std::uint32_t> tried_rounds;
      const std::uint32_t automatic = phase.AutoTailRound(1u << 17);
      for (std::uint32_t rounds : {automatic, 1u, 2u, 3u, 4u, 5u, 6u, 8u, phase.rounds}) {
        SetPhaseRounds(rounds);
        if (std::find(tried_rounds.begin(), tried_rounds.end(), phase_rounds) !=
            tried_rounds.end())
          continue;
        tried_rounds.push_back(phase_rounds);
        const float ms = TimeSteps(operation, repeats);
        ++tried;
        if (ms < best.kernel_ms) {
          best.kernel_ms = ms;
          best.schedule = THMM_SCHEDULE_PHASES;
          best.phase_rounds = phase_rounds;
        }
      }
    }
    best.candidates = tried;
    best.stripes = stripes_setting;
    ApplyTuning(best);
    return best;
  }

  void ApplyTuning(const thmm_tuning &tuning) {
    if (tuning.schedule != THMM_SCHEDULE_TEAMS && tuning.schedule != THMM_SCHEDULE_PHASES)
      throw std::invalid_argument("unknown schedule");
    schedule = phase.enabled ? tuning.schedule : THMM_SCHEDULE_TEAMS;
    if (phase.enabled && tuning.phase_rounds != phase_rounds)
      SetPhaseRounds(tuning.phase_rounds);
    ApplyThreshold(tuning.team_threshold);
    for (int slot = 0; slot < 4; ++slot)
      cta_cap[slot] = static_cast<int>(tuning.ctas_per_sm[slot]);
    stripes_setting = std::min(tuning.stripes, kMaxStripes);
    tuned_ms = tuning.kernel_ms;
  }

  thmm_tuning CurrentTuning() const {
    thmm_tuning tuning{};
    tuning.team_threshold = team_threshold;
    for (int slot = 0; slot < 4; ++slot)
      tuning.ctas_per_sm[slot] = static_cast<std::uint32_t>(cta_cap[slot]);
    tuning.stripes = stripes_setting;
    tuning.kernel_ms = tuned_ms;
    tuning.schedule = schedule;
    tuning.phase_rounds = phase_rounds;
    return tuning;
  }

  struct Outcome {
    thmm_timings timings;
    std::uint32_t error;
  };

  Outcome Run(int operation, std::size_t batch, const std::vector<Upload> &uploads,
              Clock::time_point wall_start) {
    RequireStaging();
    Check(cudaSetDevice(device), "cudaSetDevice");
    for (const Upload &upload : uploads)
      if (upload.source != upload.staging->ptr && upload.bytes != 0)
        std::memcpy(upload.staging->ptr, upload.source, upload.bytes);
    if (StripeCount(batch) > 1)
      return RunStriped(operation, batch, uploads, wall_start);
    Check(cudaEventRecord(events[0], stream), "cudaEventRecord");
    for (const Upload &upload : uploads)
      if (upload.bytes != 0)
        Check(cudaMemcpyAsync(upload.device->ptr, upload.staging->ptr, upload.bytes,
                              cudaMemcpyHostToDevice, stream),
              "cudaMemcpyAsync input upload");
    if (UploadsObservations(uploads))
      OrderObservations(stream);
    Check(cudaEventRecord(events[1], stream), "cudaEventRecord");
    Check(cudaEventRecord(events[2], stream), "cudaEventRecord");
    EnqueueDevice(operation, batch);
    Check(cudaEventRecord(events[3], stream), "cudaEventRecord");
    Check(cudaEventRecord(events[4], stream), "cudaEventRecord");
    const std::size_t S = ScalarBytes();
    const std::size_t items = forest ? capacity : batch;
    const auto download = [&](HostBuffer &host, DeviceBuffer &dev, std::size_t n) {
      if (n != 0)
        Check(cudaMemcpyAsync(host.ptr, dev.ptr, n, cudaMemcpyDeviceToHost, stream),
              "cudaMemcpyAsync result download");
    };
    download(h_values, values, items * S);
    download(h_control, control, 16);
    if (operation == THMM_OP_MARGINALS) {
      download(h_node_out, node_out, NodesFor(batch) * states * S);
      download(h_edge_out, edge_out, EdgeOutFor(batch) * states * states * S);
    }
    if (operation == THMM_OP_MAXIMUM || operation == THMM_OP_SAMPLE)
      download(h_states, states_out, NodesFor(batch) * sizeof(std::uint32_t));
    Check(cudaEventRecord(events[5], stream), "cudaEventRecord");
    Check(cudaEventSynchronize(events[5]), "tree-HMM accelerator execution");
    last_batch = batch;
    has_run = true;
    float upload_ms = 0, kernel_ms = 0, download_ms = 0;
    Check(cudaEventElapsedTime(&upload_ms, events[0], events[1]), "cudaEventElapsedTime");
    Check(cudaEventElapsedTime(&kernel_ms, events[2], events[3]), "cudaEventElapsedTime");
    Check(cudaEventElapsedTime(&download_ms, events[4], events[5]), "cudaEventElapsedTime");
    Outcome outcome{};
    outcome.timings.upload_ms = upload_ms;
    outcome.timings.kernel_ms = kernel_ms;
    outcome.timings.download_ms = download_ms;
    outcome.error = h_control.as<std::uint32_t>()[2];
    if (outcome.error & kErrorTensorTimeout)
      throw std::runtime_error("tree-HMM accelerator tensor-core wait timed out");
    outcome.timings.wall_ms =
        std::chrono::duration<double, std::milli>(Clock::now() - wall_start).count();
    return outcome;
  }

  // ------------------------------------------------------ striped calls
  std::uint32_t StripeCount(std::size_t batch) const {
    const std::size_t items = forest ? capacity : batch;
    std::uint64_t want = stripes_setting;
    if (want == 0)
      want = std::clamp<std::uint64_t>(NodesFor(batch) / kNodesPerStripe, 1, kMaxStripes);
    return static_cast<std::uint32_t>(
        std::min<std::uint64_t>({want, items, kMaxStripes}));
  }

  // Cuts instances [0, items) into stripes of about equal node count and
  // uploads each stripe's largest-first order.
  void PlanStripes(std::size_t batch, std::uint32_t wanted) {
    const std::size_t items = forest ? capacity : batch;
    if (stripe_batch == batch && stripe_threshold == team_threshold &&
        stripe_wanted == wanted && !stripe_plan.empty())
      return;
    std::vector<std::uint32_t> bounds{0};
    const std::uint64_t total = off_nodes[items];
    for (std::uint32_t c = 1; c < wanted; ++c) {
      const std::uint64_t target = total * c / wanted;
      const auto at = std::lower_bound(off_nodes.begin(), off_nodes.begin() + items + 1,
                                       target) - off_nodes.begin();
      const auto index = static_cast<std::uint32_t>(at);
      if (index > bounds.back() && index < items)
        bounds.push_back(index);
    }
    bounds.push_back(static_cast<std::uint32_t>(items));
    std::vector<std::uint32_t> order(items);
    stripe_plan.clear();
    for (std::size_t c = 0; c + 1 < bounds.size(); ++c) {
      const std::uint32_t a = bounds[c], b = bounds[c + 1];
      std::iota(order.begin() + a, order.begin() + b, a);
      std::stable_sort(order.begin() + a, order.begin() + b,
                       [&](std::uint32_t x, std::uint32_t y) {
                         return tree_nodes[x] > tree_nodes[y];
                       });
      std::uint32_t big = 0;
      while (a + big < b && tree_nodes[order[a + big]] >= team_threshold)
        ++big;
      stripe_plan.push_back({a, b, big, (b - a) - big});
    }
    stripe_order.Upload(order, stream);
    stripe_batch = batch;
    stripe_threshold = team_threshold;
    stripe_wanted = wanted;
  }

  // Byte range [offset, offset + size) of a buffer owned by instances [a, b).
  std::pair<std::size_t, std::size_t> SliceRange(Slice slice, std::size_t unit,
                                                 std::size_t bytes, std::uint32_t a,
                                                 std::uint32_t b, bool first) const {
    const std::vector<std::uint64_t> *offsets =
        slice == kNodes ? &off_nodes : slice == kEdges ? &off_edges
        : slice == kObservations ? &off_obs : nullptr;
    if (offsets == nullptr)
      return {0, first ? bytes : 0};
    return {(*offsets)[a] * unit, ((*offsets)[b] - (*offsets)[a]) * unit};
  }

  // A prepared call cut into stripes: per stripe, input copies on copy_in,
  // kernels on the workspace stream after that stripe's inputs arrived, and
  // output copies on copy_out after its kernels. Timings: upload_ms spans the
  // input copies, kernel_ms the kernels, download_ms the output copies; they
  // overlap.
  Outcome RunStriped(int operation, std::size_t batch, const std::vector<Upload> &uploads,
                     Clock::time_point wall_start) {
    PlanStripes(batch, StripeCount(batch));
    const auto P = static_cast<std::uint32_t>(stripe_plan.size());
    const std::size_t S = ScalarBytes();
    const std::size_t K = states;
    cudaEvent_t *t = stripe_timing;
    Check(cudaEventRecord(t[0], stream), "cudaEventRecord");
    Check(cudaStreamWaitEvent(copy_in, t[0], 0), "cudaStreamWaitEvent");
    Check(cudaStreamWaitEvent(copy_out, t[0], 0), "cudaStreamWaitEvent");
    Check(cudaMemsetAsync(control.ptr, 0, (8 + 8 * P) * sizeof(std::uint32_t), stream),
          "cudaMemsetAsync");
    const auto device_bytes = [](DeviceBuffer &buffer) {
      return static_cast<unsigned char *>(buffer.ptr);
    };
    const auto host_bytes = [](HostBuffer &buffer) {
      return static_cast<unsigned char *>(buffer.ptr);
    };
    // With the phase schedule the observations arrive whole with the first
    // stripe: their phase-ordered copy is rebuilt before any stripe runs.
    const bool order_observations = UploadsObservations(uploads) && phase.enabled;
    for (std::uint32_t c = 0; c < P; ++c) {
      const Stripe &stripe = stripe_plan[c];
      for (const Upload &upload : uploads) {
        const Slice slice =
            order_observations && upload.slice == kObservations ? kWhole : upload.slice;
        const auto [offset, size] = SliceRange(slice, upload.unit, upload.bytes,
                                               stripe.first, stripe.last, c == 0);
        if (size != 0)
          Check(cudaMemcpyAsync(device_bytes(*upload.device) + offset,
                                host_bytes(*upload.staging) + offset, size,
                                cudaMemcpyHostToDevice, copy_in),
                "cudaMemcpyAsync input upload");
      }
      Check(cudaEventRecord(arrived[c], copy_in), "cudaEventRecord");
    }
    Check(cudaEventRecord(t[1], copy_in), "cudaEventRecord");
    const EngineArgs base = MakeArgs(operation);
    std::uint64_t count = 0;
    for (std::uint32_t c = 0; c < P; ++c) {
      const Stripe &stripe = stripe_plan[c];
      Check(cudaStreamWaitEvent(stream, arrived[c], 0), "cudaStreamWaitEvent");
      if (c == 0)
        Check(cudaEventRecord(t[2], stream), "cudaEventRecord");
      if (c == 0 && order_observations)
        OrderObservations(stream);
      EngineArgs args = base;
      args.big_items = stripe_order.as<std::uint32_t>() + stripe.first;
      args.big_count = stripe.big;
      args.small_items = stripe_order.as<std::uint32_t>() + stripe.first + stripe.big;
      args.small_count = stripe.small;
      count += static_cast<std::uint64_t>(
          UsePhases(operation)
              ? LaunchPhases(operation, stripe.first, stripe.last)
              : LaunchTeams(operation, args, control.as<std::uint32_t>() + 8 + 8 * c));
      Check(cudaEventRecord(computed[c], stream), "cudaEventRecord");
    }
    Check(cudaEventRecord(t[3], stream), "cudaEventRecord");
    const auto download = [&](HostBuffer &host, DeviceBuffer &dev, Slice slice,
                              std::size_t unit, const Stripe &stripe) {
      std::size_t offset, size;
      if (slice == kWhole) {
        offset = stripe.first * unit;
        size = (stripe.last - stripe.first) * unit;
      } else {
        std::tie(offset, size) = SliceRange(slice, unit, 0, stripe.first, stripe.last,
                                            false);
      }
      if (size != 0)
        Check(cudaMemcpyAsync(host_bytes(host) + offset, device_bytes(dev) + offset, size,
                              cudaMemcpyDeviceToHost, copy_out),
              "cudaMemcpyAsync result download");
    };
    for (std::uint32_t c = 0; c < P; ++c) {
      const Stripe &stripe = stripe_plan[c];
      Check(cudaStreamWaitEvent(copy_out, computed[c], 0), "cudaStreamWaitEvent");
      if (c == 0)
        Check(cudaEventRecord(t[4], copy_out), "cudaEventRecord");
      download(h_values, values, kWhole, S, stripe); // one value per instance
      if (operation == THMM_OP_MARGINALS) {
        download(h_node_out, node_out, kNodes, K * S, stripe);
        download(h_edge_out, edge_out, kEdges, K * K * S, stripe);
      }
      if (operation == THMM_OP_MAXIMUM || operation == THMM_OP_SAMPLE)
        download(h_states, states_out, kNodes, sizeof(std::uint32_t), stripe);
    }
    Check(cudaMemcpyAsync(h_control.ptr, control.ptr, 16, cudaMemcpyDeviceToHost, copy_out),
          "cudaMemcpyAsync result download");
    Check(cudaEventRecord(t[5], copy_out), "cudaEventRecord");
    // Later work on the workspace stream follows this call's downloads.
    Check(cudaStreamWaitEvent(stream, t[5], 0), "cudaStreamWaitEvent");
    Check(cudaEventSynchronize(t[5]), "tree-HMM accelerator execution");
    launches = count;
    last_batch = batch;
    has_run = true;
    float upload_ms = 0, kernel_ms = 0, download_ms = 0;
    Check(cudaEventElapsedTime(&upload_ms, t[0], t[1]), "cudaEventElapsedTime");
    Check(cudaEventElapsedTime(&kernel_ms, t[2], t[3]), "cudaEventElapsedTime");
    Check(cudaEventElapsedTime(&download_ms, t[4], t[5]), "cudaEventElapsedTime");
    Outcome outcome{};
    outcome.timings.upload_ms = upload_ms;
    outcome.timings.kernel_ms = kernel_ms;
    outcome.timings.download_ms = download_ms;
    outcome.error = h_control.as<std::uint32_t>()[2];
    if (outcome.error & kErrorTensorTimeout)
      throw std::runtime_error("tree-HMM accelerator tensor-core wait timed out");
    outcome.timings.wall_ms =
        std::chrono::duration<double, std::milli>(Clock::now() - wall_start).count();
    return outcome;
  }

  double Value(std::size_t index) const {
    return scalar == 8 ? h_values.as<double>()[index]
                       : static_cast<double>(h_values.as<float>()[index]);
  }

  void RequireAllFinite(std::size_t count, const char *message) const {
    for (std::size_t i = 0; i < count; ++i)
      if (!std::isfinite(Value(i)))
        throw std::domain_error(message);
  }

  static constexpr int kWarpsPerCta = 4;
};

namespace {

template <class Body> thmm_status Guard(Body body) {
  try {
    body();
    g_last_error.clear();
    return THMM_OK;
  } catch (const std::invalid_argument &error) {
    g_last_error = error.what();
    return THMM_INVALID_ARGUMENT;
  } catch (const std::domain_error &error) {
    g_last_error = error.what();
    return THMM_DOMAIN_ERROR;
  } catch (const std::length_error &error) {
    g_last_error = error.what();
    return THMM_LENGTH_ERROR;
  } catch (const std::logic_error &error) {
    g_last_error = error.what();
    return THMM_LOGIC_ERROR;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return THMM_RUNTIME_ERROR;
  } catch (const std::exception &error) {
    g_last_error = error.what();
    return THMM_RUNTIME_ERROR;
  }
}

Workspace &AsWorkspace(thmm_workspace *workspace) {
  if (workspace == nullptr)
    throw std::invalid_argument("workspace must not be null");
  return *reinterpret_cast<Workspace *>(workspace);
}

// Shape and reservation checks shared by the dense calls
// (src/gpu_backend_impl.inc:2162-2187,2809-2818).
void CheckDense(const Workspace &ws, const thmm_dense_model &model,
                const char *requirement, bool reserved_for_operation) {
  if (!ws.reserved)
    throw std::invalid_argument(requirement);
  if (ws.categorical)
    throw std::invalid_argument(
        "dense accelerator inference cannot use a categorical workspace");
  if ((!ws.forest && reinterpret_cast<const btrc::Plan *>(model.plan) != ws.plan) ||
      model.states != ws.states || !reserved_for_operation)
    throw std::invalid_argument(requirement);
  ws.CheckBatch(model.batch, "input");
  if (model.node_count != ws.NodesFor(model.batch) * ws.states ||
      (model.node_count != 0 && model.node_potentials == nullptr))
    throw std::invalid_argument("accelerator node input shape is wrong");
  if (model.edge_count != ws.edge_inputs * ws.states * ws.states ||
      (model.edge_count != 0 && model.edge_potentials == nullptr))
    throw std::invalid_argument("accelerator edge input shape is wrong");
}

Workspace::Slice EdgeSlice(const Workspace &ws) {
  return ws.shared_edge_input ? Workspace::kWhole : Workspace::kEdges;
}

std::vector<Workspace::Upload> DenseUploads(Workspace &ws,
                                            const thmm_dense_model &model) {
  const std::size_t S = ws.ScalarBytes();
  const std::size_t K = ws.states;
  return {{model.node_potentials, &ws.h_node_in, &ws.node_in, model.node_count * S,
           Workspace::kNodes, K * S},
          {model.edge_potentials, &ws.h_edge_in, &ws.edge_in, model.edge_count * S,
           EdgeSlice(ws), K * K * S}};
}

// Categorical checks and residency rules (src/gpu_backend_impl.inc:2842-2946).
std::vector<Workspace::Upload> CategoricalUploads(Workspace &ws,
                                                  const thmm_categorical_model &model,
                                                  int update,
                                                  const char *requirement,
                                                  bool reserved_for_operation) {
  if (!ws.reserved || !ws.categorical || model.categories != ws.categories ||
      model.observation_node_count != ws.observation_nodes.size() ||
      (model.observation_node_count != 0 &&
       (model.observation_nodes == nullptr ||
        (model.observation_nodes != ws.observation_nodes.data() &&
         !std::equal(model.observation_nodes,
                     model.observation_nodes + model.observation_node_count,
                     ws.observation_nodes.begin())))))
    throw std::invalid_argument(
        "categorical accelerator model does not match the reserved workspace");
  if (update != THMM_UPDATE_ALL && update != THMM_UPDATE_FACTORS &&
      update != THMM_UPDATE_NONE)
    throw std::invalid_argument("unknown categorical input update policy");
  if ((!ws.forest && reinterpret_cast<const btrc::Plan *>(model.plan) != ws.plan) ||
      model.states != ws.states || !reserved_for_operation)
    throw std::invalid_argument(requirement);
  ws.CheckBatch(model.batch, "categorical input");
  if (model.observation_count != ws.ObservationsFor(model.batch) ||
      model.root_count != ws.states ||
      model.emission_count != ws.categories * ws.states ||
      (model.observation_count != 0 && model.observations == nullptr) ||
      model.root_potential == nullptr || model.emission_potentials == nullptr)
    throw std::invalid_argument("accelerator categorical input shapes are wrong");
  if (model.edge_count != ws.edge_inputs * ws.states * ws.states ||
      (model.edge_count != 0 && model.edge_potentials == nullptr))
    throw std::invalid_argument("accelerator edge input shape is wrong");
  const bool update_observations = update == THMM_UPDATE_ALL;
  const bool update_factors = update != THMM_UPDATE_NONE;
  if (!update_observations && ws.resident_observation_batch != model.batch)
    throw std::logic_error(
        "categorical observations are not resident for this batch; use kAll");
  if (!update_factors && !ws.resident_factors)
    throw std::logic_error(
        "categorical factors are not resident; use kAll or kFactors");
  const std::size_t S = ws.ScalarBytes();
  std::vector<Workspace::Upload> uploads;
  if (update_observations)
    uploads.push_back({model.observations, &ws.h_observations, &ws.observations,
                       model.observation_count, Workspace::kObservations, 1});
  if (update_factors) {
    uploads.push_back({model.root_potential, &ws.h_root, &ws.root_potential,
                       model.root_count * S});
    uploads.push_back({model.emission_potentials, &ws.h_emission, &ws.emission,
                       model.emission_count * S});
    uploads.push_back({model.edge_potentials, &ws.h_edge_in, &ws.edge_in,
                       model.edge_count * S, EdgeSlice(ws), ws.states * ws.states * S});
  }
  return uploads;
}

void MarkResident(Workspace &ws, std::size_t batch, int update) {
  if (update == THMM_UPDATE_ALL)
    ws.resident_observation_batch = batch;
  if (update != THMM_UPDATE_NONE)
    ws.resident_factors = true;
}

std::vector<Workspace::Upload> UniformUpload(Workspace &ws, std::size_t batch,
                                             const void *uniforms,
                                             std::size_t count) {
  if (count != ws.NodesFor(batch) || (count != 0 && uniforms == nullptr))
    throw std::invalid_argument(
        "prepared accelerator posterior sampling requires ReserveSampling and "
        "one uniform variate per batch item and node");
  return {{uniforms, &ws.h_uniforms, &ws.uniforms, count * ws.ScalarBytes(),
           Workspace::kNodes, ws.ScalarBytes()}};
}

void CheckSamplingOutcome(const Workspace &ws, const Workspace::Outcome &outcome,
                          std::size_t items) {
  if (outcome.error & kErrorInvalidUniform)
    throw std::invalid_argument("posterior-sampling variates must lie in [0, 1)");
  ws.RequireAllFinite(items, "the tree HMM has a nonpositive partition function");
  if (outcome.error & kErrorEmptyConditional)
    throw std::domain_error("cannot sample from an empty conditional distribution");
}

constexpr const char *kReserveMessage =
    "prepared accelerator inference requires Workspace::Reserve for this plan, "
    "state count, and batch capacity";
constexpr const char *kReserveMaximumMessage =
    "prepared accelerator MAP inference requires ReserveMaximum for this plan, "
    "state count, and batch capacity";
constexpr const char *kReserveSamplingMessage =
    "prepared accelerator posterior sampling requires ReserveSampling and one "
    "uniform variate per batch item and node";
constexpr const char *kReserveMarginalsMessage =
    "prepared accelerator marginal inference requires ReserveMarginals for "
    "this plan, state count, and batch capacity";

} // namespace

void SetLastError(const char *message) { g_last_error = message; }

} // namespace thmm

using thmm::Guard;
using thmm::Workspace;

// ======================================================================= C ABI
extern "C" {

const char *thmm_last_error(void) { return thmm::g_last_error.c_str(); }

thmm_status thmm_plan_create(const int64_t *parents, size_t count,
                             thmm_plan **out) {
  return Guard([&] {
    if (out == nullptr || (count != 0 && parents == nullptr))
      throw std::invalid_argument("plan arguments must not be null");
    auto plan = std::make_unique<btrc::Plan>(
        btrc::MakePlan(std::span<const std::int64_t>(parents, count)));
    *out = reinterpret_cast<thmm_plan *>(plan.release());
  });
}

thmm_status thmm_plan_create_many(const int64_t *parents, const size_t *offsets,
                                  size_t tree_count, unsigned threads, thmm_plan **out) {
  return Guard([&] {
    if (out == nullptr || offsets == nullptr || (tree_count != 0 && parents == nullptr))
      throw std::invalid_argument("plan arguments must not be null");
    for (size_t t = 0; t < tree_count; ++t) {
      out[t] = nullptr;
      if (offsets[t + 1] < offsets[t])
        throw std::invalid_argument("plan offsets must not decrease");
    }
    unsigned workers = threads != 0 ? threads : std::thread::hardware_concurrency();
    workers = static_cast<unsigned>(
        std::max<size_t>(1, std::min<size_t>(workers == 0 ? 1 : workers, tree_count)));
    // Trees are dealt round-robin; each worker keeps the first error it meets.
    std::vector<std::exception_ptr> errors(workers);
    std::vector<size_t> failed(workers, tree_count);
    const auto work = [&](unsigned w) {
      for (size_t t = w; t < tree_count; t += workers) {
        try {
          auto plan = std::make_unique<btrc::Plan>(btrc::MakePlan(std::span<const std::int64_t>(
              parents + offsets[t], offsets[t + 1] - offsets[t])));
          out[t] = reinterpret_cast<thmm_plan *>(plan.release());
        } catch (...) {
          errors[w] = std::current_exception();
          failed[w] = t;
          return;
        }
      }
    };
    std::vector<std::thread> pool;
    for (unsigned w = 1; w < workers; ++w)
      pool.emplace_back(work, w);
    work(0);
    for (std::thread &thread : pool)
      thread.join();
    // Report the error of the lowest failing tree and release everything.
    unsigned first = workers;
    for (unsigned w = 0; w < workers; ++w)
      if (errors[w] && (first == workers || failed[w] < failed[first]))
        first = w;
    if (first != workers) {
      for (size_t t = 0; t < tree_count; ++t) {
        delete reinterpret_cast<btrc::Plan *>(out[t]);
        out[t] = nullptr;
      }
      std::rethrow_exception(errors[first]);
    }
  });
}

void thmm_plan_destroy(thmm_plan *plan) {
  delete reinterpret_cast<btrc::Plan *>(plan);
}

thmm_status thmm_plan_get_info(const thmm_plan *plan, thmm_plan_info *out) {
  return Guard([&] {
    const btrc::Plan &p = thmm::AsPlan(plan);
    if (out == nullptr)
      throw std::invalid_argument("output must not be null");
    *out = {p.num_nodes(),
            p.num_edges(),
            p.num_branches(),
            p.num_compressions(),
            p.branch_combinations().size(),
            p.branch_absorptions().size(),
            p.primitive_batches().size(),
            p.rounds().size(),
            p.root()};
  });
}

thmm_status thmm_plan_get_arrays(const thmm_plan *plan, thmm_plan_arrays *out) {
  return Guard([&] {
    const btrc::Plan &p = thmm::AsPlan(plan);
    if (out == nullptr)
      throw std::invalid_argument("output must not be null");
    static_assert(sizeof(btrc::PrimitiveBatch) == 12);
    out->edge_parents = p.edge_parents().data();
    out->edge_children = p.edge_children().data();
    out->rakes = reinterpret_cast<const uint32_t *>(p.rakes().data());
    out->combinations =
        reinterpret_cast<const uint32_t *>(p.branch_combinations().data());
    out->absorptions =
        reinterpret_cast<const uint32_t *>(p.branch_absorptions().data());
    out->compressions = reinterpret_cast<const uint32_t *>(p.compressions().data());
    out->batches = reinterpret_cast<const uint32_t *>(p.primitive_batches().data());
  });
}

int thmm_available(void) {
  int count = 0;
  return cudaGetDeviceCount(&count) == cudaSuccess && count > 0 ? 1 : 0;
}

thmm_status thmm_device_description(int device, char *buffer, size_t size) {
  return Guard([&] {
    cudaDeviceProp properties{};
    thmm::Check(cudaGetDeviceProperties(&properties, device),
                "cudaGetDeviceProperties");
    const std::string text = std::string(properties.name) + " (compute " +
                             std::to_string(properties.major) + "." +
                             std::to_string(properties.minor) + ")";
    if (buffer == nullptr || size == 0)
      throw std::invalid_argument("description buffer must not be empty");
    std::snprintf(buffer, size, "%s", text.c_str());
  });
}

thmm_status thmm_workspace_create(thmm_workspace **out) {
  return Guard([&] {
    if (out == nullptr)
      throw std::invalid_argument("output must not be null");
    *out = reinterpret_cast<thmm_workspace *>(new Workspace());
  });
}

void thmm_workspace_destroy(thmm_workspace *workspace) {
  delete reinterpret_cast<Workspace *>(workspace);
}

thmm_status thmm_reserve(thmm_workspace *workspace, const thmm_plan *plan,
                         size_t states, size_t batch_capacity, int device,
                         uint32_t flags, uint32_t scalar) {
  return Guard([&] {
    thmm::AsWorkspace(workspace).ReserveBatch(thmm::AsPlan(plan), states,
                                              batch_capacity, device, flags,
                                              scalar, false, 0, {});
  });
}

thmm_status thmm_reserve_categorical(thmm_workspace *workspace,
                                     const thmm_plan *plan, size_t states,
                                     size_t batch_capacity, size_t categories,
                                     const uint32_t *observation_nodes,
                                     size_t observation_node_count, int device,
                                     uint32_t flags, uint32_t scalar) {
  return Guard([&] {
    if (observation_node_count != 0 && observation_nodes == nullptr)
      throw std::invalid_argument("observation nodes must not be null");
    thmm::AsWorkspace(workspace).ReserveBatch(
        thmm::AsPlan(plan), states, batch_capacity, device, flags, scalar, true,
        categories,
        std::span<const std::uint32_t>(observation_nodes, observation_node_count));
  });
}

thmm_status thmm_reserve_forest(thmm_workspace *workspace,
                                const thmm_plan *const *plans,
                                size_t tree_count, size_t states, int device,
                                uint32_t flags, uint32_t scalar) {
  return Guard([&] {
    if (plans == nullptr)
      throw std::invalid_argument("forest plans must not be null");
    thmm::AsWorkspace(workspace).ReserveForest(
        std::span<const btrc::Plan *const>(
            reinterpret_cast<const btrc::Plan *const *>(plans), tree_count),
        states, device, flags, scalar, false, 0, nullptr, nullptr);
  });
}

thmm_status thmm_reserve_forest_categorical(
    thmm_workspace *workspace, const thmm_plan *const *plans, size_t tree_count,
    size_t states, size_t categories, const uint32_t *observation_nodes,
    const size_t *observation_counts, int device, uint32_t flags,
    uint32_t scalar) {
  return Guard([&] {
    if (plans == nullptr || observation_counts == nullptr)
      throw std::invalid_argument("forest arrays must not be null");
    thmm::AsWorkspace(workspace).ReserveForest(
        std::span<const btrc::Plan *const>(
            reinterpret_cast<const btrc::Plan *const *>(plans), tree_count),
        states, device, flags, scalar, true, categories, observation_nodes,
        observation_counts);
  });
}

thmm_status thmm_inputs(thmm_workspace *workspace, size_t batch,
                        thmm_dense_input_view *out) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    ws.RequireReserved();
    ws.RequireStaging();
    if (ws.categorical)
      throw std::logic_error(
          "accelerator dense Inputs cannot be used after ReserveCategorical");
    ws.CheckBatch(batch, "input");
    *out = {ws.states,
            batch,
            ws.h_node_in.ptr,
            ws.NodesFor(batch) * ws.states,
            ws.h_edge_in.ptr,
            static_cast<size_t>(ws.edge_inputs * ws.states * ws.states)};
  });
}

thmm_status thmm_categorical_inputs(thmm_workspace *workspace, size_t batch,
                                    thmm_categorical_input_view *out) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (!ws.reserved || !ws.categorical)
      throw std::logic_error("accelerator Workspace::ReserveCategorical must "
                             "precede CategoricalInputs");
    ws.RequireStaging();
    ws.CheckBatch(batch, "categorical input");
    *out = {ws.states,
            batch,
            ws.categories,
            ws.observation_nodes.data(),
            ws.observation_nodes.size(),
            ws.h_observations.as<uint8_t>(),
            ws.ObservationsFor(batch),
            ws.h_root.ptr,
            ws.states,
            ws.h_emission.ptr,
            ws.categories * ws.states,
            ws.h_edge_in.ptr,
            static_cast<size_t>(ws.edge_inputs * ws.states * ws.states)};
  });
}

thmm_status thmm_uniforms(thmm_workspace *workspace, size_t batch, void **out,
                          size_t *count) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (!ws.reserved || !ws.sampling)
      throw std::logic_error(
          "accelerator Workspace::ReserveSampling must precede Uniforms");
    ws.RequireStaging();
    ws.CheckBatch(batch, "uniform");
    *out = ws.h_uniforms.ptr;
    *count = ws.NodesFor(batch);
  });
}

// ------------------------------------------------------------ dense calls
static thmm_status DensePartition(thmm_workspace *workspace,
                                  const thmm_dense_model *model, int operation,
                                  thmm_partition_result *out) {
  const auto wall_start = thmm::Clock::now();
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (model == nullptr || out == nullptr)
      throw std::invalid_argument("model and result must not be null");
    thmm::CheckDense(ws, *model, thmm::kReserveMessage, true);
    const auto outcome = ws.Run(operation, model->batch,
                                thmm::DenseUploads(ws, *model), wall_start);
    *out = {ws.h_values.ptr, ws.forest ? ws.capacity : model->batch, outcome.timings};
  });
}

thmm_status thmm_partition_function(thmm_workspace *workspace,
                                    const thmm_dense_model *model,
                                    thmm_partition_result *out) {
  return DensePartition(workspace, model, THMM_OP_PARTITION, out);
}

thmm_status thmm_log_partition_function(thmm_workspace *workspace,
                                        const thmm_dense_model *model,
                                        thmm_partition_result *out) {
  return DensePartition(workspace, model, THMM_OP_LOG_PARTITION, out);
}

thmm_status thmm_maximum_a_posteriori(thmm_workspace *workspace,
                                      const thmm_dense_model *model,
                                      thmm_maximum_result *out) {
  const auto wall_start = thmm::Clock::now();
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (model == nullptr || out == nullptr)
      throw std::invalid_argument("model and result must not be null");
    thmm::CheckDense(ws, *model, thmm::kReserveMaximumMessage, ws.maximum);
    const auto outcome = ws.Run(THMM_OP_MAXIMUM, model->batch,
                                thmm::DenseUploads(ws, *model), wall_start);
    const std::size_t items = ws.forest ? ws.capacity : model->batch;
    ws.RequireAllFinite(items, "the tree HMM has no positive-weight assignment");
    *out = {ws.h_values.ptr, items, ws.h_states.as<uint32_t>(),
            ws.NodesFor(model->batch), outcome.timings};
  });
}

thmm_status thmm_posterior_sample(thmm_workspace *workspace,
                                  const thmm_dense_model *model,
                                  const void *uniforms, size_t uniform_count,
                                  thmm_sample_result *out) {
  const auto wall_start = thmm::Clock::now();
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (model == nullptr || out == nullptr)
      throw std::invalid_argument("model and result must not be null");
    thmm::CheckDense(ws, *model, thmm::kReserveSamplingMessage, ws.sampling);
    auto uploads = thmm::DenseUploads(ws, *model);
    const auto uniform = thmm::UniformUpload(ws, model->batch, uniforms, uniform_count);
    uploads.insert(uploads.end(), uniform.begin(), uniform.end());
    const auto outcome = ws.Run(THMM_OP_SAMPLE, model->batch, uploads, wall_start);
    const std::size_t items = ws.forest ? ws.capacity : model->batch;
    thmm::CheckSamplingOutcome(ws, outcome, items);
    *out = {ws.h_states.as<uint32_t>(), ws.NodesFor(model->batch), outcome.timings};
  });
}

thmm_status thmm_posterior_marginals(thmm_workspace *workspace,
                                     const thmm_dense_model *model,
                                     thmm_marginal_result *out) {
  const auto wall_start = thmm::Clock::now();
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (model == nullptr || out == nullptr)
      throw std::invalid_argument("model and result must not be null");
    thmm::CheckDense(ws, *model, thmm::kReserveMarginalsMessage, ws.marginals);
    const auto outcome = ws.Run(THMM_OP_MARGINALS, model->batch,
                                thmm::DenseUploads(ws, *model), wall_start);
    const std::size_t items = ws.forest ? ws.capacity : model->batch;
    ws.RequireAllFinite(items, "the tree HMM has a nonpositive partition function");
    *out = {ws.h_values.ptr,
            items,
            ws.h_node_out.ptr,
            ws.NodesFor(model->batch) * ws.states,
            ws.h_edge_out.ptr,
            ws.EdgeOutFor(model->batch) * ws.states * ws.states,
            outcome.timings};
  });
}

// ------------------------------------------------------ categorical calls
static thmm_status CategoricalPartition(thmm_workspace *workspace,
                                        const thmm_categorical_model *model,
                                        int update, int operation,
                                        thmm_partition_result *out) {
  const auto wall_start = thmm::Clock::now();
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (model == nullptr || out == nullptr)
      throw std::invalid_argument("model and result must not be null");
    const auto uploads =
        thmm::CategoricalUploads(ws, *model, update, thmm::kReserveMessage, true);
    const auto outcome = ws.Run(operation, model->batch, uploads, wall_start);
    thmm::MarkResident(ws, model->batch, update);
    *out = {ws.h_values.ptr, ws.forest ? ws.capacity : model->batch, outcome.timings};
  });
}

thmm_status thmm_categorical_partition_function(
    thmm_workspace *workspace, const thmm_categorical_model *model, int update,
    thmm_partition_result *out) {
  return CategoricalPartition(workspace, model, update, THMM_OP_PARTITION, out);
}

thmm_status thmm_categorical_log_partition_function(
    thmm_workspace *workspace, const thmm_categorical_model *model, int update,
    thmm_partition_result *out) {
  return CategoricalPartition(workspace, model, update, THMM_OP_LOG_PARTITION, out);
}

thmm_status thmm_categorical_maximum_a_posteriori(
    thmm_workspace *workspace, const thmm_categorical_model *model, int update,
    thmm_maximum_result *out) {
  const auto wall_start = thmm::Clock::now();
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (model == nullptr || out == nullptr)
      throw std::invalid_argument("model and result must not be null");
    const auto uploads = thmm::CategoricalUploads(
        ws, *model, update, thmm::kReserveMaximumMessage, ws.maximum);
    const auto outcome = ws.Run(THMM_OP_MAXIMUM, model->batch, uploads, wall_start);
    const std::size_t items = ws.forest ? ws.capacity : model->batch;
    ws.RequireAllFinite(items, "the tree HMM has no positive-weight assignment");
    thmm::MarkResident(ws, model->batch, update);
    *out = {ws.h_values.ptr, items, ws.h_states.as<uint32_t>(),
            ws.NodesFor(model->batch), outcome.timings};
  });
}

thmm_status thmm_categorical_posterior_sample(
    thmm_workspace *workspace, const thmm_categorical_model *model,
    const void *uniforms, size_t uniform_count, int update,
    thmm_sample_result *out) {
  const auto wall_start = thmm::Clock::now();
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (model == nullptr || out == nullptr)
      throw std::invalid_argument("model and result must not be null");
    auto uploads = thmm::CategoricalUploads(
        ws, *model, update, thmm::kReserveSamplingMessage, ws.sampling);
    const auto uniform = thmm::UniformUpload(ws, model->batch, uniforms, uniform_count);
    uploads.insert(uploads.end(), uniform.begin(), uniform.end());
    const auto outcome = ws.Run(THMM_OP_SAMPLE, model->batch, uploads, wall_start);
    const std::size_t items = ws.forest ? ws.capacity : model->batch;
    thmm::CheckSamplingOutcome(ws, outcome, items);
    thmm::MarkResident(ws, model->batch, update);
    *out = {ws.h_states.as<uint32_t>(), ws.NodesFor(model->batch), outcome.timings};
  });
}

thmm_status thmm_categorical_posterior_marginals(
    thmm_workspace *workspace, const thmm_categorical_model *model, int update,
    thmm_marginal_result *out) {
  const auto wall_start = thmm::Clock::now();
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (model == nullptr || out == nullptr)
      throw std::invalid_argument("model and result must not be null");
    const auto uploads = thmm::CategoricalUploads(
        ws, *model, update, thmm::kReserveMarginalsMessage, ws.marginals);
    const auto outcome = ws.Run(THMM_OP_MARGINALS, model->batch, uploads, wall_start);
    const std::size_t items = ws.forest ? ws.capacity : model->batch;
    ws.RequireAllFinite(items, "the tree HMM has a nonpositive partition function");
    thmm::MarkResident(ws, model->batch, update);
    *out = {ws.h_values.ptr,
            items,
            ws.h_node_out.ptr,
            ws.NodesFor(model->batch) * ws.states,
            ws.h_edge_out.ptr,
            ws.EdgeOutFor(model->batch) * ws.states * ws.states,
            outcome.timings};
  });
}

// ------------------------------------------------------- device-only path
thmm_status thmm_enqueue(thmm_workspace *workspace, int operation,
                         uint64_t *nodes_out) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (!ws.reserved || !ws.has_run)
      throw std::logic_error(
          "thmm_enqueue needs inputs left resident by a prepared call");
    if (operation < THMM_OP_PARTITION || operation > THMM_OP_MARGINALS)
      throw std::invalid_argument("unknown operation");
    if ((operation == THMM_OP_MAXIMUM && !ws.maximum) ||
        (operation == THMM_OP_SAMPLE && !ws.sampling) ||
        (operation == THMM_OP_MARGINALS && !ws.marginals))
      throw std::invalid_argument("operation was not reserved");
    thmm::Check(cudaSetDevice(ws.device), "cudaSetDevice");
    ws.EnqueueGraph(operation, ws.last_batch);
    if (nodes_out != nullptr)
      *nodes_out = ws.NodesFor(ws.last_batch);
  });
}

thmm_status thmm_device_buffers_get(thmm_workspace *workspace, thmm_device_buffers *out) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (out == nullptr)
      throw std::invalid_argument("output must not be null");
    ws.RequireReserved();
    *out = thmm_device_buffers{};
    out->node_potentials = ws.node_in.ptr;
    out->edge_potentials = ws.edge_in.ptr;
    out->observations = ws.observations.as<std::uint8_t>();
    out->root_potential = ws.root_potential.ptr;
    out->emission_potentials = ws.emission.ptr;
    out->uniforms = ws.uniforms.ptr;
    out->values = ws.values.ptr;
    out->node_marginals = ws.node_out.ptr;
    out->edge_marginals = ws.edge_out.ptr;
    out->states = ws.states_out.as<std::uint32_t>();
  });
}

thmm_status thmm_device_inputs_ready(thmm_workspace *workspace, size_t batch) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    ws.RequireReserved();
    ws.CheckBatch(batch, "device input");
    thmm::Check(cudaSetDevice(ws.device), "cudaSetDevice");
    if (ws.categorical)
      ws.OrderObservations(ws.stream);
    ws.resident_observation_batch = batch;
    ws.resident_factors = true;
    ws.last_batch = batch;
    ws.has_run = true;
  });
}

thmm_status thmm_autotune(thmm_workspace *workspace, int operation, int repeats,
                          thmm_tuning *out) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (!ws.reserved || !ws.has_run)
      throw std::logic_error(
          "thmm_autotune needs inputs left resident by a prepared call");
    if (operation < THMM_OP_PARTITION || operation > THMM_OP_MARGINALS)
      throw std::invalid_argument("unknown operation");
    if ((operation == THMM_OP_MAXIMUM && !ws.maximum) ||
        (operation == THMM_OP_SAMPLE && !ws.sampling) ||
        (operation == THMM_OP_MARGINALS && !ws.marginals))
      throw std::invalid_argument("operation was not reserved");
    if (repeats < 1)
      throw std::invalid_argument("autotune needs at least one timed repeat");
    thmm::Check(cudaSetDevice(ws.device), "cudaSetDevice");
    const thmm_tuning tuning = ws.Autotune(operation, repeats);
    if (out != nullptr)
      *out = tuning;
  });
}

thmm_status thmm_get_tuning(const thmm_workspace *workspace, thmm_tuning *out) {
  return Guard([&] {
    if (workspace == nullptr || out == nullptr)
      throw std::invalid_argument("workspace and result must not be null");
    *out = reinterpret_cast<const Workspace *>(workspace)->CurrentTuning();
  });
}

thmm_status thmm_set_tuning(thmm_workspace *workspace, const thmm_tuning *tuning) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (tuning == nullptr)
      throw std::invalid_argument("tuning must not be null");
    if (!ws.reserved)
      throw std::logic_error("thmm_set_tuning needs a reserved workspace");
    if (tuning->team_threshold == 0)
      throw std::invalid_argument("team threshold must be positive");
    ws.ApplyTuning(*tuning);
  });
}

void *thmm_workspace_stream(thmm_workspace *workspace) {
  return workspace == nullptr
             ? nullptr
             : static_cast<void *>(reinterpret_cast<Workspace *>(workspace)->stream);
}

thmm_status thmm_workspace_synchronize(thmm_workspace *workspace) {
  return Guard([&] {
    Workspace &ws = thmm::AsWorkspace(workspace);
    if (ws.stream != nullptr)
      thmm::Check(cudaStreamSynchronize(ws.stream), "cudaStreamSynchronize");
  });
}

thmm_status thmm_wait_timeout_check(int device, uint64_t cycles) {
  return Guard([&] {
    if (cycles == 0 || cycles > (1ull << 34))
      throw std::invalid_argument("wait budget must be between 1 and 2^34 cycles");
    thmm::Check(cudaSetDevice(device), "cudaSetDevice");
    thmm::DeviceBuffer error;
    error.Allocate(sizeof(std::uint32_t));
    thmm::Check(cudaMemset(error.ptr, 0, sizeof(std::uint32_t)), "cudaMemset");
    thmm::Check(thmm::LaunchWaitTimeoutCheck(error.as<std::uint32_t>(),
                                             static_cast<long long>(cycles), nullptr),
                "wait check launch");
    std::uint32_t bits = 0;
    thmm::Check(cudaMemcpy(&bits, error.ptr, sizeof bits, cudaMemcpyDeviceToHost),
                "wait check result");
    if (bits & thmm::kErrorTensorTimeout)
      throw std::runtime_error("tree-HMM accelerator tensor-core wait timed out");
  });
}

uint64_t thmm_workspace_launches(const thmm_workspace *workspace) {
  return workspace == nullptr
             ? 0
             : reinterpret_cast<const Workspace *>(workspace)->launches;
}

} // extern "C"
