// Level-synchronous phase schedule of the sum-product calls (every state
// count up to 128).
//
// The per-tree engine (engine.cuh) contracts one tree per team and walks the
// tree's plan step by step with a team barrier in between; a tree has 20-50
// such steps but most of its work sits in the first rounds (on the uneven
// K=4 forest, round 0 eliminates 69 % of all nodes and rounds 0-2 eliminate
// 95 %). The phase schedule instead runs round r of EVERY instance in one
// grid-wide launch: the forward sweep is the launch sequence
//   gather(0), compress(0), gather(1), compress(1), ..., finish
// and the adjoint sweep
//   compress-reverse(R-1), rake-reverse(R-1), ..., compress-reverse(0),
//   rake-reverse(0),
// one thread per operation, with no barriers inside a launch. The
// operations of one round of one tree are independent (a btrc primitive
// batch), and different trees never share an operand, so each launch is
// embarrassingly parallel.
//
// Every operand is addressed by an absolute index resolved on the host, so
// the kernels read no instance or program table. The power-of-two exponents
// that the per-tree engine sums per thread travel with the stored values
// instead (one int32 per stored node value and per compressed path), so the
// root's exponent is log2 of the tree's scale; the floating-point arithmetic
// of every operation is the per-tree engine's, operation for operation, so
// both schedules give bit-identical results.
#ifndef THMM_PHASE_H_
#define THMM_PHASE_H_

#include <cstddef>
#include <cstdint>
#include <span>
#include <vector>

#include <cuda_runtime.h>

#include "engine.h"
#include "program_builder.h"

namespace thmm {

// Phase kinds, in launch order within a round.
enum PhaseKind : int {
  kPhaseGather = 0,          // fused rakes + absorption into each parent
  kPhaseCompress = 1,        // compressions of the round
  kPhaseFinish = 2,          // log Z (and the root marginal) per instance
  kPhaseRakeReverse = 3,     // adjoint of the round's rakes
  kPhaseCompressReverse = 4, // adjoint of the round's compressions
  kPhaseTailForward = 5,     // rounds >= the tail round, one warp per tree
  kPhaseTailReverse = 6,     // their adjoint, one warp per tree
};

// The last rounds of a forest hold few operations (rounds 5 and later of the
// uneven K=4 forest hold 0.4 % of them) but one launch each, and a launch
// costs microseconds however little it does. From the tail round on, the
// schedule can switch to one warp per tree that walks the tree's remaining
// rounds with a warp barrier between steps (the same operation functions,
// so the same bits). Tail records:
//   tail item   uint4: instance, first tail round entry, tail rounds, 0
//   tail round  uint4: first gather, gathers, first compression, compressions
//   tail rakes  uint2: first rake, rakes (of the same round)

// Records (absolute indices; kFlag marks a stored value / a compressed path):
//  rake     uint4: path (edge-out index, or kFlag | global compression),
//                  leaf node (kFlag: stored), leaf observation (kNone), parent node
//  gather   uint4: node (kFlag: first absorption, start from the input factor),
//                  node observation, first rake, rake count | kRootBit (node is a root)
//  compress uint4: left path, middle node (kFlag: stored), right path,
//                  middle observation; compression i writes path i
//  root     uint2: root node (kFlag: stored), root observation
// Observation fields index the phase-ordered copy of the observations
// (PhasePlan::observation_order), not the caller's array.
inline constexpr std::uint32_t kRootBit = 0x40000000u;
inline constexpr std::uint32_t kCountMask = 0x3fffffffu;

struct PhaseArgs {
  const uint4 *rakes;
  const uint4 *gathers;
  const uint4 *compress;
  const uint2 *roots;
  std::uint32_t offset; // first operation (or instance, for finish) of the launch
  std::uint32_t count;  // operations (instances) of the launch
  const void *node_in;
  const std::uint8_t *observations;
  const void *root_potential;
  const void *emission;
  std::uint32_t categories;
  std::uint32_t categorical;
  const void *edge_in;
  std::uint32_t edge_modulus; // > 0: shared edge input, row = path % edge_modulus
  std::uint32_t states;
  void *nodes;        // [node][K] stored (normalised) node values, compute type
  int *node_exp;      // [node] their power-of-two exponents
  void *comps;        // [compression][K][K] compressed paths, compute type
  int *comp_exp;      // [compression]
  void *comp_mu;      // [compression][K][K] adjoints of compressed paths
  void *values;       // [instance] log Z or Z
  void *node_out;     // node marginals
  void *edge_out;     // edge marginals
  std::uint32_t raw;     // output exp(log Z)
  std::uint32_t reverse; // finish: also write the root marginal
  const uint4 *tail_items;
  const uint4 *tail_rounds;
  const uint2 *tail_rakes;
  // Shared-topology layout only (BatchPhaseKernel): items [first_item,
  // first_item + items) of a batch whose stored objects are `item_stride`
  // items apart, each with item_nodes nodes and item_edges edges.
  std::uint32_t batch;
  std::uint32_t first_item;
  std::uint32_t items;
  std::uint64_t item_stride;
  std::uint64_t item_nodes;
  std::uint64_t item_edges;
  // Wide-state kinds (32 < K <= 128) only: the error word (tensor-core wait
  // time-outs) and the BF16 product tier.
  std::uint32_t *error;
  std::uint32_t bf16;
};

// Operation counts of one program per round and kind.
struct ProgramRounds {
  std::uint32_t rounds = 0;
  std::vector<std::uint32_t> gathers, rakes, compressions; // [round]
};

// The phase schedule of a workspace: per round, the records of every
// instance, instance-major (instance i's operations of a round are
// contiguous and precede instance i+1's), so a contiguous instance range
// is a contiguous operation range in every phase.
struct PhasePlan {
  bool enabled = false;
  std::uint32_t rounds = 0;
  std::vector<Uint4> rakes, gathers, compress;
  std::vector<Uint2> roots;
  // First operation of each round in the global arrays ([rounds + 1]).
  std::vector<std::uint64_t> rake_base, gather_base, compress_base;
  // Per-program round counts and each instance's program, to locate the
  // operations of an instance range (OpRange).
  std::vector<ProgramRounds> program_rounds;
  std::vector<std::uint32_t> instance_program;
  std::uint64_t total_compressions = 0;
  // Caller observation index of each slot of the phase-ordered copy.
  std::vector<std::uint32_t> observation_order;

  // [first, last) operations of round `round` and kind (gather, rake or
  // compress) that belong to instances [a, b).
  std::pair<std::uint64_t, std::uint64_t> OpRange(int kind, std::uint32_t round,
                                                  std::uint32_t a, std::uint32_t b) const;

  // Tail records (see kPhaseTailForward) for rounds >= `tail_round`, over
  // the instances with more rounds than that, in instance order.
  struct Tail {
    std::vector<Uint4> items, rounds;
    std::vector<Uint2> rakes;
  };
  Tail BuildTail(std::uint32_t tail_round) const;
  // Default tail round: the first round with fewer than `ops` gathers and
  // compressions over all instances.
  std::uint32_t AutoTailRound(std::uint64_t ops) const;
};

struct PhaseInstance {
  std::uint32_t program;
  std::uint64_t node_base, edge_out_base, obs_base;
};

// Builds the phase schedule of `instances` over the compiled `set`. Returns
// a disabled plan when an index would not fit the 31-bit record fields or a
// tree is large enough for its exponent sum to leave int32 range.
struct ProgramSet;
PhasePlan BuildPhasePlan(const ProgramSet &set, std::span<const PhaseInstance> instances,
                         std::uint64_t total_nodes, std::uint64_t total_edges_out,
                         unsigned threads);

// Launches one phase (or reports its occupancy when blocks_per_sm is
// non-null). scalar_bytes: 4 or 8 (input/output type); compute_f64: FP64
// arithmetic. Padded state count 4 (K <= 4) runs one thread per operation
// (phase_engine.cuh); 4 < K <= 32 (forest layout, no tail kinds) one lane
// group per operation (phase_groups.cuh); 32 < K <= 128 (FP32 only, forest
// layout, no tail kinds) one CTA per operation (wide_phase.cuh).
cudaError_t LaunchPhase(int scalar_bytes, bool compute_f64, int kind, const PhaseArgs &args,
                        cudaStream_t stream, int *blocks_per_sm);
cudaError_t LaunchWidePhase(int kind, const PhaseArgs &args, cudaStream_t stream,
                            int *blocks_per_sm);
// 4 < K <= 32: one lane group per operation (phase_groups.cuh), per padded
// state count and arithmetic type.
#define THMM_GROUP_PHASE_LAUNCHER(name)                                                    \
  cudaError_t name(int scalar_bytes, int kind, const PhaseArgs &args, cudaStream_t stream, \
                   int *blocks_per_sm);
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase8F32)
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase8F64)
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase16F32)
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase16F64)
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase32F32)
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase32F64)
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase20F32)
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase24F32)
THMM_GROUP_PHASE_LAUNCHER(LaunchGroupPhase28F32)
#undef THMM_GROUP_PHASE_LAUNCHER

// The phase-ordered copy of the observations: ordered[j * items + b] =
// observations[b * per_item + order[j]] for j < count, b < items (a forest:
// items = 1, per_item = 0).
cudaError_t LaunchObservationGather(const std::uint8_t *observations,
                                    const std::uint32_t *order, std::uint8_t *ordered,
                                    std::uint64_t count, std::uint64_t items,
                                    std::uint64_t per_item, cudaStream_t stream);

} // namespace thmm

#endif // THMM_PHASE_H_
