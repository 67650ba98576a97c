// Device-side plan format shared by the host compiler (program.cc) and the
// kernels (engine.cuh).
//
// A btrc::Plan is compiled into a *program*: its primitive batches become
// steps, and every operand is resolved statically. In particular each path
// operand names a *path version*: version v < E is input edge v, and version
// kFlag | t is the output of compression t. The reference instead overwrites
// the compression's left path in place and snapshots tapes
// (src/inference.cc:297-324, src/gpu_backend_impl.inc:459-526); versioned
// paths make every value the reverse sweep needs addressable without tapes.
#ifndef THMM_ENGINE_H_
#define THMM_ENGINE_H_

#include <cstddef>
#include <cstdint>

namespace thmm {

inline constexpr std::uint32_t kFlag = 0x80000000u;
inline constexpr std::uint32_t kMask = 0x7fffffffu;

enum StepKind : std::uint32_t {
  kStepRake = 0,
  kStepCombine = 1,
  kStepAbsorb = 2,
  kStepCompress = 3,
  kStepGather = 4,
};

// Operation records (all indices are program-local):
// Rake op (uint4):     path version, leaf (kFlag: value stored), parent,
//                      observation slot of the leaf (kNone if unobserved).
//                      The branch is implicit: rake i of the program fills
//                      branch i (btrc numbers branches in rake order).
// Combine op (uint2):  destination branch, source branch
// Absorb op (uint4):   node (kFlag: first absorption, start from the input
//                      factor), branch, observation slot of the node, 0
// Compress op (uint4): left version, middle (kFlag: stored), right version,
//                      observation slot of the middle node. The tape is
//                      implicit: compression i of the program writes tape i.
// Compress ends (uint2): parent, child (read only by MAP/sample expansion).
// Gather op (uint4):   node (kFlag: first absorption), observation slot of
//                      the node, first rake, rake count. Used only by the
//                      sum-product forward: one round's rakes, branch
//                      combinations and absorption into one parent fused into
//                      a single operation (the rakes of a round are stored
//                      grouped by parent so a gather's rakes are contiguous).
//
// A program has two step lists over the same operation arrays: the plan's
// own primitive batches (MAP, sampling and the reverse sweep) and the fused
// sum-product forward list (gather and compress steps).
inline constexpr std::uint32_t kNone = 0xffffffffu;

struct alignas(16) DevProgram {
  std::uint32_t step_begin;
  std::uint32_t step_count;
  std::uint32_t num_nodes;
  std::uint32_t num_edges;
  std::uint32_t num_rakes;
  std::uint32_t num_compressions;
  std::uint32_t root;     // kFlag: the root has a stored (absorbed) value
  std::uint32_t root_obs; // observation slot of the root, kNone if none
  std::uint32_t rake_base;     // first rake op of the program
  std::uint32_t compress_base; // first compress op of the program
  std::uint32_t fused_begin;   // fused sum-product forward steps
  std::uint32_t fused_count;
};

struct alignas(16) DevStep {
  std::uint32_t kind;
  std::uint32_t offset;
  std::uint32_t count;
  std::uint32_t aux_offset; // gather steps: the round's rakes
  std::uint32_t aux_count;
  std::uint32_t pad0;
  std::uint32_t pad1;
  std::uint32_t pad2;
};

// One tree instance: a program applied to one batch item (or one tree of a
// forest). Offsets are in elements of the arrays they index.
struct alignas(16) DevInstance {
  std::uint32_t program;
  std::uint32_t pad;
  std::uint64_t node_base;     // node inputs/outputs: (node_base + node) * K
  std::uint64_t edge_in_base;  // edge inputs: (edge_in_base + edge) * K * K
  std::uint64_t edge_out_base; // edge marginals: (edge_out_base + edge) * K*K
  std::uint64_t obs_base;      // observation bytes
  std::uint64_t scratch_base;  // compute-typed scratch
  std::uint64_t byte_base;     // byte scratch (choices, exponents)
};

enum EngineMode : std::uint32_t {
  kModeLinear = 0, // partition / log partition / marginals
  kModeMaximum = 1,
  kModeSample = 2,
};

enum ErrorBits : std::uint32_t {
  kErrorInvalidUniform = 1u,
  kErrorEmptyConditional = 2u,
  kErrorTensorTimeout = 4u, // a tensor-core completion wait gave up
};

struct EngineArgs {
  const DevProgram *programs;
  const DevStep *steps;
  const void *rakes;    // uint4
  const void *combines; // uint2
  const void *absorbs;  // uint4
  const void *compress; // uint4
  const void *compress_ends; // uint2
  const void *gathers;       // uint4
  const DevInstance *instances;
  const std::uint32_t *big_items; // instances run by a whole CTA
  std::uint32_t big_count;
  const std::uint32_t *small_items; // instances run by one warp
  std::uint32_t small_count;
  std::uint32_t *queue; // [2] work counters, zeroed before each launch
  std::uint32_t *error; // [1] ErrorBits
  const void *node_in;  // dense node factors
  const std::uint8_t *observations;
  const void *root_potential;
  const void *emission;
  std::uint32_t categories;
  std::uint32_t categorical;
  const void *edge_in;
  std::uint32_t states;
  std::uint32_t reverse; // linear mode: run the marginal (adjoint) sweep
  std::uint32_t raw;     // linear mode: output exp(log Z)
  void *scratch;
  std::uint8_t *bytes;
  void *values;   // [instance]: log Z, Z or MAP log weight
  void *node_out; // node marginals
  void *edge_out; // edge marginals
  std::uint32_t *states_out;
  const void *uniforms;
  std::uint32_t bf16; // wide-state engine: BF16 tensor products (the BF16 tier)
};

// Scratch sizes of one instance, in compute elements and bytes.
struct ScratchSize {
  std::uint64_t elements;
  std::uint64_t bytes;
};

inline ScratchSize InstanceScratch(std::uint64_t nodes, std::uint64_t rakes,
                                   std::uint64_t compressions,
                                   std::uint64_t states, EngineMode mode,
                                   bool reverse) {
  const std::uint64_t matrix = states * states;
  ScratchSize size{};
  size.elements = nodes * states + rakes * states + compressions * matrix;
  if (mode == kModeLinear && reverse)
    size.elements += compressions * matrix; // adjoints of compressed paths
  if (mode == kModeMaximum)
    size.bytes = rakes * states + compressions * matrix; // choice tapes
  size.bytes = (size.bytes + 15) & ~std::uint64_t{15};
  size.elements = (size.elements + 3) & ~std::uint64_t{3};
  return size;
}

} // namespace thmm

#endif // THMM_ENGINE_H_
