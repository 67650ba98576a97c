/* C ABI of the GB300 tree-HMM accelerator (libthmm_gb300.so).
 *
 * This is the drop-in boundary for the reference's batched accelerator path,
 * `tree_hmm::cuda` (include/tree_hmm/detail/gpu_backend_api.inc:1-142 and its
 * implementation src/gpu_backend_impl.inc:1636-3130). Every entry point below
 * names the reference declaration it replaces. The C++ API with the
 * reference's exact types and overloads is the header-only layer
 * include/tree_hmm/gb300.h, built on these functions.
 *
 * Conventions
 *   - Plain pointers and sizes only. Floating-point buffers are `void *` in the
 *     workspace's scalar width (THMM_SCALAR_F32 = float, THMM_SCALAR_F64 =
 *     double), the reference's compile-time tree_hmm::Scalar.
 *   - Every function returns a thmm_status. A non-zero status corresponds to
 *     the C++ exception type the reference throws in the same situation; the
 *     message is available from thmm_last_error() on the calling thread.
 *   - Result pointers refer to workspace-owned pinned host memory and stay
 *     valid until the workspace is reserved again or destroyed
 *     (include/tree_hmm/accelerator.h:113-114).
 *   - A workspace is not thread-safe; separate workspaces are independent.
 *     Every call is synchronous, like the reference (src/gpu_backend_impl.inc:
 *     2376), except thmm_enqueue.
 */
#ifndef THMM_GB300_H_
#define THMM_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  THMM_OK = 0,
  THMM_INVALID_ARGUMENT = 1, /* std::invalid_argument */
  THMM_LOGIC_ERROR = 2,      /* std::logic_error */
  THMM_DOMAIN_ERROR = 3,     /* std::domain_error */
  THMM_LENGTH_ERROR = 4,     /* std::length_error */
  THMM_RUNTIME_ERROR = 5,    /* std::runtime_error (CUDA runtime failure) */
} thmm_status;

enum {
  THMM_SCALAR_F32 = 4,
  THMM_SCALAR_F64 = 8,
};

/* Reservation flags: which recovery tapes the workspace keeps
 * (gpu_backend_api.inc:29-46). 0 reserves likelihood only. */
enum {
  THMM_RESERVE_MAXIMUM = 1u,
  THMM_RESERVE_SAMPLING = 2u,
  THMM_RESERVE_MARGINALS = 4u,
  /* Extension: inputs and results stay on the device. No pinned host staging
   * is allocated; Inputs/CategoricalInputs/Uniforms and the prepared calls
   * raise THMM_LOGIC_ERROR. Write inputs through thmm_device_buffers_get,
   * then thmm_device_inputs_ready and thmm_enqueue. */
  THMM_RESERVE_DEVICE_ONLY = 8u,
  /* Extension: run the sum-product paths (partition, log partition,
   * marginals) in FP64 instead of the default FP32 with exact power-of-two
   * scaling. MAP and sampling always compute in the scalar width. */
  THMM_COMPUTE_F64 = 0x100u,
  /* Extension: the BF16 tier of the tensor-core engine (more than 32 states):
   * compress products and their adjoint products in one pass of BF16
   * operands with FP32 accumulation, instead of the default 3xTF32 (FP32
   * accuracy). About 8 significant bits per operand: faster tensor-core
   * work, looser results (against FP64 on lognormal(0, 2) factors, log Z
   * within about 1.5e-5 relative and marginals within about 5e-3, where the
   * default tier gives 1e-6 and 1e-5). */
  THMM_COMPUTE_BF16 = 0x200u,
};

/* tree_hmm::CategoricalInputUpdate (include/tree_hmm/accelerator.h:89-93). */
enum {
  THMM_UPDATE_ALL = 0,
  THMM_UPDATE_FACTORS = 1,
  THMM_UPDATE_NONE = 2,
};

/* Operations for thmm_enqueue. */
enum {
  THMM_OP_PARTITION = 0,
  THMM_OP_LOG_PARTITION = 1,
  THMM_OP_MAXIMUM = 2,
  THMM_OP_SAMPLE = 3,
  THMM_OP_MARGINALS = 4,
};

/* Message of the last failing call on this thread ("" if none). */
const char *thmm_last_error(void);

/* ---------------------------------------------------------------- plans -- */
/* Opaque handle; in C++ it is exactly a btrc::Plan (include/btrc/plan.h). */
typedef struct thmm_plan thmm_plan;

typedef struct {
  size_t num_nodes;
  size_t num_edges;
  size_t num_branches;
  size_t num_compressions;
  size_t num_combinations;
  size_t num_absorptions;
  size_t num_batches;
  size_t num_rounds;
  uint32_t root;
} thmm_plan_info;

/* Raw operation arrays of a plan; pointers stay valid while the plan lives.
 * Layouts: rakes [n][4] (edge, leaf, branch, parent); combinations [n][3]
 * (destination, source, parent); absorptions [n][3] (parent, branch, round);
 * compressions [n][6] (left_edge, middle, right_edge, tape, parent, child);
 * batches [n][3] (primitive 0..3, offset, count). */
typedef struct {
  const uint32_t *edge_parents;
  const uint32_t *edge_children;
  const uint32_t *rakes;
  const uint32_t *combinations;
  const uint32_t *absorptions;
  const uint32_t *compressions;
  const uint32_t *batches;
} thmm_plan_arrays;

/* btrc::MakePlan(parents) (consumed at tests/accelerator_test.h:19-20). */
thmm_status thmm_plan_create(const int64_t *parents, size_t count,
                             thmm_plan **out);
/* Extension (no reference counterpart): the plans of `tree_count` trees at
 * once, built on `threads` host threads (0: all hardware threads). Tree t's
 * parent array is parents[offsets[t] .. offsets[t + 1]). On error no plan is
 * returned (every out[t] is null) and the status is that of the lowest
 * failing tree, as thmm_plan_create would report it. */
thmm_status thmm_plan_create_many(const int64_t *parents, const size_t *offsets,
                                  size_t tree_count, unsigned threads, thmm_plan **out);
void thmm_plan_destroy(thmm_plan *plan);
thmm_status thmm_plan_get_info(const thmm_plan *plan, thmm_plan_info *out);
thmm_status thmm_plan_get_arrays(const thmm_plan *plan, thmm_plan_arrays *out);

/* -------------------------------------------------------------- devices -- */
/* tree_hmm::cuda::Available() (gpu_backend_api.inc:1;
 * src/gpu_backend_impl.inc:1779-1782). */
int thmm_available(void);
/* tree_hmm::cuda::DeviceDescription(device) (gpu_backend_api.inc:2;
 * src/gpu_backend_impl.inc:1784-1797). Writes a NUL-terminated string. */
thmm_status thmm_device_description(int device, char *buffer, size_t size);

/* ----------------------------------------------------------- workspaces -- */
typedef struct thmm_workspace thmm_workspace;

/* Workspace() / ~Workspace() (gpu_backend_api.inc:4-14). */
thmm_status thmm_workspace_create(thmm_workspace **out);
void thmm_workspace_destroy(thmm_workspace *workspace);

/* Reserve / ReserveMaximum / ReserveSampling / ReserveMarginals
 * (gpu_backend_api.inc:17-21,29-31,36-37,43-44; src/gpu_backend_impl.inc:
 * 1803-1966,2021-2063). `flags` selects the variant. */
thmm_status thmm_reserve(thmm_workspace *workspace, const thmm_plan *plan,
                         size_t states, size_t batch_capacity, int device,
                         uint32_t flags, uint32_t scalar);

/* ReserveCategorical and its Maximum / Sampling / Marginals variants
 * (gpu_backend_api.inc:23-27,32-35,38-42,45-48; src/gpu_backend_impl.inc:
 * 1978-2019). */
thmm_status thmm_reserve_categorical(thmm_workspace *workspace,
                                     const thmm_plan *plan, size_t states,
                                     size_t batch_capacity, size_t categories,
                                     const uint32_t *observation_nodes,
                                     size_t observation_node_count, int device,
                                     uint32_t flags, uint32_t scalar);

/* Extension (no reference counterpart: the reference batch shares one
 * topology, include/tree_hmm/accelerator.h:13-23). A forest of `tree_count`
 * independent trees, each with its own plan and its own edge factors, run by
 * the same persistent launches. Node and edge arrays are the per-tree arrays concatenated in
 * tree order. */
thmm_status thmm_reserve_forest(thmm_workspace *workspace,
                                const thmm_plan *const *plans,
                                size_t tree_count, size_t states, int device,
                                uint32_t flags, uint32_t scalar);
/* Categorical forest: `observation_nodes` holds each tree's strictly
 * increasing observed nodes back to back, `observation_counts[t]` of them for
 * tree t. The root and emission factors are shared by the forest. */
thmm_status thmm_reserve_forest_categorical(
    thmm_workspace *workspace, const thmm_plan *const *plans, size_t tree_count,
    size_t states, size_t categories, const uint32_t *observation_nodes,
    const size_t *observation_counts, int device, uint32_t flags,
    uint32_t scalar);

/* Pinned staging storage (Inputs / CategoricalInputs / Uniforms,
 * gpu_backend_api.inc:52-59; src/gpu_backend_impl.inc:2065-2150).
 * For a forest, `batch` must equal the tree count. */
typedef struct {
  size_t states;
  size_t batch;
  void *node_potentials; /* [batch, node, state] */
  size_t node_count;
  void *edge_potentials; /* [edge, parent, child] */
  size_t edge_count;
} thmm_dense_input_view;

typedef struct {
  size_t states;
  size_t batch;
  size_t categories;
  const uint32_t *observation_nodes;
  size_t observation_node_count;
  uint8_t *observations; /* [batch, observation node] */
  size_t observation_count;
  void *root_potential; /* [state] */
  size_t root_count;
  void *emission_potentials; /* [category, state] */
  size_t emission_count;
  void *edge_potentials; /* [edge, parent, child] */
  size_t edge_count;
} thmm_categorical_input_view;

thmm_status thmm_inputs(thmm_workspace *workspace, size_t batch,
                        thmm_dense_input_view *out);
thmm_status thmm_categorical_inputs(thmm_workspace *workspace, size_t batch,
                                    thmm_categorical_input_view *out);
thmm_status thmm_uniforms(thmm_workspace *workspace, size_t batch, void **out,
                          size_t *count);

/* tree_hmm::BatchedModelView (include/tree_hmm/accelerator.h:13-23). For a
 * forest workspace `plan` is ignored and `batch` is the tree count. */
typedef struct {
  const thmm_plan *plan;
  size_t states;
  size_t batch;
  const void *node_potentials;
  size_t node_count;
  const void *edge_potentials;
  size_t edge_count;
} thmm_dense_model;

/* tree_hmm::BatchedCategoricalModelView (include/tree_hmm/accelerator.h:
 * 41-58). */
typedef struct {
  const thmm_plan *plan;
  size_t states;
  size_t batch;
  size_t categories;
  const uint32_t *observation_nodes;
  size_t observation_node_count;
  const uint8_t *observations;
  size_t observation_count;
  const void *root_potential;
  size_t root_count;
  const void *emission_potentials;
  size_t emission_count;
  const void *edge_potentials;
  size_t edge_count;
} thmm_categorical_model;

/* tree_hmm::AcceleratorTimings (include/tree_hmm/accelerator.h:98-111). */
typedef struct {
  double upload_ms;
  double kernel_ms;
  double download_ms;
  double wall_ms;
} thmm_timings;

/* PartitionView (accelerator.h:115-118). */
typedef struct {
  const void *values;
  size_t count;
  thmm_timings timings;
} thmm_partition_result;

/* BatchedMaximumAssignmentView (accelerator.h:123-127). */
typedef struct {
  const void *log_weights;
  size_t count;
  const uint32_t *states;
  size_t state_count;
  thmm_timings timings;
} thmm_maximum_result;

/* BatchedPosteriorSampleView (accelerator.h:131-134). */
typedef struct {
  const uint32_t *states;
  size_t count;
  thmm_timings timings;
} thmm_sample_result;

/* BatchedMarginalView (accelerator.h:140-145). */
typedef struct {
  const void *log_partitions;
  size_t count;
  const void *nodes;
  size_t node_count;
  const void *edges;
  size_t edge_count;
  thmm_timings timings;
} thmm_marginal_result;

/* Dense prepared calls (gpu_backend_api.inc:97-99,103-104,110-111,117-119,
 * 127-129; src/gpu_backend_impl.inc:3021-3118). */
thmm_status thmm_partition_function(thmm_workspace *workspace,
                                    const thmm_dense_model *model,
                                    thmm_partition_result *out);
thmm_status thmm_log_partition_function(thmm_workspace *workspace,
                                        const thmm_dense_model *model,
                                        thmm_partition_result *out);
thmm_status thmm_maximum_a_posteriori(thmm_workspace *workspace,
                                      const thmm_dense_model *model,
                                      thmm_maximum_result *out);
thmm_status thmm_posterior_sample(thmm_workspace *workspace,
                                  const thmm_dense_model *model,
                                  const void *uniforms, size_t uniform_count,
                                  thmm_sample_result *out);
thmm_status thmm_posterior_marginals(thmm_workspace *workspace,
                                     const thmm_dense_model *model,
                                     thmm_marginal_result *out);

/* Categorical prepared calls with a CategoricalInputUpdate policy
 * (gpu_backend_api.inc:100-102,105-109,112-116,120-126,130-142;
 * src/gpu_backend_impl.inc:2842-2946). */
thmm_status thmm_categorical_partition_function(
    thmm_workspace *workspace, const thmm_categorical_model *model,
    int update, thmm_partition_result *out);
thmm_status thmm_categorical_log_partition_function(
    thmm_workspace *workspace, const thmm_categorical_model *model,
    int update, thmm_partition_result *out);
thmm_status thmm_categorical_maximum_a_posteriori(
    thmm_workspace *workspace, const thmm_categorical_model *model,
    int update, thmm_maximum_result *out);
thmm_status thmm_categorical_posterior_sample(
    thmm_workspace *workspace, const thmm_categorical_model *model,
    const void *uniforms, size_t uniform_count, int update,
    thmm_sample_result *out);
thmm_status thmm_categorical_posterior_marginals(
    thmm_workspace *workspace, const thmm_categorical_model *model,
    int update, thmm_marginal_result *out);

/* Extension for device-resident timing (no reference counterpart). Enqueues
 * only the device work of `operation` on the workspace stream, reading the
 * inputs left resident by the previous prepared call of the same workspace;
 * no host copies and no synchronisation. The step (work-counter memset and
 * kernel launches) is captured into a CUDA graph on its first use per
 * operation and batch and replayed afterwards; a new tuning or reservation
 * drops the graphs. `nodes_out` (optional) receives the number of tree nodes
 * processed. */
thmm_status thmm_enqueue(thmm_workspace *workspace, int operation,
                         uint64_t *nodes_out);

/* Extension (no reference counterpart): inputs and results on the device.
 * Device addresses of the workspace's input and result buffers, in the
 * layouts of the prepared calls ([item][node][K], [edge][K][K], observation
 * bytes, ...); null where the workspace has no such buffer. They stay valid
 * until the workspace is reserved again or destroyed. For inputs produced on
 * the GPU (for example by another kernel, or too large to stage through the
 * host): write them here, then call thmm_device_inputs_ready; results of
 * thmm_enqueue can be read here without a host copy. */
typedef struct {
  void *node_potentials;     /* dense: [batch][node][K] */
  void *edge_potentials;     /* [edge][K][K] */
  uint8_t *observations;     /* categorical: observation bytes */
  void *root_potential;      /* categorical: [K] */
  void *emission_potentials; /* categorical: [category][K] */
  void *uniforms;            /* sampling: [batch][node] */
  void *values;              /* [item]: log Z, Z or MAP log weight */
  void *node_marginals;      /* [batch][node][K] */
  void *edge_marginals;      /* [batch][edge][K][K] */
  uint32_t *states;          /* [batch][node] MAP states or samples */
} thmm_device_buffers;
thmm_status thmm_device_buffers_get(thmm_workspace *workspace, thmm_device_buffers *out);
/* Declares the device inputs the caller wrote into thmm_device_buffers_get's
 * buffers resident for `batch` items (a forest: all its trees), as a prepared
 * call with kAll leaves them, so that thmm_enqueue runs on them, and rebuilds
 * the data the kernels derive from them. Work is queued on the workspace
 * stream: the caller's writes must be complete (or queued earlier on that
 * stream) when this is called. */
thmm_status thmm_device_inputs_ready(thmm_workspace *workspace, size_t batch);

/* Launch tuning of a workspace (extension, no reference counterpart). Trees
 * with at least `team_threshold` nodes are contracted by a whole CTA, smaller
 * ones by a single warp. `ctas_per_sm[k]` caps the resident CTAs per SM of
 * kernel k (0: forward sum-product sweep, 1: MAP, 2: sampling, 3: adjoint
 * sweep of the marginals); 0 means the occupancy limit. A prepared call is
 * cut into `stripes` (1 to 8; 0: one per 2 Mi nodes) contiguous runs of
 * instances whose input copies, kernels and output copies overlap.
 * `schedule` picks how sum-product calls (partition, log partition,
 * marginals) are scheduled: THMM_SCHEDULE_TEAMS contracts each tree with one
 * CTA or warp walking its plan step by step; THMM_SCHEDULE_PHASES runs each
 * round of every tree in one grid-wide launch per operation kind (the
 * default where available: forests at every state count, and the batch API
 * up to 4 states; the batch API above 4 states always uses
 * THMM_SCHEDULE_TEAMS). Under THMM_SCHEDULE_PHASES with up to 4 states, the
 * first `phase_rounds` rounds run as grid-wide launches and the remaining
 * rounds of each tree of a forest run in one warp per tree (0: chosen from
 * the operation counts; at least the tree's round count: every round
 * grid-wide); the batch API's shared-topology layout and every workspace
 * above 4 states run every round grid-wide. Up to 32 states no setting
 * changes any result bit; above 32 the two schedules round the tensor-core
 * products differently (both within the same bounds of FP64). */
#define THMM_SCHEDULE_TEAMS 0
#define THMM_SCHEDULE_PHASES 1
typedef struct thmm_tuning {
  uint32_t team_threshold;
  uint32_t ctas_per_sm[4];
  uint32_t stripes;
  float kernel_ms;     /* device time per step of the chosen setting */
  uint32_t candidates; /* settings timed by the last autotune */
  uint32_t schedule;   /* THMM_SCHEDULE_TEAMS or THMM_SCHEDULE_PHASES */
  uint32_t phase_rounds; /* grid-wide rounds of THMM_SCHEDULE_PHASES; 0: automatic */
} thmm_tuning;
/* Times candidate settings for `operation` on the inputs left resident by a
 * prepared call (`repeats` timed steps each, after one untimed step), keeps
 * the fastest and returns it. Overwrites the workspace outputs with the same
 * values. */
thmm_status thmm_autotune(thmm_workspace *workspace, int operation, int repeats,
                          thmm_tuning *out);
thmm_status thmm_get_tuning(const thmm_workspace *workspace, thmm_tuning *out);
thmm_status thmm_set_tuning(thmm_workspace *workspace, const thmm_tuning *tuning);
/* The workspace's cudaStream_t, as an opaque pointer. */
void *thmm_workspace_stream(thmm_workspace *workspace);
thmm_status thmm_workspace_synchronize(thmm_workspace *workspace);

/* Kernel launches made by the most recent prepared call or enqueue. */
uint64_t thmm_workspace_launches(const thmm_workspace *workspace);

/* Diagnostic (no reference counterpart): exercises the error path of the
 * tensor-core engine's bounded waits on `device`. One warp takes tensor
 * memory, waits on an mbarrier whose phase cannot complete (bulk-copy bytes
 * announced, no copy issued) for at most `cycles` SM cycles, records the
 * timeout exactly as the wide-state kernels do and releases the tensor
 * memory. The host then reports the recorded timeout as the prepared calls
 * do: THMM_RUNTIME_ERROR with the same message. THMM_OK would mean the wait
 * did not give up. Nothing else on the device is affected. */
thmm_status thmm_wait_timeout_check(int device, uint64_t cycles);

/* ---------------------------------------------------- allocation-free path */
/* Size of the device array that holds every intermediate of
 * thmm_log_partition_static. */
#define THMM_STATIC_SCRATCH_BYTES (16u * 1024u * 1024u)

/* No counterpart in the reference: an allocation-free variant of the batched
 * log partition function (the scaled sum-product kernel behind
 * thmm_log_partition_function), for callers that cannot call cudaMalloc, such
 * as code whose device memory is owned by another allocator or code running
 * where new allocations are not permitted. It makes no device, pinned or heap
 * allocation on success: the compiled plan and all scratch of the contraction
 * live in one static device array of THMM_STATIC_SCRATCH_BYTES that every GPU
 * loading the library keeps until exit.
 *
 * Inputs and outputs are the caller's device buffers, FP32: node factors
 * [batch, node, state], edge factors [edge, parent, child] shared by the batch,
 * and log Z [batch]. Work is enqueued on `stream` (a cudaStream_t; NULL for
 * the default stream). The compiled plan reaches the device by an ordinary
 * copy from host memory, so the call first waits for work already queued on
 * `stream`; it returns once the plan is handed over, without waiting for the
 * contraction itself.
 *
 * Results and errors: THMM_OK means the contraction was enqueued. It has no
 * failure mode of its own on the device, so nothing is reported later. A tree
 * whose partition is zero (every assignment has zero weight) gets log Z =
 * -inf in `log_partitions`; unlike thmm_log_partition_function, which waits
 * for the result and raises THMM_DOMAIN_ERROR, this call does not wait, so the
 * caller checks the outputs. Argument errors return a status at once, with
 * the message in thmm_last_error(), which a successful call clears.
 *
 * Limits and sharing: 1 to 32 states; a plan and batch whose program and
 * scratch exceed the static array are rejected with THMM_INVALID_ARGUMENT. The first call on a
 * device resolves the array's device address (cudaGetSymbolAddress) and must
 * come before any stream capture. Every call reuses the same array, which keeps
 * the last call's contents; calls whose GPU work overlaps race, and the host
 * side is not thread-safe. */
thmm_status thmm_log_partition_static(const thmm_plan *plan, size_t states,
                                      size_t batch, const float *node_potentials,
                                      const float *edge_potentials,
                                      float *log_partitions, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* THMM_GB300_H_ */
