/* ORACLE - test infrastructure only.
 *
 * A plain-C restatement of the reference CPU algebras of parallel_tree_hmm
 * (src/inference.cc), used as the checker for the GPU path. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product never links or calls it.
 *
 * Every function follows the reference operation by operation and in the same
 * floating-point evaluation order, so with ORACLE_MATH_LIBM it reproduces the
 * reference build bit for bit (checked in tests/test_oracle_pin.py against the
 * reference compiled from its own sources). ORACLE_MATH_PORTABLE swaps the C
 * library exp/log for the reproducible pair in portable_math.h, which the GPU
 * MAP and sampling kernels use, so those discrete results can be compared
 * bit for bit with the device.
 *
 * The plan is passed as the raw operation arrays of a btrc::Plan.
 */
#ifndef THMM_ORACLE_H_
#define THMM_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  uint32_t num_nodes;
  uint32_t num_edges;
  uint32_t root;
  uint32_t num_rakes;
  uint32_t num_combinations;
  uint32_t num_absorptions;
  uint32_t num_compressions;
  uint32_t num_batches;
  const uint32_t *edge_parents;  /* [num_edges] */
  const uint32_t *edge_children; /* [num_edges] */
  const uint32_t *rakes;         /* [num_rakes][4] edge, leaf, branch, parent */
  const uint32_t *combinations;  /* [n][3] destination, source, parent */
  const uint32_t *absorptions;   /* [n][3] parent, branch, round */
  const uint32_t *compressions;  /* [n][6] left, middle, right, tape, parent, child */
  const uint32_t *batches;       /* [n][3] primitive, offset, count */
} oracle_plan;

enum {
  ORACLE_OK = 0,
  ORACLE_INVALID_ARGUMENT = 1,
  ORACLE_DOMAIN_ERROR = 3,
  ORACLE_NO_MEMORY = 6,
};

enum {
  ORACLE_MATH_LIBM = 0,
  ORACLE_MATH_PORTABLE = 1,
};

/* Raw partition function Z (src/inference.cc:148-245,885-890). */
int oracle_partition_f64(const oracle_plan *plan, size_t states,
                         const double *nodes, const double *edges, double *out);
int oracle_partition_f32(const oracle_plan *plan, size_t states,
                         const float *nodes, const float *edges, float *out);

/* Scaled log partition (src/inference.cc:697-836,892-903). */
int oracle_log_partition_f64(const oracle_plan *plan, size_t states,
                             const double *nodes, const double *edges,
                             double *out);
int oracle_log_partition_f32(const oracle_plan *plan, size_t states,
                             const float *nodes, const float *edges,
                             float *out);

/* Log-domain marginals (src/inference.cc:247-562,905-917). */
int oracle_marginals_f64(const oracle_plan *plan, size_t states,
                         const double *nodes, const double *edges,
                         double *log_partition, double *partition,
                         double *node_marginals, double *edge_marginals);
int oracle_marginals_f32(const oracle_plan *plan, size_t states,
                         const float *nodes, const float *edges,
                         float *log_partition, float *partition,
                         float *node_marginals, float *edge_marginals);

/* Max-product MAP (src/inference.cc:564-695,919-927). */
int oracle_map_f64(const oracle_plan *plan, size_t states, const double *nodes,
                   const double *edges, int math, double *log_weight,
                   uint32_t *assignment);
int oracle_map_f32(const oracle_plan *plan, size_t states, const float *nodes,
                   const float *edges, int math, float *log_weight,
                   uint32_t *assignment);

/* Posterior sample (src/inference.cc:128-146,345-414,929-939). */
int oracle_sample_f64(const oracle_plan *plan, size_t states,
                      const double *nodes, const double *edges,
                      const double *uniforms, int math, uint32_t *assignment);
int oracle_sample_f32(const oracle_plan *plan, size_t states,
                      const float *nodes, const float *edges,
                      const float *uniforms, int math, uint32_t *assignment);

/* The same MAP and sample with, for every node, the margin of the
 * comparison that decided its state (diagnostic, for classifying
 * disagreements between two implementations): for MAP the gap between the
 * chosen maximum and the best other candidate of its choice, relative to
 * max(1, |maximum|); for sampling
 * the distance from the node's uniform to the nearer end of the chosen
 * state's cumulative interval. */
int oracle_map_margins_f64(const oracle_plan *plan, size_t states, const double *nodes,
                           const double *edges, int math, double *log_weight,
                           uint32_t *assignment, double *margins);
int oracle_map_margins_f32(const oracle_plan *plan, size_t states, const float *nodes,
                           const float *edges, int math, float *log_weight,
                           uint32_t *assignment, float *margins);
int oracle_sample_margins_f64(const oracle_plan *plan, size_t states,
                              const double *nodes, const double *edges,
                              const double *uniforms, int math, uint32_t *assignment,
                              double *margins);
int oracle_sample_margins_f32(const oracle_plan *plan, size_t states,
                              const float *nodes, const float *edges,
                              const float *uniforms, int math, uint32_t *assignment,
                              float *margins);

/* Portable exp/log exposed for the error-bound tests. */
float oracle_portable_expf(float x);
float oracle_portable_logf(float x);
double oracle_portable_exp(double x);
double oracle_portable_log(double x);

#ifdef __cplusplus
}
#endif

#endif /* THMM_ORACLE_H_ */
