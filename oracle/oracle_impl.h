/* ORACLE - test infrastructure only. Body of the C restatement of the
 * reference CPU algebras, instantiated for double and float by oracle.c
 * through the macros S (scalar type), SFX (name suffix), XEXP/XLOG (exp/log
 * selected by the `math` argument) and XLOGREF/XEXPREF (always the C library,
 * as in the reference scaled path). Each block cites the reference lines it
 * restates; the floating-point evaluation order is the reference's.
 */

typedef struct {
  size_t states;
  size_t matrix;
  S *nodes;
  S *paths;
  S *branches;
  S *node_scales;
  S *path_scales;
  S *branch_scales;
  S *node_adjoints;
  S *path_adjoints;
  S *branch_adjoints;
  S *rake_paths;
  S *rake_leaves;
  S *compression_left;
  S *compression_middle;
  S *compression_right;
  S *scratch;
  uint32_t *rake_choices;
  uint32_t *compression_choices;
  S *rake_margins;        /* optional: runner-up gap of every rake choice */
  S *compression_margins; /* optional: same for every compression choice */
  uint32_t *assignment;
  S log_partition;
  S max_log_weight;
  int math;
} SFX(store);

static void SFX(store_free)(SFX(store) * st) {
  free(st->nodes);
  free(st->paths);
  free(st->branches);
  free(st->node_scales);
  free(st->path_scales);
  free(st->branch_scales);
  free(st->node_adjoints);
  free(st->path_adjoints);
  free(st->branch_adjoints);
  free(st->rake_paths);
  free(st->rake_leaves);
  free(st->compression_left);
  free(st->compression_middle);
  free(st->compression_right);
  free(st->scratch);
  free(st->rake_choices);
  free(st->compression_choices);
  free(st->rake_margins);
  free(st->compression_margins);
}

static S *SFX(zeros)(size_t count) {
  return (S *)calloc(count == 0 ? 1 : count, sizeof(S));
}

/* Workspace::Reserve (src/inference.cc:845-883) followed by Prepare's copy
 * (src/inference.cc:78-93). Validation follows src/inference.cc:53-76. */
static int SFX(prepare)(const oracle_plan *plan, size_t states, const S *nodes,
                        const S *edges, int want_adjoints, int want_tapes,
                        int want_choices, SFX(store) * st) {
  memset(st, 0, sizeof *st);
  if (states == 0 || states > 256) /* terms[] buffers hold 256 entries */
    return ORACLE_INVALID_ARGUMENT;
  const size_t matrix = states * states;
  const size_t node_values = (size_t)plan->num_nodes * states;
  const size_t path_values = (size_t)plan->num_edges * matrix;
  for (size_t index = 0; index < node_values; ++index)
    if (!isfinite(nodes[index]) || nodes[index] < (S)0)
      return ORACLE_INVALID_ARGUMENT;
  for (size_t index = 0; index < path_values; ++index)
    if (!isfinite(edges[index]) || edges[index] < (S)0)
      return ORACLE_INVALID_ARGUMENT;
  st->states = states;
  st->matrix = matrix;
  st->nodes = SFX(zeros)(node_values);
  st->paths = SFX(zeros)(path_values);
  st->branches = SFX(zeros)((size_t)plan->num_rakes * states);
  st->node_scales = SFX(zeros)(plan->num_nodes);
  st->path_scales = SFX(zeros)(plan->num_edges);
  st->branch_scales = SFX(zeros)(plan->num_rakes);
  st->scratch = SFX(zeros)(matrix);
  if (!st->nodes || !st->paths || !st->branches || !st->node_scales ||
      !st->path_scales || !st->branch_scales || !st->scratch)
    return ORACLE_NO_MEMORY;
  if (want_adjoints) {
    st->node_adjoints = SFX(zeros)(node_values);
    st->path_adjoints = SFX(zeros)(path_values);
    st->branch_adjoints = SFX(zeros)((size_t)plan->num_rakes * states);
    if (!st->node_adjoints || !st->path_adjoints || !st->branch_adjoints)
      return ORACLE_NO_MEMORY;
  }
  if (want_tapes) {
    st->rake_paths = SFX(zeros)((size_t)plan->num_rakes * matrix);
    st->rake_leaves = SFX(zeros)((size_t)plan->num_rakes * states);
    st->compression_left = SFX(zeros)((size_t)plan->num_compressions * matrix);
    st->compression_middle =
        SFX(zeros)((size_t)plan->num_compressions * states);
    st->compression_right = SFX(zeros)((size_t)plan->num_compressions * matrix);
    if (!st->rake_paths || !st->rake_leaves || !st->compression_left ||
        !st->compression_middle || !st->compression_right)
      return ORACLE_NO_MEMORY;
  }
  if (want_choices) {
    st->rake_choices = (uint32_t *)calloc(
        (size_t)plan->num_rakes * states + 1, sizeof(uint32_t));
    st->compression_choices = (uint32_t *)calloc(
        (size_t)plan->num_compressions * matrix + 1, sizeof(uint32_t));
    if (!st->rake_choices || !st->compression_choices)
      return ORACLE_NO_MEMORY;
  }
  memcpy(st->nodes, nodes, node_values * sizeof(S));
  memcpy(st->paths, edges, path_values * sizeof(S));
  return ORACLE_OK;
}

#define NODE(st, i) ((st)->nodes + (size_t)(i) * (st)->states)
#define PATH(st, i) ((st)->paths + (size_t)(i) * (st)->matrix)
#define BRANCH(st, i) ((st)->branches + (size_t)(i) * (st)->states)

/* PotentialLog (src/inference.cc:95-98). */
static S SFX(potential_log)(S value, int math) {
  return value > (S)0 ? XLOG(value, math) : (S)(-INFINITY);
}

/* std::max(a, b) as used by LogSumExp (src/inference.cc:103). */
static S SFX(smax)(S left, S right) { return left < right ? right : left; }

/* LogSumExp over `size` precomputed terms (src/inference.cc:100-110). */
static S SFX(log_sum_exp)(size_t size, const S *terms, int math) {
  S maximum = (S)(-INFINITY);
  for (size_t index = 0; index < size; ++index)
    maximum = SFX(smax)(maximum, terms[index]);
  if (!isfinite(maximum))
    return maximum;
  S sum = (S)0;
  for (size_t index = 0; index < size; ++index)
    sum += XEXP(terms[index] - maximum, math);
  return maximum + XLOG(sum, math);
}

/* Argmax (src/inference.cc:112-126): first maximum wins. */
static size_t SFX(argmax)(size_t size, const S *terms, S *maximum) {
  size_t result = 0;
  S value = terms[0];
  for (size_t index = 1; index < size; ++index) {
    if (terms[index] > value) {
      result = index;
      value = terms[index];
    }
  }
  *maximum = value;
  return result;
}

/* Gap between the chosen maximum and the best other term, relative to the
 * magnitude of the maximum (max(1, |maximum|)): the margin of the deciding
 * comparison of an argmax (+inf when no other term is finite). Diagnostic
 * only; not part of the reference algorithm. */
static S SFX(runner_up_gap)(size_t size, const S *terms, size_t chosen) {
  S second = (S)(-INFINITY);
  for (size_t index = 0; index < size; ++index)
    if (index != chosen && terms[index] > second)
      second = terms[index];
  if (!isfinite(second))
    return (S)INFINITY;
  const S scale = fabs(terms[chosen]) > (S)1 ? fabs(terms[chosen]) : (S)1;
  return (terms[chosen] - second) / scale;
}

/* SampleLogWeights (src/inference.cc:128-146). Returns size on failure.
 * Also reports the margin of its deciding comparisons, the distance from the
 * uniform to the nearer end of the chosen state's cumulative interval
 * (diagnostic only; the draw is the reference's). */
static size_t SFX(sample_log_weights)(size_t size, const S *terms,
                                      S normalizer, S uniform, int math,
                                      S *margin) {
  S cumulative = (S)0;
  S below = (S)0;
  size_t last_supported = size;
  for (size_t index = 0; index < size; ++index) {
    const S log_weight = terms[index];
    if (!isfinite(log_weight))
      continue;
    last_supported = index;
    below = cumulative;
    cumulative += XEXP(log_weight - normalizer, math);
    if (uniform < cumulative) {
      const S up = cumulative - uniform;
      const S down = uniform - below;
      *margin = below == (S)0 ? up : (up < down ? up : down);
      return index;
    }
  }
  *margin = uniform - cumulative;
  return last_supported;
}

static const uint32_t *SFX(op)(const uint32_t *base, size_t width,
                               size_t index) {
  return base + index * width;
}

/* ---------- SumProductDispatcher (src/inference.cc:148-245) ---------- */
static void SFX(sum_rake)(const oracle_plan *plan, SFX(store) * st,
                          uint32_t offset, uint32_t count) {
  const size_t K = st->states;
  for (uint32_t i = offset; i < offset + count; ++i) {
    const uint32_t *op = SFX(op)(plan->rakes, 4, i);
    const S *path = PATH(st, op[0]);
    const S *leaf = NODE(st, op[1]);
    S *message = BRANCH(st, op[2]);
    for (size_t p = 0; p < K; ++p) {
      S value = (S)0;
      for (size_t c = 0; c < K; ++c)
        value += path[p * K + c] * leaf[c];
      message[p] = value;
    }
  }
}

static void SFX(mul_combine)(const oracle_plan *plan, SFX(store) * st,
                             uint32_t offset, uint32_t count) {
  for (uint32_t i = offset; i < offset + count; ++i) {
    const uint32_t *op = SFX(op)(plan->combinations, 3, i);
    S *left = BRANCH(st, op[0]);
    const S *right = BRANCH(st, op[1]);
    for (size_t k = 0; k < st->states; ++k)
      left[k] *= right[k];
  }
}

static void SFX(mul_absorb)(const oracle_plan *plan, SFX(store) * st,
                            uint32_t offset, uint32_t count) {
  for (uint32_t i = offset; i < offset + count; ++i) {
    const uint32_t *op = SFX(op)(plan->absorptions, 3, i);
    S *node = NODE(st, op[0]);
    const S *branch = BRANCH(st, op[1]);
    for (size_t k = 0; k < st->states; ++k)
      node[k] *= branch[k];
  }
}

static void SFX(sum_compress)(const oracle_plan *plan, SFX(store) * st,
                              uint32_t offset, uint32_t count) {
  const size_t K = st->states;
  for (uint32_t i = offset; i < offset + count; ++i) {
    const uint32_t *op = SFX(op)(plan->compressions, 6, i);
    S *left = PATH(st, op[0]);
    const S *middle = NODE(st, op[1]);
    const S *right = PATH(st, op[2]);
    memcpy(st->scratch, left, st->matrix * sizeof(S));
    for (size_t p = 0; p < K; ++p) {
      for (size_t c = 0; c < K; ++c) {
        S value = (S)0;
        for (size_t m = 0; m < K; ++m)
          value += st->scratch[p * K + m] * middle[m] * right[m * K + c];
        left[p * K + c] = value;
      }
    }
  }
}

/* ---------- ScaledSumProductDispatcher (src/inference.cc:697-836) -------- */
/* Normalize (src/inference.cc:787-797). */
static S SFX(normalize)(S *values, size_t size, S input_scale) {
  size_t best = 0;
  for (size_t index = 1; index < size; ++index)
    if (values[best] < values[index])
      best = index;
  const S maximum = values[best];
  if (!(maximum > (S)0))
    return (S)(-INFINITY);
  const S inverse = (S)1 / maximum;
  for (size_t index = 0; index < size; ++index)
    values[index] *= inverse;
  return input_scale + XLOGREF(maximum);
}

static void SFX(scaled_batch)(const oracle_plan *plan, SFX(store) * st,
                              uint32_t primitive, uint32_t offset,
                              uint32_t count) {
  const size_t K = st->states;
  switch (primitive) {
  case 0:
    SFX(sum_rake)(plan, st, offset, count);
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->rakes, 4, i);
      st->branch_scales[op[2]] =
          SFX(normalize)(BRANCH(st, op[2]), K,
                         st->path_scales[op[0]] + st->node_scales[op[1]]);
    }
    break;
  case 1:
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->combinations, 3, i);
      S *destination = BRANCH(st, op[0]);
      const S *source = BRANCH(st, op[1]);
      for (size_t k = 0; k < K; ++k)
        destination[k] *= source[k];
      st->branch_scales[op[0]] = SFX(normalize)(
          destination, K, st->branch_scales[op[0]] + st->branch_scales[op[1]]);
    }
    break;
  case 2:
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->absorptions, 3, i);
      S *node = NODE(st, op[0]);
      const S *branch = BRANCH(st, op[1]);
      for (size_t k = 0; k < K; ++k)
        node[k] *= branch[k];
      st->node_scales[op[0]] = SFX(normalize)(
          node, K, st->node_scales[op[0]] + st->branch_scales[op[1]]);
    }
    break;
  case 3:
    SFX(sum_compress)(plan, st, offset, count);
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->compressions, 6, i);
      st->path_scales[op[0]] = SFX(normalize)(
          PATH(st, op[0]), st->matrix,
          st->path_scales[op[0]] + st->node_scales[op[1]] +
              st->path_scales[op[2]]);
    }
    break;
  }
}

/* ---------- LogSumProductDispatcher (src/inference.cc:247-562) ---------- */
static void SFX(take_logs)(const oracle_plan *plan, SFX(store) * st) {
  const size_t node_values = (size_t)plan->num_nodes * st->states;
  const size_t path_values = (size_t)plan->num_edges * st->matrix;
  for (size_t i = 0; i < node_values; ++i)
    st->nodes[i] = SFX(potential_log)(st->nodes[i], st->math);
  for (size_t i = 0; i < path_values; ++i)
    st->paths[i] = SFX(potential_log)(st->paths[i], st->math);
}

static void SFX(log_batch)(const oracle_plan *plan, SFX(store) * st,
                           uint32_t primitive, uint32_t offset,
                           uint32_t count) {
  const size_t K = st->states;
  const size_t KK = st->matrix;
  S terms[256];
  switch (primitive) {
  case 0: /* Rake, src/inference.cc:259-277 */
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->rakes, 4, i);
      const S *path = PATH(st, op[0]);
      const S *leaf = NODE(st, op[1]);
      memcpy(st->rake_paths + (size_t)op[2] * KK, path, KK * sizeof(S));
      memcpy(st->rake_leaves + (size_t)op[2] * K, leaf, K * sizeof(S));
      S *message = BRANCH(st, op[2]);
      for (size_t p = 0; p < K; ++p) {
        for (size_t c = 0; c < K; ++c)
          terms[c] = path[p * K + c] + leaf[c];
        message[p] = SFX(log_sum_exp)(K, terms, st->math);
      }
    }
    break;
  case 1: /* CombineBranches, src/inference.cc:279-286 */
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->combinations, 3, i);
      S *destination = BRANCH(st, op[0]);
      const S *source = BRANCH(st, op[1]);
      for (size_t k = 0; k < K; ++k)
        destination[k] += source[k];
    }
    break;
  case 2: /* AbsorbBranches, src/inference.cc:288-295 */
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->absorptions, 3, i);
      S *node = NODE(st, op[0]);
      const S *branch = BRANCH(st, op[1]);
      for (size_t k = 0; k < K; ++k)
        node[k] += branch[k];
    }
    break;
  case 3: /* Compress, src/inference.cc:297-324 */
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->compressions, 6, i);
      S *left = PATH(st, op[0]);
      const S *middle = NODE(st, op[1]);
      const S *right = PATH(st, op[2]);
      S *saved_left = st->compression_left + (size_t)op[3] * KK;
      S *saved_middle = st->compression_middle + (size_t)op[3] * K;
      S *saved_right = st->compression_right + (size_t)op[3] * KK;
      memcpy(saved_left, left, KK * sizeof(S));
      memcpy(saved_middle, middle, K * sizeof(S));
      memcpy(saved_right, right, KK * sizeof(S));
      for (size_t p = 0; p < K; ++p) {
        for (size_t c = 0; c < K; ++c) {
          for (size_t m = 0; m < K; ++m)
            terms[m] = saved_left[p * K + m] + saved_middle[m] +
                       saved_right[m * K + c];
          left[p * K + c] = SFX(log_sum_exp)(K, terms, st->math);
        }
      }
    }
    break;
  }
}

/* FinishRoot (src/inference.cc:326-336). */
static int SFX(log_finish)(const oracle_plan *plan, SFX(store) * st) {
  st->log_partition = SFX(log_sum_exp)(st->states, NODE(st, plan->root),
                                       st->math);
  if (!isfinite(st->log_partition))
    return ORACLE_DOMAIN_ERROR;
  return ORACLE_OK;
}

/* ReverseCompressions (src/inference.cc:416-464). */
static void SFX(reverse_compressions)(const oracle_plan *plan, SFX(store) * st,
                                      uint32_t offset, uint32_t count) {
  const size_t K = st->states;
  const size_t KK = st->matrix;
  S terms[256];
  for (uint32_t i = offset + count; i-- > offset;) {
    const uint32_t *op = SFX(op)(plan->compressions, 6, i);
    const S *left = st->compression_left + (size_t)op[3] * KK;
    const S *middle = st->compression_middle + (size_t)op[3] * K;
    const S *right = st->compression_right + (size_t)op[3] * KK;
    S *output_adjoint = st->path_adjoints + (size_t)op[0] * KK;
    for (size_t e = 0; e < KK; ++e)
      st->scratch[e] = (S)0;
    S *middle_adjoint = st->node_adjoints + (size_t)op[1] * K;
    S *right_adjoint = st->path_adjoints + (size_t)op[2] * KK;
    for (size_t p = 0; p < K; ++p) {
      for (size_t c = 0; c < K; ++c) {
        const size_t output_index = p * K + c;
        const S adjoint = output_adjoint[output_index];
        for (size_t m = 0; m < K; ++m)
          terms[m] = left[p * K + m] + middle[m] + right[m * K + c];
        const S output = SFX(log_sum_exp)(K, terms, st->math);
        if (adjoint == (S)0 || !isfinite(output))
          continue;
        for (size_t m = 0; m < K; ++m) {
          const size_t left_index = p * K + m;
          const size_t right_index = m * K + c;
          const S term = left[left_index] + middle[m] + right[right_index];
          if (!isfinite(term))
            continue;
          const S contribution = adjoint * XEXP(term - output, st->math);
          st->scratch[left_index] += contribution;
          middle_adjoint[m] += contribution;
          right_adjoint[right_index] += contribution;
        }
      }
    }
    memcpy(output_adjoint, st->scratch, KK * sizeof(S));
  }
}

/* ReverseRakes (src/inference.cc:488-518). */
static void SFX(reverse_rakes)(const oracle_plan *plan, SFX(store) * st,
                               uint32_t offset, uint32_t count) {
  const size_t K = st->states;
  const size_t KK = st->matrix;
  S terms[256];
  for (uint32_t i = offset + count; i-- > offset;) {
    const uint32_t *op = SFX(op)(plan->rakes, 4, i);
    const S *path = st->rake_paths + (size_t)op[2] * KK;
    const S *leaf = st->rake_leaves + (size_t)op[2] * K;
    const S *message_adjoint = st->branch_adjoints + (size_t)op[2] * K;
    S *path_adjoint = st->path_adjoints + (size_t)op[0] * KK;
    S *leaf_adjoint = st->node_adjoints + (size_t)op[1] * K;
    for (size_t p = 0; p < K; ++p) {
      for (size_t c = 0; c < K; ++c)
        terms[c] = path[p * K + c] + leaf[c];
      const S message = SFX(log_sum_exp)(K, terms, st->math);
      if (!isfinite(message))
        continue;
      for (size_t c = 0; c < K; ++c) {
        const size_t path_index = p * K + c;
        const S term = path[path_index] + leaf[c];
        if (!isfinite(term))
          continue;
        const S contribution =
            message_adjoint[p] * XEXP(term - message, st->math);
        path_adjoint[path_index] += contribution;
        leaf_adjoint[c] += contribution;
      }
    }
  }
}

static void SFX(reverse_batch)(const oracle_plan *plan, SFX(store) * st,
                               uint32_t primitive, uint32_t offset,
                               uint32_t count) {
  const size_t K = st->states;
  switch (primitive) {
  case 0:
    SFX(reverse_rakes)(plan, st, offset, count);
    break;
  case 1: /* ReverseCombineBranches, src/inference.cc:477-486 */
    for (uint32_t i = offset + count; i-- > offset;) {
      const uint32_t *op = SFX(op)(plan->combinations, 3, i);
      const S *destination = st->branch_adjoints + (size_t)op[0] * K;
      S *source = st->branch_adjoints + (size_t)op[1] * K;
      for (size_t k = 0; k < K; ++k)
        source[k] += destination[k];
    }
    break;
  case 2: /* ReverseAbsorbBranches, src/inference.cc:466-475 */
    for (uint32_t i = offset + count; i-- > offset;) {
      const uint32_t *op = SFX(op)(plan->absorptions, 3, i);
      const S *node = st->node_adjoints + (size_t)op[0] * K;
      S *branch = st->branch_adjoints + (size_t)op[1] * K;
      for (size_t k = 0; k < K; ++k)
        branch[k] += node[k];
    }
    break;
  case 3:
    SFX(reverse_compressions)(plan, st, offset, count);
    break;
  }
}

/* ---------- MaxProductDispatcher (src/inference.cc:564-695) ---------- */
static void SFX(max_batch)(const oracle_plan *plan, SFX(store) * st,
                           uint32_t primitive, uint32_t offset,
                           uint32_t count) {
  const size_t K = st->states;
  const size_t KK = st->matrix;
  S terms[256];
  switch (primitive) {
  case 0: /* src/inference.cc:576-594 */
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->rakes, 4, i);
      const S *path = PATH(st, op[0]);
      const S *leaf = NODE(st, op[1]);
      S *message = BRANCH(st, op[2]);
      uint32_t *choices = st->rake_choices + (size_t)op[2] * K;
      for (size_t p = 0; p < K; ++p) {
        for (size_t c = 0; c < K; ++c)
          terms[c] = path[p * K + c] + leaf[c];
        choices[p] = (uint32_t)SFX(argmax)(K, terms, &message[p]);
        if (st->rake_margins != NULL)
          st->rake_margins[(size_t)op[2] * K + p] = SFX(runner_up_gap)(K, terms, choices[p]);
      }
    }
    break;
  case 1:
  case 2:
    SFX(log_batch)(plan, st, primitive, offset, count);
    break;
  case 3: /* src/inference.cc:614-639 */
    for (uint32_t i = offset; i < offset + count; ++i) {
      const uint32_t *op = SFX(op)(plan->compressions, 6, i);
      S *left = PATH(st, op[0]);
      const S *middle = NODE(st, op[1]);
      const S *right = PATH(st, op[2]);
      memcpy(st->scratch, left, KK * sizeof(S));
      uint32_t *choices = st->compression_choices + (size_t)op[3] * KK;
      for (size_t p = 0; p < K; ++p) {
        for (size_t c = 0; c < K; ++c) {
          for (size_t m = 0; m < K; ++m)
            terms[m] = st->scratch[p * K + m] + middle[m] + right[m * K + c];
          choices[p * K + c] =
              (uint32_t)SFX(argmax)(K, terms, &left[p * K + c]);
          if (st->compression_margins != NULL)
            st->compression_margins[(size_t)op[3] * KK + p * K + c] =
                SFX(runner_up_gap)(K, terms, choices[p * K + c]);
        }
      }
    }
    break;
  }
}

/* ---------- public entry points ---------- */
int SFX(oracle_partition)(const oracle_plan *plan, size_t states,
                          const S *nodes, const S *edges, S *out) {
  SFX(store) st;
  int status = SFX(prepare)(plan, states, nodes, edges, 0, 0, 0, &st);
  if (status == ORACLE_OK) {
    for (uint32_t b = 0; b < plan->num_batches; ++b) {
      const uint32_t *batch = plan->batches + 3 * (size_t)b;
      switch (batch[0]) {
      case 0:
        SFX(sum_rake)(plan, &st, batch[1], batch[2]);
        break;
      case 1:
        SFX(mul_combine)(plan, &st, batch[1], batch[2]);
        break;
      case 2:
        SFX(mul_absorb)(plan, &st, batch[1], batch[2]);
        break;
      case 3:
        SFX(sum_compress)(plan, &st, batch[1], batch[2]);
        break;
      }
    }
    /* FinishRoot, src/inference.cc:216-220 */
    S sum = (S)0;
    const S *root = NODE(&st, plan->root);
    for (size_t k = 0; k < states; ++k)
      sum += root[k];
    *out = sum;
  }
  SFX(store_free)(&st);
  return status;
}

int SFX(oracle_log_partition)(const oracle_plan *plan, size_t states,
                              const S *nodes, const S *edges, S *out) {
  SFX(store) st;
  int status = SFX(prepare)(plan, states, nodes, edges, 0, 0, 0, &st);
  if (status == ORACLE_OK) {
    for (uint32_t b = 0; b < plan->num_batches; ++b) {
      const uint32_t *batch = plan->batches + 3 * (size_t)b;
      SFX(scaled_batch)(plan, &st, batch[0], batch[1], batch[2]);
    }
    /* FinishRoot, src/inference.cc:778-784 */
    S sum = (S)0;
    const S *root = NODE(&st, plan->root);
    for (size_t k = 0; k < states; ++k)
      sum += root[k];
    *out = !(sum > (S)0) ? (S)(-INFINITY)
                         : st.node_scales[plan->root] + XLOGREF(sum);
  }
  SFX(store_free)(&st);
  return status;
}

int SFX(oracle_marginals)(const oracle_plan *plan, size_t states,
                          const S *nodes, const S *edges, S *log_partition,
                          S *partition, S *node_marginals, S *edge_marginals) {
  SFX(store) st;
  int status = SFX(prepare)(plan, states, nodes, edges, 1, 1, 0, &st);
  if (status == ORACLE_OK) {
    st.math = ORACLE_MATH_LIBM;
    SFX(take_logs)(plan, &st);
    for (uint32_t b = 0; b < plan->num_batches; ++b) {
      const uint32_t *batch = plan->batches + 3 * (size_t)b;
      SFX(log_batch)(plan, &st, batch[0], batch[1], batch[2]);
    }
    status = SFX(log_finish)(plan, &st);
  }
  if (status == ORACLE_OK) {
    /* SeedRootAdjoint, src/inference.cc:338-343 */
    const S *root = NODE(&st, plan->root);
    S *root_adjoint = st.node_adjoints + (size_t)plan->root * states;
    for (size_t k = 0; k < states; ++k)
      root_adjoint[k] = XEXP(root[k] - st.log_partition, st.math);
    for (uint32_t b = plan->num_batches; b-- > 0;) {
      const uint32_t *batch = plan->batches + 3 * (size_t)b;
      SFX(reverse_batch)(plan, &st, batch[0], batch[1], batch[2]);
    }
    *log_partition = st.log_partition;
    *partition = XEXP(st.log_partition, st.math);
    memcpy(node_marginals, st.node_adjoints,
           (size_t)plan->num_nodes * states * sizeof(S));
    memcpy(edge_marginals, st.path_adjoints,
           (size_t)plan->num_edges * st.matrix * sizeof(S));
  }
  SFX(store_free)(&st);
  return status;
}

int SFX(oracle_map_margins)(const oracle_plan *plan, size_t states, const S *nodes,
                            const S *edges, int math, S *log_weight,
                            uint32_t *assignment, S *margins) {
  SFX(store) st;
  int status = SFX(prepare)(plan, states, nodes, edges, 0, 0, 1, &st);
  if (status == ORACLE_OK && margins != NULL) {
    st.rake_margins = SFX(zeros)((size_t)plan->num_rakes * states);
    st.compression_margins = SFX(zeros)((size_t)plan->num_compressions * st.matrix);
    if (st.rake_margins == NULL || st.compression_margins == NULL)
      status = ORACLE_NO_MEMORY;
  }
  if (status == ORACLE_OK) {
    st.math = math;
    SFX(take_logs)(plan, &st);
    for (uint32_t b = 0; b < plan->num_batches; ++b) {
      const uint32_t *batch = plan->batches + 3 * (size_t)b;
      SFX(max_batch)(plan, &st, batch[0], batch[1], batch[2]);
    }
    /* FinishRoot, src/inference.cc:641-649 */
    assignment[plan->root] = (uint32_t)SFX(argmax)(
        states, NODE(&st, plan->root), &st.max_log_weight);
    if (margins != NULL)
      margins[plan->root] =
          SFX(runner_up_gap)(states, NODE(&st, plan->root), assignment[plan->root]);
    if (!isfinite(st.max_log_weight))
      status = ORACLE_DOMAIN_ERROR;
  }
  if (status == ORACLE_OK) {
    /* ExpandRakes / ExpandCompressions, src/inference.cc:651-667 */
    for (uint32_t b = plan->num_batches; b-- > 0;) {
      const uint32_t *batch = plan->batches + 3 * (size_t)b;
      if (batch[0] == 0) {
        for (uint32_t i = batch[1]; i < batch[1] + batch[2]; ++i) {
          const uint32_t *op = SFX(op)(plan->rakes, 4, i);
          assignment[op[1]] =
              st.rake_choices[(size_t)op[2] * states + assignment[op[3]]];
          if (margins != NULL)
            margins[op[1]] = st.rake_margins[(size_t)op[2] * states + assignment[op[3]]];
        }
      } else if (batch[0] == 3) {
        for (uint32_t i = batch[1]; i < batch[1] + batch[2]; ++i) {
          const uint32_t *op = SFX(op)(plan->compressions, 6, i);
          const size_t entry = (size_t)op[3] * st.matrix +
                               (size_t)assignment[op[4]] * states + assignment[op[5]];
          assignment[op[1]] = st.compression_choices[entry];
          if (margins != NULL)
            margins[op[1]] = st.compression_margins[entry];
        }
      }
    }
    *log_weight = st.max_log_weight;
  }
  SFX(store_free)(&st);
  return status;
}

int SFX(oracle_map)(const oracle_plan *plan, size_t states, const S *nodes,
                    const S *edges, int math, S *log_weight,
                    uint32_t *assignment) {
  return SFX(oracle_map_margins)(plan, states, nodes, edges, math, log_weight,
                                 assignment, NULL);
}

int SFX(oracle_sample_margins)(const oracle_plan *plan, size_t states, const S *nodes,
                               const S *edges, const S *uniforms, int math,
                               uint32_t *assignment, S *margins) {
  SFX(store) st;
  int status = SFX(prepare)(plan, states, nodes, edges, 0, 1, 0, &st);
  S terms[256];
  if (status == ORACLE_OK) {
    st.math = math;
    SFX(take_logs)(plan, &st);
    for (uint32_t b = 0; b < plan->num_batches; ++b) {
      const uint32_t *batch = plan->batches + 3 * (size_t)b;
      SFX(log_batch)(plan, &st, batch[0], batch[1], batch[2]);
    }
    status = SFX(log_finish)(plan, &st);
  }
  if (status == ORACLE_OK) {
    /* SeedRootSample, src/inference.cc:345-361 */
    for (uint32_t n = 0; n < plan->num_nodes; ++n)
      if (!isfinite(uniforms[n]) || uniforms[n] < (S)0 || uniforms[n] >= (S)1)
        status = ORACLE_INVALID_ARGUMENT;
  }
  if (status == ORACLE_OK) {
    S gap = (S)0;
    size_t choice = SFX(sample_log_weights)(states, NODE(&st, plan->root),
                                                   st.log_partition,
                                                   uniforms[plan->root], math, &gap);
    if (margins != NULL)
      margins[plan->root] = gap;
    if (choice == states)
      status = ORACLE_DOMAIN_ERROR;
    assignment[plan->root] = (uint32_t)choice;
    /* ExpandRakes / ExpandCompressions, src/inference.cc:363-412 */
    for (uint32_t b = plan->num_batches; status == ORACLE_OK && b-- > 0;) {
      const uint32_t *batch = plan->batches + 3 * (size_t)b;
      if (batch[0] == 0) {
        for (uint32_t i = batch[1]; i < batch[1] + batch[2]; ++i) {
          const uint32_t *op = SFX(op)(plan->rakes, 4, i);
          const size_t p = assignment[op[3]];
          const S *path = st.rake_paths + (size_t)op[2] * st.matrix;
          const S *leaf = st.rake_leaves + (size_t)op[2] * states;
          for (size_t c = 0; c < states; ++c)
            terms[c] = path[p * states + c] + leaf[c];
          const S normalizer = SFX(log_sum_exp)(states, terms, math);
          choice = SFX(sample_log_weights)(states, terms, normalizer,
                                                  uniforms[op[1]], math, &gap);
          if (choice == states)
            status = ORACLE_DOMAIN_ERROR;
          assignment[op[1]] = (uint32_t)choice;
          if (margins != NULL)
            margins[op[1]] = gap;
        }
      } else if (batch[0] == 3) {
        for (uint32_t i = batch[1]; i < batch[1] + batch[2]; ++i) {
          const uint32_t *op = SFX(op)(plan->compressions, 6, i);
          const size_t p = assignment[op[4]];
          const size_t c = assignment[op[5]];
          const S *left = st.compression_left + (size_t)op[3] * st.matrix;
          const S *middle = st.compression_middle + (size_t)op[3] * states;
          const S *right = st.compression_right + (size_t)op[3] * st.matrix;
          for (size_t m = 0; m < states; ++m)
            terms[m] = left[p * states + m] + middle[m] + right[m * states + c];
          const S normalizer = SFX(log_sum_exp)(states, terms, math);
          choice = SFX(sample_log_weights)(states, terms, normalizer,
                                                  uniforms[op[1]], math, &gap);
          if (choice == states)
            status = ORACLE_DOMAIN_ERROR;
          assignment[op[1]] = (uint32_t)choice;
          if (margins != NULL)
            margins[op[1]] = gap;
        }
      }
    }
  }
  SFX(store_free)(&st);
  return status;
}

int SFX(oracle_sample)(const oracle_plan *plan, size_t states, const S *nodes,
                       const S *edges, const S *uniforms, int math,
                       uint32_t *assignment) {
  return SFX(oracle_sample_margins)(plan, states, nodes, edges, uniforms, math,
                                    assignment, NULL);
}

#undef NODE
#undef PATH
#undef BRANCH
