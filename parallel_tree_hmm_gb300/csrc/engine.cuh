// Persistent tree-contraction kernels for sm_103a.
//
// Work decomposition. A *team* contracts one tree instance at a time: a whole
// CTA for large trees, a single warp for small ones. Instances come from two
// queues (largest first) through one atomic counter each; a CTA drains the
// large-tree queue first and then splits into four warp teams for the small
// trees. Inside a team the plan's steps run in order with a team barrier in
// between (the operations of one step are independent, as in a
// btrc::PrimitiveBatch). Each operation of a step is handled by a *group* of
// KMAX consecutive lanes of one warp, lane r owning row/state r, so K-vectors
// and K x K matrices are read row-coalesced and reductions over states are
// warp shuffles. There are no grid-wide barriers and no spin waits.
//
// Sum-product (LinearEngine) runs in the linear domain and renormalises every
// produced message by an exact power of two, accumulating the exponents in an
// integer; log Z = ln2 * sum(exponents) + log(sum(root)). This is the
// reference's scaled algebra (src/inference.cc:697-836,
// src/gpu_device_algebra.h:16-52) with the natural-log scale replaced by an
// exact binary exponent. The marginals are the adjoint of that contraction
// (d log Z / d log factor): because every path version and every node value is
// consumed exactly once, the adjoint of a rake's branch equals the marginal of
// the rake's parent node, so the reverse sweep only revisits rake and
// compression steps (the reference revisits every primitive in the log domain,
// src/inference.cc:416-518, src/gpu_backend_impl.inc:554-744).
//
// MAP (MaxEngine) and sampling (SampleEngine) follow the reference CPU
// algebras operation by operation in the log domain (src/inference.cc:
// 100-146,247-414,564-695), with the reproducible exp/log of portable_math.h,
// so their discrete outputs can be compared bit for bit with the oracle.
#ifndef THMM_ENGINE_CUH_
#define THMM_ENGINE_CUH_

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"
#include "portable_math.h"

namespace thmm {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;

template <bool kCta> struct Team {
  unsigned tid;
  unsigned size;
  __device__ __forceinline__ void sync() const {
    if constexpr (kCta)
      __syncthreads();
    else
      __syncwarp();
  }
};

// ------------------------------------------------------------- numerics --
__device__ __forceinline__ int Pow2Exponent(float m) {
  const unsigned bits = __float_as_uint(m);
  if (bits >= 0x00800000u)
    return static_cast<int>((bits >> 23) & 0xffu) - 126;
  int e;
  frexpf(m, &e);
  return e;
}
__device__ __forceinline__ int Pow2Exponent(double m) {
  const unsigned long long bits = static_cast<unsigned long long>(
      __double_as_longlong(m));
  if (bits >= 0x0010000000000000ull)
    return static_cast<int>((bits >> 52) & 0x7ffull) - 1022;
  int e;
  frexp(m, &e);
  return e;
}
// v * 2^s, exact unless the result is subnormal.
__device__ __forceinline__ float ScalePow2(float v, int s) {
  if (s >= -126 && s <= 127)
    return v * __uint_as_float(static_cast<unsigned>(127 + s) << 23);
  return ldexpf(v, s);
}
__device__ __forceinline__ double ScalePow2(double v, int s) {
  if (s >= -1022 && s <= 1023)
    return v * __longlong_as_double(static_cast<long long>(1023 + s) << 52);
  return ldexp(v, s);
}

__device__ __forceinline__ float PortableExp(float x) { return thmm_expf(x); }
__device__ __forceinline__ double PortableExp(double x) { return thmm_exp(x); }
__device__ __forceinline__ float PortableLog(float x) { return thmm_logf(x); }
__device__ __forceinline__ double PortableLog(double x) { return thmm_log(x); }

template <typename T> __device__ __forceinline__ T NegInf();
template <> __device__ __forceinline__ float NegInf<float>() {
  return __uint_as_float(0xff800000u);
}
template <> __device__ __forceinline__ double NegInf<double>() {
  return __longlong_as_double(static_cast<long long>(0xfff0000000000000ull));
}

// PotentialLog (src/inference.cc:95-98).
template <typename T> __device__ __forceinline__ T PotentialLog(T v) {
  return v > T(0) ? PortableLog(v) : NegInf<T>();
}

template <int G, typename T> __device__ __forceinline__ T GroupMax(T v) {
#pragma unroll
  for (int offset = G / 2; offset > 0; offset >>= 1) {
    const T other = __shfl_xor_sync(kFull, v, offset, G);
    v = v < other ? other : v;
  }
  return v;
}

template <int G, typename T>
__device__ __forceinline__ T GroupBroadcast(T v, int source) {
  if constexpr (G == 1)
    return v;
  else
    return __shfl_sync(kFull, v, source, G);
}

// Iterates the `count` operations of a step over groups of G lanes with a
// trip count that is uniform across the team, so warp shuffles inside `body`
// always see all 32 lanes. Idle groups re-run operation 0 with stores off.
template <int G, bool kCta, class Body>
__device__ __forceinline__ void ForGroups(const Team<kCta> &team,
                                          unsigned count, Body body) {
  const unsigned groups = team.size / G;
  const unsigned group = team.tid / G;
  const unsigned lane = team.tid % G;
  for (unsigned first = 0; first < count; first += groups) {
    const unsigned index = first + group;
    const bool active = index < count;
    body(active ? index : 0u, active, lane);
  }
}

template <bool kCta, class Body>
__device__ __forceinline__ void ForThreads(const Team<kCta> &team,
                                           unsigned count, Body body) {
  for (unsigned index = team.tid; index < count; index += team.size)
    body(index);
}

// Team-wide sum of an exponent total and OR of a flag.
template <bool kCta>
__device__ __forceinline__ void TeamReduce(const Team<kCta> &team,
                                           long long &total, int &flag,
                                           long long *warp_totals,
                                           int *warp_flags) {
#pragma unroll
  for (int offset = 16; offset > 0; offset >>= 1) {
    total += __shfl_xor_sync(kFull, total, offset);
    flag |= __shfl_xor_sync(kFull, flag, offset);
  }
  if constexpr (kCta) {
    const unsigned warp = team.tid / 32;
    if ((team.tid & 31) == 0) {
      warp_totals[warp] = total;
      warp_flags[warp] = flag;
    }
    __syncthreads();
    total = 0;
    flag = 0;
    for (unsigned w = 0; w < team.size / 32; ++w) {
      total += warp_totals[w];
      flag |= warp_flags[w];
    }
    __syncthreads();
  }
}

struct SharedState {
  unsigned item;
  long long warp_totals[kWarps];
  int warp_flags[kWarps];
};

// ------------------------------------------------------- shared context --
template <typename Scalar, typename Compute, int KMAX> struct Context {
  const EngineArgs &a;
  DevInstance inst;
  DevProgram prog;
  unsigned K;
  unsigned KK;
  Compute *nodes;
  Compute *branches;
  Compute *comps;
  const Scalar *edge_in;

  __device__ Context(const EngineArgs &args, unsigned item) : a(args) {
    inst = a.instances[item];
    prog = a.programs[inst.program];
    K = a.states;
    KK = K * K;
    Compute *base = static_cast<Compute *>(a.scratch) + inst.scratch_base;
    nodes = base;
    branches = nodes + static_cast<std::size_t>(prog.num_nodes) * K;
    comps = branches + static_cast<std::size_t>(prog.num_rakes) * K;
    edge_in = static_cast<const Scalar *>(a.edge_in) +
              inst.edge_in_base * static_cast<std::uint64_t>(KK);
  }

  // Input node factor, as src/gpu_backend_impl.inc:326-382 builds it for a
  // categorical model: (root ? root_potential : 1) * emission[observation].
  __device__ __forceinline__ Scalar InputNode(unsigned node, unsigned j) const {
    if (!a.categorical)
      return static_cast<const Scalar *>(
          a.node_in)[(inst.node_base + node) * K + j];
    const Scalar base = node == (prog.root & kMask)
                            ? static_cast<const Scalar *>(a.root_potential)[j]
                            : Scalar(1);
    const int slot = a.obs_map[prog.obs_map + node];
    if (slot < 0)
      return base;
    const unsigned category = a.observations[inst.obs_base + slot];
    const Scalar emission =
        category < a.categories
            ? static_cast<const Scalar *>(a.emission)[category * K + j]
            : Scalar(0);
    return base * emission;
  }

  __device__ __forceinline__ Scalar InputEdge(unsigned edge, unsigned i,
                                              unsigned j) const {
    return edge_in[static_cast<std::size_t>(edge) * KK + i * K + j];
  }
};

// ------------------------------------------------------- sum-product --
template <typename Scalar, typename Compute, int KMAX> struct LinearEngine {
  static constexpr int G = KMAX;
  using Ctx = Context<Scalar, Compute, KMAX>;
  Ctx c;
  Compute *comp_mu;
  int *comp_exp;
  Compute *group_buffer; // K*K values per group (reverse compressions)
  int exponent = 0;      // this thread's share of the log-scale exponent
  int zero = 0;          // some renormalised message was identically zero

  __device__ LinearEngine(const EngineArgs &args, unsigned item,
                          Compute *warp_buffer, unsigned lane_in_warp)
      : c(args, item) {
    comp_mu = c.comps + static_cast<std::size_t>(c.prog.num_compressions) * c.KK;
    comp_exp = reinterpret_cast<int *>(args.bytes + c.inst.byte_base);
    group_buffer = warp_buffer + (lane_in_warp / G) * KMAX * KMAX;
  }

  __device__ __forceinline__ Compute Node(unsigned ref, unsigned j) const {
    return (ref & kFlag) ? c.nodes[static_cast<std::size_t>(ref & kMask) * c.K + j]
                         : static_cast<Compute>(c.InputNode(ref, j));
  }
  __device__ __forceinline__ Compute Path(unsigned ref, unsigned i,
                                          unsigned j) const {
    return (ref & kFlag)
               ? c.comps[static_cast<std::size_t>(ref & kMask) * c.KK +
                         i * c.K + j]
               : static_cast<Compute>(c.InputEdge(ref, i, j));
  }

  // Renormalises the group's K values (one per lane) by a power of two.
  __device__ __forceinline__ Compute Normalize(Compute v, bool active,
                                               unsigned r) {
    const Compute m = GroupMax<G>(v);
    if (m > Compute(0)) {
      const int e = Pow2Exponent(m);
      if (active && r == 0)
        exponent += e;
      return ScalePow2(v, -e);
    }
    if (active && r == 0)
      zero = 1;
    return v;
  }

  template <bool kCta> __device__ void Forward(const Team<kCta> &team) {
    const unsigned K = c.K;
    for (unsigned s = 0; s < c.prog.step_count; ++s) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      switch (step.kind) {
      case kStepRake:
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          const uint4 op = static_cast<const uint4 *>(c.a.rakes)[step.offset + i];
          Compute v = Compute(0);
          if (r < K) {
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              if (j < K)
                v = fma(Path(op.x, r, j), Node(op.y, j), v);
          }
          v = Normalize(v, active, r);
          if (active && r < K)
            c.branches[static_cast<std::size_t>(op.z) * K + r] = v;
        });
        break;
      case kStepCombine:
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          const uint2 op = static_cast<const uint2 *>(c.a.combines)[step.offset + i];
          Compute v = Compute(0);
          if (r < K)
            v = c.branches[static_cast<std::size_t>(op.x) * K + r] *
                c.branches[static_cast<std::size_t>(op.y) * K + r];
          v = Normalize(v, active, r);
          if (active && r < K)
            c.branches[static_cast<std::size_t>(op.x) * K + r] = v;
        });
        break;
      case kStepAbsorb:
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          const uint2 op = static_cast<const uint2 *>(c.a.absorbs)[step.offset + i];
          const unsigned node = op.x & kMask;
          Compute v = Compute(0);
          if (r < K) {
            const Compute previous =
                (op.x & kFlag) ? static_cast<Compute>(c.InputNode(node, r))
                               : c.nodes[static_cast<std::size_t>(node) * K + r];
            v = previous * c.branches[static_cast<std::size_t>(op.y) * K + r];
          }
          v = Normalize(v, active, r);
          if (active && r < K)
            c.nodes[static_cast<std::size_t>(node) * K + r] = v;
        });
        break;
      case kStepCompress:
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          const uint4 op = static_cast<const uint4 *>(c.a.compress)[2 * (step.offset + i)];
          Compute out[KMAX];
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            out[j] = Compute(0);
          if (r < K) {
            for (unsigned m = 0; m < K; ++m) {
              const Compute weight = Path(op.x, r, m) * Node(op.y, m);
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                if (j < K)
                  out[j] = fma(weight, Path(op.z, m, j), out[j]);
            }
          }
          Compute row_max = Compute(0);
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            row_max = row_max < out[j] ? out[j] : row_max;
          const Compute m = GroupMax<G>(row_max);
          int e = 0;
          if (m > Compute(0))
            e = Pow2Exponent(m);
          if (active && r == 0) {
            if (m > Compute(0))
              exponent += e;
            else
              zero = 1;
            if (c.a.reverse)
              comp_exp[op.w] = e;
          }
          if (active && r < K) {
            Compute *dst = c.comps + static_cast<std::size_t>(op.w) * c.KK + r * K;
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              if (j < K)
                dst[j] = ScalePow2(out[j], -e);
          }
        });
        break;
      }
      team.sync();
    }
  }

  // d log Z / d log(factor) for every node and edge of the instance.
  template <bool kCta> __device__ void Reverse(const Team<kCta> &team) {
    const unsigned K = c.K;
    Scalar *node_out = static_cast<Scalar *>(c.a.node_out) + c.inst.node_base * K;
    Scalar *edge_out = static_cast<Scalar *>(c.a.edge_out) +
                       c.inst.edge_out_base * static_cast<std::uint64_t>(c.KK);
    // Stores the adjoint of one row entry of path version `ref`.
    const auto store_path_adjoint = [&](unsigned ref, unsigned i, unsigned j,
                                        Compute value) {
      if (ref & kFlag)
        comp_mu[static_cast<std::size_t>(ref & kMask) * c.KK + i * K + j] = value;
      else
        edge_out[static_cast<std::size_t>(ref) * c.KK + i * K + j] =
            static_cast<Scalar>(value);
    };
    for (unsigned s = c.prog.step_count; s-- > 0;) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      if (step.kind == kStepRake) {
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          const uint4 op = static_cast<const uint4 *>(c.a.rakes)[step.offset + i];
          Compute leaf[KMAX];
          Compute row[KMAX];
          Compute unnormalised = Compute(0);
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j) {
            leaf[j] = j < K ? Node(op.y, j) : Compute(0);
            row[j] = (r < K && j < K) ? Path(op.x, r, j) : Compute(0);
            unnormalised = fma(row[j], leaf[j], unnormalised);
          }
          const Compute parent_adjoint =
              r < K ? static_cast<Compute>(
                          node_out[static_cast<std::size_t>(op.w) * K + r])
                    : Compute(0);
          const Compute ratio = unnormalised > Compute(0)
                                    ? parent_adjoint / unnormalised
                                    : Compute(0);
          if (active && r < K) {
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              if (j < K)
                store_path_adjoint(op.x, r, j, ratio * row[j] * leaf[j]);
          }
          // Leaf adjoint of state r: leaf[r] * sum_p ratio_p * path[p][r].
          Compute column = Compute(0);
          for (unsigned p = 0; p < K; ++p) {
            const Compute ratio_p = GroupBroadcast<G>(ratio, static_cast<int>(p));
            if (r < K)
              column = fma(ratio_p, Path(op.x, p, r), column);
          }
          if (active && r < K)
            node_out[static_cast<std::size_t>(op.y & kMask) * K + r] =
                static_cast<Scalar>(Node(op.y, r) * column);
        });
        team.sync();
      } else if (step.kind == kStepCompress) {
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          const uint4 op = static_cast<const uint4 *>(c.a.compress)[2 * (step.offset + i)];
          const int e = comp_exp[op.w];
          const Compute *output = c.comps + static_cast<std::size_t>(op.w) * c.KK;
          const Compute *output_adjoint = comp_mu + static_cast<std::size_t>(op.w) * c.KK;
          // ratio[j] = adjoint / unnormalised output, row r.
          Compute ratio[KMAX];
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j) {
            ratio[j] = Compute(0);
            if (r < K && j < K) {
              const Compute value = output[r * K + j];
              if (value > Compute(0))
                ratio[j] = ScalePow2(output_adjoint[r * K + j] / value, -e);
            }
          }
          // Left adjoint, row r: left[r][m] middle[m] sum_j right[m][j] ratio[j].
          if (r < K) {
            for (unsigned m = 0; m < K; ++m) {
              Compute dot = Compute(0);
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                if (j < K)
                  dot = fma(Path(op.z, m, j), ratio[j], dot);
              if (active)
                store_path_adjoint(op.x, r, m, Path(op.x, r, m) * Node(op.y, m) * dot);
            }
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              if (j < K)
                group_buffer[r * K + j] = ratio[j];
          }
          __syncwarp();
          // Right adjoint, row m = r: right[m][j] middle[m] sum_p left[p][m] ratio[p][j].
          if (r < K) {
            Compute acc[KMAX];
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              acc[j] = Compute(0);
            for (unsigned p = 0; p < K; ++p) {
              const Compute left = Path(op.x, p, r);
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                if (j < K)
                  acc[j] = fma(left, group_buffer[p * K + j], acc[j]);
            }
            const Compute middle = Node(op.y, r);
            Compute middle_adjoint = Compute(0);
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j) {
              if (j < K) {
                const Compute value = Path(op.z, r, j) * middle * acc[j];
                middle_adjoint += value;
                if (active)
                  store_path_adjoint(op.z, r, j, value);
              }
            }
            if (active)
              node_out[static_cast<std::size_t>(op.y & kMask) * K + r] =
                  static_cast<Scalar>(middle_adjoint);
          }
          __syncwarp();
        });
        team.sync();
      }
    }
  }

  template <bool kCta>
  __device__ void Run(const Team<kCta> &team, unsigned item, SharedState &sh) {
    Forward(team);
    long long total = exponent;
    int flag = zero;
    TeamReduce(team, total, flag, sh.warp_totals, sh.warp_flags);
    const unsigned K = c.K;
    if (team.tid == 0) {
      double sum = 0.0;
      for (unsigned j = 0; j < K; ++j)
        sum += static_cast<double>(Node(c.prog.root, j));
      const double log_z =
          (flag || !(sum > 0.0))
              ? -INFINITY
              : static_cast<double>(total) * 0.6931471805599453094 + log(sum);
      static_cast<Scalar *>(c.a.values)[item] =
          static_cast<Scalar>(c.a.raw ? exp(log_z) : log_z);
      if (c.a.reverse) {
        Scalar *root_out = static_cast<Scalar *>(c.a.node_out) +
                           (c.inst.node_base + (c.prog.root & kMask)) * K;
        const bool finite = log_z > -INFINITY;
        for (unsigned j = 0; j < K; ++j)
          root_out[j] = static_cast<Scalar>(
              finite ? static_cast<double>(Node(c.prog.root, j)) / sum : 0.0);
      }
    }
    if (c.a.reverse) {
      team.sync();
      Reverse(team);
    }
  }
};

// -------------------------------------------------------- max-product --
template <typename T, int KMAX> struct MaxEngine {
  static constexpr int G = KMAX;
  using Ctx = Context<T, T, KMAX>;
  Ctx c;
  std::uint8_t *rake_choices;
  std::uint8_t *comp_choices;

  __device__ MaxEngine(const EngineArgs &args, unsigned item, T *, unsigned)
      : c(args, item) {
    rake_choices = args.bytes + c.inst.byte_base;
    comp_choices = rake_choices + static_cast<std::size_t>(c.prog.num_rakes) * c.K;
  }

  __device__ __forceinline__ T Node(unsigned ref, unsigned j) const {
    return (ref & kFlag) ? c.nodes[static_cast<std::size_t>(ref & kMask) * c.K + j]
                         : PotentialLog(c.InputNode(ref, j));
  }
  __device__ __forceinline__ T Path(unsigned ref, unsigned i, unsigned j) const {
    return (ref & kFlag)
               ? c.comps[static_cast<std::size_t>(ref & kMask) * c.KK + i * c.K + j]
               : PotentialLog(c.InputEdge(ref, i, j));
  }

  template <bool kCta>
  __device__ void Run(const Team<kCta> &team, unsigned item, SharedState &) {
    const unsigned K = c.K;
    for (unsigned s = 0; s < c.prog.step_count; ++s) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      switch (step.kind) {
      case kStepRake: // src/inference.cc:576-594
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          if (!active || r >= K)
            return;
          const uint4 op = static_cast<const uint4 *>(c.a.rakes)[step.offset + i];
          T best = Path(op.x, r, 0) + Node(op.y, 0);
          unsigned choice = 0;
          for (unsigned j = 1; j < K; ++j) {
            const T term = Path(op.x, r, j) + Node(op.y, j);
            if (term > best) {
              best = term;
              choice = j;
            }
          }
          c.branches[static_cast<std::size_t>(op.z) * K + r] = best;
          rake_choices[static_cast<std::size_t>(op.z) * K + r] =
              static_cast<std::uint8_t>(choice);
        });
        break;
      case kStepCombine: // src/inference.cc:596-603
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          if (!active || r >= K)
            return;
          const uint2 op = static_cast<const uint2 *>(c.a.combines)[step.offset + i];
          T *dst = c.branches + static_cast<std::size_t>(op.x) * K + r;
          *dst = *dst + c.branches[static_cast<std::size_t>(op.y) * K + r];
        });
        break;
      case kStepAbsorb: // src/inference.cc:605-612
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          if (!active || r >= K)
            return;
          const uint2 op = static_cast<const uint2 *>(c.a.absorbs)[step.offset + i];
          const unsigned node = op.x & kMask;
          T *dst = c.nodes + static_cast<std::size_t>(node) * K + r;
          const T previous =
              (op.x & kFlag) ? PotentialLog(c.InputNode(node, r)) : *dst;
          *dst = previous + c.branches[static_cast<std::size_t>(op.y) * K + r];
        });
        break;
      case kStepCompress: // src/inference.cc:614-639
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          if (!active || r >= K)
            return;
          const uint4 op = static_cast<const uint4 *>(c.a.compress)[2 * (step.offset + i)];
          T best[KMAX];
          unsigned char choice[KMAX];
          {
            const T head = Path(op.x, r, 0) + Node(op.y, 0);
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j) {
              best[j] = j < K ? head + Path(op.z, 0, j) : T(0);
              choice[j] = 0;
            }
          }
          for (unsigned m = 1; m < K; ++m) {
            const T head = Path(op.x, r, m) + Node(op.y, m);
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j) {
              if (j < K) {
                const T term = head + Path(op.z, m, j);
                if (term > best[j]) {
                  best[j] = term;
                  choice[j] = static_cast<unsigned char>(m);
                }
              }
            }
          }
          T *dst = c.comps + static_cast<std::size_t>(op.w) * c.KK + r * K;
          std::uint8_t *ch = comp_choices + static_cast<std::size_t>(op.w) * c.KK + r * K;
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j) {
            if (j < K) {
              dst[j] = best[j];
              ch[j] = choice[j];
            }
          }
        });
        break;
      }
      team.sync();
    }
    std::uint32_t *states = c.a.states_out + c.inst.node_base;
    const unsigned root = c.prog.root & kMask;
    if (team.tid == 0) { // FinishRoot, src/inference.cc:641-649
      T best = Node(c.prog.root, 0);
      unsigned choice = 0;
      for (unsigned j = 1; j < K; ++j) {
        const T value = Node(c.prog.root, j);
        if (value > best) {
          best = value;
          choice = j;
        }
      }
      static_cast<T *>(c.a.values)[item] = best;
      states[root] = choice;
    }
    team.sync();
    // ExpandRakes / ExpandCompressions, src/inference.cc:651-667.
    for (unsigned s = c.prog.step_count; s-- > 0;) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      if (step.kind == kStepRake) {
        ForThreads(team, step.count, [&](unsigned i) {
          const uint4 op = static_cast<const uint4 *>(c.a.rakes)[step.offset + i];
          states[op.y & kMask] =
              rake_choices[static_cast<std::size_t>(op.z) * K + states[op.w]];
        });
        team.sync();
      } else if (step.kind == kStepCompress) {
        ForThreads(team, step.count, [&](unsigned i) {
          const uint4 *ops = static_cast<const uint4 *>(c.a.compress) + 2 * (step.offset + i);
          const uint4 op = ops[0];
          const uint4 ends = ops[1];
          states[op.y & kMask] =
              comp_choices[static_cast<std::size_t>(op.w) * c.KK +
                           states[ends.x] * K + states[ends.y]];
        });
        team.sync();
      }
    }
  }
};

// ------------------------------------------------------------ sampling --
// LogSumExp (src/inference.cc:100-110) over terms[0..K).
template <typename T, int KMAX>
__device__ __forceinline__ T LogSumExp(const T *terms, unsigned K) {
  T maximum = NegInf<T>();
#pragma unroll
  for (unsigned j = 0; j < KMAX; ++j)
    if (j < K)
      maximum = maximum < terms[j] ? terms[j] : maximum;
  if (!isfinite(maximum))
    return maximum;
  T sum = T(0);
#pragma unroll
  for (unsigned j = 0; j < KMAX; ++j)
    if (j < K)
      sum = sum + PortableExp(terms[j] - maximum);
  return maximum + PortableLog(sum);
}

// SampleLogWeights (src/inference.cc:128-146); returns K when no term is
// finite.
template <typename T, int KMAX>
__device__ __forceinline__ unsigned SampleLogWeights(const T *terms, unsigned K,
                                                     T normalizer, T uniform) {
  T cumulative = T(0);
  unsigned last = K;
#pragma unroll
  for (unsigned j = 0; j < KMAX; ++j) {
    if (j < K && isfinite(terms[j])) {
      last = j;
      cumulative = cumulative + PortableExp(terms[j] - normalizer);
      if (uniform < cumulative)
        return j;
    }
  }
  return last;
}

template <typename T, int KMAX> struct SampleEngine {
  static constexpr int G = KMAX;
  using Ctx = Context<T, T, KMAX>;
  Ctx c;

  __device__ SampleEngine(const EngineArgs &args, unsigned item, T *, unsigned)
      : c(args, item) {}

  __device__ __forceinline__ T Node(unsigned ref, unsigned j) const {
    return (ref & kFlag) ? c.nodes[static_cast<std::size_t>(ref & kMask) * c.K + j]
                         : PotentialLog(c.InputNode(ref, j));
  }
  __device__ __forceinline__ T Path(unsigned ref, unsigned i, unsigned j) const {
    return (ref & kFlag)
               ? c.comps[static_cast<std::size_t>(ref & kMask) * c.KK + i * c.K + j]
               : PotentialLog(c.InputEdge(ref, i, j));
  }

  __device__ __forceinline__ unsigned Draw(const T *terms, T normalizer,
                                           unsigned node) const {
    const T uniform = static_cast<const T *>(c.a.uniforms)[c.inst.node_base + node];
    if (!(uniform >= T(0) && uniform < T(1)))
      atomicOr(c.a.error, kErrorInvalidUniform);
    const unsigned choice = SampleLogWeights<T, KMAX>(terms, c.K, normalizer, uniform);
    if (choice >= c.K) {
      atomicOr(c.a.error, kErrorEmptyConditional);
      return 0;
    }
    return choice;
  }

  template <bool kCta>
  __device__ void Run(const Team<kCta> &team, unsigned item, SharedState &) {
    const unsigned K = c.K;
    for (unsigned s = 0; s < c.prog.step_count; ++s) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      switch (step.kind) {
      case kStepRake: // src/inference.cc:259-277
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          if (!active || r >= K)
            return;
          const uint4 op = static_cast<const uint4 *>(c.a.rakes)[step.offset + i];
          T terms[KMAX];
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            terms[j] = j < K ? Path(op.x, r, j) + Node(op.y, j) : T(0);
          c.branches[static_cast<std::size_t>(op.z) * K + r] =
              LogSumExp<T, KMAX>(terms, K);
        });
        break;
      case kStepCombine: // src/inference.cc:279-286
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          if (!active || r >= K)
            return;
          const uint2 op = static_cast<const uint2 *>(c.a.combines)[step.offset + i];
          T *dst = c.branches + static_cast<std::size_t>(op.x) * K + r;
          *dst = *dst + c.branches[static_cast<std::size_t>(op.y) * K + r];
        });
        break;
      case kStepAbsorb: // src/inference.cc:288-295
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          if (!active || r >= K)
            return;
          const uint2 op = static_cast<const uint2 *>(c.a.absorbs)[step.offset + i];
          const unsigned node = op.x & kMask;
          T *dst = c.nodes + static_cast<std::size_t>(node) * K + r;
          const T previous =
              (op.x & kFlag) ? PotentialLog(c.InputNode(node, r)) : *dst;
          *dst = previous + c.branches[static_cast<std::size_t>(op.y) * K + r];
        });
        break;
      case kStepCompress: // src/inference.cc:297-324
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned r) {
          if (!active || r >= K)
            return;
          const uint4 op = static_cast<const uint4 *>(c.a.compress)[2 * (step.offset + i)];
          T head[KMAX];
#pragma unroll
          for (unsigned m = 0; m < KMAX; ++m)
            head[m] = m < K ? Path(op.x, r, m) + Node(op.y, m) : T(0);
          T *dst = c.comps + static_cast<std::size_t>(op.w) * c.KK + r * K;
          for (unsigned j = 0; j < K; ++j) {
            T terms[KMAX];
#pragma unroll
            for (unsigned m = 0; m < KMAX; ++m)
              terms[m] = m < K ? head[m] + Path(op.z, m, j) : T(0);
            dst[j] = LogSumExp<T, KMAX>(terms, K);
          }
        });
        break;
      }
      team.sync();
    }
    std::uint32_t *states = c.a.states_out + c.inst.node_base;
    const unsigned root = c.prog.root & kMask;
    if (team.tid == 0) { // FinishRoot + SeedRootSample, src/inference.cc:326-361
      T terms[KMAX];
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        terms[j] = j < K ? Node(c.prog.root, j) : T(0);
      const T log_z = LogSumExp<T, KMAX>(terms, K);
      static_cast<T *>(c.a.values)[item] = log_z;
      states[root] = isfinite(log_z) ? Draw(terms, log_z, root) : 0u;
    }
    team.sync();
    // ExpandRakes / ExpandCompressions, src/inference.cc:363-412.
    for (unsigned s = c.prog.step_count; s-- > 0;) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      if (step.kind == kStepRake) {
        ForThreads(team, step.count, [&](unsigned i) {
          const uint4 op = static_cast<const uint4 *>(c.a.rakes)[step.offset + i];
          const unsigned parent_state = states[op.w];
          T terms[KMAX];
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            terms[j] = j < K ? Path(op.x, parent_state, j) + Node(op.y, j) : T(0);
          const T normalizer = LogSumExp<T, KMAX>(terms, K);
          states[op.y & kMask] = Draw(terms, normalizer, op.y & kMask);
        });
        team.sync();
      } else if (step.kind == kStepCompress) {
        ForThreads(team, step.count, [&](unsigned i) {
          const uint4 *ops = static_cast<const uint4 *>(c.a.compress) + 2 * (step.offset + i);
          const uint4 op = ops[0];
          const uint4 ends = ops[1];
          const unsigned parent_state = states[ends.x];
          const unsigned child_state = states[ends.y];
          T terms[KMAX];
#pragma unroll
          for (unsigned m = 0; m < KMAX; ++m)
            terms[m] = m < K ? Path(op.x, parent_state, m) + Node(op.y, m) +
                                   Path(op.z, m, child_state)
                             : T(0);
          const T normalizer = LogSumExp<T, KMAX>(terms, K);
          states[op.y & kMask] = Draw(terms, normalizer, op.y & kMask);
        });
        team.sync();
      }
    }
  }
};

// --------------------------------------------------------------- kernel --
template <class Engine, typename Buffer>
__global__ void __launch_bounds__(kThreads) EngineKernel(EngineArgs args) {
  extern __shared__ __align__(16) unsigned char dynamic_smem[];
  __shared__ SharedState shared;
  Buffer *buffers = reinterpret_cast<Buffer *>(dynamic_smem);
  const unsigned warp = threadIdx.x / 32;
  const unsigned lane = threadIdx.x & 31;
  Buffer *warp_buffer = buffers + warp * 32 * Engine::G;

  const Team<true> cta{threadIdx.x, blockDim.x};
  for (;;) {
    if (threadIdx.x == 0)
      shared.item = atomicAdd(&args.queue[0], 1u);
    __syncthreads();
    const unsigned index = shared.item;
    __syncthreads();
    if (index >= args.big_count)
      break;
    const unsigned item = args.big_items[index];
    Engine engine(args, item, warp_buffer, lane);
    engine.Run(cta, item, shared);
    __syncthreads();
  }
  const Team<false> single{lane, 32};
  for (;;) {
    unsigned index = 0;
    if (lane == 0)
      index = atomicAdd(&args.queue[1], 1u);
    index = __shfl_sync(kFull, index, 0);
    if (index >= args.small_count)
      break;
    const unsigned item = args.small_items[index];
    Engine engine(args, item, warp_buffer, lane);
    engine.Run(single, item, shared);
    __syncwarp();
  }
}

} // namespace thmm

#endif // THMM_ENGINE_CUH_
