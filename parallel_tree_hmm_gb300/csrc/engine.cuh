// Persistent tree-contraction kernels for sm_103a.
//
// Work decomposition. A *team* contracts one tree instance at a time: a whole
// CTA (128 threads) for large trees, a single warp for small ones. Instances
// come from two queues (largest first) through one atomic counter each; a CTA
// drains the large-tree queue first and then splits into four warp teams for
// the small trees. Inside a team the plan's steps run in order with a team
// barrier in between (the operations of one step are independent, as in a
// btrc::PrimitiveBatch). Each operation of a step is handled by a *group* of
// G lanes of one warp: G = 1 for K <= 4 (one thread per operation, K-vectors
// and K x K matrices in registers, 16-byte vector loads), G = KMAX otherwise
// (lane r owns row r; state reductions are warp shuffles). There are no
// grid-wide barriers and no spin waits.
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

// 128-thread CTAs: measured fastest on the uneven K=4 forest against
// 64/256/512 threads.
#ifndef THMM_CTA_THREADS
#define THMM_CTA_THREADS 128
#endif
#ifndef THMM_FORWARD_MIN_CTAS_K4
#define THMM_FORWARD_MIN_CTAS_K4 6
#endif
#ifndef THMM_REVERSE_MIN_CTAS_K4
#define THMM_REVERSE_MIN_CTAS_K4 5
#endif
constexpr int kThreads = THMM_CTA_THREADS;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;

// Lanes per operation group for a padded state count: one lane per row, the
// group a power of two (shuffle width); lanes beyond K hold zero rows.
template <int KMAX> constexpr int GroupLanes() {
  return KMAX <= 4 ? 1 : KMAX <= 8 ? 8 : KMAX <= 16 ? 16 : 32;
}

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
  const unsigned long long bits =
      static_cast<unsigned long long>(__double_as_longlong(m));
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

// a[i] for a register array without dynamic indexing (no local memory).
template <int N, typename T>
__device__ __forceinline__ T Select(const T (&a)[N], unsigned i) {
  T v = a[0];
#pragma unroll
  for (unsigned j = 1; j < N; ++j)
    if (j == i)
      v = a[j];
  return v;
}

// Loads K <= KMAX values (zero-padded to KMAX), converting to Dst; uses one
// or two 16-byte loads for a full row of four floats or doubles.
template <int KMAX, typename Src, typename Dst>
__device__ __forceinline__ void LoadRow(const Src *p, unsigned K, Dst (&out)[KMAX]) {
  if constexpr (KMAX == 4 && sizeof(Src) == 4) {
    if (K == 4) {
      const float4 v = *reinterpret_cast<const float4 *>(p);
      out[0] = static_cast<Dst>(v.x);
      out[1] = static_cast<Dst>(v.y);
      out[2] = static_cast<Dst>(v.z);
      out[3] = static_cast<Dst>(v.w);
      return;
    }
  }
  if constexpr (KMAX == 4 && sizeof(Src) == 8) {
    if (K == 4) {
      const double2 a = reinterpret_cast<const double2 *>(p)[0];
      const double2 b = reinterpret_cast<const double2 *>(p)[1];
      out[0] = static_cast<Dst>(a.x);
      out[1] = static_cast<Dst>(a.y);
      out[2] = static_cast<Dst>(b.x);
      out[3] = static_cast<Dst>(b.y);
      return;
    }
  }
  if constexpr (KMAX >= 16 && KMAX % 4 == 0 && sizeof(Src) == 4) {
    // Rows of K % 4 == 0 floats start on 16-byte boundaries: quads (from 16
    // states up, where they cut the load count; at 8 they measured no gain).
    if (K % 4 == 0 && (reinterpret_cast<std::uintptr_t>(p) & 15u) == 0) {
#pragma unroll
      for (unsigned q = 0; q < KMAX / 4; ++q) {
        if (4 * q < K) {
          const float4 v = reinterpret_cast<const float4 *>(p)[q];
          out[4 * q] = static_cast<Dst>(v.x);
          out[4 * q + 1] = static_cast<Dst>(v.y);
          out[4 * q + 2] = static_cast<Dst>(v.z);
          out[4 * q + 3] = static_cast<Dst>(v.w);
        } else {
          out[4 * q] = out[4 * q + 1] = out[4 * q + 2] = out[4 * q + 3] = Dst(0);
        }
      }
      return;
    }
  }
#pragma unroll
  for (unsigned j = 0; j < KMAX; ++j)
    out[j] = j < K ? static_cast<Dst>(p[j]) : Dst(0);
}

template <int KMAX, typename Dst, typename Src>
__device__ __forceinline__ void StoreRow(Dst *p, unsigned K, const Src (&in)[KMAX]) {
  if constexpr (KMAX == 4 && sizeof(Dst) == 4) {
    if (K == 4) {
      *reinterpret_cast<float4 *>(p) =
          make_float4(static_cast<float>(in[0]), static_cast<float>(in[1]),
                      static_cast<float>(in[2]), static_cast<float>(in[3]));
      return;
    }
  }
  if constexpr (KMAX == 4 && sizeof(Dst) == 8) {
    if (K == 4) {
      reinterpret_cast<double2 *>(p)[0] =
          make_double2(static_cast<double>(in[0]), static_cast<double>(in[1]));
      reinterpret_cast<double2 *>(p)[1] =
          make_double2(static_cast<double>(in[2]), static_cast<double>(in[3]));
      return;
    }
  }
  if constexpr (KMAX >= 16 && KMAX % 4 == 0 && sizeof(Dst) == 4) {
    if (K % 4 == 0 && (reinterpret_cast<std::uintptr_t>(p) & 15u) == 0) {
#pragma unroll
      for (unsigned q = 0; q < KMAX / 4; ++q)
        if (4 * q < K)
          reinterpret_cast<float4 *>(p)[q] =
              make_float4(static_cast<float>(in[4 * q]), static_cast<float>(in[4 * q + 1]),
                          static_cast<float>(in[4 * q + 2]), static_cast<float>(in[4 * q + 3]));
      return;
    }
  }
#pragma unroll
  for (unsigned j = 0; j < KMAX; ++j)
    if (j < K)
      p[j] = static_cast<Dst>(in[j]);
}

// StoreRow with streaming (evict-first) stores, for outputs that are never
// read back by the kernel.
template <int KMAX, typename Dst, typename Src>
__device__ __forceinline__ void StoreRowStreaming(Dst *p, unsigned K,
                                                  const Src (&in)[KMAX]) {
  if constexpr (KMAX == 4 && sizeof(Dst) == 4) {
    if (K == 4) {
      __stcs(reinterpret_cast<float4 *>(p),
             make_float4(static_cast<float>(in[0]), static_cast<float>(in[1]),
                         static_cast<float>(in[2]), static_cast<float>(in[3])));
      return;
    }
  }
  if constexpr (KMAX == 4 && sizeof(Dst) == 8) {
    if (K == 4) {
      __stcs(reinterpret_cast<double2 *>(p),
             make_double2(static_cast<double>(in[0]), static_cast<double>(in[1])));
      __stcs(reinterpret_cast<double2 *>(p) + 1,
             make_double2(static_cast<double>(in[2]), static_cast<double>(in[3])));
      return;
    }
  }
#pragma unroll
  for (unsigned j = 0; j < KMAX; ++j)
    if (j < K)
      __stcs(p + j, static_cast<Dst>(in[j]));
}

// Asks the L2 to fetch [p, p + bytes) ahead of use (Blackwell bulk prefetch;
// a hint that changes no data). The range is trimmed to whole 16-byte blocks
// inside the given span.
__device__ __forceinline__ void PrefetchL2(const void *p, std::size_t bytes) {
  const std::size_t begin = (reinterpret_cast<std::size_t>(p) + 15) & ~std::size_t{15};
  const std::size_t end = (reinterpret_cast<std::size_t>(p) + bytes) & ~std::size_t{15};
  if (end <= begin)
    return;
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;"
               :
               : "l"(begin), "r"(static_cast<unsigned>(end - begin))
               : "memory");
}

// Prefetches the operation records of `step` (and, for a gather step, of its
// rakes) into L2.
__device__ __forceinline__ void PrefetchStep(const EngineArgs &a, const DevStep &step) {
  switch (step.kind) {
  case kStepRake:
    PrefetchL2(static_cast<const uint4 *>(a.rakes) + step.offset, step.count * 16ull);
    break;
  case kStepCombine:
    PrefetchL2(static_cast<const uint2 *>(a.combines) + step.offset, step.count * 8ull);
    break;
  case kStepAbsorb:
    PrefetchL2(static_cast<const uint4 *>(a.absorbs) + step.offset, step.count * 16ull);
    break;
  case kStepCompress:
    PrefetchL2(static_cast<const uint4 *>(a.compress) + step.offset, step.count * 16ull);
    break;
  case kStepGather:
    PrefetchL2(static_cast<const uint4 *>(a.gathers) + step.offset, step.count * 16ull);
    PrefetchL2(static_cast<const uint4 *>(a.rakes) + step.aux_offset,
               step.aux_count * 16ull);
    break;
  }
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

struct SharedState {
  unsigned item;
  long long warp_totals[kWarps];
  int warp_flags[kWarps];
};

// Team-wide sum of an exponent total and OR of a flag.
template <bool kCta>
__device__ __forceinline__ void TeamReduce(const Team<kCta> &team,
                                           long long &total, int &flag,
                                           SharedState &shared) {
#pragma unroll
  for (int offset = 16; offset > 0; offset >>= 1) {
    total += __shfl_xor_sync(kFull, total, offset);
    flag |= __shfl_xor_sync(kFull, flag, offset);
  }
  if constexpr (kCta) {
    const unsigned warp = team.tid / 32;
    if ((team.tid & 31) == 0) {
      shared.warp_totals[warp] = total;
      shared.warp_flags[warp] = flag;
    }
    __syncthreads();
    total = 0;
    flag = 0;
    for (unsigned w = 0; w < team.size / 32; ++w) {
      total += shared.warp_totals[w];
      flag |= shared.warp_flags[w];
    }
    __syncthreads();
  }
}

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

  // Input factor vector of `node`; for a categorical model the reference's
  // (root ? root_potential : 1) * emission[observation]
  // (src/gpu_backend_impl.inc:326-382), computed in Scalar precision.
  __device__ __forceinline__ void InputNode(unsigned node, unsigned obs,
                                            Scalar (&out)[KMAX]) const {
    if (!a.categorical) {
      LoadRow<KMAX>(static_cast<const Scalar *>(a.node_in) +
                        (inst.node_base + node) * K,
                    K, out);
      return;
    }
    const bool root = node == (prog.root & kMask);
    const Scalar *root_potential = static_cast<const Scalar *>(a.root_potential);
    if (obs == kNone) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = j < K ? (root ? root_potential[j] : Scalar(1)) : Scalar(0);
      return;
    }
    const unsigned category = a.observations[inst.obs_base + obs];
    if (category >= a.categories) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = Scalar(0);
      return;
    }
    LoadRow<KMAX>(static_cast<const Scalar *>(a.emission) + category * K, K, out);
    if (root) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = j < K ? root_potential[j] * out[j] : Scalar(0);
    }
  }

  __device__ __forceinline__ const Scalar *InputEdge(unsigned edge) const {
    return edge_in + static_cast<std::size_t>(edge) * KK;
  }
};

// ------------------------------------------------------- sum-product --
// The sum-product forward sweep (log Z, and the root marginal when marginals
// are wanted) and the adjoint sweep are separate launches: each gets its own
// register allocation, so the smaller forward runs at a higher occupancy.
enum LinearPart : int { kLinearForward = 0, kLinearReverse = 1 };

// Minimum resident CTAs per SM requested from the compiler for each part,
// padded state count and arithmetic width (a register cap of
// 65536 / (128 * n) per thread), chosen so that no variant spills much.
template <int KMAX, int kPart, bool kWide> constexpr int LinearMinBlocks() {
  if constexpr (KMAX <= 4 && !kWide)
    return kPart == kLinearForward ? THMM_FORWARD_MIN_CTAS_K4 : THMM_REVERSE_MIN_CTAS_K4;
  else if constexpr (KMAX <= 4)
    return kPart == kLinearForward ? 4 : 2;
  else if constexpr (KMAX <= 8 || (KMAX <= 16 && !kWide))
    return 4;
  else if constexpr (KMAX <= 24 && !kWide)
    return 3;
  else
    return 2;
}

template <typename Scalar, typename Compute, int KMAX, int kPart = kLinearForward>
struct LinearEngine {
  static constexpr int kMinBlocks = LinearMinBlocks<KMAX, kPart, sizeof(Compute) == 8>();
  static constexpr int G = GroupLanes<KMAX>();
  static constexpr int ROWS = (KMAX + G - 1) / G;
  using Ctx = Context<Scalar, Compute, KMAX>;
  Ctx c;
  Compute *comp_mu;
  Compute *group_tile; // K*K values per group (reverse compressions, G > 1)
  int exponent = 0;    // this thread's share of the log-scale exponent
  int zero = 0;        // some renormalised message was identically zero

  __device__ LinearEngine(const EngineArgs &args, unsigned item,
                          Compute *warp_buffer, unsigned lane_in_warp)
      : c(args, item) {
    comp_mu = c.comps + static_cast<std::size_t>(c.prog.num_compressions) * c.KK;
    group_tile = warp_buffer + (lane_in_warp / G) * KMAX * KMAX;
  }

  __device__ __forceinline__ void NodeVector(unsigned ref, unsigned obs,
                                             Compute (&out)[KMAX]) const {
    if (ref & kFlag) {
      LoadRow<KMAX>(c.nodes + static_cast<std::size_t>(ref & kMask) * c.K, c.K, out);
    } else {
      Scalar raw[KMAX];
      c.InputNode(ref, obs, raw);
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = static_cast<Compute>(raw[j]);
    }
  }
  __device__ __forceinline__ void PathRow(unsigned ref, unsigned r,
                                          Compute (&out)[KMAX]) const {
    if (r >= c.K) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = Compute(0);
    } else if (ref & kFlag) {
      LoadRow<KMAX>(c.comps + static_cast<std::size_t>(ref & kMask) * c.KK + r * c.K,
                    c.K, out);
    } else {
      LoadRow<KMAX>(c.InputEdge(ref) + r * c.K, c.K, out);
    }
  }
  __device__ __forceinline__ Compute PathElem(unsigned ref, unsigned i,
                                              unsigned j) const {
    return (ref & kFlag)
               ? c.comps[static_cast<std::size_t>(ref & kMask) * c.KK + i * c.K + j]
               : static_cast<Compute>(c.InputEdge(ref)[i * c.K + j]);
  }

  // Exponent e of the group maximum m = f 2^e, f in [0.5, 1); records it
  // (or the zero flag) once per operation.
  __device__ __forceinline__ int GroupExponent(Compute local_max, bool active,
                                               unsigned lane) {
    const Compute m = GroupMax<G>(local_max);
    if (m > Compute(0)) {
      const int e = Pow2Exponent(m);
      if (active && lane == 0)
        exponent += e;
      return e;
    }
    if (active && lane == 0)
      zero = 1;
    return 0;
  }

  // Multiplies rake message `rake` (path times leaf, renormalised) into the
  // K values v held by this group, then renormalises the product.
  __device__ __forceinline__ void AbsorbRake(const uint4 &rake, Compute (&v)[KMAX],
                                             bool active, unsigned lane) {
    Compute leaf[KMAX];
    NodeVector(rake.y, rake.w, leaf);
    Compute message[KMAX];
    Compute m = Compute(0);
#pragma unroll
    for (int q = 0; q < ROWS; ++q) {
      Compute row[KMAX];
      PathRow(rake.x, lane + q * G, row);
      Compute dot = Compute(0);
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        dot = fma(row[j], leaf[j], dot);
      message[q] = dot;
      m = m < dot ? dot : m;
    }
    int e = GroupExponent(m, active, lane);
    m = Compute(0);
#pragma unroll
    for (int q = 0; q < ROWS; ++q) {
      v[q] = v[q] * ScalePow2(message[q], -e);
      m = m < v[q] ? v[q] : m;
    }
    e = GroupExponent(m, active, lane);
#pragma unroll
    for (int q = 0; q < ROWS; ++q)
      v[q] = ScalePow2(v[q], -e);
  }

  // Sum-product forward over the fused step list (gather + compress).
  template <bool kCta> __device__ void Forward(const Team<kCta> &team) {
    const unsigned K = c.K;
    const uint4 *rakes = static_cast<const uint4 *>(c.a.rakes);
    const uint4 *gathers = static_cast<const uint4 *>(c.a.gathers);
    const uint4 *compress = static_cast<const uint4 *>(c.a.compress);
    if (team.tid == 0 && c.prog.fused_count != 0)
      PrefetchStep(c.a, c.a.steps[c.prog.fused_begin]);
    for (unsigned s = 0; s < c.prog.fused_count; ++s) {
      const DevStep step = c.a.steps[c.prog.fused_begin + s];
      if (team.tid == 0 && s + 1 < c.prog.fused_count)
        PrefetchStep(c.a, c.a.steps[c.prog.fused_begin + s + 1]);
      switch (step.kind) {
      case kStepGather:
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          const uint4 op = gathers[step.offset + i];
          const unsigned node = op.x & kMask;
          Compute *dst = c.nodes + static_cast<std::size_t>(node) * K;
          Compute v[KMAX];
          if constexpr (G == 1) {
            if (op.x & kFlag)
              NodeVector(node, op.y, v);
            else
              LoadRow<KMAX>(dst, K, v);
            for (unsigned k = 0; k < op.w; ++k)
              AbsorbRake(rakes[op.z + k], v, active, lane);
            if (active)
              StoreRow<KMAX>(dst, K, v);
          } else {
            if (op.x & kFlag) {
              Compute input[KMAX];
              NodeVector(node, op.y, input);
              v[0] = Select(input, lane);
            } else {
              v[0] = lane < K ? dst[lane] : Compute(0);
            }
            // Uniform trip count across the warp (groups share shuffles).
            const unsigned rounds = __reduce_max_sync(kFull, active ? op.w : 0u);
            for (unsigned k = 0; k < rounds; ++k) {
              const bool live = active && k < op.w;
              const uint4 rake = rakes[op.z + (live ? k : 0u)];
              Compute trial[KMAX];
              trial[0] = v[0];
              AbsorbRake(rake, trial, live, lane);
              if (live)
                v[0] = trial[0];
            }
            if (active && lane < K)
              dst[lane] = v[0];
          }
        });
        break;
      case kStepCompress:
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          const unsigned g = step.offset + i;
          const unsigned tape = g - c.prog.compress_base;
          const uint4 op = compress[g];
          Compute middle[KMAX];
          NodeVector(op.y, op.w, middle);
          Compute left[ROWS][KMAX];
          Compute out[ROWS][KMAX];
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            PathRow(op.x, lane + q * G, left[q]);
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              out[q][j] = Compute(0);
          }
#pragma unroll
          for (unsigned mid = 0; mid < KMAX; ++mid) {
            if (mid < K) {
              Compute right[KMAX];
              PathRow(op.z, mid, right);
#pragma unroll
              for (int q = 0; q < ROWS; ++q) {
                const Compute weight = left[q][mid] * middle[mid];
#pragma unroll
                for (unsigned j = 0; j < KMAX; ++j)
                  out[q][j] = fma(weight, right[j], out[q][j]);
              }
            }
          }
          Compute m = Compute(0);
#pragma unroll
          for (int q = 0; q < ROWS; ++q)
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              m = m < out[q][j] ? out[q][j] : m;
          const int e = GroupExponent(m, active, lane);
          if (active) {
#pragma unroll
            for (int q = 0; q < ROWS; ++q) {
              const unsigned r = lane + q * G;
              if (r < K) {
#pragma unroll
                for (unsigned j = 0; j < KMAX; ++j)
                  out[q][j] = ScalePow2(out[q][j], -e);
                StoreRow<KMAX>(c.comps + static_cast<std::size_t>(tape) * c.KK + r * K,
                               K, out[q]);
              }
            }
          }
        });
        break;
      }
      team.sync();
    }
  }

  // Stores row r of the adjoint of path version `ref` (an edge marginal for
  // an input edge, scratch for a compressed version).
  __device__ __forceinline__ void StorePathAdjoint(unsigned ref, unsigned r,
                                                   const Compute (&row)[KMAX],
                                                   Scalar *edge_out) const {
    if (ref & kFlag)
      StoreRow<KMAX>(comp_mu + static_cast<std::size_t>(ref & kMask) * c.KK + r * c.K,
                     c.K, row);
    else
      StoreRowStreaming<KMAX>(edge_out + static_cast<std::size_t>(ref) * c.KK + r * c.K,
                              c.K, row);
  }

  // d log Z / d log(factor) for every node and edge of the instance.
  template <bool kCta> __device__ void Reverse(const Team<kCta> &team) {
    const unsigned K = c.K;
    Scalar *node_out = static_cast<Scalar *>(c.a.node_out) + c.inst.node_base * K;
    Scalar *edge_out = static_cast<Scalar *>(c.a.edge_out) +
                       c.inst.edge_out_base * static_cast<std::uint64_t>(c.KK);
    const uint4 *rakes = static_cast<const uint4 *>(c.a.rakes);
    const uint4 *compress = static_cast<const uint4 *>(c.a.compress);
    for (unsigned s = c.prog.step_count; s-- > 0;) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      if (team.tid == 0) {
        for (unsigned ahead = s; ahead-- > 0;) {
          const DevStep next = c.a.steps[c.prog.step_begin + ahead];
          if (next.kind == kStepRake || next.kind == kStepCompress) {
            PrefetchStep(c.a, next);
            break;
          }
        }
      }
      if (step.kind == kStepRake) {
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          const uint4 op = rakes[step.offset + i];
          Compute leaf[KMAX];
          NodeVector(op.y, op.w, leaf);
          Compute parent_adjoint[KMAX];
          if constexpr (G == 1) {
            LoadRow<KMAX>(node_out + static_cast<std::size_t>(op.z) * K, K,
                          parent_adjoint);
          } else {
            parent_adjoint[0] =
                lane < K ? static_cast<Compute>(
                               node_out[static_cast<std::size_t>(op.z) * K + lane])
                         : Compute(0);
          }
          Compute ratio[ROWS];
          Compute rows[ROWS][KMAX];
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            PathRow(op.x, r, rows[q]);
            Compute unnormalised = Compute(0);
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              unnormalised = fma(rows[q][j], leaf[j], unnormalised);
            ratio[q] = unnormalised > Compute(0) ? parent_adjoint[q] / unnormalised
                                                 : Compute(0);
            if (active && r < K) {
              Compute w[KMAX];
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                w[j] = ratio[q] * rows[q][j] * leaf[j];
              StorePathAdjoint(op.x, r, w, edge_out);
            }
          }
          // Leaf adjoint: leaf[j] * sum_p ratio_p * path[p][j].
          if constexpr (G == 1) {
            Compute adjoint[KMAX];
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j) {
              Compute column = Compute(0);
#pragma unroll
              for (int p = 0; p < ROWS; ++p)
                column = fma(ratio[p], rows[p][j], column);
              adjoint[j] = leaf[j] * column;
            }
            if (active)
              StoreRow<KMAX>(node_out + static_cast<std::size_t>(op.y & kMask) * K, K,
                             adjoint);
          } else {
            Compute column = Compute(0);
            for (unsigned p = 0; p < K; ++p) {
              const Compute ratio_p = GroupBroadcast<G>(ratio[0], static_cast<int>(p));
              if (lane < K)
                column = fma(ratio_p, PathElem(op.x, p, lane), column);
            }
            if (active && lane < K) {
              Compute own = Compute(0);
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                if (j == lane)
                  own = leaf[j];
              node_out[static_cast<std::size_t>(op.y & kMask) * K + lane] =
                  static_cast<Scalar>(own * column);
            }
          }
        });
        team.sync();
      } else if (step.kind == kStepCompress) {
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          const unsigned g = step.offset + i;
          const unsigned tape = g - c.prog.compress_base;
          const uint4 op = compress[g];
          const Compute *output_adjoint = comp_mu + static_cast<std::size_t>(tape) * c.KK;
          Compute middle[KMAX];
          NodeVector(op.y, op.w, middle);
          // Unnormalised output rows r = lane + q G, recomputed with the
          // forward's operation order, and ratio = adjoint / output.
          Compute left[ROWS][KMAX];
          Compute ratio[ROWS][KMAX];
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            PathRow(op.x, lane + q * G, left[q]);
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              ratio[q][j] = Compute(0);
          }
#pragma unroll
          for (unsigned mid = 0; mid < KMAX; ++mid) {
            if (mid < K) {
              Compute right[KMAX];
              PathRow(op.z, mid, right);
#pragma unroll
              for (int q = 0; q < ROWS; ++q) {
                const Compute weight = left[q][mid] * middle[mid];
#pragma unroll
                for (unsigned j = 0; j < KMAX; ++j)
                  ratio[q][j] = fma(weight, right[j], ratio[q][j]);
              }
            }
          }
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            Compute adjoint[KMAX];
            if (r < K) {
              LoadRow<KMAX>(output_adjoint + r * K, K, adjoint);
            } else {
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                adjoint[j] = Compute(0);
            }
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              ratio[q][j] = ratio[q][j] > Compute(0) ? adjoint[j] / ratio[q][j]
                                                     : Compute(0);
          }
          // Left adjoint rows: left[r][m] middle[m] sum_j right[m][j] ratio[r][j],
          // one row at a time (stored as soon as it is complete).
          Compute rights[G == 1 ? KMAX : 1][KMAX];
          if constexpr (G == 1) {
#pragma unroll
            for (unsigned mid = 0; mid < KMAX; ++mid)
              PathRow(op.z, mid, rights[mid]);
          }
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            Compute left_adjoint[KMAX];
#pragma unroll
            for (unsigned mid = 0; mid < KMAX; ++mid) {
              left_adjoint[mid] = Compute(0);
              if (mid < K) {
                Compute right[KMAX];
                if constexpr (G == 1) {
#pragma unroll
                  for (unsigned j = 0; j < KMAX; ++j)
                    right[j] = rights[mid][j];
                } else {
                  PathRow(op.z, mid, right);
                }
                Compute dot = Compute(0);
#pragma unroll
                for (unsigned j = 0; j < KMAX; ++j)
                  dot = fma(right[j], ratio[q][j], dot);
                left_adjoint[mid] = left[q][mid] * middle[mid] * dot;
              }
            }
            if (active && lane + q * G < K)
              StorePathAdjoint(op.x, lane + q * G, left_adjoint, edge_out);
          }
          // Right adjoint rows m: right[m][j] middle[m] sum_p left[p][m] ratio[p][j].
          if constexpr (G == 1) {
            Compute middle_adjoint[KMAX];
#pragma unroll
            for (unsigned mid = 0; mid < KMAX; ++mid) {
              Compute right_adjoint[KMAX];
              Compute total = Compute(0);
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j) {
                Compute acc = Compute(0);
#pragma unroll
                for (int p = 0; p < ROWS; ++p)
                  acc = fma(left[p][mid], ratio[p][j], acc);
                right_adjoint[j] = rights[mid][j] * middle[mid] * acc;
                total += right_adjoint[j];
              }
              middle_adjoint[mid] = total;
              if (active && mid < K)
                StorePathAdjoint(op.z, mid, right_adjoint, edge_out);
            }
            if (active)
              StoreRow<KMAX>(node_out + static_cast<std::size_t>(op.y & kMask) * K, K,
                             middle_adjoint);
          } else {
            if (lane < K) {
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                if (j < K)
                  group_tile[lane * K + j] = ratio[0][j];
            }
            __syncwarp();
            if (lane < K) {
              Compute acc[KMAX];
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                acc[j] = Compute(0);
              for (unsigned p = 0; p < K; ++p) {
                const Compute left_p = PathElem(op.x, p, lane);
#pragma unroll
                for (unsigned j = 0; j < KMAX; ++j)
                  if (j < K)
                    acc[j] = fma(left_p, group_tile[p * K + j], acc[j]);
              }
              Compute own_middle = Compute(0);
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j)
                if (j == lane)
                  own_middle = middle[j];
              Compute right[KMAX];
              PathRow(op.z, lane, right);
              Compute right_adjoint[KMAX];
              Compute total = Compute(0);
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j) {
                right_adjoint[j] = right[j] * own_middle * acc[j];
                total += right_adjoint[j];
              }
              if (active) {
                StorePathAdjoint(op.z, lane, right_adjoint, edge_out);
                node_out[static_cast<std::size_t>(op.y & kMask) * K + lane] =
                    static_cast<Scalar>(total);
              }
            }
            __syncwarp();
          }
        });
        team.sync();
      }
    }
  }

  template <bool kCta>
  __device__ void Run(const Team<kCta> &team, unsigned item, SharedState &sh) {
    if constexpr (kPart == kLinearReverse) {
      Reverse(team);
      return;
    }
    Forward(team);
    long long total = exponent;
    int flag = zero;
    TeamReduce(team, total, flag, sh);
    const unsigned K = c.K;
    if (team.tid == 0) {
      Compute root[KMAX];
      NodeVector(c.prog.root, c.prog.root_obs, root);
      double sum = 0.0;
      for (unsigned j = 0; j < KMAX; ++j)
        sum += static_cast<double>(root[j]);
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
        for (unsigned j = 0; j < K; ++j) {
          double value = 0.0;
#pragma unroll
          for (unsigned k = 0; k < KMAX; ++k)
            if (k == j)
              value = static_cast<double>(root[k]);
          root_out[j] = static_cast<Scalar>(finite ? value / sum : 0.0);
        }
      }
    }
  }
};

// -------------------------------------------------- log-domain helpers --
template <typename T, int KMAX> struct LogContext {
  Context<T, T, KMAX> c;
  __device__ LogContext(const EngineArgs &args, unsigned item) : c(args, item) {}

  __device__ __forceinline__ void NodeVector(unsigned ref, unsigned obs,
                                             T (&out)[KMAX]) const {
    if (ref & kFlag) {
      LoadRow<KMAX>(c.nodes + static_cast<std::size_t>(ref & kMask) * c.K, c.K, out);
    } else {
      c.InputNode(ref, obs, out);
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = PotentialLog(out[j]);
    }
  }
  __device__ __forceinline__ void PathRow(unsigned ref, unsigned r,
                                          T (&out)[KMAX]) const {
    if (ref & kFlag) {
      LoadRow<KMAX>(c.comps + static_cast<std::size_t>(ref & kMask) * c.KK + r * c.K,
                    c.K, out);
    } else {
      LoadRow<KMAX>(c.InputEdge(ref) + r * c.K, c.K, out);
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = PotentialLog(out[j]);
    }
  }
  __device__ __forceinline__ T PathElem(unsigned ref, unsigned i, unsigned j) const {
    return (ref & kFlag)
               ? c.comps[static_cast<std::size_t>(ref & kMask) * c.KK + i * c.K + j]
               : PotentialLog(c.InputEdge(ref)[i * c.K + j]);
  }
};

// -------------------------------------------------------- max-product --
template <typename T, int KMAX> struct MaxEngine {
  static constexpr int kMinBlocks = KMAX <= 8 ? 4 : 2;
  static constexpr int G = GroupLanes<KMAX>();
  static constexpr int ROWS = (KMAX + G - 1) / G;
  LogContext<T, KMAX> lc;
  const Context<T, T, KMAX> &c;
  std::uint8_t *rake_choices;
  std::uint8_t *comp_choices;

  __device__ MaxEngine(const EngineArgs &args, unsigned item, T *, unsigned)
      : lc(args, item), c(lc.c) {
    rake_choices = args.bytes + c.inst.byte_base;
    comp_choices = rake_choices + static_cast<std::size_t>(c.prog.num_rakes) * c.K;
  }

  template <bool kCta>
  __device__ void Run(const Team<kCta> &team, unsigned item, SharedState &) {
    const unsigned K = c.K;
    const uint4 *rakes = static_cast<const uint4 *>(c.a.rakes);
    const uint2 *combines = static_cast<const uint2 *>(c.a.combines);
    const uint4 *absorbs = static_cast<const uint4 *>(c.a.absorbs);
    const uint4 *compress = static_cast<const uint4 *>(c.a.compress);
    for (unsigned s = 0; s < c.prog.step_count; ++s) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      switch (step.kind) {
      case kStepRake: // src/inference.cc:576-594
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          if (!active)
            return;
          const unsigned g = step.offset + i;
          const unsigned branch = g - c.prog.rake_base;
          const uint4 op = rakes[g];
          T leaf[KMAX];
          lc.NodeVector(op.y, op.w, leaf);
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            if (r >= K)
              continue;
            T row[KMAX];
            lc.PathRow(op.x, r, row);
            T best = row[0] + leaf[0];
            unsigned choice = 0;
#pragma unroll
            for (unsigned j = 1; j < KMAX; ++j) {
              if (j < K) {
                const T term = row[j] + leaf[j];
                if (term > best) {
                  best = term;
                  choice = j;
                }
              }
            }
            c.branches[static_cast<std::size_t>(branch) * K + r] = best;
            rake_choices[static_cast<std::size_t>(branch) * K + r] =
                static_cast<std::uint8_t>(choice);
          }
        });
        break;
      case kStepCombine: // src/inference.cc:596-603
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          if (!active)
            return;
          const uint2 op = combines[step.offset + i];
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            if (r < K) {
              T *dst = c.branches + static_cast<std::size_t>(op.x) * K + r;
              *dst = *dst + c.branches[static_cast<std::size_t>(op.y) * K + r];
            }
          }
        });
        break;
      case kStepAbsorb: // src/inference.cc:605-612
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          if (!active)
            return;
          const uint4 op = absorbs[step.offset + i];
          const unsigned node = op.x & kMask;
          T input[KMAX];
          if (op.x & kFlag)
            lc.NodeVector(node, op.z, input);
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            if (r < K) {
              T *dst = c.nodes + static_cast<std::size_t>(node) * K + r;
              T previous = *dst;
              if (op.x & kFlag) {
#pragma unroll
                for (unsigned j = 0; j < KMAX; ++j)
                  if (j == r)
                    previous = input[j];
              }
              *dst = previous + c.branches[static_cast<std::size_t>(op.y) * K + r];
            }
          }
        });
        break;
      case kStepCompress: // src/inference.cc:614-639
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          if (!active)
            return;
          const unsigned g = step.offset + i;
          const unsigned tape = g - c.prog.compress_base;
          const uint4 op = compress[g];
          T middle[KMAX];
          lc.NodeVector(op.y, op.w, middle);
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            if (r >= K)
              continue;
            T left[KMAX];
            lc.PathRow(op.x, r, left);
            T best[KMAX];
            unsigned char choice[KMAX];
            {
              T right[KMAX];
              lc.PathRow(op.z, 0, right);
              const T head = left[0] + middle[0];
#pragma unroll
              for (unsigned j = 0; j < KMAX; ++j) {
                best[j] = head + right[j];
                choice[j] = 0;
              }
            }
#pragma unroll
            for (unsigned m = 1; m < KMAX; ++m) {
              if (m < K) {
                T right[KMAX];
                lc.PathRow(op.z, m, right);
                const T head = left[m] + middle[m];
#pragma unroll
                for (unsigned j = 0; j < KMAX; ++j) {
                  const T term = head + right[j];
                  if (term > best[j]) {
                    best[j] = term;
                    choice[j] = static_cast<unsigned char>(m);
                  }
                }
              }
            }
            StoreRow<KMAX>(c.comps + static_cast<std::size_t>(tape) * c.KK + r * K, K,
                           best);
            std::uint8_t *ch =
                comp_choices + static_cast<std::size_t>(tape) * c.KK + r * K;
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              if (j < K)
                ch[j] = choice[j];
          }
        });
        break;
      }
      team.sync();
    }
    std::uint32_t *states = c.a.states_out + c.inst.node_base;
    const unsigned root = c.prog.root & kMask;
    if (team.tid == 0) { // FinishRoot, src/inference.cc:641-649
      T values[KMAX];
      lc.NodeVector(c.prog.root, c.prog.root_obs, values);
      T best = values[0];
      unsigned choice = 0;
#pragma unroll
      for (unsigned j = 1; j < KMAX; ++j) {
        if (j < K && values[j] > best) {
          best = values[j];
          choice = j;
        }
      }
      static_cast<T *>(c.a.values)[item] = best;
      states[root] = choice;
    }
    team.sync();
    // ExpandRakes / ExpandCompressions, src/inference.cc:651-667.
    const uint2 *ends = static_cast<const uint2 *>(c.a.compress_ends);
    for (unsigned s = c.prog.step_count; s-- > 0;) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      if (step.kind == kStepRake) {
        ForThreads(team, step.count, [&](unsigned i) {
          const unsigned g = step.offset + i;
          const uint4 op = rakes[g];
          states[op.y & kMask] =
              rake_choices[static_cast<std::size_t>(g - c.prog.rake_base) * K +
                           states[op.z]];
        });
        team.sync();
      } else if (step.kind == kStepCompress) {
        ForThreads(team, step.count, [&](unsigned i) {
          const unsigned g = step.offset + i;
          const uint4 op = compress[g];
          const uint2 end = ends[g];
          states[op.y & kMask] =
              comp_choices[static_cast<std::size_t>(g - c.prog.compress_base) * c.KK +
                           states[end.x] * K + states[end.y]];
        });
        team.sync();
      }
    }
  }
};

// ------------------------------------------------------------ sampling --
// LogSumExp (src/inference.cc:100-110) over terms[0..K).
template <typename T, int KMAX>
__device__ __forceinline__ T LogSumExp(const T (&terms)[KMAX], unsigned K) {
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
__device__ __forceinline__ unsigned SampleLogWeights(const T (&terms)[KMAX],
                                                     unsigned K, T normalizer,
                                                     T uniform) {
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
  static constexpr int kMinBlocks = KMAX <= 8 ? 4 : 2;
  static constexpr int G = GroupLanes<KMAX>();
  static constexpr int ROWS = (KMAX + G - 1) / G;
  LogContext<T, KMAX> lc;
  const Context<T, T, KMAX> &c;

  __device__ SampleEngine(const EngineArgs &args, unsigned item, T *, unsigned)
      : lc(args, item), c(lc.c) {}

  __device__ __forceinline__ unsigned Draw(const T (&terms)[KMAX], T normalizer,
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
    const uint4 *rakes = static_cast<const uint4 *>(c.a.rakes);
    const uint2 *combines = static_cast<const uint2 *>(c.a.combines);
    const uint4 *absorbs = static_cast<const uint4 *>(c.a.absorbs);
    const uint4 *compress = static_cast<const uint4 *>(c.a.compress);
    for (unsigned s = 0; s < c.prog.step_count; ++s) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      switch (step.kind) {
      case kStepRake: // src/inference.cc:259-277
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          if (!active)
            return;
          const unsigned g = step.offset + i;
          const unsigned branch = g - c.prog.rake_base;
          const uint4 op = rakes[g];
          T leaf[KMAX];
          lc.NodeVector(op.y, op.w, leaf);
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            if (r >= K)
              continue;
            T terms[KMAX];
            lc.PathRow(op.x, r, terms);
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              terms[j] = terms[j] + leaf[j];
            c.branches[static_cast<std::size_t>(branch) * K + r] =
                LogSumExp<T, KMAX>(terms, K);
          }
        });
        break;
      case kStepCombine: // src/inference.cc:279-286
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          if (!active)
            return;
          const uint2 op = combines[step.offset + i];
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            if (r < K) {
              T *dst = c.branches + static_cast<std::size_t>(op.x) * K + r;
              *dst = *dst + c.branches[static_cast<std::size_t>(op.y) * K + r];
            }
          }
        });
        break;
      case kStepAbsorb: // src/inference.cc:288-295
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          if (!active)
            return;
          const uint4 op = absorbs[step.offset + i];
          const unsigned node = op.x & kMask;
          T input[KMAX];
          if (op.x & kFlag)
            lc.NodeVector(node, op.z, input);
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            if (r < K) {
              T *dst = c.nodes + static_cast<std::size_t>(node) * K + r;
              T previous = *dst;
              if (op.x & kFlag) {
#pragma unroll
                for (unsigned j = 0; j < KMAX; ++j)
                  if (j == r)
                    previous = input[j];
              }
              *dst = previous + c.branches[static_cast<std::size_t>(op.y) * K + r];
            }
          }
        });
        break;
      case kStepCompress: // src/inference.cc:297-324
        ForGroups<G>(team, step.count, [&](unsigned i, bool active, unsigned lane) {
          if (!active)
            return;
          const unsigned g = step.offset + i;
          const unsigned tape = g - c.prog.compress_base;
          const uint4 op = compress[g];
          T middle[KMAX];
          lc.NodeVector(op.y, op.w, middle);
#pragma unroll
          for (int q = 0; q < ROWS; ++q) {
            const unsigned r = lane + q * G;
            if (r >= K)
              continue;
            T head[KMAX];
            lc.PathRow(op.x, r, head);
#pragma unroll
            for (unsigned m = 0; m < KMAX; ++m)
              head[m] = head[m] + middle[m];
            T *dst = c.comps + static_cast<std::size_t>(tape) * c.KK + r * K;
            for (unsigned j = 0; j < K; ++j) {
              T terms[KMAX];
#pragma unroll
              for (unsigned m = 0; m < KMAX; ++m)
                terms[m] = m < K ? head[m] + lc.PathElem(op.z, m, j) : T(0);
              dst[j] = LogSumExp<T, KMAX>(terms, K);
            }
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
      lc.NodeVector(c.prog.root, c.prog.root_obs, terms);
      const T log_z = LogSumExp<T, KMAX>(terms, K);
      static_cast<T *>(c.a.values)[item] = log_z;
      states[root] = isfinite(log_z) ? Draw(terms, log_z, root) : 0u;
    }
    team.sync();
    // ExpandRakes / ExpandCompressions, src/inference.cc:363-412.
    const uint2 *ends = static_cast<const uint2 *>(c.a.compress_ends);
    for (unsigned s = c.prog.step_count; s-- > 0;) {
      const DevStep step = c.a.steps[c.prog.step_begin + s];
      if (step.kind == kStepRake) {
        ForThreads(team, step.count, [&](unsigned i) {
          const uint4 op = rakes[step.offset + i];
          T leaf[KMAX], terms[KMAX];
          lc.NodeVector(op.y, op.w, leaf);
          lc.PathRow(op.x, states[op.z], terms);
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            terms[j] = terms[j] + leaf[j];
          const T normalizer = LogSumExp<T, KMAX>(terms, K);
          states[op.y & kMask] = Draw(terms, normalizer, op.y & kMask);
        });
        team.sync();
      } else if (step.kind == kStepCompress) {
        ForThreads(team, step.count, [&](unsigned i) {
          const unsigned g = step.offset + i;
          const uint4 op = compress[g];
          const uint2 end = ends[g];
          const unsigned parent_state = states[end.x];
          const unsigned child_state = states[end.y];
          T middle[KMAX], terms[KMAX];
          lc.NodeVector(op.y, op.w, middle);
          lc.PathRow(op.x, parent_state, terms);
#pragma unroll
          for (unsigned m = 0; m < KMAX; ++m)
            terms[m] = m < K ? terms[m] + middle[m] + lc.PathElem(op.z, m, child_state)
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
__global__ void __launch_bounds__(kThreads, Engine::kMinBlocks)
EngineKernel(EngineArgs args) {
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
