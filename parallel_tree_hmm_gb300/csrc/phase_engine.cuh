// Phase kernels of the level-synchronous schedule (phase.h) for padded state
// count 4 (K <= 4): one thread per operation (one warp per tree in the tail
// rounds), the K-vectors and K x K matrices in registers, 16-byte vector
// loads and stores.
//
// Each kernel performs exactly the floating-point operations of the
// one-thread-per-operation (G = 1) branch of LinearEngine (engine.cuh) in
// the same order, so the two schedules agree bit for bit; only the
// bookkeeping of the power-of-two exponents differs (carried per stored
// object here, summed per team there; both are exact integer sums).
#ifndef THMM_PHASE_ENGINE_CUH_
#define THMM_PHASE_ENGINE_CUH_

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.cuh"
#include "phase.h"

namespace thmm {

constexpr int kPhaseThreads = 128;

// Where the operands of one operation live. Forest layout: the records hold
// absolute indices of every tree's nodes, edges and compressions, so every
// map is the identity (a shared edge input is read modulo its edge count).
struct ForestIndex {
  __device__ __forceinline__ std::size_t Store(std::uint32_t node) const { return node; }
  __device__ __forceinline__ std::size_t Io(std::uint32_t node) const { return node; }
  __device__ __forceinline__ std::size_t Comp(std::uint32_t tape) const { return tape; }
  __device__ __forceinline__ std::size_t Out(std::uint32_t edge) const { return edge; }
  __device__ __forceinline__ std::size_t In(const PhaseArgs &a, std::uint32_t edge) const {
    return a.edge_modulus != 0 ? edge % a.edge_modulus : edge;
  }
  __device__ __forceinline__ std::size_t Obs(std::uint32_t slot) const { return slot; }
};

// Shared-topology layout (the reference's batch API: one plan, B node-factor
// sets, one edge input): the records are those of ONE tree and are read by
// every batch item, and consecutive threads take consecutive batch items of
// the same operation, so a warp reads each record and each edge row once
// (the addresses coincide) instead of once per item. Stored values are
// item-minor ([node][item]) so the warp's accesses are contiguous; the
// phase-ordered observations likewise ([slot][item]). Caller-visible arrays
// keep the reference's item-major layouts.
struct BatchIndex {
  std::uint32_t item;   // batch item of this thread
  std::uint64_t stride; // items per stored object (the batch capacity)
  std::uint64_t nodes;  // nodes per item
  std::uint64_t edges;  // edges per item
  __device__ __forceinline__ std::size_t Store(std::uint32_t node) const {
    return node * stride + item;
  }
  __device__ __forceinline__ std::size_t Io(std::uint32_t node) const {
    return item * nodes + node;
  }
  __device__ __forceinline__ std::size_t Comp(std::uint32_t tape) const {
    return tape * stride + item;
  }
  __device__ __forceinline__ std::size_t Out(std::uint32_t edge) const {
    return item * edges + edge;
  }
  __device__ __forceinline__ std::size_t In(const PhaseArgs &, std::uint32_t edge) const {
    return edge;
  }
  __device__ __forceinline__ std::size_t Obs(std::uint32_t slot) const {
    return slot * stride + item;
  }
};

template <typename Scalar, typename Compute, class Index> struct PhaseOps {
  static constexpr int KMAX = 4;
  const PhaseArgs &a;
  Index ix;
  unsigned K;
  unsigned KK;

  __device__ PhaseOps(const PhaseArgs &args, const Index &index)
      : a(args), ix(index), K(args.states), KK(args.states * args.states) {}

  // Input factor vector of `node`: dense row, or the reference's categorical
  // (root ? root_potential : 1) * emission[observation]
  // (src/gpu_backend_impl.inc:326-382), as Context::InputNode.
  __device__ __forceinline__ void Input(std::uint32_t node, std::uint32_t obs, bool root,
                                        Compute (&out)[KMAX]) const {
    Scalar raw[KMAX];
    if (!a.categorical) {
      LoadRow<KMAX>(static_cast<const Scalar *>(a.node_in) + ix.Io(node) * K, K, raw);
    } else {
      const Scalar *root_potential = static_cast<const Scalar *>(a.root_potential);
      if (obs == kNone) {
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          raw[j] = j < K ? (root ? root_potential[j] : Scalar(1)) : Scalar(0);
      } else {
        const unsigned category = a.observations[ix.Obs(obs)];
        if (category >= a.categories) {
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            raw[j] = Scalar(0);
        } else {
          LoadRow<KMAX>(static_cast<const Scalar *>(a.emission) + category * K, K, raw);
          if (root) {
#pragma unroll
            for (unsigned j = 0; j < KMAX; ++j)
              raw[j] = j < K ? root_potential[j] * raw[j] : Scalar(0);
          }
        }
      }
    }
#pragma unroll
    for (unsigned j = 0; j < KMAX; ++j)
      out[j] = static_cast<Compute>(raw[j]);
  }

  // Value of a rake leaf or compression middle: the stored value (adding its
  // exponent to `e`) or the input factor.
  __device__ __forceinline__ void Node(std::uint32_t ref, std::uint32_t obs,
                                       Compute (&out)[KMAX], int &e) const {
    if (ref & kFlag) {
      const std::size_t at = ix.Store(ref & kMask);
      LoadRow<KMAX>(static_cast<const Compute *>(a.nodes) + at * K, K, out);
      e += a.node_exp[at];
    } else {
      Input(ref, obs, false, out);
    }
  }

  __device__ __forceinline__ const Scalar *EdgeIn(std::uint32_t path) const {
    return static_cast<const Scalar *>(a.edge_in) + ix.In(a, path) * KK;
  }

  // Row r of path `ref` (zero for padded rows).
  __device__ __forceinline__ void PathRow(std::uint32_t ref, unsigned r,
                                          Compute (&out)[KMAX]) const {
    if (r >= K) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = Compute(0);
    } else if (ref & kFlag) {
      LoadRow<KMAX>(static_cast<const Compute *>(a.comps) + ix.Comp(ref & kMask) * KK + r * K,
                    K, out);
    } else {
      LoadRow<KMAX>(EdgeIn(ref) + r * K, K, out);
    }
  }
  __device__ __forceinline__ int PathExp(std::uint32_t ref) const {
    return (ref & kFlag) ? a.comp_exp[ix.Comp(ref & kMask)] : 0;
  }

  __device__ __forceinline__ static int Exponent(Compute m) {
    return m > Compute(0) ? Pow2Exponent(m) : 0;
  }

  // ---------------------------------------------------------- forward
  __device__ __forceinline__ void Gather(std::uint32_t i) const {
    const uint4 op = a.gathers[i];
    const std::uint32_t node = op.x & kMask;
    const std::size_t at = ix.Store(node);
    Compute *dst = static_cast<Compute *>(a.nodes) + at * K;
    Compute v[KMAX];
    int e = 0;
    if (op.x & kFlag) {
      Input(node, op.y, (op.w & kRootBit) != 0, v);
    } else {
      LoadRow<KMAX>(dst, K, v);
      e = a.node_exp[at];
    }
    const std::uint32_t count = op.w & kCountMask;
    for (std::uint32_t k = 0; k < count; ++k) {
      const uint4 rake = a.rakes[op.z + k];
      Compute leaf[KMAX];
      Node(rake.y, rake.z, leaf, e);
      e += PathExp(rake.x);
      Compute message[KMAX];
      Compute m = Compute(0);
#pragma unroll
      for (int q = 0; q < KMAX; ++q) {
        Compute row[KMAX];
        PathRow(rake.x, q, row);
        Compute dot = Compute(0);
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          dot = fma(row[j], leaf[j], dot);
        message[q] = dot;
        m = m < dot ? dot : m;
      }
      int s = Exponent(m);
      e += s;
      m = Compute(0);
#pragma unroll
      for (int q = 0; q < KMAX; ++q) {
        v[q] = v[q] * ScalePow2(message[q], -s);
        m = m < v[q] ? v[q] : m;
      }
      s = Exponent(m);
      e += s;
#pragma unroll
      for (int q = 0; q < KMAX; ++q)
        v[q] = ScalePow2(v[q], -s);
    }
    StoreRow<KMAX>(dst, K, v);
    a.node_exp[at] = e;
  }

  __device__ __forceinline__ void Compress(std::uint32_t i) const {
    const uint4 op = a.compress[i];
    int e = PathExp(op.x) + PathExp(op.z);
    Compute middle[KMAX];
    Node(op.y, op.w, middle, e);
    Compute left[KMAX][KMAX];
    Compute out[KMAX][KMAX];
#pragma unroll
    for (int q = 0; q < KMAX; ++q) {
      PathRow(op.x, q, left[q]);
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
        for (int q = 0; q < KMAX; ++q) {
          const Compute weight = left[q][mid] * middle[mid];
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            out[q][j] = fma(weight, right[j], out[q][j]);
        }
      }
    }
    Compute m = Compute(0);
#pragma unroll
    for (int q = 0; q < KMAX; ++q)
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        m = m < out[q][j] ? out[q][j] : m;
    const int s = Exponent(m);
    const std::size_t at = ix.Comp(i);
    Compute *dst = static_cast<Compute *>(a.comps) + at * KK;
#pragma unroll
    for (int q = 0; q < KMAX; ++q) {
      if (q < static_cast<int>(K)) {
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          out[q][j] = ScalePow2(out[q][j], -s);
        StoreRow<KMAX>(dst + q * K, K, out[q]);
      }
    }
    a.comp_exp[at] = e + s;
  }

  // log Z = ln 2 * (root exponent) + log(sum(root)), as LinearEngine::Run.
  // Root record `i`; the result is instance `value`'s.
  __device__ __forceinline__ void Finish(std::uint32_t i, std::uint32_t value) const {
    const uint2 rec = a.roots[i];
    const std::uint32_t node = rec.x & kMask;
    Compute root[KMAX];
    long long total = 0;
    if (rec.x & kFlag) {
      const std::size_t at = ix.Store(node);
      LoadRow<KMAX>(static_cast<const Compute *>(a.nodes) + at * K, K, root);
      total = a.node_exp[at];
    } else {
      Input(node, rec.y, true, root);
    }
    double sum = 0.0;
    for (unsigned j = 0; j < KMAX; ++j)
      sum += static_cast<double>(root[j]);
    const double log_z = !(sum > 0.0)
                             ? -INFINITY
                             : static_cast<double>(total) * 0.6931471805599453094 + log(sum);
    static_cast<Scalar *>(a.values)[value] = static_cast<Scalar>(a.raw ? exp(log_z) : log_z);
    if (a.reverse) {
      Scalar *root_out = static_cast<Scalar *>(a.node_out) + ix.Io(node) * K;
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

  // ---------------------------------------------------------- adjoint
  __device__ __forceinline__ void StorePathAdjoint(std::uint32_t ref, unsigned r,
                                                   const Compute (&row)[KMAX]) const {
    if (ref & kFlag)
      StoreRow<KMAX>(static_cast<Compute *>(a.comp_mu) + ix.Comp(ref & kMask) * KK + r * K, K,
                     row);
    else
      StoreRowStreaming<KMAX>(static_cast<Scalar *>(a.edge_out) + ix.Out(ref) * KK + r * K, K,
                              row);
  }

  __device__ __forceinline__ void RakeReverse(std::uint32_t i) const {
    const uint4 op = a.rakes[i];
    Scalar *node_out = static_cast<Scalar *>(a.node_out);
    Compute leaf[KMAX];
    int unused = 0;
    Node(op.y, op.z, leaf, unused);
    Compute parent_adjoint[KMAX];
    LoadRow<KMAX>(node_out + ix.Io(op.w) * K, K, parent_adjoint);
    Compute ratio[KMAX];
    Compute rows[KMAX][KMAX];
#pragma unroll
    for (int q = 0; q < KMAX; ++q) {
      PathRow(op.x, q, rows[q]);
      Compute unnormalised = Compute(0);
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        unnormalised = fma(rows[q][j], leaf[j], unnormalised);
      ratio[q] = unnormalised > Compute(0) ? parent_adjoint[q] / unnormalised : Compute(0);
      if (q < static_cast<int>(K)) {
        Compute w[KMAX];
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          w[j] = ratio[q] * rows[q][j] * leaf[j];
        StorePathAdjoint(op.x, q, w);
      }
    }
    Compute adjoint[KMAX];
#pragma unroll
    for (unsigned j = 0; j < KMAX; ++j) {
      Compute column = Compute(0);
#pragma unroll
      for (int p = 0; p < KMAX; ++p)
        column = fma(ratio[p], rows[p][j], column);
      adjoint[j] = leaf[j] * column;
    }
    StoreRow<KMAX>(node_out + ix.Io(op.y & kMask) * K, K, adjoint);
  }

  __device__ __forceinline__ void CompressReverse(std::uint32_t i) const {
    const uint4 op = a.compress[i];
    const Compute *output_adjoint = static_cast<const Compute *>(a.comp_mu) + ix.Comp(i) * KK;
    Compute middle[KMAX];
    int unused = 0;
    Node(op.y, op.w, middle, unused);
    Compute left[KMAX][KMAX];
    Compute ratio[KMAX][KMAX];
#pragma unroll
    for (int q = 0; q < KMAX; ++q) {
      PathRow(op.x, q, left[q]);
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
        for (int q = 0; q < KMAX; ++q) {
          const Compute weight = left[q][mid] * middle[mid];
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            ratio[q][j] = fma(weight, right[j], ratio[q][j]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < KMAX; ++q) {
      Compute adjoint[KMAX];
      if (q < static_cast<int>(K)) {
        LoadRow<KMAX>(output_adjoint + q * K, K, adjoint);
      } else {
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          adjoint[j] = Compute(0);
      }
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        ratio[q][j] = ratio[q][j] > Compute(0) ? adjoint[j] / ratio[q][j] : Compute(0);
    }
    Compute rights[KMAX][KMAX];
#pragma unroll
    for (unsigned mid = 0; mid < KMAX; ++mid)
      PathRow(op.z, mid, rights[mid]);
#pragma unroll
    for (int q = 0; q < KMAX; ++q) {
      Compute left_adjoint[KMAX];
#pragma unroll
      for (unsigned mid = 0; mid < KMAX; ++mid) {
        left_adjoint[mid] = Compute(0);
        if (mid < K) {
          Compute dot = Compute(0);
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            dot = fma(rights[mid][j], ratio[q][j], dot);
          left_adjoint[mid] = left[q][mid] * middle[mid] * dot;
        }
      }
      if (q < static_cast<int>(K))
        StorePathAdjoint(op.x, q, left_adjoint);
    }
    Compute middle_adjoint[KMAX];
#pragma unroll
    for (unsigned mid = 0; mid < KMAX; ++mid) {
      Compute right_adjoint[KMAX];
      Compute total = Compute(0);
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j) {
        Compute acc = Compute(0);
#pragma unroll
        for (int p = 0; p < KMAX; ++p)
          acc = fma(left[p][mid], ratio[p][j], acc);
        right_adjoint[j] = rights[mid][j] * middle[mid] * acc;
        total += right_adjoint[j];
      }
      middle_adjoint[mid] = total;
      if (mid < K)
        StorePathAdjoint(op.z, mid, right_adjoint);
    }
    StoreRow<KMAX>(static_cast<Scalar *>(a.node_out) + ix.Io(op.y & kMask) * K, K,
                   middle_adjoint);
  }
};

// Tail rounds of one tree per warp (kPhaseTailForward / kPhaseTailReverse):
// the lanes take the operations of a step in turn, with a warp barrier
// (which also orders the lanes' global-memory accesses) between steps.
// Starts moving `count` 16-byte records from `p` into L2 (a hint).
__device__ __forceinline__ void PrefetchRecords(const void *p, std::uint32_t count) {
  if (count != 0)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(count * 16u)
                 : "memory");
}

template <typename Scalar, typename Compute, bool kReverse>
__device__ __forceinline__ void TailTree(const PhaseOps<Scalar, Compute, ForestIndex> &ops,
                                         const PhaseArgs &a, std::uint32_t item) {
  const unsigned lane = threadIdx.x & 31u;
  const uint4 tree = a.tail_items[item];
  // The walk below is a chain of dependent loads per round; first bring
  // every tail round's records of this tree into L2 (lane e: round e).
  for (std::uint32_t e = lane; e < tree.z; e += 32) {
    const uint4 round = a.tail_rounds[tree.y + e];
    const uint2 rakes = a.tail_rakes[tree.y + e];
    PrefetchRecords(a.gathers + round.x, round.y);
    PrefetchRecords(a.compress + round.z, round.w);
    PrefetchRecords(a.rakes + rakes.x, rakes.y);
  }
  for (std::uint32_t e = 0; e < tree.z; ++e) {
    const std::uint32_t at = tree.y + (kReverse ? tree.z - 1 - e : e);
    const uint4 round = a.tail_rounds[at];
    if constexpr (!kReverse) {
      for (std::uint32_t i = lane; i < round.y; i += 32)
        ops.Gather(round.x + i);
      __syncwarp();
      for (std::uint32_t i = lane; i < round.w; i += 32)
        ops.Compress(round.z + i);
      __syncwarp();
    } else {
      for (std::uint32_t i = lane; i < round.w; i += 32)
        ops.CompressReverse(round.z + i);
      __syncwarp();
      const uint2 rakes = a.tail_rakes[at];
      for (std::uint32_t i = lane; i < rakes.y; i += 32)
        ops.RakeReverse(rakes.x + i);
      __syncwarp();
    }
  }
}

template <typename Scalar, typename Compute, class Index, int kKind>
__device__ __forceinline__ void RunOp(const PhaseArgs &args, const Index &index,
                                      std::uint32_t i, std::uint32_t value) {
  const PhaseOps<Scalar, Compute, Index> ops(args, index);
  if constexpr (kKind == kPhaseGather)
    ops.Gather(i);
  else if constexpr (kKind == kPhaseCompress)
    ops.Compress(i);
  else if constexpr (kKind == kPhaseFinish)
    ops.Finish(i, value);
  else if constexpr (kKind == kPhaseRakeReverse)
    ops.RakeReverse(i);
  else if constexpr (kKind == kPhaseCompressReverse)
    ops.CompressReverse(i);
}

// Forest layout: thread t runs operation offset + t (finish: instance), or
// warp w the tail of tree offset + w.
template <typename Scalar, typename Compute, int kKind>
__global__ void __launch_bounds__(kPhaseThreads) PhaseKernel(PhaseArgs args) {
  if constexpr (kKind == kPhaseTailForward || kKind == kPhaseTailReverse) {
    const std::uint32_t w = blockIdx.x * (kPhaseThreads / 32) + threadIdx.x / 32;
    if (w >= args.count)
      return;
    const PhaseOps<Scalar, Compute, ForestIndex> ops(args, ForestIndex{});
    TailTree<Scalar, Compute, kKind == kPhaseTailReverse>(ops, args, args.offset + w);
  } else {
    const std::uint32_t t = blockIdx.x * kPhaseThreads + threadIdx.x;
    if (t >= args.count)
      return;
    const std::uint32_t i = args.offset + t;
    RunOp<Scalar, Compute, ForestIndex, kKind>(args, ForestIndex{}, i, i);
  }
}

// Shared-topology layout: thread t runs operation offset + t / items of
// batch item first_item + t % items (finish: the root record for that item).
template <typename Scalar, typename Compute, int kKind>
__global__ void __launch_bounds__(kPhaseThreads) BatchPhaseKernel(PhaseArgs args) {
  const std::uint64_t t = static_cast<std::uint64_t>(blockIdx.x) * kPhaseThreads + threadIdx.x;
  if (t >= static_cast<std::uint64_t>(args.count) * args.items)
    return;
  BatchIndex index;
  index.item = args.first_item + static_cast<std::uint32_t>(t % args.items);
  index.stride = args.item_stride;
  index.nodes = args.item_nodes;
  index.edges = args.item_edges;
  const std::uint32_t i = args.offset + static_cast<std::uint32_t>(t / args.items);
  RunOp<Scalar, Compute, BatchIndex, kKind>(args, index, i, index.item);
}

} // namespace thmm

#endif // THMM_PHASE_ENGINE_CUH_
