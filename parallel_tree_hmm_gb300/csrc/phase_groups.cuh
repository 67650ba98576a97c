// Phase kernels of the level-synchronous schedule (phase.h) for 4 < K <= 32
// states: one lane group of G = K_P lanes per operation (K_P = 8, 16 or 32,
// the padded state count), lane r holding row r of the operation's K x K
// matrices, as the lane-group (G > 1) branch of LinearEngine (engine.cuh).
// Above 16 states the FP32 kernels size their register rows to K rounded
// up to a multiple of 4 (20, 24, 28 or 32) rather than 32, which cuts the
// padded arithmetic and the registers (at K = 20, 2.6x fewer multiply-adds
// per compression) without changing a bit.
//
// Each operation performs exactly that branch's floating-point operations
// in the same order, so the phase and per-tree schedules agree bit for bit;
// as in the K <= 4 phase kernels only the bookkeeping of the power-of-two
// exponents differs (carried per stored object here, summed per team
// there; both are exact integer sums). Forest layout only, and no tail
// kinds: every round runs grid-wide.
#ifndef THMM_PHASE_GROUPS_CUH_
#define THMM_PHASE_GROUPS_CUH_

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.cuh"
#include "phase.h"

namespace thmm {

constexpr int kGroupPhaseThreads = 128;

// Minimum resident blocks per SM (a register cap of 65536 / (128 n) per
// thread), chosen so that no FP32 variant spills.
template <int KMAX, bool kWide> constexpr int GroupPhaseMinBlocks() {
  if constexpr (KMAX <= 16)
    return kWide ? 3 : 4;
  else if constexpr (KMAX <= 24)
    return kWide ? 2 : 4;
  else
    return kWide ? 2 : 3;
}

template <typename Scalar, typename Compute, int KMAX> struct GroupPhaseOps {
  // KMAX: the register arrays' length (K rounded up to a multiple of 4
  // above 16 states, else the padded state count); G >= KMAX lanes per
  // group, lane r holding row r (lanes >= K hold zero rows). Terms past K
  // are exact zeros, so every KMAX >= K gives the same bits.
  static constexpr int G = GroupLanes<KMAX>();
  static_assert(G >= KMAX, "one row per lane");
  const PhaseArgs &a;
  unsigned K;
  unsigned KK;

  __device__ explicit GroupPhaseOps(const PhaseArgs &args)
      : a(args), K(args.states), KK(args.states * args.states) {}

  __device__ __forceinline__ Compute *Nodes() const { return static_cast<Compute *>(a.nodes); }
  __device__ __forceinline__ Compute *Comps() const { return static_cast<Compute *>(a.comps); }
  __device__ __forceinline__ Compute *CompMu() const { return static_cast<Compute *>(a.comp_mu); }
  __device__ __forceinline__ Scalar *NodeOut() const { return static_cast<Scalar *>(a.node_out); }

  // Input factor vector of `node`: dense row, or the reference's categorical
  // (root ? root_potential : 1) * emission[observation]
  // (src/gpu_backend_impl.inc:326-382), as Context::InputNode.
  __device__ __forceinline__ void Input(std::uint32_t node, std::uint32_t obs, bool root,
                                        Compute (&out)[KMAX]) const {
    Scalar raw[KMAX];
    if (!a.categorical) {
      LoadRow<KMAX>(static_cast<const Scalar *>(a.node_in) + static_cast<std::size_t>(node) * K,
                    K, raw);
    } else {
      const Scalar *root_potential = static_cast<const Scalar *>(a.root_potential);
      if (obs == kNone) {
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          raw[j] = j < K ? (root ? root_potential[j] : Scalar(1)) : Scalar(0);
      } else {
        const unsigned category = a.observations[obs];
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

  // Value of a rake leaf or compression middle (every lane the whole
  // vector): the stored value (adding its exponent to `e`) or the input.
  __device__ __forceinline__ void Node(std::uint32_t ref, std::uint32_t obs,
                                       Compute (&out)[KMAX], int &e) const {
    if (ref & kFlag) {
      const std::uint32_t node = ref & kMask;
      LoadRow<KMAX>(Nodes() + static_cast<std::size_t>(node) * K, K, out);
      e += a.node_exp[node];
    } else {
      Input(ref, obs, false, out);
    }
  }

  __device__ __forceinline__ const Scalar *EdgeIn(std::uint32_t path) const {
    const std::size_t edge = a.edge_modulus != 0 ? path % a.edge_modulus : path;
    return static_cast<const Scalar *>(a.edge_in) + edge * KK;
  }
  __device__ __forceinline__ void PathRow(std::uint32_t ref, unsigned r,
                                          Compute (&out)[KMAX]) const {
    if (r >= K) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = Compute(0);
    } else if (ref & kFlag) {
      LoadRow<KMAX>(Comps() + static_cast<std::size_t>(ref & kMask) * KK + r * K, K, out);
    } else {
      LoadRow<KMAX>(EdgeIn(ref) + r * K, K, out);
    }
  }
  __device__ __forceinline__ Compute PathElem(std::uint32_t ref, unsigned i, unsigned j) const {
    return (ref & kFlag) ? Comps()[static_cast<std::size_t>(ref & kMask) * KK + i * K + j]
                         : static_cast<Compute>(EdgeIn(ref)[i * K + j]);
  }
  __device__ __forceinline__ int PathExp(std::uint32_t ref) const {
    return (ref & kFlag) ? a.comp_exp[ref & kMask] : 0;
  }
  __device__ __forceinline__ static int Exponent(Compute m) {
    return m > Compute(0) ? Pow2Exponent(m) : 0;
  }
  __device__ __forceinline__ void StorePathAdjoint(std::uint32_t ref, unsigned r,
                                                   const Compute (&row)[KMAX]) const {
    if (ref & kFlag)
      StoreRow<KMAX>(CompMu() + static_cast<std::size_t>(ref & kMask) * KK + r * K, K, row);
    else
      StoreRowStreaming<KMAX>(static_cast<Scalar *>(a.edge_out) +
                                  static_cast<std::size_t>(ref) * KK + r * K,
                              K, row);
  }

  // ---------------------------------------------------------- forward
  // Rakes of gather i absorbed into its parent (LinearEngine::AbsorbRake):
  // lane r holds element r of the parent's value. Groups of a warp share
  // the shuffles, so every group runs the warp's largest rake count and a
  // group past its own rakes computes on a stand-in and keeps nothing.
  __device__ __forceinline__ void Gather(std::uint32_t i, bool active, unsigned lane) const {
    const uint4 op = a.gathers[i];
    const std::uint32_t node = op.x & kMask;
    Compute v;
    int e = 0;
    if (op.x & kFlag) {
      Compute input[KMAX];
      Input(node, op.y, (op.w & kRootBit) != 0, input);
      v = lane < K ? Select(input, lane) : Compute(0);
    } else {
      v = lane < K ? Nodes()[static_cast<std::size_t>(node) * K + lane] : Compute(0);
      e = a.node_exp[node];
    }
    const std::uint32_t count = op.w & kCountMask;
    const unsigned rounds = __reduce_max_sync(kFull, active ? count : 0u);
    for (unsigned k = 0; k < rounds; ++k) {
      const bool live = active && k < count;
      // rounds > 0: some group has a rake, so rake 0 (and its path) exist.
      const uint4 rake = a.rakes[live ? op.z + k : 0u];
      int le = 0;
      Compute leaf[KMAX];
      Node(rake.y, rake.z, leaf, le);
      le += PathExp(rake.x);
      Compute row[KMAX];
      PathRow(rake.x, lane, row);
      Compute dot = Compute(0);
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        dot = fma(row[j], leaf[j], dot);
      const int s1 = Exponent(GroupMax<G>(dot));
      const Compute value = v * ScalePow2(dot, -s1);
      const int s2 = Exponent(GroupMax<G>(value));
      if (live) {
        v = ScalePow2(value, -s2);
        e += le + s1 + s2;
      }
    }
    if (active && lane < K)
      Nodes()[static_cast<std::size_t>(node) * K + lane] = v;
    if (active && lane == 0)
      a.node_exp[node] = e;
  }

  // Compressed path i = left * diag(middle) * right; lane r computes row r.
  __device__ __forceinline__ void Compress(std::uint32_t i, bool active, unsigned lane) const {
    const uint4 op = a.compress[i];
    int e = PathExp(op.x) + PathExp(op.z);
    Compute middle[KMAX];
    Node(op.y, op.w, middle, e);
    Compute left[KMAX];
    Compute out[KMAX];
    PathRow(op.x, lane, left);
#pragma unroll
    for (unsigned j = 0; j < KMAX; ++j)
      out[j] = Compute(0);
#pragma unroll
    for (unsigned mid = 0; mid < KMAX; ++mid) {
      if (mid < K) {
        Compute right[KMAX];
        PathRow(op.z, mid, right);
        const Compute weight = left[mid] * middle[mid];
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          out[j] = fma(weight, right[j], out[j]);
      }
    }
    Compute m = Compute(0);
#pragma unroll
    for (unsigned j = 0; j < KMAX; ++j)
      m = m < out[j] ? out[j] : m;
    const int s = Exponent(GroupMax<G>(m));
    if (active && lane < K) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = ScalePow2(out[j], -s);
      StoreRow<KMAX>(Comps() + static_cast<std::size_t>(i) * KK + lane * K, K, out);
    }
    if (active && lane == 0)
      a.comp_exp[i] = e + s;
  }

  // log Z = ln 2 * (root exponent) + log(sum(root)), as LinearEngine::Run
  // (one thread per instance).
  __device__ __forceinline__ void Finish(std::uint32_t i) const {
    const uint2 rec = a.roots[i];
    const std::uint32_t node = rec.x & kMask;
    Compute root[KMAX];
    long long total = 0;
    if (rec.x & kFlag) {
      LoadRow<KMAX>(Nodes() + static_cast<std::size_t>(node) * K, K, root);
      total = a.node_exp[node];
    } else {
      Input(node, rec.y, true, root);
    }
    double sum = 0.0;
    for (unsigned j = 0; j < KMAX; ++j)
      sum += static_cast<double>(root[j]);
    const double log_z = !(sum > 0.0)
                             ? -INFINITY
                             : static_cast<double>(total) * 0.6931471805599453094 + log(sum);
    static_cast<Scalar *>(a.values)[i] = static_cast<Scalar>(a.raw ? exp(log_z) : log_z);
    if (a.reverse) {
      Scalar *root_out = NodeOut() + static_cast<std::size_t>(node) * K;
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
  __device__ __forceinline__ void RakeReverse(std::uint32_t i, bool active, unsigned lane) const {
    const uint4 op = a.rakes[i];
    Compute leaf[KMAX];
    int unused = 0;
    Node(op.y, op.z, leaf, unused);
    const Compute parent_adjoint =
        lane < K ? static_cast<Compute>(NodeOut()[static_cast<std::size_t>(op.w) * K + lane])
                 : Compute(0);
    Compute row[KMAX];
    PathRow(op.x, lane, row);
    Compute unnormalised = Compute(0);
#pragma unroll
    for (unsigned j = 0; j < KMAX; ++j)
      unnormalised = fma(row[j], leaf[j], unnormalised);
    const Compute ratio = unnormalised > Compute(0) ? parent_adjoint / unnormalised : Compute(0);
    if (active && lane < K) {
      Compute w[KMAX];
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        w[j] = ratio * row[j] * leaf[j];
      StorePathAdjoint(op.x, lane, w);
    }
    // Leaf adjoint: leaf[j] * sum_p ratio_p * path[p][j].
    Compute column = Compute(0);
    for (unsigned p = 0; p < K; ++p) {
      const Compute ratio_p = GroupBroadcast<G>(ratio, static_cast<int>(p));
      if (lane < K)
        column = fma(ratio_p, PathElem(op.x, p, lane), column);
    }
    if (active && lane < K)
      NodeOut()[static_cast<std::size_t>(op.y & kMask) * K + lane] =
          static_cast<Scalar>(Select(leaf, lane) * column);
  }

  // Adjoint of compression i; `tile` is this group's K x K shared-memory
  // scratch for the ratio matrix.
  __device__ __forceinline__ void CompressReverse(std::uint32_t i, bool active, unsigned lane,
                                                  Compute *tile) const {
    const uint4 op = a.compress[i];
    const Compute *output_adjoint = CompMu() + static_cast<std::size_t>(i) * KK;
    Compute middle[KMAX];
    int unused = 0;
    Node(op.y, op.w, middle, unused);
    // Unnormalised output row `lane`, recomputed with the forward's
    // operation order, and ratio = adjoint / output.
    Compute left[KMAX];
    Compute ratio[KMAX];
    PathRow(op.x, lane, left);
#pragma unroll
    for (unsigned j = 0; j < KMAX; ++j)
      ratio[j] = Compute(0);
#pragma unroll
    for (unsigned mid = 0; mid < KMAX; ++mid) {
      if (mid < K) {
        Compute right[KMAX];
        PathRow(op.z, mid, right);
        const Compute weight = left[mid] * middle[mid];
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          ratio[j] = fma(weight, right[j], ratio[j]);
      }
    }
    {
      Compute adjoint[KMAX];
      if (lane < K) {
        LoadRow<KMAX>(output_adjoint + lane * K, K, adjoint);
      } else {
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          adjoint[j] = Compute(0);
      }
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        ratio[j] = ratio[j] > Compute(0) ? adjoint[j] / ratio[j] : Compute(0);
    }
    // Left adjoint row `lane`: left[r][m] middle[m] sum_j right[m][j] ratio[r][j].
    {
      Compute left_adjoint[KMAX];
#pragma unroll
      for (unsigned mid = 0; mid < KMAX; ++mid) {
        left_adjoint[mid] = Compute(0);
        if (mid < K) {
          Compute right[KMAX];
          PathRow(op.z, mid, right);
          Compute dot = Compute(0);
#pragma unroll
          for (unsigned j = 0; j < KMAX; ++j)
            dot = fma(right[j], ratio[j], dot);
          left_adjoint[mid] = left[mid] * middle[mid] * dot;
        }
      }
      if (active && lane < K)
        StorePathAdjoint(op.x, lane, left_adjoint);
    }
    // Right adjoint row m = lane: right[m][j] middle[m] sum_p left[p][m] ratio[p][j],
    // with the ratio rows of the group in shared memory.
    if (lane < K) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        if (j < K)
          tile[lane * K + j] = ratio[j];
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
            acc[j] = fma(left_p, tile[p * K + j], acc[j]);
      }
      const Compute own_middle = Select(middle, lane);
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
        StorePathAdjoint(op.z, lane, right_adjoint);
        NodeOut()[static_cast<std::size_t>(op.y & kMask) * K + lane] = static_cast<Scalar>(total);
      }
    }
    __syncwarp();
  }
};

// Shared memory of a block: one K_P x K_P ratio tile per lane group (the
// reverse compression kind only).
template <typename Compute, int KMAX>
constexpr unsigned GroupPhaseSmem(int kind) {
  return kind == kPhaseCompressReverse
             ? (kGroupPhaseThreads / GroupLanes<KMAX>()) * KMAX * KMAX *
                   static_cast<unsigned>(sizeof(Compute))
             : 0u;
}

// One kind of one round: lane group g of the grid runs operation offset + g
// (finish: thread t the root record of instance offset + t).
template <typename Scalar, typename Compute, int KMAX, int kKind>
__global__ void __launch_bounds__(kGroupPhaseThreads,
                                  GroupPhaseMinBlocks<KMAX, sizeof(Compute) == 8>())
    GroupPhaseKernel(PhaseArgs args) {
  using Ops = GroupPhaseOps<Scalar, Compute, KMAX>;
  constexpr int G = Ops::G;
  const Ops ops(args);
  const std::uint32_t t = blockIdx.x * kGroupPhaseThreads + threadIdx.x;
  if constexpr (kKind == kPhaseFinish) {
    if (t < args.count)
      ops.Finish(args.offset + t);
  } else {
    // Whole warps past the last group leave together (no shuffle partner
    // of a live group leaves).
    if ((t & ~31u) / G >= args.count)
      return;
    const std::uint32_t group = t / G;
    const unsigned lane = threadIdx.x % G;
    const bool active = group < args.count;
    // A padding group of a live warp reads the last operation, writes nothing.
    const std::uint32_t i = args.offset + (active ? group : args.count - 1);
    if constexpr (kKind == kPhaseGather) {
      ops.Gather(i, active, lane);
    } else if constexpr (kKind == kPhaseCompress) {
      ops.Compress(i, active, lane);
    } else if constexpr (kKind == kPhaseRakeReverse) {
      ops.RakeReverse(i, active, lane);
    } else if constexpr (kKind == kPhaseCompressReverse) {
      extern __shared__ __align__(16) unsigned char group_smem[];
      Compute *tile = reinterpret_cast<Compute *>(group_smem) + (threadIdx.x / G) * KMAX * KMAX;
      ops.CompressReverse(i, active, lane, tile);
    }
  }
}

} // namespace thmm

#endif // THMM_PHASE_GROUPS_CUH_
