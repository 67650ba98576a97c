// Phase kernels of the level-synchronous schedule (phase.h) for padded state
// count 4 (K <= 4): one thread per operation, the K-vectors and K x K
// matrices in registers, 16-byte vector loads and stores.
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

constexpr int kPhaseThreads = 256;

template <typename Scalar, typename Compute> struct PhaseOps {
  static constexpr int KMAX = 4;
  const PhaseArgs &a;
  unsigned K;
  unsigned KK;

  __device__ explicit PhaseOps(const PhaseArgs &args)
      : a(args), K(args.states), KK(args.states * args.states) {}

  // Input factor vector of `node`: dense row, or the reference's categorical
  // (root ? root_potential : 1) * emission[observation]
  // (src/gpu_backend_impl.inc:326-382), as Context::InputNode.
  __device__ __forceinline__ void Input(std::uint32_t node, std::uint32_t obs, bool root,
                                        Compute (&out)[KMAX]) const {
    Scalar raw[KMAX];
    if (!a.categorical) {
      LoadRow<KMAX>(static_cast<const Scalar *>(a.node_in) +
                        static_cast<std::size_t>(node) * K,
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

  // Value of a rake leaf or compression middle: the stored value (adding its
  // exponent to `e`) or the input factor.
  __device__ __forceinline__ void Node(std::uint32_t ref, std::uint32_t obs,
                                       Compute (&out)[KMAX], int &e) const {
    if (ref & kFlag) {
      const std::uint32_t node = ref & kMask;
      LoadRow<KMAX>(static_cast<const Compute *>(a.nodes) + static_cast<std::size_t>(node) * K,
                    K, out);
      e += a.node_exp[node];
    } else {
      Input(ref, obs, false, out);
    }
  }

  __device__ __forceinline__ const Scalar *EdgeIn(std::uint32_t path) const {
    const std::uint32_t row = a.edge_modulus != 0 ? path % a.edge_modulus : path;
    return static_cast<const Scalar *>(a.edge_in) + static_cast<std::size_t>(row) * KK;
  }

  // Row r of path `ref` (zero for padded rows).
  __device__ __forceinline__ void PathRow(std::uint32_t ref, unsigned r,
                                          Compute (&out)[KMAX]) const {
    if (r >= K) {
#pragma unroll
      for (unsigned j = 0; j < KMAX; ++j)
        out[j] = Compute(0);
    } else if (ref & kFlag) {
      LoadRow<KMAX>(static_cast<const Compute *>(a.comps) +
                        static_cast<std::size_t>(ref & kMask) * KK + r * K,
                    K, out);
    } else {
      LoadRow<KMAX>(EdgeIn(ref) + r * K, K, out);
    }
  }
  __device__ __forceinline__ int PathExp(std::uint32_t ref) const {
    return (ref & kFlag) ? a.comp_exp[ref & kMask] : 0;
  }

  __device__ __forceinline__ static int Exponent(Compute m) {
    return m > Compute(0) ? Pow2Exponent(m) : 0;
  }

  // ---------------------------------------------------------- forward
  __device__ __forceinline__ void Gather(std::uint32_t i) const {
    const uint4 op = a.gathers[i];
    const std::uint32_t node = op.x & kMask;
    Compute *dst = static_cast<Compute *>(a.nodes) + static_cast<std::size_t>(node) * K;
    Compute v[KMAX];
    int e = 0;
    if (op.x & kFlag) {
      Input(node, op.y, (op.w & kRootBit) != 0, v);
    } else {
      LoadRow<KMAX>(dst, K, v);
      e = a.node_exp[node];
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
    a.node_exp[node] = e;
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
    Compute *dst = static_cast<Compute *>(a.comps) + static_cast<std::size_t>(i) * KK;
#pragma unroll
    for (int q = 0; q < KMAX; ++q) {
      if (q < static_cast<int>(K)) {
#pragma unroll
        for (unsigned j = 0; j < KMAX; ++j)
          out[q][j] = ScalePow2(out[q][j], -s);
        StoreRow<KMAX>(dst + q * K, K, out[q]);
      }
    }
    a.comp_exp[i] = e + s;
  }

  // log Z = ln 2 * (root exponent) + log(sum(root)), as LinearEngine::Run.
  __device__ __forceinline__ void Finish(std::uint32_t i) const {
    const uint2 rec = a.roots[i];
    const std::uint32_t node = rec.x & kMask;
    Compute root[KMAX];
    long long total = 0;
    if (rec.x & kFlag) {
      LoadRow<KMAX>(static_cast<const Compute *>(a.nodes) + static_cast<std::size_t>(node) * K,
                    K, root);
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
      Scalar *root_out = static_cast<Scalar *>(a.node_out) + static_cast<std::size_t>(node) * K;
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
      StoreRow<KMAX>(static_cast<Compute *>(a.comp_mu) +
                         static_cast<std::size_t>(ref & kMask) * KK + r * K,
                     K, row);
    else
      StoreRowStreaming<KMAX>(static_cast<Scalar *>(a.edge_out) +
                                  static_cast<std::size_t>(ref) * KK + r * K,
                              K, row);
  }

  __device__ __forceinline__ void RakeReverse(std::uint32_t i) const {
    const uint4 op = a.rakes[i];
    Scalar *node_out = static_cast<Scalar *>(a.node_out);
    Compute leaf[KMAX];
    int unused = 0;
    Node(op.y, op.z, leaf, unused);
    Compute parent_adjoint[KMAX];
    LoadRow<KMAX>(node_out + static_cast<std::size_t>(op.w) * K, K, parent_adjoint);
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
    StoreRow<KMAX>(node_out + static_cast<std::size_t>(op.y & kMask) * K, K, adjoint);
  }

  __device__ __forceinline__ void CompressReverse(std::uint32_t i) const {
    const uint4 op = a.compress[i];
    const Compute *output_adjoint =
        static_cast<const Compute *>(a.comp_mu) + static_cast<std::size_t>(i) * KK;
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
    StoreRow<KMAX>(static_cast<Scalar *>(a.node_out) + static_cast<std::size_t>(op.y & kMask) * K,
                   K, middle_adjoint);
  }
};

template <typename Scalar, typename Compute, int kKind>
__global__ void __launch_bounds__(kPhaseThreads) PhaseKernel(PhaseArgs args) {
  const std::uint32_t t = blockIdx.x * kPhaseThreads + threadIdx.x;
  if (t >= args.count)
    return;
  const std::uint32_t i = args.offset + t;
  const PhaseOps<Scalar, Compute> ops(args);
  if constexpr (kKind == kPhaseGather)
    ops.Gather(i);
  else if constexpr (kKind == kPhaseCompress)
    ops.Compress(i);
  else if constexpr (kKind == kPhaseFinish)
    ops.Finish(i);
  else if constexpr (kKind == kPhaseRakeReverse)
    ops.RakeReverse(i);
  else
    ops.CompressReverse(i);
}

} // namespace thmm

#endif // THMM_PHASE_ENGINE_CUH_
