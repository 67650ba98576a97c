// Forward and adjoint sweeps of the wide-state engine (included by
// wide_engine_tree.cuh).
#ifndef THMM_WIDE_ENGINE_SWEEPS_CUH_
#define THMM_WIDE_ENGINE_SWEEPS_CUH_

namespace thmm {
namespace wide {

// Scaled sum-product over the fused step list (src/inference.cc:697-836 with
// exact power-of-two scaling, as LinearEngine::Forward).
template <int KP> __device__ void Tree<KP>::Forward() {
  const uint4 *rakes = static_cast<const uint4 *>(a.rakes);
  const uint4 *gathers = static_cast<const uint4 *>(a.gathers);
  const uint4 *compress = static_cast<const uint4 *>(a.compress);
  const unsigned j = threadIdx.x;
  for (unsigned s = 0; s < prog.fused_count; ++s) {
    const DevStep step = a.steps[prog.fused_begin + s];
    if (step.kind == kStepGather) {
      for (unsigned i = 0; i < step.count; ++i) {
        const uint4 op = gathers[step.offset + i];
        const unsigned node = op.x & kMask;
        float *dst = nodes + static_cast<std::size_t>(node) * K;
        if (op.x & kFlag)
          NodeVector(node, op.y, v);
        else if (j < K)
          v[j] = dst[j];
        for (unsigned k = 0; k < op.w; ++k) {
          const uint4 rake = rakes[op.z + k];
          NodeVector(rake.y, rake.w, leaf);
          const float *path = Path(rake.x);
          if (bulk) {
            // Next rake of this step: the following one of this gather, or
            // the first one of the next gather.
            const float *next = nullptr;
            if (k + 1 < op.w) {
              next = Path(rakes[op.z + k + 1].x);
            } else if (i + 1 < step.count) {
              const uint4 following = gathers[step.offset + i + 1];
              if (following.w != 0)
                next = Path(rakes[following.z].x);
            }
            Fetch(path, nullptr, nullptr, 1, next != nullptr, next, nullptr, nullptr);
            path = raw[0];
          }
          __syncthreads();
          MatVec(path, leaf, msg);
          __syncthreads();
          const float message = j < K ? msg[j] : 0.0f;
          int e = Renormaliser(message);
          float value = j < K ? v[j] * ScalePow2(message, -e) : 0.0f;
          e = Renormaliser(value);
          if (j < K)
            v[j] = ScalePow2(value, -e);
        }
        __syncthreads();
        if (j < K)
          dst[j] = v[j];
        __syncthreads();
      }
    } else if (step.kind == kStepCompress) {
      for (unsigned i = 0; i < step.count; ++i) {
        const unsigned g = step.offset + i;
        const unsigned tape = g - prog.compress_base;
        const uint4 op = compress[g];
        NodeVector(op.y, op.w, middle);
        const float *left = Path(op.x);
        const float *right = Path(op.z);
        if (bulk) {
          const bool has_next = i + 1 < step.count;
          const uint4 next = has_next ? compress[g + 1] : op;
          Fetch(left, right, nullptr, 2, has_next, Path(next.x), Path(next.z), nullptr);
          left = raw[0];
          right = raw[1];
        }
        __syncthreads();
        // X(r, d) = left[r][d] * middle[d]; Y(n, d) = right[d][n].
        // Split accumulators (see Product): log Z is formed from these
        // products alone, so they get the more accurate accumulation.
        ok = Product<KP, RowMajor, Transposed, true>(smem, sh, phase,
                                                     tmem + Layout<KP>::kProductColumn, K,
                                                     RowMajor{left, middle},
                                                     Transposed{right}, a.bf16 != 0) &&
             ok;
        // Row j of the product is tensor-memory lane j: maximum, then scale.
        const std::uint32_t lane_base =
            tmem + Layout<KP>::kProductColumn + ((threadIdx.x & ~31u) << 16);
        float m = 0.0f;
#pragma unroll 1
        for (unsigned c = 0; c < KP; c += 32) {
          float row[32];
          SplitSum32<KP>(lane_base, c, row, a.bf16 != 0);
#pragma unroll
          for (unsigned q = 0; q < 32; ++q)
            if (j < K && c + q < K)
              m = m < row[q] ? row[q] : m;
        }
        const int e = Renormaliser(m);
        float *out = comps + static_cast<std::size_t>(tape) * KK + static_cast<std::size_t>(j) * K;
#pragma unroll 1
        for (unsigned c = 0; c < KP; c += 32) {
          float row[32];
          SplitSum32<KP>(lane_base, c, row, a.bf16 != 0);
#pragma unroll
          for (unsigned q = 0; q < 32; ++q)
            if (j < K && c + q < K)
              out[c + q] = ScalePow2(row[q], -e);
        }
        // The compressed path may later arrive by bulk copy (async proxy).
        umma::FenceProxy();
        umma::FenceBeforeSync();
        __syncthreads();
      }
    }
    __syncthreads();
  }
}

// log Z (and the root marginal when the adjoint follows), FP64 as in
// LinearEngine::Run.
template <int KP> __device__ void Tree<KP>::Finish(unsigned item) {
  NodeVector(prog.root, prog.root_obs, v);
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (unsigned q = 0; q < K; ++q)
      sum += static_cast<double>(v[q]);
    const double log_z = (zero || !(sum > 0.0))
                             ? -INFINITY
                             : static_cast<double>(exponent) * 0.6931471805599453094 +
                                   log(sum);
    static_cast<float *>(a.values)[item] =
        static_cast<float>(a.raw ? exp(log_z) : log_z);
    sh.root_sum = sum;
    sh.root_finite = log_z > -INFINITY;
  }
  __syncthreads();
  if (a.reverse && threadIdx.x < K) {
    float *root_out = static_cast<float *>(a.node_out) +
                      (inst.node_base + (prog.root & kMask)) * K;
    root_out[threadIdx.x] =
        sh.root_finite ? static_cast<float>(static_cast<double>(v[threadIdx.x]) / sh.root_sum)
                       : 0.0f;
  }
  if (!ok && threadIdx.x == 0)
    atomicOr(a.error, kErrorTensorTimeout);
  __syncthreads();
}

} // namespace wide
} // namespace thmm

#include "wide_engine_reverse.cuh"

#endif // THMM_WIDE_ENGINE_SWEEPS_CUH_
