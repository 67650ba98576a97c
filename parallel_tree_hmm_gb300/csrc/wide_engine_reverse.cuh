// Adjoint sweep and kernel of the wide-state engine (included by
// wide_engine_sweeps.cuh).
#ifndef THMM_WIDE_ENGINE_REVERSE_CUH_
#define THMM_WIDE_ENGINE_REVERSE_CUH_

namespace thmm {
namespace wide {

// d log Z / d log(factor) for every node and edge, revisiting rakes and
// compressions in reverse (the adjoint of a branch is the marginal of the
// rake's parent, as in LinearEngine::Reverse).
template <int KP> __device__ void Tree<KP>::Reverse() {
  float *node_out = static_cast<float *>(a.node_out) + inst.node_base * K;
  float *edge_out = static_cast<float *>(a.edge_out) +
                    inst.edge_out_base * static_cast<std::uint64_t>(KK);
  const uint4 *rakes = static_cast<const uint4 *>(a.rakes);
  const uint4 *compress = static_cast<const uint4 *>(a.compress);
  const unsigned j = threadIdx.x;
  const unsigned warp = threadIdx.x / 32, lane = threadIdx.x & 31;
  const auto adjoint_of = [&](unsigned ref) {
    return (ref & kFlag) ? comp_mu + static_cast<std::size_t>(ref & kMask) * KK
                         : edge_out + static_cast<std::size_t>(ref) * KK;
  };
  for (unsigned s = prog.step_count; s-- > 0;) {
    const DevStep step = a.steps[prog.step_begin + s];
    if (step.kind == kStepRake) {
      for (unsigned i = 0; i < step.count; ++i) {
        const uint4 op = rakes[step.offset + i];
        const float *path = Path(op.x);
        if (bulk) {
          const bool has_next = i + 1 < step.count;
          const float *next = has_next ? Path(rakes[step.offset + i + 1].x) : nullptr;
          Fetch(path, nullptr, nullptr, 1, has_next, next, nullptr, nullptr);
          path = raw[0];
        }
        NodeVector(op.y, op.w, leaf);
        if (j < K)
          v[j] = node_out[static_cast<std::size_t>(op.z) * K + j]; // parent marginal
        __syncthreads();
        MatVec(path, leaf, msg);
        __syncthreads();
        if (j < K)
          ratio[j] = msg[j] > 0.0f ? v[j] / msg[j] : 0.0f;
        __syncthreads();
        // Path adjoint rows ratio[r] * path[r][c] * leaf[c] (warp w: rows
        // w, w + 4, ...; lanes: columns, coalesced), and each warp's partial
        // column sums sum_r ratio[r] * path[r][c] for the leaf adjoint.
        float *out = adjoint_of(op.x);
        float column[KP / 32];
#pragma unroll
        for (unsigned q = 0; q < KP / 32; ++q)
          column[q] = 0.0f;
#pragma unroll 2
        for (unsigned r = warp; r < K; r += kThreads / 32) {
          const float ratio_r = ratio[r];
#pragma unroll
          for (unsigned q = 0; q < KP / 32; ++q) {
            const unsigned c = lane + 32 * q;
            if (c < K) {
              const float p = path[static_cast<std::size_t>(r) * K + c];
              out[static_cast<std::size_t>(r) * K + c] = ratio_r * p * leaf[c];
              column[q] = fmaf(ratio_r, p, column[q]);
            }
          }
        }
        // Reduce the four warps' column sums through the message vector.
#pragma unroll 1
        for (unsigned w = 0; w < kThreads / 32; ++w) {
          if (warp == w) {
#pragma unroll
            for (unsigned q = 0; q < KP / 32; ++q) {
              const unsigned c = lane + 32 * q;
              if (c < K)
                msg[c] = (w == 0 ? 0.0f : msg[c]) + column[q];
            }
          }
          __syncthreads();
        }
        // Leaf adjoint: leaf[c] * sum_r ratio[r] * path[r][c].
        if (j < K)
          node_out[static_cast<std::size_t>(op.y & kMask) * K + j] = leaf[j] * msg[j];
        umma::FenceProxy(); // path adjoints may later arrive by bulk copy
        __syncthreads();
      }
    } else if (step.kind == kStepCompress) {
      for (unsigned i = 0; i < step.count; ++i) {
        const unsigned g = step.offset + i;
        const unsigned tape = g - prog.compress_base;
        const uint4 op = compress[g];
        const float *left = Path(op.x);
        const float *right = Path(op.z);
        float *output_adjoint = comp_mu + static_cast<std::size_t>(tape) * KK;
        float *left_out_base = adjoint_of(op.x);
        float *right_out_base = adjoint_of(op.z);
        if (bulk) {
          // Left and right path versions and this compression's output
          // adjoint; the ratio below then lives in shared memory only.
          const bool has_next = i + 1 < step.count;
          const uint4 next = has_next ? compress[g + 1] : op;
          Fetch(left, right, output_adjoint, 3, has_next, Path(next.x), Path(next.z),
                comp_mu + static_cast<std::size_t>(tape + 1) * KK);
          left = raw[0];
          right = raw[1];
          output_adjoint = raw[2];
        }
        NodeVector(op.y, op.w, middle);
        __syncthreads();
        const float *mid = middle;
        // Unnormalised output, recomputed: left * diag(middle) * right.
        ok = Product<KP>(smem, sh, phase, tmem + Layout<KP>::kProductColumn, K,
                         RowMajor{left, middle}, Transposed{right}, a.bf16 != 0) &&
             ok;
        // ratio = adjoint / output, written over the output adjoint (each
        // path version's adjoint is read only here).
        // (tcgen05.ld is warp-collective: every lane loads, lanes j >= K
        // discard.)
        const std::uint32_t lane_base = (threadIdx.x & ~31u) << 16;
        float *row_adjoint = output_adjoint + static_cast<std::size_t>(j) * K;
#pragma unroll 1
        for (unsigned c = 0; c < KP; c += 32) {
          float row[32];
          umma::Load32(tmem + Layout<KP>::kProductColumn + lane_base + c, row);
          if (j < K) {
#pragma unroll
            for (unsigned q = 0; q < 32; ++q)
              if (c + q < K) {
                const float adjoint = row_adjoint[c + q];
                row_adjoint[c + q] = row[q] > 0.0f ? adjoint / row[q] : 0.0f;
              }
          }
        }
        umma::FenceBeforeSync();
        __syncthreads();
        const float *ratio_matrix = output_adjoint;
        // P1[r][m] = sum_c ratio[r][c] right[m][c]  (left adjoint factor).
        ok = Product<KP>(smem, sh, phase, tmem + Layout<KP>::kLeftColumn, K,
                         RowMajor{ratio_matrix, nullptr}, RowMajor{right, nullptr},
                         a.bf16 != 0) &&
             ok;
        // P2[m][c] = sum_r left[r][m] ratio[r][c]  (right adjoint factor).
        ok = Product<KP>(smem, sh, phase, tmem + Layout<KP>::kRightColumn, K, Transposed{left},
                         Transposed{ratio_matrix}, a.bf16 != 0) &&
             ok;
        // Row j: left adjoint left[j][m] middle[m] P1[j][m]; right adjoint
        // right[j][c] middle[j] P2[j][c]; middle adjoint sum_c of the latter.
        float *left_out = left_out_base + static_cast<std::size_t>(j) * K;
        float *right_out = right_out_base + static_cast<std::size_t>(j) * K;
        float total = 0.0f;
#pragma unroll 1
        for (unsigned c = 0; c < KP; c += 32) {
          float p1[32], p2[32];
          umma::Load32(tmem + Layout<KP>::kLeftColumn + lane_base + c, p1);
          umma::Load32(tmem + Layout<KP>::kRightColumn + lane_base + c, p2);
          if (j < K) {
#pragma unroll
            for (unsigned q = 0; q < 32; ++q) {
              if (c + q < K) {
                const unsigned col = c + q;
                left_out[col] = left[static_cast<std::size_t>(j) * K + col] * mid[col] * p1[q];
                const float r_adj = right[static_cast<std::size_t>(j) * K + col] * mid[j] * p2[q];
                right_out[col] = r_adj;
                total += r_adj;
              }
            }
          }
        }
        if (j < K)
          node_out[static_cast<std::size_t>(op.y & kMask) * K + j] = total;
        umma::FenceProxy(); // path adjoints may later arrive by bulk copy
        umma::FenceBeforeSync();
        __syncthreads();
      }
    }
  }
  if (!ok && threadIdx.x == 0)
    atomicOr(a.error, kErrorTensorTimeout);
  __syncthreads();
}

// Persistent kernel: one or two CTAs per SM (Layout), trees from the
// large-instance queue.
template <int KP, int kPart>
__global__ void __launch_bounds__(kThreads, Layout<KP>::kCtasPerSm) WideKernel(EngineArgs args) {
  extern __shared__ __align__(1024) unsigned char dynamic_smem[];
  __shared__ Shared sh;
  ClearOperands<KP>(dynamic_smem);
  if (threadIdx.x == 0) {
    umma::BarrierInit(&sh.barrier);
    umma::BarrierInit(&sh.copy_barrier[0]);
    umma::BarrierInit(&sh.copy_barrier[1]);
  }
  if (threadIdx.x < 32)
    umma::Allocate(&sh.tmem, Layout<KP>::kTmemColumns);
  umma::FenceBeforeSync();
  __syncthreads();
  umma::FenceAfterSync();
  const std::uint32_t tmem = sh.tmem;
  std::uint32_t phase = 0, copy_phase = 0;
  for (;;) {
    if (threadIdx.x == 0)
      sh.item = atomicAdd(&args.queue[0], 1u);
    __syncthreads();
    const unsigned index = sh.item;
    __syncthreads();
    if (index >= args.big_count)
      break;
    const unsigned item = args.big_items[index];
    Tree<KP> tree(args, item, sh, dynamic_smem, tmem, phase, copy_phase);
    if constexpr (kPart == kLinearForward) {
      tree.Forward();
      tree.Finish(item);
    } else {
      tree.Reverse();
    }
    __syncthreads();
  }
  umma::FenceBeforeSync();
  __syncthreads();
  umma::FenceAfterSync();
  if (threadIdx.x < 32)
    umma::Deallocate(tmem, Layout<KP>::kTmemColumns);
}

template <int KP, int kPart>
cudaError_t LaunchWidePart(const EngineArgs &args, int grid, cudaStream_t stream,
                           int *blocks_per_sm) {
  auto kernel = WideKernel<KP, kPart>;
  const cudaError_t status = cudaFuncSetAttribute(
      kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(Layout<KP>::kSmemBytes));
  if (status != cudaSuccess)
    return status;
  if (blocks_per_sm != nullptr)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel, kThreads,
                                                         Layout<KP>::kSmemBytes);
  kernel<<<grid, kThreads, Layout<KP>::kSmemBytes, stream>>>(args);
  return cudaGetLastError();
}

} // namespace wide
} // namespace thmm

#endif // THMM_WIDE_ENGINE_REVERSE_CUH_
