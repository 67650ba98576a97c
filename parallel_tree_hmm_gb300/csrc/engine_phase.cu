// Launchers of the phase kernels (phase_engine.cuh) for every input and
// arithmetic type, and the gather of the phase-ordered observations.
#include "phase_engine.cuh"

namespace thmm {
namespace {

template <typename Scalar, typename Compute, int kKind>
cudaError_t LaunchKind(const PhaseArgs &args, cudaStream_t stream, int *blocks_per_sm) {
  constexpr bool kTail = kKind == kPhaseTailForward || kKind == kPhaseTailReverse;
  if constexpr (!kTail) {
    if (args.batch) {
      auto kernel = BatchPhaseKernel<Scalar, Compute, kKind>;
      if (blocks_per_sm != nullptr)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel,
                                                             kPhaseThreads, 0);
      const std::uint64_t threads = static_cast<std::uint64_t>(args.count) * args.items;
      if (threads == 0)
        return cudaSuccess;
      const std::uint64_t grid = (threads + kPhaseThreads - 1) / kPhaseThreads;
      if (grid > 0x7fffffffull)
        return cudaErrorInvalidConfiguration;
      kernel<<<static_cast<unsigned>(grid), kPhaseThreads, 0, stream>>>(args);
      return cudaGetLastError();
    }
  } else if (args.batch) {
    return cudaErrorInvalidValue; // no tail in the shared-topology layout
  }
  auto kernel = PhaseKernel<Scalar, Compute, kKind>;
  if (blocks_per_sm != nullptr)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel,
                                                         kPhaseThreads, 0);
  if (args.count == 0)
    return cudaSuccess;
  // One thread per operation, or one warp per tree for the tail kinds.
  const unsigned per_block = kTail ? kPhaseThreads / 32 : kPhaseThreads;
  const unsigned grid = (args.count + per_block - 1) / per_block;
  kernel<<<grid, kPhaseThreads, 0, stream>>>(args);
  return cudaGetLastError();
}

template <typename Scalar, typename Compute>
cudaError_t LaunchTyped(int kind, const PhaseArgs &args, cudaStream_t stream,
                        int *blocks_per_sm) {
  switch (kind) {
  case kPhaseGather:
    return LaunchKind<Scalar, Compute, kPhaseGather>(args, stream, blocks_per_sm);
  case kPhaseCompress:
    return LaunchKind<Scalar, Compute, kPhaseCompress>(args, stream, blocks_per_sm);
  case kPhaseFinish:
    return LaunchKind<Scalar, Compute, kPhaseFinish>(args, stream, blocks_per_sm);
  case kPhaseRakeReverse:
    return LaunchKind<Scalar, Compute, kPhaseRakeReverse>(args, stream, blocks_per_sm);
  case kPhaseCompressReverse:
    return LaunchKind<Scalar, Compute, kPhaseCompressReverse>(args, stream, blocks_per_sm);
  case kPhaseTailForward:
    return LaunchKind<Scalar, Compute, kPhaseTailForward>(args, stream, blocks_per_sm);
  case kPhaseTailReverse:
    return LaunchKind<Scalar, Compute, kPhaseTailReverse>(args, stream, blocks_per_sm);
  default:
    return cudaErrorInvalidValue;
  }
}

__global__ void __launch_bounds__(kPhaseThreads)
ObservationGather(const std::uint8_t *observations, const std::uint32_t *order,
                  std::uint8_t *ordered, std::uint64_t count, std::uint64_t items,
                  std::uint64_t per_item) {
  const std::uint64_t t = static_cast<std::uint64_t>(blockIdx.x) * kPhaseThreads + threadIdx.x;
  if (t >= count * items)
    return;
  const std::uint64_t j = t / items, b = t % items;
  ordered[t] = observations[b * per_item + order[j]];
}

} // namespace

cudaError_t LaunchObservationGather(const std::uint8_t *observations,
                                    const std::uint32_t *order, std::uint8_t *ordered,
                                    std::uint64_t count, std::uint64_t items,
                                    std::uint64_t per_item, cudaStream_t stream) {
  const std::uint64_t threads = count * items;
  if (threads == 0)
    return cudaSuccess;
  const std::uint64_t grid = (threads + kPhaseThreads - 1) / kPhaseThreads;
  if (grid > 0x7fffffffull)
    return cudaErrorInvalidConfiguration;
  ObservationGather<<<static_cast<unsigned>(grid), kPhaseThreads, 0, stream>>>(
      observations, order, ordered, count, items, per_item);
  return cudaGetLastError();
}

cudaError_t LaunchPhase(int scalar_bytes, bool compute_f64, int kind, const PhaseArgs &args,
                        cudaStream_t stream, int *blocks_per_sm) {
  if (args.states > 32)
    return scalar_bytes == 4 && !compute_f64 && !args.batch
               ? LaunchWidePhase(kind, args, stream, blocks_per_sm)
               : cudaErrorInvalidValue;
  if (args.states > 4) {
    if (args.batch)
      return cudaErrorInvalidValue;
    if (args.states <= 8)
      return compute_f64
                 ? LaunchGroupPhase8F64(scalar_bytes, kind, args, stream, blocks_per_sm)
                 : LaunchGroupPhase8F32(scalar_bytes, kind, args, stream, blocks_per_sm);
    if (args.states <= 16)
      return compute_f64
                 ? LaunchGroupPhase16F64(scalar_bytes, kind, args, stream, blocks_per_sm)
                 : LaunchGroupPhase16F32(scalar_bytes, kind, args, stream, blocks_per_sm);
    if (compute_f64)
      return LaunchGroupPhase32F64(scalar_bytes, kind, args, stream, blocks_per_sm);
    if (args.states <= 20)
      return LaunchGroupPhase20F32(scalar_bytes, kind, args, stream, blocks_per_sm);
    if (args.states <= 24)
      return LaunchGroupPhase24F32(scalar_bytes, kind, args, stream, blocks_per_sm);
    if (args.states <= 28)
      return LaunchGroupPhase28F32(scalar_bytes, kind, args, stream, blocks_per_sm);
    return LaunchGroupPhase32F32(scalar_bytes, kind, args, stream, blocks_per_sm);
  }
  if (scalar_bytes == 8)
    return compute_f64 ? LaunchTyped<double, double>(kind, args, stream, blocks_per_sm)
                       : LaunchTyped<double, float>(kind, args, stream, blocks_per_sm);
  return compute_f64 ? LaunchTyped<float, double>(kind, args, stream, blocks_per_sm)
                     : LaunchTyped<float, float>(kind, args, stream, blocks_per_sm);
}

} // namespace thmm
