// Launchers of the phase kernels (phase_engine.cuh) for every input and
// arithmetic type.
#include "phase_engine.cuh"

namespace thmm {
namespace {

template <typename Scalar, typename Compute, int kKind>
cudaError_t LaunchKind(const PhaseArgs &args, cudaStream_t stream, int *blocks_per_sm) {
  auto kernel = PhaseKernel<Scalar, Compute, kKind>;
  if (blocks_per_sm != nullptr)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel,
                                                         kPhaseThreads, 0);
  if (args.count == 0)
    return cudaSuccess;
  const unsigned grid = (args.count + kPhaseThreads - 1) / kPhaseThreads;
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
  default:
    return cudaErrorInvalidValue;
  }
}

} // namespace

cudaError_t LaunchPhase(int scalar_bytes, bool compute_f64, int kind, const PhaseArgs &args,
                        cudaStream_t stream, int *blocks_per_sm) {
  if (scalar_bytes == 8)
    return compute_f64 ? LaunchTyped<double, double>(kind, args, stream, blocks_per_sm)
                       : LaunchTyped<double, float>(kind, args, stream, blocks_per_sm);
  return compute_f64 ? LaunchTyped<float, double>(kind, args, stream, blocks_per_sm)
                     : LaunchTyped<float, float>(kind, args, stream, blocks_per_sm);
}

} // namespace thmm
