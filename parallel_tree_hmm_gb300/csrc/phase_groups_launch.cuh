// Launchers of the lane-group phase kernels (phase_groups.cuh) for one
// padded state count; included by engine_phase_groups_*.cu, one translation
// unit per padded state count so that the build compiles them in parallel.
#ifndef THMM_PHASE_GROUPS_LAUNCH_CUH_
#define THMM_PHASE_GROUPS_LAUNCH_CUH_

#include "phase_groups.cuh"

namespace thmm {
namespace group_phase {

template <typename Scalar, typename Compute, int KMAX, int kKind>
cudaError_t LaunchKind(const PhaseArgs &args, cudaStream_t stream, int *blocks_per_sm) {
  auto kernel = GroupPhaseKernel<Scalar, Compute, KMAX, kKind>;
  const unsigned smem = GroupPhaseSmem<Compute, KMAX>(kKind);
  if (smem > 48 * 1024) {
    const cudaError_t status = cudaFuncSetAttribute(
        kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (status != cudaSuccess)
      return status;
  }
  if (blocks_per_sm != nullptr)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel,
                                                         kGroupPhaseThreads, smem);
  if (args.count == 0)
    return cudaSuccess;
  // Finish: one thread per instance; the other kinds one lane group per
  // operation.
  const std::uint64_t threads =
      kKind == kPhaseFinish ? static_cast<std::uint64_t>(args.count)
                            : static_cast<std::uint64_t>(args.count) * GroupLanes<KMAX>();
  const std::uint64_t grid = (threads + kGroupPhaseThreads - 1) / kGroupPhaseThreads;
  if (grid > 0x7fffffffull)
    return cudaErrorInvalidConfiguration;
  kernel<<<static_cast<unsigned>(grid), kGroupPhaseThreads, smem, stream>>>(args);
  return cudaGetLastError();
}

template <typename Scalar, typename Compute, int KMAX>
cudaError_t LaunchTyped(int kind, const PhaseArgs &args, cudaStream_t stream,
                        int *blocks_per_sm) {
  switch (kind) {
  case kPhaseGather:
    return LaunchKind<Scalar, Compute, KMAX, kPhaseGather>(args, stream, blocks_per_sm);
  case kPhaseCompress:
    return LaunchKind<Scalar, Compute, KMAX, kPhaseCompress>(args, stream, blocks_per_sm);
  case kPhaseFinish:
    return LaunchKind<Scalar, Compute, KMAX, kPhaseFinish>(args, stream, blocks_per_sm);
  case kPhaseRakeReverse:
    return LaunchKind<Scalar, Compute, KMAX, kPhaseRakeReverse>(args, stream, blocks_per_sm);
  case kPhaseCompressReverse:
    return LaunchKind<Scalar, Compute, KMAX, kPhaseCompressReverse>(args, stream,
                                                                    blocks_per_sm);
  default:
    return cudaErrorInvalidValue; // no tail kinds: every round runs grid-wide
  }
}

// Compute type fixed by the translation unit; scalar_bytes picks the
// input/output type.
template <typename Compute, int KMAX>
cudaError_t Launch(int scalar_bytes, int kind, const PhaseArgs &args, cudaStream_t stream,
                   int *blocks_per_sm) {
  return scalar_bytes == 8
             ? LaunchTyped<double, Compute, KMAX>(kind, args, stream, blocks_per_sm)
             : LaunchTyped<float, Compute, KMAX>(kind, args, stream, blocks_per_sm);
}

} // namespace group_phase
} // namespace thmm

#endif // THMM_PHASE_GROUPS_LAUNCH_CUH_
