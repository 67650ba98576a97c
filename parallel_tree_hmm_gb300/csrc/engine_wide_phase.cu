// Launchers of the wide-state phase kernels (wide_phase.cuh), 32 < K <= 128.
#include "wide_phase.cuh"

namespace thmm {
namespace {

template <int KP, int kKind>
cudaError_t LaunchWideKind(const PhaseArgs &args, cudaStream_t stream, int *blocks_per_sm) {
  constexpr bool kTensor = kKind == kPhaseCompress || kKind == kPhaseCompressReverse;
  using L = wide::PhaseLayout<KP>;
  auto kernel = wide::WidePhaseKernel<KP, kKind>;
  const int smem = static_cast<int>(kTensor ? L::kSmemBytes : wide::kVectorBytes);
  cudaError_t status =
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  // The largest shared-memory carve-out, so that the occupancy query (and
  // the SM) count on as many resident CTAs as the layout allows.
  if (status == cudaSuccess && kTensor)
    status = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  cudaSharedmemCarveoutMaxShared);
  if (status != cudaSuccess)
    return status;
  int per_sm = 0;
  status = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, L::kThreads, smem);
  if (status != cudaSuccess || blocks_per_sm != nullptr) {
    if (blocks_per_sm != nullptr)
      *blocks_per_sm = per_sm;
    return status;
  }
  if (args.count == 0)
    return cudaSuccess;
  if (kTensor)
    per_sm = L::kResident;
  int device = 0, sms = 0;
  status = cudaGetDevice(&device);
  if (status == cudaSuccess)
    status = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (status != cudaSuccess)
    return status;
  // A persistent grid: every CTA resident at once, each taking every
  // grid-th operation.
  const std::uint64_t slots =
      static_cast<std::uint64_t>(sms) * static_cast<std::uint64_t>(per_sm > 0 ? per_sm : 1);
  const unsigned grid = static_cast<unsigned>(args.count < slots ? args.count : slots);
  kernel<<<grid, L::kThreads, smem, stream>>>(args);
  return cudaGetLastError();
}

template <int KP>
cudaError_t LaunchWideTyped(int kind, const PhaseArgs &args, cudaStream_t stream,
                            int *blocks_per_sm) {
  switch (kind) {
  case kPhaseGather:
    return LaunchWideKind<KP, kPhaseGather>(args, stream, blocks_per_sm);
  case kPhaseCompress:
    return LaunchWideKind<KP, kPhaseCompress>(args, stream, blocks_per_sm);
  case kPhaseFinish:
    return LaunchWideKind<KP, kPhaseFinish>(args, stream, blocks_per_sm);
  case kPhaseRakeReverse:
    return LaunchWideKind<KP, kPhaseRakeReverse>(args, stream, blocks_per_sm);
  case kPhaseCompressReverse:
    return LaunchWideKind<KP, kPhaseCompressReverse>(args, stream, blocks_per_sm);
  default:
    return cudaErrorInvalidValue; // no tail kinds: every round runs grid-wide
  }
}

} // namespace

cudaError_t LaunchWidePhase(int kind, const PhaseArgs &args, cudaStream_t stream,
                            int *blocks_per_sm) {
  if (args.states > 32 && args.states <= 64)
    return LaunchWideTyped<64>(kind, args, stream, blocks_per_sm);
  if (args.states > 64 && args.states <= 128)
    return LaunchWideTyped<128>(kind, args, stream, blocks_per_sm);
  return cudaErrorInvalidValue;
}

} // namespace thmm
