// Launch helper shared by the engine_*.cu translation units.
#ifndef THMM_ENGINE_LAUNCH_CUH_
#define THMM_ENGINE_LAUNCH_CUH_

#include "engine.cuh"
#include "program.h"

namespace thmm {

// Launches EngineKernel<Engine> with `grid` CTAs, or reports its occupancy
// when `blocks_per_sm` is non-null. Linear engines get one K*K scratch tile
// per lane group in shared memory for the reverse sweep.
template <class Engine, typename Buffer, bool kGroupTiles>
cudaError_t LaunchOrQuery(const EngineArgs &args, int grid, cudaStream_t stream,
                          int *blocks_per_sm) {
  // Group tiles are only used when several lanes share an operation.
  const std::size_t smem = kGroupTiles && Engine::G > 1
                               ? std::size_t{kWarps} * 32 * Engine::G * sizeof(Buffer)
                               : 0;
  auto kernel = EngineKernel<Engine, Buffer>;
  if (smem > 48 * 1024) {
    const cudaError_t status = cudaFuncSetAttribute(
        kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (status != cudaSuccess)
      return status;
  }
  if (blocks_per_sm != nullptr)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kernel,
                                                         kThreads, smem);
  kernel<<<grid, kThreads, smem, stream>>>(args);
  return cudaGetLastError();
}

template <typename Scalar, typename Compute, int kPart>
cudaError_t LaunchLinearPart(unsigned kmax, const EngineArgs &args, int grid,
                             cudaStream_t stream, int *blocks_per_sm) {
  switch (kmax) {
  case 4:
    return LaunchOrQuery<LinearEngine<Scalar, Compute, 4, kPart>, Compute, true>(
        args, grid, stream, blocks_per_sm);
  case 8:
    return LaunchOrQuery<LinearEngine<Scalar, Compute, 8, kPart>, Compute, true>(
        args, grid, stream, blocks_per_sm);
  case 16:
    return LaunchOrQuery<LinearEngine<Scalar, Compute, 16, kPart>, Compute, true>(
        args, grid, stream, blocks_per_sm);
  case 32:
    return LaunchOrQuery<LinearEngine<Scalar, Compute, 32, kPart>, Compute, true>(
        args, grid, stream, blocks_per_sm);
  default:
    return cudaErrorInvalidValue;
  }
}

// `part` selects the forward sweep (kLinearForward) or the adjoint sweep
// (kLinearReverse).
template <typename Scalar, typename Compute>
cudaError_t LaunchLinearTyped(unsigned kmax, int part, const EngineArgs &args, int grid,
                              cudaStream_t stream, int *blocks_per_sm) {
  return part == kLinearReverse
             ? LaunchLinearPart<Scalar, Compute, kLinearReverse>(kmax, args, grid, stream,
                                                                 blocks_per_sm)
             : LaunchLinearPart<Scalar, Compute, kLinearForward>(kmax, args, grid, stream,
                                                                 blocks_per_sm);
}

template <template <typename, int> class Engine, typename T>
cudaError_t LaunchLogTyped(unsigned kmax, const EngineArgs &args, int grid,
                           cudaStream_t stream, int *blocks_per_sm) {
  switch (kmax) {
  case 4:
    return LaunchOrQuery<Engine<T, 4>, T, false>(args, grid, stream, blocks_per_sm);
  case 8:
    return LaunchOrQuery<Engine<T, 8>, T, false>(args, grid, stream, blocks_per_sm);
  case 16:
    return LaunchOrQuery<Engine<T, 16>, T, false>(args, grid, stream, blocks_per_sm);
  case 32:
    return LaunchOrQuery<Engine<T, 32>, T, false>(args, grid, stream, blocks_per_sm);
  default:
    return cudaErrorInvalidValue;
  }
}

} // namespace thmm

#endif // THMM_ENGINE_LAUNCH_CUH_
