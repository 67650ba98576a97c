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

// Launches (or queries) the sum-product kernel of one part for padded state
// count kmax, restricted to kmax <= 16 (kSmall) or > 16 so that each half
// compiles in its own translation unit.
template <typename Scalar, typename Compute, int kPart, bool kSmall>
cudaError_t LaunchLinearHalf(unsigned kmax, const EngineArgs &args, int grid,
                             cudaStream_t stream, int *blocks_per_sm) {
  if constexpr (kSmall) {
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
    default:
      return cudaErrorInvalidValue;
    }
  } else {
    switch (kmax) {
    case 20:
      return LaunchOrQuery<LinearEngine<Scalar, Compute, 20, kPart>, Compute, true>(
          args, grid, stream, blocks_per_sm);
    case 24:
      return LaunchOrQuery<LinearEngine<Scalar, Compute, 24, kPart>, Compute, true>(
          args, grid, stream, blocks_per_sm);
    case 32:
      return LaunchOrQuery<LinearEngine<Scalar, Compute, 32, kPart>, Compute, true>(
          args, grid, stream, blocks_per_sm);
    default:
      return cudaErrorInvalidValue;
    }
  }
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
  case 20:
    return LaunchOrQuery<Engine<T, 20>, T, false>(args, grid, stream, blocks_per_sm);
  case 24:
    return LaunchOrQuery<Engine<T, 24>, T, false>(args, grid, stream, blocks_per_sm);
  case 32:
    return LaunchOrQuery<Engine<T, 32>, T, false>(args, grid, stream, blocks_per_sm);
  default:
    return cudaErrorInvalidValue;
  }
}

} // namespace thmm

#endif // THMM_ENGINE_LAUNCH_CUH_
