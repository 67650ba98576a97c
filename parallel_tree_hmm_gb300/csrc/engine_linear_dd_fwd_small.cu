// Sum-product kernels, double inputs/outputs with double arithmetic, forward sweep,
// padded state counts 4, 8 and 16 (one translation unit per instance group so
// the build compiles them in parallel).
#include "engine_launch.cuh"

namespace thmm {

cudaError_t LaunchLinearDDForwardSmall(unsigned kmax, const EngineArgs &args, int grid,
                          cudaStream_t stream, int *blocks_per_sm) {
  return LaunchLinearHalf<double, double, kLinearForward, true>(kmax, args, grid, stream, blocks_per_sm);
}

} // namespace thmm
