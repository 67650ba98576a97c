// Sum-product kernels, double inputs/outputs with float arithmetic, forward sweep,
// padded state counts 20, 24 and 32 (one translation unit per instance group so
// the build compiles them in parallel).
#include "engine_launch.cuh"

namespace thmm {

cudaError_t LaunchLinearDFForwardLarge(unsigned kmax, const EngineArgs &args, int grid,
                          cudaStream_t stream, int *blocks_per_sm) {
  return LaunchLinearHalf<double, float, kLinearForward, false>(kmax, args, grid, stream, blocks_per_sm);
}

} // namespace thmm
