// Posterior-sampling kernels; arithmetic in the scalar width.
#include "engine_launch.cuh"

namespace thmm {

cudaError_t LaunchSample(int scalar_bytes, unsigned kmax, const EngineArgs &args,
                         int grid, cudaStream_t stream, int *blocks_per_sm) {
  return scalar_bytes == 8
             ? LaunchLogTyped<SampleEngine, double>(kmax, args, grid, stream,
                                                    blocks_per_sm)
             : LaunchLogTyped<SampleEngine, float>(kmax, args, grid, stream,
                                                   blocks_per_sm);
}

} // namespace thmm
