// Posterior-sampling kernels, double arithmetic (one translation unit per
// instance so the build compiles them in parallel).
#include "engine_launch.cuh"

namespace thmm {

cudaError_t LaunchSampleF64(unsigned kmax, const EngineArgs &args, int grid, cudaStream_t stream,
                 int *blocks_per_sm) {
  return LaunchLogTyped<SampleEngine, double>(kmax, args, grid, stream, blocks_per_sm);
}

} // namespace thmm
