// Max-product (MAP) kernels, float arithmetic (one translation unit per
// instance so the build compiles them in parallel).
#include "engine_launch.cuh"

namespace thmm {

cudaError_t LaunchMaximumF32(unsigned kmax, const EngineArgs &args, int grid, cudaStream_t stream,
                 int *blocks_per_sm) {
  return LaunchLogTyped<MaxEngine, float>(kmax, args, grid, stream, blocks_per_sm);
}

} // namespace thmm
