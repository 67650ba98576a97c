// Max-product (MAP) kernels; arithmetic in the scalar width.
#include "engine_launch.cuh"

namespace thmm {

cudaError_t LaunchMaximum(int scalar_bytes, unsigned kmax,
                          const EngineArgs &args, int grid, cudaStream_t stream,
                          int *blocks_per_sm) {
  return scalar_bytes == 8
             ? LaunchLogTyped<MaxEngine, double>(kmax, args, grid, stream,
                                                 blocks_per_sm)
             : LaunchLogTyped<MaxEngine, float>(kmax, args, grid, stream,
                                                blocks_per_sm);
}

} // namespace thmm
