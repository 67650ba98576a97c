// Sum-product kernels, float inputs/outputs with double arithmetic, adjoint sweep,
// padded state counts 20, 24 and 32 (one translation unit per instance group so
// the build compiles them in parallel).
#include "engine_launch.cuh"

namespace thmm {

cudaError_t LaunchLinearFDReverseLarge(unsigned kmax, const EngineArgs &args, int grid,
                          cudaStream_t stream, int *blocks_per_sm) {
  return LaunchLinearHalf<float, double, kLinearReverse, false>(kmax, args, grid, stream, blocks_per_sm);
}

} // namespace thmm
