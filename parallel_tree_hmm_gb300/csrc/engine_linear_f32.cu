// Sum-product kernels for float inputs/outputs (FP32 or FP64 arithmetic).
#include "engine_launch.cuh"

namespace thmm {

cudaError_t LaunchLinearF32(bool compute_f64, unsigned kmax, int part,
                            const EngineArgs &args, int grid,
                            cudaStream_t stream, int *blocks_per_sm) {
  if (kmax > 32)
    return compute_f64 ? cudaErrorInvalidValue
                       : LaunchWide(kmax, part, args, grid, stream, blocks_per_sm);
  return compute_f64 ? LaunchLinearTyped<float, double>(kmax, part, args, grid, stream,
                                                        blocks_per_sm)
                     : LaunchLinearTyped<float, float>(kmax, part, args, grid, stream,
                                                       blocks_per_sm);
}

} // namespace thmm
