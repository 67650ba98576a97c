// Tensor-core sum-product kernels for 32 < K <= 128 states (FP32).
#include "program.h"
#include "wide_engine.cuh"

namespace thmm {

cudaError_t LaunchWide(unsigned kmax, int part, const EngineArgs &args, int grid,
                       cudaStream_t stream, int *blocks_per_sm) {
  switch (kmax) {
  case 64:
    return part == kLinearReverse
               ? wide::LaunchWidePart<64, kLinearReverse>(args, grid, stream, blocks_per_sm)
               : wide::LaunchWidePart<64, kLinearForward>(args, grid, stream, blocks_per_sm);
  case 128:
    return part == kLinearReverse
               ? wide::LaunchWidePart<128, kLinearReverse>(args, grid, stream, blocks_per_sm)
               : wide::LaunchWidePart<128, kLinearForward>(args, grid, stream, blocks_per_sm);
  default:
    return cudaErrorInvalidValue;
  }
}

} // namespace thmm
