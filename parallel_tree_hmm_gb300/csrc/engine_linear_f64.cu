// Sum-product dispatch for double inputs/outputs (FP32 or FP64 arithmetic).
// The kernel instances live in engine_linear_d{f,d}_{fwd,rev}_{small,large}.cu.
#include "program.h"

namespace thmm {

cudaError_t LaunchLinearF64(bool compute_f64, unsigned kmax, int part,
                            const EngineArgs &args, int grid,
                            cudaStream_t stream, int *blocks_per_sm) {
  if (kmax > 32)
    return cudaErrorInvalidValue;
  const bool small = kmax <= 16;
  if (compute_f64) {
    if (part == 1)
      return small ? LaunchLinearDDReverseSmall(kmax, args, grid, stream, blocks_per_sm)
                   : LaunchLinearDDReverseLarge(kmax, args, grid, stream, blocks_per_sm);
    return small ? LaunchLinearDDForwardSmall(kmax, args, grid, stream, blocks_per_sm)
                 : LaunchLinearDDForwardLarge(kmax, args, grid, stream, blocks_per_sm);
  }
  if (part == 1)
    return small ? LaunchLinearDFReverseSmall(kmax, args, grid, stream, blocks_per_sm)
                 : LaunchLinearDFReverseLarge(kmax, args, grid, stream, blocks_per_sm);
  return small ? LaunchLinearDFForwardSmall(kmax, args, grid, stream, blocks_per_sm)
               : LaunchLinearDFForwardLarge(kmax, args, grid, stream, blocks_per_sm);
}

} // namespace thmm
