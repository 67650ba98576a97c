// Sum-product dispatch for float inputs/outputs (FP32 or FP64 arithmetic;
// tensor-core engine above 32 states). The kernel instances live in
// engine_linear_f{f,d}_{fwd,rev}_{small,large}.cu.
#include "program.h"

namespace thmm {

cudaError_t LaunchLinearF32(bool compute_f64, unsigned kmax, int part,
                            const EngineArgs &args, int grid,
                            cudaStream_t stream, int *blocks_per_sm) {
  if (kmax > 32)
    return compute_f64 ? cudaErrorInvalidValue
                       : LaunchWide(kmax, part, args, grid, stream, blocks_per_sm);
  const bool small = kmax <= 16;
  if (compute_f64) {
    if (part == 1)
      return small ? LaunchLinearFDReverseSmall(kmax, args, grid, stream, blocks_per_sm)
                   : LaunchLinearFDReverseLarge(kmax, args, grid, stream, blocks_per_sm);
    return small ? LaunchLinearFDForwardSmall(kmax, args, grid, stream, blocks_per_sm)
                 : LaunchLinearFDForwardLarge(kmax, args, grid, stream, blocks_per_sm);
  }
  if (part == 1)
    return small ? LaunchLinearFFReverseSmall(kmax, args, grid, stream, blocks_per_sm)
                 : LaunchLinearFFReverseLarge(kmax, args, grid, stream, blocks_per_sm);
  return small ? LaunchLinearFFForwardSmall(kmax, args, grid, stream, blocks_per_sm)
               : LaunchLinearFFForwardLarge(kmax, args, grid, stream, blocks_per_sm);
}

} // namespace thmm
