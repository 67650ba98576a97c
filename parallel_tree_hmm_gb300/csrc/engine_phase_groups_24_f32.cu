// Lane-group phase kernels with register rows of 24 (K in (20, 24]), float
// arithmetic.
#include "phase_groups_launch.cuh"

namespace thmm {

cudaError_t LaunchGroupPhase24F32(int scalar_bytes, int kind, const PhaseArgs &args,
                                   cudaStream_t stream, int *blocks_per_sm) {
  return group_phase::Launch<float, 24>(scalar_bytes, kind, args, stream, blocks_per_sm);
}

} // namespace thmm
