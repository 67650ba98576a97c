// Lane-group phase kernels for padded state count 16, float arithmetic.
#include "phase_groups_launch.cuh"

namespace thmm {

cudaError_t LaunchGroupPhase16F32(int scalar_bytes, int kind, const PhaseArgs &args,
                                   cudaStream_t stream, int *blocks_per_sm) {
  return group_phase::Launch<float, 16>(scalar_bytes, kind, args, stream, blocks_per_sm);
}

} // namespace thmm
