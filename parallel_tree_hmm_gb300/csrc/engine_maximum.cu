// Max-product (MAP) dispatch; arithmetic in the scalar width. The kernel
// instances live in engine_maximum_f{32,64}.cu.
#include "program.h"

namespace thmm {

cudaError_t LaunchMaximum(int scalar_bytes, unsigned kmax,
                          const EngineArgs &args, int grid, cudaStream_t stream,
                          int *blocks_per_sm) {
  return scalar_bytes == 8 ? LaunchMaximumF64(kmax, args, grid, stream, blocks_per_sm)
                           : LaunchMaximumF32(kmax, args, grid, stream, blocks_per_sm);
}

} // namespace thmm
