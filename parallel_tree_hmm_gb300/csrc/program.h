// Host-side compilation of btrc plans into the device program format of
// engine.h, and the kernel launch entry points implemented by the engine_*.cu
// translation units.
#ifndef THMM_PROGRAM_H_
#define THMM_PROGRAM_H_

#include <cstddef>
#include <cstdint>
#include <span>
#include <vector>

#include <cuda_runtime.h>

#include "btrc/plan.h"
#include "engine.h"
#include "program_builder.h"

namespace thmm {

// Programs of every distinct plan of a workspace, concatenated.
struct ProgramSet {
  std::vector<DevProgram> programs;
  std::vector<DevStep> steps;
  std::vector<Uint4> rakes;
  std::vector<Uint2> combines;
  std::vector<Uint4> absorbs;
  std::vector<Uint4> compress;
  std::vector<Uint2> compress_ends;
  std::vector<Uint4> gathers;

  template <class T> std::vector<T> Temp(std::size_t count, T value) {
    return std::vector<T>(count, value);
  }

  // Appends the program of `plan`; `observation_nodes` (strictly increasing)
  // gives each observed node its observation slot (categorical models).
  std::uint32_t Add(const btrc::Plan &plan,
                    std::span<const std::uint32_t> observation_nodes,
                    bool categorical);
};

struct ProgramRequest {
  const btrc::Plan *plan;
  std::span<const std::uint32_t> observation_nodes;
};

// Programs of `requests`, in order, as one ProgramSet. Contiguous runs of
// requests are compiled on up to `threads` host threads (0: all hardware
// threads) into separate sets that are then concatenated with their array
// offsets shifted, which gives exactly the arrays of a one-thread build.
ProgramSet BuildPrograms(std::span<const ProgramRequest> requests, bool categorical,
                         unsigned threads);

// Kernel entry points. `kmax` is the padded state count (4, 8, 16, 20, 24
// or 32; 64 or 128 for the wide-state engine).
// With `blocks_per_sm` non-null the call only reports the occupancy. The
// linear (sum-product) kernels come in two parts: 0 = forward sweep (log Z,
// root marginal), 1 = adjoint sweep (marginals), launched in that order.
cudaError_t LaunchLinearF32(bool compute_f64, unsigned kmax, int part,
                            const EngineArgs &args, int grid,
                            cudaStream_t stream, int *blocks_per_sm);
cudaError_t LaunchLinearF64(bool compute_f64, unsigned kmax, int part,
                            const EngineArgs &args, int grid,
                            cudaStream_t stream, int *blocks_per_sm);
cudaError_t LaunchMaximum(int scalar_bytes, unsigned kmax,
                          const EngineArgs &args, int grid, cudaStream_t stream,
                          int *blocks_per_sm);
cudaError_t LaunchSample(int scalar_bytes, unsigned kmax, const EngineArgs &args,
                         int grid, cudaStream_t stream, int *blocks_per_sm);

// Per-instance launchers behind the dispatchers above, one translation unit
// each (engine_linear_<scalar><compute>_<part>_<half>.cu for padded state
// counts up to 16 (Small) or above (Large), engine_maximum_f*.cu,
// engine_sample_f*.cu) so that the build compiles them in parallel.
#define THMM_DECLARE_LAUNCHER(NAME)                                                  \
  cudaError_t NAME(unsigned kmax, const EngineArgs &args, int grid, cudaStream_t stream, \
                   int *blocks_per_sm);
#define THMM_DECLARE_LINEAR(TYPES)                                                   \
  THMM_DECLARE_LAUNCHER(LaunchLinear##TYPES##ForwardSmall)                            \
  THMM_DECLARE_LAUNCHER(LaunchLinear##TYPES##ForwardLarge)                            \
  THMM_DECLARE_LAUNCHER(LaunchLinear##TYPES##ReverseSmall)                            \
  THMM_DECLARE_LAUNCHER(LaunchLinear##TYPES##ReverseLarge)
THMM_DECLARE_LINEAR(FF)
THMM_DECLARE_LINEAR(FD)
THMM_DECLARE_LINEAR(DF)
THMM_DECLARE_LINEAR(DD)
THMM_DECLARE_LAUNCHER(LaunchMaximumF32)
THMM_DECLARE_LAUNCHER(LaunchMaximumF64)
THMM_DECLARE_LAUNCHER(LaunchSampleF32)
THMM_DECLARE_LAUNCHER(LaunchSampleF64)
#undef THMM_DECLARE_LINEAR
#undef THMM_DECLARE_LAUNCHER

// Tensor-core sum-product kernels for 32 < K <= 128 (kmax 64 or 128, FP32).
cudaError_t LaunchWide(unsigned kmax, int part, const EngineArgs &args, int grid,
                       cudaStream_t stream, int *blocks_per_sm);
// One warp whose bounded mbarrier wait cannot complete and gives up after
// `budget` cycles, setting kErrorTensorTimeout in *error.
cudaError_t LaunchWaitTimeoutCheck(std::uint32_t *error, long long budget,
                                   cudaStream_t stream);

inline unsigned PaddedStates(std::size_t states) {
  return states <= 4    ? 4u
         : states <= 8  ? 8u
         : states <= 16 ? 16u
         : states <= 20 ? 20u
         : states <= 24 ? 24u
         : states <= 32 ? 32u
         : states <= 64 ? 64u
                        : 128u;
}

} // namespace thmm

#endif // THMM_PROGRAM_H_
