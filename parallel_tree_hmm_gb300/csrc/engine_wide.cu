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

namespace {

// One warp: takes 32 tensor-memory columns, announces 16 bytes of bulk copy
// on an mbarrier but issues no copy and no MMA, so the phase never completes
// and every lane's bounded wait gives up after `budget` cycles; the timeout
// is recorded exactly as the wide-state kernels record it, and the columns
// are released as those kernels release them.
__global__ void __launch_bounds__(32) WaitTimeoutKernel(std::uint32_t *error,
                                                        long long budget) {
  __shared__ std::uint64_t barrier;
  __shared__ std::uint32_t tmem;
  umma::Allocate(&tmem, 32);
  if (threadIdx.x == 0) {
    umma::BarrierInit(&barrier);
    umma::ExpectBytes(&barrier, 16);
  }
  __syncwarp();
  umma::FenceAfterSync();
  const bool ok = umma::Wait(&barrier, 0, budget);
  if (!ok && threadIdx.x == 0)
    atomicOr(error, kErrorTensorTimeout);
  umma::FenceBeforeSync();
  __syncwarp();
  umma::Deallocate(tmem, 32);
}

} // namespace

cudaError_t LaunchWaitTimeoutCheck(std::uint32_t *error, long long budget,
                                   cudaStream_t stream) {
  WaitTimeoutKernel<<<1, 32, 0, stream>>>(error, budget);
  return cudaGetLastError();
}

} // namespace thmm
