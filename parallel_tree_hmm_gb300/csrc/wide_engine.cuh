// Sum-product kernels for 32 < K <= 128 states ("wide" states) on sm_103a.
//
// One CTA of 128 threads contracts one tree at a time (trees come from the
// same largest-first queue as the narrow engines), and handles the operations
// of a step one after another with the whole CTA:
//   * rake messages (K x K matrix times vector): warp w takes rows w, w+4, ...,
//     lanes stride the columns with coalesced loads, shuffle reductions;
//   * compress products left * diag(middle) * right, and the two products of
//     their adjoint, run on the tensor cores (tcgen05, kind::tf32) with the
//     accumulators in tensor memory. Each FP32 operand x is split into
//     hi = x rounded to the nearest TF32 value and lo = x - hi (exact), and
//     the product is accumulated in FP32 as
//     lo*hi + hi*lo + hi*hi ("3xTF32"; the dropped lo*lo term is below
//     2^-22 relative), so the result has close to FP32 accuracy.
// Renormalisation and the log-scale bookkeeping are those of the narrow
// LinearEngine (engine.cuh): every produced message or compressed path is
// divided by an exact power of two, exponents are summed in an integer and
// log Z = ln2 * sum + log(sum(root)) is formed in FP64.
//
// Shared memory: four 32 KB operand buffers (X hi/lo, Y hi/lo for a product
// depth of 64) plus a few K-vectors, so one CTA runs per SM and it may hold
// all 512 tensor-memory columns. Every tensor-core wait is bounded; a wait
// that gives up sets kErrorTensorTimeout and the host reports an error.
#ifndef THMM_WIDE_ENGINE_CUH_
#define THMM_WIDE_ENGINE_CUH_

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.cuh"
#include "umma.cuh"

namespace thmm {
namespace wide {

constexpr unsigned kThreads = 128;
constexpr unsigned kChunk = 64;                      // product depth staged at once
constexpr unsigned kOperandBytes = 128 * kChunk * 4; // one hi or lo operand (32 KB)
constexpr std::uint32_t kSbo = kChunk / 4 * 128;     // 2048 bytes between 8-row groups
constexpr unsigned kVectors = 6;                     // K-vectors of 128 floats
constexpr unsigned kSmemBytes = 4 * kOperandBytes + kVectors * 128 * 4;
constexpr std::uint32_t kTmemColumns = 512;
// Tensor-memory columns of the three accumulators of a reverse compression.
constexpr std::uint32_t kProductColumn = 0, kLeftColumn = 128, kRightColumn = 256;

struct Shared {
  std::uint64_t barrier;
  double root_sum;
  std::uint32_t tmem;
  unsigned item;
  int root_finite;
  float reduce[kThreads / 32];
};

// The TF32 part of v, rounded to nearest (ties away from zero) so that the
// remainder v - Hi(v), exact in FP32, has either sign and the split carries
// no bias.
__device__ __forceinline__ float Hi(float v) {
  return __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xffffe000u);
}

__device__ __forceinline__ float WarpSum(float v) {
#pragma unroll
  for (int offset = 16; offset > 0; offset >>= 1)
    v += __shfl_xor_sync(kFull, v, offset);
  return v;
}

__device__ __forceinline__ float WarpMax(float v) {
#pragma unroll
  for (int offset = 16; offset > 0; offset >>= 1) {
    const float other = __shfl_xor_sync(kFull, v, offset);
    v = v < other ? other : v;
  }
  return v;
}

// Maximum of `v` over the CTA (values are nonnegative).
__device__ __forceinline__ float BlockMax(float v, Shared &sh) {
  v = WarpMax(v);
  if ((threadIdx.x & 31) == 0)
    sh.reduce[threadIdx.x / 32] = v;
  __syncthreads();
  float m = sh.reduce[0];
#pragma unroll
  for (unsigned w = 1; w < kThreads / 32; ++w)
    m = m < sh.reduce[w] ? sh.reduce[w] : m;
  __syncthreads();
  return m;
}

// Tensor-memory lanes 0..127 (one per thread), columns [column, column + KP):
//   D[r][n] = sum_d X(r, d) * Y(n, d),  r < 128, n < KP, d < KP,
// in 3xTF32 with FP32 accumulation. The functors return 0 outside the K x K
// block. kXRows (kYRows): the source of X (Y) is read with d running fastest
// across threads (row-major source); otherwise r (n) runs fastest. Returns
// false if a tensor-core wait timed out.
template <int KP, bool kXRows, bool kYRows, class XF, class YF>
__device__ bool Product(unsigned char *smem, Shared &sh, std::uint32_t &phase,
                        std::uint32_t tmem, XF x, YF y) {
  static_assert(KP % kChunk == 0 && KP <= 128, "padded state count");
  const unsigned tid = threadIdx.x;
  unsigned char *const xh = smem;
  unsigned char *const xl = smem + kOperandBytes;
  unsigned char *const yh = smem + 2 * kOperandBytes;
  unsigned char *const yl = smem + 3 * kOperandBytes;
  constexpr std::uint32_t kDescriptor = umma::Tf32Descriptor(128, KP);
  bool ok = true;
#pragma unroll 1
  for (unsigned chunk = 0; chunk < KP / kChunk; ++chunk) {
    const unsigned d0 = chunk * kChunk;
#pragma unroll 4
    for (unsigned idx = tid; idx < 128 * kChunk; idx += kThreads) {
      const unsigned r = kXRows ? idx / kChunk : idx % 128;
      const unsigned d = kXRows ? idx % kChunk : idx / 128;
      const float v = x(r, d0 + d);
      const float h = Hi(v);
      const std::uint32_t at = umma::CoreOffset(r, d, kSbo);
      *reinterpret_cast<float *>(xh + at) = h;
      *reinterpret_cast<float *>(xl + at) = v - h;
    }
#pragma unroll 4
    for (unsigned idx = tid; idx < KP * kChunk; idx += kThreads) {
      const unsigned n = kYRows ? idx / kChunk : idx % KP;
      const unsigned d = kYRows ? idx % kChunk : idx / KP;
      const float v = y(n, d0 + d);
      const float h = Hi(v);
      const std::uint32_t at = umma::CoreOffset(n, d, kSbo);
      *reinterpret_cast<float *>(yh + at) = h;
      *reinterpret_cast<float *>(yl + at) = v - h;
    }
    umma::FenceOperands();
    umma::FenceBeforeSync();
    __syncthreads();
    umma::FenceAfterSync();
    if (tid == 0) {
      const std::uint32_t xh_at = umma::SmemAddress(xh), xl_at = umma::SmemAddress(xl);
      const std::uint32_t yh_at = umma::SmemAddress(yh), yl_at = umma::SmemAddress(yl);
      const std::uint32_t a_parts[3] = {xl_at, xh_at, xh_at};
      const std::uint32_t b_parts[3] = {yh_at, yl_at, yh_at};
#pragma unroll
      for (int part = 0; part < 3; ++part) {
#pragma unroll
        for (unsigned k = 0; k < kChunk / 8; ++k) {
          const std::uint64_t a = umma::SmemDescriptor(a_parts[part] + k * 256, kSbo);
          const std::uint64_t b = umma::SmemDescriptor(b_parts[part] + k * 256, kSbo);
          umma::MmaTf32(tmem, a, b, kDescriptor, chunk != 0 || part != 0 || k != 0);
        }
      }
      umma::Commit(&sh.barrier);
    }
    ok = umma::Wait(&sh.barrier, phase) && ok;
    phase ^= 1u;
    umma::FenceAfterSync();
  }
  return ok;
}

} // namespace wide
} // namespace thmm

#include "wide_engine_tree.cuh"

#endif // THMM_WIDE_ENGINE_CUH_
