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
// Shared memory: four operand buffers (X hi/lo, Y hi/lo for a product depth
// of 64) plus a few K-vectors; one CTA per SM (see Layout). Every tensor-core wait is bounded; a wait
// that gives up sets kErrorTensorTimeout and the host reports an error.
#ifndef THMM_WIDE_ENGINE_CUH_
#define THMM_WIDE_ENGINE_CUH_

#include <cstdint>
#include <type_traits>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "engine.cuh"
#include "umma.cuh"

namespace thmm {
namespace wide {

constexpr unsigned kThreads = 128;
constexpr unsigned kChunk = 64;                  // product depth staged at once
constexpr std::uint32_t kSbo = kChunk / 4 * 128; // 2048 bytes between 8-row groups
constexpr unsigned kVectors = 6;                 // K-vectors of 128 floats

// Shared- and tensor-memory layout for padded state count KP. X operands
// have M = 128 rows, Y operands N = KP rows, both a depth chunk of 64; the
// three accumulators of a reverse compression sit at columns 0, KP and 2 KP.
// One CTA per SM holds all 512 TMEM columns: the dynamic shared memory is
// padded to more than half of the SM's 228 KB so that a second CTA cannot
// be resident (and wait on the allocation). Two CTAs per SM at KP = 64 (99 KB
// each, 256 columns) measured slower: the shared-memory carve-out left the
// operand-staging loads too little L1.
template <int KP> struct Layout {
  static constexpr unsigned kXBytes = 128 * kChunk * 4;
  static constexpr unsigned kYBytes = KP * kChunk * 4;
  static constexpr unsigned kXh = 0, kXl = kXBytes;
  static constexpr unsigned kYh = 2 * kXBytes, kYl = 2 * kXBytes + kYBytes;
  static constexpr unsigned kVectorsAt = 2 * kXBytes + 2 * kYBytes;
  // At KP = 64, two sets of three raw K x K matrices (path versions and the
  // adjoint): one set feeds the current operation while the bulk copy of the
  // next operation's set is in flight.
  static constexpr unsigned kRawCount = KP == 64 ? 6 : 0;
  static constexpr unsigned kRawBytes = KP * KP * 4;
  static constexpr unsigned kRawAt = kVectorsAt + kVectors * 128 * 4;
  static constexpr unsigned kUsedBytes = kRawAt + kRawCount * kRawBytes;
  static constexpr unsigned kSmemBytes = kUsedBytes > 116 * 1024 ? kUsedBytes : 116 * 1024;
  static constexpr std::uint32_t kTmemColumns = 512;
  static constexpr std::uint32_t kProductColumn = 0, kLeftColumn = KP, kRightColumn = 2 * KP;
  static constexpr int kCtasPerSm = 1;
  static_assert(2 * kSmemBytes > 228 * 1024, "a second CTA would wait on TMEM");
};

struct Shared {
  std::uint64_t barrier;         // tensor-core completion
  std::uint64_t copy_barrier[2]; // bulk-copy completion, one per raw set
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

// Operand sources. A product operand is a K x K block of a row-major K x K
// matrix in global memory, read either as stored (element (r, d) at
// p[r * K + d], optionally times scale[d]) or transposed (element (r, d) at
// p[d * K + r]).
struct RowMajor {
  const float *p;
  const float *scale; // shared-memory column scale, or null
  __device__ __forceinline__ float operator()(unsigned K, unsigned r, unsigned d) const {
    const float v = p[static_cast<std::size_t>(r) * K + d];
    return scale != nullptr ? v * scale[d] : v;
  }
  // Elements d .. d + 3 of row r (K a multiple of 4, so 16-byte aligned).
  __device__ __forceinline__ float4 Quad(unsigned K, unsigned r, unsigned d) const {
    float4 v = *reinterpret_cast<const float4 *>(p + static_cast<std::size_t>(r) * K + d);
    if (scale != nullptr) {
      v.x *= scale[d];
      v.y *= scale[d + 1];
      v.z *= scale[d + 2];
      v.w *= scale[d + 3];
    }
    return v;
  }
};
struct Transposed {
  const float *p;
  __device__ __forceinline__ float operator()(unsigned K, unsigned r, unsigned d) const {
    return p[static_cast<std::size_t>(d) * K + r];
  }
};

__device__ __forceinline__ void StoreSplit(unsigned char *hi, unsigned char *lo,
                                           std::uint32_t at, float v) {
  const float h = Hi(v);
  *reinterpret_cast<float *>(hi + at) = h;
  *reinterpret_cast<float *>(lo + at) = v - h;
}
__device__ __forceinline__ void StoreSplit(unsigned char *hi, unsigned char *lo,
                                           std::uint32_t at, float4 v) {
  const float4 h = make_float4(Hi(v.x), Hi(v.y), Hi(v.z), Hi(v.w));
  *reinterpret_cast<float4 *>(hi + at) = h;
  *reinterpret_cast<float4 *>(lo + at) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
}

// Writes rows r < K, depths [d0, d0 + kChunk) ∩ [0, K) of one operand as
// TF32 hi/lo parts; everything else in the buffers stays zero (they are
// cleared once per launch), so padded rows and depths contribute nothing.
template <class Source>
__device__ __forceinline__ void Stage(const Source &src, unsigned K, unsigned d0,
                                      unsigned char *hi, unsigned char *lo) {
  const unsigned depth = K > d0 ? (K - d0 < kChunk ? K - d0 : kChunk) : 0u;
  if (d0 != 0 && depth < kChunk) {
    // A later chunk: clear depths [depth, kChunk) left over from the first.
    const unsigned pad = kChunk - depth;
    for (unsigned idx = threadIdx.x; idx < K * pad; idx += kThreads) {
      const std::uint32_t at = umma::CoreOffset(idx / pad, depth + idx % pad, kSbo);
      *reinterpret_cast<float *>(hi + at) = 0.0f;
      *reinterpret_cast<float *>(lo + at) = 0.0f;
    }
  }
  if constexpr (std::is_same_v<Source, RowMajor>) {
    if (K % 4 == 0) {
      const unsigned quads = depth / 4;
#pragma unroll 4
      for (unsigned idx = threadIdx.x; idx < K * quads; idx += kThreads) {
        const unsigned r = idx / quads, q = idx % quads;
        StoreSplit(hi, lo, umma::CoreOffset(r, 4 * q, kSbo), src.Quad(K, r, d0 + 4 * q));
      }
      return;
    }
#pragma unroll 4
    for (unsigned idx = threadIdx.x; idx < K * depth; idx += kThreads) {
      const unsigned r = idx / depth, d = idx % depth;
      StoreSplit(hi, lo, umma::CoreOffset(r, d, kSbo), src(K, r, d0 + d));
    }
  } else {
#pragma unroll 4
    for (unsigned idx = threadIdx.x; idx < K * depth; idx += kThreads) {
      const unsigned r = idx % K, d = idx / K;
      StoreSplit(hi, lo, umma::CoreOffset(r, d, kSbo), src(K, r, d0 + d));
    }
  }
}

// BF16 tier: the same operands as single BF16 values (round to nearest
// even), K-major core matrices of 8 rows x 8 values. Element (row, k) of a
// depth chunk sits at (row / 8) * kSbo16 + (k / 8) * 128 + (row % 8) * 16 +
// (k % 8) * 2 in the hi buffer of the operand; one kind::f16 MMA consumes a
// depth of 16 (two core matrices), so step k starts 256 bytes further.
constexpr std::uint32_t kSbo16 = kChunk / 8 * 128; // 1024 bytes between 8-row groups

__device__ __forceinline__ std::uint32_t CoreOffset16(unsigned row, unsigned k) {
  return (row / 8) * kSbo16 + (k / 8) * 128u + (row % 8) * 16u + (k % 8) * 2u;
}

__device__ __forceinline__ unsigned short Bf16Bits(float v) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

template <class Source>
__device__ __forceinline__ void StageBf16(const Source &src, unsigned K, unsigned d0,
                                          unsigned char *dst) {
  const unsigned depth = K > d0 ? (K - d0 < kChunk ? K - d0 : kChunk) : 0u;
  if (d0 != 0 && depth < kChunk) {
    // A later chunk: clear depths [depth, kChunk) left over from the first.
    const unsigned pad = kChunk - depth;
    for (unsigned idx = threadIdx.x; idx < K * pad; idx += kThreads)
      *reinterpret_cast<unsigned short *>(dst + CoreOffset16(idx / pad, depth + idx % pad)) = 0;
  }
  if constexpr (std::is_same_v<Source, RowMajor>) {
    if (K % 4 == 0) {
      const unsigned quads = depth / 4;
#pragma unroll 4
      for (unsigned idx = threadIdx.x; idx < K * quads; idx += kThreads) {
        const unsigned r = idx / quads, q = idx % quads;
        const float4 v = src.Quad(K, r, d0 + 4 * q);
        const uint2 packed = make_uint2(Bf16Bits(v.x) | (unsigned(Bf16Bits(v.y)) << 16),
                                        Bf16Bits(v.z) | (unsigned(Bf16Bits(v.w)) << 16));
        *reinterpret_cast<uint2 *>(dst + CoreOffset16(r, 4 * q)) = packed;
      }
      return;
    }
#pragma unroll 4
    for (unsigned idx = threadIdx.x; idx < K * depth; idx += kThreads) {
      const unsigned r = idx / depth, d = idx % depth;
      *reinterpret_cast<unsigned short *>(dst + CoreOffset16(r, d)) = Bf16Bits(src(K, r, d0 + d));
    }
  } else {
#pragma unroll 4
    for (unsigned idx = threadIdx.x; idx < K * depth; idx += kThreads) {
      const unsigned r = idx % K, d = idx / K;
      *reinterpret_cast<unsigned short *>(dst + CoreOffset16(r, d)) = Bf16Bits(src(K, r, d0 + d));
    }
  }
}

// Clears the four operand buffers (once per launch).
template <int KP> __device__ __forceinline__ void ClearOperands(unsigned char *smem) {
  float4 *p = reinterpret_cast<float4 *>(smem);
  for (unsigned i = threadIdx.x; i < Layout<KP>::kVectorsAt / 16; i += kThreads)
    p[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// Tensor-memory lanes 0..127 (one per thread), columns [column, column + KP):
//   D[r][n] = sum_{d < K} X(r, d) * Y(n, d)
// for r, n < K (other lanes and columns hold values nobody reads), in 3xTF32
// with FP32 accumulation. Returns false if a tensor-core wait timed out.
//
// With kSplit, the product is left in KP / kChunk + 1 accumulators of KP
// columns each instead of one: the hi*hi part of depth chunk c at column
// c * KP, and both small parts (lo*hi + hi*lo) of every chunk at column
// (KP / kChunk) * KP; SplitSum32 adds them in FP32. Each accumulator then
// takes at most 16 tensor-core steps instead of 48 at K = 128, and the
// tensor core's accumulation error grows with the steps accumulated into one
// accumulator (about 1.7e-6 relative on log Z at K = 128 with one).
//
// With `bf16` (the BF16 tier, a workspace-wide choice) each product is one
// pass of BF16 operands instead (kind::f16, FP32 accumulation, one
// accumulator whatever kSplit asks): about 8 significant bits per operand.
template <int KP, class XS, class YS, bool kSplit = false>
__device__ bool Product(unsigned char *smem, Shared &sh, std::uint32_t &phase,
                        std::uint32_t tmem, unsigned K, const XS &x, const YS &y,
                        bool bf16) {
  static_assert(KP % kChunk == 0 && KP <= 128, "padded state count");
  unsigned char *const xh = smem + Layout<KP>::kXh;
  unsigned char *const xl = smem + Layout<KP>::kXl;
  unsigned char *const yh = smem + Layout<KP>::kYh;
  unsigned char *const yl = smem + Layout<KP>::kYl;
  constexpr std::uint32_t kDescriptor = umma::Tf32Descriptor(128, KP);
  bool ok = true;
  if (bf16) {
    constexpr std::uint32_t kBf16 = umma::Bf16Descriptor(128, KP);
#pragma unroll 1
    for (unsigned chunk = 0; chunk < KP / kChunk; ++chunk) {
      StageBf16(x, K, chunk * kChunk, xh);
      StageBf16(y, K, chunk * kChunk, yh);
      umma::FenceOperands();
      umma::FenceBeforeSync();
      __syncthreads();
      umma::FenceAfterSync();
      if (threadIdx.x == 0) {
        const std::uint32_t xh_at = umma::SmemAddress(xh), yh_at = umma::SmemAddress(yh);
#pragma unroll
        for (unsigned k = 0; k < kChunk / 16; ++k)
          umma::MmaBf16(tmem, umma::SmemDescriptor(xh_at + k * 256, kSbo16),
                        umma::SmemDescriptor(yh_at + k * 256, kSbo16), kBf16,
                        chunk != 0 || k != 0);
        umma::Commit(&sh.barrier);
      }
      ok = umma::Wait(&sh.barrier, phase) && ok;
      phase ^= 1u;
      umma::FenceAfterSync();
    }
    return ok;
  }
#pragma unroll 1
  for (unsigned chunk = 0; chunk < KP / kChunk; ++chunk) {
    const unsigned d0 = chunk * kChunk;
    Stage(x, K, d0, xh, xl);
    Stage(y, K, d0, yh, yl);
    umma::FenceOperands();
    umma::FenceBeforeSync();
    __syncthreads();
    umma::FenceAfterSync();
    if (threadIdx.x == 0) {
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
          if constexpr (kSplit) {
            const bool big = part == 2;
            const std::uint32_t column = big ? chunk * KP : (KP / kChunk) * KP;
            const bool accumulate = big ? k != 0 : (chunk != 0 || part != 0 || k != 0);
            umma::MmaTf32(tmem + column, a, b, kDescriptor, accumulate);
          } else {
            umma::MmaTf32(tmem, a, b, kDescriptor, chunk != 0 || part != 0 || k != 0);
          }
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

// Columns [c, c + 32) of this thread's lane of a split product (Product with
// kSplit at `lane_base`): the hi*hi accumulators of the depth chunks in order,
// then the small-part accumulator, added in FP32.
template <int KP>
__device__ __forceinline__ void SplitSum32(std::uint32_t lane_base, unsigned c,
                                           float (&row)[32], bool bf16) {
  umma::Load32(lane_base + c, row);
  if (bf16)
    return; // the BF16 tier keeps one accumulator
#pragma unroll 1
  for (unsigned part = 1; part <= KP / kChunk; ++part) {
    float more[32];
    umma::Load32(lane_base + part * KP + c, more);
#pragma unroll
    for (unsigned q = 0; q < 32; ++q)
      row[q] += more[q];
  }
}

} // namespace wide
} // namespace thmm

#include "wide_engine_tree.cuh"

#endif // THMM_WIDE_ENGINE_CUH_
