// Phase kernels of the level-synchronous schedule (phase.h) for 32 < K <= 128
// states: round r of EVERY tree in one grid-wide launch per kind, as for
// K <= 4, but one operation per CTA (128 threads at K_P = 64, 256 at 128;
// rakes: warp-per-row K x K matrix-vector products; compressions and their
// adjoints: tcgen05 products with TMEM accumulators, as the per-tree
// tensor-core engine).
//
// The per-tree engine (wide_engine.cuh) contracts one tree per CTA, so a
// forest of 16 trees keeps 16 SMs busy and each SM runs one operation at a
// time. Here every operation of a round, over all trees, is spread across
// a persistent grid of several CTAs per SM, so staging, tensor-core work and
// epilogues of different operations overlap on an SM.
//
// Differences from the per-tree engine:
//   * power-of-two exponents travel with the stored values (one int32 per
//     stored node value and compressed path), as in the K <= 4 phase
//     schedule, instead of one running sum per tree;
//   * the adjoint of a compression reads the stored compressed path and its
//     own renormalisation exponent (comp_exp minus its inputs' exponents)
//     instead of recomputing the forward product, so a reverse compression
//     takes two tensor-core products instead of three;
//   * operand staging maps threads so that both the global loads (runs of
//     16-byte quads) and the shared-memory stores (eight rows of a core
//     matrix per 128-byte wavefront) are conflict-free, with a batch of
//     loads in flight per thread, and the next operation's matrices are
//     prefetched into L2 while the current one is worked on;
//   * at K_P = 64 the X operand's padded rows 64..127 are not stored: the
//     MMA tile has M = 128, and the lanes of rows >= 64 read whatever follows
//     the live rows (the lo part, the Y operand), results nobody reads, so
//     a CTA holds 64 KB of operands instead of 96 KB and three CTAs fit an SM.
// Every tensor-core wait is bounded; a wait that gives up sets
// kErrorTensorTimeout in the error word and the host reports an error.
#ifndef THMM_WIDE_PHASE_CUH_
#define THMM_WIDE_PHASE_CUH_

#include <cstdint>
#include <cuda_runtime.h>

#include "phase.h"
#include "wide_engine.cuh"

namespace thmm {
namespace wide {

// Shared-memory and TMEM layout of the tensor-core phase kinds for padded
// state count KP: operand parts of KP rows x a depth chunk of 64 (hi, lo of
// X, then of Y; BF16 uses the hi parts only), then the K-vectors.
template <int KP> struct PhaseLayout {
  // Threads per CTA: 128 at KP = 64 (three CTAs per SM), 256 at KP = 128
  // (one CTA per SM, so twice the warps for staging and epilogues; warps w
  // and w + 4 share TMEM lane quarter w and split the columns).
  static constexpr unsigned kThreads = KP == 64 ? 128u : 256u;
  static constexpr unsigned kPart = KP * kChunk * 4;
  static constexpr unsigned kXh = 0, kXl = kPart, kYh = 2 * kPart, kYl = 3 * kPart;
  static constexpr unsigned kVectorsAt = 4 * kPart;
  static constexpr unsigned kUsedBytes = kVectorsAt + kVectors * 128 * 4;
  // Forward: split accumulators (KP / 64 hi*hi parts + the small parts);
  // reverse: two products side by side.
  static constexpr std::uint32_t kColumns = KP == 64 ? 128 : 512;
  static_assert((KP / kChunk + 1) * KP <= kColumns && 2 * KP <= kColumns, "TMEM columns");
  static constexpr int kCtasPerSm = static_cast<int>(512 / kColumns);
  // At most kCtasPerSm CTAs fit in the SM's 228 KB (1 KB reserved per CTA),
  // so no CTA waits on a TMEM allocation.
  static constexpr unsigned kFloorBytes = 228 * 1024 / (kCtasPerSm + 1);
  static constexpr unsigned kSmemBytes = kUsedBytes > kFloorBytes ? kUsedBytes : kFloorBytes;
  static_assert(kSmemBytes <= 227 * 1024, "shared memory per CTA");
  // CTAs per SM the grid is sized for: what the shared memory (with 1 KB of
  // static and 1 KB of reserved shared memory per CTA) and TMEM allow. The
  // occupancy query reports one CTA per SM for kernels that use tcgen05,
  // whatever their resources, so it is not consulted.
  static constexpr unsigned kSmemResident = 228 * 1024 / (kSmemBytes + 2048);
  static constexpr int kResident =
      static_cast<int>(kSmemResident) < kCtasPerSm ? static_cast<int>(kSmemResident) : kCtasPerSm;
};

// Dynamic shared memory of the kinds without tensor-core work: the vectors.
constexpr unsigned kVectorBytes = kVectors * 128 * 4;

struct PhaseShared {
  std::uint64_t barrier; // tensor-core completion
  double root_sum;
  std::uint32_t tmem;
  int root_finite;
  float reduce[8]; // one per warp (at most 256 threads)
};

template <unsigned T> __device__ __forceinline__ float CtaMax(float v, PhaseShared &sh) {
  static_assert(T % 32 == 0 && T / 32 <= sizeof(PhaseShared::reduce) / sizeof(float),
                "one reduction slot per warp");
  v = WarpMax(v);
  if ((threadIdx.x & 31) == 0)
    sh.reduce[threadIdx.x / 32] = v;
  __syncthreads();
  float m = sh.reduce[0];
#pragma unroll
  for (unsigned w = 1; w < T / 32; ++w)
    m = m < sh.reduce[w] ? sh.reduce[w] : m;
  __syncthreads();
  return m;
}

__device__ __forceinline__ int ExponentOf(float m) { return m > 0.0f ? Pow2Exponent(m) : 0; }

// ------------------------------------------------------------ operand sources
// A product operand element (r, d): row r of the operand, depth d. Row
// sources read element (r, d) at p[r * K + d] (four consecutive depths per
// 16-byte Quad); column sources at p[d * K + r].
struct Rows {
  static constexpr bool kColumns = false;
  const float *p;
  const float *scale; // shared-memory depth scale, or null
  __device__ __forceinline__ float At(unsigned K, unsigned r, unsigned d) const {
    const float v = p[static_cast<std::size_t>(r) * K + d];
    return scale != nullptr ? v * scale[d] : v;
  }
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
struct Columns {
  static constexpr bool kColumns = true;
  const float *p;
  __device__ __forceinline__ float At(unsigned K, unsigned r, unsigned d) const {
    return p[static_cast<std::size_t>(d) * K + r];
  }
};

// The adjoint ratio of a compression, formed while staging: entry (r, c)
// is mu[r][c] / product[r][c] with product = stored path * 2^shift (zero
// where the product is zero). The division is the fast reciprocal form
// (stored entries are at most 1, well inside its range; about 2 ulp), and
// 2^-shift is one exact factor when it is a normal float.
struct Ratio {
  int shift;
  float factor;
  bool exact;
  __device__ __forceinline__ explicit Ratio(int s)
      : shift(s), factor(s >= -127 && s <= 126 ? ScalePow2(1.0f, -s) : 0.0f),
        exact(s >= -127 && s <= 126) {}
  __device__ __forceinline__ float operator()(float mu, float stored) const {
    if (!(stored > 0.0f))
      return 0.0f;
    const float q = __fdividef(mu, stored);
    return exact ? q * factor : ScalePow2(q, -shift);
  }
};
struct RatioRows {
  static constexpr bool kColumns = false;
  const float *mu;
  const float *stored;
  Ratio ratio;
  __device__ __forceinline__ float At(unsigned K, unsigned r, unsigned d) const {
    const std::size_t at = static_cast<std::size_t>(r) * K + d;
    return ratio(mu[at], stored[at]);
  }
  __device__ __forceinline__ float4 Quad(unsigned K, unsigned r, unsigned d) const {
    const std::size_t at = static_cast<std::size_t>(r) * K + d;
    const float4 m = *reinterpret_cast<const float4 *>(mu + at);
    const float4 s = *reinterpret_cast<const float4 *>(stored + at);
    return make_float4(ratio(m.x, s.x), ratio(m.y, s.y), ratio(m.z, s.z), ratio(m.w, s.w));
  }
};
struct RatioColumns {
  static constexpr bool kColumns = true;
  const float *mu;
  const float *stored;
  Ratio ratio;
  __device__ __forceinline__ float At(unsigned K, unsigned r, unsigned d) const {
    const std::size_t at = static_cast<std::size_t>(d) * K + r;
    return ratio(mu[at], stored[at]);
  }
};

// ------------------------------------------------------------------ staging
// An operand chunk is written as rows r < K, depths [d0, d0 + depth) (depth
// = the chunk's part of [0, K)) in TF32 hi/lo parts (bf16: as BF16 in `hi`);
// padded depths of the chunk are zero (cleared once per launch, and again
// for a later, shorter chunk), padded rows are never read.
//
// K % 4 == 0: each thread moves quads (4 consecutive depths of one row) in
// passes of kBatch: all loads of a pass for both operands are issued before
// any store, so a thread has up to 2 kBatch global loads in flight.
//   * Row sources: a warp takes 8 rows x 4 quads, so its global loads are
//     64-byte runs of 8 rows and its 16-byte shared-memory stores fill whole
//     128-byte core-matrix rows (4 wavefronts for 512 bytes);
//   * column sources: a warp takes 32 consecutive rows of one quad of
//     depths, four coalesced 128-byte loads and one 16-byte store per thread.
constexpr unsigned kBatch = 4;

// This thread's walk over the quad slots of an operand chunk: slot
// threadIdx.x, then every T-th. The row and quad of each slot are
// advanced incrementally (one division when the walk starts, none per slot).
//   * Row sources: slot idx is lane t = idx % 32 of group g = idx / 32, row
//     (g / quad_groups) * 8 + t % 8, quad (g % quad_groups) * 4 + t / 8;
//   * column sources: row idx % K, quad idx / K.
template <class Src, unsigned T> struct QuadCursor {
  unsigned K, quads, quad_groups;
  unsigned major, minor; // rows: g / quad_groups, g % quad_groups; columns: q, r
  unsigned step_major, step_minor;
  unsigned lane_row, lane_quad;
  __device__ __forceinline__ QuadCursor(unsigned states, unsigned depth)
      : K(states), quads(depth / 4), quad_groups((depth / 4 + 3) / 4) {
    if constexpr (Src::kColumns) {
      major = threadIdx.x / K;
      minor = threadIdx.x % K;
      step_major = T / K;
      step_minor = T % K;
      lane_row = lane_quad = 0;
    } else {
      const unsigned g = threadIdx.x >> 5, t = threadIdx.x & 31u;
      major = g / quad_groups;
      minor = g % quad_groups;
      step_major = (T / 32) / quad_groups;
      step_minor = (T / 32) % quad_groups;
      lane_row = t & 7u;
      lane_quad = t >> 3;
    }
  }
  __device__ __forceinline__ unsigned Row() const {
    return Src::kColumns ? minor : major * 8 + lane_row;
  }
  __device__ __forceinline__ unsigned Quad() const {
    return Src::kColumns ? major : minor * 4 + lane_quad;
  }
  // Slots remain (this one may still be padding).
  __device__ __forceinline__ bool More() const {
    return Src::kColumns ? major < quads : major * 8 < K;
  }
  __device__ __forceinline__ bool Valid() const { return More() && Row() < K && Quad() < quads; }
  __device__ __forceinline__ void Advance() {
    const unsigned limit = Src::kColumns ? K : quad_groups;
    major += step_major;
    minor += step_minor;
    if (minor >= limit) {
      minor -= limit;
      ++major;
    }
  }
};

template <class Src>
__device__ __forceinline__ float4 LoadQuad(const Src &src, unsigned K, unsigned r, unsigned d) {
  if constexpr (Src::kColumns)
    return make_float4(src.At(K, r, d), src.At(K, r, d + 1), src.At(K, r, d + 2),
                       src.At(K, r, d + 3));
  else
    return src.Quad(K, r, d);
}

template <bool kBf16>
__device__ __forceinline__ void Put(unsigned char *hi, unsigned char *lo, unsigned r,
                                   unsigned d, float v) {
  if constexpr (kBf16)
    *reinterpret_cast<unsigned short *>(hi + CoreOffset16(r, d)) = Bf16Bits(v);
  else
    StoreSplit(hi, lo, umma::CoreOffset(r, d, kSbo), v);
}

template <bool kBf16>
__device__ __forceinline__ void Put4(unsigned char *hi, unsigned char *lo, unsigned r,
                                     unsigned d, float4 v) {
  if constexpr (kBf16)
    *reinterpret_cast<uint2 *>(hi + CoreOffset16(r, d)) =
        make_uint2(Bf16Bits(v.x) | (unsigned(Bf16Bits(v.y)) << 16),
                   Bf16Bits(v.z) | (unsigned(Bf16Bits(v.w)) << 16));
  else
    StoreSplit(hi, lo, umma::CoreOffset(r, d, kSbo), v);
}

// Clears depths [depth, kChunk) of rows < K (a later, shorter chunk).
template <bool kBf16, unsigned T>
__device__ __forceinline__ void ClearTail(unsigned K, unsigned depth, unsigned char *hi,
                                          unsigned char *lo) {
  const unsigned pad = kChunk - depth;
  for (unsigned idx = threadIdx.x; idx < K * pad; idx += T)
    Put<kBf16>(hi, lo, idx / pad, depth + idx % pad, 0.0f);
}

// Any K: one element per slot (used when K % 4 != 0).
template <bool kBf16, unsigned T, class Src>
__device__ __forceinline__ void StageScalar(const Src &src, unsigned K, unsigned d0,
                                            unsigned depth, unsigned char *hi,
                                            unsigned char *lo) {
#pragma unroll 4
  for (unsigned idx = threadIdx.x; idx < K * depth; idx += T) {
    const unsigned r = Src::kColumns ? idx % K : idx / depth;
    const unsigned d = Src::kColumns ? idx / K : idx % depth;
    Put<kBf16>(hi, lo, r, d, src.At(K, r, d0 + d));
  }
}

// Stages depth chunk d0 of both operands of a product.
template <bool kBf16, unsigned T, class XS, class YS>
__device__ __forceinline__ void StageChunk(const XS &x, const YS &y, unsigned K, unsigned d0,
                                           unsigned char *xh, unsigned char *xl,
                                           unsigned char *yh, unsigned char *yl) {
  const unsigned depth = K - d0 < kChunk ? K - d0 : kChunk;
  if (d0 != 0 && depth < kChunk) {
    ClearTail<kBf16, T>(K, depth, xh, xl);
    ClearTail<kBf16, T>(K, depth, yh, yl);
  }
  if (K % 4 != 0) {
    StageScalar<kBf16, T>(x, K, d0, depth, xh, xl);
    StageScalar<kBf16, T>(y, K, d0, depth, yh, yl);
    return;
  }
  QuadCursor<XS, T> xs(K, depth);
  QuadCursor<YS, T> ys(K, depth);
#pragma unroll 1
  while (xs.More() || ys.More()) {
    float4 xv[kBatch], yv[kBatch];
    unsigned xr[kBatch], xq[kBatch], yr[kBatch], yq[kBatch];
    bool xok[kBatch], yok[kBatch];
#pragma unroll
    for (unsigned b = 0; b < kBatch; ++b) {
      xok[b] = xs.Valid();
      xr[b] = xs.Row();
      xq[b] = xs.Quad();
      xs.Advance();
      yok[b] = ys.Valid();
      yr[b] = ys.Row();
      yq[b] = ys.Quad();
      ys.Advance();
      if (xok[b])
        xv[b] = LoadQuad(x, K, xr[b], d0 + 4 * xq[b]);
      if (yok[b])
        yv[b] = LoadQuad(y, K, yr[b], d0 + 4 * yq[b]);
    }
#pragma unroll
    for (unsigned b = 0; b < kBatch; ++b) {
      if (xok[b])
        Put4<kBf16>(xh, xl, xr[b], 4 * xq[b], xv[b]);
      if (yok[b])
        Put4<kBf16>(yh, yl, yr[b], 4 * yq[b], yv[b]);
    }
  }
}

// Issues the tensor-core steps of depth chunk `chunk` of a product whose
// operands are staged (hi/lo, or BF16 in the hi parts) and waits for them
// (bounded). Returns false if the wait timed out.
template <int KP, bool kSplit>
__device__ bool MmaChunk(unsigned char *smem, PhaseShared &sh, std::uint32_t &phase,
                         std::uint32_t tmem, unsigned chunk, bool bf16) {
  using L = PhaseLayout<KP>;
  umma::FenceOperands();
  umma::FenceBeforeSync();
  __syncthreads();
  umma::FenceAfterSync();
  if (threadIdx.x == 0) {
    const std::uint32_t xh_at = umma::SmemAddress(smem + L::kXh);
    const std::uint32_t xl_at = umma::SmemAddress(smem + L::kXl);
    const std::uint32_t yh_at = umma::SmemAddress(smem + L::kYh);
    const std::uint32_t yl_at = umma::SmemAddress(smem + L::kYl);
    if (bf16) {
      constexpr std::uint32_t kBf16 = umma::Bf16Descriptor(128, KP);
#pragma unroll
      for (unsigned k = 0; k < kChunk / 16; ++k)
        umma::MmaBf16(tmem, umma::SmemDescriptor(xh_at + k * 256, kSbo16),
                      umma::SmemDescriptor(yh_at + k * 256, kSbo16), kBf16,
                      chunk != 0 || k != 0);
    } else {
      constexpr std::uint32_t kTf32 = umma::Tf32Descriptor(128, KP);
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
            umma::MmaTf32(tmem + column, a, b, kTf32, accumulate);
          } else {
            umma::MmaTf32(tmem, a, b, kTf32, chunk != 0 || part != 0 || k != 0);
          }
        }
      }
    }
    umma::Commit(&sh.barrier);
  }
  const bool ok = umma::Wait(&sh.barrier, phase);
  phase ^= 1u;
  umma::FenceAfterSync();
  return ok;
}

// Tensor-memory lanes 0..127 (one per thread), columns from `tmem`:
//   D[r][n] = sum_{d < K} X(r, d) * Y(n, d)   for r, n < K
// in 3xTF32 (split accumulators with kSplit, see Product) or, with bf16,
// one BF16 pass. Returns false if a tensor-core wait timed out.
template <int KP, bool kSplit, class XS, class YS>
__device__ bool PhaseProduct(unsigned char *smem, PhaseShared &sh, std::uint32_t &phase,
                             std::uint32_t tmem, unsigned K, const XS &x, const YS &y,
                             bool bf16) {
  using L = PhaseLayout<KP>;
  unsigned char *const xh = smem + L::kXh;
  unsigned char *const xl = smem + L::kXl;
  unsigned char *const yh = smem + L::kYh;
  unsigned char *const yl = smem + L::kYl;
  bool ok = true;
  // KP is the padded state count, so K > KP - 64 and every chunk holds
  // depths of [0, K): each split accumulator is written.
#pragma unroll 1
  for (unsigned chunk = 0; chunk < KP / kChunk; ++chunk) {
    const unsigned d0 = chunk * kChunk;
    constexpr unsigned T = L::kThreads;
    if (bf16)
      StageChunk<true, T>(x, y, K, d0, xh, nullptr, yh, nullptr);
    else
      StageChunk<false, T>(x, y, K, d0, xh, xl, yh, yl);
    ok = MmaChunk<KP, kSplit>(smem, sh, phase, tmem, chunk, bf16) && ok;
  }
  return ok;
}

// Stages depth chunk d0 of one operand (K % 4 == 0), loads batched as in
// StageChunk.
template <bool kBf16, unsigned T, class Src>
__device__ __forceinline__ void StageOne(const Src &src, unsigned K, unsigned d0,
                                         unsigned char *hi, unsigned char *lo) {
  const unsigned depth = K - d0 < kChunk ? K - d0 : kChunk;
  QuadCursor<Src, T> cursor(K, depth);
#pragma unroll 1
  while (cursor.More()) {
    float4 v[kBatch];
    unsigned rows[kBatch], quads[kBatch];
    bool ok[kBatch];
#pragma unroll
    for (unsigned b = 0; b < kBatch; ++b) {
      ok[b] = cursor.Valid();
      rows[b] = cursor.Row();
      quads[b] = cursor.Quad();
      cursor.Advance();
      if (ok[b])
        v[b] = LoadQuad(src, K, rows[b], d0 + 4 * quads[b]);
    }
#pragma unroll
    for (unsigned b = 0; b < kBatch; ++b)
      if (ok[b])
        Put4<kBf16>(hi, lo, rows[b], 4 * quads[b], v[b]);
  }
}

// Y(n, d) = X(d, n) for n, d < K (KP = 64: one depth chunk holds the whole
// staged operand): copies the staged hi and lo parts (BF16: hi) element by
// element, so the transpose holds exactly the values staged in X. A warp
// moves an 8 x 4 block of X per step: its reads cover one core matrix row
// set (32 distinct banks), its writes two.
template <bool kBf16, unsigned T>
__device__ __forceinline__ void TransposeStaged(unsigned K, const unsigned char *xh,
                                                const unsigned char *xl, unsigned char *yh,
                                                unsigned char *yl) {
  const unsigned warp = threadIdx.x / 32, lane = threadIdx.x & 31u;
  const unsigned row_blocks = (K + 7) / 8, col_blocks = (K + 3) / 4;
  for (unsigned block = warp; block < row_blocks * col_blocks; block += T / 32) {
    const unsigned d = (block / col_blocks) * 8 + lane / 4;
    const unsigned n = (block % col_blocks) * 4 + lane % 4;
    if (d < K && n < K) {
      if constexpr (kBf16) {
        *reinterpret_cast<unsigned short *>(yh + CoreOffset16(n, d)) =
            *reinterpret_cast<const unsigned short *>(xh + CoreOffset16(d, n));
      } else {
        const std::uint32_t from = umma::CoreOffset(d, n, kSbo);
        const std::uint32_t to = umma::CoreOffset(n, d, kSbo);
        *reinterpret_cast<float *>(yh + to) = *reinterpret_cast<const float *>(xh + from);
        *reinterpret_cast<float *>(yl + to) = *reinterpret_cast<const float *>(xl + from);
      }
    }
  }
}

// One operation of a wide phase kind, executed by the whole CTA.
template <int KP> struct WideOps {
  // Threads of the CTA; a thread's TMEM lane (accumulator row) is
  // threadIdx.x % 128, and with 256 threads the two halves of the CTA take
  // the two halves of the columns.
  static constexpr unsigned kThreads = PhaseLayout<KP>::kThreads;
  static constexpr unsigned kHalves = kThreads / 128;
  static constexpr unsigned kHalfColumns = KP / kHalves;
  const PhaseArgs &a;
  PhaseShared &sh;
  unsigned char *smem;
  std::uint32_t tmem;
  std::uint32_t &phase;
  bool &ok;
  unsigned K, KK;
  float *v, *leaf, *msg, *middle, *ratio;

  __device__ WideOps(const PhaseArgs &args, PhaseShared &shared, unsigned char *dynamic_smem,
                     float *vectors, std::uint32_t tmem_base, std::uint32_t &mma_phase,
                     bool &status)
      : a(args), sh(shared), smem(dynamic_smem), tmem(tmem_base), phase(mma_phase), ok(status),
        K(args.states), KK(args.states * args.states) {
    v = vectors;
    leaf = vectors + 128;
    msg = vectors + 256;
    middle = vectors + 384;
    ratio = vectors + 512;
  }

  __device__ __forceinline__ float *Nodes() const { return static_cast<float *>(a.nodes); }
  __device__ __forceinline__ float *Comps() const { return static_cast<float *>(a.comps); }
  __device__ __forceinline__ float *CompMu() const { return static_cast<float *>(a.comp_mu); }
  __device__ __forceinline__ float *NodeOut() const { return static_cast<float *>(a.node_out); }

  __device__ __forceinline__ const float *PathPtr(std::uint32_t ref) const {
    if (ref & kFlag)
      return Comps() + static_cast<std::size_t>(ref & kMask) * KK;
    const std::size_t edge = a.edge_modulus != 0 ? ref % a.edge_modulus : ref;
    return static_cast<const float *>(a.edge_in) + edge * KK;
  }
  __device__ __forceinline__ int PathExp(std::uint32_t ref) const {
    return (ref & kFlag) ? a.comp_exp[ref & kMask] : 0;
  }
  __device__ __forceinline__ float *AdjointOf(std::uint32_t ref) const {
    return (ref & kFlag) ? CompMu() + static_cast<std::size_t>(ref & kMask) * KK
                         : static_cast<float *>(a.edge_out) + static_cast<std::size_t>(ref) * KK;
  }

  // Input factor of `node` for state j < K: dense row, or the reference's
  // categorical (root ? root_potential : 1) * emission[observation]
  // (src/gpu_backend_impl.inc:326-382).
  __device__ __forceinline__ float Input(std::uint32_t node, std::uint32_t obs, bool root,
                                         unsigned j) const {
    if (!a.categorical)
      return static_cast<const float *>(a.node_in)[static_cast<std::size_t>(node) * K + j];
    const float *root_potential = static_cast<const float *>(a.root_potential);
    float value = root ? root_potential[j] : 1.0f;
    if (obs != kNone) {
      const unsigned category = a.observations[obs];
      value = category < a.categories
                  ? value * static_cast<const float *>(a.emission)[category * K + j]
                  : 0.0f;
    }
    return value;
  }

  // dst[j] (j < K) = the value of a rake leaf or compression middle: the
  // stored value or the input factor. Returns the stored value's exponent.
  __device__ __forceinline__ int NodeInto(std::uint32_t ref, std::uint32_t obs,
                                          float *dst) const {
    const unsigned j = threadIdx.x;
    if (ref & kFlag) {
      const std::uint32_t node = ref & kMask;
      if (j < K)
        dst[j] = Nodes()[static_cast<std::size_t>(node) * K + j];
      return a.node_exp[node];
    }
    if (j < K)
      dst[j] = Input(ref, obs, false, j);
    return 0;
  }

  // Row stride (floats) of a K x K tile staged in the operand buffers: K + 4,
  // so that the 16-byte row writes of eight consecutive rows (one per
  // thread) and the row reads of the coalesced passes are conflict-free.
  __device__ __forceinline__ unsigned TileStride() const { return K + 4; }
  // Writes columns [c, c + 32) ∩ [0, K) of row j of a tile (K % 4 == 0).
  __device__ __forceinline__ void TileRow(float *tile, unsigned j, unsigned c,
                                          const float (&row)[32]) const {
#pragma unroll
    for (unsigned q = 0; q < 32; q += 4)
      if (c + q < K)
        *reinterpret_cast<float4 *>(tile + j * TileStride() + c + q) =
            make_float4(row[q], row[q + 1], row[q + 2], row[q + 3]);
  }

  // This thread's walk over the quads of a row-major K x K matrix (K % 4 ==
  // 0): quad threadIdx.x, then every kThreads-th, as (row, first column).
  struct TileWalk {
    unsigned quads, row, column, step_rows, step_quads;
    __device__ __forceinline__ explicit TileWalk(unsigned K)
        : quads(K / 4), row(threadIdx.x / (K / 4)), column(4 * (threadIdx.x % (K / 4))),
          step_rows(kThreads / (K / 4)), step_quads(kThreads % (K / 4)) {}
    __device__ __forceinline__ void Advance() {
      row += step_rows;
      column += 4 * step_quads;
      if (column >= 4 * quads) {
        column -= 4 * quads;
        ++row;
      }
    }
  };

  // Rows per warp whose loads are in flight together (MatVec, RakeReverse).
  static constexpr unsigned kRows = KP == 64 ? 8 : 4;

  // out[i] = sum_j path[i][j] * x[j] for i < K: warp w takes rows w, w + 4,
  // ...; lanes stride the columns (coalesced), shuffle reductions.
  __device__ __forceinline__ void MatVec(const float *path, const float *x, float *out) const {
    const unsigned warp = threadIdx.x / 32, lane = threadIdx.x & 31;
#pragma unroll 1
    for (unsigned i0 = warp; i0 < K; i0 += kRows * (kThreads / 32)) {
      float p[kRows][KP / 32];
#pragma unroll
      for (unsigned t = 0; t < kRows; ++t) {
        const unsigned i = i0 + t * (kThreads / 32);
#pragma unroll
        for (unsigned q = 0; q < KP / 32; ++q) {
          const unsigned j = lane + 32 * q;
          p[t][q] = i < K && j < K ? path[static_cast<std::size_t>(i) * K + j] : 0.0f;
        }
      }
#pragma unroll
      for (unsigned t = 0; t < kRows; ++t) {
        const unsigned i = i0 + t * (kThreads / 32);
        float s = 0.0f;
#pragma unroll
        for (unsigned q = 0; q < KP / 32; ++q) {
          const unsigned j = lane + 32 * q;
          if (j < K)
            s = fmaf(p[t][q], x[j], s);
        }
        s = WarpSum(s);
        if (lane == 0 && i < K)
          out[i] = s;
      }
    }
  }

  // Starts moving the matrices of operation i (of this launch's kind) into
  // L2 while the CTA works on the current one (thread 0; K % 4 == 0 so the
  // matrices are 16-byte aligned and sized).
  template <int kKind> __device__ __forceinline__ void Prefetch(std::uint32_t i) const {
    if (K % 4 != 0)
      return;
    const std::uint32_t bytes = KK * 4u;
    if constexpr (kKind == kPhaseCompress || kKind == kPhaseCompressReverse) {
      const uint4 op = a.compress[i];
      umma::PrefetchL2(PathPtr(op.x), bytes);
      umma::PrefetchL2(PathPtr(op.z), bytes);
      if constexpr (kKind == kPhaseCompressReverse) {
        umma::PrefetchL2(CompMu() + static_cast<std::size_t>(i) * KK, bytes);
        umma::PrefetchL2(Comps() + static_cast<std::size_t>(i) * KK, bytes);
      }
    } else if constexpr (kKind == kPhaseRakeReverse) {
      umma::PrefetchL2(PathPtr(a.rakes[i].x), bytes);
    } else if constexpr (kKind == kPhaseGather) {
      const uint4 op = a.gathers[i];
      if ((op.w & kCountMask) != 0)
        umma::PrefetchL2(PathPtr(a.rakes[op.z].x), bytes);
    }
  }

  // ------------------------------------------------------------ forward
  // Absorbs the rakes of one gather into its parent (src/inference.cc:
  // 697-836 with exact power-of-two scaling, as LinearEngine's gather).
  __device__ void Gather(std::uint32_t i) {
    const uint4 op = a.gathers[i];
    const std::uint32_t node = op.x & kMask;
    const unsigned j = threadIdx.x;
    int e = 0;
    if (op.x & kFlag) {
      if (j < K)
        v[j] = Input(node, op.y, (op.w & kRootBit) != 0, j);
    } else {
      if (j < K)
        v[j] = Nodes()[static_cast<std::size_t>(node) * K + j];
      e = a.node_exp[node];
    }
    const std::uint32_t count = op.w & kCountMask;
    for (std::uint32_t k = 0; k < count; ++k) {
      const uint4 rake = a.rakes[op.z + k];
      e += NodeInto(rake.y, rake.z, leaf) + PathExp(rake.x);
      __syncthreads();
      MatVec(PathPtr(rake.x), leaf, msg);
      __syncthreads();
      const float message = j < K ? msg[j] : 0.0f;
      int s = ExponentOf(CtaMax<kThreads>(message, sh));
      e += s;
      const float value = j < K ? v[j] * ScalePow2(message, -s) : 0.0f;
      s = ExponentOf(CtaMax<kThreads>(value, sh));
      e += s;
      if (j < K)
        v[j] = ScalePow2(value, -s);
    }
    if (j < K)
      Nodes()[static_cast<std::size_t>(node) * K + j] = v[j];
    if (j == 0)
      a.node_exp[node] = e;
    __syncthreads();
  }

  // Compressed path i = left * diag(middle) * right, renormalised by the
  // power of two of its largest entry.
  __device__ void Compress(std::uint32_t i) {
    const uint4 op = a.compress[i];
    const int e = PathExp(op.x) + PathExp(op.z) + NodeInto(op.y, op.w, middle);
    __syncthreads();
    ok = PhaseProduct<KP, true>(smem, sh, phase, tmem, K, Rows{PathPtr(op.x), middle},
                                Columns{PathPtr(op.z)}, a.bf16 != 0) &&
         ok;
    // Accumulator row `row` (TMEM lane), columns [c0, c0 + kHalfColumns).
    const unsigned row = threadIdx.x % 128, c0 = (threadIdx.x / 128) * kHalfColumns;
    const std::uint32_t lane_base = tmem + ((row & ~31u) << 16);
    float m = 0.0f;
#pragma unroll 1
    for (unsigned c = c0; c < c0 + kHalfColumns; c += 32) {
      float values[32];
      SplitSum32<KP>(lane_base, c, values, a.bf16 != 0);
#pragma unroll
      for (unsigned q = 0; q < 32; ++q)
        if (row < K && c + q < K)
          m = m < values[q] ? values[q] : m;
    }
    const int s = ExponentOf(CtaMax<kThreads>(m, sh));
    float *out = Comps() + static_cast<std::size_t>(i) * KK;
    if (K % 4 == 0) {
      // Rows through the (now idle) operand buffers, then coalesced stores.
      float *tile = reinterpret_cast<float *>(smem);
#pragma unroll 1
      for (unsigned c = c0; c < c0 + kHalfColumns; c += 32) {
        float values[32];
        SplitSum32<KP>(lane_base, c, values, a.bf16 != 0);
        if (row < K) {
#pragma unroll
          for (unsigned q = 0; q < 32; ++q)
            values[q] = ScalePow2(values[q], -s);
          TileRow(tile, row, c, values);
        }
      }
      __syncthreads();
#pragma unroll 4
      for (TileWalk w(K); w.row < K; w.Advance())
        *reinterpret_cast<float4 *>(out + static_cast<std::size_t>(w.row) * K + w.column) =
            *reinterpret_cast<const float4 *>(tile + w.row * TileStride() + w.column);
    } else {
#pragma unroll 1
      for (unsigned c = c0; c < c0 + kHalfColumns; c += 32) {
        float values[32];
        SplitSum32<KP>(lane_base, c, values, a.bf16 != 0);
        if (row < K) {
#pragma unroll
          for (unsigned q = 0; q < 32; ++q)
            if (c + q < K)
              out[static_cast<std::size_t>(row) * K + c + q] = ScalePow2(values[q], -s);
        }
      }
    }
    if (threadIdx.x == 0)
      a.comp_exp[i] = e + s;
    umma::FenceBeforeSync();
    __syncthreads();
  }

  // log Z = ln 2 * (root exponent) + log(sum(root)) in FP64, and the root
  // marginal when the adjoint follows (as LinearEngine::Run).
  __device__ void Finish(std::uint32_t i) {
    const uint2 rec = a.roots[i];
    const std::uint32_t node = rec.x & kMask;
    const unsigned j = threadIdx.x;
    long long total = 0;
    if (rec.x & kFlag) {
      if (j < K)
        v[j] = Nodes()[static_cast<std::size_t>(node) * K + j];
      total = a.node_exp[node];
    } else if (j < K) {
      v[j] = Input(node, rec.y, true, j);
    }
    __syncthreads();
    if (j == 0) {
      double sum = 0.0;
      for (unsigned q = 0; q < K; ++q)
        sum += static_cast<double>(v[q]);
      const double log_z = !(sum > 0.0)
                               ? -INFINITY
                               : static_cast<double>(total) * 0.6931471805599453094 + log(sum);
      static_cast<float *>(a.values)[i] = static_cast<float>(a.raw ? exp(log_z) : log_z);
      sh.root_sum = sum;
      sh.root_finite = log_z > -INFINITY;
    }
    __syncthreads();
    if (a.reverse && j < K)
      NodeOut()[static_cast<std::size_t>(node) * K + j] =
          sh.root_finite ? static_cast<float>(static_cast<double>(v[j]) / sh.root_sum) : 0.0f;
    __syncthreads();
  }

  // ------------------------------------------------------------ adjoint
  // Adjoint of one rake: the path's entries ratio[r] * path[r][c] *
  // leaf[c] with ratio = parent marginal / message, and the leaf's marginal
  // leaf[c] * sum_r ratio[r] * path[r][c].
  __device__ void RakeReverse(std::uint32_t i) {
    const uint4 op = a.rakes[i];
    const unsigned j = threadIdx.x;
    const unsigned warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    NodeInto(op.y, op.z, leaf);
    if (j < K)
      v[j] = NodeOut()[static_cast<std::size_t>(op.w) * K + j];
    __syncthreads();
    const float *path = PathPtr(op.x);
    MatVec(path, leaf, msg);
    __syncthreads();
    if (j < K)
      ratio[j] = msg[j] > 0.0f ? v[j] / msg[j] : 0.0f;
    __syncthreads();
    float *out = AdjointOf(op.x);
    float column[KP / 32];
#pragma unroll
    for (unsigned q = 0; q < KP / 32; ++q)
      column[q] = 0.0f;
#pragma unroll 1
    for (unsigned r0 = warp; r0 < K; r0 += kRows * (kThreads / 32)) {
      float p[kRows][KP / 32];
#pragma unroll
      for (unsigned t = 0; t < kRows; ++t) {
        const unsigned r = r0 + t * (kThreads / 32);
#pragma unroll
        for (unsigned q = 0; q < KP / 32; ++q) {
          const unsigned c = lane + 32 * q;
          p[t][q] = r < K && c < K ? path[static_cast<std::size_t>(r) * K + c] : 0.0f;
        }
      }
#pragma unroll
      for (unsigned t = 0; t < kRows; ++t) {
        const unsigned r = r0 + t * (kThreads / 32);
        if (r < K) {
          const float ratio_r = ratio[r];
#pragma unroll
          for (unsigned q = 0; q < KP / 32; ++q) {
            const unsigned c = lane + 32 * q;
            if (c < K) {
              out[static_cast<std::size_t>(r) * K + c] = ratio_r * p[t][q] * leaf[c];
              column[q] = fmaf(ratio_r, p[t][q], column[q]);
            }
          }
        }
      }
    }
    // Reduce the four warps' column sums through the message vector.
#pragma unroll 1
    for (unsigned w = 0; w < kThreads / 32; ++w) {
      if (warp == w) {
#pragma unroll
        for (unsigned q = 0; q < KP / 32; ++q) {
          const unsigned c = lane + 32 * q;
          if (c < K)
            msg[c] = (w == 0 ? 0.0f : msg[c]) + column[q];
        }
      }
      __syncthreads();
    }
    if (j < K)
      NodeOut()[static_cast<std::size_t>(op.y & kMask) * K + j] = leaf[j] * msg[j];
    __syncthreads();
  }

  // Adjoint of compression i with ratio R = mu / (left diag(middle) right)
  // (mu: the compressed path's adjoint): left adjoint left[r][m] middle[m]
  // (R right^T)[r][m], right adjoint right[m][c] middle[m] (left^T R)[m][c],
  // middle adjoint the row sums of the latter.
  __device__ void CompressReverse(std::uint32_t i) {
    const uint4 op = a.compress[i];
    const unsigned j = threadIdx.x;
    const int inputs = PathExp(op.x) + PathExp(op.z) + NodeInto(op.y, op.w, middle);
    const int shift = a.comp_exp[i] - inputs; // the compression's renormalisation
    __syncthreads();
    const float *left = PathPtr(op.x);
    const float *right = PathPtr(op.z);
    const float *mu = CompMu() + static_cast<std::size_t>(i) * KK;
    const float *stored = Comps() + static_cast<std::size_t>(i) * KK;
    // P1[r][m] = sum_c R[r][c] right[m][c];  P2[m][c] = sum_r left[r][m] R[r][c].
    const Ratio ratio_of(shift);
    if (KP == 64 && K % 4 == 0) {
      // P1 stages R as its X operand; P2's Y operand is that staged R,
      // transposed in shared memory, so R is formed once per compression.
      using L = PhaseLayout<KP>;
      unsigned char *const xh = smem + L::kXh, *const xl = smem + L::kXl;
      unsigned char *const yh = smem + L::kYh, *const yl = smem + L::kYl;
      const bool bf16 = a.bf16 != 0;
      if (bf16)
        StageChunk<true, kThreads>(RatioRows{mu, stored, ratio_of}, Rows{right, nullptr}, K, 0,
                                   xh, nullptr, yh, nullptr);
      else
        StageChunk<false, kThreads>(RatioRows{mu, stored, ratio_of}, Rows{right, nullptr}, K, 0,
                                    xh, xl, yh, yl);
      ok = MmaChunk<KP, false>(smem, sh, phase, tmem, 0, bf16) && ok;
      if (bf16)
        TransposeStaged<true, kThreads>(K, xh, xl, yh, yl);
      else
        TransposeStaged<false, kThreads>(K, xh, xl, yh, yl);
      __syncthreads();
      if (bf16)
        StageOne<true, kThreads>(Columns{left}, K, 0, xh, nullptr);
      else
        StageOne<false, kThreads>(Columns{left}, K, 0, xh, xl);
      ok = MmaChunk<KP, false>(smem, sh, phase, tmem + KP, 0, bf16) && ok;
    } else {
      ok = PhaseProduct<KP, false>(smem, sh, phase, tmem, K, RatioRows{mu, stored, ratio_of},
                                   Rows{right, nullptr}, a.bf16 != 0) &&
           ok;
      ok = PhaseProduct<KP, false>(smem, sh, phase, tmem + KP, K, Columns{left},
                                   RatioColumns{mu, stored, ratio_of}, a.bf16 != 0) &&
           ok;
    }
    // Accumulator row `row` (TMEM lane), columns [c0, c0 + kHalfColumns).
    const unsigned row = threadIdx.x % 128, c0 = (threadIdx.x / 128) * kHalfColumns;
    const std::uint32_t lane_base = tmem + ((row & ~31u) << 16);
    float *left_out = AdjointOf(op.x);
    float *right_out = AdjointOf(op.z);
    float total = 0.0f;
    if (K % 4 == 0) {
      // Each product's rows go through the (now idle) operand buffers; the
      // adjoints are then formed and stored in coalesced passes.
      float *tile = reinterpret_cast<float *>(smem);
      const auto stage_rows = [&](std::uint32_t column) {
#pragma unroll 1
        for (unsigned c = c0; c < c0 + kHalfColumns; c += 32) {
          float values[32];
          umma::Load32(lane_base + column + c, values);
          if (row < K)
            TileRow(tile, row, c, values);
        }
        __syncthreads();
      };
      // Left adjoint left[r][m] middle[m] P1[r][m].
      stage_rows(0);
#pragma unroll 4
      for (TileWalk w(K); w.row < K; w.Advance()) {
        const unsigned r = w.row, c = w.column;
        const std::size_t at = static_cast<std::size_t>(r) * K + c;
        const float4 l = *reinterpret_cast<const float4 *>(left + at);
        const float4 p = *reinterpret_cast<const float4 *>(tile + r * TileStride() + c);
        *reinterpret_cast<float4 *>(left_out + at) =
            make_float4(l.x * middle[c] * p.x, l.y * middle[c + 1] * p.y,
                        l.z * middle[c + 2] * p.z, l.w * middle[c + 3] * p.w);
      }
      __syncthreads();
      // Right adjoint right[m][c] middle[m] P2[m][c], kept in the tile for
      // the middle adjoint (its row sums).
      stage_rows(KP);
#pragma unroll 4
      for (TileWalk w(K); w.row < K; w.Advance()) {
        const unsigned r = w.row, c = w.column;
        const std::size_t at = static_cast<std::size_t>(r) * K + c;
        const float4 rr = *reinterpret_cast<const float4 *>(right + at);
        float4 *p = reinterpret_cast<float4 *>(tile + r * TileStride() + c);
        const float mr = middle[r];
        const float4 v = *p;
        const float4 adjoint =
            make_float4(rr.x * mr * v.x, rr.y * mr * v.y, rr.z * mr * v.z, rr.w * mr * v.w);
        *reinterpret_cast<float4 *>(right_out + at) = adjoint;
        *p = adjoint;
      }
      __syncthreads();
      if (j < K) {
        const float *row_values = tile + j * TileStride();
        for (unsigned c = 0; c < K; c += 4) {
          const float4 v = *reinterpret_cast<const float4 *>(row_values + c);
          total += v.x;
          total += v.y;
          total += v.z;
          total += v.w;
        }
      }
    } else {
      // Row-per-thread stores (tcgen05.ld is warp-collective: every lane
      // loads, rows >= K discard). The halves' partial middle adjoints meet
      // in the msg and ratio vectors.
      const float *left_row = left + static_cast<std::size_t>(row) * K;
      const float *right_row = right + static_cast<std::size_t>(row) * K;
      const float middle_row = row < K ? middle[row] : 0.0f;
#pragma unroll 1
      for (unsigned c = c0; c < c0 + kHalfColumns; c += 32) {
        float p1[32];
        umma::Load32(lane_base + c, p1);
        if (row < K) {
#pragma unroll
          for (unsigned q = 0; q < 32; ++q)
            if (c + q < K)
              left_out[static_cast<std::size_t>(row) * K + c + q] =
                  left_row[c + q] * middle[c + q] * p1[q];
        }
      }
      float partial = 0.0f;
#pragma unroll 1
      for (unsigned c = c0; c < c0 + kHalfColumns; c += 32) {
        float p2[32];
        umma::Load32(lane_base + KP + c, p2);
        if (row < K) {
#pragma unroll
          for (unsigned q = 0; q < 32; ++q) {
            if (c + q < K) {
              const float adjoint = right_row[c + q] * middle_row * p2[q];
              right_out[static_cast<std::size_t>(row) * K + c + q] = adjoint;
              partial += adjoint;
            }
          }
        }
      }
      if (kHalves == 1) {
        total = partial;
      } else {
        (threadIdx.x < 128 ? msg : ratio)[row] = partial;
        __syncthreads();
        if (j < K)
          total = msg[j] + ratio[j];
      }
    }
    if (j < K)
      NodeOut()[static_cast<std::size_t>(op.y & kMask) * K + j] = total;
    umma::FenceBeforeSync();
    __syncthreads();
  }
};

// One kind of one round over operations [offset, offset + count): a
// persistent grid, CTA b taking operations b, b + grid, ...
template <int KP, int kKind>
__global__ void __launch_bounds__(PhaseLayout<KP>::kThreads, KP == 64 ? 3 : 1)
    WidePhaseKernel(PhaseArgs args) {
  constexpr bool kTensor = kKind == kPhaseCompress || kKind == kPhaseCompressReverse;
  using L = PhaseLayout<KP>;
  extern __shared__ __align__(1024) unsigned char dynamic_smem[];
  __shared__ PhaseShared sh;
  float *vectors = reinterpret_cast<float *>(dynamic_smem + (kTensor ? L::kVectorsAt : 0u));
  std::uint32_t phase = 0;
  bool ok = true;
  if constexpr (kTensor) {
    float4 *p = reinterpret_cast<float4 *>(dynamic_smem);
    for (unsigned i = threadIdx.x; i < L::kVectorsAt / 16; i += L::kThreads)
      p[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (threadIdx.x == 0)
      umma::BarrierInit(&sh.barrier);
    if (threadIdx.x < 32)
      umma::Allocate(&sh.tmem, L::kColumns);
    umma::FenceBeforeSync();
    __syncthreads();
    umma::FenceAfterSync();
  }
  WideOps<KP> ops(args, sh, dynamic_smem, vectors, kTensor ? sh.tmem : 0u, phase, ok);
  for (std::uint32_t t = blockIdx.x; t < args.count; t += gridDim.x) {
    const std::uint32_t i = args.offset + t;
    if constexpr (kKind != kPhaseFinish) {
      if (threadIdx.x == 0) {
        if (t == blockIdx.x)
          ops.template Prefetch<kKind>(i);
        if (t + gridDim.x < args.count)
          ops.template Prefetch<kKind>(i + gridDim.x);
      }
    }
    if constexpr (kKind == kPhaseGather)
      ops.Gather(i);
    else if constexpr (kKind == kPhaseCompress)
      ops.Compress(i);
    else if constexpr (kKind == kPhaseFinish)
      ops.Finish(i);
    else if constexpr (kKind == kPhaseRakeReverse)
      ops.RakeReverse(i);
    else if constexpr (kKind == kPhaseCompressReverse)
      ops.CompressReverse(i);
  }
  if constexpr (kTensor) {
    if (!ok && threadIdx.x == 0)
      atomicOr(args.error, kErrorTensorTimeout);
    umma::FenceBeforeSync();
    __syncthreads();
    umma::FenceAfterSync();
    if (threadIdx.x < 32)
      umma::Deallocate(sh.tmem, L::kColumns);
  }
}

} // namespace wide
} // namespace thmm

#endif // THMM_WIDE_PHASE_CUH_
