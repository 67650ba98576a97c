// Thin inline-PTX wrappers for the 5th-generation tensor cores (tcgen05) on
// sm_103a: tensor-memory allocation, single-CTA TF32 MMA with operands in
// shared memory, completion through an mbarrier, and accumulator read-back.
//
// Operand layout: no swizzle, K-major "core matrices" of 8 rows x 16 bytes
// (8 x 4 fp32 values, or 8 x 8 bf16 values), 128 contiguous bytes each. Element (row, k) of an
// operand lives at
//     (row / 8) * SBO + (k / 4) * LBO + (row % 8) * 16 + (k % 4) * 4
// with LBO (the byte distance between core matrices adjacent in K) = 128 and
// SBO (between core matrices adjacent in M or N) = KD / 4 * 128 for a depth
// of KD. One TF32 MMA consumes a depth of 8 (two core matrices along K), so
// step k of a product starts at the operand base + k * 2 * LBO.
//
// Every wait is bounded: a wait that gives up returns false and the caller
// records an error instead of spinning forever.
#ifndef THMM_UMMA_CUH_
#define THMM_UMMA_CUH_

#include <cstdint>

namespace thmm {
namespace umma {

__device__ __forceinline__ std::uint32_t SmemAddress(const void *p) {
  return static_cast<std::uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) in a no-swizzle K-major operand.
__device__ __forceinline__ std::uint32_t CoreOffset(unsigned row, unsigned k,
                                                    std::uint32_t sbo) {
  return (row / 8) * sbo + (k / 4) * 128u + (row % 8) * 16u + (k % 4) * 4u;
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ std::uint64_t SmemDescriptor(std::uint32_t address,
                                                        std::uint32_t sbo) {
  std::uint64_t d = 0;
  d |= static_cast<std::uint64_t>((address >> 4) & 0x3fffu);
  d |= static_cast<std::uint64_t>((128u >> 4) & 0x3fffu) << 16;
  d |= static_cast<std::uint64_t>((sbo >> 4) & 0x3fffu) << 32;
  d |= static_cast<std::uint64_t>(1) << 46;
  return d;
}

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, M x N tile.
__host__ __device__ constexpr std::uint32_t Tf32Descriptor(unsigned m, unsigned n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// Instruction descriptor of kind::f16 with BF16 A and B (the same type for
// both, as kind::f16 requires), FP32 accumulator, both K-major, M x N tile.
__host__ __device__ constexpr std::uint32_t Bf16Descriptor(unsigned m, unsigned n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// Allocates `columns` (power of two, >= 32) TMEM columns; the base address is
// written to `*slot` (shared memory). Executed by one whole warp.
__device__ __forceinline__ void Allocate(std::uint32_t *slot, std::uint32_t columns) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   SmemAddress(slot)),
               "r"(columns)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void Deallocate(std::uint32_t base, std::uint32_t columns) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base),
               "r"(columns)
               : "memory");
}

__device__ __forceinline__ void BarrierInit(std::uint64_t *barrier) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(SmemAddress(barrier))
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Makes this thread's generic-proxy shared-memory writes visible to the
// tensor cores (async proxy); follow with a CTA barrier.
__device__ __forceinline__ void FenceOperands() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void FenceBeforeSync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void FenceAfterSync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A * B for one depth-8 slice; `accumulate` false overwrites D.
__device__ __forceinline__ void MmaTf32(std::uint32_t tmem, std::uint64_t a,
                                        std::uint64_t b, std::uint32_t idesc,
                                        bool accumulate) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
               "l"(a), "l"(b), "r"(idesc), "r"(accumulate ? 1u : 0u)
               : "memory");
}

// D[tmem] (+)= A * B for one depth-16 slice of BF16 operands.
__device__ __forceinline__ void MmaBf16(std::uint32_t tmem, std::uint64_t a,
                                        std::uint64_t b, std::uint32_t idesc,
                                        bool accumulate) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
               "l"(a), "l"(b), "r"(idesc), "r"(accumulate ? 1u : 0u)
               : "memory");
}

// Arrives on `barrier` once every MMA issued so far by this thread is done.
__device__ __forceinline__ void Commit(std::uint64_t *barrier) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          SmemAddress(barrier))
      : "memory");
}

// Default wait budget: about 2^31 SM cycles (about a second at 2 GHz).
inline constexpr long long kWaitCycles = 1ll << 31;

// Waits for phase `parity` of `barrier` to complete, for at most `budget` SM
// cycles. Returns false on time-out.
__device__ __forceinline__ bool Wait(std::uint64_t *barrier, std::uint32_t parity,
                                     long long budget = kWaitCycles) {
  const long long start = clock64();
  std::uint32_t done = 0;
  while (true) {
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.b32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(SmemAddress(barrier)), "r"(parity)
                 : "memory");
    if (done)
      return true;
    if (clock64() - start > budget)
      return false;
  }
}

// Bulk (TMA, non-tensor) copies global -> shared completing on an mbarrier.
// The issuing thread announces the bytes of the phase with ExpectBytes, then
// issues the copies; every waiter uses Wait with the phase parity. Addresses
// and sizes are multiples of 16 bytes.
__device__ __forceinline__ void ExpectBytes(std::uint64_t *barrier, std::uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   SmemAddress(barrier)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void BulkLoad(void *dst, const void *src, std::uint32_t bytes,
                                         std::uint64_t *barrier) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
               "[%0], [%1], %2, [%3];" ::"r"(SmemAddress(dst)),
               "l"(src), "r"(bytes), "r"(SmemAddress(barrier))
               : "memory");
}
// Starts fetching `bytes` of global memory into L2 (a hint: nothing waits
// on it). Address and size are multiples of 16 bytes.
__device__ __forceinline__ void PrefetchL2(const void *src, std::uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Orders this thread's earlier generic-proxy memory accesses before later
// async-proxy (TMA, tensor core) accesses of the same memory, and back.
__device__ __forceinline__ void FenceProxy() {
  asm volatile("fence.proxy.async;" ::: "memory");
}

// Loads 32 consecutive FP32 accumulator columns of this thread's TMEM lane
// (warp w reads lanes 32w .. 32w + 31).
__device__ __forceinline__ void Load32(std::uint32_t address, float (&out)[32]) {
  std::uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(address));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j)
    out[j] = __uint_as_float(r[j]);
}

} // namespace umma
} // namespace thmm

#endif // THMM_UMMA_CUH_
