// Tree contraction of the wide-state engine (included by wide_engine.cuh).
#ifndef THMM_WIDE_ENGINE_TREE_CUH_
#define THMM_WIDE_ENGINE_TREE_CUH_

namespace thmm {
namespace wide {

// One tree instance contracted by the whole CTA. Scratch layout and operation
// records are those of the narrow engines (engine.h): node messages N*K,
// (unused) branch slots, compressed paths C*K*K and their adjoints C*K*K.
template <int KP> struct Tree {
  const EngineArgs &a;
  Shared &sh;
  unsigned char *smem;
  std::uint32_t tmem;
  std::uint32_t &phase;
  std::uint32_t &copy_phase; // bit s: phase parity of raw set s
  DevInstance inst;
  DevProgram prog;
  unsigned K, KK;
  float *nodes;
  float *comps;
  float *comp_mu;
  const float *edge_in;
  // K-vectors in shared memory.
  float *v, *leaf, *msg, *middle, *ratio, *spare;
  long long exponent = 0; // thread 0's log-scale exponent sum
  int zero = 0;           // some renormalised message was identically zero
  bool ok = true;         // every tensor-core and bulk-copy wait completed
  // Raw K x K matrices in shared memory, filled by bulk copy (KP = 64 and K a
  // multiple of 4, so every matrix is 16-byte aligned and sized).
  float *raw[3] = {nullptr, nullptr, nullptr}; // the current set
  float *raw_base = nullptr;  // set s, matrix i at raw_base + (3 s + i) K_P^2
  unsigned current = 0;       // raw set of the current operation
  unsigned issued = 0;        // bit s: a copy into set s is in flight
  bool bulk = false;

  __device__ Tree(const EngineArgs &args, unsigned item, Shared &shared,
                  unsigned char *dynamic_smem, std::uint32_t tmem_base,
                  std::uint32_t &mma_phase, std::uint32_t &bulk_phase)
      : a(args), sh(shared), smem(dynamic_smem), tmem(tmem_base), phase(mma_phase),
        copy_phase(bulk_phase) {
    inst = a.instances[item];
    prog = a.programs[inst.program];
    K = a.states;
    KK = K * K;
    float *base = static_cast<float *>(a.scratch) + inst.scratch_base;
    nodes = base;
    comps = nodes + static_cast<std::size_t>(prog.num_nodes) * K +
            static_cast<std::size_t>(prog.num_rakes) * K;
    comp_mu = comps + static_cast<std::size_t>(prog.num_compressions) * KK;
    edge_in = static_cast<const float *>(a.edge_in) +
              inst.edge_in_base * static_cast<std::uint64_t>(KK);
    float *vectors = reinterpret_cast<float *>(smem + Layout<KP>::kVectorsAt);
    v = vectors;
    leaf = vectors + 128;
    msg = vectors + 256;
    middle = vectors + 384;
    ratio = vectors + 512;
    spare = vectors + 640;
    if constexpr (Layout<KP>::kRawCount == 6) {
      raw_base = reinterpret_cast<float *>(smem + Layout<KP>::kRawAt);
      bulk = K % 4 == 0 && (reinterpret_cast<std::uintptr_t>(edge_in) & 15) == 0 &&
             (reinterpret_cast<std::uintptr_t>(comps) & 15) == 0 &&
             (reinterpret_cast<std::uintptr_t>(comp_mu) & 15) == 0;
    }
  }

  // Starts bulk copies of `count` K x K matrices into raw set `set` (thread 0
  // only; the set must be free: its earlier readers are behind a CTA barrier).
  __device__ __forceinline__ float *RawMatrix(unsigned set, unsigned i) const {
    return raw_base + (3 * set + i) * static_cast<unsigned>(KP * KP);
  }

  __device__ __forceinline__ void Issue(unsigned set, const float *m0, const float *m1,
                                        const float *m2, unsigned count) {
    issued |= 1u << set;
    if (threadIdx.x != 0)
      return;
    const std::uint32_t bytes = KK * 4u;
    umma::FenceProxy();
    umma::ExpectBytes(&sh.copy_barrier[set], bytes * count);
    umma::BulkLoad(RawMatrix(set, 0), m0, bytes, &sh.copy_barrier[set]);
    if (count > 1)
      umma::BulkLoad(RawMatrix(set, 1), m1, bytes, &sh.copy_barrier[set]);
    if (count > 2)
      umma::BulkLoad(RawMatrix(set, 2), m2, bytes, &sh.copy_barrier[set]);
  }

  // Makes raw set `set` current once its copies have landed (bounded wait;
  // every thread calls it).
  __device__ __forceinline__ void Await(unsigned set) {
    ok = umma::Wait(&sh.copy_barrier[set], (copy_phase >> set) & 1u) && ok;
    copy_phase ^= 1u << set;
    issued &= ~(1u << set);
    current = set;
    raw[0] = RawMatrix(set, 0);
    raw[1] = RawMatrix(set, 1);
    raw[2] = RawMatrix(set, 2);
  }

  // The matrices of the current operation: taken from the copy issued ahead
  // when there is one, else copied now; then the copy for the next operation
  // of the same step (independent of this one) is started into the other set.
  __device__ __forceinline__ void Fetch(const float *m0, const float *m1, const float *m2,
                                        unsigned count, bool has_next, const float *n0,
                                        const float *n1, const float *n2) {
    const unsigned other = current ^ 1u;
    const unsigned set = (issued >> other) & 1u ? other : current;
    if (!((issued >> set) & 1u))
      Issue(set, m0, m1, m2, count);
    Await(set);
    if (has_next)
      Issue(set ^ 1u, n0, n1, n2, count);
  }

  // Row r of path version `ref` (input edge, or compressed path kFlag | t).
  __device__ __forceinline__ const float *Path(unsigned ref) const {
    return (ref & kFlag) ? comps + static_cast<std::size_t>(ref & kMask) * KK
                         : edge_in + static_cast<std::size_t>(ref) * KK;
  }

  // dst[j] for j < K: the stored value of node `ref` (kFlag) or its input
  // factor; for a categorical model (root ? root potential : 1) times the
  // emission row of its observation (src/gpu_backend_impl.inc:326-382).
  __device__ __forceinline__ void NodeVector(unsigned ref, unsigned obs, float *dst) const {
    const unsigned j = threadIdx.x;
    if (j >= K)
      return;
    if (ref & kFlag) {
      dst[j] = nodes[static_cast<std::size_t>(ref & kMask) * K + j];
      return;
    }
    if (!a.categorical) {
      dst[j] = static_cast<const float *>(a.node_in)[(inst.node_base + ref) * K + j];
      return;
    }
    const bool root = ref == (prog.root & kMask);
    const float *root_potential = static_cast<const float *>(a.root_potential);
    float value = root ? root_potential[j] : 1.0f;
    if (obs != kNone) {
      const unsigned category = a.observations[inst.obs_base + obs];
      value = category < a.categories
                  ? value * static_cast<const float *>(a.emission)[category * K + j]
                  : 0.0f;
    }
    dst[j] = value;
  }

  // out[i] = sum_j path[i][j] * x[j] for i < K (x and out in shared memory).
  __device__ __forceinline__ void MatVec(const float *path, const float *x, float *out) const {
    const unsigned warp = threadIdx.x / 32, lane = threadIdx.x & 31;
#pragma unroll 2
    for (unsigned i = warp; i < K; i += kThreads / 32) {
      const float *row = path + static_cast<std::size_t>(i) * K;
      float s = 0.0f;
#pragma unroll
      for (unsigned q = 0; q < KP / 32; ++q) {
        const unsigned j = lane + 32 * q;
        if (j < K)
          s = fmaf(row[j], x[j], s);
      }
      s = WarpSum(s);
      if (lane == 0)
        out[i] = s;
    }
  }

  // Exponent of the CTA maximum m = f 2^e (f in [0.5, 1)), recorded once; a
  // zero maximum sets the zero flag and gives 0.
  __device__ __forceinline__ int Renormaliser(float local_max) {
    const float m = BlockMax(local_max, sh);
    if (m > 0.0f) {
      const int e = Pow2Exponent(m);
      if (threadIdx.x == 0)
        exponent += e;
      return e;
    }
    if (threadIdx.x == 0)
      zero = 1;
    return 0;
  }

  __device__ void Forward();
  __device__ void Reverse();
  __device__ void Finish(unsigned item);
};

} // namespace wide
} // namespace thmm

#include "wide_engine_sweeps.cuh"

#endif // THMM_WIDE_ENGINE_TREE_CUH_
