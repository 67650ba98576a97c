// thmm_log_partition_static: the batched log partition function without any
// memory allocation, for callers that cannot call cudaMalloc (for example
// code running under an external memory manager that owns all device memory,
// or inside a region where new allocations are forbidden).
//
// Everything the kernel needs beyond the caller's inputs and outputs (the
// compiled plan, the per-item instance table, the work queues and the
// per-tree scratch of the contraction) lives in one file-scope device array,
// kStaticBytes long, which every GPU that loads the library keeps until the
// process exits. The host side compiles the plan into a fixed host image with
// the same builder the workspaces use and copies it into that array; no heap,
// pinned or device allocation is made.
//
// The array's name is only a host-side stand-in for its device address, so
// the first call on a device resolves the address with cudaGetSymbolAddress
// (with that device current) and caches it; that first call should happen
// before any stream capture. All calls share the array and leave the last
// call's contents in it: calls whose GPU work overlaps (for example on two
// streams) race, and the host side (a static host image) is not thread-safe.
// Successive calls on one stream are ordered by that stream.
//
// The host image reaches the device by a copy from pageable host memory: the
// CUDA runtime first waits for work already queued on the stream, then stages
// the image before the call returns, so the next call may rebuild the image at
// once. The sum-product forward kernel has no device-side failure mode (its
// error word is never set); a zero partition shows up as log Z = -inf in the
// caller's output.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <algorithm>
#include <cstdlib>
#include <stdexcept>
#include <string>

#include "engine.cuh" // kWarps (CTA shape shared with the engine kernels)
#include "program.h"
#include "program_builder.h"
#include "thmm_gb300.h"

namespace thmm {
namespace {

constexpr std::size_t kStaticBytes = THMM_STATIC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// The shared scratch array (see the file comment).
static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

// Host image of everything but the scratch region, and the builder's
// temporaries. Both are fixed-size static storage.
alignas(256) unsigned char g_host_image[kStaticBytes];
alignas(256) unsigned char g_host_temp[kStaticBytes];

struct DeviceSetup {
  bool ready = false;
  unsigned char *scratch = nullptr;
  int sms = 0;
  int occupancy[6] = {0, 0, 0, 0, 0, 0}; // per padded state count 4, 8, 16, 20, 24, 32
};
DeviceSetup g_devices[kMaxDevices];

std::size_t AlignUp(std::size_t value, std::size_t alignment) {
  return (value + alignment - 1) / alignment * alignment;
}

// Bump allocator over a fixed buffer.
struct Arena {
  unsigned char *base;
  std::size_t size;
  std::size_t used = 0;
  template <class T> T *Take(std::size_t count) {
    const std::size_t offset = AlignUp(used, alignof(T) < 16 ? 16 : alignof(T));
    if (count > (size - std::min(offset, size)) / sizeof(T))
      throw std::invalid_argument(
          "plan exceeds the static scratch of thmm_log_partition_static");
    used = offset + count * sizeof(T);
    return reinterpret_cast<T *>(base + offset);
  }
};

template <class T> struct FixedVector {
  T *data = nullptr;
  std::size_t n = 0;
  std::size_t capacity = 0;
  void push_back(const T &value) {
    if (n == capacity)
      throw std::logic_error("static program image overflow");
    data[n++] = value;
  }
  std::size_t size() const { return n; }
  T &back() { return data[n - 1]; }
};

template <class T> struct TempArray {
  T *data;
  T &operator[](std::size_t i) { return data[i]; }
  const T &operator[](std::size_t i) const { return data[i]; }
};

// Storage policy for BuildProgram: outputs are laid out in the host image at
// the offsets they will occupy in the device array.
struct StaticStorage {
  Arena temp;
  FixedVector<DevProgram> programs;
  FixedVector<DevStep> steps;
  FixedVector<Uint4> rakes;
  FixedVector<Uint2> combines;
  FixedVector<Uint4> absorbs;
  FixedVector<Uint4> compress;
  FixedVector<Uint2> compress_ends;
  FixedVector<Uint4> gathers;
  template <class T> TempArray<T> Temp(std::size_t count, T value) {
    T *data = temp.Take<T>(count == 0 ? 1 : count);
    for (std::size_t i = 0; i < count; ++i)
      data[i] = value;
    return {data};
  }
};

template <class T>
void Place(Arena &image, FixedVector<T> &vector, std::size_t capacity) {
  vector.data = image.Take<T>(capacity == 0 ? 1 : capacity);
  vector.capacity = capacity;
  vector.n = 0;
}

std::size_t Offset(const Arena &image, const void *p) {
  return static_cast<std::size_t>(static_cast<const unsigned char *>(p) - image.base);
}

void Check(cudaError_t status, const char *what) {
  if (status != cudaSuccess)
    throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(status));
}

DeviceSetup &Setup(int device) {
  if (device < 0 || device >= kMaxDevices)
    throw std::runtime_error("device index out of range for static scratch");
  DeviceSetup &setup = g_devices[device];
  if (!setup.ready) {
    void *address = nullptr;
    Check(cudaGetSymbolAddress(&address, g_static_scratch),
          "cudaGetSymbolAddress(static scratch)");
    setup.scratch = static_cast<unsigned char *>(address);
    Check(cudaDeviceGetAttribute(&setup.sms, cudaDevAttrMultiProcessorCount, device),
          "cudaDeviceGetAttribute");
    const unsigned kmax[6] = {4, 8, 16, 20, 24, 32};
    EngineArgs probe{};
    for (int i = 0; i < 6; ++i)
      Check(LaunchLinearF32(false, kmax[i], kLinearForward, probe, 0, nullptr,
                                            &setup.occupancy[i]),
            "occupancy query");
    setup.ready = true;
  }
  return setup;
}

int TeamThresholdStatic() {
  if (const char *value = std::getenv("THMM_TEAM_THRESHOLD"))
    return std::max(1, std::atoi(value));
  return 1024;
}

} // namespace

// Records the message returned by thmm_last_error() (runtime.cc).
void SetLastError(const char *message);

} // namespace thmm

extern "C" thmm_status thmm_log_partition_static(
    const thmm_plan *plan_handle, size_t states, size_t batch,
    const float *node_potentials, const float *edge_potentials,
    float *log_partitions, void *stream_handle) {
  using namespace thmm;
  try {
    if (plan_handle == nullptr || node_potentials == nullptr ||
        log_partitions == nullptr)
      throw std::invalid_argument("plan, node potentials and outputs must not be null");
    const btrc::Plan &plan = *reinterpret_cast<const btrc::Plan *>(plan_handle);
    if (states == 0 || batch == 0)
      throw std::invalid_argument("accelerator state and batch counts must be nonzero");
    if (states > 32)
      throw std::invalid_argument(
          "state count exceeds the accelerator compression block limit");
    if (plan.num_edges() != 0 && edge_potentials == nullptr)
      throw std::invalid_argument("edge potentials must not be null");
    int device = 0;
    Check(cudaGetDevice(&device), "cudaGetDevice");
    DeviceSetup &setup = Setup(device);

    // Host image: control block, program, instances, items; then scratch.
    Arena image{g_host_image, kStaticBytes};
    image.Take<unsigned char>(256); // queue counters and error word
    StaticStorage storage{Arena{g_host_temp, kStaticBytes}, {}, {}, {}, {}, {}, {}, {}, {}};
    const std::size_t batches = plan.primitive_batches().size();
    Place(image, storage.programs, 1);
    Place(image, storage.steps, 2 * batches + 1);
    Place(image, storage.rakes, plan.num_branches());
    Place(image, storage.combines, plan.branch_combinations().size());
    Place(image, storage.absorbs, plan.branch_absorptions().size());
    Place(image, storage.compress, plan.num_compressions());
    Place(image, storage.compress_ends, plan.num_compressions());
    // Every gather absorbs at least one rake, and each rake belongs to one
    // gather (program_builder.h), so the rake count bounds the gathers.
    Place(image, storage.gathers, plan.num_branches());
    BuildProgram(plan, {}, false, storage);

    DevInstance *instances = image.Take<DevInstance>(batch);
    std::uint32_t *items = image.Take<std::uint32_t>(batch);
    const ScratchSize per_item = InstanceScratch(plan.num_nodes(), plan.num_branches(),
                                                 plan.num_compressions(), states,
                                                 kModeLinear, false);
    for (std::size_t b = 0; b < batch; ++b) {
      instances[b] = DevInstance{};
      instances[b].node_base = b * plan.num_nodes();
      instances[b].edge_out_base = b * plan.num_edges();
      instances[b].scratch_base = b * per_item.elements;
      items[b] = static_cast<std::uint32_t>(b);
    }
    const std::size_t image_bytes = AlignUp(image.used, 256);
    if (per_item.elements != 0 &&
        batch > (kStaticBytes - std::min(image_bytes, kStaticBytes)) /
                    (per_item.elements * sizeof(float)))
      throw std::invalid_argument(
          "batch and plan exceed the " + std::to_string(kStaticBytes >> 20) +
          " MiB static scratch of thmm_log_partition_static");

    const cudaStream_t stream = static_cast<cudaStream_t>(stream_handle);
    unsigned char *base = setup.scratch;
    Check(cudaMemcpyAsync(base + 256, g_host_image + 256, image_bytes - 256,
                          cudaMemcpyHostToDevice, stream),
          "cudaMemcpyAsync static program image");
    Check(cudaMemsetAsync(base, 0, 256, stream), "cudaMemsetAsync static control");

    const unsigned kmax = PaddedStates(states);
    const bool big = plan.num_nodes() >= static_cast<std::size_t>(TeamThresholdStatic());
    EngineArgs args{};
    args.programs = reinterpret_cast<const DevProgram *>(
        base + Offset(image, storage.programs.data));
    args.steps = reinterpret_cast<const DevStep *>(base + Offset(image, storage.steps.data));
    args.rakes = base + Offset(image, storage.rakes.data);
    args.combines = base + Offset(image, storage.combines.data);
    args.absorbs = base + Offset(image, storage.absorbs.data);
    args.compress = base + Offset(image, storage.compress.data);
    args.compress_ends = base + Offset(image, storage.compress_ends.data);
    args.gathers = base + Offset(image, storage.gathers.data);
    args.instances = reinterpret_cast<const DevInstance *>(base + Offset(image, instances));
    const std::uint32_t *device_items =
        reinterpret_cast<const std::uint32_t *>(base + Offset(image, items));
    args.big_items = device_items;
    args.small_items = device_items;
    args.big_count = big ? static_cast<std::uint32_t>(batch) : 0u;
    args.small_count = big ? 0u : static_cast<std::uint32_t>(batch);
    args.queue = reinterpret_cast<std::uint32_t *>(base);
    args.error = reinterpret_cast<std::uint32_t *>(base) + 2;
    args.node_in = node_potentials;
    args.edge_in = edge_potentials;
    args.states = static_cast<std::uint32_t>(states);
    args.scratch = base + image_bytes;
    args.values = log_partitions;
    const int index = kmax == 4    ? 0
                      : kmax == 8  ? 1
                      : kmax == 16 ? 2
                      : kmax == 20 ? 3
                      : kmax == 24 ? 4
                                   : 5;
    const std::size_t teams = big ? batch : (batch + kWarps - 1) / kWarps;
    const int grid = static_cast<int>(std::max<std::size_t>(
        1, std::min<std::size_t>(teams, static_cast<std::size_t>(setup.sms) *
                                            std::max(setup.occupancy[index], 1))));
    Check(LaunchLinearF32(false, kmax, kLinearForward, args, grid, stream, nullptr),
          "tree-HMM accelerator kernel launch");
    SetLastError("");
    return THMM_OK;
  } catch (const std::invalid_argument &error) {
    SetLastError(error.what());
    return THMM_INVALID_ARGUMENT;
  } catch (const std::length_error &error) {
    SetLastError(error.what());
    return THMM_LENGTH_ERROR;
  } catch (const std::logic_error &error) {
    SetLastError(error.what());
    return THMM_LOGIC_ERROR;
  } catch (const std::exception &error) {
    SetLastError(error.what());
    return THMM_RUNTIME_ERROR;
  }
}
