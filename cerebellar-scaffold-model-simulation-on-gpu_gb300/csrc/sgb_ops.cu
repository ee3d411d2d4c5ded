// Standalone delivery operator on caller-owned device buffers.
//
// The reference exposes its propagation as free-standing kernels called once
// per projection and step (spike_propagation, spike_propagation_mThreads,
// spike_propagation_PR; Simulation_header.cu:83-303).  sgb_deliver_spikes is
// the same operation for callers that run their own neuron update: given one
// step's spike flags it adds every synapse of every spiking cell into the
// fixed-point delay ring, event-driven.  Two kernels: a ballot compaction of
// the spike flags into an active list (scratch), then one warp per active
// cell walking its push-table row with coalesced loads and integer atomics.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "../../include/scaffold_gb300.h"
#include "sgb_device.h"
#include "sgb_model.h"

namespace sgb {
namespace {

constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kMaxDevices = 64;

// SM count of the current device, queried once per device and cached (the
// delivery kernels are sized by it on every call).
std::atomic<int> g_sms[kMaxDevices];

int device_sms() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
  int v = g_sms[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      return 1;
    g_sms[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

// Scratch layout: [0] active count, [64..] active cell ids (256-byte aligned).
constexpr uint32_t kListOffset = 64;

__global__ void __launch_bounds__(kBlock) k_ops_compact(const uint8_t* __restrict__ spikes,
                                                        uint32_t n, uint32_t* scratch) {
  const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
  const bool f = i < n && spikes[i] != 0;
  const uint32_t ballot = __ballot_sync(kFullMask, f);
  if (!ballot) return;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t off = 0;
  if (lane == 0) off = atomicAdd(scratch, (uint32_t)__popc(ballot));
  off = __shfl_sync(kFullMask, off, 0);
  if (f) scratch[kListOffset + off + __popc(ballot & ((1u << lane) - 1u))] = i;
}

template <bool BF16>
__global__ void __launch_bounds__(kBlock) k_ops_push(const uint32_t* scratch,
                                                     const uint32_t* __restrict__ row,
                                                     const uint32_t* __restrict__ syn,
                                                     const void* __restrict__ w, int* ring,
                                                     uint32_t n, uint32_t slots, uint32_t slot0) {
  // Ring slot of each delay field value d = 0..15: (step + d) % slots, exact
  // for every delay the 4-bit field can hold, whatever the ring's size.
  __shared__ uint32_t s_slot[16];
  if (threadIdx.x < 16) s_slot[threadIdx.x] = (slot0 + threadIdx.x) % slots;
  __syncthreads();
  const uint32_t n_act = scratch[0];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t nw = (gridDim.x * kBlock) >> 5;
  for (uint32_t e = (blockIdx.x * kBlock + threadIdx.x) >> 5; e < n_act; e += nw) {
    const uint32_t j = scratch[kListOffset + e];
    const uint32_t r0 = __ldg(row + j), r1 = __ldg(row + j + 1);
    for (uint32_t q = r0 + lane; q < r1; q += 32) {
      const uint32_t wd = __ldg(syn + q);
      const float wf = BF16 ? __uint_as_float(((uint32_t)__ldg((const unsigned short*)w + q)) << 16)
                            : __ldg((const float*)w + q);
      const uint32_t slot = s_slot[(wd >> kPushPostBits) & 15u];
      atomicAdd(ring + (((size_t)slot * n + (wd & kPushPostMask)) << 1) + (wd >> 31),
                __float2int_rn(wf));
    }
  }
}

}  // namespace

int deliver_check(int32_t n_cells, int32_t weight_type, int32_t ring_slots, int64_t step,
                  const void* spikes, const void* row, const void* syn, const void* w,
                  const void* ring) {
  if (n_cells < 0 || (uint32_t)n_cells > kPushPostMask)
    return set_error(SGB_ERR_ARG, "n_cells %d not in 0..2^27-1", n_cells);
  if (weight_type != SGB_WEIGHT_FP32 && weight_type != SGB_WEIGHT_BF16)
    return set_error(SGB_ERR_ARG, "unknown weight type %d", weight_type);
  if (ring_slots < 2 || ring_slots > kMaxDelay + 1)
    return set_error(SGB_ERR_ARG, "ring_slots %d not in 2..%d", ring_slots, kMaxDelay + 1);
  if (step < 0) return set_error(SGB_ERR_ARG, "step is negative");
  if (n_cells && (!spikes || !row || !syn || !w || !ring))
    return set_error(SGB_ERR_ARG, "NULL device buffer");
  return SGB_OK;
}

// Compaction + push on `scratch` (count word + list of n_cells ids).
cudaError_t deliver_enqueue(const uint8_t* spikes, int32_t n_cells, const uint32_t* row,
                            const uint32_t* syn, const void* w, int32_t weight_type, int32_t* ring,
                            int32_t ring_slots, int64_t step, uint32_t* scratch,
                            cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t), st);
  if (e || !n_cells) return e;
  const uint32_t n = (uint32_t)n_cells;
  k_ops_compact<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(spikes, n, scratch);
  if ((e = cudaGetLastError())) return e;
  const int sms = device_sms();
  const uint32_t slot0 = (uint32_t)(step % ring_slots);
  const int blocks = 2 * (sms > 0 ? sms : 1);
  if (weight_type == SGB_WEIGHT_BF16)
    k_ops_push<true><<<blocks, kBlock, 0, st>>>(scratch, row, syn, w, ring, n,
                                                 (uint32_t)ring_slots, slot0);
  else
    k_ops_push<false><<<blocks, kBlock, 0, st>>>(scratch, row, syn, w, ring, n,
                                                  (uint32_t)ring_slots, slot0);
  return cudaGetLastError();
}

}  // namespace sgb

using namespace sgb;

extern "C" int sgb_deliver_spikes(const uint8_t* spikes, int32_t n_cells, const uint32_t* row,
                                  const uint32_t* syn, const void* weights, int32_t weight_type,
                                  int32_t* ring, int32_t ring_slots, int64_t step, void* stream) {
  int rc = deliver_check(n_cells, weight_type, ring_slots, step, spikes, row, syn, weights, ring);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t* scratch = nullptr;
  const size_t bytes = ((size_t)kListOffset + (size_t)n_cells) * sizeof(uint32_t);
  cudaError_t e = cudaMallocAsync((void**)&scratch, bytes, st);
  if (e) return set_error(SGB_ERR_CUDA, "cudaMallocAsync of %zu scratch bytes: %s", bytes, cudaGetErrorString(e));
  e = deliver_enqueue(spikes, n_cells, row, syn, weights, weight_type, ring, ring_slots, step,
                      scratch, st);
  cudaError_t e2 = cudaFreeAsync(scratch, st);
  if (e) return set_error(SGB_ERR_CUDA, "delivery launch failed: %s", cudaGetErrorString(e));
  if (e2) return set_error(SGB_ERR_CUDA, "cudaFreeAsync: %s", cudaGetErrorString(e2));
  return SGB_OK;
}

// ---------------------------------------------------------------------------
// Delivery without any device allocation.
//
// Some callers cannot allocate device memory at the point where they deliver
// spikes: a real-time loop in which a cudaMalloc (which may synchronise the
// device) would break the step deadline, or a host process whose device
// memory is owned by another allocator (a framework's caching allocator, a
// fixed memory budget) that must not be bypassed.  sgb_deliver_spikes_static
// gives them the same operation as sgb_deliver_spikes with its scratch (one
// count word plus the active-cell list) in the file-scope array below, which
// every GPU that loads this library holds until the process exits.
static constexpr uint32_t kStaticMaxCells = 1u << 20;  // 1,048,576 cells: 4 MiB of scratch
static __device__ __align__(256) uint32_t g_deliver_scratch[sgb::kListOffset + kStaticMaxCells];

namespace sgb {
namespace {

std::mutex g_scratch_mu;
uint32_t* g_scratch_addr[kMaxDevices] = {};

// Device address of the static scratch on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device, with that device current, and cached.  A cudaDeviceReset
// ends the context that holds the array (as it frees every device buffer the
// caller owns), so the cached address is stale after one: this entry point is
// not for a device that the process has reset.
int static_scratch(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e) return set_error(SGB_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(SGB_ERR_UNSUPPORTED, "device %d", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_deliver_scratch);
    if (e) return set_error(SGB_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_scratch_addr[dev] = (uint32_t*)p;
  }
  *out = g_scratch_addr[dev];
  return SGB_OK;
}

}  // namespace
}  // namespace sgb

extern "C" int sgb_deliver_spikes_static(const uint8_t* spikes, int32_t n_cells,
                                         const uint32_t* row, const uint32_t* syn,
                                         const void* weights, int32_t weight_type, int32_t* ring,
                                         int32_t ring_slots, int64_t step, void* stream) {
  if (n_cells > 0 && (uint32_t)n_cells > kStaticMaxCells)
    return set_error(SGB_ERR_RANGE, "n_cells %d exceeds the static scratch of %u cells", n_cells,
                     kStaticMaxCells);
  int rc = deliver_check(n_cells, weight_type, ring_slots, step, spikes, row, syn, weights, ring);
  if (rc) return rc;
  uint32_t* scratch = nullptr;
  rc = static_scratch(&scratch);
  if (rc) return rc;
  const cudaError_t e = deliver_enqueue(spikes, n_cells, row, syn, weights, weight_type, ring,
                                        ring_slots, step, scratch, (cudaStream_t)stream);
  if (e) return set_error(SGB_ERR_CUDA, "delivery launch failed: %s", cudaGetErrorString(e));
  return SGB_OK;
}
