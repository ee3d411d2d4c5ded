// Step kernels of the scaffold simulation hot path (sm_103a).
//
// One exchange step t runs, in stream order:
//   k_update      every cell: INPUT cells draw their Philox Poisson / periodic
//                 stimulus (reference InputStimulation, UserInputFunctions.cu:
//                 86-120); LIF cells consume ring slot t and integrate
//                 `substeps` Euler substeps (reference update_lif_ch,
//                 Simulation_header.cu:305-381).  Spikes leave the kernel as
//                 a bitmap word per warp (ballot), a compacted active list
//                 (ballot + popc + one atomic per warp) and per-segment counts.
//   k_push_csr    event-driven delivery: one warp per spiking cell walks the
//                 cell's pre-major rows and adds fixed-point weights into
//                 ring slot t + delay of each target.
//   k_pull_*      dense delivery for projections in ELL mode: each post cell
//                 gathers the spike bits of its in-row from the bitmap of
//                 step t + 1 - delay and adds the sum into ring slot t + 1
//                 (the reference's pull, Simulation_header.cu:83-139, with
//                 the delay applied on read as at GPUScaffoldSimulation.cu:735).
//   k_advance     step bookkeeping (ring slot, history row, buffer parity).
// The ring holds int32 fixed-point sums, so CSR and ELL delivery, any launch
// order and any number of instances give bit-identical conductances.
#include <stdint.h>

#include "sgb_device.h"
#include "sgb_philox.h"
#include "../../include/scaffold_gb300.h"

namespace sgb {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float load_weight(const void* w, uint32_t q, bool bf16) {
  if (bf16) return __uint_as_float(((uint32_t)((const uint16_t*)w)[q]) << 16);
  return ((const float*)w)[q];
}

__device__ __forceinline__ int to_fixed(float w, float scale) {
  return __float2int_rn(__fmul_rn(w, scale));
}

__device__ __forceinline__ bool window_on(const SrcDev& s, int64_t k) {
  if (s.win_end <= s.win_start) return true;
  int64_t kk = k;
  if (s.win_period > 0) {
    kk = k % s.win_period;
    if (kk < 0) kk += s.win_period;
  }
  return kk >= s.win_start && kk < s.win_end;
}

// PeriodicFiring (UserInputFunctions.cu:8-10): fires in the substep where the
// cycle count floor((t - start) * f / 1000) increments.
__device__ __forceinline__ bool periodic_fire(const SrcDev& s, int64_t k) {
  const double x1 = __dmul_rn((double)(k - s.k_phase), s.cyc);
  const double x0 = __dmul_rn((double)(k - s.k_phase - 1), s.cyc);
  return floor(x1) != floor(x0);
}

__device__ bool input_fire(const StepArgs& a, const SegDev& sd, uint32_t local, uint32_t mask,
                           unsigned long long t) {
  bool fire = false;
  U4 r{};
  for (int s = 0; s < a.substeps; ++s) {
    if ((s & 3) == 0) r = philox_draw(sd.seed, sd.key_base + local, t, kTagInput, (uint32_t)(s >> 2));
    const uint32_t x = u4_get(r, s & 3);
    const int64_t k = (int64_t)t * a.substeps + s;
    uint32_t m = mask;
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      const SrcDev src = a.srcs[sd.src_first + b];
      if (!window_on(src, k)) continue;
      if (src.kind == SGB_INPUT_POISSON)
        fire |= (uint64_t)x < src.thresh;
      else
        fire |= periodic_fire(src, k);
    }
  }
  return fire;
}

// Conductance-based LIF, `substeps` explicit Euler steps.  Statement order is
// the reference's (Simulation_header.cu:338-370): synaptic current from the
// old conductances, conductance decay plus the step's increment on substep 0
// only, spike test on the old potential, refractory count, reset.  Every
// operation is a single IEEE-rounded FP32 op so a CPU restatement reproduces
// it bit for bit.
__device__ __forceinline__ bool lif_update(const SegDev& sd, int substeps, float4& st, int2 acc) {
  float u = st.x, g0 = st.y, g1 = st.z;
  int ref = __float_as_int(st.w);
  const float dge = __fmul_rn(__int2float_rn(acc.x), sd.inv_scale[0]);
  const float dgi = __fmul_rn(__int2float_rn(acc.y), sd.inv_scale[1]);
  const float in0 = sd.sel[0] ? dgi : dge;
  const float in1 = sd.sel[1] ? dgi : dge;
  bool spk = false;
  for (int s = 0; s < substeps; ++s) {
    const float isyn =
        __fmaf_rn(g1, __fsub_rn(u, sd.E[1]), __fmul_rn(g0, __fsub_rn(u, sd.E[0])));
    const float cur = __fsub_rn(__fmaf_rn(sd.neg_gL, __fsub_rn(u, sd.El), sd.Ie), isyn);
    const float du = __fmul_rn(sd.dt_cm, cur);
    if (s == 0) {
      g0 = __fmaf_rn(g0, sd.keep[0], __fmul_rn(sd.gw[0], in0));
      g1 = __fmaf_rn(g1, sd.keep[1], __fmul_rn(sd.gw[1], in1));
    } else {
      g0 = __fmul_rn(g0, sd.keep[0]);
      g1 = __fmul_rn(g1, sd.keep[1]);
    }
    const bool above = u > sd.Vth;
    spk |= above;
    ref = above ? sd.ref_steps : (ref > 0 ? ref - 1 : 0);
    u = ref ? sd.Vr : __fadd_rn(u, du);
  }
  st = make_float4(u, g0, g1, __int_as_float(ref));
  return spk;
}

__global__ void k_chunk_begin(StepArgs a) {
  a.ctl->t_rel = 0;
  a.ctl->raster_count = 0;
  a.raster_off[0] = 0;
}

__global__ void __launch_bounds__(kUpdateTile) k_update(StepArgs a) {
  const UpdTile tile = a.upd_tiles[blockIdx.x];
  const SegDev& sd = a.segs[tile.seg];
  const uint32_t i = tile.start + threadIdx.x;
  const uint32_t i0 = i & ~31u;
  if (i0 - sd.base >= sd.count) return;  // whole warp past the segment end
  const uint32_t local = i - sd.base;
  const bool valid = local < sd.count;
  Ctl* ctl = a.ctl;
  const unsigned long long t = ctl->step;
  bool fired = false;
  if (valid) {
    if (sd.kind == kSegInput) {
      const uint32_t mask = a.src_mask[i];
      if (mask) fired = input_fire(a, sd, local, mask, t);
    } else {
      int2* rp = reinterpret_cast<int2*>(a.ring) + (size_t)ctl->ring_slot * a.n_pad + i;
      const int2 acc = *rp;
      if (acc.x | acc.y) *rp = make_int2(0, 0);
      float4 st = a.state[i];
      fired = lif_update(sd, a.substeps, st, acc);
      a.state[i] = st;
    }
  }
  const uint32_t ballot = __ballot_sync(kFull, fired);
  const uint32_t lane = threadIdx.x & 31u;
  if (lane == 0) a.hist[(size_t)ctl->hist_row * a.n_words + (i >> 5)] = ballot;
  if (ballot == 0) return;
  const uint32_t n = __popc(ballot);
  const uint32_t rank = __popc(ballot & ((1u << lane) - 1u));
  const uint32_t ev = __reduce_add_sync(kFull, fired ? a.outdeg[i] : 0u);
  uint32_t off = 0, roff = 0;
  if (lane == 0) {
    off = atomicAdd(&ctl->active_count[t & 1], n);
    atomicAdd(&a.counts[(size_t)ctl->t_rel * a.n_segs + tile.seg], n);
    if (ev) atomicAdd(&ctl->events, (unsigned long long)ev);
    if (a.raster_cap) roff = atomicAdd(&ctl->raster_count, n);
  }
  off = __shfl_sync(kFull, off, 0);
  if (fired) a.active[(size_t)(t & 1) * a.n_pad + off + rank] = i;
  if (a.raster_cap) {
    roff = __shfl_sync(kFull, roff, 0);
    if (fired) {
      if (roff + rank < a.raster_cap)
        a.raster[roff + rank] = i;
      else
        atomicOr(&ctl->error, kErrRasterOverflow);
    }
  }
}

// One warp per spiking cell; lanes stride over the cell's CSR row so that
// synapse words and weights are read as coalesced 128-byte lines.
template <bool BF16>
__global__ void __launch_bounds__(256) k_push_csr(StepArgs a) {
  Ctl* ctl = a.ctl;
  const unsigned long long t = ctl->step;
  const uint32_t n_active = ctl->active_count[t & 1];
  const uint32_t* list = a.active + (size_t)(t & 1) * a.n_pad;
  const uint32_t slot0 = ctl->ring_slot;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t e = warp; e < n_active; e += n_warps) {
    const uint32_t j = list[e];
    const SegDev& sd = a.segs[a.seg_of_word[j >> 5]];
    const uint32_t local = j - sd.base;
    for (uint32_t o = 0; o < sd.out_count; ++o) {
      const ProjDev& P = a.projs[a.out_list[sd.out_first + o]];
      if (P.mode != SGB_PROP_CSR) continue;
      const uint32_t r0 = P.csr_row[local], r1 = P.csr_row[local + 1];
      if (lane == 0 && r1 > r0) atomicAdd(&a.ctl->delivered, (unsigned long long)(r1 - r0));
      for (uint32_t q = r0 + lane; q < r1; q += 32) {
        const uint32_t wd = P.csr_syn[q];
        const uint32_t d = wd >> kIndexBits;
        uint32_t slot = slot0 + d;
        if (slot >= a.ring_slots) slot -= a.ring_slots;
        const int fx = to_fixed(load_weight(P.csr_w, q, BF16), P.scale);
        atomicAdd(a.ring + (((size_t)slot * a.n_pad + P.post_base + (wd & kIndexMask)) << 1) +
                      P.channel,
                  fx);
      }
    }
  }
}

__device__ __forceinline__ uint32_t spike_bit(const StepArgs& a, uint32_t hist_row_t,
                                              uint32_t pre_global, uint32_t d) {
  uint32_t row = hist_row_t + 1u + a.hist_rows - d;  // row of step t + 1 - d
  row %= a.hist_rows;
  return (__ldg(a.hist + (size_t)row * a.n_words + (pre_global >> 5)) >> (pre_global & 31u)) & 1u;
}

// Column-major ELL: one thread per post cell, ELL column k of all posts is
// contiguous, so a warp reads consecutive words per k.
template <bool BF16>
__global__ void __launch_bounds__(kPullThreadTile) k_pull_thread(StepArgs a) {
  const PullTile tile = a.pull_tiles[blockIdx.x];
  const ProjDev& P = a.projs[tile.proj];
  if (P.mode != SGB_PROP_ELL) return;
  const uint32_t p = tile.post_start + threadIdx.x;
  if (p >= P.post_count) return;
  const Ctl* ctl = a.ctl;
  const uint32_t hrow = ctl->hist_row;
  int acc = 0;
  for (uint32_t k = 0; k < P.ell_K; ++k) {
    const uint32_t q = k * P.post_count + p;
    const uint32_t wd = __ldg(P.ell_syn + q);
    if (wd == kEllPad) break;  // padding is at the end of each row
    if (spike_bit(a, hrow, P.pre_base + (wd & kIndexMask), wd >> kIndexBits))
      acc += to_fixed(load_weight(P.ell_w, q, BF16), P.scale);
  }
  if (acc) {
    uint32_t slot = ctl->ring_slot + 1u;
    if (slot >= a.ring_slots) slot -= a.ring_slots;
    atomicAdd(a.ring + (((size_t)slot * a.n_pad + P.post_base + p) << 1) + P.channel, acc);
  }
}

// Row-major ELL for wide rows: one warp per (post, chunk of kPullWarpChunk).
template <bool BF16>
__global__ void __launch_bounds__(256) k_pull_warp(StepArgs a) {
  const uint32_t item_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (item_id >= a.n_pull_items) return;
  const PullItem it = a.pull_items[item_id];
  const ProjDev& P = a.projs[it.proj];
  if (P.mode != SGB_PROP_ELL) return;
  const uint32_t lane = threadIdx.x & 31u;
  const Ctl* ctl = a.ctl;
  const uint32_t hrow = ctl->hist_row;
  const uint32_t k1 = min(it.k0 + (uint32_t)kPullWarpChunk, P.ell_K);
  const size_t row = (size_t)it.post * P.ell_K;
  int acc = 0;
  for (uint32_t k = it.k0 + lane; k < k1; k += 32) {
    const uint32_t wd = __ldg(P.ell_syn + row + k);
    if (wd != kEllPad &&
        spike_bit(a, hrow, P.pre_base + (wd & kIndexMask), wd >> kIndexBits))
      acc += to_fixed(load_weight(P.ell_w, (uint32_t)(row + k), BF16), P.scale);
  }
  acc = __reduce_add_sync(kFull, acc);
  if (lane == 0 && acc) {
    uint32_t slot = ctl->ring_slot + 1u;
    if (slot >= a.ring_slots) slot -= a.ring_slots;
    atomicAdd(a.ring + (((size_t)slot * a.n_pad + P.post_base + it.post) << 1) + P.channel, acc);
  }
}

__global__ void k_advance(StepArgs a) {
  Ctl* ctl = a.ctl;
  const unsigned long long t = ctl->step + 1ull;
  ctl->step = t;
  ctl->ring_slot = ctl->ring_slot + 1u == a.ring_slots ? 0u : ctl->ring_slot + 1u;
  ctl->hist_row = ctl->hist_row + 1u == a.hist_rows ? 0u : ctl->hist_row + 1u;
  ctl->active_count[t & 1] = 0;
  const uint32_t r = ++ctl->t_rel;
  a.raster_off[r] = ctl->raster_count;
}

// Per-segment spike totals of the chunk, folded into the FP64 accumulators.
__global__ void __launch_bounds__(256) k_chunk_end(StepArgs a) {
  const uint32_t seg = blockIdx.x;
  const uint32_t steps = a.ctl->t_rel;
  unsigned long long s = 0;
  for (uint32_t r = threadIdx.x; r < steps; r += blockDim.x) s += a.counts[(size_t)r * a.n_segs + seg];
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(kFull, s, o);
  __shared__ unsigned long long part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += part[w];
    a.totals[seg] += (double)tot;
  }
}

}  // namespace

cudaError_t launch_chunk_begin(const StepArgs& a, cudaStream_t s) {
  k_chunk_begin<<<1, 1, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_update(const StepArgs& a, cudaStream_t s) {
  if (!a.n_upd_tiles) return cudaSuccess;
  k_update<<<a.n_upd_tiles, kUpdateTile, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_push(const StepArgs& a, int blocks, cudaStream_t s) {
  if (blocks <= 0) return cudaSuccess;
  if (a.bf16)
    k_push_csr<true><<<blocks, 256, 0, s>>>(a);
  else
    k_push_csr<false><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_pull_thread(const StepArgs& a, cudaStream_t s) {
  if (!a.n_pull_tiles) return cudaSuccess;
  if (a.bf16)
    k_pull_thread<true><<<a.n_pull_tiles, kPullThreadTile, 0, s>>>(a);
  else
    k_pull_thread<false><<<a.n_pull_tiles, kPullThreadTile, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_pull_warp(const StepArgs& a, cudaStream_t s) {
  if (!a.n_pull_items) return cudaSuccess;
  const unsigned blocks = (a.n_pull_items + 7u) / 8u;
  if (a.bf16)
    k_pull_warp<true><<<blocks, 256, 0, s>>>(a);
  else
    k_pull_warp<false><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_advance(const StepArgs& a, cudaStream_t s) {
  k_advance<<<1, 1, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_chunk_end(const StepArgs& a, cudaStream_t s) {
  if (!a.n_segs) return cudaSuccess;
  k_chunk_end<<<a.n_segs, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sgb
