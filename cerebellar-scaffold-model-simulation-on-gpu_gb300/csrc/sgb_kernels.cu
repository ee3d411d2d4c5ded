// Step kernels of the scaffold simulation hot path (sm_103a).
//
// One exchange step t consists of two grid-wide phases:
//   update   every cell, one warp per 32-cell word: INPUT cells draw their
//            Philox Poisson / periodic stimulus (reference InputStimulation,
//            UserInputFunctions.cu:86-120); LIF cells consume ring slot t and
//            integrate `substeps` Euler substeps (reference update_lif_ch,
//            Simulation_header.cu:305-381).  Spikes leave as a bitmap word
//            per warp (ballot), a compacted active list (ballot + popc + one
//            atomic per warp) and per-segment counts.
//   deliver  event-driven push: one warp per spiking cell walks the cell's
//            row of the push table and adds fixed-point weights into ring
//            slot t + delay of each target; dense pull for projections in ELL
//            mode: each post cell gathers the spike bits of its in-row from the
//            bitmap of step t + 1 - delay and adds the sum into ring slot t + 1
//            (the reference's pull, Simulation_header.cu:83-139, with the delay
//            applied on read as at GPUScaffoldSimulation.cu:735).
// Two drivers run these phases: per-step kernels (replayed from a CUDA graph;
// kernel boundaries order the phases) and one persistent cooperative kernel
// per chunk of steps (a bounded grid barrier orders them).  The persistent
// kernel comes in three forms: fused (every word resident in one warp, every
// projection event-driven: update and push share one phase, one barrier a
// step, push rows and items in shared memory; with one substep a step it
// publishes each step's spikes one step early, as soon as the potential that
// decides them is known, and makes a step's writes after its barrier
// arrival -- the late-push timeline, optionally with a split barrier),
// resident (words resident,
// some dense pulls: two barriers) and general (more words than warps; one
// barrier a step with the pushes in each block's shared memory when every
// projection is event-driven, else two with a global item list).  With
// plastic projections a plasticity phase runs before the deliveries.  The
// ring holds int32 fixed-point sums, so push and pull delivery, any launch
// order and any number of instances give bit-identical conductances.
#include <stdint.h>

#include <algorithm>

#include "sgb_device.h"
#include "sgb_philox.h"
#include "../../include/scaffold_gb300.h"

namespace sgb {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// Step indices shared by every phase of one step.
struct StepIdx {
  unsigned long long t;
  uint32_t slot;  // t % ring_slots
  uint32_t hrow;  // t % hist_rows
  uint32_t srow;  // t % (hist_rows + 1): spike-summary row
  uint32_t rel;   // step index within the chunk
  // Element offsets of the step's rows, computed once per step (all fit 32
  // bits: ring_slots * n_pad < 2^31, 2 * hist_rows * n_words <= 2^28).
  uint32_t roff;   // ring slot: slot * n_pad (int2 elements)
  uint32_t hoff;   // history row of step t: (hist_rows - 1 - hrow) * n_words
  uint32_t hoff2;  // its second copy, hist_rows rows further
};

template <bool BF16>
__device__ __forceinline__ float load_weight(const void* w, uint32_t q) {
  if (BF16) return __uint_as_float(((uint32_t)__ldg((const unsigned short*)w + q)) << 16);
  return __ldg((const float*)w + q);
}

__device__ __forceinline__ bool window_on(const SrcDev& s, int64_t k) {
  if (s.win_end <= s.win_start) return true;
  int64_t kk = k;
  if (s.win_period > 0) {
    if ((uint64_t)k <= 0xFFFFFFFFull && (uint64_t)s.win_period <= 0xFFFFFFFFull) {
      kk = (int64_t)((uint32_t)k % (uint32_t)s.win_period);  // same value, 32-bit divide
    } else {
      kk = k % s.win_period;
      if (kk < 0) kk += s.win_period;
    }
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

__device__ bool input_fire(const StepArgs& a, const SrcDev* srcs, const SegDev& sd, uint32_t local,
                           uint32_t mask, unsigned long long t) {
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
      const SrcDev src = srcs[sd.src_first + b];
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
// The LIF constants of a segment, fetched as four 16-byte groups (plus the
// refractory length): a word's update issues 5 loads for them, not 17.
struct LifK {
  float El, Vr, Vth, Ie, neg_gL, dt_cm, keep0, keep1, gw0, gw1, E0, E1, inv0, inv1;
  uint32_t sel0, sel1;
  int32_t ref_steps;
};
__device__ __forceinline__ LifK lif_k(const SegDev& sd) {
  const float4* p = reinterpret_cast<const float4*>(&sd.El);
  const float4 a = p[0], b = p[1], c = p[2], d = p[3];
  LifK k;
  k.El = a.x; k.Vr = a.y; k.Vth = a.z; k.Ie = a.w;
  k.neg_gL = b.x; k.dt_cm = b.y; k.keep0 = b.z; k.keep1 = b.w;
  k.gw0 = c.x; k.gw1 = c.y; k.E0 = c.z; k.E1 = c.w;
  k.inv0 = d.x; k.inv1 = d.y; k.sel0 = __float_as_uint(d.z); k.sel1 = __float_as_uint(d.w);
  k.ref_steps = sd.ref_steps;
  return k;
}

// SUB = 1: the single-substep form of the same operations (the benchmark
// configurations); SUB = 0: `substeps` substeps.
template <int SUB>
__device__ __forceinline__ bool lif_update(const LifK& k, int substeps, float4& st, int2 acc) {
  float u = st.x, g0 = st.y, g1 = st.z;
  int ref = __float_as_int(st.w);
  const float dge = __fmul_rn(__int2float_rn(acc.x), k.inv0);
  const float dgi = __fmul_rn(__int2float_rn(acc.y), k.inv1);
  const float in0 = k.sel0 ? dgi : dge;
  const float in1 = k.sel1 ? dgi : dge;
  bool spk = false;
  const int n = SUB == 1 ? 1 : substeps;
  for (int s = 0; s < n; ++s) {
    const float isyn = __fmaf_rn(g1, __fsub_rn(u, k.E1), __fmul_rn(g0, __fsub_rn(u, k.E0)));
    const float cur = __fsub_rn(__fmaf_rn(k.neg_gL, __fsub_rn(u, k.El), k.Ie), isyn);
    const float du = __fmul_rn(k.dt_cm, cur);
    if (s == 0) {
      g0 = __fmaf_rn(g0, k.keep0, __fmul_rn(k.gw0, in0));
      g1 = __fmaf_rn(g1, k.keep1, __fmul_rn(k.gw1, in1));
    } else {
      g0 = __fmul_rn(g0, k.keep0);
      g1 = __fmul_rn(g1, k.keep1);
    }
    const bool above = u > k.Vth;
    spk |= above;
    ref = above ? k.ref_steps : (ref > 0 ? ref - 1 : 0);
    u = ref ? k.Vr : __fadd_rn(u, du);
  }
  st = make_float4(u, g0, g1, __int_as_float(ref));
  return spk;
}

__device__ __forceinline__ bool lif_step(const LifK& k, int substeps, float4& st, int2 acc) {
  return substeps == 1 ? lif_update<1>(k, 1, st, acc) : lif_update<0>(k, substeps, st, acc);
}

// ---- phase 1: one warp updates the 32 cells of word w --------------------------
// Cross-block data (ring slots written by other SMs' atomics, counters, push
// items) is accessed with ld/st.global.cg so a persistent kernel never sees a
// stale L1 line.

// Push items carry the step that produced them; a consumer clears each item
// it delivers, so the delivery phase finds the end of the list without
// reading the item count.
__device__ __forceinline__ uint32_t item_tag(unsigned long long t) {
  return ((uint32_t)t & 0x3FFFFFu) | 0x400000u;  // never 0 (cleared)
}

// Spike bits of word w at step t: both copies of the history row, and, when
// any cell of the word spiked, the word's bit in the step's summary row.
__device__ __forceinline__ void put_hist(const StepArgs& a, const StepIdx& ix, uint32_t w,
                                         uint32_t bits) {
  __stcg(a.hist + (ix.hoff + w), bits);  // rows in decreasing step order
  __stcg(a.hist + (ix.hoff2 + w), bits);
  if (bits) atomicOr(a.hsum + (size_t)ix.srow * a.n_swords + (w >> 5), 1u << (w & 31u));
}

// The summary row of step t + 1 is free during step t (the oldest row a pull
// of step t reads is that of t + 1 - H); threads gtid, gtid + gthreads, ...
// clear it.
__device__ __forceinline__ void clear_next_summary(const StepArgs& a, const StepIdx& ix,
                                                   uint32_t gtid, uint32_t gthreads) {
  const uint32_t row = ix.srow == a.hist_rows ? 0u : ix.srow + 1u;
  for (uint32_t j = gtid; j < a.n_swords; j += gthreads)
    __stcg(a.hsum + (size_t)row * a.n_swords + j, 0u);
}

// One cell's step; state and constants in registers, ring slot consumed.
__device__ __forceinline__ bool cell_fire(const StepArgs& a, const SegDev& sd, uint32_t i,
                                          uint32_t local, bool valid, float4& st, uint32_t mask,
                                          const StepIdx& ix) {
  if (!valid) return false;
  if (sd.kind == kSegInput) return mask ? input_fire(a, a.srcs, sd, local, mask, ix.t) : false;
  int2* rp = reinterpret_cast<int2*>(a.ring) + (ix.roff + i);
  const int2 acc = __ldcg(rp);
  if (acc.x | acc.y) __stcg(rp, make_int2(0, 0));
  return lif_step(lif_k(sd), a.substeps, st, acc);
}

template <bool BF16>
__device__ __forceinline__ uint32_t push_item(const StepArgs& a, uint2 it, uint32_t slot0);

// A block's own push-item list (general persistent kernel with one grid
// barrier per step): items in shared memory, the step's count.
constexpr uint32_t kGenItems = 1024;  // items per block and step (8 KiB)
struct BlockItems {
  uint2* items;
  uint32_t* count;
};

// Spike bookkeeping of one word: bitmap word, per-segment count, event count,
// raster entries, and the spiking cells' push rows cut into kPushChunk items
// laid out by a warp-inclusive scan (one atomic reserves the warp's items):
// in the step's global list, or with LOCAL in the block's list, where the
// warp itself pushes the items past its capacity (their slots t + d, d >= 1,
// are read after the step's barrier).  Returns the synapses pushed here.
template <bool BF16 = false, bool LOCAL = false>
__device__ __forceinline__ uint32_t publish_word(const StepArgs& a, uint32_t w, uint32_t seg,
                                                 uint32_t i, bool fired, uint32_t r0, uint32_t r1,
                                                 uint32_t outdeg, const StepIdx& ix,
                                                 BlockItems bi = {nullptr, nullptr}) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t ballot = __ballot_sync(kFull, fired);
  if (lane == 0) put_hist(a, ix, w, ballot);
  if (ballot == 0) return 0;
  const uint32_t n = __popc(ballot);
  const uint32_t rank = __popc(ballot & ((1u << lane) - 1u));
  const uint32_t ev = __reduce_add_sync(kFull, fired ? outdeg : 0u);
  const uint32_t nit = fired ? (r1 - r0 + kPushChunk - 1) / kPushChunk : 0u;
  uint32_t incl = nit;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(kFull, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  const uint32_t tot_items = __shfl_sync(kFull, incl, 31);
  uint32_t off = 0, roff = 0;
  Ctl* ctl = a.ctl;
  if (lane == 0) {
    if (tot_items) off = LOCAL ? atomicAdd(bi.count, tot_items)
                               : atomicAdd(&ctl->active_count[ix.t & 1], tot_items);
    atomicAdd(&a.counts[(size_t)ix.rel * a.n_segs + seg], n);
    if (ev) atomicAdd(&ctl->events, (unsigned long long)ev);
    if (a.raster_cap) roff = atomicAdd(&ctl->raster_count, n);
  }
  off = __shfl_sync(kFull, off, 0) + incl - nit;
  uint32_t walked = 0;
  if (LOCAL) {
    for (uint32_t k = 0; k < nit && off + k < kGenItems; ++k) {
      const uint32_t q0 = r0 + k * kPushChunk;
      bi.items[off + k] = make_uint2(q0, min(kPushChunk, r1 - q0) << 23);
    }
    uint32_t spill = __ballot_sync(kFull, off + nit > kGenItems);
    while (spill) {
      const int src = __ffs(spill) - 1;
      spill &= spill - 1;
      const uint32_t o = __shfl_sync(kFull, off, src), c = __shfl_sync(kFull, nit, src);
      const uint32_t b0 = __shfl_sync(kFull, r0, src), b1 = __shfl_sync(kFull, r1, src);
      for (uint32_t k = o < kGenItems ? kGenItems - o : 0u; k < c; ++k) {
        const uint32_t q0 = b0 + k * kPushChunk;
        walked += push_item<BF16>(a, make_uint2(q0, min(kPushChunk, b1 - q0) << 23), ix.slot);
      }
    }
  } else {
    uint2* items = a.items + (size_t)(ix.t & 1) * a.item_cap;
    const uint32_t tag = item_tag(ix.t);
    for (uint32_t k = 0; k < nit; ++k) {
      const uint32_t q0 = r0 + k * kPushChunk;
      const uint32_t len = min(kPushChunk, r1 - q0);
      __stcg(items + off + k, make_uint2(q0, (len << 23) | tag));
    }
  }
  if (a.raster_cap) {
    roff = __shfl_sync(kFull, roff, 0);
    if (fired) {
      if (roff + rank < a.raster_cap)
        a.raster[roff + rank] = i;
      else
        atomicOr(&ctl->error, kErrRasterOverflow);
    }
  }
  return walked;
}

// General form, everything from global memory.  The word's state and ring
// slot are loaded first (their addresses depend only on the word index), the
// segment descriptor next; push-row bounds and out-degrees only for spiking
// cells.  Callers may issue load_word for the next word before finishing the
// current one (the two touch different cells).
struct WordIn {
  float u;
  float2 g;
  int2 acc;
  uint32_t seg;
};

__device__ __forceinline__ WordIn load_word(const StepArgs& a, uint32_t w, const StepIdx& ix) {
  const uint32_t i = (w << 5) + (threadIdx.x & 31u);
  WordIn in;
  in.seg = __ldg(a.seg_of_word + w);
  in.acc = __ldcg(reinterpret_cast<const int2*>(a.ring) + (ix.roff + i));
  // State streams through L2 only: no L1 allocation for the largest stream,
  // which would evict the segment descriptors every word reads.
  in.u = __ldcg(a.su + i);
  in.g = __ldcg(a.sg + i);
  return in;
}

// Register state {u, g0, g1, ref bits} from / to the stored fields.
__device__ __forceinline__ float4 state_in(float u, float2 g, float vr) {
  const int32_t ref = unpack_ref(u);
  return make_float4(ref ? vr : u, g.x, g.y, __int_as_float(ref));
}
__device__ __forceinline__ void state_out(const StepArgs& a, uint32_t i, const float4& st) {
  __stcg(a.su + i, pack_u(st.x, __float_as_int(st.w)));
  __stcg(a.sg + i, make_float2(st.y, st.z));
}

// RECENT: the handle may keep per-cell spike registers (plastic
// projections); the general persistent kernel takes the RECENT = false form
// when it has none, so the update of a network without plasticity carries
// no trace of them.
// SEGSMEM: the segment descriptors and stimulus sources are in the general
// persistent kernel's dynamic shared memory (g_dyn: descriptors, then
// sources) rather than read from global memory.
extern __shared__ __align__(16) unsigned char g_dyn[];
__host__ __device__ __forceinline__ size_t seg_table_bytes(uint32_t n_segs) {
  return ((size_t)n_segs * sizeof(SegDev) + 15) & ~(size_t)15;
}

template <bool RECENT = true, bool SEGSMEM = false, bool BF16 = false, bool LOCAL = false>
__device__ __forceinline__ uint32_t finish_word(const StepArgs& a, uint32_t w, const WordIn& in,
                                                const StepIdx& ix,
                                                BlockItems bi = {nullptr, nullptr}) {
  if (in.seg == 0xFFFFu) return 0;  // padding between segments (warp-uniform)
  const uint32_t lane = threadIdx.x & 31u;
  const SegDev& sd = SEGSMEM ? reinterpret_cast<const SegDev*>(g_dyn)[in.seg] : a.segs[in.seg];
  const uint4 hd = *reinterpret_cast<const uint4*>(&sd);  // base, count, key_base, kind
  const uint32_t i = (w << 5) + lane;
  const uint32_t local = i - hd.x;
  const bool valid = local < hd.y;
  bool fired = false;
  if (hd.w == kSegInput) {  // warp-uniform
    if (valid) {
      const uint32_t mask = __ldg(a.src_mask + i);
      const SrcDev* srcs =
          SEGSMEM ? reinterpret_cast<const SrcDev*>(g_dyn + seg_table_bytes(a.n_segs)) : a.srcs;
      if (mask) fired = input_fire(a, srcs, sd, local, mask, ix.t);
    }
  } else {
    // Every lane of a LIF word runs the update: a padding lane past the
    // segment's end integrates its own (never read) padding state and is
    // masked out of the spikes, so no lane diverges here.
    if (in.acc.x | in.acc.y)
      __stcg(reinterpret_cast<int2*>(a.ring) + (ix.roff + i), make_int2(0, 0));
    const LifK k = lif_k(sd);
    float4 st = state_in(in.u, in.g, k.Vr);
    fired = lif_step(k, a.substeps, st, in.acc) && valid;
    state_out(a, i, st);
  }
  // Handles with plastic projections: each cell's last 64 steps of spikes,
  // bit j = step t - j, for the pairing windows.
  if (RECENT && a.recent && valid)
    a.recent[(ix.t & 1ull) * a.n_pad + i] =
        (__ldcg(a.recent + ((ix.t + 1ull) & 1ull) * a.n_pad + i) << 1) | (fired ? 1ull : 0ull);
  uint32_t r0 = 0, r1 = 0, od = 0;
  if (fired) {
    od = __ldg(a.outdeg + i);
    if (a.any_push) {
      r0 = __ldg(a.push_row + i);
      r1 = __ldg(a.push_row + i + 1);
    }
  }
  return publish_word<BF16, LOCAL>(a, w, in.seg, i, fired, r0, r1, od, ix, bi);
}

__device__ __forceinline__ void update_word(const StepArgs& a, uint32_t w, const StepIdx& ix) {
  finish_word(a, w, load_word(a, w, ix), ix);
}

// Words gw, gw + nw, ... with the next word's loads in flight while the
// current one is computed.  Returns the synapses pushed on the way.
template <bool RECENT, bool SEGSMEM, bool BF16, bool LOCAL>
__device__ __forceinline__ uint32_t update_words(const StepArgs& a, uint32_t gw, uint32_t nw,
                                                 const StepIdx& ix, BlockItems bi) {
  uint32_t w = gw, walked = 0;
  if (w >= a.n_words) return 0;
  WordIn cur = load_word(a, w, ix);
  while (true) {
    const uint32_t wn = w + nw;
    WordIn nxt;
    if (wn < a.n_words) nxt = load_word(a, wn, ix);
    walked += finish_word<RECENT, SEGSMEM, BF16, LOCAL>(a, w, cur, ix, bi);
    if (wn >= a.n_words) break;
    w = wn;
    cur = nxt;
  }
  return walked;
}

// ---- two cells per lane (general persistent kernel, one-barrier form) ----------
// A pair is two consecutive words, cells 64p .. 64p + 63; lane L takes cells
// 64p + 2L and 64p + 2L + 1, both in word 2p + (L >> 4), so a lane's two cells
// share a segment (segments start on 32-cell boundaries).  A lane moves its
// cells' ring entries, potentials and conductances as one int4, float2 and
// float4 each, and the per-word work -- segment header, LIF constants, bitmap
// words, counts, push items -- is shared by twice the cells.  Each cell's
// arithmetic is exactly the one-cell form's.
struct PairIn {
  int4 acc;      // {exc, inh} of the lane's two cells
  float4 g;      // {g0, g1} of the two cells
  float2 u;      // stored potential fields of the two cells
  uint32_t seg;  // segment of the lane's word
};

__device__ __forceinline__ PairIn load_pair(const StepArgs& a, uint32_t p, const StepIdx& ix) {
  const uint32_t c = (p << 6) + 2u * (threadIdx.x & 31u);
  PairIn in;
  in.seg = __ldg(a.seg_of_word + (c >> 5));
  // ix.roff and c are even: 16-byte aligned pairs of int2 / float2.
  in.acc = __ldcg(reinterpret_cast<const int4*>(reinterpret_cast<const int2*>(a.ring) + (ix.roff + c)));
  in.u = __ldcg(reinterpret_cast<const float2*>(a.su + c));
  in.g = __ldcg(reinterpret_cast<const float4*>(a.sg + c));
  return in;
}

// Bitmap words of words w, w + 1 (w even, so both share a summary word).
__device__ __forceinline__ void put_hist2(const StepArgs& a, const StepIdx& ix, uint32_t w,
                                          uint32_t b0, uint32_t b1) {
  __stcg(reinterpret_cast<uint2*>(a.hist + (ix.hoff + w)), make_uint2(b0, b1));
  __stcg(reinterpret_cast<uint2*>(a.hist + (ix.hoff2 + w)), make_uint2(b0, b1));
  const uint32_t sbits = (b0 ? 1u << (w & 31u) : 0u) | (b1 ? 2u << (w & 31u) : 0u);
  if (sbits) atomicOr(a.hsum + (size_t)ix.srow * a.n_swords + (w >> 5), sbits);
}

// Spike bookkeeping of a pair: bitmap words, per-segment counts (one per
// word), events, raster entries, and the spiking cells' push rows cut into
// kPushChunk items in the block's list (items past its capacity are pushed
// here).  Returns the synapses pushed here.
template <bool BF16>
__device__ __forceinline__ uint32_t publish_pair(const StepArgs& a, uint32_t p, uint32_t c,
                                                 uint32_t seg, bool f0, bool f1, const StepIdx& ix,
                                                 BlockItems bi) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t packed = (f0 ? 1u : 0u) | (f1 ? 2u : 0u);
  // Cell j of word 2p is lane j >> 1's cell j & 1; of word 2p + 1, lane 16 + (j >> 1)'s.
  const uint32_t x0 = __shfl_sync(kFull, packed, lane >> 1);
  const uint32_t x1 = __shfl_sync(kFull, packed, 16u + (lane >> 1));
  const uint32_t W0 = __ballot_sync(kFull, (x0 >> (lane & 1u)) & 1u);
  const uint32_t W1 = __ballot_sync(kFull, (x1 >> (lane & 1u)) & 1u);
  if (lane == 0) put_hist2(a, ix, 2u * p, W0, W1);
  if ((W0 | W1) == 0u) return 0;
  Ctl* ctl = a.ctl;
  const uint32_t mine = lane < 16u ? W0 : W1;
  if ((lane & 15u) == 0u && mine)
    atomicAdd(&a.counts[(size_t)ix.rel * a.n_segs + seg], (uint32_t)__popc(mine));
  uint32_t ev = 0, ra = 0, rb = 0, rc = 0;
  if (packed) {
    if (f0) ev += __ldg(a.outdeg + c);
    if (f1) ev += __ldg(a.outdeg + c + 1u);
    if (a.any_push) {
      ra = __ldg(a.push_row + c);
      rb = __ldg(a.push_row + c + 1u);
      rc = __ldg(a.push_row + c + 2u);
    }
  }
  ev = __reduce_add_sync(kFull, ev);
  const uint32_t na = f0 ? (rb - ra + kPushChunk - 1) / kPushChunk : 0u;
  const uint32_t nb = f1 ? (rc - rb + kPushChunk - 1) / kPushChunk : 0u;
  const uint32_t nit = na + nb;
  uint32_t incl = nit;
  uint32_t rk = (f0 ? 1u : 0u) + (f1 ? 1u : 0u), rincl = rk;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(kFull, incl, o);
    const uint32_t r = __shfl_up_sync(kFull, rincl, o);
    if (lane >= (uint32_t)o) {
      incl += v;
      rincl += r;
    }
  }
  const uint32_t tot_items = __shfl_sync(kFull, incl, 31);
  uint32_t off = 0, roff = 0;
  if (lane == 0) {
    if (tot_items) off = atomicAdd(bi.count, tot_items);
    if (ev) atomicAdd(&ctl->events, (unsigned long long)ev);
    if (a.raster_cap) roff = atomicAdd(&ctl->raster_count, (uint32_t)(__popc(W0) + __popc(W1)));
  }
  off = __shfl_sync(kFull, off, 0) + incl - nit;
  for (uint32_t k = 0; k < nit && off + k < kGenItems; ++k) {
    const uint32_t q0 = k < na ? ra + k * kPushChunk : rb + (k - na) * kPushChunk;
    const uint32_t q1 = k < na ? rb : rc;
    bi.items[off + k] = make_uint2(q0, min(kPushChunk, q1 - q0) << 23);
  }
  uint32_t walked = 0;
  uint32_t spill = __ballot_sync(kFull, off + nit > kGenItems);
  while (spill) {
    const int src = __ffs(spill) - 1;
    spill &= spill - 1;
    const uint32_t o = __shfl_sync(kFull, off, src), cnt = __shfl_sync(kFull, nit, src);
    const uint32_t sa = __shfl_sync(kFull, na, src);
    const uint32_t pa = __shfl_sync(kFull, ra, src), pb = __shfl_sync(kFull, rb, src),
                   pc = __shfl_sync(kFull, rc, src);
    for (uint32_t k = o < kGenItems ? kGenItems - o : 0u; k < cnt; ++k) {
      const uint32_t q0 = k < sa ? pa + k * kPushChunk : pb + (k - sa) * kPushChunk;
      const uint32_t q1 = k < sa ? pb : pc;
      walked += push_item<BF16>(a, make_uint2(q0, min(kPushChunk, q1 - q0) << 23), ix.slot);
    }
  }
  if (a.raster_cap) {
    roff = __shfl_sync(kFull, roff, 0) + rincl - rk;
    uint32_t q = roff;
    if (f0) {
      if (q < a.raster_cap) a.raster[q] = c; else atomicOr(&ctl->error, kErrRasterOverflow);
      ++q;
    }
    if (f1) {
      if (q < a.raster_cap) a.raster[q] = c + 1u; else atomicOr(&ctl->error, kErrRasterOverflow);
    }
  }
  return walked;
}

template <bool SEGSMEM, bool BF16>
__device__ __forceinline__ uint32_t finish_pair(const StepArgs& a, uint32_t p, const PairIn& in,
                                                const StepIdx& ix, BlockItems bi) {
  const uint32_t c = (p << 6) + 2u * (threadIdx.x & 31u);
  bool f0 = false, f1 = false;
  if (in.seg != 0xFFFFu) {  // padding words past the last segment (half-warp uniform)
    const SegDev& sd = SEGSMEM ? reinterpret_cast<const SegDev*>(g_dyn)[in.seg] : a.segs[in.seg];
    const uint4 hd = *reinterpret_cast<const uint4*>(&sd);  // base, count, key_base, kind
    const uint32_t l0 = c - hd.x;
    const bool v0 = l0 < hd.y, v1 = l0 + 1u < hd.y;
    if (hd.w == kSegInput) {
      const SrcDev* srcs =
          SEGSMEM ? reinterpret_cast<const SrcDev*>(g_dyn + seg_table_bytes(a.n_segs)) : a.srcs;
      const uint2 m = v0 ? __ldg(reinterpret_cast<const uint2*>(a.src_mask + c)) : make_uint2(0u, 0u);
      if (m.x) f0 = input_fire(a, srcs, sd, l0, m.x, ix.t);
      if (v1 && m.y) f1 = input_fire(a, srcs, sd, l0 + 1u, m.y, ix.t);
    } else {
      // Both lanes' cells run the LIF step (a padding cell integrates its own,
      // never read, padding state and is masked out of the spikes).
      if (in.acc.x | in.acc.y | in.acc.z | in.acc.w)
        __stcg(reinterpret_cast<int4*>(reinterpret_cast<int2*>(a.ring) + (ix.roff + c)),
               make_int4(0, 0, 0, 0));
      const LifK k = lif_k(sd);
      float4 s0 = state_in(in.u.x, make_float2(in.g.x, in.g.y), k.Vr);
      float4 s1 = state_in(in.u.y, make_float2(in.g.z, in.g.w), k.Vr);
      f0 = lif_step(k, a.substeps, s0, make_int2(in.acc.x, in.acc.y)) && v0;
      f1 = lif_step(k, a.substeps, s1, make_int2(in.acc.z, in.acc.w)) && v1;
      __stcg(reinterpret_cast<float2*>(a.su + c),
             make_float2(pack_u(s0.x, __float_as_int(s0.w)), pack_u(s1.x, __float_as_int(s1.w))));
      __stcg(reinterpret_cast<float4*>(a.sg + c), make_float4(s0.y, s0.z, s1.y, s1.z));
    }
  }
  return publish_pair<BF16>(a, p, c, in.seg, f0, f1, ix, bi);
}

// Pairs gp, gp + np, ... with the next pair's loads in flight while the
// current one is computed.  Returns the synapses pushed on the way.
template <bool SEGSMEM, bool BF16>
__device__ __forceinline__ uint32_t update_pairs(const StepArgs& a, uint32_t gp, uint32_t np,
                                                 const StepIdx& ix, BlockItems bi) {
  const uint32_t n_pairs = a.n_words >> 1;
  uint32_t p = gp, walked = 0;
  if (p >= n_pairs) return 0;
  PairIn cur = load_pair(a, p, ix);
  while (true) {
    const uint32_t pn = p + np;
    PairIn nxt;
    if (pn < n_pairs) nxt = load_pair(a, pn, ix);
    walked += finish_pair<SEGSMEM, BF16>(a, p, cur, ix, bi);
    if (pn >= n_pairs) break;
    p = pn;
    cur = nxt;
  }
  return walked;
}

// ---- phase 2: deliveries ------------------------------------------------------
// One warp delivers one push item (at most kPushChunk synapses of a spiking
// cell's row): all loads of the item are issued before its atomics so the
// item costs one memory round trip; returns the item's synapse count.
template <bool BF16>
__device__ __forceinline__ uint32_t push_item(const StepArgs& a, uint2 it, uint32_t slot0) {
  constexpr int kPer = kPushChunk / 32;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t q1 = it.x + (it.y >> 23);
  uint32_t wd[kPer];
  float wv[kPer];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const uint32_t q = it.x + k * 32 + lane;
    wd[k] = q < q1 ? __ldg(a.push_syn + q) : 0u;
    wv[k] = q < q1 ? load_weight<BF16>(a.push_w, q) : 0.f;
  }
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    if (it.x + k * 32 + lane >= q1) break;
    uint32_t slot = slot0 + ((wd[k] >> kPushPostBits) & 15u);
    if (slot >= a.ring_slots) slot -= a.ring_slots;
    atomicAdd(a.ring + (((size_t)slot * a.n_pad + (wd[k] & kPushPostMask)) << 1) + (wd[k] >> 31),
              __float2int_rn(wv[k]));
  }
  return it.y >> 23;
}

// The same from a block's shared-memory copy of its cells' rows: {synapse
// word, fixed-point increment} per synapse, so the item's only memory round
// trip is its atomics.
__device__ __forceinline__ uint32_t push_item_smem(const StepArgs& a, const uint2* rows, uint2 it,
                                                   uint32_t slot0) {
  constexpr int kPer = kPushChunk / 32;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t n = it.y >> 23;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const uint32_t j = k * 32 + lane;
    if (j >= n) break;
    const uint2 e = rows[it.x + j];
    uint32_t slot = slot0 + ((e.x >> kPushPostBits) & 15u);
    if (slot >= a.ring_slots) slot -= a.ring_slots;
    atomicAdd(a.ring + (((size_t)slot * a.n_pad + (e.x & kPushPostMask)) << 1) + (e.x >> 31),
              (int)e.y);
  }
  return n;
}

// ---- dense pull (ELL) ----------------------------------------------------------
// A unit is kPullUnit consecutive entries of one projection's ELL, whatever
// its layout.  An entry is the offset of its spike bit above the step's
// history base (word e >> 5, bit e & 31); for the few entries whose pre cell
// spiked the weight is read and added into the post cell's ring slot with one
// atomic (the post is recovered from the entry's offset).
__device__ __forceinline__ const uint32_t* hist_base(const StepArgs& a, uint32_t hrow) {
  return a.hist + (size_t)(a.hist_rows - 1u - hrow) * a.n_words;  // row of step t
}

template <bool BF16>
__device__ __forceinline__ void pull_hit(const StepArgs& a, const ProjDev& P, uint32_t o,
                                         uint32_t slot1) {
  const uint32_t post = P.ell_rowmajor ? o / P.ell_K : o % P.post_count;
  // A plastic projection's weights change every step (inside a persistent
  // launch too): read at L2, not through the non-coherent read-only path.
  const float wv = BF16 ? __uint_as_float((uint32_t)__ldcg((const unsigned short*)P.ell_w + o) << 16)
                        : __ldcg((const float*)P.ell_w + o);
  const int v = __float2int_rn(wv);
  atomicAdd(a.ring + (((size_t)slot1 * a.n_pad + P.post_base + post) << 1) + P.channel, v);
}

// Persistent kernels: one of a unit's kPullParts ranges of kPullUnit /
// kPullParts entries (`part`; 8 per lane, loaded at once, within their
// 64-register budget), so a unit spreads over that many warps and a pull is
// one round of loads per warp.  Entries straight from global memory, tested
// against the block's staged summary when there is one, history words from
// L2 (other blocks write them during the launch).  Returns the lane's hits.
constexpr uint32_t kPullParts = 4;
template <bool BF16>
__device__ __forceinline__ uint32_t pull_unit(const StepArgs& a, const PullUnit un, uint32_t part,
                                              const uint32_t* hb, uint32_t slot1,
                                              const uint32_t* s_sum) {
  constexpr uint32_t B = kPullUnit / kPullParts / 32;
  const uint32_t pad = a.hist_rows * a.n_pad;
  const ProjDev& P = a.projs[un.proj];
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t hits = 0;
  const uint32_t o0 = un.o0 + part * (kPullUnit / kPullParts);
  {
    const uint32_t ob = o0 + lane;
    uint32_t e[B];
#pragma unroll
    for (uint32_t u = 0; u < B; ++u) e[u] = __ldg(P.ell_syn + ob + 32u * u);  // padded to units
    uint32_t hit = 0;
    if (s_sum) {
      // The block's staged summary settles most entries; the history word is
      // read only for those whose 32-cell word had a spike.
#pragma unroll
      for (uint32_t u = 0; u < B; ++u) {
        const uint32_t sw = s_sum[e[u] >> 10];
        if (__funnelshift_r(sw, sw, e[u] >> 5) & 1u)
          hit |= ((__ldcg(hb + (e[u] >> 5)) >> (e[u] & 31u)) & 1u) << u;
      }
    } else {
#pragma unroll
      for (uint32_t u = 0; u < B; ++u)
        if (e[u] < pad) hit |= ((__ldcg(hb + (e[u] >> 5)) >> (e[u] & 31u)) & 1u) << u;
    }
    hits += __popc(hit);
    while (hit) {
      const uint32_t u = __ffs(hit) - 1;
      hit &= hit - 1;
      pull_hit<BF16>(a, P, ob + 32u * u, slot1);
    }
  }
  return hits;
}

// The spike summary of steps t - d1, d1 = 0 .. max_delay - 1 (the delay rows
// a pull of step t reads; a longer history kept for plasticity is not) into
// shared memory as rows d1 of n_swords words, plus the zero word that
// padding entries (row hist_rows) test; threads tid, tid + nthreads, ... with
// four loads issued before their stores.  The caller synchronizes the block.
__device__ __forceinline__ void stage_summary(const StepArgs& a, const StepIdx& ix, uint32_t* s_sum,
                                              uint32_t tid, uint32_t nthreads) {
  const uint32_t R = a.hist_rows + 1u, n = a.max_delay * a.n_swords;
  for (uint32_t j0 = tid; j0 < n; j0 += 4u * nthreads) {
    uint32_t v[4];
#pragma unroll
    for (uint32_t k = 0; k < 4u; ++k) {
      const uint32_t j = j0 + k * nthreads;
      const uint32_t d1 = j / a.n_swords, w = j - d1 * a.n_swords;
      v[k] = j < n ? __ldcg(a.hsum + (size_t)((ix.srow + R - d1) % R) * a.n_swords + w) : 0u;
    }
#pragma unroll
    for (uint32_t k = 0; k < 4u; ++k)
      if (j0 + k * nthreads < n) s_sum[j0 + k * nthreads] = v[k];
  }
  if (tid == 0) s_sum[a.hist_rows * a.n_swords] = 0u;
}

// Delivery phase for one warp: push items gw, gw + nw, ... up to the first
// slot not written this step (each delivered item is cleared), then the dense
// pull units.  Returns the synapses walked by the push items.
template <bool BF16, bool PULL>
__device__ __forceinline__ uint32_t deliver_warp(const StepArgs& a, uint32_t gw, uint32_t nw,
                                                 const StepIdx& ix, const uint32_t* s_sum = nullptr) {
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t walked = 0;
  if (a.any_push) {
    uint2* list = a.items + (size_t)(ix.t & 1) * a.item_cap;
    const uint32_t tag = item_tag(ix.t);
    for (uint32_t u = gw; u < a.item_cap; u += nw) {
      const uint2 it = __ldcg(list + u);
      if ((it.y & 0x7FFFFFu) != tag) break;
      if (lane == 0) __stcg(&list[u].y, 0u);
      walked += push_item<BF16>(a, it, ix.slot);
    }
  }
  if (PULL && a.n_pull_units) {
    const uint32_t slot1 = ix.slot + 1u == a.ring_slots ? 0u : ix.slot + 1u;
    uint32_t hits = 0;
    const uint32_t* hb = hist_base(a, ix.hrow);
    for (uint32_t v = gw; v < a.n_pull_units * kPullParts; v += nw)
      hits += pull_unit<BF16>(a, a.pull_units[v / kPullParts], v % kPullParts, hb, slot1, s_sum);
    hits = __reduce_add_sync(kFull, hits);
    if (lane == 0 && hits) atomicAdd(&a.ctl->pulled, (unsigned long long)hits);
  }
  return walked;
}

__device__ __forceinline__ void ix_rows(const StepArgs& a, StepIdx& ix) {
  ix.roff = ix.slot * a.n_pad;
  ix.hoff = (a.hist_rows - 1u - ix.hrow) * a.n_words;
  ix.hoff2 = ix.hoff + a.hist_rows * a.n_words;
}

__device__ __forceinline__ StepIdx step_of(const StepArgs& a) {
  const Ctl* ctl = a.ctl;
  StepIdx ix;
  ix.t = ctl->step;
  ix.slot = ctl->ring_slot;
  ix.hrow = ctl->hist_row;
  ix.srow = (uint32_t)(ix.t % (a.hist_rows + 1ull));
  ix.rel = ctl->t_rel;
  ix_rows(a, ix);
  return ix;
}

// The next step's indices (persistent kernels).
__device__ __forceinline__ void ix_advance(const StepArgs& a, StepIdx& ix) {
  ix.slot = ix.slot + 1u == a.ring_slots ? 0u : ix.slot + 1u;
  ix.hrow = ix.hrow + 1u == a.hist_rows ? 0u : ix.hrow + 1u;
  ix.srow = ix.srow == a.hist_rows ? 0u : ix.srow + 1u;
  ix_rows(a, ix);
}

// ---- per-step kernels (CUDA-graph driver) ----------------------------------
__global__ void k_chunk_begin(StepArgs a) {
  a.ctl->t_rel = 0;
  a.ctl->raster_count = 0;
  a.raster_off[0] = 0;
}

__global__ void __launch_bounds__(kBlock) k_update(StepArgs a) {
  const uint32_t gtid = blockIdx.x * kBlock + threadIdx.x;
  const uint32_t w = gtid >> 5;
  const StepIdx ix = step_of(a);
  clear_next_summary(a, ix, gtid, gridDim.x * kBlock);
  if (w >= a.n_words) return;
  update_word(a, w, ix);
}

// Delivery of step t; the last block to finish also advances the step
// (ring slot, history row, buffer parity, raster offsets).
template <bool BF16>
__global__ void __launch_bounds__(kBlock) k_deliver(StepArgs a) {
  Ctl* ctl = a.ctl;
  const StepIdx ix = step_of(a);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t walked = deliver_warp<BF16, false>(a, (blockIdx.x * kBlock + threadIdx.x) >> 5,
                                             (gridDim.x * kBlock) >> 5, ix);
  if (lane == 0 && walked) atomicAdd(&ctl->delivered, (unsigned long long)walked);
  // Step bookkeeping by the last block to arrive.
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&ctl->barrier_gen, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    ctl->barrier_gen = 0;
    const unsigned long long t = ix.t + 1ull;
    ctl->step = t;
    ctl->ring_slot = ix.slot + 1u == a.ring_slots ? 0u : ix.slot + 1u;
    ctl->hist_row = ix.hrow + 1u == a.hist_rows ? 0u : ix.hrow + 1u;
    ctl->active_count[t & 1] = 0;
    ctl->t_rel = ix.rel + 1u;
    a.raster_off[ix.rel + 1u] = ctl->raster_count;
  }
}

// Dense pull of the per-step driver (one 1,024-thread block per SM).  Each
// block stages the summary rows of steps t + 1 - d, d = 1..H (one bit per
// 32-cell word: did any cell of it spike) in shared memory, delay-major, so
// an entry's summary word is s_sum[e >> 10]; the word after them stays zero,
// so padding entries (delay field H) never pass.  Warps stream
// units (gw, gw + nw, ...; the first one's loads overlap the staging): a lane
// loads its 32 entries of a unit at once, settles every entry whose summary
// bit is clear in shared memory, and walks the few that passed four at a
// time (usually one trip per warp), loading each entry again (an L1 hit) and
// then its history word (through L1: the history is read-only in this
// launch).  Without room for the summary (SUM false) every entry walks.
template <bool BF16, bool SUM>
__global__ void __launch_bounds__(kPullBlock, 1) k_pull(StepArgs a) {
  constexpr uint32_t E = kPullUnit / 32;  // entries per lane per unit
  constexpr uint32_t W = 4;               // entries walked per trip
  extern __shared__ uint32_t s_sum[];     // [H][n_swords] + 1 (padding's word)
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gw = (blockIdx.x * kPullBlock + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * kPullBlock) >> 5;
  const uint32_t n = a.n_pull_units;
  const StepIdx ix = step_of(a);
  const uint32_t slot1 = ix.slot + 1u == a.ring_slots ? 0u : ix.slot + 1u;
  uint32_t e[E];
  if (gw < n) {
    const PullUnit un = a.pull_units[gw];
    const uint32_t* src = a.projs[un.proj].ell_syn + un.o0 + lane;
#pragma unroll
    for (uint32_t k = 0; k < E; ++k) e[k] = __ldg(src + k * 32u);
  }
  if (SUM) {
    stage_summary(a, ix, s_sum, threadIdx.x, kPullBlock);
    __syncthreads();
  }
  const uint32_t* hb = hist_base(a, ix.hrow);
  const uint32_t pad = a.hist_rows * a.n_pad;
  uint32_t hits = 0;
  for (uint32_t u = gw; u < n; u += nw) {
    const PullUnit un = a.pull_units[u];
    const ProjDev& P = a.projs[un.proj];
    const uint32_t* src = P.ell_syn + un.o0 + lane;  // tables are padded to whole units
    if (u != gw) {
#pragma unroll
      for (uint32_t k = 0; k < E; ++k) e[k] = __ldg(src + k * 32u);
    }
    uint32_t need = 0;
#pragma unroll
    for (uint32_t k = 0; k < E; ++k) {
      if (SUM) {
        const uint32_t sw = s_sum[e[k] >> 10];
        need |= (__funnelshift_r(sw, sw, e[k] >> 5) & 1u) << k;
      } else {
        need |= (uint32_t)(e[k] < pad) << k;
      }
    }
    while (need) {
      uint32_t ks[W], ev[W], hw[W];
#pragma unroll
      for (uint32_t j = 0; j < W; ++j) {
        ks[j] = need ? __ffs(need) - 1u : E;
        need &= need - 1u;
      }
#pragma unroll
      for (uint32_t j = 0; j < W; ++j) ev[j] = ks[j] < E ? __ldg(src + ks[j] * 32u) : 0u;
#pragma unroll
      for (uint32_t j = 0; j < W; ++j)
        hw[j] = ks[j] < E ? __ldg(hb + (ev[j] >> 5)) : 0u;
#pragma unroll
      for (uint32_t j = 0; j < W; ++j) {
        if (ks[j] < E && ((hw[j] >> (ev[j] & 31u)) & 1u)) {
          ++hits;
          pull_hit<BF16>(a, P, un.o0 + ks[j] * 32u + lane, slot1);
        }
      }
    }
  }
  hits = __reduce_add_sync(kFull, hits);
  if (lane == 0 && hits) atomicAdd(&a.ctl->pulled, (unsigned long long)hits);
}

// Dense pull with 16-byte entry loads (per-step driver; one 1,024-thread
// block per SM): as k_pull with the staged summary, but a lane holds entries
// 4L .. 4L + 3 of each 128-entry row of its unit and loads them as one uint4,
// eight loads per unit instead of 32.  Entry m of the lane (0 .. 31) is at
// unit offset (m >> 2) * 128 + 4L + (m & 3).
template <bool BF16>
__global__ void __launch_bounds__(kPullBlock, 1) k_pull_vec(StepArgs a) {
  constexpr uint32_t V = kPullUnit / 128;  // 16-byte loads per lane per unit
  constexpr uint32_t E = 4 * V;            // entries per lane per unit
  constexpr uint32_t W = 4;                // entries walked per trip
  extern __shared__ uint32_t s_sum[];      // [H][n_swords] + 1 (padding's word)
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gw = (blockIdx.x * kPullBlock + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * kPullBlock) >> 5;
  const uint32_t n = a.n_pull_units;
  const StepIdx ix = step_of(a);
  const uint32_t slot1 = ix.slot + 1u == a.ring_slots ? 0u : ix.slot + 1u;
  uint4 q[V];
  if (gw < n) {
    const PullUnit un = a.pull_units[gw];
    const uint4* src = reinterpret_cast<const uint4*>(a.projs[un.proj].ell_syn + un.o0) + lane;
#pragma unroll
    for (uint32_t k = 0; k < V; ++k) q[k] = __ldg(src + 32u * k);
  }
  stage_summary(a, ix, s_sum, threadIdx.x, kPullBlock);
  __syncthreads();
  const uint32_t* hb = hist_base(a, ix.hrow);
  uint32_t hits = 0;
  for (uint32_t u = gw; u < n; u += nw) {
    const PullUnit un = a.pull_units[u];
    const ProjDev& P = a.projs[un.proj];
    const uint32_t* base = P.ell_syn + un.o0 + 4u * lane;  // tables are padded to whole units
    if (u != gw) {
#pragma unroll
      for (uint32_t k = 0; k < V; ++k) q[k] = __ldg(reinterpret_cast<const uint4*>(base) + 32u * k);
    }
    uint32_t need = 0;
#pragma unroll
    for (uint32_t k = 0; k < V; ++k) {
      const uint32_t ev4[4] = {q[k].x, q[k].y, q[k].z, q[k].w};
#pragma unroll
      for (uint32_t j = 0; j < 4; ++j) {
        const uint32_t sw = s_sum[ev4[j] >> 10];
        need |= (__funnelshift_r(sw, sw, ev4[j] >> 5) & 1u) << (4u * k + j);
      }
    }
    while (need) {
      uint32_t ms[W], ev[W], hw[W];
#pragma unroll
      for (uint32_t j = 0; j < W; ++j) {
        ms[j] = need ? __ffs(need) - 1u : E;
        need &= need - 1u;
      }
#pragma unroll
      for (uint32_t j = 0; j < W; ++j)
        ev[j] = ms[j] < E ? __ldg(base + (ms[j] >> 2) * 128u + (ms[j] & 3u)) : 0u;
#pragma unroll
      for (uint32_t j = 0; j < W; ++j) hw[j] = ms[j] < E ? __ldg(hb + (ev[j] >> 5)) : 0u;
#pragma unroll
      for (uint32_t j = 0; j < W; ++j) {
        if (ms[j] < E && ((hw[j] >> (ev[j] & 31u)) & 1u)) {
          ++hits;
          pull_hit<BF16>(a, P, un.o0 + (ms[j] >> 2) * 128u + 4u * lane + (ms[j] & 3u), slot1);
        }
      }
    }
  }
  hits = __reduce_add_sync(kFull, hits);
  if (lane == 0 && hits) atomicAdd(&a.ctl->pulled, (unsigned long long)hits);
}

// STDP of the plastic projections, step t (SynapticPlasticity.cu:40-120), run
// after the cells of step t updated and before the dense pull that delivers
// into slot t + 1, so that delivery uses the new values -- in the reference
// the propagation of the next millisecond follows invoke_stdp_plasticity.
// One warp per unit of 1,024 ELL cells, one lane per cell.  The entry of a
// cell is its pre cell's spike-bit offset for step t + 1 - d above the history
// row of step t, so the spikes of steps t - d - s are at e + (s + 1) n_pad;
// the post cell's spike of step t is at its own index, a teacher's at the
// offset precomputed per post cell.  COH: inside a persistent launch the
// history, spike registers and plastic values were written this launch by
// other SMs, so they are read at L2 (ld.global.cg); a per-step kernel reads
// data written by earlier launches and may use the read-only path.
template <bool COH>
__device__ __forceinline__ uint32_t ld_coh(const uint32_t* p) {
  return COH ? __ldcg(p) : __ldg(p);
}
template <bool COH>
__device__ __forceinline__ uint32_t hist_bit(const uint32_t* hb, uint32_t off) {
  return (ld_coh<COH>(hb + (off >> 5)) >> (off & 31u)) & 1u;
}

// A synapse whose dw is 0 keeps its value and weight bit for bit, so with a0
// = a1_j = 0 (the reference's own coefficients) only synapses of post cells
// whose post / teacher spike is set change: a row-major unit whose posts all
// lack it is skipped after one lookup per post.  Units are kStdpUnit cells
// (four per lane, loads issued together), so the rows of the few posts that
// do change spread over many warps; the window's spike count is gathered
// eight rows at a time.
template <bool BF16, bool COH>
__device__ __forceinline__ bool stdp_post_spiked(const StepArgs& a, const PlastDev& L,
                                                 const ProjDev& P, const uint32_t* hb,
                                                 uint32_t post) {
  const uint32_t so = L.rule == SGB_STDP_TEACHER ? __ldg(L.teacher + post) : P.post_base + post;
  return so != 0xFFFFFFFFu && hist_bit<COH>(hb, so);
}

// Updates the cells of one unit (the whole warp, four cells per lane).
// EARLY: run during the update of step t (a rule that reads only earlier
// steps' spikes), so the spike registers are read from the buffer of step
// t - 1, one bit lower.
// spiked: the screening found the unit inside one post cell's row with its
// post / teacher spike set, so the entries need not look it up again.
template <bool BF16, bool COH, bool EARLY>
__device__ __forceinline__ void stdp_unit(const StepArgs& a, const PullUnit un,
                                          const uint32_t* hb, uint32_t pad, unsigned long long t,
                                          bool spiked = false) {
  constexpr uint32_t B = kStdpUnit / 32;
  const uint32_t lane = threadIdx.x & 31u;
  const PlastDev& L = a.plast[un.proj];
  const ProjDev& P = a.projs[L.proj];
  const uint32_t end = min(un.o0 + kStdpUnit, P.ell_n);
  const bool all = L.a0 != 0.f || L.a1_j != 0.f;  // every synapse may change
  uint32_t e[B], n_upd = 0;
  bool sp[B];
#pragma unroll
  for (uint32_t k = 0; k < B; ++k) {
    const uint32_t o = un.o0 + lane + 32u * k;
    e[k] = o < end ? __ldg(P.ell_syn + o) : pad;
  }
#pragma unroll
  for (uint32_t k = 0; k < B; ++k) {
    const uint32_t o = un.o0 + lane + 32u * k;
    sp[k] = e[k] < pad &&
            (spiked ||
             stdp_post_spiked<BF16, COH>(a, L, P, hb, P.ell_rowmajor ? o / P.ell_K : o % P.post_count));
  }
#pragma unroll
  for (uint32_t k = 0; k < B; ++k) {
    if (e[k] >= pad || !(all || sp[k])) continue;  // padding, or dw = 0
    const uint32_t o = un.o0 + lane + 32u * k;
    ++n_upd;
    bool s_pre;
    uint32_t nwin = 0;  // pre spikes at t - d - j, j < window
    if (L.recent_ok) {
      // The pre cell's spike register: bit d is step t - d, bits d .. d +
      // window - 1 the window (d + window <= 64 for this projection).
      const uint32_t d = e[k] / a.n_pad + 1u, g = e[k] - (d - 1u) * a.n_pad;
      const unsigned long long* rb = a.recent + ((EARLY ? t + 1ull : t) & 1ull) * a.n_pad + g;
      const unsigned long long r = (COH ? __ldcg(rb) : __ldg(rb)) >> (EARLY ? d - 1u : d);
      s_pre = (r & 1ull) != 0ull;
      if (sp[k] && L.a2_ji != 0.f)
        nwin = __popcll(L.window == 64u ? r : r & ((1ull << L.window) - 1ull));
    } else {
      s_pre = hist_bit<COH>(hb, e[k] + a.n_pad) != 0u;
      if (sp[k] && L.a2_ji != 0.f) {
        for (uint32_t j0 = 0; j0 < L.window; j0 += 8u) {
          uint32_t bit[8];
#pragma unroll
          for (uint32_t j = 0; j < 8u; ++j)
            bit[j] = j0 + j < L.window ? hist_bit<COH>(hb, e[k] + (j0 + j + 1u) * a.n_pad) : 0u;
#pragma unroll
          for (uint32_t j = 0; j < 8u; ++j) nwin += bit[j];
        }
      }
    }
    // Reference order: A0, A1_J (pre), A1_I (post / teacher), A2_JI window.
    float dw = __fadd_rn(0.f, L.a0);
    if (s_pre) dw = __fadd_rn(dw, L.a1_j);
    if (sp[k]) dw = __fadd_rn(dw, L.a1_i);
    for (uint32_t j = 0; j < nwin; ++j) dw = __fadd_rn(dw, L.a2_ji);
    float v = __fadd_rn(__ldcg(L.val + o), dw);
    v = v < 0.f ? 0.f : (v > L.v_max ? L.v_max : v);
    L.val[o] = v;
    const float tw = __fmul_rn(__ldg(L.w0 + o), v);
    if (BF16)
      reinterpret_cast<uint16_t*>(L.w_table)[o] = f32_to_bf16_bits(tw);
    else
      reinterpret_cast<float*>(L.w_table)[o] = tw;
  }
  n_upd = __reduce_add_sync(kFull, n_upd);
  if (lane == 0 && n_upd) atomicAdd(&a.ctl->plast_updates, (unsigned long long)n_upd);
}

// A synapse whose dw is 0 keeps its value and weight bit for bit, so with a0
// = a1_j = 0 (the reference's own coefficients) only synapses of post cells
// whose post / teacher spike is set change.  Each warp first tests up to 32
// of its units at once, one per lane (a row-major unit: the one or two posts
// it covers), then updates only the units that can change.  Units are
// kStdpUnit cells, so the rows of the few posts that do change spread over
// many warps; the window's spike count is gathered eight rows at a time.
// The plasticity phase of step ix over warps gw, gw + nw, ... (k_stdp, or a
// phase of the persistent kernels between the update and the deliveries).
template <bool BF16, bool COH, bool EARLY>
__device__ __forceinline__ void stdp_warp(const StepArgs& a, uint32_t gw, uint32_t nw,
                                          const StepIdx& ix) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t* hb = hist_base(a, ix.hrow);
  const uint32_t pad = a.hist_rows * a.n_pad;
  for (uint32_t base = gw; base < a.n_stdp_units; base += 32u * nw) {
    const uint32_t u = base + lane * nw;
    bool active = false, one = false;  // one: a single post, whose post / teacher spike is set
    if (u < a.n_stdp_units) {
      const PullUnit un = a.stdp_units[u];
      const PlastDev& L = a.plast[un.proj];
      const ProjDev& P = a.projs[L.proj];
      if (L.a0 != 0.f || L.a1_j != 0.f || !P.ell_rowmajor) {
        active = true;
      } else {
        const uint32_t end = min(un.o0 + kStdpUnit, P.ell_n);
        const uint32_t p0 = un.o0 / P.ell_K, p1 = (end - 1u) / P.ell_K;
        for (uint32_t p = p0; p <= p1; ++p) active |= stdp_post_spiked<BF16, COH>(a, L, P, hb, p);
        one = active && p0 == p1;
      }
    }
    uint32_t act = __ballot_sync(kFull, active);
    const uint32_t ones = __ballot_sync(kFull, one);
    while (act) {
      const uint32_t j = __ffs(act) - 1;
      act &= act - 1;
      stdp_unit<BF16, COH, EARLY>(a, a.stdp_units[base + j * nw], hb, pad, ix.t, (ones >> j) & 1u);
    }
  }
}

// EARLY: launched beside k_update of the same step (rules that read only
// earlier steps' spikes), reading the spike registers of step t - 1.
template <bool BF16, bool EARLY>
__global__ void __launch_bounds__(kBlock) k_stdp(StepArgs a) {
  stdp_warp<BF16, false, EARLY>(a, (blockIdx.x * kBlock + threadIdx.x) >> 5,
                                (gridDim.x * kBlock) >> 5, step_of(a));
}

// Plastic values back to their start, v_max (the reference starts at 1, its
// clamp), and the tables to the matching weights.
template <bool BF16>
__global__ void __launch_bounds__(kBlock) k_plast_reset(StepArgs a) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gw = (blockIdx.x * kBlock + threadIdx.x) >> 5, nw = (gridDim.x * kBlock) >> 5;
  for (uint32_t u = gw; u < a.n_stdp_units; u += nw) {
    const PullUnit un = a.stdp_units[u];
    const PlastDev& L = a.plast[un.proj];
    const uint32_t end = min(un.o0 + kStdpUnit, a.projs[L.proj].ell_n);
    for (uint32_t o = un.o0 + lane; o < end; o += 32u) {
      L.val[o] = L.v_max;
      const float tw = __fmul_rn(__ldg(L.w0 + o), L.v_max);
      if (BF16)
        reinterpret_cast<uint16_t*>(L.w_table)[o] = f32_to_bf16_bits(tw);
      else
        reinterpret_cast<float*>(L.w_table)[o] = tw;
    }
  }
}

// Per-segment spike totals of the chunk, folded into the FP64 accumulators.
__global__ void __launch_bounds__(kBlock) k_chunk_end(StepArgs a) {
  const uint32_t seg = blockIdx.x;
  const uint32_t steps = a.ctl->t_rel;
  unsigned long long s = 0;
  for (uint32_t r = threadIdx.x; r < steps; r += blockDim.x) s += a.counts[(size_t)r * a.n_segs + seg];
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(kFull, s, o);
  __shared__ unsigned long long part[kBlock / 32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int w = 0; w < kBlock / 32; ++w) tot += part[w];
    a.totals[seg] += (double)tot;
  }
}

// ---- persistent driver ----------------------------------------------------------
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier over co-resident blocks (cooperative launch).  After the
// block barrier, thread 0 arrives on a counter with a gpu-scope release
// reduction (cumulative over the block's writes ordered before it by
// __syncthreads), then polls with gpu-scope acquire loads; the closing
// __syncthreads hands the acquired view to the whole block.  No separate
// fences: measured on 152 blocks, ~0.3 us per barrier less than fence +
// atomicAdd + fence.  It waits for every block's arrival at this barrier (plus
// a.bar_extra arrivals that no block makes, in the tests of this limit) -- at
// most kBarrierTimeoutNs of global time, checked every 256 polls.  On timeout it records
// kErrBarrierTimeout; every block then returns at its next barrier (or as
// soon as it sees the flag), so the kernel always ends and the host reads
// the flag as SGB_ERR_DEVICE.  grid_arrive / grid_wait are the two halves,
// for callers with work that does not depend on the other blocks in between.
__device__ __forceinline__ void grid_arrive(const StepArgs& a, unsigned long long& target) {
  __syncthreads();
  target += gridDim.x;
  if (threadIdx.x == 0)
    asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(a.bar) : "memory");
}

// One thread polls the arrival counter until it reaches target (plus the
// tests' a.bar_extra) with gpu-scope acquire loads, for at most
// kBarrierTimeoutNs of global time; false (and kErrBarrierTimeout recorded)
// when the wait ran out or another block had already recorded a timeout.
__device__ __forceinline__ bool poll_arrivals(const StepArgs& a, unsigned long long target) {
  const unsigned long long want = target + a.bar_extra;
  unsigned long long t0 = 0;
  uint32_t it = 0;
  while (ld_acquire(a.bar) < want) {
    if ((++it & 255u) == 0u) {
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      if (now - t0 > kBarrierTimeoutNs || (__ldcg(&a.ctl->error) & kErrBarrierTimeout)) {
        atomicOr(&a.ctl->error, kErrBarrierTimeout);
        return false;
      }
    }
    __nanosleep(32);
  }
  return true;
}

__device__ __forceinline__ bool grid_wait(const StepArgs& a, unsigned long long target,
                                          uint32_t poller = 0) {
  __shared__ int abort_flag;
  if (threadIdx.x == poller) abort_flag = !poll_arrivals(a, target);
  __syncthreads();
  return !abort_flag;
}

// Arrival by one thread whose gpu-scope fence comes first: the fence followed
// by the relaxed reduction is a release pattern, cumulative over the writes
// that a block barrier ordered before the fence.
__device__ __forceinline__ void grid_arrive_fenced(const StepArgs& a) {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], 1;" ::"l"(a.bar) : "memory");
}

// Block barrier 1 over the first n threads (a multiple of 32).
__device__ __forceinline__ void bar_sync_first(uint32_t n) {
  asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory");
}

__device__ __forceinline__ bool grid_barrier(const StepArgs& a, unsigned long long& target) {
  grid_arrive(a, target);
  return grid_wait(a, target);
}

__host__ __device__ __forceinline__ size_t seg_smem_bytes_dev(const StepArgs& a) {
  return seg_table_bytes(a.n_segs) + (((size_t)a.n_srcs * sizeof(SrcDev) + 15) & ~(size_t)15);
}

// Raster offsets of a launch with one grid barrier per step: a block may
// already reserve raster entries of step s while another still reads the
// count of step s - 1, so the offsets come from the step counts instead (a
// step's entries are contiguous: its reservations all follow the previous
// barrier).  After the launch's last barrier every count is final; block 0
// scans them (all its threads call this; s_wsum holds kPersistBlock / 32).
__device__ void raster_offsets_from_counts(const StepArgs& a, uint32_t n_steps, uint32_t* s_wsum) {
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const uint32_t per = (n_steps + kPersistBlock - 1) / kPersistBlock;
  const uint32_t q0 = min(n_steps, threadIdx.x * per), q1 = min(n_steps, q0 + per);
  uint32_t tot = 0;
  for (uint32_t q = q0; q < q1; ++q)
    for (uint32_t g = 0; g < a.n_segs; ++g) tot += __ldcg(a.counts + (size_t)q * a.n_segs + g);
  uint32_t incl = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(kFull, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  __syncthreads();  // s_wsum's previous readers are done
  if (lane == 31) s_wsum[wib] = incl;
  __syncthreads();
  if (wib == 0) {
    const uint32_t x = s_wsum[lane];
    uint32_t xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(kFull, xi, o);
      if (lane >= (uint32_t)o) xi += v;
    }
    s_wsum[lane] = xi - x;
  }
  __syncthreads();
  uint32_t run = s_wsum[wib] + incl - tot;
  for (uint32_t q = q0; q < q1; ++q) {
    for (uint32_t g = 0; g < a.n_segs; ++g) run += __ldcg(a.counts + (size_t)q * a.n_segs + g);
    a.raster_off[q + 1] = run;
  }
}

// General persistent kernel.  ONE (networks without dense pulls or rules that
// read the step's own spikes): a step's pushes only target ring slots
// t + 1 .. t + D while its update reads slot t, so each block collects its
// spiking cells' push items in shared memory during the update, delivers them
// right after it, and one grid barrier ends the step.  Otherwise the items go
// to a global list delivered by all warps between two grid barriers.
// LANE (one-barrier form, no plasticity): 1 one cell per lane (update_words),
// 2 two cells per lane (update_pairs).
template <bool BF16, bool ONE, int LANE = 1>
__global__ void __launch_bounds__(kPersistBlock, 1) k_persistent(StepArgs a, uint32_t n_steps) {
  // Dynamic shared memory: the segment descriptors every word reads (when
  // a.seg_smem), then the staged spike summary (dense pulls, when it fits).
  uint32_t* s_sum = reinterpret_cast<uint32_t*>(g_dyn + (a.seg_smem ? seg_smem_bytes_dev(a) : 0));
  __shared__ uint2 s_items[ONE ? kGenItems : 1];
  __shared__ uint32_t s_icnt[2];  // item count of step parity p; the other one is reset
  __shared__ uint32_t s_wsum[kPersistBlock / 32];
  if (threadIdx.x == 0) s_icnt[0] = s_icnt[1] = 0;
  if (a.seg_smem) {
    const uint4* src = reinterpret_cast<const uint4*>(a.segs);
    uint4* dst = reinterpret_cast<uint4*>(g_dyn);
    for (uint32_t j = threadIdx.x; j < a.n_segs * (uint32_t)(sizeof(SegDev) / 16); j += kPersistBlock)
      dst[j] = src[j];
    const uint2* ss = reinterpret_cast<const uint2*>(a.srcs);
    uint2* sd = reinterpret_cast<uint2*>(g_dyn + seg_table_bytes(a.n_segs));
    for (uint32_t j = threadIdx.x; j < a.n_srcs * (uint32_t)(sizeof(SrcDev) / 8); j += kPersistBlock)
      sd[j] = ss[j];
  }
  __syncthreads();
  Ctl* ctl = a.ctl;
  StepIdx ix = step_of(a);
  const unsigned long long t0 = ix.t;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gw = (blockIdx.x * kPersistBlock + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * kPersistBlock) >> 5;
  // One-barrier form: update words are dealt warp-major over the blocks
  // (slot = warp x blocks + block), so consecutive words -- a stimulated input
  // segment, say -- spread over all blocks; each row of nw words is still
  // swept together.
  const uint32_t uw = ONE ? (threadIdx.x >> 5) * gridDim.x + blockIdx.x : gw;
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long target = 0;
  uint32_t walked = 0;
  for (uint32_t s = 0; s < n_steps; ++s) {
    ix.t = t0 + s;
    ix.rel = s;
    // Item counter of step t + 1: its last user was the update of step t - 1
    // (kept zero in ONE launches too, for launches of the other form).
    if (leader) __stcg(&ctl->active_count[(ix.t + 1) & 1], 0u);
    clear_next_summary(a, ix, blockIdx.x * kPersistBlock + threadIdx.x, gridDim.x * kPersistBlock);
    const BlockItems bi{s_items, &s_icnt[s & 1u]};
    if (a.n_plast)
      walked += a.seg_smem ? update_words<true, true, BF16, ONE>(a, uw, nw, ix, bi)
                           : update_words<true, false, BF16, ONE>(a, uw, nw, ix, bi);
    else if (LANE == 2)
      walked += a.seg_smem ? update_pairs<true, BF16>(a, uw, nw, ix, bi)
                           : update_pairs<false, BF16>(a, uw, nw, ix, bi);
    else
      walked += a.seg_smem ? update_words<false, true, BF16, ONE>(a, uw, nw, ix, bi)
                           : update_words<false, false, BF16, ONE>(a, uw, nw, ix, bi);
    // Plastic values of step t before its dense deliveries: with rules that
    // read only earlier steps' spikes, in the update phase itself.
    if (a.n_plast && a.stdp_early) stdp_warp<BF16, true, true>(a, gw, nw, ix);
    if (ONE) {
      __syncthreads();
      const uint32_t n_items = min(s_icnt[s & 1u], kGenItems);
      // The other parity's count was last read before the previous barrier.
      if (threadIdx.x == 0) s_icnt[(s & 1u) ^ 1u] = 0;
      for (uint32_t u = threadIdx.x >> 5; u < n_items; u += kPersistBlock / 32)
        walked += push_item<BF16>(a, s_items[u], ix.slot);
      if (!grid_barrier(a, target)) return;
      ix_advance(a, ix);
      continue;
    }
    if (!grid_barrier(a, target)) return;
    if (a.raster_cap && leader) a.raster_off[s + 1] = __ldcg(&ctl->raster_count);
    if (a.n_plast && !a.stdp_early) {
      stdp_warp<BF16, true, false>(a, gw, nw, ix);
      if (!grid_barrier(a, target)) return;
    }
    const uint32_t* sum = nullptr;
    if (a.n_pull_units && a.pull_sum) {
      stage_summary(a, ix, s_sum, threadIdx.x, kPersistBlock);
      __syncthreads();
      sum = s_sum;
    }
    walked += deliver_warp<BF16, true>(a, gw, nw, ix, sum);
    if (!grid_barrier(a, target)) return;
    ix_advance(a, ix);
  }
  if (ONE && a.raster_cap && blockIdx.x == 0) raster_offsets_from_counts(a, n_steps, s_wsum);
  if (lane == 0 && walked) atomicAdd(&ctl->delivered, (unsigned long long)walked);
  if (leader) {
    ctl->step = t0 + n_steps;
    ctl->ring_slot = ix.slot;
    ctl->hist_row = ix.hrow;
    ctl->t_rel = n_steps;
  }
}

// Resident form for networks with at most one 32-cell word per warp: each warp
// keeps its cells' state, source masks, out-degrees and push-row bounds in
// registers for the whole chunk and writes the state back at the end, so a
// step's critical path is the ring read, the cell update and the deliveries.
template <bool BF16>
__global__ void __launch_bounds__(kPersistBlock, 1) k_persistent_resident(StepArgs a,
                                                                          uint32_t n_steps) {
  // Dynamic shared memory as in the general kernel: segment descriptors and
  // sources (when a.seg_smem), then the staged spike summary.
  uint32_t* s_sum = reinterpret_cast<uint32_t*>(g_dyn + (a.seg_smem ? seg_smem_bytes_dev(a) : 0));
  if (a.seg_smem) {
    const uint4* src = reinterpret_cast<const uint4*>(a.segs);
    uint4* dst = reinterpret_cast<uint4*>(g_dyn);
    for (uint32_t j = threadIdx.x; j < a.n_segs * (uint32_t)(sizeof(SegDev) / 16); j += kPersistBlock)
      dst[j] = src[j];
    const uint2* ss = reinterpret_cast<const uint2*>(a.srcs);
    uint2* sd = reinterpret_cast<uint2*>(g_dyn + seg_table_bytes(a.n_segs));
    for (uint32_t j = threadIdx.x; j < a.n_srcs * (uint32_t)(sizeof(SrcDev) / 8); j += kPersistBlock)
      sd[j] = ss[j];
    __syncthreads();
  }
  const SegDev* segs = a.seg_smem ? reinterpret_cast<const SegDev*>(g_dyn) : a.segs;
  Ctl* ctl = a.ctl;
  StepIdx ix = step_of(a);
  const unsigned long long t0 = ix.t;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t gw = (blockIdx.x * kPersistBlock + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * kPersistBlock) >> 5;
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  // Words are dealt round-robin over the blocks (word slot = warp x blocks +
  // block), so every SM holds about the same number of cells and spikes.
  const uint32_t ws = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  const bool has = ws < a.n_upd_words;
  uint32_t w = 0, seg = 0, i = 0, local = 0, mask = 0, r0 = 0, r1 = 0, od = 0;
  bool valid = false, lif = false;
  float4 st = make_float4(0.f, 0.f, 0.f, 0.f);
  if (has) {
    w = __ldg(a.upd_words + ws);
    seg = __ldg(a.seg_of_word + w);
    i = (w << 5) + lane;
    const SegDev& sd = a.segs[seg];
    local = i - sd.base;
    valid = local < sd.count;
    lif = sd.kind == kSegLif;
    if (valid) {
      if (lif) st = state_in(a.su[i], a.sg[i], sd.Vr); else mask = __ldg(a.src_mask + i);
      od = __ldg(a.outdeg + i);
      if (a.any_push) {
        r0 = __ldg(a.push_row + i);
        r1 = __ldg(a.push_row + i + 1);
      }
    }
  }
  unsigned long long target = 0;
  uint32_t walked = 0;
  for (uint32_t s = 0; s < n_steps; ++s) {
    ix.t = t0 + s;
    ix.rel = s;
    if (leader) __stcg(&ctl->active_count[(ix.t + 1) & 1], 0u);
    clear_next_summary(a, ix, blockIdx.x * kPersistBlock + threadIdx.x, gridDim.x * kPersistBlock);
    if (has) {
      const bool fired = cell_fire(a, segs[seg], i, local, valid, st, mask, ix);
      if (a.recent && valid)
        a.recent[(ix.t & 1ull) * a.n_pad + i] =
            (__ldcg(a.recent + ((ix.t + 1ull) & 1ull) * a.n_pad + i) << 1) | (fired ? 1ull : 0ull);
      publish_word(a, w, seg, i, fired, r0, r1, od, ix);
    }
    // Plastic values of step t before its dense deliveries: with rules that
    // read only earlier steps' spikes, in the update phase itself, on the
    // warps without a word (word slots past the last word) when there are
    // some, so that updates and plasticity run side by side.
    if (a.n_plast && a.stdp_early) {
      const uint32_t n_idle = nw > a.n_upd_words ? nw - a.n_upd_words : 0u;
      if (n_idle == 0u)
        stdp_warp<BF16, true, true>(a, gw, nw, ix);
      else if (!has)
        stdp_warp<BF16, true, true>(a, ws - a.n_upd_words, n_idle, ix);
    }
    if (!grid_barrier(a, target)) break;
    if (a.raster_cap && leader) a.raster_off[s + 1] = __ldcg(&ctl->raster_count);
    if (a.n_plast && !a.stdp_early) {
      stdp_warp<BF16, true, false>(a, gw, nw, ix);
      if (!grid_barrier(a, target)) break;
    }
    const uint32_t* sum = nullptr;
    if (a.n_pull_units && a.pull_sum) {
      stage_summary(a, ix, s_sum, threadIdx.x, kPersistBlock);
      __syncthreads();
      sum = s_sum;
    }
    walked += deliver_warp<BF16, true>(a, gw, nw, ix, sum);
    if (!grid_barrier(a, target)) break;
    ix_advance(a, ix);
  }
  if (valid && lif) state_out(a, i, st);
  if (__ldcg(&ctl->error) & kErrBarrierTimeout) return;
  if (lane == 0 && walked) atomicAdd(&ctl->delivered, (unsigned long long)walked);
  if (leader) {
    ctl->step = t0 + n_steps;
    ctl->ring_slot = ix.slot;
    ctl->hist_row = ix.hrow;
    ctl->t_rel = n_steps;
  }
}

// Fused form (resident networks whose projections are all event-driven): a
// step's deliveries only target ring slots t+1 .. t+D-1 while its update only
// reads slot t, so update and push of the same step share one phase and a
// step needs one grid barrier.  Each block gathers the push items of its
// spiking cells in shared memory, so the rows of a cell with thousands of
// synapses spread over the block's 32 warps.  With a.row_smem > 0 the block
// first copies its cells' push rows into dynamic shared memory (in word, lane
// order, each row whole or not at all; rows past the capacity stay in global
// memory), so a step's pushes read no global memory.
constexpr uint32_t kBlockItems = 2048;  // push items per block and step (16 KiB)
// Own rows are cut into items of 2^a.item_log2 synapses (32, 64 or 128; 64 =
// two per lane unless the autotuner picked another width): a block usually
// pushes one or two spikes' rows a step, and smaller items spread their
// scattered reductions over more of its warps.

// An item of the fused kernel: (first synapse, length << 23 | flags); flag 1:
// the synapses are in the block's shared-memory rows, flag 2: a shard of the
// previous step's spike (its delays count from that step's ring slot).
template <bool BF16>
__device__ __forceinline__ uint32_t push_any(const StepArgs& a, const uint2* rows, uint2 it,
                                             uint32_t slot, uint32_t prev) {
  const uint32_t s0 = (it.y & 2u) ? prev : slot;
  return (it.y & 1u) ? push_item_smem(a, rows, it, s0) : push_item<BF16>(a, it, s0);
}

// TL: the step's timeline -- 0 spikes in their own step; for one-substep steps
// 1 late push, 2 late push with a split grid barrier (see the loops below).
// ILOG: push items of 2^ILOG synapses.
template <bool BF16, uint32_t TL, uint32_t ILOG>
__global__ void __launch_bounds__(kPersistBlock, 1) k_persistent_fused(StepArgs a,
                                                                       uint32_t n_steps) {
  __shared__ uint2 s_items[kBlockItems];
  __shared__ uint32_t s_n[2];  // item count of step parity p; the other one is reset
  __shared__ uint32_t s_wsum[kPersistBlock / 32];
  __shared__ uint4 s_sh[kMaxShards];  // {cell, first synapse, length << 23 | flags, global first}
  __shared__ uint32_t s_shtot, s_ptot;
  __shared__ uint32_t s_od[kPersistBlock];  // out-degree of each thread's cell
  // Segment descriptors and stimulus sources, read every step, in shared
  // memory (when few enough): a miss in the small L1 that this kernel's
  // shared-memory carve-out leaves would cost an L2 round trip per step.
  constexpr uint32_t kSegCache = 16, kSrcCache = 16;
  __shared__ SegDev s_seg[kSegCache];
  __shared__ SrcDev s_src[kSrcCache];
  extern __shared__ uint2 s_rows[];
  const SegDev* segs = a.n_segs <= kSegCache ? s_seg : a.segs;
  const SrcDev* srcs = a.n_srcs <= kSrcCache ? s_src : a.srcs;
  if (a.n_segs <= kSegCache && threadIdx.x < a.n_segs) s_seg[threadIdx.x] = a.segs[threadIdx.x];
  if (a.n_srcs <= kSrcCache && threadIdx.x < a.n_srcs) s_src[threadIdx.x] = a.srcs[threadIdx.x];
  Ctl* ctl = a.ctl;
  StepIdx ix = step_of(a);
  const unsigned long long t0 = ix.t;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wib = threadIdx.x >> 5;
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  // Words are dealt round-robin over the blocks (word slot = warp x blocks +
  // block), so every SM holds about the same number of cells and spikes.
  const uint32_t ws = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  const bool has = ws < a.n_upd_words;
  // st: a LIF cell's state {u, g0, g1, ref}; an input cell's source mask and
  // index within its segment (bits of st.x, st.y).
  uint32_t w = 0, seg = 0, i = 0, r0 = 0, r1 = 0;
  s_od[threadIdx.x] = 0;
  bool valid = false, lif = false;
  float4 st = make_float4(0.f, 0.f, 0.f, 0.f);
  if (has) {
    w = __ldg(a.upd_words + ws);
    seg = __ldg(a.seg_of_word + w);
    i = (w << 5) + lane;
    const SegDev& sd = a.segs[seg];
    const uint32_t local = i - sd.base;
    valid = local < sd.count;
    lif = sd.kind == kSegLif;
    if (valid) {
      if (lif)
        st = state_in(a.su[i], a.sg[i], sd.Vr);
      else
        st = make_float4(__uint_as_float(__ldg(a.src_mask + i)), __uint_as_float(local), 0.f, 0.f);
      s_od[threadIdx.x] = __ldg(a.outdeg + i);
      r0 = __ldg(a.push_row + i);
      r1 = __ldg(a.push_row + i + 1);
    }
  }
  // Shards: a sharded cell pushes only its delay-1 and delay-2 synapses (r1
  // becomes its split point); the rest of its row is cut into shards dealt to
  // blocks, which push a shard in the step after the cell's spike (two steps
  // after it in the late-push timeline), reading the spike from the history.
  // Its delays d >= 3 count from the spike's ring slot, so the targets are
  // still ahead of the updates that read them.
  // This block's n_sh shards go first into shared memory while they fit.
  const bool sharded = a.n_shards != 0 && gridDim.x == a.shard_grid;
  uint32_t n_sh = 0;
  if (sharded) {
    if (valid) r1 = __ldg(a.push_split + i);
    const uint32_t h0 = __ldg(a.shard_off + blockIdx.x);
    n_sh = __ldg(a.shard_off + blockIdx.x + 1) - h0;
    if (threadIdx.x == 0) {
      const uint32_t cap = a.row_smem / (uint32_t)sizeof(uint2);
      uint32_t used = 0;
      for (uint32_t j = 0; j < n_sh; ++j) {
        const uint4 h = a.shards[h0 + j];
        const bool in = h.z <= cap - used;
        s_sh[j] = make_uint4(h.x, in ? used : h.y, (h.z << 23) | (in ? 3u : 2u), h.y);
        if (in) used += h.z;
      }
      s_shtot = used;
    }
    __syncthreads();
    for (uint32_t j = wib; j < n_sh; j += kPersistBlock / 32) {
      const uint4 h = s_sh[j];
      if (h.z & 1u)
        for (uint32_t k = lane; k < (h.z >> 23); k += 32)
          s_rows[h.y + k] = make_uint2(__ldg(a.push_syn + h.w + k),
                                       (uint32_t)__float2int_rn(load_weight<BF16>(a.push_w, h.w + k)));
    }
  }
  // Input cells: the stimulus decision of the coming step, drawn ahead (it
  // depends only on the step index) -- for later steps while the previous
  // grid barrier completes.
  const bool stim = valid && !lif && __float_as_uint(st.x) != 0u;
  // The barrier is polled from the highest warp without stimulated cells, so
  // the poll starts as soon as the block has arrived.
  __shared__ uint32_t s_poller;
  if (threadIdx.x == 0) s_poller = 0;
  __syncthreads();  // also publishes s_seg / s_src
  bool next_in = stim && input_fire(a, srcs, segs[seg], __float_as_uint(st.y), __float_as_uint(st.x), t0);
  const bool warp_stim = __any_sync(kFull, stim);
  if (lane == 0 && !warp_stim) atomicMax(&s_poller, threadIdx.x);
  // Push rows into shared memory: sb = the row's offset there, or kNoRow.
  // Rows of at least kLongRow synapses are placed first (a spike of such a
  // cell is the most work to push), then the others, each in word order.
  constexpr uint32_t kNoRow = 0xFFFFFFFFu;
  constexpr uint32_t kLongRow = 128;
  uint32_t sb = kNoRow;
  const uint32_t len = r1 - r0;
  if (a.row_smem) {
    const uint32_t cap = a.row_smem / (uint32_t)sizeof(uint2);
    uint32_t used = sharded ? s_shtot : 0u;
    for (uint32_t pass = 0; pass < 2; ++pass) {
      const uint32_t lp = (len >= kLongRow) == (pass == 0) ? len : 0u;
      uint32_t incl = lp;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(kFull, incl, o);
        if (lane >= (uint32_t)o) incl += v;
      }
      __syncthreads();  // s_wsum's previous readers are done
      if (lane == 31) s_wsum[wib] = incl;
      __syncthreads();
      if (wib == 0) {
        uint32_t x = s_wsum[lane], xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t v = __shfl_up_sync(kFull, xi, o);
          if (lane >= (uint32_t)o) xi += v;
        }
        s_wsum[lane] = xi - x;
        if (lane == 31) s_ptot = xi;
      }
      __syncthreads();
      const uint32_t base = used + s_wsum[wib] + incl - lp;
      if (lp && base <= cap && lp <= cap - base) sb = base;
      used += s_ptot;
    }
    uint32_t todo = __ballot_sync(kFull, sb != kNoRow);
    while (todo) {
      const int src = __ffs(todo) - 1;
      todo &= todo - 1;
      const uint32_t q0 = __shfl_sync(kFull, r0, src), n = __shfl_sync(kFull, len, src);
      const uint32_t b0 = __shfl_sync(kFull, sb, src);
      for (uint32_t k = lane; k < n; k += 32)
        s_rows[b0 + k] = make_uint2(__ldg(a.push_syn + q0 + k),
                                    (uint32_t)__float2int_rn(load_weight<BF16>(a.push_w, q0 + k)));
    }
  }
  // From here a row is (qb, rl): its first synapse in shared or global
  // memory and its length, with bit 31 set when it is in shared memory.
  const uint32_t qb = sb != kNoRow ? sb : r0;
  const uint32_t rl = len | (sb != kNoRow ? 0x80000000u : 0u);
  constexpr uint32_t clog = ILOG, chunk = 1u << ILOG;  // push-item width
  unsigned long long target = 0;
  uint32_t walked = 0;
  bool aborted = false;
  if (threadIdx.x == 0) s_n[0] = s_n[1] = 0;
  __syncthreads();
  // off / nit: the lane's first item in the block's list and its item count
  // (a warp delivers its own items past the list's capacity).
  uint32_t off = 0, nit = 0;
  // Spike bookkeeping of this warp's word for the spikes of step px.t (chunk
  // row `rel`): history and summary bits, per-segment count, events, raster
  // entries, and the spiking cells' rows cut into chunk-synapse items
  // in the block's list of parity `par`.
  auto publish = [&](bool fired, const StepIdx& px, uint32_t rel, uint32_t par) {
    off = 0;
    nit = 0;
    const uint32_t ballot = __ballot_sync(kFull, fired);
    if (lane == 0) put_hist(a, px, w, ballot);
    if (!ballot) return;
    const uint32_t n = __popc(ballot);
    const uint32_t rank = __popc(ballot & ((1u << lane) - 1u));
    const uint32_t ev = __reduce_add_sync(kFull, fired ? s_od[threadIdx.x] : 0u);
    nit = fired ? ((rl & 0x7FFFFFFFu) + chunk - 1) >> clog : 0u;
    uint32_t incl = nit;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(kFull, incl, o);
      if (lane >= (uint32_t)o) incl += v;
    }
    const uint32_t tot = __shfl_sync(kFull, incl, 31);
    uint32_t roff = 0;
    if (lane == 0) {
      if (tot) off = atomicAdd(&s_n[par], tot);
      atomicAdd(&a.counts[(size_t)rel * a.n_segs + seg], n);
      if (ev) atomicAdd(&ctl->events, (unsigned long long)ev);
      if (a.raster_cap) roff = atomicAdd(&ctl->raster_count, n);
    }
    off = __shfl_sync(kFull, off, 0) + incl - nit;
    for (uint32_t k = 0; k < nit && off + k < kBlockItems; ++k) {
      const uint32_t q = k << clog;
      s_items[off + k] = make_uint2(qb + q, (min(chunk, (rl & 0x7FFFFFFFu) - q) << 23) |
                                                (rl >> 31));
    }
    if (a.raster_cap) {
      roff = __shfl_sync(kFull, roff, 0);
      if (fired) {
        if (roff + rank < a.raster_cap)
          a.raster[roff + rank] = raster_record(i, rel);
        else
          atomicOr(&ctl->error, kErrRasterOverflow);
      }
    }
  };
  // A spiking shard (its cell's bit set in the history word sh_w) becomes
  // chunk-synapse items of parity par; returns the first item past the
  // list's capacity, which this thread's warp pushes itself (kNoRow: none).
  auto shard_items = [&](bool ck, uint32_t sh_w, uint32_t par) -> uint32_t {
    uint32_t from = kNoRow;
    if (ck) {
      const uint4 h = s_sh[threadIdx.x];
      if ((sh_w >> (h.x & 31u)) & 1u) {
        const uint32_t sl = h.z >> 23, ni = (sl + chunk - 1) >> clog;
        const uint32_t o = atomicAdd(&s_n[par], ni);
        for (uint32_t k = 0; k < ni && o + k < kBlockItems; ++k)
          s_items[o + k] = make_uint2(h.y + (k << clog),
                                      (min(chunk, sl - (k << clog)) << 23) | (h.z & 3u));
        if (o + ni > kBlockItems) from = o < kBlockItems ? kBlockItems - o : 0u;
      }
    }
    return from;
  };
  // The block's items of parity par, then the items past the list's
  // capacity; own rows count their delays from ring slot `own`, shards from
  // ring slot `shard` (their spike's step).
  // nw: the warps that deliver (the first nw of the block; fewer than all of
  // them meet on block barrier 1 instead of 0).
  auto deliver = [&](uint32_t par, uint32_t own, uint32_t shard, uint32_t sh_from,
                     uint32_t nw = kPersistBlock / 32) {
    if (nw == kPersistBlock / 32) __syncthreads(); else bar_sync_first(nw * 32u);
    const uint32_t n_items = min(s_n[par], kBlockItems);
    // The other parity's count was last read before this block barrier.
    if (threadIdx.x == 0) s_n[par ^ 1u] = 0;
    for (uint32_t u = wib; u < n_items; u += nw)
      walked += push_any<BF16>(a, s_rows, s_items[u], own, shard);
    uint32_t spill = __ballot_sync(kFull, off + nit > kBlockItems);
    while (spill) {
      const int src = __ffs(spill) - 1;
      spill &= spill - 1;
      const uint32_t o = __shfl_sync(kFull, off, src), c = __shfl_sync(kFull, nit, src);
      const uint32_t b0 = __shfl_sync(kFull, qb, src), bl = __shfl_sync(kFull, rl, src);
      for (uint32_t k = o < kBlockItems ? kBlockItems - o : 0; k < c; ++k) {
        const uint32_t q = k << clog;
        const uint2 it = make_uint2(b0 + q, (min(chunk, (bl & 0x7FFFFFFFu) - q) << 23) | (bl >> 31));
        walked += push_any<BF16>(a, s_rows, it, own, shard);
      }
    }
    if (n_sh) {
      uint32_t sp = __ballot_sync(kFull, sh_from != kNoRow);
      while (sp) {
        const int src = __ffs(sp) - 1;
        sp &= sp - 1;
        const uint4 h = s_sh[wib * 32u + src];
        const uint32_t sl = h.z >> 23;
        for (uint32_t q = __shfl_sync(kFull, sh_from, src) << clog; q < sl; q += chunk)
          walked += push_any<BF16>(
              a, s_rows, make_uint2(h.y + q, (min(chunk, sl - q) << 23) | (h.z & 3u)), own,
              shard);
      }
    }
  };
  // The shards of the spikes of step ix.t - 1 (ix has advanced past that
  // step): the epilogue of the timelines that push shards a step late.
  auto last_shards = [&]() {
    const uint32_t prev = ix.slot == 0u ? a.ring_slots - 1u : ix.slot - 1u;
    bool hit = false;
    if (threadIdx.x < n_sh) {
      const uint32_t c = s_sh[threadIdx.x].x;
      hit = (__ldcg(hist_base(a, ix.hrow) + a.n_words + (c >> 5)) >> (c & 31u)) & 1u;
    }
    uint32_t sp = __ballot_sync(kFull, hit);
    while (sp) {
      const int src = __ffs(sp) - 1;
      sp &= sp - 1;
      const uint4 h = s_sh[wib * 32u + src];
      walked += push_any<BF16>(a, s_rows, make_uint2(h.y, h.z), ix.slot, prev);
    }
  };
  if (TL == 0) {
    // Step t: update (ring slot t), spikes of t, their pushes and the shards
    // of step t - 1's spikes; one grid barrier.
    for (uint32_t s = 0; s < n_steps; ++s) {
      ix.t = t0 + s;
      ix.rel = s;
      const uint32_t par = s & 1u;
      clear_next_summary(a, ix, blockIdx.x * kPersistBlock + threadIdx.x, gridDim.x * kPersistBlock);
      // Shards of the previous step's spikes (none at a launch's first step:
      // each launch pushes its last step's shards itself, after the loop).
      const bool sh_ck = s > 0 && threadIdx.x < n_sh;
      const uint32_t sh_w =
          sh_ck ? __ldcg(hist_base(a, ix.hrow) + a.n_words + (s_sh[threadIdx.x].x >> 5)) : 0u;
      off = nit = 0;
      if (has) {
        const bool fired = lif ? cell_fire(a, segs[seg], i, 0u, valid, st, 0u, ix) : next_in;
        publish(fired, ix, s, par);
      }
      const uint32_t sh_from = shard_items(sh_ck, sh_w, par);
      deliver(par, ix.slot, ix.slot == 0u ? a.ring_slots - 1u : ix.slot - 1u, sh_from);
      grid_arrive(a, target);
      if (stim && s + 1 < n_steps)
        next_in = input_fire(a, srcs, segs[seg], __float_as_uint(st.y), __float_as_uint(st.x), ix.t + 1);
      if (!grid_wait(a, target, s_poller)) {
        aborted = true;
        break;
      }
      ix_advance(a, ix);
    }
    // The shards of the last step's spikes (ix has advanced past that step).
    if (!aborted && n_sh && n_steps) last_shards();
  } else if (TL == 1) {
    // Late-push timeline (one substep per step).  A cell's spike of step t + 1
    // is decided by its potential after the update of step t (the spike test
    // reads the potential before the step's integration), so step t updates
    // with ring slot t and publishes the spikes of t + 1, whose pushes target
    // slots t + 2 and later.  Those pushes are first read after the barrier of
    // step t + 1, so a block arrives at step t's barrier as soon as its cells
    // are updated, and only then makes the step's writes -- the clears of the
    // slot it consumed, the history words, counts and pushes of the new
    // spikes, the shards of step t - 1's spikes (delays >= 3) -- while the
    // other blocks arrive: the next arrival's release carries them.
    //   Slot t + 1 is complete at step t + 1's start: own pushes into it come
    // from steps <= t - 1, shards from steps <= t - 1 as well (a shard reads
    // the spike of step T in the history row written in step T - 1 and pushes
    // in step T + 1).  A clear made after step t's arrival is ordered before
    // the pushes of step t + 2 and later only; with max_delay + 3 ring slots
    // no push of step t + 1 targets slot t again.  A prologue publishes and
    // pushes the spikes of the launch's first step; the last step publishes
    // nothing, so a launch ends in the same state as with the other timelines.
    //   A warp 31 without a word of its own arrives and polls while the other
    // 31 warps make the step's writes (they meet on block barrier 1), so the
    // arrival's release stalls no warp with work; otherwise thread 0 arrives
    // and the block's poller polls after the writes.
    int2* ring2 = reinterpret_cast<int2*>(a.ring);
    const bool rd = has && lif && valid;
    const bool sync_idle = 31u * gridDim.x + blockIdx.x >= a.n_upd_words;  // block-uniform
    const uint32_t nw = sync_idle ? kPersistBlock / 32 - 1u : kPersistBlock / 32;
    __shared__ int s_ok1[2];
    bool in_next = false;  // input spike of step t + 1, drawn a step ahead
    if (n_steps) {
      if (stim && n_steps > 1)
        in_next = input_fire(a, srcs, segs[seg], __float_as_uint(st.y), __float_as_uint(st.x), t0 + 1);
      ix.rel = 0;
      clear_next_summary(a, ix, blockIdx.x * kPersistBlock + threadIdx.x, gridDim.x * kPersistBlock);
      off = nit = 0;
      if (has) publish(valid && (lif ? st.x > segs[seg].Vth : next_in), ix, 0u, 0u);
      deliver(0u, ix.slot, ix.slot, kNoRow);
      grid_arrive(a, target);
      aborted = !grid_wait(a, target, s_poller);
    }
    for (uint32_t s = 0; s < n_steps && !aborted; ++s) {
      const bool more = s + 1u < n_steps;
      int2 acc = make_int2(0, 0);
      if (rd) acc = __ldcg(ring2 + (ix.roff + i));
      const uint32_t consumed = ix.roff;
      // Shards of step t - 1's spikes (none at a launch's first step: the
      // previous launch pushed them after its loop).
      const bool sh_ck = s > 0 && threadIdx.x < n_sh;
      const uint32_t sh_w =
          sh_ck ? __ldcg(hist_base(a, ix.hrow) + a.n_words + (s_sh[threadIdx.x].x >> 5)) : 0u;
      const uint32_t shard_slot = ix.slot == 0u ? a.ring_slots - 1u : ix.slot - 1u;
      // From here on ix is step t + 1, whose spikes this step publishes.
      ix.t += 1ull;
      ix.rel = s + 1u;
      ix_advance(a, ix);
      clear_next_summary(a, ix, blockIdx.x * kPersistBlock + threadIdx.x,
                         gridDim.x * kPersistBlock);  // the row of step t + 2
      bool fired = false;
      if (has) {
        if (lif) {
          const LifK k = lif_k(segs[seg]);
          if (rd) lif_update<1>(k, 1, st, acc);
          fired = valid && st.x > k.Vth;
        } else {
          fired = in_next;
        }
      }
      __syncthreads();  // the block's updates (and the previous step's writes) are done
      target += gridDim.x;
      if (sync_idle && wib == 31u) {
        if (lane == 0) {
          asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(a.bar) : "memory");
          s_ok1[s & 1u] = poll_arrivals(a, target);
        }
        __syncwarp();
      } else {
        if (!sync_idle && threadIdx.x == 0)
          asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(a.bar) : "memory");
        if (rd && (acc.x | acc.y)) __stcg(ring2 + (consumed + i), make_int2(0, 0));
        const uint32_t par = (s + 1u) & 1u;
        off = nit = 0;
        if (has && more) publish(fired, ix, s + 1u, par);
        const uint32_t sh_from = shard_items(sh_ck, sh_w, par);
        deliver(par, ix.slot, shard_slot, sh_from, nw);
        if (stim && s + 2u < n_steps)
          in_next = input_fire(a, srcs, segs[seg], __float_as_uint(st.y), __float_as_uint(st.x), ix.t + 1ull);
        if (!sync_idle && threadIdx.x == s_poller) s_ok1[s & 1u] = poll_arrivals(a, target);
      }
      __syncthreads();
      if (!s_ok1[s & 1u]) {
        aborted = true;
        break;
      }
    }
    // The shards of the last step's spikes (ix has advanced past that step).
    if (!aborted && n_sh && n_steps) last_shards();
  } else {
    // Late-push timeline with a split grid barrier (one substep per step).
    // The steps' work and data as in the timeline above, but every write of
    // step t is first read in step t + 2, so the barrier is split: at the top
    // of step t + 1, after the block barrier that ends step t, warp 31 fences
    // the block's writes of step t and arrives; the block waits for the other
    // blocks' arrivals only at the end of step t + 1, before step t + 2 reads
    // slot t + 2.  Arrival, fence and barrier latency overlap a step's work,
    // and blocks run at most one step apart, which adds to the timeline above:
    //   * a history row is rewritten hist_rows steps later: with shards the
    //     handle keeps at least 4 rows, so that no block rewrites a row before
    //     a block one step behind has read it for its shards;
    //   * warp 31 clears the summary row of step t + 2 at the top of step t,
    //     before its fence; its bits are set in step t + 1;
    //   * the raster records of neighbouring steps may interleave (each
    //     record carries its step mod 4).
    // A warp 31 without a word of its own polls right after arriving while
    // the other 31 warps work (they meet on block barrier 1); one with a word
    // works like the others and the block's poller polls at the end.
    int2* ring2 = reinterpret_cast<int2*>(a.ring);
    const bool rd = has && lif && valid;
    const bool sync_idle = 31u * gridDim.x + blockIdx.x >= a.n_upd_words;  // block-uniform
    const uint32_t nw = sync_idle ? kPersistBlock / 32 - 1u : kPersistBlock / 32;
    __shared__ int s_ok[2];
    bool in_next = false;  // input spike of step t + 1, drawn a step ahead
    if (n_steps) {
      // Prologue: the spikes of the launch's first step, published and pushed
      // (fenced with the first arrival, read from step t0 + 1 on).
      if (stim && n_steps > 1)
        in_next = input_fire(a, srcs, segs[seg], __float_as_uint(st.y), __float_as_uint(st.x), t0 + 1);
      ix.rel = 0;
      clear_next_summary(a, ix, blockIdx.x * kPersistBlock + threadIdx.x, gridDim.x * kPersistBlock);
      off = nit = 0;
      if (has) publish(valid && (lif ? st.x > segs[seg].Vth : next_in), ix, 0u, 0u);
      deliver(0u, ix.slot, ix.slot, kNoRow);
      __syncthreads();
    }
    for (uint32_t s = 0; s < n_steps; ++s) {
      const bool more = s + 1u < n_steps;
      target += gridDim.x;
      if (wib == 31u) {
        const uint32_t row = (ix.srow + 2u) % (a.hist_rows + 1u);  // summary row of step t + 2
        for (uint32_t j = blockIdx.x * 32u + lane; j < a.n_swords; j += gridDim.x * 32u)
          __stcg(a.hsum + (size_t)row * a.n_swords + j, 0u);
        __syncwarp();
        if (lane == 0) {
          grid_arrive_fenced(a);
          if (sync_idle) s_ok[s & 1u] = poll_arrivals(a, target);
        }
        __syncwarp();
      }
      if (!sync_idle || wib != 31u) {
        int2 acc = make_int2(0, 0);
        if (rd) acc = __ldcg(ring2 + (ix.roff + i));
        const uint32_t consumed = ix.roff;
        // Shards of step t - 1's spikes (none at a launch's first step: the
        // previous launch pushed them after its loop).
        const bool sh_ck = s > 0 && threadIdx.x < n_sh;
        const uint32_t sh_w =
            sh_ck ? __ldcg(hist_base(a, ix.hrow) + a.n_words + (s_sh[threadIdx.x].x >> 5)) : 0u;
        const uint32_t shard_slot = ix.slot == 0u ? a.ring_slots - 1u : ix.slot - 1u;
        // From here on ix is step t + 1, whose spikes this step publishes.
        ix.t += 1ull;
        ix.rel = s + 1u;
        ix_advance(a, ix);
        bool fired = false;
        if (has) {
          if (lif) {
            const LifK k = lif_k(segs[seg]);
            if (rd) lif_update<1>(k, 1, st, acc);
            fired = valid && st.x > k.Vth;
          } else {
            fired = in_next;
          }
        }
        if (rd && (acc.x | acc.y)) __stcg(ring2 + (consumed + i), make_int2(0, 0));
        const uint32_t par = (s + 1u) & 1u;
        off = nit = 0;
        if (has && more) publish(fired, ix, s + 1u, par);
        const uint32_t sh_from = shard_items(sh_ck, sh_w, par);
        deliver(par, ix.slot, shard_slot, sh_from, nw);
        if (stim && s + 2u < n_steps)
          in_next = input_fire(a, srcs, segs[seg], __float_as_uint(st.y), __float_as_uint(st.x), ix.t + 1ull);
        if (!sync_idle && threadIdx.x == s_poller) s_ok[s & 1u] = poll_arrivals(a, target);
      } else {
        ix.t += 1ull;
        ix.rel = s + 1u;
        ix_advance(a, ix);
      }
      __syncthreads();  // ends the step: the next arrival fences its writes
      if (!s_ok[s & 1u]) {
        aborted = true;
        break;
      }
    }
    // The shards of the last step's spikes (ix has advanced past that step).
    if (!aborted && n_sh && n_steps) last_shards();
  }
  if (valid && lif) state_out(a, i, st);
  if (a.raster_cap && blockIdx.x == 0) raster_offsets_from_counts(a, n_steps, s_wsum);
  if (__ldcg(&ctl->error) & kErrBarrierTimeout) return;
  if (lane == 0 && walked) atomicAdd(&ctl->delivered, (unsigned long long)walked);
  if (leader) {
    ctl->step = t0 + n_steps;
    ctl->ring_slot = ix.slot;
    ctl->hist_row = ix.hrow;
    ctl->t_rel = n_steps;
  }
}

}  // namespace

cudaError_t launch_chunk_begin(const StepArgs& a, cudaStream_t s) {
  k_chunk_begin<<<1, 1, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_update(const StepArgs& a, cudaStream_t s) {
  if (!a.n_upd_words) return cudaSuccess;
  k_update<<<(a.n_words + kBlock / 32 - 1) / (kBlock / 32), kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_deliver(const StepArgs& a, int blocks, cudaStream_t s) {
  if (a.bf16)
    k_deliver<true><<<blocks, kBlock, 0, s>>>(a);
  else
    k_deliver<false><<<blocks, kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

size_t pull_sum_bytes(const StepArgs& a) { return ((size_t)a.hist_rows * a.n_swords + 1) * 4; }
size_t seg_smem_bytes(const StepArgs& a) { return seg_smem_bytes_dev(a); }

static size_t pull_smem_bytes(const StepArgs& a) { return a.pull_sum ? pull_sum_bytes(a) : 0; }

cudaError_t launch_pull(const StepArgs& a, int blocks, cudaStream_t s) {
  if (!a.n_pull_units) return cudaSuccess;
  if (a.pull_sum == 2u) {
    const size_t smem = pull_sum_bytes(a);
    if (a.bf16) k_pull_vec<true><<<blocks, kPullBlock, smem, s>>>(a);
    else k_pull_vec<false><<<blocks, kPullBlock, smem, s>>>(a);
    return cudaGetLastError();
  }
  const size_t smem = pull_smem_bytes(a);
  if (a.bf16) {
    if (a.pull_sum) k_pull<true, true><<<blocks, kPullBlock, smem, s>>>(a);
    else k_pull<true, false><<<blocks, kPullBlock, smem, s>>>(a);
  } else {
    if (a.pull_sum) k_pull<false, true><<<blocks, kPullBlock, smem, s>>>(a);
    else k_pull<false, false><<<blocks, kPullBlock, smem, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_stdp(const StepArgs& a, int blocks, cudaStream_t s, bool early) {
  if (!a.n_stdp_units) return cudaSuccess;
  if (a.bf16) {
    if (early) k_stdp<true, true><<<blocks, kBlock, 0, s>>>(a);
    else k_stdp<true, false><<<blocks, kBlock, 0, s>>>(a);
  } else {
    if (early) k_stdp<false, true><<<blocks, kBlock, 0, s>>>(a);
    else k_stdp<false, false><<<blocks, kBlock, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_plast_reset(const StepArgs& a, int blocks, cudaStream_t s) {
  if (!a.n_stdp_units) return cudaSuccess;
  if (a.bf16)
    k_plast_reset<true><<<blocks, kBlock, 0, s>>>(a);
  else
    k_plast_reset<false><<<blocks, kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t pull_setup() {
  const int mx = (int)kPullSumMax;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_pull_vec<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_pull_vec<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;

  if ((e = cudaFuncSetAttribute(k_pull<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_pull<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_pull<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_pull<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  // The persistent kernels stage the same summary rows before their deliveries.
  if ((e = cudaFuncSetAttribute(k_persistent<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_persistent<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_persistent<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_persistent<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_persistent<true, true, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_persistent<false, true, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx))) return e;
  if ((e = cudaFuncSetAttribute(k_persistent_resident<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx)))
    return e;
  return cudaFuncSetAttribute(k_persistent_resident<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

int pull_blocks_per_sm(const StepArgs& a) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_pull<true, true>, kPullBlock, pull_smem_bytes(a));
  return n > 0 ? n : 1;
}

cudaError_t launch_chunk_end(const StepArgs& a, cudaStream_t s) {
  if (!a.n_segs) return cudaSuccess;
  k_chunk_end<<<a.n_segs, kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

// The fused kernel's forms: [BF16][0: spikes in their own step, 64-synapse
// items; 1, 2: late-push timeline, 3, 4: late push with the split barrier,
// each with items of 64 and 128 synapses].
#define SGB_FUSED_FORMS(B)                                                                  \
  (const void*)k_persistent_fused<B, 0, 6>, (const void*)k_persistent_fused<B, 1, 6>,        \
      (const void*)k_persistent_fused<B, 1, 7>, (const void*)k_persistent_fused<B, 2, 6>,    \
      (const void*)k_persistent_fused<B, 2, 7>
constexpr uint32_t kFusedForms = 5;
static const void* const kFusedKernels[] = {SGB_FUSED_FORMS(false), SGB_FUSED_FORMS(true)};
#undef SGB_FUSED_FORMS

// The timeline and item width the fused kernel runs with for these arguments.
uint32_t fused_timeline(const StepArgs& a) { return a.substeps == 1 ? std::min(a.ahead, 2u) : 0u; }
uint32_t fused_item_log2(const StepArgs& a) {
  return fused_timeline(a) ? (a.item_log2 >= 7 ? 7u : 6u) : 6u;
}

static const void* fused_kernel(const StepArgs& a) {
  const uint32_t tl = fused_timeline(a);
  const uint32_t form = tl ? 2u * tl - 1u + (fused_item_log2(a) - 6u) : 0u;
  return kFusedKernels[(a.bf16 ? kFusedForms : 0u) + form];
}

static int fused_blocks_per_sm() {
  int n = 1 << 20;
  for (const void* fn : kFusedKernels) {
    int f = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, fn, kPersistBlock, 0);
    n = f < n ? f : n;
  }
  return n;
}

int persistent_blocks_per_sm(bool bf16) {
  int n = 0, m = 0;
  int f = 0;
  int o = 0;
  if (bf16) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_persistent<true, true>, kPersistBlock, 0);
    int q = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, k_persistent<true, true, 2>, kPersistBlock, 0);
    o = o < q ? o : q;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<true, false>, kPersistBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_persistent_resident<true>, kPersistBlock, 0);
    f = fused_blocks_per_sm();
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_persistent<false, true>, kPersistBlock, 0);
    int q = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, k_persistent<false, true, 2>, kPersistBlock, 0);
    o = o < q ? o : q;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<false, false>, kPersistBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_persistent_resident<false>, kPersistBlock, 0);
    f = fused_blocks_per_sm();
  }
  n = n < m ? n : m;
  n = n < o ? n : o;
  return n < f ? n : f;
}

// The general kernel's one-barrier form: no dense pulls, no plastic rule
// that reads the step's own spikes.
bool general_one_barrier(const StepArgs& a) {
  return a.n_pull_units == 0 && (a.n_plast == 0 || a.stdp_early);
}

int persistent_kernel_kind(const StepArgs& a, int blocks) {
  const bool resident = (uint64_t)a.n_upd_words * 32u <= (uint64_t)blocks * kPersistBlock;
  if (!resident) return SGB_KERNEL_GENERAL;
  return a.n_pull_units == 0 ? SGB_KERNEL_FUSED : SGB_KERNEL_RESIDENT;
}

cudaError_t launch_persistent(const StepArgs& a, uint32_t n_steps, int blocks, cudaStream_t s) {
  StepArgs args = a;
  uint32_t n = n_steps;
  void* params[] = {&args, &n};
  const int kind = persistent_kernel_kind(a, blocks);
  const bool resident = kind != SGB_KERNEL_GENERAL;
  const bool fused = kind == SGB_KERNEL_FUSED;
  const void* fn = fused      ? fused_kernel(a)
                   : resident ? (a.bf16 ? (const void*)k_persistent_resident<true>
                                        : (const void*)k_persistent_resident<false>)
                   : general_one_barrier(a)
                       ? (a.n_plast == 0 && a.lane_cells == 2u
                              ? (a.bf16 ? (const void*)k_persistent<true, true, 2>
                                        : (const void*)k_persistent<false, true, 2>)
                              : (a.bf16 ? (const void*)k_persistent<true, true>
                                        : (const void*)k_persistent<false, true>))
                       : (a.bf16 ? (const void*)k_persistent<true, false>
                                 : (const void*)k_persistent<false, false>);
  const size_t smem = fused ? a.row_smem
                     : (a.seg_smem ? seg_smem_bytes(a) : 0) +
                           ((a.n_pull_units && a.pull_sum) ? pull_sum_bytes(a) : 0);
  return cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kPersistBlock), params, smem, s);
}

uint32_t fused_row_smem_max() {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  size_t st = 0;
  for (const void* fn : kFusedKernels) {
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, fn);
    st = fa.sharedSizeBytes > st ? fa.sharedSizeBytes : st;
  }
  return (size_t)optin > st ? (uint32_t)(((size_t)optin - st) & ~(size_t)255) : 0u;
}

cudaError_t set_fused_row_smem(uint32_t bytes) {
  for (const void* fn : kFusedKernels) {
    const cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e) return e;
  }
  return cudaSuccess;
}

}  // namespace sgb
