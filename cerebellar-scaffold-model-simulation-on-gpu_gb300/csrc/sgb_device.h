// Device-resident descriptors and kernel entry points of the step loop.
//
// HBM layout (one simulation handle, all instances concatenated):
//   cells      padded index space (a multiple of 1,024 cells): every (instance,
//              population) segment starts on a 32-cell boundary, so one warp /
//              one spike-bitmap word never straddles two segments.
//   state      SoA: su (float per cell: the potential, or while refractory the
//              refractory count as a quiet-NaN payload, the cell sitting at
//              V_reset) and sg (float2 per cell: conductances of channels 0, 1).
//   ring       int2 per cell per delay slot: fixed-point conductance
//              increments {exc, inh} arriving at a future step; D = max
//              delay + 1 slots.  Integer accumulation makes every sum exact
//              and independent of the order in which spikes are delivered.
//   history    spike bitmap rows (1 bit per cell) of the last H steps, kept
//              twice in decreasing step order, so step t - d sits d rows above
//              step t's row; plus a summary bit per 32-cell word and step.
//   items      push work of the current step (per-step and general persistent
//              kernels): for every spiking cell, its push-table row cut into
//              ranges of at most kPushChunk synapses (uint2 {first synapse,
//              length << 23 | step tag}); a delivered item is cleared;
//              double-buffered by step parity.  The fused persistent kernel
//              keeps its items, and its blocks' push rows, in shared memory.
//   push table one cell-major CSR over every projection in event-driven mode
//              (all instances), each row's delay-1 synapses first, then its
//              delay-2 synapses, then the rest: synapse
//              word = padded post index | delay << 27 | accumulator << 31, plus
//              the weight pre-multiplied by its accumulator's 2^S (exact
//              power-of-two scaling) in FP32 or BF16.
//   ELL tables per projection, post-major (dense pull): entry = (delay - 1) *
//              n_pad + padded pre index, the offset of the pre cell's spike bit
//              above the history row of the pulling step; plus the pre-scaled
//              weight.  Padding entries (H * n_pad) are skipped by value.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sgb {

constexpr int kBlock = 256;           // threads per block of the per-step kernels
constexpr int kPersistBlock = 1024;   // threads per block of the persistent kernel
constexpr uint32_t kPushChunk = 256;  // synapses per push work item (8 per lane)
// Fused persistent kernel: a cell with at least kShardMin synapses of delay
// >= 3 keeps only its delay-1 and delay-2 synapses; the rest is cut into
// shards of kPushChunk synapses that other blocks push one step later (two
// in the late-push timeline; at most kMaxShards per block).
constexpr uint32_t kShardMin = 256;
constexpr uint32_t kMaxShards = 128;
constexpr uint32_t kPullUnit = 1024;  // ELL entries per dense-pull work unit (32 per lane)
constexpr uint32_t kStdpUnit = 128;   // ELL cells per plasticity work unit (4 per lane)
constexpr int kPullBlock = 1024;             // threads per k_pull block (one per SM)
constexpr size_t kPullSumMax = 192 * 1024;  // largest spike summary k_pull stages (H rows)
constexpr uint32_t kEllColMajorMaxK = 48;  // widths up to this use the column-major layout
// Push-table synapse word: 27-bit padded post index, 4-bit delay, 1-bit accumulator.
constexpr uint32_t kPushPostBits = 27;
constexpr uint32_t kPushPostMask = (1u << kPushPostBits) - 1u;
// Raster record of the fused kernel: padded cell index (< 2^27) with the
// chunk-relative step mod 4 in bits 30-31.  Its late-push timelines let blocks
// run a step apart, so a step's records may interleave with its neighbours';
// the host picks them out of the window between steps t - 2 and t + 2.  The
// other kernels write the bare index, their steps' records in step order.
constexpr uint32_t kRasterTagShift = 30;
__host__ __device__ inline uint32_t raster_record(uint32_t cell, uint32_t rel) {
  return cell | ((rel & 3u) << kRasterTagShift);
}
// Grid-barrier spin limit (iterations of ~64 ns sleeps): ~1 s, then the
// kernel records kErrBarrierTimeout and returns.
constexpr unsigned long long kBarrierTimeoutNs = 1000000000ull;  // grid-barrier wait limit (1 s)

enum SegKind : uint32_t { kSegLif = 0, kSegInput = 1 };

// 16-byte groups: the header and the four groups of LIF constants from El to
// sel are fetched with vector loads.
struct alignas(16) SegDev {
  uint32_t base;       // padded index of cell 0 (multiple of 32)
  uint32_t count;      // cells
  uint32_t key_base;   // Philox neuron id of cell 0 (instance-local, unpadded)
  uint32_t kind;       // SegKind
  float El, Vr, Vth, Ie;
  float neg_gL, dt_cm;            // -gL, dt/Cm
  float keep[2];                  // 1 - dt/tau_c
  float gw[2];                    // g_bar_c * w_c
  float E[2];
  float inv_scale[2];             // 2^-S of the exc / inh accumulators
  uint32_t sel[2];                // accumulator feeding channel c (0 exc, 1 inh)
  int32_t ref_steps;              // (int)(dt_ref / dt), computed in double
  int32_t substeps;
  uint64_t seed;       // instance seed
  uint32_t src_first, src_count;  // stimulus sources (INPUT segments)
  uint32_t out_first, out_count;  // outgoing projections (index list)
};
static_assert(offsetof(SegDev, El) == 16 && offsetof(SegDev, neg_gL) == 32 &&
                  offsetof(SegDev, gw) == 48 && offsetof(SegDev, inv_scale) == 64 &&
                  offsetof(SegDev, ref_steps) == 80,
              "SegDev vector groups");

struct ProjDev {
  uint32_t pre_base, post_base;   // padded segment bases
  uint32_t pre_count, post_count;
  uint32_t channel;               // accumulator (0 exc, 1 inh)
  uint32_t mode;                  // SGB_PROP_CSR / SGB_PROP_ELL
  float scale;                    // 2^S of the post segment's accumulator
  uint32_t ell_K;                 // ELL width (max in-degree)
  uint32_t ell_rowmajor;          // 0: [K][post_count], 1: [post_count][K]
  uint32_t ell_n;                 // entries (ell_K * post_count)
  const uint32_t* ell_syn;        // ell_entry words, ell_pad for padding
  const void* ell_w;              // weights x 2^S
};

struct SrcDev {
  uint32_t kind;                  // SGB_INPUT_POISSON / SGB_INPUT_PERIODIC
  uint32_t pad_;
  uint64_t thresh;                // Poisson: fire iff draw < thresh (2^32 = always)
  double cyc;                     // periodic: cycles per substep (dt * f / 1000)
  int64_t k_phase;                // periodic: phase, substeps
  int64_t win_period, win_start, win_end;  // window in substeps; end <= start: always on
};

static_assert(sizeof(SrcDev) % 8 == 0, "SrcDev copied in 8-byte units");

struct Ctl {
  unsigned long long step;        // exchange step about to be / being computed
  uint32_t ring_slot;             // step % D
  uint32_t hist_row;              // step % H
  uint32_t t_rel;                 // step index within the current chunk
  uint32_t active_count[2];       // push items reserved in buffer s & 1 at step s
  uint32_t raster_count;          // spikes recorded in the current chunk
  uint32_t error;                 // device error bits (kErr*)
  uint32_t barrier_gen;           // persistent-kernel grid barrier state
  unsigned long long barrier_arrive;
  unsigned long long events;      // synaptic events (spikes x out-degree) since reset
  unsigned long long delivered;   // synapses walked by the CSR push since reset
  unsigned long long pulled;      // dense-pull entries whose pre cell spiked, since reset
  unsigned long long plast_updates;  // plastic synapses updated (dw computed), since reset
};

constexpr uint32_t kErrRasterOverflow = 1u;
constexpr uint32_t kErrBarrierTimeout = 2u;

// kPullUnit consecutive entries [o0, o0 + kPullUnit) of one projection's ELL.
struct PullUnit { uint32_t proj, o0; };

// One plastic projection (STDP).  Per ELL cell: the plasticity value and the
// weight it scales (w x 2^S, FP32); per post cell: where its teacher's spike
// sits above the step's history base (~0u: none).
struct PlastDev {
  uint32_t proj;                  // index into projs
  uint32_t rule;                  // SGB_STDP_HEBB / SGB_STDP_TEACHER
  uint32_t window;                // pairing window (steps)
  uint32_t recent_ok;             // max delay + window <= 64: use the spike registers
  float a0, a1_i, a1_j, a2_ji, v_max, pad2_;
  float* val;
  const float* w0;
  const uint32_t* teacher;
  void* w_table;                  // the projection's ELL weights, rewritten each step
};

// Everything a step kernel needs, passed by value.
struct StepArgs {
  Ctl* ctl;
  const SegDev* segs;
  const ProjDev* projs;
  const SrcDev* srcs;
  const uint32_t* out_list;       // projection ids per segment (CSR by segment)
  const uint16_t* seg_of_word;    // segment of each 32-cell word
  const uint32_t* src_mask;       // per cell: bit s = covered by source s of its segment
  const uint32_t* outdeg;         // per cell: synapses leaving it (all projections)
  const uint32_t* upd_words;      // 32-cell words holding cells (padding words skipped)
  const uint32_t* push_row;       // [n_pad + 1] push-table row offsets
  const uint32_t* push_syn;
  const void* push_w;
  const PullUnit* pull_units;
  const PlastDev* plast;          // [n_plast]
  const PullUnit* stdp_units;     // {plastic projection, first of kStdpUnit ELL cells}
  float* su;                      // potential, or the refractory count (pack_u)
  float2* sg;                     // conductances of channels 0 and 1
  int* ring;                      // int2 per cell per slot, viewed as int[2]
  uint32_t* hist;                 // [2H][n_words]: rows H-1-(t mod H) and 2H-1-(t mod H) hold step t
  unsigned long long* recent;     // [2][n_pad] per-cell spike registers (plasticity), or NULL:
                                  // the update of step t writes buffer t & 1 (bit j = step
                                  // t - j) from buffer (t - 1) & 1
  uint32_t* hsum;                 // [H + 1][n_swords]: bit w of row t mod (H + 1) = word w
                                  // of step t had a spike
  uint2* items;                   // [2][item_cap] push work ranges
  uint32_t* counts;               // [chunk_steps][n_segs]
  uint32_t* raster;               // [raster_cap] padded ids
  uint32_t* raster_off;           // [chunk_steps + 1]
  double* totals;                 // [n_segs]
  unsigned long long* bar;        // grid-barrier arrival counter (zeroed per launch)
  uint32_t n_pad, n_words, n_segs, n_projs;
  uint32_t n_srcs;                // stimulus sources (all segments)
  uint32_t ring_slots, hist_rows;
  uint32_t max_delay;             // longest synaptic delay, steps (ring_slots = max_delay + 3)
  uint32_t item_log2;             // fused persistent kernel: push items of 2^item_log2 synapses
  uint32_t ahead;                 // fused persistent kernel's timeline (one substep): 0 spikes in
                                  // their own step, 1 late push, 2 late push, split barrier
  uint32_t lane_cells;            // general persistent kernel, one-barrier form: cells per lane (1, 2)
  uint32_t n_upd_words, n_pull_units;
  uint32_t n_plast, n_stdp_units;
  uint32_t stdp_early;            // every plastic rule reads only earlier steps' spikes (Teacher)
  uint32_t seg_smem;              // general persistent kernel: segment descriptors in shared memory
  uint32_t bar_extra;             // tests only: barrier arrivals that never come
  uint32_t n_swords;              // summary words per row: ceil(n_words / 32)
  uint32_t pull_sum;              // dense pulls: 0 every entry loads its history word; 1 entries
                                  // settle on a staged spike summary; 2 as 1, the per-step
                                  // kernel loading entries 16 bytes at a time (k_pull_vec)
  uint32_t any_push;
  uint32_t raster_cap;
  uint32_t item_cap;              // items per parity buffer
  uint32_t row_smem;              // fused persistent kernel: shared-memory bytes for push rows (0: none)
  uint32_t n_shards;              // fused persistent kernel: deferred shards (0: none)
  uint32_t shard_grid;            // the grid size the shards were dealt for
  const uint32_t* push_split;     // [n_pad] end of the part of a row its owner pushes (shards on)
  const uint4* shards;            // {cell, first synapse, length, 0}, grouped by block
  const uint32_t* shard_off;      // [shard_grid + 1] each block's range of shards
  int32_t bf16;
  int32_t substeps;
};

// Launch wrappers (sgb_kernels.cu).  All return the launch status.
cudaError_t launch_chunk_begin(const StepArgs& a, cudaStream_t s);
cudaError_t launch_update(const StepArgs& a, cudaStream_t s);
// Delivery of the current step; also advances the step counter.
cudaError_t launch_deliver(const StepArgs& a, int blocks, cudaStream_t s);
cudaError_t launch_chunk_end(const StepArgs& a, cudaStream_t s);
// One cooperative launch advancing n_steps; grid = blocks (all co-resident).
cudaError_t launch_persistent(const StepArgs& a, uint32_t n_steps, int blocks, cudaStream_t s);
// Largest dynamic shared memory the fused persistent kernel can take for push
// rows, and setting it (both weight types) before launches that use it.
uint32_t fused_row_smem_max();
cudaError_t set_fused_row_smem(uint32_t bytes);
int persistent_blocks_per_sm(bool bf16);
// Dense pull (per-step driver): k_pull needs pull_setup() once per device
// before its first launch.
cudaError_t launch_pull(const StepArgs& a, int blocks, cudaStream_t s);
// STDP of the plastic projections (per-step drivers, between update and pull)
// and the reset of their values to 1.
// early: beside k_update of the same step (a.stdp_early rules), on another stream.
cudaError_t launch_stdp(const StepArgs& a, int blocks, cudaStream_t s, bool early = false);
cudaError_t launch_plast_reset(const StepArgs& a, int blocks, cudaStream_t s);
cudaError_t pull_setup();
int pull_blocks_per_sm(const StepArgs& a);
size_t pull_sum_bytes(const StepArgs& a);  // shared memory of the staged summary rows
size_t seg_smem_bytes(const StepArgs& a);  // shared memory of the segment descriptors
// Which persistent kernel launch_persistent runs for these arguments (SGB_KERNEL_*).
int persistent_kernel_kind(const StepArgs& a, int blocks);
bool general_one_barrier(const StepArgs& a);
// The fused kernel's timeline (0 spikes in their own step, 1 late push, 2 late
// push with a split barrier) and push-item width (log2) for these arguments.
uint32_t fused_timeline(const StepArgs& a);
uint32_t fused_item_log2(const StepArgs& a);  // the general kernel's one-barrier form applies

}  // namespace sgb
