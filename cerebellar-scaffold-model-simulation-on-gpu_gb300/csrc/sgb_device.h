// Device-resident descriptors and kernel entry points of the step loop.
//
// HBM layout (one simulation handle, all instances concatenated):
//   cells      padded index space: every (instance, population) segment starts
//              on a 32-cell boundary, so one warp / one spike-bitmap word
//              never straddles two segments.
//   state      float4 per cell {u, g_exc_channel0, g_channel1, refractory
//              steps left (int bits)}: one 16-byte load and store per update.
//   ring       int2 per cell per delay slot: fixed-point conductance
//              increments {exc, inh} arriving at a future step; D = max
//              delay + 1 slots.  Integer accumulation makes every sum exact
//              and independent of the order in which spikes are delivered.
//   history    spike bitmaps of the last H = max delay steps (1 bit per cell).
//   active     compacted ids of the cells that fired in the current step
//              (double-buffered by step parity).
//   tables     per projection: pre-major CSR (event-driven push) and
//              post-major ELL (dense pull), 32-bit synapse words
//              (population-local index | delay << 28) plus FP32 or BF16
//              weights.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sgb {

constexpr int kUpdateTile = 256;      // cells per update block (8 warps)
constexpr int kPullThreadTile = 128;  // posts per block of the column-major ELL pull
constexpr int kPullWarpChunk = 1024;  // synapses per warp item of the row-major ELL pull
constexpr uint32_t kEllColMajorMaxK = 48;  // widths up to this use the column-major layout

enum SegKind : uint32_t { kSegLif = 0, kSegInput = 1 };

struct SegDev {
  uint32_t base;       // padded index of cell 0 (multiple of 32)
  uint32_t count;      // cells
  uint32_t key_base;   // Philox neuron id of cell 0 (instance-local, unpadded)
  uint32_t kind;       // SegKind
  uint64_t seed;       // instance seed
  uint32_t src_first, src_count;  // stimulus sources (INPUT segments)
  uint32_t out_first, out_count;  // outgoing projections (index list)
  float El, Vr, Vth, Ie;
  float neg_gL, dt_cm;            // -gL, dt/Cm
  float keep[2];                  // 1 - dt/tau_c
  float gw[2];                    // g_bar_c * w_c
  float E[2];
  float inv_scale[2];             // 2^-S of the exc / inh accumulators
  int32_t ref_steps;              // (int)(dt_ref / dt), computed in double
  int32_t substeps;
  uint32_t sel[2];                // accumulator feeding channel c (0 exc, 1 inh)
};

struct ProjDev {
  uint32_t pre_base, post_base;   // padded segment bases
  uint32_t pre_count, post_count;
  uint32_t channel;               // accumulator (0 exc, 1 inh)
  uint32_t mode;                  // SGB_PROP_CSR / SGB_PROP_ELL
  float scale;                    // 2^S of the post segment's accumulator
  uint32_t ell_K;                 // ELL width (max in-degree)
  uint32_t ell_rowmajor;          // 0: [K][post_count], 1: [post_count][K]
  uint32_t pad_;
  const uint32_t* csr_row;        // [pre_count + 1]
  const uint32_t* csr_syn;        // post | delay << 28
  const void* csr_w;
  const uint32_t* ell_syn;        // pre | delay << 28, kEllPad for padding
  const void* ell_w;
};

struct SrcDev {
  uint32_t kind;                  // SGB_INPUT_POISSON / SGB_INPUT_PERIODIC
  uint32_t pad_;
  uint64_t thresh;                // Poisson: fire iff draw < thresh (2^32 = always)
  double cyc;                     // periodic: cycles per substep (dt * f / 1000)
  int64_t k_phase;                // periodic: phase, substeps
  int64_t win_period, win_start, win_end;  // window in substeps; end <= start: always on
};

struct Ctl {
  unsigned long long step;        // exchange step about to be / being computed
  uint32_t ring_slot;             // step % D
  uint32_t hist_row;              // step % H
  uint32_t t_rel;                 // step index within the current chunk
  uint32_t active_count[2];       // spikes of step s live in buffer s & 1
  uint32_t raster_count;          // spikes recorded in the current chunk
  uint32_t error;                 // device error bits (kErr*)
  uint32_t barrier_gen;           // persistent-kernel grid barrier state
  unsigned long long barrier_arrive;
  unsigned long long events;      // synaptic events (spikes x out-degree) since reset
  unsigned long long delivered;   // synapses walked by the CSR push since reset
};

constexpr uint32_t kErrRasterOverflow = 1u;
constexpr uint32_t kErrBarrierTimeout = 2u;

struct PullTile { uint32_t proj, post_start; };
struct PullItem { uint32_t proj, post, k0; };
struct UpdTile { uint32_t seg, start; };

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
  const UpdTile* upd_tiles;
  const PullTile* pull_tiles;
  const PullItem* pull_items;
  float4* state;
  int* ring;                      // int2 per cell per slot, viewed as int[2]
  uint32_t* hist;                 // [H][n_words]
  uint32_t* active;               // [2][n_pad]
  uint32_t* counts;               // [chunk_steps][n_segs]
  uint32_t* raster;               // [raster_cap] padded ids
  uint32_t* raster_off;           // [chunk_steps + 1]
  double* totals;                 // [n_segs]
  uint32_t n_pad, n_words, n_segs, n_projs;
  uint32_t ring_slots, hist_rows;
  uint32_t n_upd_tiles, n_pull_tiles, n_pull_items;
  uint32_t raster_cap;
  int32_t bf16;
  int32_t substeps;
};

// Launch wrappers (sgb_kernels.cu).  All return the launch status.
cudaError_t launch_chunk_begin(const StepArgs& a, cudaStream_t s);
cudaError_t launch_update(const StepArgs& a, cudaStream_t s);
cudaError_t launch_push(const StepArgs& a, int blocks, cudaStream_t s);
cudaError_t launch_pull_thread(const StepArgs& a, cudaStream_t s);
cudaError_t launch_pull_warp(const StepArgs& a, cudaStream_t s);
cudaError_t launch_advance(const StepArgs& a, cudaStream_t s);
cudaError_t launch_chunk_end(const StepArgs& a, cudaStream_t s);

}  // namespace sgb
