// Simulation handle: device layout of every instance, synapse tables, step
// drivers (CUDA graph / persistent kernel / plain launches) and host I/O.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <vector>

#include "sgb_device.h"
#include "sgb_model.h"

namespace sgb {

struct ProjTables {
  int32_t net = 0, proj = 0;
  uint32_t pre_seg = 0, post_seg = 0;
  int32_t scale_bits = 0;  // of the post segment's accumulator
  int64_t nnz = 0;
  uint32_t ell_K = 0;
  bool ell_rowmajor = false;
  size_t off_ell_syn = 0, off_ell_w = 0;  // offsets inside the ELL pool
};

// Host view of one plastic projection: the ELL cell of each synapse (in the
// projection's synapse order), for reading the values back.
struct PlastHost {
  int32_t net = 0, proj = 0;
  uint32_t k = 0;                 // index into projs
  std::vector<uint32_t> cell_of_syn;
  size_t off_val = 0, cells = 0;  // in d_plast
};

struct Sim {
  sgb_config cfg{};
  std::vector<Network> nets;
  std::vector<uint64_t> seeds;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  int sm_count = 0;

  // Layout.
  std::vector<SegDev> segs;
  std::vector<int64_t> seg_first_id;  // global unpadded id of cell 0
  std::vector<int32_t> seg_net, seg_pop;
  std::vector<int32_t> net_seg0;      // first segment of each net
  std::vector<int32_t> net_proj0;     // first projection of each net
  std::vector<ProjDev> projs;
  std::vector<ProjTables> ptab;
  std::vector<SrcDev> srcs;
  std::vector<int32_t> src_net, src_idx;
  bool pull_sum_fits = false;    // the staged spike summary fits shared memory
  uint32_t n_pad = 0, n_words = 0, ring_slots = 3, hist_rows = 1, max_delay = 1;
  int64_t n_cells = 0, n_syn = 0;
  uint32_t chunk = 1000, raster_cap = 0;
  bool bf16 = false;

  // Device memory.
  void* d_ell = nullptr;    // per-projection ELL tables
  size_t ell_bytes = 0;
  void* d_push = nullptr;   // merged push table (capacity: every synapse)
  size_t push_bytes = 0;
  void* d_misc = nullptr;   // state, ring, history, lists, descriptors
  size_t misc_bytes = 0;
  StepArgs args{};
  int deliver_blocks = 0;
  int pull_blocks = 0;        // k_pull grid (resident blocks per SM x SMs)
  size_t hist_bytes = 0;      // spike history + its summary
  int persistent_blocks = 0;
  std::vector<uint32_t> upd_words;  // host copy of args.upd_words
  int64_t n_shard_cells = 0;        // cells whose delay >= 2 synapses are sharded
  // Plasticity (STDP) of plastic projections.
  void* d_plast = nullptr;
  void* d_shard = nullptr;    // fused-kernel shards: split points, shard list, per-block offsets
  size_t off_recent = 0;      // per-cell spike registers inside d_plast
  std::vector<PlastHost> plast;
  // Per-step drivers with early plasticity rules: k_stdp runs on `side`,
  // forked from and joined back into the step's stream around k_update.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // Persisting L2 window over the cell state (su, sg).
  void* l2_base = nullptr;
  size_t l2_window = 0, l2_setaside = 0, l2_prev_limit = 0;
  float l2_hit = 0.f;
  SrcDev* h_srcs = nullptr;  // pinned staging of the source table

  // Host staging for outputs.
  uint32_t* h_counts = nullptr;
  uint32_t* h_raster = nullptr;
  uint32_t* h_raster_off = nullptr;

  std::map<uint32_t, cudaGraphExec_t> graphs;  // by chunk length
  int64_t launches = 0;

  ~Sim();
};

int sim_create(const sgb_config& cfg, sgb_net* const* nets, const uint64_t* seeds, int32_t n,
               Sim** out);
int sim_run(Sim& s, int64_t n_steps, uint32_t* counts, uint32_t* raster_ids, int64_t raster_cap,
            int64_t* raster_offsets);
int sim_reset(Sim& s, const uint64_t* seeds);
int sim_enqueue(Sim& s, int64_t n_steps);
int sim_sync(Sim& s);
int sim_set_rates(Sim& s, int32_t net, int32_t n, const float* rates);
int sim_get_state(Sim& s, float* u, float* g, int32_t* ref);
int sim_set_state(Sim& s, const float* u, const float* g, const int32_t* ref);
int sim_totals(Sim& s, double* totals);
int sim_set_mode(Sim& s, int32_t net, int32_t proj, int32_t mode);
int sim_autotune(Sim& s, int32_t n_steps, const char* cache_path);
int sim_profile(Sim& s, int32_t n_steps, double* mean_us, double* bytes, int64_t* launches);
int sim_plastic_values(Sim& s, int32_t net, int32_t proj, float* values);
int sim_checkpoint_size(const Sim& s, int64_t* bytes);
int sim_checkpoint(Sim& s, void* buf, int64_t size, bool load);
int sim_set_stream(Sim& s, cudaStream_t st);

}  // namespace sgb

// Handles behind the C ABI.
struct sgb_net {
  sgb::Network net;
};
struct sgb_sim {
  sgb::Sim* sim;
};
