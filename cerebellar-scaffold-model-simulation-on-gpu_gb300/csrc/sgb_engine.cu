// Simulation engine: builds the device layout from host networks, owns the
// device memory, and drives the step kernels (see sgb_engine.h).
//
// The reference's equivalents are Initialization (GPUScaffoldSimulation.cu:
// 132-631: population split, ELL upload, Philox state setup, streams) and
// loop_n_steps (:693-791: per-ms launches on 12 streams + a device-wide
// synchronize).  Here one handle holds any number of independent instances.
// Two drivers advance a chunk of steps: a CUDA graph of two kernels per step
// whose step index lives in device memory (so one executable graph is
// replayed for every chunk), or one persistent cooperative kernel per chunk.
#include "sgb_engine.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <numeric>
#include <string>

#include "sgb_philox.h"

namespace sgb {

#define SGB_CUDA(call)                                                                        \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return set_error(SGB_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                       __FILE__, __LINE__);                                                   \
  } while (0)

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Access-policy window of the cell state on stream st (num_bytes 0 clears it).
static cudaError_t l2_window_on(const Sim& s, cudaStream_t st, bool on) {
  cudaStreamAttrValue v;
  memset(&v, 0, sizeof v);
  v.accessPolicyWindow.base_ptr = s.l2_base;
  v.accessPolicyWindow.num_bytes = on ? s.l2_window : 0;
  v.accessPolicyWindow.hitRatio = on ? s.l2_hit : 0.f;
  v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
  v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
  return cudaStreamSetAttribute(st, cudaStreamAttributeAccessPolicyWindow, &v);
}

Sim::~Sim() {
  if (stream) cudaStreamSynchronize(stream);
  if (l2_window) {
    // Hand the set-aside back: clear the window, demote persisting lines and
    // restore the context's previous limit.
    l2_window_on(*this, stream, false);
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, l2_prev_limit);
  }
  for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
  if (d_ell) cudaFree(d_ell);
  if (d_push) cudaFree(d_push);
  if (d_misc) cudaFree(d_misc);
  if (d_plast) cudaFree(d_plast);
  if (d_shard) cudaFree(d_shard);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (side) cudaStreamDestroy(side);
  if (h_counts) cudaFreeHost(h_counts);
  if (h_raster) cudaFreeHost(h_raster);
  if (h_raster_off) cudaFreeHost(h_raster_off);
  if (h_srcs) cudaFreeHost(h_srcs);
  if (own_stream) cudaStreamDestroy(own_stream);
}

// ---------------------------------------------------------------------------
// Per-segment LIF constants, folded once in double and rounded to float.
static void fill_lif(SegDev& d, const Population& p, double dt, int substeps) {
  d.El = p.El;
  d.Vr = p.Vr;
  d.Vth = p.Vth;
  d.Ie = p.Ie;
  d.neg_gL = -p.gL;
  d.dt_cm = (float)(dt / (double)p.Cm);
  // Reference: ref_step = (int)(target.dt_ref / DT) with DT a double literal
  // (Simulation_header.cu:322).
  d.ref_steps = (int32_t)((double)p.dt_ref / dt);  // at most kRefMax (checked at create)
  d.substeps = substeps;
  for (int c = 0; c < 2; ++c) {
    if (c < p.c_num) {
      d.keep[c] = (float)(1.0 - dt / (double)p.tau[c]);
      d.gw[c] = p.gbar[c] * p.w[c];
      d.E[c] = p.E[c];
      // Channel c integrates dg_exc when E_c > E_L, else dg_inh
      // (Simulation_header.cu:347).
      d.sel[c] = p.E[c] > p.El ? 0u : 1u;
    } else {
      d.keep[c] = 0.f;
      d.gw[c] = 0.f;
      d.E[c] = 0.f;
      d.sel[c] = 0u;
    }
  }
}

static uint64_t poisson_threshold(float rate_hz, double dt_ms) {
  const double p = (double)rate_hz * dt_ms / 1000.0;
  if (!(p > 0.0)) return 0;
  if (p >= 1.0) return 1ull << 32;
  return (uint64_t)floor(p * 4294967296.0);
}

static void fill_source(SrcDev& d, const sgb_input_params& p, double dt_ms) {
  memset(&d, 0, sizeof d);
  d.kind = (uint32_t)p.kind;
  d.thresh = p.kind == SGB_INPUT_POISSON ? poisson_threshold(p.rate_hz, dt_ms) : 0;
  d.cyc = p.kind == SGB_INPUT_PERIODIC ? dt_ms * (double)p.rate_hz / 1000.0 : 0.0;
  d.k_phase = llround(p.phase_ms / dt_ms);
  d.win_period = p.win_period_ms > 0 ? llround(p.win_period_ms / dt_ms) : 0;
  d.win_start = llround(p.win_start_ms / dt_ms);
  d.win_end = llround(p.win_end_ms / dt_ms);
  if (d.win_end <= d.win_start) d.win_start = d.win_end = 0;
}

// Initial potential of a LIF cell: Vr + (Vth - Vr) * U(0,1] (InitParams,
// init_params.cu:346), U from Philox(seed; neuron, step 0, tag InitU).
static float initial_u(const Population& p, uint64_t seed, uint32_t key) {
  const U4 r = philox_draw(seed, key, 0, kTagInitU, 0);
  return fmaf(p.Vth - p.Vr, u01_open0(r.x), p.Vr);
}

// Weight as stored in a device table: the (BF16-rounded) magnitude times the
// accumulator's 2^S.  Power-of-two scaling is exact, so rint(stored) equals
// rint(w * 2^S) for the table's w.
static float scaled_weight(float w, int32_t bits, bool bf16) {
  return ldexpf(table_weight(w, bf16), bits);
}

// ---------------------------------------------------------------------------
// Post-major ELL of one projection, width = max in-degree, padding at the end
// of each row; column-major for narrow rows, row-major for wide ones (either
// way the pull streams it as flat units, so the table is padded to whole
// units).  Entries are ell_entry words (at most 2^27 padded cells).
static bool build_ell(const Projection& pr, int32_t npost, uint32_t pre_base, uint32_t n_pad,
                      uint32_t pad, bool bf16, ProjTables& t, std::vector<uint32_t>& syn,
                      std::vector<float>& wf, std::vector<uint16_t>& wh,
                      std::vector<float>* w0 = nullptr, std::vector<uint32_t>* cell_of_syn = nullptr) {
  const size_t nnz = pr.pre_idx.size();
  std::vector<uint32_t> indeg((size_t)npost, 0);
  for (size_t i = 0; i < nnz; ++i) indeg[pr.post_idx[i]]++;
  uint32_t K = 0;
  for (uint32_t v : indeg) K = std::max(K, v);
  t.ell_K = K;
  t.ell_rowmajor = K > kEllColMajorMaxK;
  const size_t cells = (size_t)K * (size_t)npost;
  if (cells >= (1ull << 32) - kPullUnit) return false;  // entry offsets are 32-bit
  syn.assign(align_up(cells, kPullUnit), pad);  // whole pull units
  if (bf16) wh.assign(cells, 0); else wf.assign(cells, 0.f);
  if (w0) w0->assign(cells, 0.f);
  if (cell_of_syn) cell_of_syn->assign(nnz, 0);
  // Each row sorted by (delay, pre, synapse): neighbouring entries then test
  // bits of one history row at nearby words.  The pulled sum is an integer,
  // so the order does not change it.
  std::vector<size_t> start((size_t)npost + 1, 0);
  for (size_t p = 0; p < (size_t)npost; ++p) start[p + 1] = start[p] + indeg[p];
  std::vector<uint32_t> order(nnz);
  {
    std::vector<size_t> fill(start.begin(), start.end() - 1);
    for (size_t i = 0; i < nnz; ++i) order[fill[pr.post_idx[i]]++] = (uint32_t)i;
  }
  const auto key = [&](uint32_t i) {
    return ((uint64_t)pr.delay[i] << 32) | (uint64_t)(uint32_t)pr.pre_idx[i];
  };
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t p = 0; p < npost; ++p)
    std::sort(order.begin() + start[p], order.begin() + start[p + 1], [&](uint32_t x, uint32_t y) {
      const uint64_t kx = key(x), ky = key(y);
      return kx != ky ? kx < ky : x < y;
    });
  for (size_t p = 0; p < (size_t)npost; ++p) {
    for (size_t j = start[p]; j < start[p + 1]; ++j) {
      const uint32_t i = order[j];
      const size_t k = j - start[p];
      const size_t q = t.ell_rowmajor ? p * K + k : k * (size_t)npost + p;
      syn[q] = ell_entry(pre_base + (uint32_t)pr.pre_idx[i], pr.delay[i], n_pad);
      const float w = scaled_weight(pr.weight[i], t.scale_bits, bf16);
      if (bf16) wh[q] = f32_to_bf16_bits(w); else wf[q] = w;
      if (w0) (*w0)[q] = ldexpf(pr.weight[i], t.scale_bits);
      if (cell_of_syn) (*cell_of_syn)[i] = (uint32_t)q;
    }
  }
  return true;
}

// Rebuilds the merged push table (every projection in CSR mode, cell-major)
// and the dense-pull work lists, uploads them, and drops captured graphs.
static int upload_modes(Sim& s) {
  StepArgs& a = s.args;
  // Push table.
  std::vector<uint32_t> row((size_t)s.n_pad + 1, 0);
  int64_t total = 0;
  for (size_t k = 0; k < s.projs.size(); ++k) {
    if (s.projs[k].mode != SGB_PROP_CSR) continue;
    const ProjTables& t = s.ptab[k];
    const Projection& pr = s.nets[t.net].projs[t.proj];
    const uint32_t pre_base = s.segs[t.pre_seg].base;
    for (uint32_t p : pr.pre_idx) row[pre_base + p + 1]++;
    total += t.nnz;
  }
  if (total > 0xFFFFFFFFll) return set_error(SGB_ERR_UNSUPPORTED, "more than 2^32 push synapses");
  for (uint32_t j = 0; j < s.n_pad; ++j) row[j + 1] += row[j];
  std::vector<uint32_t> syn((size_t)total);
  std::vector<float> wf(s.bf16 ? 0 : (size_t)total);
  std::vector<uint16_t> wh(s.bf16 ? (size_t)total : 0);
  // Each row holds its delay-1 synapses first (pass 0), then its delay-2
  // synapses (pass 1), then the others: split[c] is where the delay >= 3 part
  // of cell c's row starts.
  std::vector<uint32_t> split;
  {
    std::vector<uint32_t> fill(row.begin(), row.end() - 1);
    for (int pass = 0; pass < 3; ++pass) {
      for (size_t k = 0; k < s.projs.size(); ++k) {
        if (s.projs[k].mode != SGB_PROP_CSR) continue;
        const ProjTables& t = s.ptab[k];
        const Projection& pr = s.nets[t.net].projs[t.proj];
        const uint32_t pre_base = s.segs[t.pre_seg].base, post_base = s.segs[t.post_seg].base;
        for (size_t i = 0; i < pr.pre_idx.size(); ++i) {
          if (std::min<int>(pr.delay[i], 3) - 1 != pass) continue;
          const uint32_t q = fill[pre_base + pr.pre_idx[i]]++;
          syn[q] = (post_base + pr.post_idx[i]) | ((uint32_t)pr.delay[i] << kPushPostBits) |
                   ((uint32_t)pr.channel << 31);
          const float w = scaled_weight(pr.weight[i], t.scale_bits, s.bf16);
          if (s.bf16) wh[q] = f32_to_bf16_bits(w); else wf[q] = w;
        }
      }
      if (pass == 1) split = fill;
    }
  }
  const size_t wsz = s.bf16 ? 2 : 4;
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  SGB_CUDA(cudaMemcpy((void*)a.push_row, row.data(), row.size() * 4, cudaMemcpyHostToDevice));
  if (total) {
    SGB_CUDA(cudaMemcpy((void*)a.push_syn, syn.data(), (size_t)total * 4, cudaMemcpyHostToDevice));
    SGB_CUDA(cudaMemcpy((void*)a.push_w, s.bf16 ? (const void*)wh.data() : (const void*)wf.data(),
                        (size_t)total * wsz, cudaMemcpyHostToDevice));
  }
  a.any_push = total > 0 ? 1u : 0u;
  // Dense-pull work units.
  std::vector<PullUnit> units;
  for (uint32_t pid = 0; pid < s.projs.size(); ++pid) {
    const ProjDev& P = s.projs[pid];
    if (P.mode != SGB_PROP_ELL || P.ell_n == 0) continue;
    for (uint32_t o = 0; o < P.ell_n; o += kPullUnit) {
      units.push_back({pid, o});
      if (P.ell_n - o <= kPullUnit) break;
    }
  }
  if (!units.empty())
    SGB_CUDA(cudaMemcpy((void*)a.pull_units, units.data(), units.size() * sizeof(PullUnit), cudaMemcpyHostToDevice));
  SGB_CUDA(cudaMemcpy((void*)a.projs, s.projs.data(), s.projs.size() * sizeof(ProjDev), cudaMemcpyHostToDevice));
  a.n_pull_units = (uint32_t)units.size();
  // Fused persistent kernel.  Shards: the delay >= 3 parts of long rows
  // (longest first) are cut into kPushChunk-synapse shards dealt round-robin
  // over the blocks, so one spike's pushes spread over many SMs; a cell whose
  // shards no longer fit keeps its whole row.  Then shared memory for the
  // push rows of the block holding the most synapses (word slot ws runs in
  // block ws mod blocks; a sharded cell's own part is its delay-1 and delay-2
  // synapses).
  a.row_smem = 0;
  a.n_shards = 0;
  s.n_shard_cells = 0;
  const bool fused = total > 0 && s.persistent_blocks > 0 &&
                     persistent_kernel_kind(a, s.persistent_blocks) == SGB_KERNEL_FUSED;
  std::vector<uint32_t> own_end(row.begin() + 1, row.end());
  std::vector<std::vector<uint4>> blk_sh(fused && s.d_shard ? (size_t)s.persistent_blocks : 0);
  if (!blk_sh.empty()) {
    const uint32_t B = (uint32_t)blk_sh.size();
    std::vector<uint32_t> cand;
    for (uint32_t c = 0; c < s.n_pad; ++c)
      if (row[c + 1] - split[c] >= kShardMin) cand.push_back(c);
    std::stable_sort(cand.begin(), cand.end(), [&](uint32_t x, uint32_t y) {
      return row[x + 1] - split[x] > row[y + 1] - split[y];
    });
    uint32_t cursor = 0;
    for (uint32_t c : cand) {
      std::vector<uint32_t> picked;
      for (uint32_t q = split[c]; q < row[c + 1]; q += kPushChunk) {
        uint32_t tries = 0;
        while (tries < B && blk_sh[cursor].size() >= kMaxShards) { cursor = (cursor + 1) % B; ++tries; }
        if (tries == B) break;
        blk_sh[cursor].push_back(make_uint4(c, q, std::min(kPushChunk, row[c + 1] - q), 0u));
        picked.push_back(cursor);
        cursor = (cursor + 1) % B;
      }
      if ((uint64_t)picked.size() * kPushChunk < row[c + 1] - split[c]) {
        for (uint32_t b : picked) blk_sh[b].pop_back();
        break;
      }
      own_end[c] = split[c];
      ++s.n_shard_cells;
    }
    std::vector<uint4> flat;
    std::vector<uint32_t> off(B + 1, 0);
    for (uint32_t b = 0; b < B; ++b) {
      flat.insert(flat.end(), blk_sh[b].begin(), blk_sh[b].end());
      off[b + 1] = (uint32_t)flat.size();
    }
    char* sb = (char*)s.d_shard;
    const size_t o_sh = align_up((size_t)s.n_pad * 4, 256);
    const size_t o_off = o_sh + align_up((size_t)B * kMaxShards * sizeof(uint4), 256);
    SGB_CUDA(cudaMemcpy(sb, own_end.data(), (size_t)s.n_pad * 4, cudaMemcpyHostToDevice));
    if (!flat.empty())
      SGB_CUDA(cudaMemcpy(sb + o_sh, flat.data(), flat.size() * sizeof(uint4), cudaMemcpyHostToDevice));
    SGB_CUDA(cudaMemcpy(sb + o_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
    a.push_split = (const uint32_t*)sb;
    a.shards = (const uint4*)(sb + o_sh);
    a.shard_off = (const uint32_t*)(sb + o_off);
    a.shard_grid = B;
    a.n_shards = (uint32_t)flat.size();
  }
  if (fused) {
    std::vector<uint64_t> need((size_t)s.persistent_blocks, 0);
    for (size_t ws = 0; ws < s.upd_words.size(); ++ws) {
      const uint32_t w = s.upd_words[ws];
      for (uint32_t c = w * 32; c < w * 32 + 32; ++c) need[ws % need.size()] += own_end[c] - row[c];
    }
    for (size_t b = 0; b < blk_sh.size(); ++b)
      for (const uint4& h : blk_sh[b]) need[b] += h.z;
    const uint64_t most = *std::max_element(need.begin(), need.end()) * sizeof(uint2);
    const uint64_t bytes = std::min<uint64_t>((most + 255) & ~255ull, fused_row_smem_max());
    if (bytes >= 1024) {
      SGB_CUDA(set_fused_row_smem((uint32_t)bytes));
      a.row_smem = (uint32_t)bytes;
    }
  }
  for (auto& kv : s.graphs) cudaGraphExecDestroy(kv.second);
  s.graphs.clear();
  return SGB_OK;
}

int sim_create(const sgb_config& cfg, sgb_net* const* nets, const uint64_t* seeds, int32_t n,
               Sim** out) {
  if (!out) return set_error(SGB_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (n < 1 || !nets) return set_error(SGB_ERR_ARG, "need at least one network");
  if (!(cfg.dt_ms > 0.0)) return set_error(SGB_ERR_ARG, "dt_ms must be positive");
  if (cfg.substeps < 1 || cfg.substeps > 1024)
    return set_error(SGB_ERR_ARG, "substeps %d not in 1..1024", cfg.substeps);
  if (cfg.chunk_steps < 1 || cfg.chunk_steps > 100000)
    return set_error(SGB_ERR_ARG, "chunk_steps %d not in 1..100000", cfg.chunk_steps);
  if (cfg.weight_type != SGB_WEIGHT_FP32 && cfg.weight_type != SGB_WEIGHT_BF16)
    return set_error(SGB_ERR_ARG, "unknown weight type %d", cfg.weight_type);
  if (cfg.exec_mode < SGB_EXEC_GRAPH || cfg.exec_mode > SGB_EXEC_STREAM)
    return set_error(SGB_ERR_ARG, "unknown exec mode %d", cfg.exec_mode);
  if (cfg.default_prop != SGB_PROP_AUTO && cfg.default_prop != SGB_PROP_CSR &&
      cfg.default_prop != SGB_PROP_ELL)
    return set_error(SGB_ERR_ARG, "unknown default propagation mode %d", cfg.default_prop);
  if (cfg.blocks_per_sm < 0 || cfg.blocks_per_sm > 32)
    return set_error(SGB_ERR_ARG, "blocks_per_sm %d not in 0..32", cfg.blocks_per_sm);
  if (cfg.barrier_test_extra < 0 || cfg.barrier_test_extra > 1024)
    return set_error(SGB_ERR_ARG, "barrier_test_extra %d not in 0..1024", cfg.barrier_test_extra);
  for (int32_t i = 0; i < n; ++i)
    if (!nets[i]) return set_error(SGB_ERR_ARG, "network %d is NULL", i);

  SGB_CUDA(cudaSetDevice(cfg.device));
  std::unique_ptr<Sim> S(new Sim());
  Sim& s = *S;
  s.cfg = cfg;
  s.bf16 = cfg.weight_type == SGB_WEIGHT_BF16;
  s.chunk = (uint32_t)cfg.chunk_steps;
  for (int32_t i = 0; i < n; ++i) {
    s.nets.push_back(nets[i]->net);
    s.seeds.push_back(seeds ? seeds[i] : (uint64_t)(i + 1));
  }
  SGB_CUDA(cudaDeviceGetAttribute(&s.sm_count, cudaDevAttrMultiProcessorCount, cfg.device));
  SGB_CUDA(cudaStreamCreateWithFlags(&s.own_stream, cudaStreamNonBlocking));
  s.stream = s.own_stream;

  // ---- segments (cells of every instance, each population 32-aligned) -----
  uint64_t cursor = 0;
  int64_t first_id = 0;
  int max_delay = 1;
  std::vector<std::vector<int32_t>> net_bits(n);
  for (int32_t ni = 0; ni < n; ++ni) {
    const Network& net = s.nets[ni];
    s.net_seg0.push_back((int32_t)s.segs.size());
    uint32_t key = 0;
    accumulator_scale_bits(net, s.bf16, net_bits[ni]);
    const std::vector<int32_t>& bits = net_bits[ni];
    for (size_t pi = 0; pi < net.pops.size(); ++pi) {
      const Population& p = net.pops[pi];
      SegDev d;
      memset(&d, 0, sizeof d);
      cursor = align_up(cursor, 32);
      d.base = (uint32_t)cursor;
      d.count = (uint32_t)p.num;
      d.key_base = key;
      d.kind = p.dev_type == SGB_INPUT ? kSegInput : kSegLif;
      d.seed = s.seeds[ni];
      if (d.kind == kSegLif) {
        fill_lif(d, p, cfg.dt_ms, cfg.substeps);
        if (d.ref_steps > kRefMax)
          return set_error(SGB_ERR_RANGE, "population %zu: refractory period of %d steps exceeds %d",
                           pi, d.ref_steps, kRefMax);
      }
      d.inv_scale[0] = ldexpf(1.0f, -bits[pi * 2 + 0]);
      d.inv_scale[1] = ldexpf(1.0f, -bits[pi * 2 + 1]);
      s.segs.push_back(d);
      s.seg_first_id.push_back(first_id);
      s.seg_net.push_back(ni);
      s.seg_pop.push_back((int32_t)pi);
      cursor += (uint64_t)p.num;
      key += (uint32_t)p.num;
      first_id += p.num;
      if (cursor > kPushPostMask)
        return set_error(SGB_ERR_UNSUPPORTED, "more than 2^27 cells (with padding) in one handle");
    }
    for (const auto& pr : net.projs)
      for (uint8_t d : pr.delay) max_delay = std::max(max_delay, (int)d);
  }
  if (s.segs.size() > 65535) return set_error(SGB_ERR_UNSUPPORTED, "more than 65535 segments");
  // A multiple of 1,024 cells, so dense entries (delay - 1) * n_pad + g keep
  // the word and summary-word structure of g (see ell_entry).
  s.n_pad = (uint32_t)align_up(std::max<uint64_t>(cursor, 1024), 1024);
  if (s.n_pad > kPushPostMask + 1u)
    return set_error(SGB_ERR_UNSUPPORTED, "more than 2^27 cells (with padding) in one handle");
  s.n_words = s.n_pad / 32;
  s.n_cells = first_id;
  // Ring slots t .. t + max_delay receive increments.  Networks that may run
  // the fused kernel (at most one 32-cell word per warp of the persistent
  // grid) keep two more: its late-push timelines clear slot t after step t's
  // barrier arrival, so the clear is ordered only before the pushes of step
  // t + 2 and later, while step t + 1 pushes up to slot t + 2 + max_delay.
  // The others keep one more (the layout their kernels were measured with).
  s.max_delay = (uint32_t)max_delay;
  uint64_t upd_words_n = 0;
  for (const SegDev& d : s.segs) upd_words_n += (d.count + 31u) / 32u;
  const bool may_fuse = upd_words_n * 32u <=
                        (uint64_t)std::max(1, cfg.blocks_per_sm) * s.sm_count * kPersistBlock;
  s.ring_slots = (uint32_t)max_delay + (may_fuse ? 3u : 2u);
  // History rows: one per delay; where the fused kernel may run with shards
  // (delays >= 3) at least 4: in its split-barrier timeline a block may
  // rewrite a row up to one step before a block behind it reads that row.
  s.hist_rows = (uint32_t)(may_fuse && max_delay >= 3 ? std::max(max_delay, 4) : max_delay);
  // A plastic synapse with delay d reads its pre cell's spikes d .. d +
  // window - 1 steps back, a teacher up to max_delay steps back.  Windows that
  // end within 64 steps come from the per-cell spike registers instead.
  for (const Network& net : s.nets)
    for (const Projection& pr : net.projs) {
      if (!pr.plastic) continue;
      int dmax = 1;
      for (uint8_t d : pr.delay) dmax = std::max(dmax, (int)d);
      const int back = dmax + pr.plast.window_steps <= 64 ? 0 : dmax + pr.plast.window_steps;
      s.hist_rows = std::max<uint32_t>(s.hist_rows, (uint32_t)std::max(max_delay + 1, back));
    }
  if ((uint64_t)s.hist_rows * s.n_pad > 0xFFFFFFFFull)
    return set_error(SGB_ERR_UNSUPPORTED, "spike history of %u steps x %u cells exceeds 2^32",
                     s.hist_rows, s.n_pad);

  // ---- stimulus sources ----------------------------------------------------
  std::vector<uint32_t> src_mask(s.n_pad, 0);
  for (int32_t ni = 0; ni < n; ++ni) {
    const Network& net = s.nets[ni];
    // Each segment's sources are contiguous; bit b of a cell's mask is the
    // segment's b-th source.
    for (size_t pi = 0; pi < net.pops.size(); ++pi) {
      SegDev& d = s.segs[s.net_seg0[ni] + pi];
      d.src_first = (uint32_t)s.srcs.size();
      for (size_t si = 0; si < net.inputs.size(); ++si) {
        const InputSource& src = net.inputs[si];
        if (src.pop != (int32_t)pi) continue;
        const uint32_t bit = (uint32_t)s.srcs.size() - d.src_first;
        SrcDev sd;
        fill_source(sd, src.p, cfg.dt_ms);
        s.srcs.push_back(sd);
        s.src_net.push_back(ni);
        s.src_idx.push_back((int32_t)si);
        for (uint32_t id : src.ids) src_mask[d.base + id] |= 1u << bit;
      }
      d.src_count = (uint32_t)s.srcs.size() - d.src_first;
    }
  }

  // ---- projections: ELL tables, out-degrees ---------------------------------
  std::vector<uint32_t> outdeg(s.n_pad, 0);
  std::vector<std::vector<uint32_t>> ell_syn;
  std::vector<std::vector<float>> ell_wf;
  std::vector<std::vector<uint16_t>> ell_wh;
  std::vector<std::vector<float>> plast_w0;  // per plastic projection: w x 2^S per ELL cell
  size_t pool = 0;
  const size_t wsz = s.bf16 ? 2 : 4;
  for (int32_t ni = 0; ni < n; ++ni) {
    const Network& net = s.nets[ni];
    s.net_proj0.push_back((int32_t)s.projs.size());
    const std::vector<int32_t>& bits = net_bits[ni];
    for (size_t pj = 0; pj < net.projs.size(); ++pj) {
      const Projection& pr = net.projs[pj];
      ProjTables t;
      t.net = ni;
      t.proj = (int32_t)pj;
      t.pre_seg = (uint32_t)(s.net_seg0[ni] + pr.pre);
      t.post_seg = (uint32_t)(s.net_seg0[ni] + pr.post);
      t.scale_bits = bits[pr.post * 2 + pr.channel];
      t.nnz = (int64_t)pr.pre_idx.size();
      ell_syn.emplace_back();
      ell_wf.emplace_back();
      ell_wh.emplace_back();
      if (pr.plastic) {
        PlastHost ph;
        ph.net = ni;
        ph.proj = (int32_t)pj;
        ph.k = (uint32_t)s.projs.size();
        s.plast.push_back(ph);
        plast_w0.emplace_back();
      }
      if (!build_ell(pr, net.pops[pr.post].num, s.segs[t.pre_seg].base, s.n_pad,
                     ell_pad(s.hist_rows, s.n_pad), s.bf16, t, ell_syn.back(), ell_wf.back(),
                     ell_wh.back(), pr.plastic ? &plast_w0.back() : nullptr,
                     pr.plastic ? &s.plast.back().cell_of_syn : nullptr))
        return set_error(SGB_ERR_UNSUPPORTED, "projection %zu: dense table over 2^32 entries", pj);
      t.off_ell_syn = pool;
      pool = align_up(pool + ell_syn.back().size() * 4, 256);
      t.off_ell_w = pool;
      pool = align_up(pool + (size_t)t.ell_K * net.pops[pr.post].num * wsz, 256);
      const SegDev& pre = s.segs[t.pre_seg];
      const SegDev& post = s.segs[t.post_seg];
      for (uint32_t p : pr.pre_idx) outdeg[pre.base + p]++;
      ProjDev P;
      memset(&P, 0, sizeof P);
      P.pre_base = pre.base;
      P.post_base = post.base;
      P.pre_count = pre.count;
      P.post_count = post.count;
      P.channel = (uint32_t)pr.channel;
      const int mode = pr.mode == SGB_PROP_AUTO ? cfg.default_prop : pr.mode;
      P.mode = (uint32_t)(mode == SGB_PROP_AUTO ? SGB_PROP_CSR : mode);
      P.scale = ldexpf(1.0f, t.scale_bits);
      P.ell_K = t.ell_K;
      P.ell_rowmajor = t.ell_rowmajor ? 1u : 0u;
      P.ell_n = t.ell_K * post.count;
      s.n_syn += t.nnz;
      s.projs.push_back(P);
      s.ptab.push_back(t);
    }
  }
  std::vector<uint16_t> seg_of_word(s.n_words, 0xFFFF);
  std::vector<uint32_t> upd_words;
  for (size_t si = 0; si < s.segs.size(); ++si) {
    const SegDev& d = s.segs[si];
    for (uint32_t w = d.base / 32; w < (d.base + d.count + 31) / 32; ++w) {
      seg_of_word[w] = (uint16_t)si;
      upd_words.push_back(w);
    }
  }
  size_t cap_units = 0;
  for (const ProjDev& P : s.projs) cap_units += (P.ell_n + kPullUnit - 1) / kPullUnit;

  // ---- device memory ---------------------------------------------------------
  s.ell_bytes = std::max<size_t>(pool, 256);
  SGB_CUDA(cudaMalloc(&s.d_ell, s.ell_bytes));
  for (size_t i = 0; i < s.ptab.size(); ++i) {
    const ProjTables& t = s.ptab[i];
    char* base = (char*)s.d_ell;
    if (!ell_syn[i].empty()) {
      SGB_CUDA(cudaMemcpy(base + t.off_ell_syn, ell_syn[i].data(), ell_syn[i].size() * 4, cudaMemcpyHostToDevice));
      SGB_CUDA(cudaMemcpy(base + t.off_ell_w, s.bf16 ? (const void*)ell_wh[i].data() : (const void*)ell_wf[i].data(),
                          (s.bf16 ? ell_wh[i].size() : ell_wf[i].size()) * wsz, cudaMemcpyHostToDevice));
    }
    s.projs[i].ell_syn = (const uint32_t*)(base + t.off_ell_syn);
    s.projs[i].ell_w = base + t.off_ell_w;
    std::vector<uint32_t>().swap(ell_syn[i]);
    std::vector<float>().swap(ell_wf[i]);
    std::vector<uint16_t>().swap(ell_wh[i]);
  }
  {
    size_t p = 0;
    const size_t off_row = p; p = align_up(p + ((size_t)s.n_pad + 1) * 4, 256);
    const size_t off_syn = p; p = align_up(p + std::max<int64_t>(s.n_syn, 1) * 4, 256);
    const size_t off_w = p; p = align_up(p + std::max<int64_t>(s.n_syn, 1) * wsz, 256);
    s.push_bytes = p;
    SGB_CUDA(cudaMalloc(&s.d_push, s.push_bytes));
    s.args.push_row = (const uint32_t*)((char*)s.d_push + off_row);
    s.args.push_syn = (const uint32_t*)((char*)s.d_push + off_syn);
    s.args.push_w = (const void*)((char*)s.d_push + off_w);
  }

  s.raster_cap = cfg.raster ? (uint32_t)std::min<uint64_t>((uint64_t)s.n_pad * s.chunk, 1ull << 24) : 0;
  const size_t nseg = s.segs.size();
  size_t m = 0;
  auto take = [&](size_t bytes) { size_t o = m; m = align_up(m + std::max<size_t>(bytes, 1), 256); return o; };
  const size_t o_ctl = take(sizeof(Ctl));
  const size_t o_bar = take(sizeof(unsigned long long));
  const size_t o_segs = take(nseg * sizeof(SegDev));
  const size_t o_projs = take(std::max<size_t>(s.projs.size(), 1) * sizeof(ProjDev));
  const size_t o_srcs = take(std::max<size_t>(s.srcs.size(), 1) * sizeof(SrcDev));
  const size_t o_sow = take((size_t)s.n_words * 2);
  const size_t o_mask = take((size_t)s.n_pad * 4);
  const size_t o_outdeg = take((size_t)s.n_pad * 4);
  const size_t o_words = take(std::max<size_t>(upd_words.size(), 1) * 4);
  const size_t o_units = take(std::max<size_t>(cap_units, 1) * sizeof(PullUnit));
  const size_t o_su = take((size_t)s.n_pad * sizeof(float));
  const size_t o_sg = take((size_t)s.n_pad * sizeof(float2));
  const size_t o_ring = take((size_t)s.ring_slots * s.n_pad * 8);
  // Spike history (two copies of H rows) followed by its summary (H + 1 rows
  // of one bit per word): one region, cleared and snapshotted together.
  const uint32_t n_swords = (s.n_words + 31) / 32;
  s.hist_bytes = ((size_t)2 * s.hist_rows * s.n_words + (size_t)(s.hist_rows + 1) * n_swords) * 4;
  const size_t o_hist = take(s.hist_bytes);
  const uint64_t item_cap = (uint64_t)s.n_pad + (uint64_t)(s.n_syn / kPushChunk) + 1;
  if (item_cap > 0xFFFFFFFFull) return set_error(SGB_ERR_UNSUPPORTED, "push work list too large");
  const size_t o_items_push = take((size_t)2 * item_cap * sizeof(uint2));
  const size_t o_counts = take((size_t)s.chunk * nseg * 4);
  const size_t o_raster = take((size_t)std::max<uint32_t>(s.raster_cap, 1) * 4);
  const size_t o_roff = take((size_t)(s.chunk + 1) * 4);
  const size_t o_totals = take(nseg * sizeof(double));
  s.misc_bytes = m;
  SGB_CUDA(cudaMalloc(&s.d_misc, s.misc_bytes));
  SGB_CUDA(cudaMemset(s.d_misc, 0, s.misc_bytes));
  char* mb = (char*)s.d_misc;

  StepArgs& a = s.args;
  a.ctl = (Ctl*)(mb + o_ctl);
  a.bar = (unsigned long long*)(mb + o_bar);
  a.segs = (const SegDev*)(mb + o_segs);
  a.projs = (const ProjDev*)(mb + o_projs);
  a.srcs = (const SrcDev*)(mb + o_srcs);
  a.seg_of_word = (const uint16_t*)(mb + o_sow);
  a.src_mask = (const uint32_t*)(mb + o_mask);
  a.outdeg = (const uint32_t*)(mb + o_outdeg);
  a.upd_words = (const uint32_t*)(mb + o_words);
  a.pull_units = (const PullUnit*)(mb + o_units);
  a.su = (float*)(mb + o_su);
  a.sg = (float2*)(mb + o_sg);
  a.ring = (int*)(mb + o_ring);
  a.hist = (uint32_t*)(mb + o_hist);
  a.hsum = a.hist + (size_t)2 * s.hist_rows * s.n_words;
  a.n_swords = n_swords;
  a.hist_rows = s.hist_rows;
  a.pull_sum = pull_sum_bytes(a) <= kPullSumMax ? 1u : 0u;
  a.items = (uint2*)(mb + o_items_push);
  a.item_cap = (uint32_t)item_cap;
  a.counts = (uint32_t*)(mb + o_counts);
  a.raster = (uint32_t*)(mb + o_raster);
  a.raster_off = (uint32_t*)(mb + o_roff);
  a.totals = (double*)(mb + o_totals);
  a.n_pad = s.n_pad;
  a.n_words = s.n_words;
  a.n_segs = (uint32_t)nseg;
  a.n_srcs = (uint32_t)s.srcs.size();
  // The general persistent kernel keeps the segment descriptors and sources
  // in shared memory when they fit beside the staged summary (one limit).
  a.seg_smem = seg_smem_bytes(a) + (a.pull_sum ? pull_sum_bytes(a) : 0) <= kPullSumMax ? 1u : 0u;
  a.n_projs = (uint32_t)s.projs.size();
  a.ring_slots = s.ring_slots;
  a.hist_rows = s.hist_rows;
  a.max_delay = s.max_delay;
  a.n_upd_words = (uint32_t)upd_words.size();
  a.raster_cap = s.raster_cap;
  a.bf16 = s.bf16 ? 1 : 0;
  a.substeps = cfg.substeps;
  a.bar_extra = (uint32_t)cfg.barrier_test_extra;
  s.deliver_blocks = 2 * s.sm_count;
  a.item_log2 = 7;  // fused kernel's late-push timelines: push items of 128 synapses (or 64)
  a.ahead = 2;      // fused kernel, one substep: late push with the split barrier (or another)
  a.lane_cells = 2;  // general kernel, one-barrier form: two cells per lane (or one: autotuner)
  // Dense pulls settle entries on the staged summary where it fits; the
  // per-step pull kernel may also stage its entry stream (the autotuner's
  // choice, where that fits too).
  s.pull_sum_fits = a.pull_sum != 0;
  if (a.pull_sum) a.pull_sum = 2u;  // summary staged; the per-step pull loads entries 16 B at a time
  // The cell state is read and rewritten every step; where the device lets
  // this context set L2 aside for persisting accesses, the state window
  // stays in L2 across steps while ring slots, tables and history stream
  // past it.  The limit is a property of this process's context.
  if (cfg.l2_persist) {
    int maxp = 0, maxw = 0;
    cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, cfg.device);
    cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, cfg.device);
    const size_t region = (size_t)((char*)(a.sg + s.n_pad) - (char*)a.su);
    if (maxp > 0 && maxw > 0 && region > 0) {
      SGB_CUDA(cudaDeviceGetLimit(&s.l2_prev_limit, cudaLimitPersistingL2CacheSize));
      const size_t want = std::min(region, (size_t)maxp);
      if (want > s.l2_prev_limit) SGB_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want));
      SGB_CUDA(cudaDeviceGetLimit(&s.l2_setaside, cudaLimitPersistingL2CacheSize));
      s.l2_base = a.su;
      s.l2_window = std::min(region, (size_t)maxw);
      s.l2_hit = (float)std::min(1.0, (double)s.l2_setaside / (double)s.l2_window);
      SGB_CUDA(l2_window_on(s, s.stream, true));
    }
  }
  // ---- plastic projections: values, scaled weights, teachers, work units ----
  if (!s.plast.empty()) {
    std::vector<PlastDev> pd(s.plast.size());
    std::vector<PullUnit> units;
    size_t bytes = align_up(pd.size() * sizeof(PlastDev), 256);
    const size_t off_units = bytes;
    for (size_t i = 0; i < s.plast.size(); ++i) {
      const ProjDev& P = s.projs[s.plast[i].k];
      for (uint32_t o = 0; o < P.ell_n; o += kStdpUnit) units.push_back({(uint32_t)i, o});
    }
    bytes = align_up(bytes + std::max<size_t>(units.size(), 1) * sizeof(PullUnit), 256);
    s.off_recent = bytes;
    bytes = align_up(bytes + (size_t)s.n_pad * 16, 256);  // two buffers
    std::vector<size_t> off_w0(s.plast.size()), off_t(s.plast.size());
    for (size_t i = 0; i < s.plast.size(); ++i) {
      PlastHost& ph = s.plast[i];
      const ProjDev& P = s.projs[ph.k];
      ph.cells = P.ell_n;
      ph.off_val = bytes;
      bytes = align_up(bytes + std::max<size_t>(ph.cells, 1) * 4, 256);
      off_w0[i] = bytes;
      bytes = align_up(bytes + std::max<size_t>(ph.cells, 1) * 4, 256);
      off_t[i] = bytes;
      bytes = align_up(bytes + std::max<size_t>(P.post_count, 1) * 4, 256);
    }
    SGB_CUDA(cudaMalloc(&s.d_plast, bytes));
    char* pb = (char*)s.d_plast;
    for (size_t i = 0; i < s.plast.size(); ++i) {
      const PlastHost& ph = s.plast[i];
      const ProjDev& P = s.projs[ph.k];
      const Projection& pr = s.nets[ph.net].projs[ph.proj];
      const sgb_plasticity_params& q = pr.plast;
      // Teacher of each post cell: its synapse of the teacher projection with
      // the lowest (delay, pre id); its spike sits `delay` rows above step t.
      std::vector<uint32_t> teacher(P.post_count, 0xFFFFFFFFu);
      if (q.rule == SGB_STDP_TEACHER) {
        const Projection& tp = s.nets[ph.net].projs[q.teacher_proj];
        const uint32_t tbase = s.segs[s.net_seg0[ph.net] + tp.pre].base;
        std::vector<uint64_t> best(P.post_count, ~0ull);
        for (size_t j = 0; j < tp.pre_idx.size(); ++j) {
          const uint64_t key = ((uint64_t)tp.delay[j] << 32) | tp.pre_idx[j];
          uint64_t& b = best[tp.post_idx[j]];
          if (key < b) b = key;
        }
        for (uint32_t p = 0; p < P.post_count; ++p)
          if (best[p] != ~0ull)
            teacher[p] = (uint32_t)(best[p] >> 32) * s.n_pad + tbase + (uint32_t)(best[p] & 0xFFFFFFFFu);
      }
      SGB_CUDA(cudaMemcpy(pb + off_w0[i], plast_w0[i].data(), ph.cells * 4, cudaMemcpyHostToDevice));
      SGB_CUDA(cudaMemcpy(pb + off_t[i], teacher.data(), (size_t)P.post_count * 4, cudaMemcpyHostToDevice));
      PlastDev& d = pd[i];
      memset(&d, 0, sizeof d);
      d.proj = ph.k;
      d.rule = (uint32_t)q.rule;
      d.window = (uint32_t)q.window_steps;
      {
        int dmax = 1;
        for (uint8_t dl : pr.delay) dmax = std::max(dmax, (int)dl);
        d.recent_ok = dmax + q.window_steps <= 64 ? 1u : 0u;
      }
      d.a0 = q.a0;
      d.a1_i = q.a1_i;
      d.a1_j = q.a1_j;
      d.a2_ji = q.a2_ji;
      d.v_max = q.v_max;
      d.val = (float*)(pb + ph.off_val);
      d.w0 = (const float*)(pb + off_w0[i]);
      d.teacher = (const uint32_t*)(pb + off_t[i]);
      d.w_table = const_cast<void*>(P.ell_w);
    }
    std::vector<std::vector<float>>().swap(plast_w0);
    SGB_CUDA(cudaMemcpy(pb, pd.data(), pd.size() * sizeof(PlastDev), cudaMemcpyHostToDevice));
    if (!units.empty())
      SGB_CUDA(cudaMemcpy(pb + off_units, units.data(), units.size() * sizeof(PullUnit), cudaMemcpyHostToDevice));
    a.plast = (const PlastDev*)pb;
    a.recent = (unsigned long long*)(pb + s.off_recent);
    a.n_plast = (uint32_t)pd.size();
    a.stdp_early = 1u;  // the Teacher rule reads its teacher's and pre cells' earlier spikes
    for (const PlastDev& d : pd)
      if (d.rule != SGB_STDP_TEACHER) a.stdp_early = 0u;
    if (a.stdp_early) {
      SGB_CUDA(cudaStreamCreateWithFlags(&s.side, cudaStreamNonBlocking));
      SGB_CUDA(cudaEventCreateWithFlags(&s.ev_fork, cudaEventDisableTiming));
      SGB_CUDA(cudaEventCreateWithFlags(&s.ev_join, cudaEventDisableTiming));
    }
    a.stdp_units = (const PullUnit*)(pb + off_units);
    a.n_stdp_units = (uint32_t)units.size();
  }
  SGB_CUDA(pull_setup());
  s.pull_blocks = pull_blocks_per_sm(a) * s.sm_count;
  const int bpsm = std::min(cfg.blocks_per_sm > 0 ? cfg.blocks_per_sm : 1,
                            persistent_blocks_per_sm(s.bf16));
  s.persistent_blocks = std::max(1, bpsm) * s.sm_count;

  SGB_CUDA(cudaMemcpy((void*)a.segs, s.segs.data(), nseg * sizeof(SegDev), cudaMemcpyHostToDevice));
  SGB_CUDA(cudaMallocHost(&s.h_srcs, std::max<size_t>(s.srcs.size(), 1) * sizeof(SrcDev)));
  if (!s.srcs.empty()) {
    memcpy(s.h_srcs, s.srcs.data(), s.srcs.size() * sizeof(SrcDev));
    SGB_CUDA(cudaMemcpy((void*)a.srcs, s.h_srcs, s.srcs.size() * sizeof(SrcDev), cudaMemcpyHostToDevice));
  }
  SGB_CUDA(cudaMemcpy((void*)a.seg_of_word, seg_of_word.data(), seg_of_word.size() * 2, cudaMemcpyHostToDevice));
  SGB_CUDA(cudaMemcpy((void*)a.src_mask, src_mask.data(), src_mask.size() * 4, cudaMemcpyHostToDevice));
  SGB_CUDA(cudaMemcpy((void*)a.outdeg, outdeg.data(), outdeg.size() * 4, cudaMemcpyHostToDevice));
  if (!upd_words.empty())
    SGB_CUDA(cudaMemcpy((void*)a.upd_words, upd_words.data(), upd_words.size() * 4, cudaMemcpyHostToDevice));
  s.upd_words = upd_words;
  if ((uint64_t)upd_words.size() * 32 <= (uint64_t)s.persistent_blocks * kPersistBlock) {
    // Resident networks may run the fused kernel: room for its shards.
    const size_t bytes = align_up((size_t)s.n_pad * 4, 256) +
                         align_up((size_t)s.persistent_blocks * kMaxShards * sizeof(uint4), 256) +
                         ((size_t)s.persistent_blocks + 1) * 4;
    SGB_CUDA(cudaMalloc(&s.d_shard, bytes));
    s.push_bytes += bytes;
  }
  int rc = upload_modes(s);
  if (rc) return rc;

  SGB_CUDA(cudaMallocHost(&s.h_counts, (size_t)s.chunk * nseg * 4));
  SGB_CUDA(cudaMallocHost(&s.h_raster_off, (size_t)(s.chunk + 1) * 4));
  if (s.raster_cap) SGB_CUDA(cudaMallocHost(&s.h_raster, (size_t)s.raster_cap * 4));

  rc = sim_reset(s, nullptr);
  if (rc) return rc;
  *out = S.release();
  return SGB_OK;
}

// ---------------------------------------------------------------------------
int sim_reset(Sim& s, const uint64_t* seeds) {
  if (seeds) {
    for (size_t i = 0; i < s.nets.size(); ++i) s.seeds[i] = seeds[i];
    for (size_t si = 0; si < s.segs.size(); ++si) s.segs[si].seed = s.seeds[s.seg_net[si]];
    SGB_CUDA(cudaMemcpyAsync((void*)s.args.segs, s.segs.data(), s.segs.size() * sizeof(SegDev),
                             cudaMemcpyHostToDevice, s.stream));
  }
  std::vector<float> su(s.n_pad, 0.f);
  for (size_t si = 0; si < s.segs.size(); ++si) {
    const SegDev& d = s.segs[si];
    if (d.kind != kSegLif) continue;
    const Population& p = s.nets[s.seg_net[si]].pops[s.seg_pop[si]];
    for (uint32_t j = 0; j < d.count; ++j) su[d.base + j] = initial_u(p, d.seed, d.key_base + j);
  }
  const StepArgs& a = s.args;
  SGB_CUDA(cudaMemcpyAsync(a.su, su.data(), su.size() * sizeof(float), cudaMemcpyHostToDevice, s.stream));
  SGB_CUDA(cudaMemsetAsync(a.sg, 0, (size_t)s.n_pad * sizeof(float2), s.stream));
  SGB_CUDA(cudaMemsetAsync(a.ring, 0, (size_t)s.ring_slots * s.n_pad * 8, s.stream));
  SGB_CUDA(cudaMemsetAsync(a.hist, 0, s.hist_bytes, s.stream));
  SGB_CUDA(cudaMemsetAsync(a.ctl, 0, sizeof(Ctl), s.stream));
  if (a.n_plast) {
    SGB_CUDA(launch_plast_reset(a, s.deliver_blocks, s.stream));
    SGB_CUDA(cudaMemsetAsync(a.recent, 0, (size_t)s.n_pad * 16, s.stream));
  }
  SGB_CUDA(cudaMemsetAsync(a.items, 0, (size_t)2 * a.item_cap * sizeof(uint2), s.stream));
  SGB_CUDA(cudaMemsetAsync(a.totals, 0, s.segs.size() * sizeof(double), s.stream));
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  return SGB_OK;
}

// ---------------------------------------------------------------------------
// One chunk of c steps issued on `st` (direct launches; also the body that is
// captured into a graph).  *nlaunch receives the number of kernel launches.
static cudaError_t issue_chunk(Sim& s, uint32_t c, cudaStream_t st, int64_t* nlaunch) {
  const StepArgs& a = s.args;
  cudaError_t e;
  int64_t L = 0;
  if ((e = cudaMemsetAsync(a.counts, 0, (size_t)c * a.n_segs * 4, st))) return e;
  if ((e = launch_chunk_begin(a, st))) return e;
  L++;
  if (s.cfg.exec_mode == SGB_EXEC_PERSISTENT) {
    if ((e = cudaMemsetAsync(a.bar, 0, sizeof(unsigned long long), st))) return e;
    if ((e = launch_persistent(a, c, s.persistent_blocks, st))) return e;
    L++;
  } else {
    for (uint32_t i = 0; i < c; ++i) {
      if (a.n_plast && s.side) {
        // Early rule: the step's plasticity does not read its update, so the
        // two run side by side (fork / join; also inside a graph capture).
        if ((e = cudaEventRecord(s.ev_fork, st))) return e;
        if ((e = cudaStreamWaitEvent(s.side, s.ev_fork, 0))) return e;
        if ((e = launch_stdp(a, s.deliver_blocks, s.side, true))) return e;
        if ((e = launch_update(a, st))) return e;
        if ((e = cudaEventRecord(s.ev_join, s.side))) return e;
        if ((e = cudaStreamWaitEvent(st, s.ev_join, 0))) return e;
        L++;
      } else {
        if ((e = launch_update(a, st))) return e;
        if (a.n_plast) {
          if ((e = launch_stdp(a, s.deliver_blocks, st))) return e;
          L++;
        }
      }
      if (a.n_pull_units) {
        if ((e = launch_pull(a, s.pull_blocks, st))) return e;
        L++;
      }
      if ((e = launch_deliver(a, s.deliver_blocks, st))) return e;
      L += 2;
    }
  }
  if ((e = launch_chunk_end(a, st))) return e;
  L++;
  if (nlaunch) *nlaunch = L;
  return cudaSuccess;
}

static int launch_chunk(Sim& s, uint32_t c) {
  int64_t L = 0;
  if (s.cfg.exec_mode == SGB_EXEC_GRAPH) {
    auto it = s.graphs.find(c);
    if (it == s.graphs.end()) {
      cudaGraph_t g;
      SGB_CUDA(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = issue_chunk(s, c, s.stream, &L);
      cudaError_t e2 = cudaStreamEndCapture(s.stream, &g);
      if (e != cudaSuccess)
        return set_error(SGB_ERR_CUDA, "capture of a %u-step chunk failed: %s", c, cudaGetErrorString(e));
      if (e2 != cudaSuccess) return set_error(SGB_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e2));
      cudaGraphExec_t ge;
      e = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return set_error(SGB_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
      it = s.graphs.emplace(c, ge).first;
    }
    SGB_CUDA(cudaGraphLaunch(it->second, s.stream));
    L = 2 + 2 * (int64_t)c;
  } else {
    cudaError_t e = issue_chunk(s, c, s.stream, &L);
    if (e != cudaSuccess) return set_error(SGB_ERR_CUDA, "step launch failed: %s", cudaGetErrorString(e));
  }
  s.launches += L;
  return SGB_OK;
}

static int check_device_error(Sim& s, uint32_t* bits) {
  uint32_t err = 0;
  SGB_CUDA(cudaMemcpyAsync(&err, &s.args.ctl->error, 4, cudaMemcpyDeviceToHost, s.stream));
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  if (bits) *bits = err;
  return SGB_OK;
}

int sim_enqueue(Sim& s, int64_t n_steps) {
  if (n_steps < 0) return set_error(SGB_ERR_ARG, "n_steps is negative");
  for (int64_t done = 0; done < n_steps;) {
    const uint32_t c = (uint32_t)std::min<int64_t>(s.chunk, n_steps - done);
    int rc = launch_chunk(s, c);
    if (rc) return rc;
    done += c;
  }
  return SGB_OK;
}

int sim_sync(Sim& s) {
  uint32_t err = 0;
  int rc = check_device_error(s, &err);
  if (rc) return rc;
  SGB_CUDA(cudaMemsetAsync(&s.args.ctl->error, 0, 4, s.stream));
  if (err & kErrBarrierTimeout)
    return set_error(SGB_ERR_DEVICE, "a device-side grid barrier hit its wait limit; reset the handle");

  return SGB_OK;
}

int sim_run(Sim& s, int64_t n_steps, uint32_t* counts, uint32_t* raster_ids, int64_t raster_cap,
            int64_t* raster_offsets) {
  if (n_steps < 0) return set_error(SGB_ERR_ARG, "n_steps is negative");
  const bool want_raster = raster_ids || raster_offsets;
  if (want_raster && !s.raster_cap)
    return set_error(SGB_ERR_STATE, "raster output needs a handle created with cfg.raster = 1");
  if (want_raster && (!raster_ids || !raster_offsets))
    return set_error(SGB_ERR_ARG, "raster_ids and raster_offsets go together");
  const size_t nseg = s.segs.size();
  int64_t done = 0, rfill = 0;
  bool overflow = false;
  if (raster_offsets) raster_offsets[0] = 0;
  while (done < n_steps) {
    const uint32_t c = (uint32_t)std::min<int64_t>(s.chunk, n_steps - done);
    int rc = launch_chunk(s, c);
    if (rc) return rc;
    if (counts || want_raster) {
      const StepArgs& a = s.args;
      SGB_CUDA(cudaMemcpyAsync(s.h_counts, a.counts, (size_t)c * nseg * 4, cudaMemcpyDeviceToHost, s.stream));
      if (want_raster)
        SGB_CUDA(cudaMemcpyAsync(s.h_raster_off, a.raster_off, (size_t)(c + 1) * 4, cudaMemcpyDeviceToHost, s.stream));
      SGB_CUDA(cudaStreamSynchronize(s.stream));
      if (counts) memcpy(counts + (size_t)done * nseg, s.h_counts, (size_t)c * nseg * 4);
      if (want_raster) {
        const uint32_t nrec = std::min<uint32_t>(s.h_raster_off[c], s.raster_cap);
        if (nrec) {
          SGB_CUDA(cudaMemcpyAsync(s.h_raster, a.raster, (size_t)nrec * 4, cudaMemcpyDeviceToHost, s.stream));
          SGB_CUDA(cudaStreamSynchronize(s.stream));
        }
        // Records are in step order, except from the fused kernel's late-push
        // timelines: there step r's records lie after every record of step
        // r - 2 and before every record of step r + 2 (blocks run at most a
        // step apart), and carry r mod 4.
        const bool windowed = s.cfg.exec_mode == SGB_EXEC_PERSISTENT &&
                              persistent_kernel_kind(a, s.persistent_blocks) == SGB_KERNEL_FUSED &&
                              fused_timeline(a) != 0;
        for (uint32_t r = 0; r < c; ++r) {
          const uint32_t b = s.h_raster_off[windowed && r > 0 ? r - 1 : r];
          const uint32_t e = std::min<uint32_t>(s.h_raster_off[windowed ? std::min(r + 2, c) : r + 1],
                                                s.raster_cap);
          const uint32_t need = s.h_raster_off[r + 1] - s.h_raster_off[r];
          const int64_t start = rfill;
          for (uint32_t q = b; q < e && rfill - start < (int64_t)need; ++q) {
            if (windowed && (s.h_raster[q] >> kRasterTagShift) != (r & 3u)) continue;
            if (rfill >= raster_cap) {
              overflow = true;
              break;
            }
            const uint32_t pid = s.h_raster[q] & ((1u << kRasterTagShift) - 1u);
            // Segment of the padded id by binary search over segment bases.
            size_t lo = 0, hi = nseg;
            while (hi - lo > 1) {
              const size_t mid = (lo + hi) / 2;
              if (s.segs[mid].base <= pid) lo = mid; else hi = mid;
            }
            raster_ids[rfill++] = (uint32_t)(s.seg_first_id[lo] + (pid - s.segs[lo].base));
          }
          if (rfill - start < (int64_t)need) overflow = true;  // records past a capacity
          std::sort(raster_ids + start, raster_ids + rfill);
          raster_offsets[done + r + 1] = rfill;
        }
      }
    }
    done += c;
  }
  uint32_t err = 0;
  int rc = check_device_error(s, &err);
  if (rc) return rc;
  SGB_CUDA(cudaMemsetAsync(&s.args.ctl->error, 0, 4, s.stream));
  if (err & kErrBarrierTimeout)
    return set_error(SGB_ERR_DEVICE, "a device-side grid barrier hit its wait limit; reset the handle");

  if (overflow || (want_raster && (err & kErrRasterOverflow)))
    return set_error(SGB_ERR_OVERFLOW, "raster buffer too small; counts and state are intact");
  return SGB_OK;
}

int sim_set_rates(Sim& s, int32_t net, int32_t n, const float* rates) {
  if (net < 0 || net >= (int32_t)s.nets.size()) return set_error(SGB_ERR_ARG, "net %d out of range", net);
  const int32_t nsrc = (int32_t)s.nets[net].inputs.size();
  if (n != nsrc || (!rates && n)) return set_error(SGB_ERR_ARG, "net %d has %d sources, got %d rates", net, nsrc, n);
  for (int32_t i = 0; i < n; ++i)
    if (!(rates[i] >= 0.f)) return set_error(SGB_ERR_ARG, "rate %d must be >= 0", i);
  for (size_t k = 0; k < s.srcs.size(); ++k) {
    if (s.src_net[k] != net) continue;
    sgb_input_params& p = s.nets[net].inputs[s.src_idx[k]].p;
    p.rate_hz = rates[s.src_idx[k]];
    fill_source(s.srcs[k], p, s.cfg.dt_ms);
  }
  if (!s.srcs.empty()) {
    // The pinned staging copy is reused only after the previous upload ended.
    SGB_CUDA(cudaStreamSynchronize(s.stream));
    memcpy(s.h_srcs, s.srcs.data(), s.srcs.size() * sizeof(SrcDev));
    SGB_CUDA(cudaMemcpyAsync((void*)s.args.srcs, s.h_srcs, s.srcs.size() * sizeof(SrcDev),
                             cudaMemcpyHostToDevice, s.stream));
  }
  return SGB_OK;
}

int sim_get_state(Sim& s, float* u, float* g, int32_t* ref) {
  std::vector<float> su(s.n_pad);
  std::vector<float2> sg(s.n_pad);
  SGB_CUDA(cudaMemcpyAsync(su.data(), s.args.su, su.size() * sizeof(float), cudaMemcpyDeviceToHost, s.stream));
  SGB_CUDA(cudaMemcpyAsync(sg.data(), s.args.sg, sg.size() * sizeof(float2), cudaMemcpyDeviceToHost, s.stream));
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  for (size_t si = 0; si < s.segs.size(); ++si) {
    const SegDev& d = s.segs[si];
    const int64_t f = s.seg_first_id[si];
    const bool lif = d.kind == kSegLif;
    for (uint32_t j = 0; j < d.count; ++j) {
      const float x = su[d.base + j];
      const int32_t r = lif ? unpack_ref(x) : 0;
      if (u) u[f + j] = r ? d.Vr : x;
      if (g) { g[2 * (f + j)] = sg[d.base + j].x; g[2 * (f + j) + 1] = sg[d.base + j].y; }
      if (ref) ref[f + j] = r;
    }
  }
  return SGB_OK;
}

// A refractory cell's potential is V_reset (the update pins it there and the
// stored state keeps only the count), so a state with ref > 0 and another
// potential is refused.
int sim_set_state(Sim& s, const float* u, const float* g, const int32_t* ref) {
  std::vector<float> su(s.n_pad);
  std::vector<float2> sg(s.n_pad);
  SGB_CUDA(cudaMemcpyAsync(su.data(), s.args.su, su.size() * sizeof(float), cudaMemcpyDeviceToHost, s.stream));
  SGB_CUDA(cudaMemcpyAsync(sg.data(), s.args.sg, sg.size() * sizeof(float2), cudaMemcpyDeviceToHost, s.stream));
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  for (size_t si = 0; si < s.segs.size(); ++si) {
    const SegDev& d = s.segs[si];
    if (d.kind != kSegLif) continue;
    const int64_t f = s.seg_first_id[si];
    for (uint32_t j = 0; j < d.count; ++j) {
      float& x = su[d.base + j];
      int32_t r = unpack_ref(x);
      float v = r ? d.Vr : x;
      if (u) v = u[f + j];
      if (ref) {
        if (ref[f + j] < 0 || ref[f + j] > kRefMax)
          return set_error(SGB_ERR_ARG, "refractory count %d out of 0..%d", ref[f + j], kRefMax);
        r = ref[f + j];
      }
      if (r > 0 && v != d.Vr)
        return set_error(SGB_ERR_ARG, "cell %lld is refractory but its potential is not V_reset",
                         (long long)(f + j));
      x = pack_u(v, r);
      if (g) sg[d.base + j] = make_float2(g[2 * (f + j)], g[2 * (f + j) + 1]);
    }
  }
  SGB_CUDA(cudaMemcpyAsync(s.args.su, su.data(), su.size() * sizeof(float), cudaMemcpyHostToDevice, s.stream));
  SGB_CUDA(cudaMemcpyAsync(s.args.sg, sg.data(), sg.size() * sizeof(float2), cudaMemcpyHostToDevice, s.stream));
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  return SGB_OK;
}

int sim_totals(Sim& s, double* totals) {
  if (!totals) return set_error(SGB_ERR_ARG, "totals is NULL");
  SGB_CUDA(cudaMemcpyAsync(totals, s.args.totals, s.segs.size() * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  return SGB_OK;
}

// A change of propagation modes at a step boundary (step T about to run).
// A projection's spikes of steps S < T reach their targets' ring slots S + d
// either pushed in (or before) step S, or pulled in step S + d - 1: at the
// boundary, a projection that pushed has already delivered its recent
// spikes' contributions to slots T + 1 and later, which its pulls would add
// again, and one that pulled has not yet delivered them.  So for every
// projection whose mode changed, each synapse of delay d >= 2 whose pre cell
// spiked in step S = T - k (k = 1 .. d - 1; from the spike history) has its
// fixed-point increment taken out of slot S + d (push -> pull) or added to it
// (pull -> push).  The ring holds integer sums, so the run continues exactly
// as if the new modes had been in place from the start.
static int handover_modes(Sim& s, const std::vector<uint32_t>& before) {
  std::vector<size_t> changed;
  for (size_t k = 0; k < s.projs.size(); ++k)
    if (before[k] != s.projs[k].mode) changed.push_back(k);
  if (changed.empty() || s.max_delay < 2) return SGB_OK;
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  Ctl ctl;
  SGB_CUDA(cudaMemcpy(&ctl, s.args.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  const uint64_t T = ctl.step;
  if (T == 0) return SGB_OK;
  const uint32_t H = s.hist_rows, R = s.ring_slots, D = s.max_delay;
  std::vector<uint32_t> hist((size_t)2 * H * s.n_words);
  SGB_CUDA(cudaMemcpy(hist.data(), s.args.hist, hist.size() * 4, cudaMemcpyDeviceToHost));
  // Row of step T - k: the rows run in decreasing step order from that of T
  // (the second copy covers the wrap).
  auto spiked = [&](uint32_t k, uint32_t cell) {
    const size_t row = (size_t)(H - 1u - ctl.hist_row + k) * s.n_words;
    return (hist[row + (cell >> 5)] >> (cell & 31u)) & 1u;
  };
  // Ring slots T + 1 .. T + D - 1.
  std::vector<int2> slots((size_t)(D - 1) * s.n_pad);
  auto slot_of = [&](uint32_t ahead) { return (ctl.ring_slot + ahead) % R; };
  for (uint32_t j = 1; j < D; ++j)
    SGB_CUDA(cudaMemcpy(slots.data() + (size_t)(j - 1) * s.n_pad,
                        (const int2*)s.args.ring + (size_t)slot_of(j) * s.n_pad,
                        (size_t)s.n_pad * 8, cudaMemcpyDeviceToHost));
  for (size_t k : changed) {
    const ProjTables& t = s.ptab[k];
    const Projection& pr = s.nets[t.net].projs[t.proj];
    const uint32_t pre_base = s.segs[t.pre_seg].base, post_base = s.segs[t.post_seg].base;
    const int32_t sign = s.projs[k].mode == SGB_PROP_ELL ? -1 : 1;
    for (size_t i = 0; i < pr.pre_idx.size(); ++i) {
      const uint32_t d = pr.delay[i];
      const uint32_t pre = pre_base + pr.pre_idx[i];
      for (uint32_t back = 1; back < d && back <= T; ++back) {
        if (!spiked(back, pre)) continue;
        const int32_t inc = (int32_t)lrintf(scaled_weight(pr.weight[i], t.scale_bits, s.bf16));
        int2& e = slots[(size_t)(d - back - 1) * s.n_pad + post_base + pr.post_idx[i]];
        (pr.channel ? e.y : e.x) += sign * inc;
      }
    }
  }
  for (uint32_t j = 1; j < D; ++j)
    SGB_CUDA(cudaMemcpy((int2*)s.args.ring + (size_t)slot_of(j) * s.n_pad,
                        slots.data() + (size_t)(j - 1) * s.n_pad, (size_t)s.n_pad * 8,
                        cudaMemcpyHostToDevice));
  return SGB_OK;
}

static std::vector<uint32_t> current_modes(const Sim& s) {
  std::vector<uint32_t> m(s.projs.size());
  for (size_t k = 0; k < m.size(); ++k) m[k] = s.projs[k].mode;
  return m;
}

int sim_set_mode(Sim& s, int32_t net, int32_t proj, int32_t mode) {
  if (net < 0 || net >= (int32_t)s.nets.size()) return set_error(SGB_ERR_ARG, "net %d out of range", net);
  if (proj < 0 || proj >= (int32_t)s.nets[net].projs.size())
    return set_error(SGB_ERR_ARG, "projection %d out of range", proj);
  if (mode != SGB_PROP_CSR && mode != SGB_PROP_ELL) return set_error(SGB_ERR_ARG, "mode must be CSR or ELL");
  if (s.nets[net].projs[proj].plastic && mode != SGB_PROP_ELL)
    return set_error(SGB_ERR_UNSUPPORTED, "projection %d is plastic: it stays in dense pull", proj);
  const std::vector<uint32_t> before = current_modes(s);
  s.projs[s.net_proj0[net] + proj].mode = (uint32_t)mode;
  int rc = upload_modes(s);
  return rc ? rc : handover_modes(s, before);
}

int sim_set_stream(Sim& s, cudaStream_t st) {
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  cudaStream_t next = st ? st : s.own_stream;
  if (s.l2_window && next != s.stream) {
    // The state window follows the handle's launches; a caller's stream is
    // left without it once the handle moves on.
    if (s.stream != s.own_stream) SGB_CUDA(l2_window_on(s, s.stream, false));
    SGB_CUDA(l2_window_on(s, next, true));
  }
  s.stream = next;
  for (auto& kv : s.graphs) cudaGraphExecDestroy(kv.second);
  s.graphs.clear();
  return SGB_OK;
}

// ---------------------------------------------------------------------------
// Autotuner.  Decisions: propagation mode per projection group (projection j
// of every instance; instances of one handle share an architecture or are
// tuned per net when they do not) and the step driver (persistent vs graph).
// Each candidate runs n_steps of the live simulation, timed with CUDA events
// on the handle's stream, from the same snapshot of the device state; the
// snapshot is restored at the end, so tuning does not advance the simulation.

static uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
  return h;
}

static std::string tune_signature(const Sim& s) {
  uint64_t h = 1469598103934665603ull;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, s.cfg.device) == cudaSuccess)
    h = fnv1a(h, prop.name, strlen(prop.name));
  const int32_t hdr[4] = {(int32_t)s.nets.size(), s.cfg.substeps, s.cfg.weight_type, (int32_t)s.chunk};
  h = fnv1a(h, hdr, sizeof hdr);
  h = fnv1a(h, &s.cfg.dt_ms, sizeof s.cfg.dt_ms);
  for (const Network& net : s.nets) {
    for (const Population& p : net.pops) h = fnv1a(h, &p.num, sizeof p.num);
    for (const Projection& pr : net.projs) {
      const int64_t v[4] = {pr.pre, pr.post, pr.channel, (int64_t)pr.pre_idx.size()};
      h = fnv1a(h, v, sizeof v);
    }
  }
  char buf[32];
  snprintf(buf, sizeof buf, "%016llx", (unsigned long long)h);
  return buf;
}

// Launch shapes the autotuner picks beside the modes and the driver.
struct TuneShape {
  int32_t item_log2;     // fused kernel: push items of 2^item_log2 synapses (6 or 7)
  int32_t deliver_mult;  // per-step driver: delivery blocks per SM
  int32_t pull_sum;      // dense pulls: 0 no summary, 1 staged summary, 2 also 16-byte entry loads
  int32_t ahead;         // fused kernel's timeline: 0 spikes in their own step, 1 late push,
                         // 2 late push with a split barrier
  int32_t lane_cells;    // general kernel's one-barrier form: cells per lane (1 or 2)
};

static TuneShape current_shape(const Sim& s) {
  return {(int32_t)s.args.item_log2, std::max(1, s.deliver_blocks / std::max(1, s.sm_count)),
          (int32_t)s.args.pull_sum, (int32_t)s.args.ahead, (int32_t)s.args.lane_cells};
}

// Applies a shape (kept within what the handle supports); captured graphs
// hold the old kernel arguments and are dropped.
static void apply_shape(Sim& s, const TuneShape& t) {
  s.args.item_log2 = (uint32_t)std::min(7, std::max(6, t.item_log2));
  s.deliver_blocks = std::min(8, std::max(1, t.deliver_mult)) * s.sm_count;
  const bool ok = t.pull_sum == 0 || (s.pull_sum_fits && t.pull_sum >= 1 && t.pull_sum <= 2);
  s.args.pull_sum = ok ? (uint32_t)t.pull_sum : (s.pull_sum_fits ? 2u : 0u);
  s.args.ahead = (uint32_t)std::min(2, std::max(0, t.ahead));
  s.args.lane_cells = t.lane_cells >= 2 ? 2u : 1u;
  for (auto& kv : s.graphs) cudaGraphExecDestroy(kv.second);
  s.graphs.clear();
}

// Reads the cached decision for `sig` from a JSON-lines file:
// {"signature": "<hex>", "exec_mode": m, "modes": [a, b, ...],
//  "shape": [item_log2, deliver_mult, pull_sum], "us_per_step": x}
static bool tune_cache_read(const char* path, const std::string& sig, int32_t* exec_mode,
                            std::vector<int32_t>& modes, TuneShape* shape) {
  FILE* f = path ? fopen(path, "rb") : nullptr;
  if (!f) return false;
  char line[1 << 16];
  bool found = false;
  while (!found && fgets(line, sizeof line, f)) {
    if (!strstr(line, ("\"signature\": \"" + sig + "\"").c_str())) continue;
    const char* e = strstr(line, "\"exec_mode\":");
    const char* m = strstr(line, "\"modes\": [");
    if (!e || !m) continue;
    *exec_mode = atoi(e + 12);
    modes.clear();
    for (const char* p = m + 10; *p && *p != ']';) {
      char* q;
      const long v = strtol(p, &q, 10);
      if (q == p) { ++p; continue; }
      modes.push_back((int32_t)v);
      p = q;
    }
    const char* sh = strstr(line, "\"shape\": [");
    if (sh && shape) {
      int32_t v[5] = {6, 2, 1, 1, 1};
      if (sscanf(sh + 10, "%d , %d , %d , %d , %d", &v[0], &v[1], &v[2], &v[3], &v[4]) >= 3)
        *shape = {v[0], v[1], v[2], v[3], v[4]};
    }
    found = true;
  }
  fclose(f);
  return found;
}

static void tune_cache_write(const char* path, const std::string& sig, int32_t exec_mode,
                             const std::vector<int32_t>& modes, const TuneShape& shape,
                             double us_per_step) {
  if (!path) return;
  FILE* f = fopen(path, "ab");
  if (!f) return;
  fprintf(f, "{\"signature\": \"%s\", \"exec_mode\": %d, \"modes\": [", sig.c_str(), exec_mode);
  for (size_t i = 0; i < modes.size(); ++i) fprintf(f, "%s%d", i ? ", " : "", modes[i]);
  fprintf(f, "], \"shape\": [%d, %d, %d, %d, %d], \"us_per_step\": %.4f}\n", shape.item_log2,
          shape.deliver_mult, shape.pull_sum, shape.ahead, shape.lane_cells, us_per_step);
  fclose(f);
}

static int apply_modes(Sim& s, const std::vector<int32_t>& modes) {
  if (modes.size() != s.projs.size()) return set_error(SGB_ERR_ARG, "mode vector length mismatch");
  for (size_t k = 0; k < modes.size(); ++k) s.projs[k].mode = (uint32_t)modes[k];
  return upload_modes(s);
}

int sim_autotune(Sim& s, int32_t n_steps, const char* cache_path) {
  if (!s.plast.empty())
    return set_error(SGB_ERR_UNSUPPORTED,
                     "handles with plastic projections keep their modes and driver (not tuned)");
  if (n_steps < 1) return set_error(SGB_ERR_ARG, "n_steps must be >= 1");
  const std::string sig = tune_signature(s);
  std::vector<int32_t> modes;
  int32_t exec_mode = s.cfg.exec_mode;
  TuneShape shape = current_shape(s);
  const std::vector<uint32_t> modes0 = current_modes(s);
  if (tune_cache_read(cache_path, sig, &exec_mode, modes, &shape) &&
      modes.size() == s.projs.size()) {
    s.cfg.exec_mode = exec_mode;
    apply_shape(s, shape);
    int rc = apply_modes(s, modes);
    return rc ? rc : handover_modes(s, modes0);
  }
  // Snapshot of the device state a run changes.
  const StepArgs& a = s.args;
  const size_t b_su = (size_t)s.n_pad * sizeof(float), b_sg = (size_t)s.n_pad * sizeof(float2);
  const size_t b_ring = (size_t)s.ring_slots * s.n_pad * 8;
  const size_t b_hist = s.hist_bytes;
  const size_t b_tot = s.segs.size() * sizeof(double);
  const size_t total = b_su + b_sg + b_ring + b_hist + sizeof(Ctl) + b_tot;
  char* snap = nullptr;
  SGB_CUDA(cudaMalloc(&snap, total));
  auto save = [&](bool restore) -> cudaError_t {
    struct { void* dev; size_t n; } parts[6] = {{a.su, b_su}, {a.sg, b_sg}, {a.ring, b_ring}, {a.hist, b_hist},
                                              {a.ctl, sizeof(Ctl)}, {a.totals, b_tot}};
    size_t o = 0;
    for (auto& p : parts) {
      cudaError_t e = restore ? cudaMemcpyAsync(p.dev, snap + o, p.n, cudaMemcpyDeviceToDevice, s.stream)
                              : cudaMemcpyAsync(snap + o, p.dev, p.n, cudaMemcpyDeviceToDevice, s.stream);
      if (e) return e;
      o += p.n;
    }
    return cudaStreamSynchronize(s.stream);
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = SGB_OK;
  auto fail = [&](int code) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(snap);
    return code;
  };
  if (save(false) || cudaEventCreate(&e0) || cudaEventCreate(&e1))
    return fail(set_error(SGB_ERR_CUDA, "autotune snapshot failed"));
  // One candidate: restore, warm up, time n_steps.
  auto measure = [&](double* us) -> int {
    if (save(true)) return set_error(SGB_ERR_CUDA, "autotune restore failed");
    int r = sim_enqueue(s, std::max(1, n_steps / 4));
    if (r) return r;
    cudaEventRecord(e0, s.stream);
    r = sim_enqueue(s, n_steps);
    if (r) return r;
    cudaEventRecord(e1, s.stream);
    r = sim_sync(s);
    if (r) return r;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e0, e1)) return set_error(SGB_ERR_CUDA, "autotune timing failed");
    *us = 1000.0 * ms / n_steps;
    return SGB_OK;
  };
  // Projection groups: the j-th projection of every net with j projections.
  size_t max_proj = 0;
  for (const Network& net : s.nets) max_proj = std::max(max_proj, net.projs.size());
  modes.assign(s.projs.size(), SGB_PROP_CSR);
  for (size_t k = 0; k < s.projs.size(); ++k)
    if (!s.projs[k].ell_K) modes[k] = SGB_PROP_CSR;
  double best = 0;
  if ((rc = apply_modes(s, modes)) || (rc = measure(&best))) return fail(rc);
  for (size_t j = 0; j < max_proj; ++j) {
    std::vector<int32_t> trial = modes;
    bool any = false;
    for (size_t k = 0; k < s.ptab.size(); ++k)
      if ((size_t)s.ptab[k].proj == j && s.projs[k].ell_K) { trial[k] = SGB_PROP_ELL; any = true; }
    if (!any) continue;
    double us = 0;
    if ((rc = apply_modes(s, trial)) || (rc = measure(&us))) return fail(rc);
    if (us < best * 0.98) { best = us; modes = trial; }
  }
  if ((rc = apply_modes(s, modes))) return fail(rc);
  // Step driver.
  const int32_t other = s.cfg.exec_mode == SGB_EXEC_PERSISTENT ? SGB_EXEC_GRAPH : SGB_EXEC_PERSISTENT;
  const int32_t mine = s.cfg.exec_mode;
  s.cfg.exec_mode = other;
  for (auto& kv : s.graphs) cudaGraphExecDestroy(kv.second);
  s.graphs.clear();
  double us_other = 0;
  if ((rc = measure(&us_other))) return fail(rc);
  if (us_other < best * 0.98) best = us_other; else s.cfg.exec_mode = mine;
  for (auto& kv : s.graphs) cudaGraphExecDestroy(kv.second);
  s.graphs.clear();
  // Launch shapes for the chosen driver and modes, one dimension at a time:
  // the fused kernel's timeline and push-item width, the general kernel's
  // cells per lane, the per-step delivery grid, and the dense-pull variant.
  {
    TuneShape cur = current_shape(s);
    std::vector<TuneShape> cands;
    const bool persistent = s.cfg.exec_mode == SGB_EXEC_PERSISTENT;
    if (persistent && persistent_kernel_kind(s.args, s.persistent_blocks) == SGB_KERNEL_FUSED &&
        s.cfg.substeps == 1) {
      // The three timelines; the two late-push ones with each item width.
      for (int32_t tl = 0; tl <= 2; ++tl)
        for (int32_t w = 6; w <= (tl ? 7 : 6); ++w)
          if (tl != cur.ahead || w != cur.item_log2)
            cands.push_back({w, cur.deliver_mult, cur.pull_sum, tl, cur.lane_cells});
    }
    if (persistent && persistent_kernel_kind(s.args, s.persistent_blocks) == SGB_KERNEL_GENERAL &&
        general_one_barrier(s.args) && s.args.n_plast == 0)
      cands.push_back({cur.item_log2, cur.deliver_mult, cur.pull_sum, cur.ahead,
                       3 - cur.lane_cells});  // one or two cells per lane
    if (!persistent)
      for (int32_t m : {1, 4}) cands.push_back({cur.item_log2, m, cur.pull_sum, cur.ahead, cur.lane_cells});
    // The other dense-pull variants: no summary; summary; summary with
    // 16-byte entry loads (the per-step kernel; the persistent kernels treat 2 as 1).
    for (int32_t ps = 0; s.args.n_pull_units && ps <= 2; ++ps) {
      const bool ok = ps == 0 || s.pull_sum_fits;
      if (ok && ps != cur.pull_sum && (ps < 2 || !persistent)) cands.push_back({-1 - ps, -1, -1, -1, -1});
    }
    for (TuneShape c : cands) {
      if (c.item_log2 < 0)
        c = {cur.item_log2, cur.deliver_mult, -1 - c.item_log2, cur.ahead, cur.lane_cells};
      apply_shape(s, c);
      double us = 0;
      if ((rc = measure(&us))) return fail(rc);
      if (us < best * 0.98) { best = us; cur = c; }
    }
    apply_shape(s, cur);
    shape = cur;
  }
  if (save(true)) return fail(set_error(SGB_ERR_CUDA, "autotune restore failed"));
  // The restored state carries the deliveries in flight under the modes the
  // handle had before tuning.
  if ((rc = handover_modes(s, modes0))) return fail(rc);
  tune_cache_write(cache_path, sig, s.cfg.exec_mode, modes, shape, best);
  return fail(SGB_OK);
}

// Instrumented run: the per-step kernels launched one by one, each bracketed
// by CUDA events on the handle's stream, synchronised per step so that the
// spike and delivery counters of every step can be read.
int sim_profile(Sim& s, int32_t n_steps, double* mean_us, double* bytes, int64_t* launches) {
  if (n_steps < 1) return set_error(SGB_ERR_ARG, "n_steps must be >= 1");
  constexpr int K = SGB_KCLASS_COUNT;
  const StepArgs& a = s.args;
  const double W = s.bf16 ? 2.0 : 4.0;
  // Algorithmic bytes: update = state 12 B read + 12 B write + ring 8 B per
  // LIF cell, mask 4 B per input cell, 8 B per bitmap word (two history
  // copies), 8 B per push item written; deliver = per walked push synapse 4 B
  // word + W weight + 8 B atomic, 8 B per push item read; pull = 4 B per
  // stored dense entry plus, per entry whose pre cell spiked, W weight + 8 B
  // atomic; plasticity = per updated plastic synapse 4 B entry + 4 B value
  // read + 4 B value write + 4 B base weight + W table weight written (a rule
  // without a0 / a1_j updates only the rows of posts whose post / teacher
  // spike is set).
  double upd_bytes = (double)a.n_words * 8.0;
  for (const SegDev& d : s.segs) upd_bytes += d.kind == kSegLif ? 32.0 * d.count : 4.0 * d.count;
  double pull_entries = 0;
  for (const ProjDev& P : s.projs)
    if (P.mode == SGB_PROP_ELL) pull_entries += (double)P.ell_n;
  cudaEvent_t ev[2 * K];
  for (auto& e : ev) SGB_CUDA(cudaEventCreate(&e));
  double tot_ms[K] = {0}, tot_bytes[K] = {0};
  int64_t nl[K] = {0};
  Ctl before, after;
  int32_t done = 0;
  while (done < n_steps) {
    const uint32_t c = (uint32_t)std::min<int64_t>(s.chunk, n_steps - done);
    SGB_CUDA(cudaMemsetAsync(a.counts, 0, (size_t)c * a.n_segs * 4, s.stream));
    SGB_CUDA(launch_chunk_begin(a, s.stream));
    for (uint32_t i = 0; i < c; ++i) {
      SGB_CUDA(cudaMemcpyAsync(&before, a.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s.stream));
      SGB_CUDA(cudaEventRecord(ev[0], s.stream));
      SGB_CUDA(launch_update(a, s.stream));
      SGB_CUDA(cudaEventRecord(ev[1], s.stream));
      SGB_CUDA(cudaEventRecord(ev[6], s.stream));
      SGB_CUDA(launch_stdp(a, s.deliver_blocks, s.stream));
      SGB_CUDA(cudaEventRecord(ev[7], s.stream));
      SGB_CUDA(cudaEventRecord(ev[4], s.stream));
      SGB_CUDA(launch_pull(a, s.pull_blocks, s.stream));
      SGB_CUDA(cudaEventRecord(ev[5], s.stream));
      SGB_CUDA(cudaEventRecord(ev[2], s.stream));
      SGB_CUDA(launch_deliver(a, s.deliver_blocks, s.stream));
      SGB_CUDA(cudaEventRecord(ev[3], s.stream));
      SGB_CUDA(cudaMemcpyAsync(&after, a.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s.stream));
      SGB_CUDA(cudaStreamSynchronize(s.stream));
      const double items = (double)after.active_count[before.step & 1];
      const double walked = (double)(after.delivered - before.delivered);
      const double pulled = (double)(after.pulled - before.pulled);
      const double plast_upd = (double)(after.plast_updates - before.plast_updates);
      const double step_bytes[K] = {upd_bytes + items * 8.0, walked * (12.0 + W) + items * 8.0,
                                    pull_entries * 4.0 + pulled * (8.0 + W),
                                    plast_upd * (16.0 + W)};
      for (int k = 0; k < K; ++k) {
        if (k == 2 && !a.n_pull_units) continue;
        if (k == 3 && !a.n_plast) continue;
        float ms = 0.f;
        SGB_CUDA(cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]));
        tot_ms[k] += ms;
        tot_bytes[k] += step_bytes[k];
        nl[k]++;
      }
    }
    SGB_CUDA(launch_chunk_end(a, s.stream));
    s.launches += 2;
    done += (int32_t)c;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  for (int k = 0; k < K; ++k) {
    s.launches += nl[k];
    if (mean_us) mean_us[k] = nl[k] ? 1000.0 * tot_ms[k] / (double)nl[k] : 0.0;
    if (bytes) bytes[k] = nl[k] ? tot_bytes[k] / (double)nl[k] : 0.0;
    if (launches) launches[k] = nl[k];
  }
  return SGB_OK;
}

}  // namespace sgb

namespace sgb {

int sim_plastic_values(Sim& s, int32_t net, int32_t proj, float* values) {
  if (!values) return set_error(SGB_ERR_ARG, "values is NULL");
  for (const PlastHost& ph : s.plast) {
    if (ph.net != net || ph.proj != proj) continue;
    std::vector<float> v(std::max<size_t>(ph.cells, 1));
    SGB_CUDA(cudaStreamSynchronize(s.stream));
    SGB_CUDA(cudaMemcpy(v.data(), (char*)s.d_plast + ph.off_val, ph.cells * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < ph.cell_of_syn.size(); ++i) values[i] = v[ph.cell_of_syn[i]];
    return SGB_OK;
  }
  return set_error(SGB_ERR_ARG, "projection %d of net %d is not plastic", proj, net);
}

}  // namespace sgb

namespace sgb {

// ---------------------------------------------------------------------------
// Checkpoints: a header with a layout signature, then the device regions in
// a fixed order and the host copy of the stimulus sources.
namespace {
struct CkptHeader {
  char magic[8];          // "SGBCKPT1"
  uint64_t signature;     // layout hash (cells, delays, history, tables, plasticity)
  uint64_t bytes;         // whole checkpoint
};

struct CkptPart {
  void* dev;
  size_t n;
};

uint64_t ckpt_signature(const Sim& s) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (v >> (8 * i)) & 0xFFu;
      h *= 1099511628211ull;
    }
  };
  mix(s.n_pad);
  mix(s.ring_slots);
  mix(s.hist_rows);
  mix(s.segs.size());
  mix(s.srcs.size());
  mix(s.projs.size());
  mix(s.bf16 ? 1 : 0);
  for (const SegDev& d : s.segs) mix(((uint64_t)d.base << 32) | d.count);
  for (size_t k = 0; k < s.projs.size(); ++k) mix(((uint64_t)s.projs[k].ell_n << 32) ^ (uint64_t)s.ptab[k].nnz);
  for (const PlastHost& ph : s.plast) mix(((uint64_t)ph.k << 32) | ph.cells);
  return h;
}

std::vector<CkptPart> ckpt_parts(const Sim& s) {
  const StepArgs& a = s.args;
  std::vector<CkptPart> v = {{a.su, (size_t)s.n_pad * sizeof(float)},
                             {a.sg, (size_t)s.n_pad * sizeof(float2)},
                             {a.ring, (size_t)s.ring_slots * s.n_pad * 8},
                             {a.hist, s.hist_bytes},
                             {a.ctl, sizeof(Ctl)},
                             {a.totals, s.segs.size() * sizeof(double)}};
  const size_t wsz = s.bf16 ? 2 : 4;
  if (!s.plast.empty()) v.push_back({a.recent, (size_t)s.n_pad * 16});
  for (const PlastHost& ph : s.plast) {
    v.push_back({(char*)s.d_plast + ph.off_val, ph.cells * 4});
    v.push_back({const_cast<void*>(s.projs[ph.k].ell_w), ph.cells * wsz});
  }
  return v;
}
}  // namespace

int sim_checkpoint_size(const Sim& s, int64_t* bytes) {
  if (!bytes) return set_error(SGB_ERR_ARG, "bytes is NULL");
  size_t n = sizeof(CkptHeader) + s.srcs.size() * sizeof(SrcDev);
  for (const CkptPart& p : ckpt_parts(s)) n += p.n;
  *bytes = (int64_t)n;
  return SGB_OK;
}

int sim_checkpoint(Sim& s, void* buf, int64_t size, bool load) {
  if (!buf) return set_error(SGB_ERR_ARG, "buffer is NULL");
  int64_t need = 0;
  sim_checkpoint_size(s, &need);
  if (size < need)
    return set_error(SGB_ERR_ARG, "checkpoint buffer of %lld bytes, %lld needed", (long long)size,
                     (long long)need);
  char* p = (char*)buf;
  CkptHeader h;
  if (load) {
    memcpy(&h, p, sizeof h);
    if (memcmp(h.magic, "SGBCKPT1", 8) != 0) return set_error(SGB_ERR_FORMAT, "not a checkpoint");
    if (h.signature != ckpt_signature(s) || h.bytes != (uint64_t)need)
      return set_error(SGB_ERR_FORMAT, "checkpoint of a different network layout");
  } else {
    memcpy(h.magic, "SGBCKPT1", 8);
    h.signature = ckpt_signature(s);
    h.bytes = (uint64_t)need;
    memcpy(p, &h, sizeof h);
  }
  p += sizeof h;
  SGB_CUDA(cudaStreamSynchronize(s.stream));
  for (const CkptPart& part : ckpt_parts(s)) {
    if (load)
      SGB_CUDA(cudaMemcpy(part.dev, p, part.n, cudaMemcpyHostToDevice));
    else
      SGB_CUDA(cudaMemcpy(p, part.dev, part.n, cudaMemcpyDeviceToHost));
    p += part.n;
  }
  const size_t nsrc = s.srcs.size() * sizeof(SrcDev);
  if (load) {
    if (nsrc) {
      memcpy(s.srcs.data(), p, nsrc);
      memcpy(s.h_srcs, s.srcs.data(), nsrc);
      SGB_CUDA(cudaMemcpy((void*)s.args.srcs, s.h_srcs, nsrc, cudaMemcpyHostToDevice));
    }
  } else if (nsrc) {
    memcpy(p, s.srcs.data(), nsrc);
  }
  return SGB_OK;
}

}  // namespace sgb
