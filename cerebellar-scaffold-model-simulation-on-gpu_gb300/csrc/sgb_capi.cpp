// extern "C" entry points declared in include/scaffold_gb300.h.  Thin
// argument checks and exception fences around the host model (sgb_model.cpp)
// and the engine (sgb_engine.cu); no function here exits the process.
#include <algorithm>
#include <math.h>
#include <string.h>

#include <new>

#include "../../include/scaffold_gb300.h"
#include "sgb_engine.h"

using namespace sgb;

#define SGB_GUARD(...)                                                        \
  try {                                                                       \
    __VA_ARGS__                                                               \
  } catch (const std::bad_alloc&) {                                           \
    return set_error(SGB_ERR_NOMEM, "host allocation failed");                \
  } catch (const std::exception& ex) {                                        \
    return set_error(SGB_ERR_STATE, "internal error: %s", ex.what());         \
  }

extern "C" {

void sgb_config_init(sgb_config* cfg) {
  if (!cfg) return;
  memset(cfg, 0, sizeof *cfg);
  cfg->dt_ms = 0.1;
  cfg->substeps = 1;
  cfg->weight_type = SGB_WEIGHT_FP32;
  cfg->exec_mode = SGB_EXEC_GRAPH;
  cfg->chunk_steps = 1000;
  cfg->device = 0;
  cfg->default_prop = SGB_PROP_AUTO;
  cfg->raster = 0;
  cfg->blocks_per_sm = 0;
  cfg->l2_persist = 1;
}

const char* sgb_last_error(void) { return last_error(); }

int32_t sgb_abi_version(void) { return 3; }

int sgb_net_create(sgb_net** out) {
  if (!out) return set_error(SGB_ERR_ARG, "out is NULL");
  SGB_GUARD(*out = new sgb_net(); return SGB_OK;)
}

void sgb_net_destroy(sgb_net* net) { delete net; }

int sgb_net_add_population(sgb_net* net, const char* name, int32_t num, float Cm, float El,
                           float dt_ref, float Ie, float Vr, float Vth, float gL,
                           int32_t dev_type, int32_t c_num, const float* channels,
                           int32_t* pop_id) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  SGB_GUARD(return add_population(net->net, name, num, Cm, El, dt_ref, Ie, Vr, Vth, gL, dev_type,
                                  c_num, channels, pop_id);)
}

int sgb_net_add_projection_dat(sgb_net* net, const char* path, int32_t pre_pop,
                               int32_t post_pop, float initial_weight, int32_t delay_steps,
                               int32_t mode, int32_t* proj_id) {
  if (!net || !path) return set_error(SGB_ERR_ARG, "net or path is NULL");
  SGB_GUARD(return load_projection_dat(net->net, path, pre_pop, post_pop, initial_weight,
                                       delay_steps, mode, proj_id);)
}

int sgb_net_add_projection_arrays(sgb_net* net, int32_t pre_pop, int32_t post_pop,
                                  int64_t n_syn, const uint32_t* pre, const uint32_t* post,
                                  const float* weight, const uint8_t* delay, int32_t delay_all,
                                  int32_t channel, int32_t mode, int32_t* proj_id) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  if (n_syn < 0) return set_error(SGB_ERR_ARG, "negative synapse count");
  if (n_syn && (!pre || !post || !weight)) return set_error(SGB_ERR_ARG, "NULL synapse array");
  if (!delay && (delay_all < 1 || delay_all > kMaxDelay))
    return set_error(SGB_ERR_RANGE, "delay %d not in 1..%d steps", delay_all, kMaxDelay);
  SGB_GUARD({
    Projection pr;
    pr.pre = pre_pop;
    pr.post = post_pop;
    pr.channel = channel;
    pr.mode = mode;
    pr.pre_idx.assign(pre, pre + n_syn);
    pr.post_idx.assign(post, post + n_syn);
    pr.weight.assign(weight, weight + n_syn);
    if (delay)
      pr.delay.assign(delay, delay + n_syn);
    else
      pr.delay.assign((size_t)n_syn, (uint8_t)delay_all);
    return add_projection(net->net, std::move(pr), proj_id);
  })
}

int sgb_net_add_projection_random(sgb_net* net, int32_t pre_pop, int32_t post_pop,
                                  int32_t in_degree, float w_mean, float w_lo, float w_hi,
                                  int32_t d_min, int32_t d_max, int32_t channel, uint64_t seed,
                                  int32_t mode, int32_t* proj_id) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  SGB_GUARD(return add_random_projection(net->net, pre_pop, post_pop, in_degree, w_mean, w_lo,
                                         w_hi, d_min, d_max, channel, seed, mode, proj_id);)
}

int sgb_net_add_input(sgb_net* net, int32_t pop, int64_t n_ids, const uint32_t* ids,
                      const sgb_input_params* params, int32_t* src_id) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  SGB_GUARD(return add_input(net->net, pop, n_ids, ids, params, src_id);)
}

int sgb_net_add_input_dat(sgb_net* net, const char* path, int32_t pop,
                          const sgb_input_params* params, int32_t* src_id) {
  if (!net || !path) return set_error(SGB_ERR_ARG, "net or path is NULL");
  SGB_GUARD(return load_input_dat(net->net, path, pop, params, src_id);)
}

int sgb_net_build_scaffold(sgb_net* net, int32_t config, double scale, uint64_t seed) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  SGB_GUARD(return build_scaffold(net->net, config, scale, seed);)
}

int sgb_net_counts(const sgb_net* net, int32_t* n_pops, int32_t* n_projs, int32_t* n_inputs,
                   int64_t* n_neurons, int64_t* n_synapses) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  if (n_pops) *n_pops = (int32_t)net->net.pops.size();
  if (n_projs) *n_projs = (int32_t)net->net.projs.size();
  if (n_inputs) *n_inputs = (int32_t)net->net.inputs.size();
  if (n_neurons) *n_neurons = net->net.n_neurons();
  if (n_synapses) *n_synapses = net->net.n_synapses();
  return SGB_OK;
}

int sgb_net_population_info(const sgb_net* net, int32_t pop, sgb_population_info* info) {
  if (!net || !info) return set_error(SGB_ERR_ARG, "NULL argument");
  if (pop < 0 || pop >= (int32_t)net->net.pops.size())
    return set_error(SGB_ERR_ARG, "population %d out of range", pop);
  const Population& p = net->net.pops[pop];
  memset(info, 0, sizeof *info);
  info->num = p.num;
  info->dev_type = p.dev_type;
  info->c_num = p.c_num;
  for (const auto& pr : net->net.projs) info->n_in_projections += pr.post == pop;
  info->Cm = p.Cm; info->El = p.El; info->dt_ref = p.dt_ref; info->Ie = p.Ie;
  info->Vr = p.Vr; info->Vth = p.Vth; info->gL = p.gL;
  for (int c = 0; c < 2; ++c) {
    info->ch_w[c] = p.w[c]; info->ch_E[c] = p.E[c];
    info->ch_gbar[c] = p.gbar[c]; info->ch_tau[c] = p.tau[c];
  }
  strncpy(info->name, p.name.c_str(), sizeof info->name - 1);
  return SGB_OK;
}

int sgb_net_projection_info(const sgb_net* net, int32_t proj, sgb_projection_info* info) {
  if (!net || !info) return set_error(SGB_ERR_ARG, "NULL argument");
  if (proj < 0 || proj >= (int32_t)net->net.projs.size())
    return set_error(SGB_ERR_ARG, "projection %d out of range", proj);
  SGB_GUARD({
    const Projection& pr = net->net.projs[proj];
    memset(info, 0, sizeof *info);
    info->pre_pop = pr.pre;
    info->post_pop = pr.post;
    info->channel = pr.channel;
    info->mode = pr.mode;
    info->n_synapses = (int64_t)pr.pre_idx.size();
    std::vector<int32_t> in((size_t)net->net.pops[pr.post].num, 0),
        out((size_t)net->net.pops[pr.pre].num, 0);
    int dmin = 0, dmax = 0;
    for (size_t i = 0; i < pr.pre_idx.size(); ++i) {
      in[pr.post_idx[i]]++;
      out[pr.pre_idx[i]]++;
      const int d = pr.delay[i];
      dmin = (i == 0 || d < dmin) ? d : dmin;
      dmax = d > dmax ? d : dmax;
    }
    for (int32_t v : in) info->max_in_degree = v > info->max_in_degree ? v : info->max_in_degree;
    for (int32_t v : out) info->max_out_degree = v > info->max_out_degree ? v : info->max_out_degree;
    info->min_delay = dmin;
    info->max_delay = dmax;
    strncpy(info->name, pr.name.c_str(), sizeof info->name - 1);
    return SGB_OK;
  })
}

int sgb_net_projection_synapses(const sgb_net* net, int32_t proj, uint32_t* pre, uint32_t* post,
                                float* weight, uint8_t* delay) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  if (proj < 0 || proj >= (int32_t)net->net.projs.size())
    return set_error(SGB_ERR_ARG, "projection %d out of range", proj);
  const Projection& pr = net->net.projs[proj];
  const size_t n = pr.pre_idx.size();
  if (pre) memcpy(pre, pr.pre_idx.data(), n * 4);
  if (post) memcpy(post, pr.post_idx.data(), n * 4);
  if (weight) memcpy(weight, pr.weight.data(), n * 4);
  if (delay) memcpy(delay, pr.delay.data(), n);
  return SGB_OK;
}

int sgb_net_input_info(const sgb_net* net, int32_t src, sgb_input_info* info) {
  if (!net || !info) return set_error(SGB_ERR_ARG, "NULL argument");
  if (src < 0 || src >= (int32_t)net->net.inputs.size())
    return set_error(SGB_ERR_ARG, "source %d out of range", src);
  const InputSource& s = net->net.inputs[src];
  info->pop = s.pop;
  info->n_ids = (int32_t)s.ids.size();
  info->params = s.p;
  return SGB_OK;
}

int sgb_net_input_ids(const sgb_net* net, int32_t src, uint32_t* ids) {
  if (!net || !ids) return set_error(SGB_ERR_ARG, "NULL argument");
  if (src < 0 || src >= (int32_t)net->net.inputs.size())
    return set_error(SGB_ERR_ARG, "source %d out of range", src);
  const InputSource& s = net->net.inputs[src];
  memcpy(ids, s.ids.data(), s.ids.size() * 4);
  return SGB_OK;
}

int sgb_net_add_plasticity(sgb_net* net, int32_t proj, const sgb_plasticity_params* params) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  SGB_GUARD(return add_plasticity(net->net, proj, params);)
}

int sgb_net_plasticity_info(const sgb_net* net, int32_t proj, int32_t* plastic,
                            sgb_plasticity_params* params) {
  if (!net || !plastic) return set_error(SGB_ERR_ARG, "NULL argument");
  if (proj < 0 || proj >= (int32_t)net->net.projs.size())
    return set_error(SGB_ERR_ARG, "projection %d out of range", proj);
  const Projection& pr = net->net.projs[proj];
  *plastic = pr.plastic ? 1 : 0;
  if (params) {
    if (pr.plastic) *params = pr.plast; else memset(params, 0, sizeof *params);
  }
  return SGB_OK;
}

int sgb_net_write_projection_dat(const sgb_net* net, int32_t proj, const char* path) {
  if (!net || !path) return set_error(SGB_ERR_ARG, "net or path is NULL");
  SGB_GUARD(return write_projection_dat(net->net, proj, path);)
}

// ---------------------------------------------------------------------------
int sgb_sim_create(const sgb_config* cfg, sgb_net* const* nets, const uint64_t* seeds,
                   int32_t n_nets, sgb_sim** out) {
  if (!out) return set_error(SGB_ERR_ARG, "out is NULL");
  *out = nullptr;
  sgb_config c;
  if (cfg) c = *cfg; else sgb_config_init(&c);
  SGB_GUARD({
    Sim* s = nullptr;
    int rc = sim_create(c, nets, seeds, n_nets, &s);
    if (rc) return rc;
    *out = new sgb_sim{s};
    return SGB_OK;
  })
}

void sgb_sim_destroy(sgb_sim* sim) {
  if (!sim) return;
  delete sim->sim;
  delete sim;
}

#define SIM_CHECK(sim) \
  if (!(sim) || !(sim)->sim) return set_error(SGB_ERR_ARG, "sim is NULL")

int sgb_sim_set_stream(sgb_sim* sim, void* stream) {
  SIM_CHECK(sim);
  return sim_set_stream(*sim->sim, (cudaStream_t)stream);
}

int sgb_sim_set_input_rates(sgb_sim* sim, int32_t net, int32_t n, const float* rates_hz) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_set_rates(*sim->sim, net, n, rates_hz);)
}

int sgb_sim_run(sgb_sim* sim, int64_t n_steps, uint32_t* counts, uint32_t* raster_ids,
                int64_t raster_cap, int64_t* raster_offsets) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_run(*sim->sim, n_steps, counts, raster_ids, raster_cap, raster_offsets);)
}

int sgb_sim_enqueue(sgb_sim* sim, int64_t n_steps) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_enqueue(*sim->sim, n_steps);)
}

int sgb_sim_sync(sgb_sim* sim) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_sync(*sim->sim);)
}

int sgb_sim_reset(sgb_sim* sim, const uint64_t* seeds) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_reset(*sim->sim, seeds);)
}

int sgb_sim_get_info(const sgb_sim* sim, sgb_sim_info* info) {
  SIM_CHECK(sim);
  if (!info) return set_error(SGB_ERR_ARG, "info is NULL");
  const Sim& s = *sim->sim;
  memset(info, 0, sizeof *info);
  info->n_nets = (int32_t)s.nets.size();
  info->n_segments = (int32_t)s.segs.size();
  info->n_projections = (int32_t)s.projs.size();
  info->ring_slots = (int32_t)s.ring_slots;
  info->n_neurons = s.n_cells;
  info->n_synapses = s.n_syn;
  Ctl ctl;
  if (cudaStreamSynchronize(s.stream) != cudaSuccess ||
      cudaMemcpy(&ctl, s.args.ctl, sizeof ctl, cudaMemcpyDeviceToHost) != cudaSuccess)
    return set_error(SGB_ERR_CUDA, "reading the step counter failed");
  info->step = (int64_t)ctl.step;
  info->events = (int64_t)ctl.events;
  info->delivered = (int64_t)ctl.delivered;
  info->pulled = (int64_t)ctl.pulled;
  info->l2_persist_bytes = (int64_t)s.l2_setaside;
  for (const ProjDev& P : s.projs)
    if (P.mode == SGB_PROP_ELL) info->pull_entries += P.ell_n;
  info->step_kernel = s.cfg.exec_mode == SGB_EXEC_PERSISTENT
                          ? persistent_kernel_kind(s.args, s.persistent_blocks)
                          : SGB_KERNEL_GRAPH;
  info->push_smem_bytes = info->step_kernel == SGB_KERNEL_FUSED ? (int32_t)s.args.row_smem : 0;
  info->shard_cells = info->step_kernel == SGB_KERNEL_FUSED ? s.n_shard_cells : 0;
  info->item_width = 1 << fused_item_log2(s.args);
  info->deliver_blocks = s.deliver_blocks;
  info->pull_summary = (int32_t)s.args.pull_sum;
  info->spike_ahead = info->step_kernel == SGB_KERNEL_FUSED ? (int32_t)fused_timeline(s.args) : 0;
  info->lane_cells = (int32_t)s.args.lane_cells;
  info->device_bytes = (int64_t)(s.ell_bytes + s.push_bytes + s.misc_bytes);
  info->exec_mode = s.cfg.exec_mode;
  info->weight_type = s.cfg.weight_type;
  info->substeps = s.cfg.substeps;
  info->chunk_steps = (int32_t)s.chunk;
  info->dt_ms = s.cfg.dt_ms;
  return SGB_OK;
}

int sgb_sim_segment_info(const sgb_sim* sim, int32_t seg, sgb_segment_info* info) {
  SIM_CHECK(sim);
  const Sim& s = *sim->sim;
  if (!info) return set_error(SGB_ERR_ARG, "info is NULL");
  if (seg < 0 || seg >= (int32_t)s.segs.size()) return set_error(SGB_ERR_ARG, "segment %d out of range", seg);
  info->net = s.seg_net[seg];
  info->pop = s.seg_pop[seg];
  info->dev_type = s.nets[info->net].pops[info->pop].dev_type;
  info->count = (int32_t)s.segs[seg].count;
  info->first_id = s.seg_first_id[seg];
  for (int c = 0; c < 2; ++c) info->scale_bits[c] = -ilogbf(s.segs[seg].inv_scale[c]);
  return SGB_OK;
}

int sgb_sim_get_state(sgb_sim* sim, float* u, float* g, int32_t* ref) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_get_state(*sim->sim, u, g, ref);)
}

int sgb_sim_set_state(sgb_sim* sim, const float* u, const float* g, const int32_t* ref) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_set_state(*sim->sim, u, g, ref);)
}

int sgb_sim_spike_totals(sgb_sim* sim, double* totals) {
  SIM_CHECK(sim);
  return sim_totals(*sim->sim, totals);
}

int sgb_sim_set_propagation(sgb_sim* sim, int32_t net, int32_t proj, int32_t mode) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_set_mode(*sim->sim, net, proj, mode);)
}

int sgb_sim_get_propagation(const sgb_sim* sim, int32_t net, int32_t proj, int32_t* mode) {
  SIM_CHECK(sim);
  const Sim& s = *sim->sim;
  if (!mode) return set_error(SGB_ERR_ARG, "mode is NULL");
  if (net < 0 || net >= (int32_t)s.nets.size()) return set_error(SGB_ERR_ARG, "net %d out of range", net);
  if (proj < 0 || proj >= (int32_t)s.nets[net].projs.size())
    return set_error(SGB_ERR_ARG, "projection %d out of range", proj);
  *mode = (int32_t)s.projs[s.net_proj0[net] + proj].mode;
  return SGB_OK;
}

int sgb_sim_checkpoint_size(const sgb_sim* sim, int64_t* bytes) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_checkpoint_size(*sim->sim, bytes);)
}

int sgb_sim_save_checkpoint(sgb_sim* sim, void* buf, int64_t capacity) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_checkpoint(*sim->sim, buf, capacity, false);)
}

int sgb_sim_load_checkpoint(sgb_sim* sim, const void* buf, int64_t size) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_checkpoint(*sim->sim, const_cast<void*>(buf), size, true);)
}

int sgb_sim_plastic_values(sgb_sim* sim, int32_t net, int32_t proj, float* values) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_plastic_values(*sim->sim, net, proj, values);)
}

int sgb_sim_autotune(sgb_sim* sim, int32_t n_steps, const char* cache_path) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_autotune(*sim->sim, n_steps, cache_path);)
}

int sgb_sim_launch_count(const sgb_sim* sim, int64_t* launches) {
  SIM_CHECK(sim);
  if (!launches) return set_error(SGB_ERR_ARG, "launches is NULL");
  *launches = sim->sim->launches;
  return SGB_OK;
}

int sgb_sim_profile(sgb_sim* sim, int32_t n_steps, double* mean_us, double* bytes_per_launch,
                    int64_t* launches) {
  SIM_CHECK(sim);
  SGB_GUARD(return sim_profile(*sim->sim, n_steps, mean_us, bytes_per_launch, launches);)
}

}  // extern "C"
