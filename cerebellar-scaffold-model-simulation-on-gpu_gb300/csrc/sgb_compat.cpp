// Reference-structure mode and the reference-named driver API.
//
//  * sgb_net_build_reference_scaffold: the reference's hard-coded 96,737-cell
//    scaffold (init_neurons_params / init_connectivity_params,
//    init_params.cu:367-766) over .dat files in the reference's names and
//    format, with its stimulus lists (UserInputFunctions.cu:72-81).
//  * sgb_sim_write_raster: spike rasters in the reference's text format
//    "t\tlocal_id\ttype_id" (GPUScaffoldSimulation.cu:81).
//  * CreateNetworkEnv ... FinalizeNetworkEnv (include/scaffold_compat.h): the
//    six calls a main.cu-style driver makes (GPUScaffoldSimulation.h:40-47),
//    with the reference's behaviour on error (message on stderr, exit).
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/scaffold_compat.h"
#include "../../include/scaffold_gb300.h"
#include "sgb_engine.h"

using namespace sgb;

namespace {

// Populations in the reference's array order: NORMAL types first, then the
// CPU-side types from the end (set_neuron_params, init_params.cu:255-270).
struct RefPop {
  const char* name;
  int32_t num, dev_type, enum_id;  // enum_id: NeuronType (struct_enum_def.h:10-20)
  float Cm, El, dt_ref, Ie, Vr, Vth, gL;
  float ch[8];
};
const RefPop kRefPops[] = {
    {"granule_cell", 88158, SGB_NORMAL, 0, 3.0f, -74.0f, 1.5f, 0.0f, -84.0f, -42.0f, 1.5f,
     {1.f, 0.f, 1.f, 0.5f, 1.f, -85.f, 1.f, 10.f}},
    {"purkinje_cell", 69, SGB_NORMAL, 2, 620.0f, -62.0f, 0.8f, 600.0f, -72.0f, -47.0f, 7.0f,
     {1.f, 0.f, 1.f, 0.5f, 1.f, -85.f, 1.f, 1.6f}},
    {"golgi_cell", 219, SGB_NORMAL, 3, 76.0f, -65.0f, 2.0f, 36.75f, -75.0f, -55.0f, 3.6f,
     {1.f, 0.f, 1.f, 0.5f, 1.f, -85.f, 1.f, 15.f}},
    {"stellate_cell", 603, SGB_NORMAL, 4, 14.6f, -68.0f, 1.6f, 15.6f, -78.0f, -53.0f, 1.0f,
     {1.f, 0.f, 1.f, 0.64f, 1.f, -85.f, 1.f, 2.f}},
    {"basket_cell", 603, SGB_NORMAL, 5, 14.6f, -68.0f, 1.6f, 15.6f, -78.0f, -53.0f, 1.0f,
     {1.f, 0.f, 1.f, 0.64f, 1.f, -85.f, 1.f, 2.f}},
    {"dcn_cell", 12, SGB_OUTPUT, 6, 89.0f, -59.0f, 3.7f, 55.8f, -69.0f, -48.0f, 1.56f,
     {1.f, 0.f, 1.f, 7.1f, 4.f, -85.f, 1.f, 13.6f}},
    {"glomerulus", 7073, SGB_INPUT, 1, 0, 0, 0, 0, 0, 0, 0, {0}},
};
enum { kGrC = 0, kPC, kGoC, kSC, kBC, kDCN, kGlom, kRefPopCount };

struct RefProj {
  const char* file;
  int32_t pre, post;
  float weight, delay_ms;
};
// init_connectivity_params (init_params.cu:531-766), in its order.
const RefProj kRefProjs[] = {
    {"parallel_fiber_to_purkinje.dat", kGrC, kPC, 0.02f, 5.0f},
    {"parallel_fiber_to_golgi.dat", kGrC, kGoC, 0.4f, 5.0f},
    {"parallel_fiber_to_stellate.dat", kGrC, kSC, 0.2f, 5.0f},
    {"parallel_fiber_to_basket.dat", kGrC, kBC, 0.2f, 5.0f},
    {"ascending_axon_to_golgi.dat", kGrC, kGoC, 20.0f, 2.0f},
    {"ascending_axon_to_purkinje.dat", kGrC, kPC, 75.0f, 2.0f},
    {"golgi_to_golgi.dat", kGoC, kGoC, -8.0f, 1.0f},
    {"stellate_to_stellate.dat", kSC, kSC, -2.0f, 1.0f},
    {"basket_to_basket.dat", kBC, kBC, -2.5f, 1.0f},
    {"glomerulus_to_dcn.dat", kGlom, kDCN, 0.006f, 4.0f},
    {"purkinje_to_dcn.dat", kPC, kDCN, -0.0075f, 4.0f},
    {"basket_to_purkinje.dat", kBC, kPC, -9.0f, 4.0f},
    {"stellate_to_purkinje.dat", kSC, kPC, -8.5f, 5.0f},
    {"glomerulus_to_granule.dat", kGlom, kGrC, 9.0f, 4.0f},
    {"glomerulus_to_golgi.dat", kGlom, kGoC, 2.0f, 4.0f},
    {"golgi_to_granule.dat", kGoC, kGrC, -5.0f, 2.0f},
};

std::string join(const char* dir, const char* file) {
  std::string p = dir && *dir ? dir : ".";
  if (p.back() != '/') p += '/';
  return p + file;
}

}  // namespace

extern "C" int sgb_net_build_reference_scaffold(sgb_net* net, const char* dat_dir,
                                                const int32_t* sizes) {
  if (!net) return set_error(SGB_ERR_ARG, "net is NULL");
  if (!net->net.pops.empty()) return set_error(SGB_ERR_STATE, "network must be empty");
  try {
    for (int p = 0; p < kRefPopCount; ++p) {
      const RefPop& r = kRefPops[p];
      const int32_t num = sizes ? sizes[p] : r.num;
      const int rc = add_population(net->net, r.name, num, r.Cm, r.El, r.dt_ref, r.Ie, r.Vr,
                                    r.Vth, r.gL, r.dev_type, r.dev_type == SGB_INPUT ? 0 : 2,
                                    r.dev_type == SGB_INPUT ? nullptr : r.ch, nullptr);
      if (rc) return rc;
    }
    for (const RefProj& pr : kRefProjs) {
      // Delays are whole ms; with the reference's 1-ms exchange step (10
      // substeps of 0.1 ms) they are exchange steps.
      const int rc = load_projection_dat(net->net, join(dat_dir, pr.file).c_str(), pr.pre,
                                         pr.post, pr.weight, (int32_t)pr.delay_ms,
                                         SGB_PROP_AUTO, nullptr);
      if (rc) return rc;
    }
    // background_noise: Poisson 1 Hz (UserInputFunctions.cu:19-23);
    // tone_stim: periodic 140 Hz from 292.8 ms inside [300, 351) ms, or
    // Poisson 1 Hz (:25-29).
    const sgb_input_params bg{SGB_INPUT_POISSON, 1.0f, 0.0, 0.0, 0.0, 0.0};
    const sgb_input_params tone{SGB_INPUT_PERIODIC, 140.0f, 292.8, 0.0, 300.0, 351.0};
    int rc = load_input_dat(net->net, join(dat_dir, "background_noise.dat").c_str(), kGlom, &bg,
                            nullptr);
    if (rc) return rc;
    rc = load_input_dat(net->net, join(dat_dir, "tone_stim.dat").c_str(), kGlom, &tone, nullptr);
    if (rc) return rc;
    return load_input_dat(net->net, join(dat_dir, "tone_stim.dat").c_str(), kGlom, &bg, nullptr);
  } catch (const std::bad_alloc&) {
    return set_error(SGB_ERR_NOMEM, "host allocation failed");
  }
}

extern "C" int32_t sgb_reference_type_id(int32_t pop) {
  return pop >= 0 && pop < kRefPopCount ? kRefPops[pop].enum_id : -1;
}

extern "C" int sgb_sim_write_raster(const sgb_sim* sim, const char* path, const uint32_t* ids,
                                    const int64_t* offsets, int64_t n_steps, int64_t first_step,
                                    const int32_t* type_ids, int32_t append) {
  if (!sim || !sim->sim || !path) return set_error(SGB_ERR_ARG, "NULL argument");
  if (n_steps < 0 || (n_steps && (!ids || !offsets)))
    return set_error(SGB_ERR_ARG, "raster arrays missing");
  const Sim& s = *sim->sim;
  FILE* f = fopen(path, append ? "ab" : "wb");
  if (!f) return set_error(SGB_ERR_IO, "cannot open '%s': %s", path, strerror(errno));
  const double step_ms = s.cfg.dt_ms * s.cfg.substeps;
  const size_t nseg = s.segs.size();
  for (int64_t k = 0; k < n_steps; ++k) {
    const float t = (float)((double)(first_step + k) * step_ms);
    for (int64_t q = offsets[k]; q < offsets[k + 1]; ++q) {
      const int64_t id = ids[q];
      // Segment of a global id: last segment whose first id <= id.
      const size_t seg =
          (size_t)(std::upper_bound(s.seg_first_id.begin(), s.seg_first_id.end(), id) -
                   s.seg_first_id.begin()) - 1;
      if (seg >= nseg) continue;
      const int32_t pop = s.seg_pop[seg];
      fprintf(f, "%f\t%lld\t%d\n", t, (long long)(id - s.seg_first_id[seg]),
              type_ids ? type_ids[pop] : pop);
    }
  }
  if (fclose(f)) return set_error(SGB_ERR_IO, "write to '%s' failed", path);
  return SGB_OK;
}

// ---------------------------------------------------------------------------
// Reference-named driver API.
namespace {
void die(const char* what) {
  fprintf(stderr, "[Error] %s: %s\n", what, sgb_last_error());
  exit(1);
}
}  // namespace

extern "C" {

void CreateNetworkEnv(NetworkEnvironment* env, int num_of_dev, int num_of_neuron_types,
                      int num_of_connectivity_types, int num_of_inputs,
                      int num_of_plasticities) {
  (void)num_of_dev;
  (void)num_of_plasticities;
  if (!env) die("CreateNetworkEnv");
  memset(env, 0, sizeof *env);
  env->num_of_neuron_types = num_of_neuron_types;
  env->num_of_connectivity_types = num_of_connectivity_types;
  env->num_of_inputs = num_of_inputs;
  const char* dir = getenv("SGB_DAT_DIR");
  snprintf(env->dat_dir, sizeof env->dat_dir, "%s", dir ? dir : ".");
  snprintf(env->out_dir, sizeof env->out_dir, "spike_output");
  env->seed = 1;
  if (sgb_net_create(&env->net)) die("CreateNetworkEnv");
}

void InitializeNetworkEnv(NetworkEnvironment* env, int T_print, int T_cpu_sim) {
  if (!env || !env->net) die("InitializeNetworkEnv");
  if (T_print < T_cpu_sim || T_cpu_sim < 1 || T_print % T_cpu_sim) {
    fprintf(stderr, "Consistency between T_print and T_cpu_sim is corrupt.\n "
                    "T_print must be multiples of T_cpu_sim\n");
    exit(1);
  }
  env->T_print = T_print;
  env->T_cpu_sim = T_cpu_sim;
  if (sgb_net_build_reference_scaffold(env->net, env->dat_dir, nullptr))
    die("InitializeNetworkEnv");
  sgb_config cfg;
  sgb_config_init(&cfg);
  cfg.dt_ms = 0.1;     // DT (option.h:4)
  cfg.substeps = 10;   // STEP_MAX (option.h:6)
  cfg.chunk_steps = T_cpu_sim;
  cfg.raster = 1;
  if (sgb_sim_create(&cfg, &env->net, &env->seed, 1, &env->sim)) die("InitializeNetworkEnv");
  sgb_sim_info si;
  if (sgb_sim_get_info(env->sim, &si)) die("InitializeNetworkEnv");
  env->Host_sim_val[0].Host.neuron_num = (int)si.n_neurons;
  sgb_population_info pi;
  sgb_net_population_info(env->net, kDCN, &pi);
  const int32_t n_out = pi.num;
  env->n_output = n_out;
  env->output_spike_train = (char*)calloc((size_t)T_cpu_sim * (n_out > 0 ? n_out : 1), 1);
  env->raster_cap = (int64_t)T_cpu_sim * 200000;
  env->raster_ids = (uint32_t*)malloc((size_t)env->raster_cap * sizeof(uint32_t));
  env->raster_off = (int64_t*)malloc((size_t)(T_cpu_sim + 1) * sizeof(int64_t));
  if (!env->output_spike_train || !env->raster_ids || !env->raster_off) {
    fprintf(stderr, "[Error] InitializeNetworkEnv: out of host memory\n");
    exit(1);
  }
  mkdir(env->out_dir, 0755);
  ResetNetworkEnv(env, 0);
}

void SetInputFreq(NetworkEnvironment* env, const float* freq_list) {
  // Stored per input list as the reference does (GPUScaffoldSimulation.cu:883-890);
  // its stimulus functions never read it (background_noise and tone_stim use
  // fixed rates, UserInputFunctions.cu:19-29), so the rates stay as defined.
  if (!env || !freq_list) return;
  for (int i = 0; i < env->num_of_inputs && i < 8; ++i) env->freq[i] = freq_list[i];
}

void loop_n_steps(NetworkEnvironment* env, int start_step, int n_steps, int trial,
                  char** output_spike_train) {
  (void)trial;
  if (!env || !env->sim) die("loop_n_steps");
  if (n_steps > env->T_cpu_sim) {
    fprintf(stderr, "[Error] loop_n_steps: n_steps %d exceeds T_cpu_sim %d\n", n_steps,
            env->T_cpu_sim);
    exit(1);
  }
  if (sgb_sim_run(env->sim, n_steps, nullptr, env->raster_ids, env->raster_cap, env->raster_off))
    die("loop_n_steps");
  int32_t type_ids[kRefPopCount];
  for (int p = 0; p < kRefPopCount; ++p) type_ids[p] = kRefPops[p].enum_id;
  char path[600];
  snprintf(path, sizeof path, "%s/spike_dev0_0.dat", env->out_dir);
  if (sgb_sim_write_raster(env->sim, path, env->raster_ids, env->raster_off, n_steps, start_step,
                           type_ids, 1))
    die("loop_n_steps");
  // OUTPUT-population spike flags of the chunk, [step][output cell], as the
  // reference's CPU side returns them (GPUScaffoldSimulation.cu:777).
  sgb_segment_info si;
  sgb_sim_segment_info(env->sim, kDCN, &si);
  memset(env->output_spike_train, 0, (size_t)env->T_cpu_sim * (env->n_output > 0 ? env->n_output : 1));
  for (int k = 0; k < n_steps; ++k)
    for (int64_t q = env->raster_off[k]; q < env->raster_off[k + 1]; ++q) {
      const int64_t id = env->raster_ids[q];
      if (id >= si.first_id && id < si.first_id + si.count)
        env->output_spike_train[(size_t)k * env->n_output + (id - si.first_id)] = 1;
    }
  if (output_spike_train) *output_spike_train = env->output_spike_train;
}

void ResetNetworkEnv(NetworkEnvironment* env, int trial) {
  if (!env || !env->sim) die("ResetNetworkEnv");
  char src[600], dst[600];
  snprintf(src, sizeof src, "%s/spike_dev0_0.dat", env->out_dir);
  if (env->resets > 0) {
    snprintf(dst, sizeof dst, "%s/spike_result_trial%d.dat", env->out_dir, trial);
    rename(src, dst);
  }
  FILE* f = fopen(src, "wb");
  if (f) fclose(f);
  env->resets++;
  if (sgb_sim_reset(env->sim, nullptr)) die("ResetNetworkEnv");
}

void FinalizeNetworkEnv(NetworkEnvironment* env) {
  if (!env) return;
  sgb_sim_destroy(env->sim);
  sgb_net_destroy(env->net);
  free(env->output_spike_train);
  free(env->raster_ids);
  free(env->raster_off);
  env->sim = nullptr;
  env->net = nullptr;
}

}  // extern "C"
