/*
 * scaffold_compat.h -- the reference's six driver calls on top of scaffold_gb300.h.
 *
 * A main.cu-style driver of the reference (SimulationModule/Scaffold/main.cu)
 * compiles against this header unchanged at its call sites: the names,
 * arguments and behaviour of CreateNetworkEnv, InitializeNetworkEnv,
 * loop_n_steps, SetInputFreq, ResetNetworkEnv and FinalizeNetworkEnv
 * (GPUScaffoldSimulation.h:40-47) are kept, including the reference's
 * handling of errors (message on stderr, process exit).  The network is the
 * reference's hard-coded scaffold (init_params.cu:367-766) read from .dat files
 * in the directory named by the SGB_DAT_DIR environment variable (default:
 * the working directory, where the reference reads them), simulated with the
 * reference's 1-ms exchange step of 10 substeps of 0.1 ms.  Rasters are
 * written in the reference's text format to spike_output/.  The reference's
 * own main.cu also takes constants and enumerations from its
 * GPUScaffoldSimulation.h: include/compat/GPUScaffoldSimulation.h provides
 * them under that name.
 */
#ifndef SCAFFOLD_COMPAT_H
#define SCAFFOLD_COMPAT_H

#include "scaffold_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The part of the reference's per-device record (cpu_sim_thread_val /
 * Sim_cond_lif_exp, struct_enum_def.h:132-171) that its driver reads:
 * Env.Host_sim_val[0].Host.neuron_num, the cells of the (one) device. */
typedef struct sgb_compat_host {
  int neuron_num;
} sgb_compat_host;
typedef struct sgb_compat_sim_val {
  sgb_compat_host Host;
} sgb_compat_sim_val;

typedef struct NetworkEnvironment {
  sgb_compat_sim_val Host_sim_val[1];  /* set by InitializeNetworkEnv */
  sgb_net* net;
  sgb_sim* sim;
  int num_of_neuron_types, num_of_connectivity_types, num_of_inputs;
  int T_print, T_cpu_sim;
  uint64_t seed;
  char dat_dir[512];
  char out_dir[512];
  char* output_spike_train;  /* [T_cpu_sim][DCN cells] spike flags of the last chunk */
  int32_t n_output;
  uint32_t* raster_ids;
  int64_t* raster_off;
  int64_t raster_cap;
  int resets;
  float freq[8];
} NetworkEnvironment;

void CreateNetworkEnv(NetworkEnvironment* env, int num_of_dev, int num_of_neuron_types,
                      int num_of_connectivity_types, int num_of_inputs, int num_of_plasticities);
void InitializeNetworkEnv(NetworkEnvironment* env, int T_print, int T_cpu_sim);
void loop_n_steps(NetworkEnvironment* env, int start_step, int n_steps, int trial,
                  char** output_spike_train);
void SetInputFreq(NetworkEnvironment* env, const float* freq_list);
void ResetNetworkEnv(NetworkEnvironment* env, int trial);
void FinalizeNetworkEnv(NetworkEnvironment* env);

#ifdef __cplusplus
}
#endif
#endif /* SCAFFOLD_COMPAT_H */
