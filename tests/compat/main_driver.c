/* A driver written like the reference's main.cu (SimulationModule/Scaffold/
 * main.cu:17-75): trials of T_MAX ms in chunks of T_cpu_sim, the six
 * environment calls, the DCN spike flags of each chunk summed.  Built and run
 * by tests/test_gpu_reference_mode.py against scaffold_compat.h. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "scaffold_compat.h"

#define T_MAX 1000
#define INPUT_STIM_NUM 2

static void CalcFreq(float* freq_list, int t) {
  freq_list[0] = 4.f;
  freq_list[1] = (30.f - 4) / 2 * (1 - cosf(2 * 3.14159265f * ((float)t / 1000.f) / 2.f));
}

int main(int argc, char** argv) {
  int trials = argc > 1 ? atoi(argv[1]) : 1;
  int T_cpu_sim = argc > 2 ? atoi(argv[2]) : 25;
  int T_print = argc > 3 ? atoi(argv[3]) : 50;
  char* spike_train = NULL;
  NetworkEnvironment Env;
  CreateNetworkEnv(&Env, 1, 7, 16, INPUT_STIM_NUM, 0);
  InitializeNetworkEnv(&Env, T_print, T_cpu_sim);
  fprintf(stderr, "neuron_num = %d\n", Env.Host_sim_val[0].Host.neuron_num);
  float freq_list[INPUT_STIM_NUM];
  long dcn_spikes = 0;
  for (int trial = 0; trial < trials; trial++) {
    int t = 0;
    while (t < T_MAX) {
      CalcFreq(freq_list, t);
      SetInputFreq(&Env, freq_list);
      loop_n_steps(&Env, t, T_cpu_sim, trial, &spike_train);
      for (int k = 0; k < T_cpu_sim * Env.n_output; ++k) dcn_spikes += spike_train[k];
      t += T_cpu_sim;
    }
    ResetNetworkEnv(&Env, trial);
  }
  FinalizeNetworkEnv(&Env);
  printf("dcn_spikes %ld\n", dcn_spikes);
  return 0;
}
