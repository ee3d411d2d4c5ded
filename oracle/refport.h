/*
 * Restatement of the reference's own CPU path -- TEST INFRASTRUCTURE ONLY.
 *
 * host_update_lif_ch and host_spike_propagation (Simulation_header.cu:385-493)
 * are the reference's CPU loops for the path: a dense pull over every stored
 * synapse of every projection each step, and the LIF update in the
 * reference's mixed precision (FP32 state, double DT).  rp_* restates those
 * loops in C with OpenMP over post cells; it is the timed CPU baseline on
 * machines where the reference itself cannot be compiled, and a test pins it
 * bit for bit to the reference's compiled functions (ref_harness.cu) where
 * they can.
 *
 * Per-synapse delays are handled the way the reference handles one delay
 * per projection (GPUScaffoldSimulation.cu:734-735): each projection is split
 * into one ELL table per delay value, each read from spike row t - delay.
 */
#ifndef SGB_REFPORT_H
#define SGB_REFPORT_H
#include <stdint.h>

#include "oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rp_tab {
  int32_t proj, pre, post, channel, delay, max_conv;
  int32_t* cind;  /* [post_num][max_conv], -1 padded, population-local pre ids */
  float* w;       /* [post_num][max_conv] */
} rp_tab;

typedef struct rp_sim {
  orc_net net;
  orc_sim* inputs;   /* input-cell stimulus (same Philox streams as the oracle) */
  int64_t N;
  int64_t* base;     /* [n_pops + 1] */
  int32_t R;         /* spike ring rows: max delay + 1 */
  int32_t n_tabs;
  rp_tab* tabs;
  float *u, *g, *dg_exc, *dg_inh, *Inoise;
  int32_t* ref;
  char* spk;         /* [R][N] */
  uint64_t step;
} rp_sim;

int rp_create(const orc_net* net, rp_sim** out);
void rp_destroy(rp_sim* s);
/* Same outputs as orc_run; `threads` OpenMP threads (0: all). */
int rp_run(rp_sim* s, int64_t n_steps, int32_t threads, uint32_t* counts, uint32_t* raster,
           int64_t raster_cap, int64_t* raster_off);
int rp_get_state(const rp_sim* s, float* u, float* g, int32_t* ref);
/* Shared by rp_run and the compiled-reference harness: step inputs and
 * bookkeeping around the two compute loops. */
void rp_begin_step(rp_sim* s, char* row);
int rp_end_step(rp_sim* s, const char* row, int64_t step, uint32_t* counts, uint32_t* raster,
                int64_t raster_cap, int64_t* rfill);

#ifdef __cplusplus
}
#endif
#endif
