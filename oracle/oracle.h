/*
 * CPU oracle of the scaffold simulation hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only to check or time against the CUDA path; the
 * product never calls it.
 *
 * A plain-C restatement of the reference's per-step algorithm:
 *   input cells   InputStimulation + PoissonProcess / PeriodicFiring
 *                 (UserInputFunctions.cu:4-10, 86-120), with the random draw
 *                 keyed on (seed, neuron, step) instead of a cuRAND state;
 *   LIF cells     update_lif_ch / host_update_lif_ch
 *                 (Simulation_header.cu:305-381, 385-465);
 *   propagation   spike_propagation / host_spike_propagation
 *                 (Simulation_header.cu:83-101, 468-493) with per-synapse
 *                 delays, restated as delivery of each spike into the
 *                 accumulator of step t + delay;
 *   plasticity    Hebb_plasticity / Teacher_plasticity (SynapticPlasticity.cu:
 *                 40-120), applied after the cells of step t; a plastic
 *                 projection is delivered on arrival (the spike of step
 *                 t + 1 - d into the accumulator of t + 1, after step t's
 *                 plasticity), as the reference reads it d steps late.
 *                 The reference has this code switched off and no test of
 *                 it: this part of the oracle is unpinned.
 * Two arithmetic modes:
 *   ORC_FP32  the FP32 formulation of the CUDA kernels, one rounding per
 *             operation (compiled with -ffp-contract=off), fixed-point
 *             increment sums -- bit-identical to the device when the code
 *             is right;
 *   ORC_FP64  the same equations in double precision with exact double
 *             increment sums and unrounded (FP32) weights.
 */
#ifndef SGB_ORACLE_H
#define SGB_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_FP32 0
#define ORC_FP64 1

typedef struct orc_pop {
  int32_t num, is_input;
  float Cm, El, dt_ref, Ie, Vr, Vth, gL;
  int32_t c_num;
  float w[2], E[2], gbar[2], tau[2];
} orc_pop;

typedef struct orc_proj {
  int32_t pre, post, channel, pad_;
  int64_t n;
  const uint32_t* pre_idx;
  const uint32_t* post_idx;
  const float* weight;
  const uint8_t* delay;
} orc_proj;

typedef struct orc_src {
  int32_t pop, kind;
  float rate_hz, pad_;
  double phase_ms, win_period_ms, win_start_ms, win_end_ms;
  int64_t n_ids;
  const uint32_t* ids;
} orc_src;

/* Plasticity of one projection (SynapticPlasticity.cu:40-120): rule 0 Hebb,
 * 1 Teacher; constant coefficients; values clamped to [0, v_max]. */
typedef struct orc_plast {
  int32_t proj, rule, teacher_proj, window;
  float a0, a1_i, a1_j, a2_ji, v_max, pad_;
} orc_plast;

typedef struct orc_net {
  int32_t n_pops, n_projs, n_srcs, substeps;
  const orc_pop* pops;
  const orc_proj* projs;
  const orc_src* srcs;
  double dt_ms;
  uint64_t seed;
  int32_t bf16, mode;
  int32_t n_plast, pad_;
  const orc_plast* plast;
} orc_net;

typedef struct orc_sim orc_sim;

/* Philox4x32-10 of one counter block. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Largest S <= 30 such that every post cell's sum of rint(w * 2^S) fits int32. */
int32_t orc_scale_bits(const orc_net* net, int32_t pop, int32_t channel);

int orc_create(const orc_net* net, orc_sim** out);
void orc_destroy(orc_sim* s);
/* rates: one per source of the net (the net's source order). */
int orc_set_rates(orc_sim* s, const float* rates);
/* Advances n steps.  counts[n][n_pops]; raster ids (ascending within a step),
 * raster_off[n+1] relative to this call; any output may be NULL. */
int orc_run(orc_sim* s, int64_t n_steps, uint32_t* counts, uint32_t* raster, int64_t raster_cap,
            int64_t* raster_off);
/* State in global-id order (INPUT cells report zeros). */
int orc_get_state(const orc_sim* s, float* u, float* g, int32_t* ref);
int orc_set_state(orc_sim* s, const float* u, const float* g, const int32_t* ref);
int64_t orc_events(const orc_sim* s);
/* Plasticity values of plastic projection `proj` (the net's projection index),
 * in its synapse order; -1 if it is not plastic. */
int orc_plastic_values(const orc_sim* s, int32_t proj, float* values);
/* Input-cell spike flags of step t (1 byte per cell in global-id order; LIF
 * cells are left untouched).  Does not advance the simulation. */
int orc_input_flags(const orc_sim* s, uint64_t t, uint8_t* flags);

/* Synthetic benchmark networks (netgen.c): one fixed in-degree projection
 * drawn from `seed` into caller arrays of npost * in_degree entries, and the
 * scaffold architecture of configurations 1, 2 and 5. */
int orc_random_projection(int64_t npre, int64_t npost, int32_t in_degree, float w_mean,
                          float w_lo, float w_hi, int32_t d_min, int32_t d_max, uint64_t seed,
                          uint32_t* pre_idx, uint32_t* post_idx, float* weight, uint8_t* delay);
int orc_scaffold_spec(int32_t config, double scale, int32_t* sizes, int32_t* proj, float* drive,
                      int32_t* burst_n);

#ifdef __cplusplus
}
#endif
#endif
