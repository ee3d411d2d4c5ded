/*
 * scaffold_gb300.h -- C ABI of the GB300 cerebellar-scaffold simulation hot path.
 *
 * This is the drop-in boundary for the reference simulator's per-timestep loop
 * (Rkuriyama/Cerebellar-Scaffold-Model-Simulation-on-GPU, directory
 * SimulationModule/Scaffold/).  Every entry point below names the reference
 * interface it replaces.  All functions are plain C: opaque handles, plain
 * pointers and sizes, no CUDA or torch types.  Every function returns an int
 * status (SGB_OK == 0, negative on error) and never exits the process; the
 * text of the last error on the calling thread is available from
 * sgb_last_error().  (The reference calls exit() from CUDA_SAFE_CALL,
 * Simulation_header.h:11-18, and from its file loaders, init_params.cu:33-36.)
 *
 * Ownership: the library owns every device buffer behind a handle; every host
 * buffer passed in is owned by the caller and only read or written during the
 * call.  A handle is single-thread-affine; independent handles may be driven
 * from different threads and streams.
 *
 * Units: times in milliseconds, rates in Hz, potentials in mV, capacitances in
 * pF, conductances in nS (the reference's units, init_params.cu:367-529).  One
 * "step" is one exchange step of `substeps` Euler substeps of `dt_ms` each:
 * spikes are exchanged once per step and synaptic delays count steps.
 */
#ifndef SCAFFOLD_GB300_H
#define SCAFFOLD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SGB_OK 0
#define SGB_ERR_ARG (-1)          /* invalid argument or out-of-range index     */
#define SGB_ERR_IO (-2)           /* file cannot be opened or read              */
#define SGB_ERR_FORMAT (-3)       /* malformed .dat line                        */
#define SGB_ERR_RANGE (-4)        /* id outside its population, delay too long  */
#define SGB_ERR_CUDA (-5)         /* CUDA runtime error (text in last_error)    */
#define SGB_ERR_STATE (-6)        /* call not valid in the handle's state       */
#define SGB_ERR_OVERFLOW (-7)     /* raster buffer too small (counts still ok)  */
#define SGB_ERR_DEVICE (-8)       /* device-side error flag (e.g. wait limit)   */
#define SGB_ERR_NOMEM (-9)        /* host or device allocation failed           */
#define SGB_ERR_UNSUPPORTED (-10) /* feature outside this build's limits        */

/* ---- enums ------------------------------------------------------------- */
/* Population device type: reference DeviceType, struct_enum_def.h:43-47.
 * OUTPUT populations (DCN) run on the GPU like NORMAL ones here; the flag only
 * marks them as the output of sgb_loop_n_steps-style drivers. */
#define SGB_NORMAL 0
#define SGB_INPUT 1
#define SGB_OUTPUT 2

/* Conductance accumulator a projection feeds: the reference picks dg_exc or
 * dg_inh from the sign of initial_weight (GPUScaffoldSimulation.cu:732-733). */
#define SGB_CH_EXC 0
#define SGB_CH_INH 1

/* Propagation mode per projection (the reference picks its kernel from
 * max_conv, GPUScaffoldSimulation.cu:573-578,737-743). */
#define SGB_PROP_AUTO 0 /* decided by sgb_sim_autotune (default: CSR)   */
#define SGB_PROP_CSR 1  /* event-driven push of each spike's out-row     */
#define SGB_PROP_ELL 2  /* dense pull over every post's in-row each step */

#define SGB_WEIGHT_FP32 0
#define SGB_WEIGHT_BF16 1

/* Step driver: a CUDA graph replaying per-step kernels over a chunk, one
 * cooperative persistent launch per chunk, or plain per-step launches. */
#define SGB_EXEC_GRAPH 0
#define SGB_EXEC_PERSISTENT 1
#define SGB_EXEC_STREAM 2

/* Input stimulus kinds: reference PoissonProcess and PeriodicFiring,
 * UserInputFunctions.cu:4-10. */
#define SGB_INPUT_POISSON 0
#define SGB_INPUT_PERIODIC 1

/* ---- plain structs ------------------------------------------------------ */
typedef struct sgb_config {
  double dt_ms;          /* Euler substep length; reference DT (option.h:4)            */
  int32_t substeps;      /* Euler substeps per exchange step; reference STEP_MAX (option.h:6) */
  int32_t weight_type;   /* SGB_WEIGHT_FP32 or SGB_WEIGHT_BF16 synapse tables           */
  int32_t exec_mode;     /* SGB_EXEC_*                                                  */
  int32_t chunk_steps;   /* steps per graph replay / persistent launch (default 1000)   */
  int32_t device;        /* CUDA device ordinal                                          */
  int32_t default_prop;  /* mode for projections added with SGB_PROP_AUTO                */
  int32_t raster;        /* 1: record every spike for sgb_sim_run's raster output        */
  int32_t blocks_per_sm; /* persistent driver: resident blocks per SM (0: 1)              */
  int32_t l2_persist;    /* 1 (default): keep the cell state in a persisting L2 window    */
                         /* (within this process's context); 0: plain caching          */
  int32_t barrier_test_extra; /* tests of the bounded wait only: the persistent kernels'   */
                         /* grid barrier waits for this many arrivals beyond the grid, so */
                         /* it runs out its 1 s limit and the run returns SGB_ERR_DEVICE; */
                         /* 0 (default) otherwise                                         */
  int32_t reserved[6];
} sgb_config;

typedef struct sgb_input_params {
  int32_t kind;          /* SGB_INPUT_POISSON or SGB_INPUT_PERIODIC                     */
  float rate_hz;         /* Poisson rate, or periodic frequency                          */
  double phase_ms;       /* periodic: time of the first period start ("start" argument)  */
  double win_period_ms;  /* > 0: the window below repeats with this period               */
  double win_start_ms;   /* active window [start, end); end <= start means always active */
  double win_end_ms;
} sgb_input_params;

/* Synaptic plasticity of one projection: the reference's STDP rules
 * (SynapticPlasticity.cu:40-120, invoke_stdp_plasticity :123-140; compiled
 * in but switched off there, NumOfPlasticity = 0, struct_enum_def.h:50-53).
 * Every synapse carries a value v (v_max at start) that scales its weight; each
 * step, after the cells update, every synapse of the projection adds
 *   a0 + a1_j [pre spiked at t - d] + a1_i [post (Hebb) / teacher spiked]
 *      + a2_ji [post / teacher spiked] * #{s < window : pre spiked at t - d - s}
 * (in that order, FP32) and is clamped to [0, v_max]; the delivery of the
 * next step uses the new value.  Teacher: the teacher of a post cell is the
 * first synapse of `teacher_proj` onto it (lowest delay, then lowest pre id;
 * the reference takes the first ELL entry, :89, of a single-delay
 * projection), its spike read at t - its delay.  The reference's
 * coefficients are functions of (v, s); the ones it defines are constants
 * (:8-17), which is what these are. */
#define SGB_STDP_HEBB 0
#define SGB_STDP_TEACHER 1
typedef struct sgb_plasticity_params {
  int32_t rule;          /* SGB_STDP_HEBB or SGB_STDP_TEACHER                          */
  int32_t teacher_proj;  /* Teacher: projection onto the same post population       */
  int32_t window_steps;  /* pairing window of the a2_ji term (reference: 50), 0..64  */
  float a0, a1_i, a1_j, a2_ji;
  float v_max;           /* start value and upper clamp, 0 < v_max <= 1 (reference: 1;  */
                         /* its Teacher rule has no upper clamp and only depresses)     */
} sgb_plasticity_params;

typedef struct sgb_population_info {
  int32_t num, dev_type, c_num, n_in_projections;
  float Cm, El, dt_ref, Ie, Vr, Vth, gL;
  float ch_w[2], ch_E[2], ch_gbar[2], ch_tau[2];
  char name[32];
} sgb_population_info;

typedef struct sgb_projection_info {
  int32_t pre_pop, post_pop, channel, mode;
  int64_t n_synapses;
  int32_t max_in_degree, max_out_degree, min_delay, max_delay;
  char name[32];
} sgb_projection_info;

typedef struct sgb_input_info {
  int32_t pop, n_ids;
  sgb_input_params params;
} sgb_input_info;

typedef struct sgb_segment_info {
  int32_t net, pop, dev_type, count;
  int64_t first_id;      /* global id (all nets concatenated) of the segment's cell 0 */
  int32_t scale_bits[2]; /* fixed-point fraction bits of the exc / inh accumulators    */
} sgb_segment_info;

typedef struct sgb_sim_info {
  int32_t n_nets, n_segments, n_projections, ring_slots;
  int64_t n_neurons, n_synapses, step;
  int64_t device_bytes;  /* device memory held by the handle                           */
  int32_t exec_mode, weight_type, substeps, chunk_steps;
  double dt_ms;
  int64_t events;        /* synaptic events (spikes x out-degree) since the last reset */
  int64_t delivered;     /* synapses walked by event-driven delivery since the last reset */
  int32_t step_kernel;   /* SGB_KERNEL_*: the kernel a chunk of steps runs in            */
  int32_t push_smem_bytes; /* SGB_KERNEL_FUSED: shared memory per block holding push rows (0: none) */
  int64_t pulled;        /* dense-pull entries whose pre cell had spiked (deliveries) since the last reset */
  int64_t pull_entries;  /* dense-table entries streamed per step (0 without dense projections) */
  int64_t l2_persist_bytes; /* L2 set aside for the persisting state window (0: none)   */
  int64_t shard_cells;   /* SGB_KERNEL_FUSED: cells whose delay >= 3 synapses other blocks push */
  /* Launch shapes (defaults, or the autotuner's choice): */
  int32_t item_width;     /* SGB_KERNEL_FUSED: synapses per push item (32, 64 or 128)      */
  int32_t deliver_blocks; /* per-step driver: blocks of the delivery kernel               */
  int32_t pull_summary;   /* dense pulls: 0 every entry reads its history word; 1 entries   */
                          /* settle on a staged spike summary; 2 as 1, the per-step pull  */
                          /* loading its entries 16 bytes at a time                       */
  int32_t spike_ahead;    /* SGB_KERNEL_FUSED: the step's timeline; 0 spikes in their own  */
                          /* step (always with substeps > 1); 1 late push: a step         */
                          /* publishes the next step's spikes and makes its writes after  */
                          /* its grid-barrier arrival; 2 late push with the barrier split */
                          /* across steps                                                 */
  int32_t lane_cells;     /* SGB_KERNEL_GENERAL, one-barrier form: cells per lane (1, 2)  */
  int32_t reserved_;
} sgb_sim_info;

/* Step kernels (sgb_sim_info.step_kernel). */
#define SGB_KERNEL_GRAPH 0      /* k_update + k_deliver per step, CUDA graph or stream */
#define SGB_KERNEL_GENERAL 1    /* persistent; one grid barrier per step (two with dense  */
                                /* pulls or a Hebbian rule)                               */
#define SGB_KERNEL_RESIDENT 2   /* persistent, state in registers, two barriers        */
#define SGB_KERNEL_FUSED 3      /* persistent, state in registers, one barrier         */

typedef struct sgb_net sgb_net;
typedef struct sgb_sim sgb_sim;

/* ---- library ------------------------------------------------------------ */
void sgb_config_init(sgb_config* cfg);
const char* sgb_last_error(void);
int32_t sgb_abi_version(void);

/* ---- network description (host only; no GPU needed) ------------------- */
/* Replaces CreateNetworkEnv's host allocations (GPUScaffoldSimulation.cu:634-657). */
int sgb_net_create(sgb_net** out);
void sgb_net_destroy(sgb_net* net);

/* Replaces set_neuron_params (init_params.cu:255-302): `channels` holds c_num
 * records {w, E, g_bar, tau} in the order of the reference's varargs.  c_num
 * must be 1 or 2 for NORMAL/OUTPUT and 0 for INPUT populations. */
int sgb_net_add_population(sgb_net* net, const char* name, int32_t num, float Cm, float El,
                           float dt_ref, float Ie, float Vr, float Vth, float gL,
                           int32_t dev_type, int32_t c_num, const float* channels,
                           int32_t* pop_id);

/* Replaces set_connectivity_params + GetMaxConv + LoadConnectivityFile_ELL
 * (init_params.cu:304-332, 96-128, 13-67): reads "pre post" lines, gives each
 * synapse |initial_weight| (the loader's val=1 times w_bar,
 * GPUScaffoldSimulation.cu:733) and the one delay, and picks the accumulator
 * from the sign of initial_weight.  Lines with ids outside the populations
 * are rejected with SGB_ERR_RANGE (the reference skips them in GetMaxConv and
 * writes out of bounds in the loader). */
int sgb_net_add_projection_dat(sgb_net* net, const char* path, int32_t pre_pop,
                               int32_t post_pop, float initial_weight, int32_t delay_steps,
                               int32_t mode, int32_t* proj_id);

/* Per-synapse arrays (pre, post population-local ids; weight magnitude;
 * delay in steps, 1..15).  delay may be NULL when all equal `delay_all`. */
int sgb_net_add_projection_arrays(sgb_net* net, int32_t pre_pop, int32_t post_pop,
                                  int64_t n_syn, const uint32_t* pre, const uint32_t* post,
                                  const float* weight, const uint8_t* delay,
                                  int32_t delay_all, int32_t channel, int32_t mode,
                                  int32_t* proj_id);

/* Synthetic fixed in-degree projection: every post cell draws `in_degree`
 * distinct pre cells uniformly; weights uniform in [w_lo, w_hi) x w_mean;
 * delays uniform in d_min..d_max steps.  Deterministic in `seed`. */
int sgb_net_add_projection_random(sgb_net* net, int32_t pre_pop, int32_t post_pop,
                                  int32_t in_degree, float w_mean, float w_lo, float w_hi,
                                  int32_t d_min, int32_t d_max, int32_t channel,
                                  uint64_t seed, int32_t mode, int32_t* proj_id);

/* Replaces setInputStim (UserInputFunctions.cu:41-70): a stimulus source over
 * the listed cells of an INPUT population (ids == NULL: every cell).  A cell
 * covered by several sources fires when any of them fires. */
int sgb_net_add_input(sgb_net* net, int32_t pop, int64_t n_ids, const uint32_t* ids,
                      const sgb_input_params* params, int32_t* src_id);
/* Same, reading the id list from a file with one id per line. */
int sgb_net_add_input_dat(sgb_net* net, const char* path, int32_t pop,
                          const sgb_input_params* params, int32_t* src_id);

/* Builds one of the synthetic scaffolds (1: 9,256-cell net, 2: 92,550-cell
 * scaffold with burst input, 5: ~925k-cell scaffold), population sizes times
 * `scale`, connectivity and weights drawn from `seed`.  The network must be
 * empty.  Replaces the hard-coded init_neurons_params/init_connectivity_params
 * (init_params.cu:367-766) for the synthetic workloads. */
int sgb_net_build_scaffold(sgb_net* net, int32_t config, double scale, uint64_t seed);

/* Reference-structure mode: the reference's hard-coded scaffold (populations
 * and parameters of init_neurons_params, the 16 projections, weights and ms
 * delays of init_connectivity_params; init_params.cu:367-766) over the .dat
 * files in `dat_dir` (the reference's file names and format), and its two
 * stimulus lists background_noise.dat (Poisson 1 Hz) and tone_stim.dat
 * (periodic 140 Hz from 292.8 ms within [300, 351) ms, or Poisson 1 Hz;
 * UserInputFunctions.cu:19-29,72-81).  Delays in ms are exchange steps, as
 * with the reference's 1-ms step (cfg.dt_ms = 0.1, cfg.substeps = 10).
 * Populations are in the reference's array order (granule, purkinje, golgi,
 * stellate, basket, dcn, glomerulus); `sizes` (NULL: the reference's)
 * overrides the population sizes. */
int sgb_net_build_reference_scaffold(sgb_net* net, const char* dat_dir, const int32_t* sizes);
/* NeuronType enum value (struct_enum_def.h:10-20) of population `pop` of the
 * reference scaffold, as the reference prints it in rasters; -1 if none. */
int32_t sgb_reference_type_id(int32_t pop);

int sgb_net_counts(const sgb_net* net, int32_t* n_pops, int32_t* n_projs, int32_t* n_inputs,
                   int64_t* n_neurons, int64_t* n_synapses);
int sgb_net_population_info(const sgb_net* net, int32_t pop, sgb_population_info* info);
int sgb_net_projection_info(const sgb_net* net, int32_t proj, sgb_projection_info* info);
/* Makes projection `proj` plastic (replaces the reference's Init_Plasticity,
 * SynapticPlasticity.cu:20-34).  A plastic projection is delivered by dense
 * pull (its weights change every step), after the step's plasticity, with any
 * driver (persistent: resident or general kernel); autotuning is refused. */
int sgb_net_add_plasticity(sgb_net* net, int32_t proj, const sgb_plasticity_params* params);
/* *plastic = 1 and the parameters when projection `proj` is plastic, else 0. */
int sgb_net_plasticity_info(const sgb_net* net, int32_t proj, int32_t* plastic,
                            sgb_plasticity_params* params);
/* Copies the synapse arrays of a projection (any pointer may be NULL). */
int sgb_net_projection_synapses(const sgb_net* net, int32_t proj, uint32_t* pre, uint32_t* post,
                                float* weight, uint8_t* delay);
int sgb_net_input_info(const sgb_net* net, int32_t src, sgb_input_info* info);
int sgb_net_input_ids(const sgb_net* net, int32_t src, uint32_t* ids);
/* Writes a projection in the reference's .dat format ("pre\tpost" lines,
 * sorted by post then pre, as convert.py:62-81 writes them). */
int sgb_net_write_projection_dat(const sgb_net* net, int32_t proj, const char* path);

/* ---- simulation (needs a GPU) ------------------------------------------- */
/* Replaces InitializeNetworkEnv + Initialization (GPUScaffoldSimulation.cu:659-691,
 * 132-631): builds the device synapse tables of every net, allocates the
 * state, and draws the initial potentials u0 = Vr + (Vth-Vr)*U(0,1]
 * (InitParams, init_params.cu:343-352).  Several nets are simulated as
 * independent instances in the same launches; seeds[i] keys net i's random
 * streams. */
int sgb_sim_create(const sgb_config* cfg, sgb_net* const* nets, const uint64_t* seeds,
                   int32_t n_nets, sgb_sim** out);
/* Replaces FinalizeNetworkEnv (GPUScaffoldSimulation.cu:856-880). */
void sgb_sim_destroy(sgb_sim* sim);

/* Stream every later launch and copy is issued on (a cudaStream_t passed as
 * void*; NULL restores the handle's own stream). */
int sgb_sim_set_stream(sgb_sim* sim, void* stream);

/* Replaces SetInputFreq (GPUScaffoldSimulation.cu:883-890): new rate of each
 * input source of net `net` (n == number of sources), from the next step on. */
int sgb_sim_set_input_rates(sgb_sim* sim, int32_t net, int32_t n, const float* rates_hz);

/* Replaces loop_n_steps (GPUScaffoldSimulation.cu:693-791): advances every
 * instance by n_steps exchange steps.  Optional host outputs:
 *   counts[n_steps][n_segments]  spikes per segment per step;
 *   raster_ids / raster_offsets  spikes of step s are raster_ids[offsets[s] ..
 *                                offsets[s+1]) as global ids, ascending
 *                                (needs cfg.raster = 1; offsets has n_steps+1
 *                                entries; SGB_ERR_OVERFLOW when raster_cap is
 *                                too small -- the simulation itself is intact).
 * Returns after the device has finished the steps. */
int sgb_sim_run(sgb_sim* sim, int64_t n_steps, uint32_t* counts, uint32_t* raster_ids,
                int64_t raster_cap, int64_t* raster_offsets);

/* Asynchronous form of sgb_sim_run without host outputs: enqueues n_steps on
 * the handle's stream and returns at once (spike counts stay on the device and
 * are folded into the FP64 totals).  sgb_sim_sync waits for the stream and
 * reports device-side error flags.  These two calls have no counterpart in the
 * reference, whose loop_n_steps always blocks (GPUScaffoldSimulation.cu:756). */
int sgb_sim_enqueue(sgb_sim* sim, int64_t n_steps);
int sgb_sim_sync(sgb_sim* sim);

/* Replaces ResetNetworkEnv (GPUScaffoldSimulation.cu:802-853): step counter to
 * 0, conductances, refractory counters, delay rings and spike history cleared,
 * initial potentials redrawn with the (possibly new) seeds (NULL: keep). */
int sgb_sim_reset(sgb_sim* sim, const uint64_t* seeds);

int sgb_sim_get_info(const sgb_sim* sim, sgb_sim_info* info);
int sgb_sim_segment_info(const sgb_sim* sim, int32_t seg, sgb_segment_info* info);

/* Neuron state in global-id order: u[n], g[n][2], refractory steps left[n]
 * (any pointer may be NULL).  INPUT cells report zeros. */
int sgb_sim_get_state(sgb_sim* sim, float* u, float* g, int32_t* ref);
int sgb_sim_set_state(sgb_sim* sim, const float* u, const float* g, const int32_t* ref);

/* Checkpoint / resume.  A checkpoint holds the whole evolving device state of
 * a handle: cell state, pending synaptic increments, spike history, step and
 * event counters, long-horizon totals, stimulus rates and plastic values.
 * sgb_sim_checkpoint_size gives its size; save copies it into caller memory
 * (at a chunk boundary: after sgb_sim_run or sgb_sim_sync); load restores it
 * into a handle built from the same networks and configuration, which then
 * continues exactly as the saved one would have when its seeds are the same
 * (inputs are keyed on seed, cell and step).  The reference has no
 * counterpart (ResetNetworkEnv, GPUScaffoldSimulation.cu:802-854, only
 * re-draws the potentials). */
int sgb_sim_checkpoint_size(const sgb_sim* sim, int64_t* bytes);
int sgb_sim_save_checkpoint(sgb_sim* sim, void* buf, int64_t capacity);
int sgb_sim_load_checkpoint(sgb_sim* sim, const void* buf, int64_t size);

/* Writes a raster returned by sgb_sim_run in the reference's text format,
 * one "t\tlocal_id\ttype_id" line per spike (print_spike_train,
 * GPUScaffoldSimulation.cu:77-85): t in ms as %f (step index first_step + k
 * times the exchange step), the cell's index within its population, and
 * type_ids[population] (NULL: the population index). */
int sgb_sim_write_raster(const sgb_sim* sim, const char* path, const uint32_t* ids,
                         const int64_t* offsets, int64_t n_steps, int64_t first_step,
                         const int32_t* type_ids, int32_t append);

/* Long-horizon spike totals per segment (FP64 accumulators, updated on the
 * device at the end of every chunk). */
int sgb_sim_spike_totals(sgb_sim* sim, double* totals);

/* Propagation mode of projection `proj` of net `net` (SGB_PROP_CSR/ELL), from
 * the next step on.  Any time between runs: the contributions of the last
 * (max delay - 1) steps' spikes still on their way are handed over (taken back
 * out of the ring when the projection starts pulling, added when it starts
 * pushing), so the run continues bit for bit as if the new mode had been in
 * place from the start; the autotuner does the same with its choice. */
int sgb_sim_set_propagation(sgb_sim* sim, int32_t net, int32_t proj, int32_t mode);
int sgb_sim_get_propagation(const sgb_sim* sim, int32_t net, int32_t proj, int32_t* mode);

/* Current plasticity values v of the synapses of plastic projection `proj`
 * of net `net`, in the projection's synapse order (sgb_net_projection_synapses). */
int sgb_sim_plastic_values(sgb_sim* sim, int32_t net, int32_t proj, float* values);

/* Autotuner: times the CSR and ELL propagation of every projection over
 * `n_steps` steps of the running simulation (restoring its state afterwards)
 * and keeps the faster mode.  With a cache path, decisions are read from and
 * written to that JSON file. */
int sgb_sim_autotune(sgb_sim* sim, int32_t n_steps, const char* cache_path);

/* Number of kernel launches issued so far (graph nodes count one each). */
int sgb_sim_launch_count(const sgb_sim* sim, int64_t* launches);

/* Instrumented run: advances n_steps with the per-step kernels launched one by
 * one, each bracketed by CUDA events on the handle's stream, and returns per
 * kernel class (0 update, 1 event-driven delivery, 2 dense pull, 3
 * plasticity) the mean device time per launch in microseconds, the mean
 * algorithmic bytes per launch, and the number of launches (0 for the pull
 * without dense projections and for plasticity without plastic ones). */
#define SGB_KCLASS_COUNT 4
int sgb_sim_profile(sgb_sim* sim, int32_t n_steps, double* mean_us, double* bytes_per_launch,
                    int64_t* launches);

/* ---- standalone operator (caller-owned device buffers) -------------------- */
/* Replaces the reference's per-projection propagation kernels spike_propagation,
 * spike_propagation_mThreads and spike_propagation_PR (Simulation_header.cu:
 * 83-303) as one operator for callers that run their own neuron update.  For
 * every cell j with spikes[j] != 0 and every synapse q in [row[j], row[j+1]):
 *   post = syn[q] & (2^27 - 1), d = (syn[q] >> 27) & 15, a = syn[q] >> 31,
 *   ring[((step + d) % ring_slots) * n_cells + post][a] += rint(weights[q]),
 * where weights are FP32 or BF16 already multiplied by the accumulator's 2^S.
 * Every delay field value 0..15 is taken modulo ring_slots, so a table whose
 * delays reach ring_slots or beyond wraps around the ring (it never writes
 * outside it); a simulation that needs every spike to land in its own future
 * slot keeps all delays < ring_slots.  All pointers are device pointers; work is enqueued on `stream` (a
 * cudaStream_t as void*, NULL = legacy default stream) and the call returns
 * without waiting.  Scratch for the active-cell list is taken from the
 * stream-ordered pool (cudaMallocAsync) and released on the same stream. */
int sgb_deliver_spikes(const uint8_t* spikes, int32_t n_cells, const uint32_t* row,
                       const uint32_t* syn, const void* weights, int32_t weight_type,
                       int32_t* ring, int32_t ring_slots, int64_t step, void* stream);

/* Same operation as sgb_deliver_spikes, allocating nothing.  This entry point
 * has no counterpart in the reference.  It is for callers that cannot
 * allocate device memory when they deliver spikes: a real-time step loop in
 * which a device allocation (which may synchronise the device) would break
 * the deadline, or a process whose device memory belongs to another allocator
 * (a framework's caching allocator, a fixed budget) that must not be bypassed.
 * The caller passes inputs and outputs as above; the scratch (one count word
 * and the list of active cells) is a file-scope device array of the library,
 * sized for n_cells <= 1,048,576 (4 MiB), which every GPU that loads the
 * library holds until the process exits.  Larger n_cells return
 * SGB_ERR_RANGE.  The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress) with the device current; make that first
 * call before any stream capture.  A cudaDeviceReset of that device ends the
 * context holding the array, so the cached address is stale afterwards: do
 * not call this entry point on a device the process has reset.  Every call
 * clears the count word on its stream and shares the one array, so calls
 * that overlap on the GPU (other streams, other host threads) race:
 * serialise them. */
int sgb_deliver_spikes_static(const uint8_t* spikes, int32_t n_cells, const uint32_t* row,
                              const uint32_t* syn, const void* weights, int32_t weight_type,
                              int32_t* ring, int32_t ring_slots, int64_t step, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SCAFFOLD_GB300_H */
