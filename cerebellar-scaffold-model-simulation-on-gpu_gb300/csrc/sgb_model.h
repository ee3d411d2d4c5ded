// Host-side network description: populations, projections and stimulus
// sources of one scaffold instance, plus the rules every later stage shares
// (fixed-point accumulator scales, synthetic scaffold definitions).
//
// The reference keeps the same information in its Neuron / Connectivity /
// InputFunctionsStruct records (struct_enum_def.h:56-102) filled by
// set_neuron_params / set_connectivity_params / setInputStim
// (init_params.cu:255-332, UserInputFunctions.cu:41-70).  Here synapses are
// stored as flat per-projection arrays with a weight and a delay each; the
// device tables (post-major ELL and pre-major CSR) are built from them.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/scaffold_gb300.h"

namespace sgb {

struct Population {
  std::string name;
  int32_t num = 0;
  float Cm = 0, El = 0, dt_ref = 0, Ie = 0, Vr = 0, Vth = 0, gL = 0;
  int32_t dev_type = SGB_NORMAL;
  int32_t c_num = 0;
  float w[2] = {0, 0}, E[2] = {0, 0}, gbar[2] = {0, 0}, tau[2] = {1, 1};
};

struct Projection {
  std::string name;
  int32_t pre = -1, post = -1, channel = SGB_CH_EXC, mode = SGB_PROP_AUTO;
  std::vector<uint32_t> pre_idx, post_idx;  // population-local ids
  std::vector<float> weight;                // magnitude added to the accumulator
  std::vector<uint8_t> delay;               // exchange steps, 1..kMaxDelay
  bool plastic = false;                     // STDP (add_plasticity)
  sgb_plasticity_params plast{};
};

struct InputSource {
  int32_t pop = -1;
  std::vector<uint32_t> ids;  // population-local ids, sorted, unique
  sgb_input_params p{};
};

struct Network {
  std::vector<Population> pops;
  std::vector<Projection> projs;
  std::vector<InputSource> inputs;
  int64_t n_neurons() const;
  int64_t n_synapses() const;
};

// Status plumbing shared by every translation unit of the library.
int set_error(int code, const char* fmt, ...);
const char* last_error();

// Network construction (validated; return SGB_OK or a negative status).
int add_population(Network& net, const char* name, int32_t num, float Cm, float El,
                   float dt_ref, float Ie, float Vr, float Vth, float gL, int32_t dev_type,
                   int32_t c_num, const float* channels, int32_t* pop_id);
int add_projection(Network& net, Projection&& proj, int32_t* proj_id);
int load_projection_dat(Network& net, const char* path, int32_t pre_pop, int32_t post_pop,
                        float initial_weight, int32_t delay_steps, int32_t mode,
                        int32_t* proj_id);
int add_random_projection(Network& net, int32_t pre_pop, int32_t post_pop, int32_t in_degree,
                          float w_mean, float w_lo, float w_hi, int32_t d_min, int32_t d_max,
                          int32_t channel, uint64_t seed, int32_t mode, int32_t* proj_id);
int add_input(Network& net, int32_t pop, int64_t n_ids, const uint32_t* ids,
              const sgb_input_params* params, int32_t* src_id);
int load_input_dat(Network& net, const char* path, int32_t pop, const sgb_input_params* params,
                   int32_t* src_id);
int write_projection_dat(const Network& net, int32_t proj, const char* path);
int add_plasticity(Network& net, int32_t proj, const sgb_plasticity_params* params);
constexpr int kMaxStdpWindow = 64;  // longest pairing window (steps)
int build_scaffold(Network& net, int32_t config, double scale, uint64_t seed);

// Fixed-point fraction bits of each (population, accumulator) pair: the
// largest S <= kMaxScaleBits such that, for every post cell, the sum of
// rint(w * 2^S) over all synapses feeding that accumulator is <= INT32_MAX.
// Every synapse contributes at most once to one delay slot, so no sum of
// delivered increments can overflow.  Weights are the values the device
// tables hold (BF16-rounded when bf16 is set).
constexpr int kMaxScaleBits = 30;
void accumulator_scale_bits(const Network& net, bool bf16, std::vector<int32_t>& bits);

// Weight as held by the device table.
inline float table_weight(float w, bool bf16);

}  // namespace sgb

#include "sgb_philox.h"
inline float sgb::table_weight(float w, bool bf16) {
  return bf16 ? bf16_bits_to_f32(f32_to_bf16_bits(w)) : w;
}
