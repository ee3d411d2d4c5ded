// Host-side network description (see sgb_model.h).
#include "sgb_model.h"

#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <numeric>

#include "sgb_philox.h"

namespace sgb {

static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

const char* last_error() { return g_last_error.c_str(); }

int64_t Network::n_neurons() const {
  int64_t n = 0;
  for (const auto& p : pops) n += p.num;
  return n;
}

int64_t Network::n_synapses() const {
  int64_t n = 0;
  for (const auto& p : projs) n += (int64_t)p.pre_idx.size();
  return n;
}

// ---------------------------------------------------------------------------
// Populations: set_neuron_params (init_params.cu:255-302).  The reference
// re-orders populations (NORMAL first, INPUT/OUTPUT last) to split GPU and
// CPU work; everything runs on the GPU here, so definition order is kept.
int add_population(Network& net, const char* name, int32_t num, float Cm, float El,
                   float dt_ref, float Ie, float Vr, float Vth, float gL, int32_t dev_type,
                   int32_t c_num, const float* channels, int32_t* pop_id) {
  if (num < 0) return set_error(SGB_ERR_ARG, "population size %d is negative", num);
  if ((int64_t)num > (int64_t)kIndexMask)
    return set_error(SGB_ERR_UNSUPPORTED, "population size %d exceeds 2^28-1", num);
  if (dev_type != SGB_NORMAL && dev_type != SGB_INPUT && dev_type != SGB_OUTPUT)
    return set_error(SGB_ERR_ARG, "unknown device type %d", dev_type);
  if (dev_type == SGB_INPUT) {
    if (c_num != 0) return set_error(SGB_ERR_ARG, "INPUT populations take no channels");
  } else {
    if (c_num < 1 || c_num > 2)
      return set_error(SGB_ERR_UNSUPPORTED, "c_num=%d: this build supports 1 or 2 channels",
                       c_num);
    if (!channels) return set_error(SGB_ERR_ARG, "channels is NULL");
    if (!(Cm > 0.f)) return set_error(SGB_ERR_ARG, "Cm must be positive");
    for (int c = 0; c < c_num; ++c)
      if (!(channels[4 * c + 3] > 0.f))
        return set_error(SGB_ERR_ARG, "channel %d: tau must be positive", c);
  }
  Population p;
  p.name = name ? name : "";
  if (p.name.size() > 31) p.name.resize(31);
  p.num = num;
  p.Cm = Cm; p.El = El; p.dt_ref = dt_ref; p.Ie = Ie; p.Vr = Vr; p.Vth = Vth; p.gL = gL;
  p.dev_type = dev_type;
  p.c_num = c_num;
  for (int c = 0; c < c_num; ++c) {
    p.w[c] = channels[4 * c + 0];
    p.E[c] = channels[4 * c + 1];
    p.gbar[c] = channels[4 * c + 2];
    p.tau[c] = channels[4 * c + 3];
  }
  net.pops.push_back(p);
  if (pop_id) *pop_id = (int32_t)net.pops.size() - 1;
  return SGB_OK;
}

// ---------------------------------------------------------------------------
// Projections.
int add_projection(Network& net, Projection&& pr, int32_t* proj_id) {
  const int32_t npop = (int32_t)net.pops.size();
  if (pr.pre < 0 || pr.pre >= npop || pr.post < 0 || pr.post >= npop)
    return set_error(SGB_ERR_ARG, "projection populations (%d -> %d) out of range", pr.pre,
                     pr.post);
  if (net.pops[pr.post].dev_type == SGB_INPUT)
    return set_error(SGB_ERR_ARG, "projection onto INPUT population '%s'",
                     net.pops[pr.post].name.c_str());
  if (pr.channel != SGB_CH_EXC && pr.channel != SGB_CH_INH)
    return set_error(SGB_ERR_ARG, "channel %d is neither SGB_CH_EXC nor SGB_CH_INH", pr.channel);
  if (pr.mode < SGB_PROP_AUTO || pr.mode > SGB_PROP_ELL)
    return set_error(SGB_ERR_ARG, "unknown propagation mode %d", pr.mode);
  const size_t n = pr.pre_idx.size();
  if (pr.post_idx.size() != n || pr.weight.size() != n || pr.delay.size() != n)
    return set_error(SGB_ERR_ARG, "synapse arrays differ in length");
  const uint32_t npre = (uint32_t)net.pops[pr.pre].num, npost = (uint32_t)net.pops[pr.post].num;
  for (size_t i = 0; i < n; ++i) {
    if (pr.pre_idx[i] >= npre || pr.post_idx[i] >= npost)
      return set_error(SGB_ERR_RANGE, "synapse %zu: (%u -> %u) outside populations of %u / %u",
                       i, pr.pre_idx[i], pr.post_idx[i], npre, npost);
    if (pr.delay[i] < 1 || pr.delay[i] > kMaxDelay)
      return set_error(SGB_ERR_RANGE, "synapse %zu: delay %u not in 1..%d steps", i,
                       (unsigned)pr.delay[i], kMaxDelay);
    if (!(pr.weight[i] >= 0.f) || !isfinite(pr.weight[i]))
      return set_error(SGB_ERR_ARG, "synapse %zu: weight must be a finite magnitude >= 0", i);
  }
  if (pr.name.empty())
    pr.name = net.pops[pr.pre].name + "_to_" + net.pops[pr.post].name;
  if (pr.name.size() > 31) pr.name.resize(31);
  net.projs.push_back(std::move(pr));
  if (proj_id) *proj_id = (int32_t)net.projs.size() - 1;
  return SGB_OK;
}

// Reads whitespace-separated integer pairs, one synapse per line, as
// LoadConnectivityFile_ELL does with sscanf("%d %d") (init_params.cu:38-53).
// Blank lines are skipped; anything else that is not two integers is a
// format error.
static int read_pairs(const char* path, std::vector<int64_t>& a, std::vector<int64_t>& b) {
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(SGB_ERR_IO, "cannot open '%s': %s", path, strerror(errno));
  std::string text;
  char buf[1 << 16];
  size_t got;
  while ((got = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
  fclose(f);
  const char* s = text.c_str();
  const char* end = s + text.size();
  int64_t line = 0;
  while (s < end) {
    ++line;
    const char* eol = (const char*)memchr(s, '\n', (size_t)(end - s));
    if (!eol) eol = end;
    const char* p = s;
    while (p < eol && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    if (p < eol) {
      char* q;
      errno = 0;
      long long x = strtoll(p, &q, 10);
      if (q == p || errno) return set_error(SGB_ERR_FORMAT, "%s:%lld: expected integer", path, line);
      p = q;
      long long y = strtoll(p, &q, 10);
      if (q == p || errno) return set_error(SGB_ERR_FORMAT, "%s:%lld: expected two integers", path, line);
      p = q;
      while (p < eol && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
      if (p < eol) return set_error(SGB_ERR_FORMAT, "%s:%lld: trailing characters", path, line);
      a.push_back(x);
      b.push_back(y);
    }
    s = eol + 1;
  }
  return SGB_OK;
}

int load_projection_dat(Network& net, const char* path, int32_t pre_pop, int32_t post_pop,
                        float initial_weight, int32_t delay_steps, int32_t mode,
                        int32_t* proj_id) {
  const int32_t npop = (int32_t)net.pops.size();
  if (pre_pop < 0 || pre_pop >= npop || post_pop < 0 || post_pop >= npop)
    return set_error(SGB_ERR_ARG, "population index out of range");
  if (delay_steps < 1 || delay_steps > kMaxDelay)
    return set_error(SGB_ERR_RANGE, "delay %d not in 1..%d steps", delay_steps, kMaxDelay);
  std::vector<int64_t> a, b;
  int rc = read_pairs(path, a, b);
  if (rc) return rc;
  Projection pr;
  pr.pre = pre_pop;
  pr.post = post_pop;
  pr.mode = mode;
  // Sign picks the accumulator, magnitude is the weight
  // (GPUScaffoldSimulation.cu:732-733; val = 1 from init_params.cu:45).
  pr.channel = initial_weight > 0.f ? SGB_CH_EXC : SGB_CH_INH;
  const float w = fabsf(initial_weight);
  const int64_t npre = net.pops[pre_pop].num, npost = net.pops[post_pop].num;
  pr.pre_idx.reserve(a.size());
  for (size_t i = 0; i < a.size(); ++i) {
    if (a[i] < 0 || a[i] >= npre || b[i] < 0 || b[i] >= npost)
      return set_error(SGB_ERR_RANGE, "%s: synapse %zu (%lld -> %lld) outside populations of "
                       "%lld / %lld", path, i, (long long)a[i], (long long)b[i],
                       (long long)npre, (long long)npost);
    pr.pre_idx.push_back((uint32_t)a[i]);
    pr.post_idx.push_back((uint32_t)b[i]);
  }
  pr.weight.assign(a.size(), w);
  pr.delay.assign(a.size(), (uint8_t)delay_steps);
  const char* base = strrchr(path, '/');
  pr.name = base ? base + 1 : path;
  const size_t dot = pr.name.rfind(".dat");
  if (dot != std::string::npos) pr.name.resize(dot);
  return add_projection(net, std::move(pr), proj_id);
}

// One Philox stream for synthetic connectivity: draw i of purpose `purpose`
// for post cell `post` is component i%4 of philox(seed; post, i/4, tag, purpose).
struct GenStream {
  uint64_t seed;
  uint32_t post, purpose;
  uint64_t next = 0;
  U4 cur{};
  uint32_t draw() {
    if ((next & 3) == 0) cur = philox_draw(seed, post, next >> 2, kTagNetGen, purpose);
    return u4_get(cur, (int)(next++ & 3));
  }
};

int add_random_projection(Network& net, int32_t pre_pop, int32_t post_pop, int32_t in_degree,
                          float w_mean, float w_lo, float w_hi, int32_t d_min, int32_t d_max,
                          int32_t channel, uint64_t seed, int32_t mode, int32_t* proj_id) {
  const int32_t npop = (int32_t)net.pops.size();
  if (pre_pop < 0 || pre_pop >= npop || post_pop < 0 || post_pop >= npop)
    return set_error(SGB_ERR_ARG, "population index out of range");
  const int64_t npre = net.pops[pre_pop].num, npost = net.pops[post_pop].num;
  if (in_degree < 0 || in_degree > npre)
    return set_error(SGB_ERR_ARG, "in-degree %d not in 0..%lld", in_degree, (long long)npre);
  if (d_min < 1 || d_max < d_min || d_max > kMaxDelay)
    return set_error(SGB_ERR_RANGE, "delays %d..%d not within 1..%d", d_min, d_max, kMaxDelay);
  if (!(w_mean >= 0.f) || !(w_hi >= w_lo) || !(w_lo >= 0.f))
    return set_error(SGB_ERR_ARG, "weight range must be non-negative and ordered");
  Projection pr;
  pr.pre = pre_pop;
  pr.post = post_pop;
  pr.channel = channel;
  pr.mode = mode;
  const int64_t nsyn = (int64_t)in_degree * npost;
  pr.pre_idx.resize(nsyn);
  pr.post_idx.resize(nsyn);
  pr.weight.resize(nsyn);
  pr.delay.resize(nsyn);
  const uint32_t dspan = (uint32_t)(d_max - d_min + 1);
  const float wspan = w_hi - w_lo;
#pragma omp parallel
  {
    // Floyd's sampling of in_degree distinct ids from [0, npre), bitmap-marked.
    std::vector<uint64_t> mark((size_t)(npre + 63) / 64, 0);
    std::vector<uint32_t> pick;
    pick.reserve(in_degree);
#pragma omp for schedule(dynamic, 16)
    for (int64_t p = 0; p < npost; ++p) {
      GenStream gi{seed, (uint32_t)p, 0u}, gw{seed, (uint32_t)p, 1u}, gd{seed, (uint32_t)p, 2u};
      pick.clear();
      for (int64_t j = npre - in_degree; j < npre; ++j) {
        uint32_t t = (uint32_t)(((uint64_t)gi.draw() * (uint64_t)(j + 1)) >> 32);
        if (mark[t >> 6] >> (t & 63) & 1ull) t = (uint32_t)j;
        mark[t >> 6] |= 1ull << (t & 63);
        pick.push_back(t);
      }
      std::sort(pick.begin(), pick.end());
      const int64_t o = p * in_degree;
      for (int32_t k = 0; k < in_degree; ++k) {
        const uint32_t t = pick[k];
        mark[t >> 6] &= ~(1ull << (t & 63));
        pr.pre_idx[o + k] = t;
        pr.post_idx[o + k] = (uint32_t)p;
        const float u = (float)(gw.draw() >> 8) * (1.0f / 16777216.0f);  // [0, 1)
        pr.weight[o + k] = w_mean * (w_lo + wspan * u);
        pr.delay[o + k] = (uint8_t)(d_min + (int32_t)(((uint64_t)gd.draw() * dspan) >> 32));
      }
    }
  }
  return add_projection(net, std::move(pr), proj_id);
}

// ---------------------------------------------------------------------------
// Stimulus sources: setInputStim (UserInputFunctions.cu:41-70).
int add_input(Network& net, int32_t pop, int64_t n_ids, const uint32_t* ids,
              const sgb_input_params* params, int32_t* src_id) {
  if (pop < 0 || pop >= (int32_t)net.pops.size())
    return set_error(SGB_ERR_ARG, "population index %d out of range", pop);
  if (net.pops[pop].dev_type != SGB_INPUT)
    return set_error(SGB_ERR_ARG, "population '%s' is not an INPUT population",
                     net.pops[pop].name.c_str());
  if (!params) return set_error(SGB_ERR_ARG, "params is NULL");
  if (params->kind != SGB_INPUT_POISSON && params->kind != SGB_INPUT_PERIODIC)
    return set_error(SGB_ERR_ARG, "unknown input kind %d", params->kind);
  if (!(params->rate_hz >= 0.f)) return set_error(SGB_ERR_ARG, "rate must be >= 0");
  if (params->win_period_ms < 0.0) return set_error(SGB_ERR_ARG, "window period must be >= 0");
  if (net.inputs.size() >= 32) return set_error(SGB_ERR_UNSUPPORTED, "at most 32 sources per net");
  InputSource s;
  s.pop = pop;
  s.p = *params;
  const uint32_t num = (uint32_t)net.pops[pop].num;
  if (ids) {
    if (n_ids < 0) return set_error(SGB_ERR_ARG, "negative id count");
    s.ids.assign(ids, ids + n_ids);
    for (uint32_t id : s.ids)
      if (id >= num)
        return set_error(SGB_ERR_RANGE, "input id %u outside population of %u", id, num);
    std::sort(s.ids.begin(), s.ids.end());
    s.ids.erase(std::unique(s.ids.begin(), s.ids.end()), s.ids.end());
  } else {
    s.ids.resize(num);
    std::iota(s.ids.begin(), s.ids.end(), 0u);
  }
  net.inputs.push_back(std::move(s));
  if (src_id) *src_id = (int32_t)net.inputs.size() - 1;
  return SGB_OK;
}

// One unsigned id per line (UserInputFunctions.cu:53-57).
int load_input_dat(Network& net, const char* path, int32_t pop, const sgb_input_params* params,
                   int32_t* src_id) {
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(SGB_ERR_IO, "cannot open '%s': %s", path, strerror(errno));
  std::vector<uint32_t> ids;
  char line[256];
  int64_t ln = 0;
  while (fgets(line, sizeof line, f)) {
    ++ln;
    char* p = line;
    while (*p == ' ' || *p == '\t') ++p;
    if (*p == '\n' || *p == '\r' || *p == 0) continue;
    char* q;
    errno = 0;
    long long v = strtoll(p, &q, 10);
    if (q == p || errno || v < 0 || v > 0xFFFFFFFFll) {
      fclose(f);
      return set_error(SGB_ERR_FORMAT, "%s:%lld: expected an unsigned id", path, ln);
    }
    ids.push_back((uint32_t)v);
  }
  fclose(f);
  return add_input(net, pop, (int64_t)ids.size(), ids.data(), params, src_id);
}

// "pre\tpost" sorted by post then pre, as convert.py:79-81 writes them.
int write_projection_dat(const Network& net, int32_t proj, const char* path) {
  if (proj < 0 || proj >= (int32_t)net.projs.size())
    return set_error(SGB_ERR_ARG, "projection index %d out of range", proj);
  const Projection& pr = net.projs[proj];
  std::vector<size_t> order(pr.pre_idx.size());
  std::iota(order.begin(), order.end(), (size_t)0);
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return pr.post_idx[a] != pr.post_idx[b] ? pr.post_idx[a] < pr.post_idx[b]
                                            : pr.pre_idx[a] < pr.pre_idx[b];
  });
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(SGB_ERR_IO, "cannot create '%s': %s", path, strerror(errno));
  for (size_t i : order) fprintf(f, "%u\t%u\n", pr.pre_idx[i], pr.post_idx[i]);
  if (fclose(f)) return set_error(SGB_ERR_IO, "write to '%s' failed", path);
  return SGB_OK;
}

// ---------------------------------------------------------------------------
// Accumulator scales (see header).
// Plastic values start at v_max and stay in [0, v_max], v_max <= 1, so a plastic synapse
// never delivers more than its initial weight and the accumulator scales
// need no headroom.
int add_plasticity(Network& net, int32_t proj, const sgb_plasticity_params* p) {
  if (!p) return set_error(SGB_ERR_ARG, "params is NULL");
  if (proj < 0 || proj >= (int32_t)net.projs.size())
    return set_error(SGB_ERR_ARG, "projection %d out of range", proj);
  Projection& pr = net.projs[proj];
  if (pr.plastic) return set_error(SGB_ERR_ARG, "projection %d is already plastic", proj);
  if (p->rule != SGB_STDP_HEBB && p->rule != SGB_STDP_TEACHER)
    return set_error(SGB_ERR_ARG, "unknown plasticity rule %d", p->rule);
  if (p->window_steps < 0 || p->window_steps > kMaxStdpWindow)
    return set_error(SGB_ERR_RANGE, "window of %d steps not in 0..%d", p->window_steps,
                     kMaxStdpWindow);
  if (!(p->v_max > 0.f && p->v_max <= 1.f))
    return set_error(SGB_ERR_RANGE, "v_max %g not in (0, 1]", (double)p->v_max);
  if (!std::isfinite(p->a0) || !std::isfinite(p->a1_i) || !std::isfinite(p->a1_j) ||
      !std::isfinite(p->a2_ji))
    return set_error(SGB_ERR_ARG, "coefficients must be finite");
  if (p->rule == SGB_STDP_TEACHER) {
    if (p->teacher_proj < 0 || p->teacher_proj >= (int32_t)net.projs.size() ||
        p->teacher_proj == proj)
      return set_error(SGB_ERR_ARG, "teacher projection %d out of range", p->teacher_proj);
    if (net.projs[p->teacher_proj].post != pr.post)
      return set_error(SGB_ERR_ARG, "teacher projection %d does not target population %d",
                       p->teacher_proj, pr.post);
  }
  pr.plastic = true;
  pr.plast = *p;
  if (p->rule == SGB_STDP_HEBB) pr.plast.teacher_proj = -1;
  pr.mode = SGB_PROP_ELL;
  return SGB_OK;
}

void accumulator_scale_bits(const Network& net, bool bf16, std::vector<int32_t>& bits) {
  const size_t np = net.pops.size();
  bits.assign(np * 2, kMaxScaleBits);
  for (size_t pop = 0; pop < np; ++pop) {
    for (int ch = 0; ch < 2; ++ch) {
      std::vector<const Projection*> in;
      for (const auto& pr : net.projs)
        if (pr.post == (int32_t)pop && pr.channel == ch && !pr.pre_idx.empty()) in.push_back(&pr);
      if (in.empty()) continue;
      const size_t npost = (size_t)net.pops[pop].num;
      std::vector<double> sum(npost, 0.0);
      for (const Projection* pr : in)
        for (size_t i = 0; i < pr->pre_idx.size(); ++i)
          sum[pr->post_idx[i]] += (double)table_weight(pr->weight[i], bf16);
      double mx = 0.0;
      for (double v : sum) mx = v > mx ? v : mx;
      int s = kMaxScaleBits;
      if (mx > 0.0) {
        const int est = (int)floor(log2(2147483647.0 / mx));
        s = est + 1 < kMaxScaleBits ? est + 1 : kMaxScaleBits;
      }
      // Exact check, lowering S until every post cell's integer sum fits.
      std::vector<int64_t> isum(npost);
      for (;; --s) {
        std::fill(isum.begin(), isum.end(), 0);
        const float scale = ldexpf(1.0f, s);
        for (const Projection* pr : in)
          for (size_t i = 0; i < pr->pre_idx.size(); ++i)
            isum[pr->post_idx[i]] += (int64_t)rintf(table_weight(pr->weight[i], bf16) * scale);
        int64_t m = 0;
        for (int64_t v : isum) m = v > m ? v : m;
        if (m <= 2147483647ll || s <= -100) break;
      }
      bits[pop * 2 + ch] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// Synthetic scaffolds.  Population sizes and in-degrees are those of the
// benchmark configurations; every cell uses the same conductance-based LIF
// (C=3 pF, gL=0.2 nS, EL=-70 mV, Vth=-50 mV, Vreset=-70 mV, 2 ms refractory,
// tau_exc=0.5 ms, tau_inh=10 ms, E_exc=0 mV, E_inh=-80 mV).  Projection means
// are given as the total drive (mean weight x in-degree) so that the 9k- and
// 92k-cell nets with different in-degrees stay in the same dynamical regime;
// weights are uniform in [0.5, 1.5) x mean and delays uniform in 1..4 steps.
namespace {
struct ScaffoldSpec {
  int32_t mossy, granule, golgi, stellate, basket, purkinje, dcn;
  int32_t k_grc_mf, k_grc_goc, k_goc_grc, k_goc_mf, k_sc_grc, k_bc_grc, k_pc_grc, k_pc_sc,
      k_pc_bc, k_dcn_pc, k_dcn_mf;
  bool burst;
};
// Total drive per projection (nS summed over the in-degree), calibrated once
// with the oracle for a sparse granule layer (~3-4 Hz), Golgi / stellate /
// basket at ~30-40 Hz, Purkinje at ~60-90 Hz and DCN at ~10-20 Hz under 4 Hz
// mossy input, then frozen.
constexpr float kDriveGrcMf = 11.0f, kDriveGrcGoc = 3.0f, kDriveGocGrc = 30.0f,
                kDriveGocMf = 12.0f, kDriveScGrc = 45.0f, kDriveBcGrc = 45.0f,
                kDrivePcGrc = 450.0f, kDrivePcSc = 3.0f, kDrivePcBc = 3.0f,
                kDriveDcnPc = 2.0f, kDriveDcnMf = 60.0f;
}  // namespace

int build_scaffold(Network& net, int32_t config, double scale, uint64_t seed) {
  if (!net.pops.empty()) return set_error(SGB_ERR_STATE, "build_scaffold needs an empty network");
  if (!(scale > 0.0)) return set_error(SGB_ERR_ARG, "scale must be positive");
  ScaffoldSpec s;
  switch (config) {
    case 1:
      s = {512, 8192, 128, 256, 128, 32, 8, 4, 4, 200, 20, 100, 100, 2000, 10, 10, 8, 20, false};
      break;
    case 2:
      s = {2400, 88000, 220, 600, 1200, 70, 60, 4, 4, 400, 20, 100, 100, 25000, 10, 10, 12, 50, true};
      break;
    case 5:
      s = {24000, 880000, 2200, 6000, 12000, 700, 600, 4, 4, 400, 20, 100, 100, 25000, 10, 10, 12,
           50, true};
      break;
    default:
      return set_error(SGB_ERR_ARG, "unknown scaffold config %d (1, 2 or 5)", config);
  }
  auto sz = [&](int32_t n) { return (int32_t)std::max(1.0, floor(n * scale + 0.5)); };
  const float ch[8] = {1.0f, 0.0f, 1.0f, 0.5f, 1.0f, -80.0f, 1.0f, 10.0f};
  int32_t mf, grc, goc, sc, bc, pc, dcn;
  int rc = 0;
#define LIF(name, n, type, id) \
  rc = add_population(net, name, sz(n), 3.0f, -70.0f, 2.0f, 0.0f, -70.0f, -50.0f, 0.2f, type, 2, ch, &id); \
  if (rc) return rc;
  rc = add_population(net, "mossy", sz(s.mossy), 0, 0, 0, 0, 0, 0, 0, SGB_INPUT, 0, nullptr, &mf);
  if (rc) return rc;
  LIF("granule", s.granule, SGB_NORMAL, grc)
  LIF("golgi", s.golgi, SGB_NORMAL, goc)
  LIF("stellate", s.stellate, SGB_NORMAL, sc)
  LIF("basket", s.basket, SGB_NORMAL, bc)
  LIF("purkinje", s.purkinje, SGB_NORMAL, pc)
  LIF("dcn", s.dcn, SGB_OUTPUT, dcn)
#undef LIF
  auto kdeg = [&](int32_t k, int32_t pre) { return std::min(k, net.pops[pre].num); };
  struct P { int32_t pre, post, k, ch; float drive; };
  const P projs[] = {
      {mf, grc, s.k_grc_mf, SGB_CH_EXC, kDriveGrcMf},   {goc, grc, s.k_grc_goc, SGB_CH_INH, kDriveGrcGoc},
      {grc, goc, s.k_goc_grc, SGB_CH_EXC, kDriveGocGrc}, {mf, goc, s.k_goc_mf, SGB_CH_EXC, kDriveGocMf},
      {grc, sc, s.k_sc_grc, SGB_CH_EXC, kDriveScGrc},    {grc, bc, s.k_bc_grc, SGB_CH_EXC, kDriveBcGrc},
      {grc, pc, s.k_pc_grc, SGB_CH_EXC, kDrivePcGrc},    {sc, pc, s.k_pc_sc, SGB_CH_INH, kDrivePcSc},
      {bc, pc, s.k_pc_bc, SGB_CH_INH, kDrivePcBc},       {pc, dcn, s.k_dcn_pc, SGB_CH_INH, kDriveDcnPc},
      {mf, dcn, s.k_dcn_mf, SGB_CH_EXC, kDriveDcnMf},
  };
  int i = 0;
  for (const P& p : projs) {
    const int32_t k = kdeg(p.k, p.pre);
    const float mean = k > 0 ? p.drive / (float)k : 0.f;
    rc = add_random_projection(net, p.pre, p.post, k, mean, 0.5f, 1.5f, 1, 4, p.ch,
                               seed * 1000003ull + (uint64_t)(++i), SGB_PROP_AUTO, nullptr);
    if (rc) return rc;
  }
  sgb_input_params bg{SGB_INPUT_POISSON, 4.0f, 0.0, 0.0, 0.0, 0.0};
  rc = add_input(net, mf, -1, nullptr, &bg, nullptr);
  if (rc) return rc;
  if (s.burst) {
    const int32_t nb = std::max(1, net.pops[mf].num / 10);
    std::vector<uint32_t> ids(nb);
    std::iota(ids.begin(), ids.end(), 0u);
    sgb_input_params burst{SGB_INPUT_POISSON, 100.0f, 0.0, 1000.0, 260.0, 300.0};
    rc = add_input(net, mf, nb, ids.data(), &burst, nullptr);
    if (rc) return rc;
  }
  return SGB_OK;
}

}  // namespace sgb
