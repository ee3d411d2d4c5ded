/*
 * Restatement of the reference's CPU loops -- TEST INFRASTRUCTURE ONLY
 * (see refport.h).
 */
#include "refport.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static float bf16r(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
  memcpy(&f, &u, 4);
  return f;
}

int rp_create(const orc_net* net, rp_sim** out) {
  rp_sim* s = (rp_sim*)calloc(1, sizeof(rp_sim));
  if (!s) return -9;
  s->net = *net;
  orc_net in = *net;
  in.mode = ORC_FP32;
  int rc = orc_create(&in, &s->inputs);
  if (rc) { free(s); return rc; }
  const int np = net->n_pops;
  s->base = (int64_t*)calloc((size_t)np + 1, sizeof(int64_t));
  for (int p = 0; p < np; ++p) s->base[p + 1] = s->base[p] + net->pops[p].num;
  s->N = s->base[np];
  int maxd = 1;
  for (int i = 0; i < net->n_projs; ++i)
    for (int64_t q = 0; q < net->projs[i].n; ++q)
      if (net->projs[i].delay[q] > maxd) maxd = net->projs[i].delay[q];
  s->R = maxd + 1;
  /* One ELL table per (projection, delay) that has synapses, in projection
   * order then ascending delay; rows keep the stored synapse order
   * (LoadConnectivityFile_ELL fills rows in file order, init_params.cu:38-53). */
  s->tabs = (rp_tab*)calloc((size_t)(net->n_projs * maxd + 1), sizeof(rp_tab));
  for (int i = 0; i < net->n_projs; ++i) {
    const orc_proj* pr = &net->projs[i];
    const int64_t npost = net->pops[pr->post].num;
    int32_t* col = (int32_t*)calloc((size_t)(npost > 0 ? npost : 1), sizeof(int32_t));
    for (int d = 1; d <= maxd; ++d) {
      memset(col, 0, (size_t)npost * sizeof(int32_t));
      int32_t mc = 0;
      for (int64_t q = 0; q < pr->n; ++q)
        if (pr->delay[q] == d && ++col[pr->post_idx[q]] > mc) mc = col[pr->post_idx[q]];
      if (!mc) continue;
      rp_tab* t = &s->tabs[s->n_tabs++];
      t->proj = i; t->pre = pr->pre; t->post = pr->post; t->channel = pr->channel;
      t->delay = d; t->max_conv = mc;
      t->cind = (int32_t*)malloc((size_t)npost * mc * sizeof(int32_t));
      t->w = (float*)calloc((size_t)npost * mc, sizeof(float));
      for (int64_t k = 0; k < npost * mc; ++k) t->cind[k] = -1;
      memset(col, 0, (size_t)npost * sizeof(int32_t));
      for (int64_t q = 0; q < pr->n; ++q) {
        if (pr->delay[q] != d) continue;
        const int64_t at = (int64_t)pr->post_idx[q] * mc + col[pr->post_idx[q]]++;
        t->cind[at] = (int32_t)pr->pre_idx[q];
        t->w[at] = net->bf16 ? bf16r(pr->weight[q]) : pr->weight[q];
      }
    }
    free(col);
  }
  const int64_t N = s->N > 0 ? s->N : 1;
  s->u = (float*)calloc((size_t)N, 4);
  s->g = (float*)calloc((size_t)N * 2, 4);
  s->dg_exc = (float*)calloc((size_t)N, 4);
  s->dg_inh = (float*)calloc((size_t)N, 4);
  s->Inoise = (float*)calloc((size_t)N, 4);
  s->ref = (int32_t*)calloc((size_t)N, 4);
  s->spk = (char*)calloc((size_t)s->R * N, 1);
  /* Same initial potentials as the oracle (one Philox draw per cell). */
  orc_get_state(s->inputs, s->u, NULL, NULL);
  *out = s;
  return 0;
}

void rp_destroy(rp_sim* s) {
  if (!s) return;
  for (int i = 0; i < s->n_tabs; ++i) { free(s->tabs[i].cind); free(s->tabs[i].w); }
  free(s->tabs); free(s->base); free(s->u); free(s->g); free(s->dg_exc); free(s->dg_inh);
  free(s->Inoise); free(s->ref); free(s->spk);
  orc_destroy(s->inputs);
  free(s);
}

void rp_begin_step(rp_sim* s, char* row) {
  /* Input cells of this step (InputStimulation writes row target_row,
   * GPUScaffoldSimulation.cu:720-725). */
  orc_input_flags(s->inputs, s->step, (uint8_t*)row);
}

int rp_end_step(rp_sim* s, const char* row, int64_t step, uint32_t* counts, uint32_t* raster,
                int64_t raster_cap, int64_t* rfill) {
  int overflow = 0;
  for (int p = 0; p < s->net.n_pops; ++p) {
    uint32_t c = 0;
    for (int64_t id = s->base[p]; id < s->base[p + 1]; ++id) {
      if (!row[id]) continue;
      ++c;
      if (raster) {
        if (*rfill < raster_cap) raster[(*rfill)++] = (uint32_t)id; else overflow = 1;
      }
    }
    if (counts) counts[step * s->net.n_pops + p] = c;
  }
  s->step++;
  return overflow;
}

/* host_spike_propagation (Simulation_header.cu:468-493) for one table:
 * for every post cell, sum spike[pre] * weight over its row (stopping at the
 * first -1), then dg[post] += sum * w_bar. */
static void propagate(rp_sim* s, const rp_tab* t, const char* read_row, float* dg) {
  const int64_t npost = s->net.pops[t->post].num;
  const int64_t pre0 = s->base[t->pre], post0 = s->base[t->post];
  const int32_t mc = t->max_conv;
  const float w_bar = 1.0f;
#pragma omp parallel for schedule(static)
  for (int64_t post = 0; post < npost; ++post) {
    float _dg = 0;
    const int32_t* ci = t->cind + post * mc;
    const float* w = t->w + post * mc;
    for (int32_t i = 0; i < mc; ++i) {
      if (ci[i] < 0) break;
      _dg += (read_row[pre0 + ci[i]]) * w[i];
    }
    dg[post0 + post] += _dg * w_bar;
  }
}

/* host_update_lif_ch (Simulation_header.cu:385-465): FP32 state, double DT. */
static void update(rp_sim* s, int p, char* row) {
  const orc_pop* P = &s->net.pops[p];
  const double DT = s->net.dt_ms;
  const int STEP_MAX = s->net.substeps;
  const int c_num = P->c_num;
  const float u_rest = P->El, u_reset = P->Vr, u_th = P->Vth;
  const int ref_step = (int)(P->dt_ref / DT);
  const float Cm = P->Cm, Ie = P->Ie, gL = P->gL;
  float* g = s->g;
  const int64_t b0 = s->base[p], b1 = s->base[p + 1];
#pragma omp parallel for schedule(static)
  for (int64_t global_id = b0; global_id < b1; ++global_id) {
    const int64_t ch_base = global_id * 2;
    float u_ = s->u[global_id];
    float du_ = 0;
    int IsRef = s->ref[global_id];
    int spike_ = 0;
    float Isyn = 0;
    {
      Isyn = 0;
      for (int c = 0; c < c_num; c++) Isyn += g[ch_base + c] * (u_ - P->E[c]);
      du_ = (DT / Cm) * (Ie - gL * (u_ - u_rest) - Isyn);
      for (int c = 0; c < c_num; c++)
        g[ch_base + c] += -(DT / P->tau[c]) * g[ch_base + c] +
                          P->gbar[c] * P->w[c] *
                              ((P->E[c] > u_rest) ? s->dg_exc[global_id] : s->dg_inh[global_id]);
      spike_ = (u_ > u_th);
      IsRef = (u_ > u_th) ? ref_step : (IsRef > 0) ? IsRef - 1 : 0;
      u_ = (IsRef > 0) ? u_reset : u_ + du_;
    }
    for (int step = 1; step < STEP_MAX; step++) {
      Isyn = 0;
      for (int c = 0; c < c_num; c++) Isyn += g[ch_base + c] * (u_ - P->E[c]);
      du_ = (DT / Cm) * (Ie - gL * (u_ - u_rest) - Isyn);
      for (int c = 0; c < c_num; c++) g[ch_base + c] += -(DT / P->tau[c]) * g[ch_base + c];
      spike_ += (u_ > u_th);
      IsRef = (u_ > u_th) ? ref_step : (IsRef > 0) ? IsRef - 1 : 0;
      u_ = (IsRef > 0) ? u_reset : u_ + du_;
    }
    s->u[global_id] = u_;
    row[global_id] = (spike_ > 0) ? 1 : 0;
    s->ref[global_id] = IsRef;
    s->dg_exc[global_id] = 0;
    s->dg_inh[global_id] = 0;
  }
}

int rp_run(rp_sim* s, int64_t n_steps, int32_t threads, uint32_t* counts, uint32_t* raster,
           int64_t raster_cap, int64_t* raster_off) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  int64_t rfill = 0;
  int overflow = 0;
  if (raster_off) raster_off[0] = 0;
  for (int64_t k = 0; k < n_steps; ++k) {
    const int32_t r = (int32_t)(s->step % (uint64_t)s->R);
    char* row = s->spk + (int64_t)r * s->N;
    rp_begin_step(s, row);
    for (int i = 0; i < s->n_tabs; ++i) {
      const rp_tab* t = &s->tabs[i];
      const int32_t rr = (int32_t)((r + s->R - t->delay) % s->R);
      propagate(s, t, s->spk + (int64_t)rr * s->N, t->channel ? s->dg_inh : s->dg_exc);
    }
    for (int p = 0; p < s->net.n_pops; ++p)
      if (!s->net.pops[p].is_input) update(s, p, row);
    overflow |= rp_end_step(s, row, k, counts, raster, raster_cap, &rfill);
    if (raster_off) raster_off[k + 1] = rfill;
  }
  return overflow ? -7 : 0;
}

int rp_get_state(const rp_sim* s, float* u, float* g, int32_t* ref) {
  for (int p = 0; p < s->net.n_pops; ++p) {
    const int inp = s->net.pops[p].is_input;
    for (int64_t id = s->base[p]; id < s->base[p + 1]; ++id) {
      if (u) u[id] = inp ? 0.f : s->u[id];
      if (g) { g[2 * id] = inp ? 0.f : s->g[2 * id]; g[2 * id + 1] = inp ? 0.f : s->g[2 * id + 1]; }
      if (ref) ref[id] = inp ? 0 : s->ref[id];
    }
  }
  return 0;
}
