// Harness around the reference's compiled CPU functions -- TEST INFRASTRUCTURE ONLY.
//
// Links host_update_lif_ch and host_spike_propagation compiled from the
// reference's own Simulation_header.cu (build_ref.py; the source is never
// copied) and drives them over a network description with the same step
// order as the reference's loops (inputs, every projection's pull, every LIF
// population's update; GPUScaffoldSimulation.cu:717-765 and :20-46).  Setup,
// input cells and bookkeeping come from refport.c, so rh_run and rp_run
// differ only in whose compute loops they call.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <new>

#include "Simulation_header.h"  // reference declarations (-I <reference>/SimulationModule/Scaffold)
#include "refport.h"
#ifdef _OPENMP
#include <omp.h>
#endif

struct rh_sim {
  rp_sim* rp;
  Sim_cond_lif_exp* dev;
  pthread_val* pa;
  float* chan[7][4];  // w, E, g_bar, tau per population
  int type_ids[TotalNumOfCellTypes];
  FILE* sink;
};

extern "C" {

int rh_step_max(void) { return STEP_MAX; }

int rh_create(const orc_net* net, rh_sim** out) {
  if (net->n_pops > (int)TotalNumOfCellTypes) return -10;
  if (net->substeps != STEP_MAX || net->dt_ms != (double)DT) return -10;
  for (int p = 0; p < net->n_pops; ++p)
    if (!net->pops[p].is_input && net->pops[p].c_num != 2) return -10;
  rh_sim* h = new (std::nothrow) rh_sim();
  if (!h) return -9;
  int rc = rp_create(net, &h->rp);
  if (rc) { delete h; return rc; }
  h->dev = new Sim_cond_lif_exp();
  h->pa = new pthread_val();
  h->dev->print_arg = h->pa;
  h->pa->host_spike = h->rp->spk;
  h->dev->total_neuron_num = (int)h->rp->N;
  for (int p = 0; p < net->n_pops; ++p) {
    h->dev->neurons[p].base_id = (int)h->rp->base[p];
    h->dev->start[p] = 0;
    h->dev->end[p] = (unsigned)net->pops[p].num;
    h->type_ids[p] = p;
    for (int k = 0; k < 4; ++k) h->chan[p][k] = (float*)calloc(2, sizeof(float));
    for (int c = 0; c < net->pops[p].c_num; ++c) {
      h->chan[p][0][c] = net->pops[p].w[c];
      h->chan[p][1][c] = net->pops[p].E[c];
      h->chan[p][2][c] = net->pops[p].gbar[c];
      h->chan[p][3][c] = net->pops[p].tau[c];
    }
  }
  h->sink = fopen("/dev/null", "w");
  *out = h;
  return 0;
}

void rh_destroy(rh_sim* h) {
  if (!h) return;
  for (int p = 0; p < h->rp->net.n_pops; ++p)
    for (int k = 0; k < 4; ++k) free(h->chan[p][k]);
  rp_destroy(h->rp);
  delete h->dev;
  delete h->pa;
  if (h->sink) fclose(h->sink);
  delete h;
}

int rh_run(rh_sim* h, int64_t n_steps, int32_t threads, uint32_t* counts, uint32_t* raster,
           int64_t raster_cap, int64_t* raster_off) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  rp_sim* s = h->rp;
  const orc_net& net = s->net;
  int64_t rfill = 0;
  int overflow = 0;
  if (raster_off) raster_off[0] = 0;
  for (int64_t k = 0; k < n_steps; ++k) {
    const int32_t r = (int32_t)(s->step % (uint64_t)s->R);
    char* row = s->spk + (int64_t)r * s->N;
    rp_begin_step(s, row);
    for (int i = 0; i < s->n_tabs; ++i) {
      const rp_tab* t = &s->tabs[i];
      const int32_t rr = (r + s->R - t->delay) % s->R;
      const int npost = net.pops[t->post].num;
      const int chunk = 256;
      float* dg = t->channel ? s->dg_inh : s->dg_exc;
#pragma omp parallel for schedule(static)
      for (int c0 = 0; c0 < npost; c0 += chunk) {
        const int len = npost - c0 < chunk ? npost - c0 : chunk;
        host_spike_propagation(t->pre, len, (int)s->base[t->post] + c0, dg, t->max_conv,
                               t->cind + (int64_t)c0 * t->max_conv,
                               t->w + (int64_t)c0 * t->max_conv, 1.0f, rr, 0, h->dev);
      }
    }
    for (int p = 0; p < net.n_pops; ++p) {
      const orc_pop& P = net.pops[p];
      if (P.is_input) continue;
      const int chunk = 1024;
#pragma omp parallel for schedule(static)
      for (int c0 = 0; c0 < P.num; c0 += chunk) {
        Neuron target;
        memset(&target, 0, sizeof target);
        target.type = p;
        target.num = P.num - c0 < chunk ? P.num - c0 : chunk;
        target.base_id = (int)s->base[p] + c0;
        target.Cm = P.Cm; target.El = P.El; target.dt_ref = P.dt_ref; target.Ie = P.Ie;
        target.Vr = P.Vr; target.Vth = P.Vth; target.gL = P.gL;
        target.w = h->chan[p][0]; target.E = h->chan[p][1];
        target.g_bar = h->chan[p][2]; target.tau = h->chan[p][3];
        target.g = s->g;
        target.c_num = P.c_num;
        target.dev_type = NORMAL;
        host_update_lif_ch(s->u, s->dg_exc, s->dg_inh, s->Inoise, row, s->ref, target, r,
                           (float)s->step, h->sink, h->type_ids);
      }
    }
    overflow |= rp_end_step(s, row, k, counts, raster, raster_cap, &rfill);
    if (raster_off) raster_off[k + 1] = rfill;
  }
  return overflow ? -7 : 0;
}

int rh_get_state(const rh_sim* h, float* u, float* g, int32_t* ref) {
  return rp_get_state(h->rp, u, g, ref);
}

}  // extern "C"
