/*
 * CPU oracle of the scaffold simulation hot path -- TEST INFRASTRUCTURE ONLY
 * (see oracle.h).  Build: make -C oracle  (gcc, -ffp-contract=off).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---- Philox4x32-10 (Salmon et al., SC'11) ------------------------------ */
static uint32_t mulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    const uint32_t a = 0xD2511F53u, b = 0xCD9E8D57u;
    const uint32_t n0 = mulhi(b, c2) ^ c1 ^ k0;
    const uint32_t n1 = b * c2;
    const uint32_t n2 = mulhi(a, c0) ^ c3 ^ k1;
    const uint32_t n3 = a * c0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Draw block of (seed; neuron, step, tag, block): counter {neuron, step lo,
 * step hi, tag | block << 8}, key {seed lo, seed hi}. */
static void draw4(uint64_t seed, uint32_t neuron, uint64_t step, uint32_t tag, uint32_t block,
                  uint32_t out[4]) {
  const uint32_t c[4] = {neuron, (uint32_t)step, (uint32_t)(step >> 32), tag | (block << 8)};
  const uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  orc_philox4x32_10(c, k, out);
}

#define TAG_INPUT 1u
#define TAG_INIT_U 2u

static float bf16_round(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
  memcpy(&f, &u, 4);
  return f;
}

static float table_w(const orc_net* n, float w) { return n->bf16 ? bf16_round(w) : w; }

/* ---- accumulator scale rule -------------------------------------------- */
int32_t orc_scale_bits(const orc_net* net, int32_t pop, int32_t ch) {
  const int64_t npost = net->pops[pop].num;
  int64_t* sum = (int64_t*)calloc((size_t)(npost > 0 ? npost : 1), sizeof(int64_t));
  int any = 0;
  for (int i = 0; i < net->n_projs; ++i)
    any |= net->projs[i].post == pop && net->projs[i].channel == ch && net->projs[i].n > 0;
  int32_t s = 30;
  if (any) {
    for (; s > -100; --s) {
      memset(sum, 0, (size_t)npost * sizeof(int64_t));
      const float scale = ldexpf(1.0f, s);
      int64_t mx = 0;
      for (int i = 0; i < net->n_projs; ++i) {
        const orc_proj* p = &net->projs[i];
        if (p->post != pop || p->channel != ch) continue;
        for (int64_t q = 0; q < p->n; ++q) {
          int64_t* v = &sum[p->post_idx[q]];
          *v += (int64_t)rintf(table_w(net, p->weight[q]) * scale);
          if (*v > mx) mx = *v;
        }
      }
      if (mx <= 2147483647ll) break;
    }
  }
  free(sum);
  return s;
}

/* ---- simulation state ---------------------------------------------------- */
typedef struct {
  int64_t* row;     /* [npre + 1] */
  uint32_t* post;
  uint8_t* delay;
  int32_t* wfix;    /* FP32 mode */
  double* wd;       /* FP64 mode */
} push_rows;

/* One plastic projection. */
typedef struct {
  const orc_plast* p;
  float* v32;         /* per synapse */
  double* v64;
  float* w0;          /* w * 2^S per synapse (FP32 mode) */
  int64_t* teacher;   /* per post: global id of the teacher cell, -1 none */
  int32_t* tdelay;    /* per post: delay of the teacher synapse */
} plast_state;

struct orc_sim {
  orc_net net;
  plast_state* pl;          /* [n_plast] */
  int32_t* plast_of;        /* [n_projs]: index into pl or -1 */
  uint8_t* hist;            /* [H][n_cells] spikes, row = step % H */
  int32_t H;
  int64_t n_cells;
  int64_t* base;            /* [n_pops] first global id */
  int32_t D;                /* ring slots */
  int32_t* scale_bits;      /* [n_pops][2] */
  push_rows* rows;          /* [n_projs] */
  uint32_t* src_mask;       /* [n_cells] */
  uint64_t* thresh;         /* [n_srcs] */
  float* rates;             /* [n_srcs] */
  /* state */
  float *u32, *g32;         /* FP32 */
  double *u64, *g64;        /* FP64 */
  int32_t* ref;
  int32_t* ring_fix;        /* [D][n_cells][2] */
  double* ring_d;
  uint8_t* spk;             /* spikes of the current step */
  uint64_t step;
  int64_t events;
};

static uint64_t thresh_of(float rate, double dt) {
  const double p = (double)rate * dt / 1000.0;
  if (!(p > 0.0)) return 0;
  if (p >= 1.0) return 1ull << 32;
  return (uint64_t)floor(p * 4294967296.0);
}

int orc_set_rates(orc_sim* s, const float* rates) {
  for (int i = 0; i < s->net.n_srcs; ++i) {
    s->rates[i] = rates ? rates[i] : s->net.srcs[i].rate_hz;
    s->thresh[i] = thresh_of(s->rates[i], s->net.dt_ms);
  }
  return 0;
}

int orc_create(const orc_net* net, orc_sim** out) {
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  if (!s) return -9;
  s->net = *net;
  const int np = net->n_pops;
  s->base = (int64_t*)calloc((size_t)np + 1, sizeof(int64_t));
  for (int p = 0; p < np; ++p) s->base[p + 1] = s->base[p] + net->pops[p].num;
  s->n_cells = s->base[np];
  const int64_t N = s->n_cells > 0 ? s->n_cells : 1;
  int maxd = 1;
  for (int i = 0; i < net->n_projs; ++i)
    for (int64_t q = 0; q < net->projs[i].n; ++q)
      if (net->projs[i].delay[q] > maxd) maxd = net->projs[i].delay[q];
  s->D = maxd + 1;
  s->scale_bits = (int32_t*)calloc((size_t)np * 2, sizeof(int32_t));
  for (int p = 0; p < np; ++p)
    for (int c = 0; c < 2; ++c) s->scale_bits[p * 2 + c] = orc_scale_bits(net, p, c);
  /* Pre-major rows of every projection (delivery loops over spiking pres). */
  s->rows = (push_rows*)calloc((size_t)(net->n_projs > 0 ? net->n_projs : 1), sizeof(push_rows));
  for (int i = 0; i < net->n_projs; ++i) {
    const orc_proj* p = &net->projs[i];
    push_rows* r = &s->rows[i];
    const int64_t npre = net->pops[p->pre].num;
    r->row = (int64_t*)calloc((size_t)npre + 1, sizeof(int64_t));
    r->post = (uint32_t*)malloc((size_t)(p->n > 0 ? p->n : 1) * 4);
    r->delay = (uint8_t*)malloc((size_t)(p->n > 0 ? p->n : 1));
    r->wfix = (int32_t*)malloc((size_t)(p->n > 0 ? p->n : 1) * 4);
    r->wd = (double*)malloc((size_t)(p->n > 0 ? p->n : 1) * 8);
    for (int64_t q = 0; q < p->n; ++q) r->row[p->pre_idx[q] + 1]++;
    for (int64_t j = 0; j < npre; ++j) r->row[j + 1] += r->row[j];
    int64_t* fill = (int64_t*)malloc((size_t)(npre > 0 ? npre : 1) * sizeof(int64_t));
    memcpy(fill, r->row, (size_t)npre * sizeof(int64_t));
    const float scale = ldexpf(1.0f, s->scale_bits[p->post * 2 + p->channel]);
    for (int64_t q = 0; q < p->n; ++q) {
      const int64_t o = fill[p->pre_idx[q]]++;
      r->post[o] = p->post_idx[q];
      r->delay[o] = p->delay[q];
      r->wfix[o] = (int32_t)rintf(table_w(net, p->weight[q]) * scale);
      r->wd[o] = (double)p->weight[q];
    }
    free(fill);
  }
  s->src_mask = (uint32_t*)calloc((size_t)N, sizeof(uint32_t));
  s->thresh = (uint64_t*)calloc((size_t)(net->n_srcs > 0 ? net->n_srcs : 1), sizeof(uint64_t));
  s->rates = (float*)calloc((size_t)(net->n_srcs > 0 ? net->n_srcs : 1), sizeof(float));
  for (int i = 0; i < net->n_srcs; ++i) {
    const orc_src* src = &net->srcs[i];
    for (int64_t q = 0; q < src->n_ids; ++q) s->src_mask[s->base[src->pop] + src->ids[q]] |= 1u << i;
  }
  orc_set_rates(s, NULL);
  s->u32 = (float*)calloc((size_t)N, 4);
  s->g32 = (float*)calloc((size_t)N * 2, 4);
  s->u64 = (double*)calloc((size_t)N, 8);
  s->g64 = (double*)calloc((size_t)N * 2, 8);
  s->ref = (int32_t*)calloc((size_t)N, 4);
  s->ring_fix = (int32_t*)calloc((size_t)s->D * N * 2, 4);
  s->ring_d = (double*)calloc((size_t)s->D * N * 2, 8);
  s->spk = (uint8_t*)calloc((size_t)N, 1);
  /* Plasticity: values start at 1; history deep enough for the window. */
  s->plast_of = (int32_t*)malloc((size_t)(net->n_projs > 0 ? net->n_projs : 1) * 4);
  for (int i = 0; i < net->n_projs; ++i) s->plast_of[i] = -1;
  s->pl = (plast_state*)calloc((size_t)(net->n_plast > 0 ? net->n_plast : 1), sizeof(plast_state));
  s->H = 0;
  for (int k = 0; k < net->n_plast; ++k) {
    const orc_plast* pp = &net->plast[k];
    const orc_proj* p = &net->projs[pp->proj];
    plast_state* ps = &s->pl[k];
    s->plast_of[pp->proj] = k;
    ps->p = pp;
    const int64_t m = p->n > 0 ? p->n : 1;
    ps->v32 = (float*)malloc((size_t)m * 4);
    ps->v64 = (double*)malloc((size_t)m * 8);
    ps->w0 = (float*)malloc((size_t)m * 4);
    const float scale = ldexpf(1.0f, s->scale_bits[p->post * 2 + p->channel]);
    int dmax = 1;
    for (int64_t q = 0; q < p->n; ++q) {
      ps->v32[q] = pp->v_max;  /* values start at the clamp (reference: 1) */
      ps->v64[q] = (double)pp->v_max;
      ps->w0[q] = p->weight[q] * scale; /* power of two: exact */
      if (p->delay[q] > dmax) dmax = p->delay[q];
    }
    const int need = (maxd + 1 > dmax + pp->window) ? maxd + 1 : dmax + pp->window;
    if (need > s->H) s->H = need;
    const int64_t npost = net->pops[p->post].num > 0 ? net->pops[p->post].num : 1;
    ps->teacher = (int64_t*)malloc((size_t)npost * 8);
    ps->tdelay = (int32_t*)calloc((size_t)npost, 4);
    for (int64_t j = 0; j < npost; ++j) ps->teacher[j] = -1;
    if (pp->rule == 1) {
      /* teacher of a post: its teacher synapse of lowest (delay, pre id) */
      const orc_proj* tp = &net->projs[pp->teacher_proj];
      for (int64_t q = 0; q < tp->n; ++q) {
        const uint32_t j = tp->post_idx[q];
        const int64_t g = s->base[tp->pre] + tp->pre_idx[q];
        const int32_t d = tp->delay[q];
        if (ps->teacher[j] < 0 || d < ps->tdelay[j] ||
            (d == ps->tdelay[j] && g < ps->teacher[j])) {
          ps->teacher[j] = g;
          ps->tdelay[j] = d;
        }
      }
    }
  }
  s->hist = s->H ? (uint8_t*)calloc((size_t)s->H * N, 1) : NULL;
  /* u0 = Vr + (Vth - Vr) * U(0,1] (init_params.cu:346); id = global index. */
  for (int p = 0; p < np; ++p) {
    const orc_pop* P = &net->pops[p];
    if (P->is_input) continue;
    for (int64_t j = 0; j < P->num; ++j) {
      const int64_t id = s->base[p] + j;
      uint32_t r[4];
      draw4(net->seed, (uint32_t)id, 0, TAG_INIT_U, 0, r);
      const float U = (float)((r[0] >> 8) + 1u) * (1.0f / 16777216.0f);
      s->u32[id] = fmaf(P->Vth - P->Vr, U, P->Vr);
      s->u64[id] = (double)P->Vr + ((double)P->Vth - (double)P->Vr) * (double)U;
    }
  }
  *out = s;
  return 0;
}

void orc_destroy(orc_sim* s) {
  if (!s) return;
  for (int i = 0; i < s->net.n_projs; ++i) {
    free(s->rows[i].row); free(s->rows[i].post); free(s->rows[i].delay);
    free(s->rows[i].wfix); free(s->rows[i].wd);
  }
  free(s->rows); free(s->base); free(s->scale_bits); free(s->src_mask); free(s->thresh);
  free(s->rates); free(s->u32); free(s->g32); free(s->u64); free(s->g64); free(s->ref);
  free(s->ring_fix); free(s->ring_d); free(s->spk);
  for (int k = 0; k < s->net.n_plast; ++k) {
    free(s->pl[k].v32); free(s->pl[k].v64); free(s->pl[k].w0);
    free(s->pl[k].teacher); free(s->pl[k].tdelay);
  }
  free(s->pl); free(s->plast_of); free(s->hist);
  free(s);
}

/* ---- one input cell (InputStimulation, UserInputFunctions.cu:86-120) ----- */
static int src_window(const orc_src* src, double dt, int64_t k) {
  int64_t w0 = llround(src->win_start_ms / dt), w1 = llround(src->win_end_ms / dt);
  if (w1 <= w0) return 1;
  int64_t kk = k;
  const int64_t per = src->win_period_ms > 0 ? llround(src->win_period_ms / dt) : 0;
  if (per > 0) {
    kk = k % per;
    if (kk < 0) kk += per;
  }
  return kk >= w0 && kk < w1;
}

static int input_cell(const orc_sim* s, int64_t id, uint64_t t) {
  const uint32_t mask = s->src_mask[id];
  if (!mask) return 0;
  const orc_net* n = &s->net;
  int fire = 0;
  uint32_t r[4] = {0, 0, 0, 0};
  for (int sub = 0; sub < n->substeps; ++sub) {
    if (sub % 4 == 0) draw4(n->seed, (uint32_t)id, t, TAG_INPUT, (uint32_t)(sub / 4), r);
    const uint32_t x = r[sub % 4];
    const int64_t k = (int64_t)t * n->substeps + sub;
    for (int i = 0; i < n->n_srcs; ++i) {
      if (!((mask >> i) & 1u)) continue;
      const orc_src* src = &n->srcs[i];
      if (!src_window(src, n->dt_ms, k)) continue;
      if (src->kind == 0) {
        fire |= (uint64_t)x < s->thresh[i];
      } else {
        /* PeriodicFiring: the cycle count floor((t - start) f / 1000) steps up. */
        const double cyc = n->dt_ms * (double)s->rates[i] / 1000.0;
        const int64_t kp = llround(src->phase_ms / n->dt_ms);
        fire |= floor((double)(k - kp) * cyc) != floor((double)(k - kp - 1) * cyc);
      }
    }
  }
  return fire;
}

/* ---- per-population LIF constants -------------------------------------- */
typedef struct {
  float dt_cm, keep[2], gw[2], E[2];
  double dt_cm_d, keep_d[2], gw_d[2];
  int32_t ref_steps;
  int sel[2];
} lif_k;

static void lif_consts(const orc_pop* P, double dt, lif_k* k) {
  memset(k, 0, sizeof *k);
  k->dt_cm = (float)(dt / (double)P->Cm);
  k->dt_cm_d = dt / (double)P->Cm;
  /* ref_step = (int)(dt_ref / DT) in double (Simulation_header.cu:322) */
  k->ref_steps = (int32_t)((double)P->dt_ref / dt);
  for (int c = 0; c < P->c_num; ++c) {
    k->keep[c] = (float)(1.0 - dt / (double)P->tau[c]);
    k->keep_d[c] = 1.0 - dt / (double)P->tau[c];
    k->gw[c] = P->gbar[c] * P->w[c];
    k->gw_d[c] = (double)P->gbar[c] * (double)P->w[c];
    k->E[c] = P->E[c];
    /* channel c integrates dg_exc iff E_c > E_L (Simulation_header.cu:347) */
    k->sel[c] = P->E[c] > P->El ? 0 : 1;
  }
}

/* ---- LIF cell, FP32 formulation of the device kernel -------------------- */
static int lif32(const orc_pop* P, const lif_k* k, int substeps, float* u_, float* g,
                 int32_t* ref_, int32_t acc_e, int32_t acc_i, float inv_e, float inv_i) {
  const float dge = (float)acc_e * inv_e;
  const float dgi = (float)acc_i * inv_i;
  const float in0 = k->sel[0] ? dgi : dge, in1 = k->sel[1] ? dgi : dge;
  float u = *u_, g0 = g[0], g1 = g[1];
  int32_t ref = *ref_;
  int spk = 0;
  for (int sub = 0; sub < substeps; ++sub) {
    const float isyn = fmaf(g1, u - k->E[1], g0 * (u - k->E[0]));
    const float cur = fmaf(-P->gL, u - P->El, P->Ie) - isyn;
    const float du = k->dt_cm * cur;
    if (sub == 0) {
      g0 = fmaf(g0, k->keep[0], k->gw[0] * in0);
      g1 = fmaf(g1, k->keep[1], k->gw[1] * in1);
    } else {
      g0 = g0 * k->keep[0];
      g1 = g1 * k->keep[1];
    }
    const int above = u > P->Vth;
    spk |= above;
    ref = above ? k->ref_steps : (ref > 0 ? ref - 1 : 0);
    u = ref ? P->Vr : u + du;
  }
  *u_ = u; g[0] = g0; g[1] = g1; *ref_ = ref;
  return spk;
}

/* ---- LIF cell, FP64 ----------------------------------------------------- */
static int lif64(const orc_pop* P, const lif_k* k, int substeps, double* u_, double* g,
                 int32_t* ref_, double dge, double dgi) {
  const double in0 = k->sel[0] ? dgi : dge, in1 = k->sel[1] ? dgi : dge;
  const double E0 = P->c_num > 0 ? P->E[0] : 0.0, E1 = P->c_num > 1 ? P->E[1] : 0.0;
  double u = *u_, g0 = g[0], g1 = g[1];
  int32_t ref = *ref_;
  int spk = 0;
  for (int sub = 0; sub < substeps; ++sub) {
    const double isyn = g0 * (u - E0) + g1 * (u - E1);
    const double du = k->dt_cm_d * ((double)P->Ie - (double)P->gL * (u - (double)P->El) - isyn);
    if (sub == 0) {
      g0 = g0 * k->keep_d[0] + k->gw_d[0] * in0;
      g1 = g1 * k->keep_d[1] + k->gw_d[1] * in1;
    } else {
      g0 *= k->keep_d[0];
      g1 *= k->keep_d[1];
    }
    const int above = u > (double)P->Vth;
    spk |= above;
    ref = above ? k->ref_steps : (ref > 0 ? ref - 1 : 0);
    u = ref ? (double)P->Vr : u + du;
  }
  *u_ = u; g[0] = g0; g[1] = g1; *ref_ = ref;
  return spk;
}

/* ---- plasticity ------------------------------------------------------------ */
/* Spike of global cell g at step `step` (no spikes before step 0). */
static int spiked(const orc_sim* s, int64_t g, int64_t step) {
  if (step < 0) return 0;
  return s->hist[(step % s->H) * s->n_cells + g];
}

/* One step of Hebb_plasticity / Teacher_plasticity (SynapticPlasticity.cu:
 * 40-75, 78-120) over every synapse of the projection: dw = A0 + A1_J [pre
 * at t - d] + A1_I [post at t / teacher at t - its delay] + A2_JI x #window
 * pre spikes at t - d - s, summed in that order; v = clamp(v + dw). */
static void stdp_step(orc_sim* s, plast_state* ps, uint64_t t) {
  const orc_plast* pp = ps->p;
  const orc_proj* pr = &s->net.projs[pp->proj];
  const int fp64 = s->net.mode == ORC_FP64;
  const int64_t tt = (int64_t)t;
  for (int64_t q = 0; q < pr->n; ++q) {
    const int64_t pre_g = s->base[pr->pre] + pr->pre_idx[q];
    const int64_t d = pr->delay[q];
    const uint32_t j = pr->post_idx[q];
    int s_post;
    if (pp->rule == 0)
      s_post = s->spk[s->base[pr->post] + j];
    else
      s_post = ps->teacher[j] >= 0 && spiked(s, ps->teacher[j], tt - ps->tdelay[j]);
    const int s_pre = spiked(s, pre_g, tt - d);
    int nwin = 0;
    if (s_post && pp->a2_ji != 0.0f)
      for (int k = 0; k < pp->window; ++k) nwin += spiked(s, pre_g, tt - d - k);
    if (!fp64) {
      float dw = 0.0f + pp->a0;
      if (s_pre) dw = dw + pp->a1_j;
      if (s_post) dw = dw + pp->a1_i;
      for (int k = 0; k < nwin; ++k) dw = dw + pp->a2_ji;
      float v = ps->v32[q] + dw;
      v = v < 0.0f ? 0.0f : (v > pp->v_max ? pp->v_max : v);
      ps->v32[q] = v;
    } else {
      double dw = 0.0 + (double)pp->a0;
      if (s_pre) dw += (double)pp->a1_j;
      if (s_post) dw += (double)pp->a1_i;
      dw += (double)nwin * (double)pp->a2_ji;
      double v = ps->v64[q] + dw;
      v = v < 0.0 ? 0.0 : (v > (double)pp->v_max ? (double)pp->v_max : v);
      ps->v64[q] = v;
    }
  }
}

int orc_plastic_values(const orc_sim* s, int32_t proj, float* values) {
  if (proj < 0 || proj >= s->net.n_projs || s->plast_of[proj] < 0) return -1;
  const plast_state* ps = &s->pl[s->plast_of[proj]];
  const orc_proj* pr = &s->net.projs[proj];
  for (int64_t q = 0; q < pr->n; ++q)
    values[q] = s->net.mode == ORC_FP64 ? (float)ps->v64[q] : ps->v32[q];
  return 0;
}

int orc_run(orc_sim* s, int64_t n_steps, uint32_t* counts, uint32_t* raster, int64_t raster_cap,
            int64_t* raster_off) {
  const orc_net* n = &s->net;
  const int64_t N = s->n_cells;
  const int fp64 = n->mode == ORC_FP64;
  int64_t rfill = 0;
  int overflow = 0;
  if (raster_off) raster_off[0] = 0;
  for (int64_t step = 0; step < n_steps; ++step) {
    const uint64_t t = s->step;
    const int32_t slot = (int32_t)(t % (uint64_t)s->D);
    /* 1. cells of step t */
    for (int p = 0; p < n->n_pops; ++p) {
      const orc_pop* P = &n->pops[p];
      lif_k k;
      lif_consts(P, n->dt_ms, &k);
      const float inv_e = ldexpf(1.0f, -s->scale_bits[p * 2]);
      const float inv_i = ldexpf(1.0f, -s->scale_bits[p * 2 + 1]);
      uint32_t cnt = 0;
      for (int64_t j = 0; j < P->num; ++j) {
        const int64_t id = s->base[p] + j;
        int f;
        if (P->is_input) {
          f = input_cell(s, id, t);
        } else if (!fp64) {
          int32_t* acc = &s->ring_fix[((int64_t)slot * N + id) * 2];
          f = lif32(P, &k, n->substeps, &s->u32[id], &s->g32[id * 2], &s->ref[id], acc[0],
                    acc[1], inv_e, inv_i);
          acc[0] = acc[1] = 0;
        } else {
          double* acc = &s->ring_d[((int64_t)slot * N + id) * 2];
          f = lif64(P, &k, n->substeps, &s->u64[id], &s->g64[id * 2], &s->ref[id], acc[0],
                    acc[1]);
          acc[0] = acc[1] = 0.0;
        }
        s->spk[id] = (uint8_t)f;
        cnt += (uint32_t)f;
        if (f && raster) {
          if (rfill < raster_cap) raster[rfill++] = (uint32_t)id; else overflow = 1;
        }
      }
      if (counts) counts[step * n->n_pops + p] = cnt;
    }
    if (raster_off) raster_off[step + 1] = rfill;
    if (s->H) memcpy(&s->hist[(int64_t)(t % (uint64_t)s->H) * N], s->spk, (size_t)N);
    /* 2. plasticity of step t, then delivery of plastic projections on
     * arrival: spikes of step t + 1 - d into the accumulators of t + 1 */
    for (int k = 0; k < n->n_plast; ++k) stdp_step(s, &s->pl[k], t);
    for (int k = 0; k < n->n_plast; ++k) {
      const plast_state* ps = &s->pl[k];
      const orc_proj* pr = &n->projs[ps->p->proj];
      const int64_t sl = (int64_t)((t + 1) % (uint64_t)s->D);
      for (int64_t q = 0; q < pr->n; ++q) {
        const int64_t pre_g = s->base[pr->pre] + pr->pre_idx[q];
        if (!spiked(s, pre_g, (int64_t)t + 1 - pr->delay[q])) continue;
        const int64_t at = (sl * N + s->base[pr->post] + pr->post_idx[q]) * 2 + pr->channel;
        if (fp64)
          s->ring_d[at] += (double)pr->weight[q] * ps->v64[q];
        else
          s->ring_fix[at] += (int32_t)rintf(table_w(n, ps->w0[q] * ps->v32[q]));
      }
    }
    /* 3. delivery of step t's spikes into the accumulators of t + delay
     * (plastic projections: counted here, delivered above) */
    for (int i = 0; i < n->n_projs; ++i) {
      const orc_proj* pr = &n->projs[i];
      const push_rows* r = &s->rows[i];
      const int64_t pre0 = s->base[pr->pre], post0 = s->base[pr->post];
      for (int64_t j = 0; j < n->pops[pr->pre].num; ++j) {
        if (!s->spk[pre0 + j]) continue;
        s->events += r->row[j + 1] - r->row[j];
        if (s->plast_of[i] >= 0) continue;
        for (int64_t q = r->row[j]; q < r->row[j + 1]; ++q) {
          const int64_t sl = (int64_t)((t + r->delay[q]) % (uint64_t)s->D);
          const int64_t at = (sl * N + post0 + r->post[q]) * 2 + pr->channel;
          if (fp64) s->ring_d[at] += r->wd[q]; else s->ring_fix[at] += r->wfix[q];
        }
      }
    }
    s->step++;
  }
  return overflow ? -7 : 0;
}

int orc_get_state(const orc_sim* s, float* u, float* g, int32_t* ref) {
  const int fp64 = s->net.mode == ORC_FP64;
  for (int p = 0; p < s->net.n_pops; ++p) {
    for (int64_t j = 0; j < s->net.pops[p].num; ++j) {
      const int64_t id = s->base[p] + j;
      const int inp = s->net.pops[p].is_input;
      if (u) u[id] = inp ? 0.f : (fp64 ? (float)s->u64[id] : s->u32[id]);
      if (g) {
        g[2 * id] = inp ? 0.f : (fp64 ? (float)s->g64[2 * id] : s->g32[2 * id]);
        g[2 * id + 1] = inp ? 0.f : (fp64 ? (float)s->g64[2 * id + 1] : s->g32[2 * id + 1]);
      }
      if (ref) ref[id] = inp ? 0 : s->ref[id];
    }
  }
  return 0;
}

int orc_set_state(orc_sim* s, const float* u, const float* g, const int32_t* ref) {
  for (int64_t id = 0; id < s->n_cells; ++id) {
    if (u) { s->u32[id] = u[id]; s->u64[id] = u[id]; }
    if (g) {
      s->g32[2 * id] = g[2 * id]; s->g32[2 * id + 1] = g[2 * id + 1];
      s->g64[2 * id] = g[2 * id]; s->g64[2 * id + 1] = g[2 * id + 1];
    }
    if (ref) s->ref[id] = ref[id];
  }
  return 0;
}

int64_t orc_events(const orc_sim* s) { return s->events; }

int orc_input_flags(const orc_sim* s, uint64_t t, uint8_t* flags) {
  for (int p = 0; p < s->net.n_pops; ++p) {
    if (!s->net.pops[p].is_input) continue;
    for (int64_t j = 0; j < s->net.pops[p].num; ++j)
      flags[s->base[p] + j] = (uint8_t)input_cell(s, s->base[p] + j, t);
  }
  return 0;
}
