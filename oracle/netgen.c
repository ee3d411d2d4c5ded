/*
 * Synthetic scaffold generator of the oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * The benchmark networks are synthetic (the reference's .dat connectivity is
 * not available): seeded fixed in-degree projections with U[0.5, 1.5) x mean
 * weights and U{1..4}-step delays.  This file draws the same networks as the
 * library's generator without loading the library, so the CPU arms of the
 * benchmark (the reference's CPU loops and their restatement) build their
 * network from oracle code alone; a CPU test checks that both generators
 * return identical synapse arrays.
 *
 * Draw i of purpose q (0 pre ids, 1 weights, 2 delays) for post cell p of a
 * projection with seed s is component i % 4 of
 * Philox4x32-10(counter = (p, i / 4, 0, tag 3), key = s).  Pre ids are drawn
 * by Floyd's algorithm (distinct ids of [0, npre), sorted ascending).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define NETGEN_TAG 3u

typedef struct gen_stream {
  uint64_t seed;
  uint32_t post, purpose;
  uint64_t next;
  uint32_t cur[4];
} gen_stream;

static uint32_t gen_draw(gen_stream* g) {
  if ((g->next & 3) == 0) {
    const uint64_t blk = g->next >> 2;
    const uint32_t c[4] = {g->post, (uint32_t)blk, (uint32_t)(blk >> 32),
                           NETGEN_TAG | (g->purpose << 8)};
    const uint32_t k[2] = {(uint32_t)g->seed, (uint32_t)(g->seed >> 32)};
    orc_philox4x32_10(c, k, g->cur);
  }
  return g->cur[g->next++ & 3];
}

static int cmp_u32(const void* a, const void* b) {
  const uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return (x > y) - (x < y);
}

int orc_random_projection(int64_t npre, int64_t npost, int32_t in_degree, float w_mean,
                          float w_lo, float w_hi, int32_t d_min, int32_t d_max, uint64_t seed,
                          uint32_t* pre_idx, uint32_t* post_idx, float* weight, uint8_t* delay) {
  if (in_degree < 0 || in_degree > npre || d_min < 1 || d_max < d_min) return -1;
  const uint32_t dspan = (uint32_t)(d_max - d_min + 1);
  const float wspan = w_hi - w_lo;
  int rc = 0;
#pragma omp parallel
  {
    uint64_t* mark = (uint64_t*)calloc((size_t)(npre + 63) / 64 + 1, sizeof(uint64_t));
    uint32_t* pick = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(in_degree + 1));
    if (!mark || !pick) {
#pragma omp atomic write
      rc = -2;
    }
#pragma omp for schedule(dynamic, 16)
    for (int64_t p = 0; p < npost; ++p) {
      if (!mark || !pick) continue;
      gen_stream gi = {seed, (uint32_t)p, 0u, 0, {0}};
      gen_stream gw = {seed, (uint32_t)p, 1u, 0, {0}};
      gen_stream gd = {seed, (uint32_t)p, 2u, 0, {0}};
      int32_t n = 0;
      for (int64_t j = npre - in_degree; j < npre; ++j) {
        uint32_t t = (uint32_t)(((uint64_t)gen_draw(&gi) * (uint64_t)(j + 1)) >> 32);
        if ((mark[t >> 6] >> (t & 63)) & 1ull) t = (uint32_t)j;
        mark[t >> 6] |= 1ull << (t & 63);
        pick[n++] = t;
      }
      qsort(pick, (size_t)n, sizeof(uint32_t), cmp_u32);
      const int64_t o = p * in_degree;
      for (int32_t k = 0; k < in_degree; ++k) {
        const uint32_t t = pick[k];
        mark[t >> 6] &= ~(1ull << (t & 63));
        pre_idx[o + k] = t;
        post_idx[o + k] = (uint32_t)p;
        const float u = (float)(gen_draw(&gw) >> 8) * (1.0f / 16777216.0f);
        weight[o + k] = w_mean * (w_lo + wspan * u);
        delay[o + k] = (uint8_t)(d_min + (int32_t)(((uint64_t)gen_draw(&gd) * dspan) >> 32));
      }
    }
    free(mark);
    free(pick);
  }
  return rc;
}

/* Benchmark scaffold architecture (populations mossy, granule, Golgi,
 * stellate, basket, Purkinje, DCN; eleven projections), configurations 1, 2
 * and 5.  sizes[7]; proj[11][4] = {pre, post, in-degree, channel};
 * drive[11] = total drive (mean weight x in-degree, nS); *burst_n = number of
 * mossy fibres with the 100 Hz burst (0: none). */
int orc_scaffold_spec(int32_t config, double scale, int32_t* sizes, int32_t* proj, float* drive,
                      int32_t* burst_n) {
  static const int32_t base1[7] = {512, 8192, 128, 256, 128, 32, 8};
  static const int32_t base2[7] = {2400, 88000, 220, 600, 1200, 70, 60};
  static const int32_t base5[7] = {24000, 880000, 2200, 6000, 12000, 700, 600};
  static const int32_t deg1[11] = {4, 4, 200, 20, 100, 100, 2000, 10, 10, 8, 20};
  static const int32_t deg2[11] = {4, 4, 400, 20, 100, 100, 25000, 10, 10, 12, 50};
  /* pre, post, channel (0 exc, 1 inh), total drive */
  static const int32_t pp[11][3] = {{0, 1, 0}, {2, 1, 1}, {1, 2, 0}, {0, 2, 0},
                                    {1, 3, 0}, {1, 4, 0}, {1, 5, 0}, {3, 5, 1},
                                    {4, 5, 1}, {5, 6, 1}, {0, 6, 0}};
  static const float drv[11] = {11.0f, 3.0f, 30.0f, 12.0f, 45.0f, 45.0f,
                                450.0f, 3.0f, 3.0f, 2.0f, 60.0f};
  const int32_t* base;
  const int32_t* deg;
  int burst;
  switch (config) {
    case 1: base = base1; deg = deg1; burst = 0; break;
    case 2: base = base2; deg = deg2; burst = 1; break;
    case 5: base = base5; deg = deg2; burst = 1; break;
    default: return -1;
  }
  if (!(scale > 0.0)) return -1;
  for (int i = 0; i < 7; ++i) {
    const double f = floor((double)base[i] * scale + 0.5);
    sizes[i] = (int32_t)(f < 1.0 ? 1.0 : f);
  }
  for (int j = 0; j < 11; ++j) {
    const int32_t pre = pp[j][0];
    proj[4 * j + 0] = pre;
    proj[4 * j + 1] = pp[j][1];
    proj[4 * j + 2] = deg[j] < sizes[pre] ? deg[j] : sizes[pre];
    proj[4 * j + 3] = pp[j][2];
    drive[j] = drv[j];
  }
  *burst_n = burst ? (sizes[0] / 10 > 1 ? sizes[0] / 10 : 1) : 0;
  return 0;
}
