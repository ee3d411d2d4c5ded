// Counter-based random numbers and bit-exact scalar helpers shared by the
// host library and the device kernels.
//
// Philox4x32-10 follows the construction published by Salmon, Moraes, Dror
// and Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11): ten rounds
// of two 32x32->64 multiplies on a 128-bit counter, with a 64-bit key bumped
// by the Weyl constants between rounds.  The reference draws its mossy-fibre
// and initial-potential randoms from stateful cuRAND Philox4_32_10 generators
// (UserInputFunctions.cu:104, init_params.cu:346, seeded from time(NULL) at
// GPUScaffoldSimulation.cu:135,316,358); here the generator is stateless and
// keyed on (instance seed, neuron id, step), so any step of any neuron can be
// regenerated independently and a run is reproducible.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define SGB_HD __host__ __device__ __forceinline__
#else
#define SGB_HD inline
#endif

namespace sgb {

// Round multipliers and key increments of Philox4x32 (SC'11, table 2).
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

// Stream tags: the fourth counter word separates independent uses of the
// same (seed, neuron, step) triple.
constexpr uint32_t kTagInput = 1u;    // mossy-fibre / input-cell draws
constexpr uint32_t kTagInitU = 2u;    // initial membrane potential
constexpr uint32_t kTagNetGen = 3u;   // synthetic connectivity generation

struct U4 { uint32_t x, y, z, w; };

SGB_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

SGB_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#if defined(__CUDACC__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = mulhi32(kPhiloxM0, c.x);
    const uint32_t lo0 = kPhiloxM0 * c.x;
    const uint32_t hi1 = mulhi32(kPhiloxM1, c.z);
    const uint32_t lo1 = kPhiloxM1 * c.z;
    U4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
  return c;
}

// Counter layout used by every draw in the library:
//   x = neuron id (instance-local, unpadded), y/z = step (low/high word),
//   w = tag | (block << 8), where block numbers successive groups of four
//   draws inside one step (substeps > 4).
SGB_HD U4 philox_draw(uint64_t seed, uint32_t neuron, uint64_t step,
                      uint32_t tag, uint32_t block) {
  U4 c;
  c.x = neuron;
  c.y = (uint32_t)step;
  c.z = (uint32_t)(step >> 32);
  c.w = tag | (block << 8);
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

SGB_HD uint32_t u4_get(const U4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// Uniform in (0, 1] with 24-bit resolution: exact in float, never zero.
SGB_HD float u01_open0(uint32_t x) {
  return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f);
}

// Round-to-nearest-even float -> bfloat16 bits (finite inputs), and back.
SGB_HD uint16_t f32_to_bf16_bits(float f) {
  union { float f; uint32_t u; } v;
  v.f = f;
  const uint32_t lsb = (v.u >> 16) & 1u;
  return (uint16_t)((v.u + 0x7FFFu + lsb) >> 16);
}
SGB_HD float bf16_bits_to_f32(uint16_t h) {
  union { float f; uint32_t u; } v;
  v.u = ((uint32_t)h) << 16;
  return v.f;
}

// Population sizes are bounded by the 28-bit index space; delays are 1..15
// exchange steps.
constexpr uint32_t kIndexBits = 28;
constexpr uint32_t kIndexMask = (1u << kIndexBits) - 1u;
constexpr int kMaxDelay = 15;

// Stored LIF state: the potential u (4 B) and the two conductances (8 B).
// A cell that is refractory after a step sits at V_reset (the update pins it
// there), so its potential field carries the refractory count instead, as a
// quiet-NaN payload: 0x7FC00000 | ref, ref in 1..2^22 - 1.  Arithmetic NaNs
// have an empty payload and read back as themselves with ref 0.
constexpr uint32_t kRefTag = 0x7FC00000u;
constexpr int32_t kRefMax = (1 << 22) - 1;
SGB_HD float pack_u(float u, int32_t ref) {
  union { float f; uint32_t b; } v;
  if (ref > 0) { v.b = kRefTag | (uint32_t)ref; return v.f; }
  return u;
}
// Unpacks the potential field: the refractory count (0 if none) and the
// potential (vr while refractory).
SGB_HD int32_t unpack_ref(float x) {
  union { float f; uint32_t b; } v;
  v.f = x;
  return v.b - (kRefTag + 1u) < (uint32_t)kRefMax ? (int32_t)(v.b - kRefTag) : 0;
}

// Dense-pull (ELL) entry: (delay - 1) * n_pad + g for the pre cell's global
// (padded) index g, with n_pad a multiple of 1,024.  The spike history keeps
// its rows in decreasing step order (and twice, so no wrap), so the history
// word of the pre cell at step t + 1 - d sits at base_t + (e >> 5), its bit
// is e & 31, and, with the summary rows of steps t, t - 1, ... laid out the
// same way at one bit per history word, its summary word is e >> 10 and the
// bit there (e >> 5) & 31.  Padding carries delay field H, one past the
// deepest delay: ell_pad = H * n_pad.
SGB_HD uint32_t ell_entry(uint32_t g, uint32_t delay, uint32_t n_pad) {
  return (delay - 1u) * n_pad + g;
}
SGB_HD uint32_t ell_pad(uint32_t hist_rows, uint32_t n_pad) { return hist_rows * n_pad; }

}  // namespace sgb
