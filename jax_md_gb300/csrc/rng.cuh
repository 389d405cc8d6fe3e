// Counter-based normal draws for the Langevin O step: Philox4x32-10
// (J. K. Salmon, M. A. Moraes, R. O. Dror and D. E. Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11) maps (counter, key) to four 32-bit
// words with no state, so every atom and step gets its own draw from
// (seed, step, atom) and a run can be replayed exactly.  Box-Muller turns the
// four words into four standard normals.  Host and device code: the host copy
// is unit-tested against an independent NumPy restatement.
#pragma once

#include <cmath>
#include <cstdint>

namespace jmd {

struct Words4 {
  uint32_t w[4];
};

__host__ __device__ inline Words4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;  // round multipliers
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;  // key schedule (Weyl) increments
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * c0, p1 = (uint64_t)M1 * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  Words4 o;
  o.w[0] = c0;
  o.w[1] = c1;
  o.w[2] = c2;
  o.w[3] = c3;
  return o;
}

// A word as a uniform in (0, 1): the top 23 bits k give (2k + 1) / 2^24, the
// centre of the k-th interval of width 2^-23.  2k + 1 < 2^24 fits a float32
// significand, so the value is exact (no rounding, never 0 or 1, and the
// logarithm is finite); the oracle forms the same number.
__host__ __device__ inline float word_to_unit(uint32_t w) {
  return (float)(w >> 9) * (1.0f / 8388608.0f) + (1.0f / 16777216.0f);
}

// Box-Muller on word pairs (0, 1) and (2, 3): sqrt(-2 ln u0) (cos, sin)(2 pi u1).
__host__ __device__ inline void normals_from_words(const Words4& r, float z[4]) {
  const float two_pi = 6.283185307179586f;
  for (int h = 0; h < 2; ++h) {
    const float u0 = word_to_unit(r.w[2 * h]), u1 = word_to_unit(r.w[2 * h + 1]);
    const float rad = sqrtf(-2.0f * logf(u0));
    z[2 * h] = rad * cosf(two_pi * u1);
    z[2 * h + 1] = rad * sinf(two_pi * u1);
  }
}

// Four standard normals of atom `atom` at step `step` under `seed`: Philox on
// counter (atom, 0, step lo, step hi) and key (seed lo, seed hi), then
// Box-Muller on the four words.
__host__ __device__ inline void langevin_normals(uint64_t seed, uint64_t step, uint32_t atom,
                                                 float z[4]) {
  const Words4 r = philox4x32_10(atom, 0u, (uint32_t)step, (uint32_t)(step >> 32), (uint32_t)seed,
                                 (uint32_t)(seed >> 32));
  normals_from_words(r, z);
}

}  // namespace jmd
