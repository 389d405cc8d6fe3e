// Pair-potential derivatives and gradient bins shared by the adjoint
// kernels (adjoint.cu, batched.cu).
//
// Reference: the derivatives jax.grad takes through energy.lennard_jones x
// multiplicative_isotropic_cutoff, energy.soft_sphere and energy.morse x
// multiplicative_isotropic_cutoff (energy.py:125-173, 246-272, 346-440,
// 534-580), with the LJ cutoff radii following max(sigma) (energy.py:319-320);
// the Morse radii are absolute.
#pragma once

#include <algorithm>
#include <cstring>

#include "pair.cuh"

namespace jmd {
namespace {

// Bins of the parameter gradient: [a*8+b] sigma, [64 + a*8+b] epsilon,
// [128] the cutoff scale (max sigma) when the cutoff is global.
constexpr int kBins = 130;

// Per-pair quantities of the potential and their parameter derivatives.
struct PairD {
  float g, hh;              // U'/r and U''
  float U;                  // energy
  float dg_s, dg_e, dg_k;   // d g / d sigma, d eps, d cutoff scale
  float dU_s, dU_e, dU_k;   // d U / ...
};

template <int KIND>
__device__ __forceinline__ PairD pair_derivs(float r2, const PairCoef& c, float sigma, float kappa) {
  PairD o;
  if (KIND == JMD_MORSE) {
    const MorseTerms m = morse_terms(r2, sigma, c.eps, c.alpha, c.ro2, c.rc2, c.inv_den);
    o.U = m.U;
    o.g = m.g;
    o.hh = m.hh;
    o.dU_e = m.dU_e;
    o.dg_e = m.dg_e;
    o.dU_s = m.dU_s;
    o.dg_s = m.dg_s;
    o.dU_k = 0.f;
    o.dg_k = 0.f;
    return o;
  }
  if (KIND == JMD_SOFT_SPHERE) {
    const float r = sqrtf(r2);
    const float is = c.inv_sig;
    const float b = 1.0f - r * is;
    const float al = c.alpha;
    const float pa2 = al == 2.0f ? 1.0f : __powf(b, al - 2.0f);
    const float pa1 = al == 2.0f ? b : __powf(b, al - 1.0f);
    const float U = c.eps / al * pa1 * b;
    const float dU = -c.eps * is * pa1;            // U'
    const float d2U = c.eps * (al - 1.0f) * is * is * pa2;
    o.U = U;
    o.g = dU / r;
    o.hh = d2U;
    o.dU_e = U / c.eps;
    o.dg_e = o.g / c.eps;
    o.dU_s = c.eps * pa1 * r * is * is;
    const float dUp_s = c.eps * is * is * pa1 - c.eps * is * (al - 1.0f) * pa2 * r * is * is;
    o.dg_s = dUp_s / r;
    o.dg_k = 0.f;
    o.dU_k = 0.f;
    return o;
  }
  const float ir2 = 1.0f / r2;
  const float s2 = c.sig2 * ir2;
  const float s6 = s2 * s2 * s2, s12 = s6 * s6;
  const float e4 = 4.0f * c.eps;
  const float U0 = e4 * (s12 - s6);
  const float U0p_r = e4 * (6.0f * s6 - 12.0f * s12) * ir2;    // U0' / r
  const float U0pp = e4 * (156.0f * s12 - 42.0f * s6) * ir2;   // U0''
  const float is = 1.0f / sigma;
  const float dU0_s = e4 * (12.0f * s12 - 6.0f * s6) * is;
  const float dU0p_r_s = e4 * (36.0f * s6 - 144.0f * s12) * ir2 * is;  // d(U0'/r)/d sigma
  float S = 1.f, Su = 0.f, Suu = 0.f, dS_k = 0.f, dSu_k = 0.f;
  if (KIND == JMD_LJ && r2 > c.ro2) {
    const float A = c.rc2 - r2;
    const float B = c.rc2 + 2.0f * r2 - 3.0f * c.ro2;
    const float idn = c.inv_den;
    const float w = c.rc2 - c.ro2;
    S = A * A * B * idn;
    Su = 6.0f * A * (c.ro2 - r2) * idn;
    Suu = 6.0f * (2.0f * r2 - c.rc2 - c.ro2) * idn;
    const float dS_rc = (2.0f * A * B + A * A) * idn - 3.0f * S / w;
    const float dS_ro = -3.0f * A * A * idn + 3.0f * S / w;
    const float dSu_rc = 6.0f * (c.ro2 - r2) * idn - 3.0f * Su / w;
    const float dSu_ro = 6.0f * A * idn + 3.0f * Su / w;
    const float ik = 2.0f / kappa;  // d(r^2_cut)/d kappa = 2 r^2_cut / kappa
    dS_k = (dS_ro * c.ro2 + dS_rc * c.rc2) * ik;
    dSu_k = (dSu_ro * c.ro2 + dSu_rc * c.rc2) * ik;
  }
  // U = U0 S ; U'/r = (U0'/r) S + 2 U0 Su ; U'' = U0'' S + 2 U0' S' + U0 S''
  o.U = U0 * S;
  o.g = U0p_r * S + 2.0f * U0 * Su;
  const float Sp_r = 2.0f * Su;                        // S'/r
  o.hh = U0pp * S + 2.0f * (U0p_r * r2) * Sp_r + U0 * (4.0f * r2 * Suu + 2.0f * Su);
  o.dU_e = o.U / c.eps;
  o.dg_e = o.g / c.eps;
  o.dU_s = dU0_s * S;
  o.dg_s = dU0p_r_s * S + 2.0f * dU0_s * Su;
  o.dU_k = U0 * dS_k;
  o.dg_k = U0p_r * dS_k + 2.0f * U0 * dSu_k;
  return o;
}

// Per-thread accumulators of one row of bins (the row is the species of the
// thread's atom; NB = 8 with species, 1 without).  Entries are picked with
// unrolled compares so the arrays stay in registers.
template <int NB>
struct BinAcc {
  float s[NB], e[NB], k;
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int b = 0; b < NB; ++b) s[b] = e[b] = 0.f;
    k = 0.f;
  }
  __device__ __forceinline__ void add(int col, float vs, float ve, float vk, bool per_pair) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      if (b == col) {
        s[b] += per_pair ? vs + vk : vs;
        e[b] += ve;
      }
    }
    if (!per_pair) k += vk;
  }
  // Sums over the `width` lanes of a lane group (all of them share a row).
  // Every lane of the warp must take part (ncol is uniform across the warp).
  __device__ __forceinline__ void group_sum(int width, int ncol) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      if (b < ncol) {
        for (int o = width / 2; o > 0; o >>= 1) {
          s[b] += __shfl_xor_sync(0xffffffffu, s[b], o, width);
          e[b] += __shfl_xor_sync(0xffffffffu, e[b], o, width);
        }
      }
    }
    for (int o = width / 2; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o, width);
  }
  __device__ __forceinline__ void flush(float* bins, int row, int ncol) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      if (b < ncol && s[b] != 0.f) atomicAdd(&bins[row * JMD_MAX_SPECIES + b], s[b]);
      if (b < ncol && e[b] != 0.f) atomicAdd(&bins[64 + row * JMD_MAX_SPECIES + b], e[b]);
    }
    if (k != 0.f) atomicAdd(&bins[128], k);
  }
};

__device__ __forceinline__ void zero_bins(float* bins) {
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) bins[b] = 0.f;
}

__device__ __forceinline__ void publish_bins(const float* bins, double* out, double scale) {
  for (int b = threadIdx.x; b < kBins; b += blockDim.x)
    if (out && bins[b] != 0.f) atomicAdd(out + b, scale * (double)bins[b]);
}

// Shared sigma lookups of the derivative formulas: sigma of each (a, b) in the
// pad slot of a second table, max sigma (the global cutoff scale) in its pad.
inline PairTable sigma_table(const jmd_pair& pp) {
  PairTable sg;
  memset(&sg, 0, sizeof(sg));
  const int S = pp.n_species > 0 ? pp.n_species : 1;
  float maxs = 0.f;
  for (int a = 0; a < S; ++a)
    for (int b = 0; b < S; ++b) {
      sg.c[a * JMD_MAX_SPECIES + b].pad = pp.sigma[a][b];
      maxs = std::max(maxs, pp.sigma[a][b]);
    }
  sg.pad = maxs;
  return sg;
}

}  // namespace
}  // namespace jmd
