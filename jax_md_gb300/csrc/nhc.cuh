// Nose-Hoover chain of simulate.nvt_nose_hoover as device functions: the
// substep (simulate.py:444-490), the half step with update_mass
// (simulate.py:492-517) and its reverse by forward-mode dual numbers.  Used by
// the single-system chain kernels (integrate.cu) and the batched ones, one
// chain per system (batched.cu).
#pragma once

#include "common.cuh"

namespace jmd {
namespace {
struct NhcArgs {
  int M1;  // chain length
  int chain_steps;
  int sy_steps;
  double dof;
  double dt;
  double tau;
  double w[7];
  int update_mass;
};

// Chain layout: xi[16] p[16] Q[16] spare[16] KE kT (f64 in memory).  The
// substeps run in float32, the arithmetic of the reference's default float32
// state (simulate.py:444-507): a single thread walks a long serial chain of
// exp / divide steps, and float32 keeps it on the fast pipes.
template <typename T>
__device__ void nhc_substep(T delta, T* xi, T* p, const T* Q, T& KE, T& scale_total, int M1, T dof,
                            T kT) {
  const int M = M1 - 1;
  const T d2 = delta / T(2), d4 = d2 / T(2), d8 = d4 / T(2);
  T G = p[M - 1] * p[M - 1] / Q[M - 1] - kT;
  p[M] += d4 * G;
  T pnew = p[M];
  for (int m = M - 1; m > 0; --m) {
    G = p[m - 1] * p[m - 1] / Q[m - 1] - kT;
    T s = exp(-d8 * pnew / Q[m + 1]);
    pnew = s * (s * p[m] + d4 * G);
    p[m] = pnew;
  }
  G = T(2) * KE - dof * kT;
  T s = exp(-d8 * p[1] / Q[1]);
  p[0] = s * (s * p[0] + d4 * G);
  s = exp(-d2 * p[0] / Q[0]);
  KE = KE * s * s;
  scale_total *= s;
  for (int m = 0; m <= M; ++m) xi[m] += d2 * p[m] / Q[m];
  G = T(2) * KE - dof * kT;
  for (int m = 0; m < M; ++m) {
    T sc = exp(-d8 * p[m + 1] / Q[m + 1]);
    p[m] = sc * (sc * p[m] + d4 * G);
    G = p[m] * p[m] / Q[m] - kT;
  }
  p[M] += d4 * G;
}

// update_mass (when a.update_mass) and one half step of the chain at `chain`
// (66 doubles: xi[16] p[16] Q[16] spare[16] KE kT) with kinetic energy KE and
// dof degrees of freedom.  The chain is worked on in thread-local copies (the
// substeps are a long serial dependency chain) and written back once, with the
// rescaled kinetic energy in chain[64]; returns the total momentum scale.
__device__ inline float nhc_half_chain(const NhcArgs& a, double* chain, float KE, float dof) {
  float xi[16], p[16], Q[16];
  const int M1 = a.M1;
  for (int m = 0; m < M1; ++m) {
    xi[m] = (float)chain[m];
    p[m] = (float)chain[16 + m];
    Q[m] = (float)chain[32 + m];
  }
  const float kT = (float)chain[65];
  if (a.update_mass) {
    const float tau = (float)a.tau;
    for (int m = 0; m < M1; ++m) Q[m] = kT * tau * tau;
    Q[0] *= dof;
  }
  float scale = 1.f;
  if (a.chain_steps == 1 && a.sy_steps == 1) {
    nhc_substep<float>((float)a.dt, xi, p, Q, KE, scale, M1, dof, kT);
  } else {
    const float delta = (float)a.dt / (float)a.chain_steps;
    for (int k = 0; k < a.chain_steps * a.sy_steps; ++k)
      nhc_substep<float>(delta * (float)a.w[k % a.sy_steps], xi, p, Q, KE, scale, M1, dof, kT);
  }
  for (int m = 0; m < M1; ++m) {
    chain[m] = xi[m];
    chain[16 + m] = p[m];
    chain[32 + m] = Q[m];
  }
  chain[64] = KE;
  return scale;
}

// Forward-mode dual number with 8 tangents: the chain half step run on it
// gives the Jacobian of (p_xi', scale) with respect to (p_xi, KE) in one
// pass (chains of up to 7 thermostats).
struct Dual8 {
  float v;
  float d[8];
  __device__ Dual8() : v(0.f) {
#pragma unroll
    for (int i = 0; i < 8; ++i) d[i] = 0.f;
  }
  __device__ Dual8(float x) : v(x) {
#pragma unroll
    for (int i = 0; i < 8; ++i) d[i] = 0.f;
  }
  __device__ Dual8& operator+=(const Dual8& b) {
    v += b.v;
#pragma unroll
    for (int i = 0; i < 8; ++i) d[i] += b.d[i];
    return *this;
  }
  __device__ Dual8& operator*=(const Dual8& b) {
#pragma unroll
    for (int i = 0; i < 8; ++i) d[i] = d[i] * b.v + v * b.d[i];
    v *= b.v;
    return *this;
  }
};
__device__ inline Dual8 operator+(Dual8 a, const Dual8& b) { return a += b; }
__device__ inline Dual8 operator-(const Dual8& a) {
  Dual8 r(-a.v);
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = -a.d[i];
  return r;
}
__device__ inline Dual8 operator-(const Dual8& a, const Dual8& b) { return a + (-b); }
__device__ inline Dual8 operator*(Dual8 a, const Dual8& b) { return a *= b; }
__device__ inline Dual8 operator/(const Dual8& a, const Dual8& b) {
  Dual8 r(a.v / b.v);
  const float ib = 1.f / b.v;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
__device__ inline Dual8 exp(const Dual8& a) {
  Dual8 r(expf(a.v));
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = r.v * a.d[i];
  return r;
}

// Reverse of nhc_half_chain: given the chain state before it (unchanged), the
// kinetic energy it used and the cotangents of its outputs (p_xi' [M1],
// scale), writes the cotangents of p_xi [M1] and of the kinetic energy.
// Chains of up to 7 thermostats (8 tangents: M1 chain momenta and KE).
__device__ inline void nhc_half_chain_vjp(const NhcArgs& a, const double* chain, float ke,
                                          float dof, const double* cot_pxi, double cot_scale,
                                          double* out_pxi, double* out_ke) {
  const int M1 = a.M1;
  Dual8 xi[8], p[8], Q[8];
  const float kT = (float)chain[65];
  for (int m = 0; m < M1; ++m) {
    xi[m] = Dual8((float)chain[m]);
    p[m] = Dual8((float)chain[16 + m]);
    p[m].d[m] = 1.f;
    Q[m] = Dual8(a.update_mass ? kT * (float)a.tau * (float)a.tau : (float)chain[32 + m]);
  }
  if (a.update_mass) Q[0] = Q[0] * Dual8(dof);
  Dual8 KE(ke);
  KE.d[M1] = 1.f;
  Dual8 scale(1.f);
  if (a.chain_steps == 1 && a.sy_steps == 1) {
    nhc_substep<Dual8>(Dual8((float)a.dt), xi, p, Q, KE, scale, M1, Dual8(dof), Dual8(kT));
  } else {
    const float delta = (float)a.dt / (float)a.chain_steps;
    for (int k = 0; k < a.chain_steps * a.sy_steps; ++k)
      nhc_substep<Dual8>(Dual8(delta * (float)a.w[k % a.sy_steps]), xi, p, Q, KE, scale, M1,
                         Dual8(dof), Dual8(kT));
  }
  for (int j = 0; j <= M1; ++j) {
    double g = cot_scale * (double)scale.d[j];
    for (int m = 0; m < M1; ++m) g += cot_pxi[m] * (double)p[m].d[j];
    if (j < M1) out_pxi[j] = g;
    else *out_ke = g;
  }
}

// Arguments of the chain kernels; Suzuki-Yoshida weights (Yoshida 1990): the
// values simulate.py:328-347 uses.
inline NhcArgs nhc_args(const jmd_nhc& c, int32_t update_mass) {
  static const double w3[3] = {0.828981543588751, -0.657963087177502, 0.828981543588751};
  static const double w5[5] = {0.2967324292201065, 0.2967324292201065, -0.186929716880426,
                               0.2967324292201065, 0.2967324292201065};
  static const double w7[7] = {0.784513610477560, 0.235573213359357, -1.17767998417887,
                               1.31518632068391, -1.17767998417887, 0.235573213359357,
                               0.784513610477560};
  NhcArgs a;
  a.M1 = c.chain_length;
  a.chain_steps = c.chain_steps;
  a.sy_steps = c.sy_steps;
  a.dof = (double)c.dof;
  a.dt = c.dt;
  a.tau = c.tau;
  a.update_mass = update_mass;
  for (int k = 0; k < 7; ++k) a.w[k] = 0.0;
  const double* src = c.sy_steps == 3 ? w3 : c.sy_steps == 5 ? w5 : c.sy_steps == 7 ? w7 : nullptr;
  if (src) for (int k = 0; k < c.sy_steps; ++k) a.w[k] = src[k];
  else a.w[0] = 1.0;
  return a;
}

}  // namespace
}  // namespace jmd
