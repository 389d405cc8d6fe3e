// Packed-FP32x2 evaluation of two neighbour pairs per lane for the Dense
// pair kernels (sm_100+ FFMA2 / FADD2 / FMUL2: two FP32 results per issued
// instruction).  The pair arithmetic is the same as pair_eval in pair.cuh,
// element by element, with IEEE round-to-nearest in every operation.
#pragma once

#include "pair.cuh"

namespace jmd {

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b, exact as a scalar subtraction (b * -1 is exact)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2s(-1.f), a); }

__device__ __forceinline__ float2 rcp2(float2 x) {
  float2 y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y.x) : "f"(x.x));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y.y) : "f"(x.y));
  float2 e = fma2(make_float2(-x.x, -x.y), y, f2s(1.f));
  return fma2(y, e, y);
}

__device__ __forceinline__ float2 rsqrt2(float2 x) {
  float2 y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y.x) : "f"(x.x));
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y.y) : "f"(x.y));
  // one Newton step: y (1.5 - 0.5 x y^2)
  float2 hx = mul2(f2s(0.5f), x);
  float2 t = fma2(mul2(hx, y), make_float2(-y.x, -y.y), f2s(1.5f));
  return mul2(y, t);
}

// Coefficients of two pairs, packed.
struct Coef2 {
  float2 sig2, eps, alpha, ro2, rc2, inv_den, inv_sig, sig;
};

__device__ __forceinline__ Coef2 coef2(const PairCoef& a, const PairCoef& b) {
  Coef2 c;
  c.sig2 = f2(a.sig2, b.sig2);
  c.eps = f2(a.eps, b.eps);
  c.alpha = f2(a.alpha, b.alpha);
  c.ro2 = f2(a.ro2, b.ro2);
  c.rc2 = f2(a.rc2, b.rc2);
  c.inv_den = f2(a.inv_den, b.inv_den);
  c.inv_sig = f2(a.inv_sig, b.inv_sig);
  c.sig = f2(a.pad, b.pad);
  return c;
}

__device__ __forceinline__ Coef2 coef2(const PairCoef& a) { return coef2(a, a); }

// U and g = U'(r)/r for two pairs at squared distances r2 (> 0, callers mask
// pairs beyond the cutoff afterwards).
template <int KIND, bool NEED_U>
__device__ __forceinline__ void pair_eval2(float2 r2, const Coef2& c, float2& U, float2& g) {
  if (KIND == JMD_MORSE) {
    // two scalar evaluations: the exponential has no packed form
    const MorseTerms a = morse_terms(r2.x, c.sig.x, c.eps.x, c.alpha.x, c.ro2.x, c.rc2.x,
                                     c.inv_den.x);
    const MorseTerms b = morse_terms(r2.y, c.sig.y, c.eps.y, c.alpha.y, c.ro2.y, c.rc2.y,
                                     c.inv_den.y);
    g = f2(a.g, b.g);
    if (NEED_U) U = f2(a.U, b.U);
    return;
  }
  if (KIND == JMD_SOFT_SPHERE) {
    float2 rs = rsqrt2(r2);            // 1/r
    float2 r = mul2(r2, rs);           // r
    float2 x = mul2(r, c.inv_sig);
    float2 base = fma2(x, f2s(-1.f), f2s(1.f));
    if (c.alpha.x == 2.0f && c.alpha.y == 2.0f) {
      if (NEED_U) U = mul2(mul2(f2s(0.5f), c.eps), mul2(base, base));
      // U'(r) = -eps/sigma (1 - r/sigma)
      g = mul2(mul2(make_float2(-c.eps.x, -c.eps.y), c.inv_sig), mul2(base, rs));
    } else {
      float p0 = __powf(base.x, c.alpha.x - 1.0f), p1 = __powf(base.y, c.alpha.y - 1.0f);
      if (NEED_U) U = f2(c.eps.x / c.alpha.x * p0 * base.x, c.eps.y / c.alpha.y * p1 * base.y);
      g = f2(-c.eps.x * c.inv_sig.x * p0 * rs.x, -c.eps.y * c.inv_sig.y * p1 * rs.y);
    }
    return;
  }
  float2 ir2 = rcp2(r2);
  float2 s2 = mul2(c.sig2, ir2);
  float2 s6 = mul2(mul2(s2, s2), s2);
  float2 e4s6 = mul2(mul2(f2s(4.f), c.eps), s6);
  // U = 4 eps (s12 - s6) = e4s6 (s6 - 1); U'/r = e4s6 (6 - 12 s6) / r^2
  float2 u = mul2(e4s6, add2(s6, f2s(-1.f)));
  float2 gr = mul2(mul2(e4s6, fma2(s6, f2s(-12.f), f2s(6.f))), ir2);
  if (KIND == JMD_LJ) {
    float2 a = sub2(c.rc2, r2);
    float2 bq = fma2(f2s(2.f), r2, fma2(c.ro2, f2s(-3.f), c.rc2));
    float2 aid = mul2(a, c.inv_den);
    float2 S = mul2(mul2(a, aid), bq);
    float2 dSr = mul2(mul2(f2s(12.f), aid), sub2(c.ro2, r2));
    float2 gs = fma2(gr, S, mul2(u, dSr));
    float2 us = mul2(u, S);
    g.x = r2.x > c.ro2.x ? gs.x : gr.x;
    g.y = r2.y > c.ro2.y ? gs.y : gr.y;
    if (NEED_U) {
      U.x = r2.x > c.ro2.x ? us.x : u.x;
      U.y = r2.y > c.ro2.y ? us.y : u.y;
    }
  } else {
    g = gr;
    if (NEED_U) U = u;
  }
}

// L2 policy that asks to keep lines (evict_last): the positions are
// re-gathered ~n_neighbours times per step while the index rows stream
// through once (those use evict-first loads).  Created once per thread.
__device__ __forceinline__ uint64_t policy_keep() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// Read-only float4 gather under an L2 cache policy (positions do not change
// while a kernel runs; the step kernels write the next positions elsewhere).
__device__ __forceinline__ float4 ldg_keep(const float4* p, uint64_t pol) {
  float4 r;
  asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
      : "l"(p), "l"(pol));
  return r;
}

template <int DIM>
__device__ __forceinline__ bool interior(const float4& x, const Geo& g, float m) {
  if (!g.periodic) return true;
  bool in = x.x >= m && x.x <= g.L[0] - m && x.y >= m && x.y <= g.L[1] - m;
  if (DIM == 3) in = in && x.z >= m && x.z <= g.L[2] - m;
  return in;
}

}  // namespace jmd
