// Pair-potential evaluation shared by the force, fused-step and adjoint
// kernels.
//
// Reference: jax_md/energy.py
//   lennard_jones                     :246-272  4 eps ((s/r)^12 - (s/r)^6)
//   multiplicative_isotropic_cutoff   :534-580  S(r) between r_onset, r_cutoff
//   soft_sphere                       :125-173  eps/alpha (1 - r/sigma)^alpha
//   morse                             :346-371  eps (1 - exp(-alpha (r - sigma)))^2 - eps
#pragma once

#include <functional>
#include <string>

#include "common.cuh"
#include "segment.cuh"

namespace jmd {

// Per species-pair coefficients (host-precomputed, 32 bytes).
struct PairCoef {
  float sig2;     // sigma^2
  float eps;      // epsilon
  float alpha;    // soft-sphere exponent
  float ro2;      // r_onset^2 (LJ smoothing)
  float rc2;      // interaction cutoff^2 (LJ r_cutoff, soft sphere sigma^2)
  float inv_den;  // 1 / (rc2 - ro2)^3
  float inv_sig;  // 1 / sigma
  float pad;      // sigma (the Morse minimum; unused by the other kinds)
};

struct PairTable {
  int kind;
  int nsp;         // 0: scalar (entry 0)
  float rc2_max;   // largest rc2 in the table
  float pad;
  PairCoef c[JMD_MAX_SPECIES * JMD_MAX_SPECIES];
  // per-particle parameters (generic kernels only): per-atom sigma / epsilon
  // combined as 0.5 (p_i + p_j); maxs = max sigma, the cutoff scale
  const float* psig;
  const float* peps;
  int per_pair_cutoff;
  float maxs, r_onset, r_cutoff;
};

PairTable make_pair_table(const jmd_pair& pp);
// allow_particle: the caller's kernels read per-particle parameters
int validate_pair(const jmd_pair* pp, bool allow_particle = false);

// Coefficients of pair (i, j) under per-particle parameters: the reference's
// 0.5 (p_i + p_j) in float32 (smap.py:704-713), then the table's derived
// values for that sigma / epsilon (make_pair_table).
__device__ __forceinline__ PairCoef particle_coef(const PairTable& t, int i, int j) {
  PairCoef c = t.c[0];
  if (t.peps) c.eps = 0.5f * (__ldg(t.peps + i) + __ldg(t.peps + j));
  if (t.psig) {
    const float sig = 0.5f * (__ldg(t.psig + i) + __ldg(t.psig + j));
    c.sig2 = sig * sig;
    c.inv_sig = 1.0f / sig;
    c.pad = sig;
    if (t.kind == JMD_SOFT_SPHERE) {
      c.rc2 = sig * sig;
      c.ro2 = c.rc2;
    } else if (t.per_pair_cutoff && t.maxs > 0.f) {
      const float ro = t.r_onset * sig / t.maxs, rc = t.r_cutoff * sig / t.maxs;
      c.ro2 = ro * ro;
      c.rc2 = rc * rc;
      const double den = (double)c.rc2 - (double)c.ro2;
      c.inv_den = den > 0 ? (float)(1.0 / (den * den * den)) : 0.f;
      if (t.kind == JMD_LJ_TRUNCATED) c.ro2 = c.rc2;
    }
  }
  return c;
}

// Packed float4 Dense path (fused.cu).
int dense_tpa();
bool dense2_applicable(const float* x, int64_t xs, const int32_t* idx, int64_t ld, const float* f,
                       int64_t fs);
int dense2_forces(const jmd_pair* pp, const jmd_space* space, const float* x, const int32_t* species,
                  int64_t n, const int32_t* idx, int64_t ld, int64_t width, const int32_t* cnt,
                  float* f, double* energy, float* e_atom, double* virial, double* partials,
                  unsigned int* counter, double* totals, cudaStream_t st);

// 1/x to ~0.5 ulp: hardware approximation plus one Newton step.
__device__ __forceinline__ float rcp_nr(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  float e = fmaf(-x, y, 1.0f);
  return fmaf(y, e, y);
}

// Morse pair under the multiplicative cutoff with absolute radii: U0 =
// eps ((1 - e)^2 - 1), e = exp(-alpha (r - sigma)); U = U0 S(r^2) with S of
// multiplicative_isotropic_cutoff for ro2 < r^2 (S = 1 below).  Gives U,
// g = U'(r)/r, hh = U''(r) and the derivatives of U and g with respect to
// sigma (U0 depends on r - sigma only, the radii not at all) and epsilon (U
// is linear in it).  Host and device code: the host copy is unit-tested
// against the FP64 oracle.
struct MorseTerms {
  float U, g, hh, dU_s, dg_s, dU_e, dg_e;
};

__host__ __device__ inline MorseTerms morse_terms(float r2, float sigma, float eps, float alpha,
                                                  float ro2, float rc2, float inv_den) {
  MorseTerms o;
  const float r = sqrtf(r2);
  const float ir = 1.0f / r;
  const float e = expf(-alpha * (r - sigma));
  const float om = 1.0f - e;
  const float U0 = eps * om * om - eps;
  const float U0p = 2.0f * eps * alpha * e * om;                          // U0'
  const float U0pp = 2.0f * eps * alpha * alpha * e * (2.0f * e - 1.0f);  // U0''
  float S = 1.f, Su = 0.f, Suu = 0.f;  // S and its derivatives in u = r^2
  if (r2 > ro2) {
    const float A = rc2 - r2;
    const float B = rc2 + 2.0f * r2 - 3.0f * ro2;
    S = A * A * B * inv_den;
    Su = 6.0f * A * (ro2 - r2) * inv_den;
    Suu = 6.0f * (2.0f * r2 - rc2 - ro2) * inv_den;
  }
  // U' = U0' S + U0 S' with S' = 2 r Su;  U'' = U0'' S + 2 U0' S' + U0 (4 r^2 Suu + 2 Su)
  o.U = U0 * S;
  o.g = U0p * ir * S + 2.0f * U0 * Su;
  o.hh = U0pp * S + 4.0f * r * U0p * Su + U0 * (4.0f * r2 * Suu + 2.0f * Su);
  o.dU_s = -U0p * S;
  o.dg_s = -U0pp * ir * S - 2.0f * U0p * Su;
  const float U0e = om * om - 1.0f, U0pe = 2.0f * alpha * e * om;  // d/d eps of U0, U0'
  o.dU_e = U0e * S;
  o.dg_e = U0pe * ir * S + 2.0f * U0e * Su;
  return o;
}

// Evaluates one pair at squared distance r2 (0 < r2 < c.rc2 is the caller's
// job).  Returns U and g = U'(r)/r; d2 = U''(r) (second derivative) when
// SECOND, for the adjoint.
template <int KIND, bool SECOND>
__device__ __forceinline__ void pair_eval(float r2, const PairCoef& c, float& U, float& g,
                                          float& h) {
  if (KIND == JMD_MORSE) {
    const MorseTerms m = morse_terms(r2, c.pad, c.eps, c.alpha, c.ro2, c.rc2, c.inv_den);
    U = m.U;
    g = m.g;
    if (SECOND) h = m.hh;
    return;
  }
  if (KIND == JMD_SOFT_SPHERE) {
    float r = sqrtf(r2);
    float x = r * c.inv_sig;
    float base = 1.0f - x;
    float inv_r = rcp_nr(r);
    if (c.alpha == 2.0f) {
      U = 0.5f * c.eps * base * base;
      float dU = -c.eps * c.inv_sig * base;  // U'(r)
      g = dU * inv_r;
      if (SECOND) h = c.eps * c.inv_sig * c.inv_sig;
    } else {
      float pa1 = __powf(base, c.alpha - 1.0f);
      U = c.eps / c.alpha * pa1 * base;
      float dU = -c.eps * c.inv_sig * pa1;
      g = dU * inv_r;
      if (SECOND) h = c.eps * (c.alpha - 1.0f) * c.inv_sig * c.inv_sig * __powf(base, c.alpha - 2.0f);
    }
    return;
  }
  float inv_r2 = rcp_nr(r2);
  float s2 = c.sig2 * inv_r2;
  float s6 = s2 * s2 * s2;
  float s12 = s6 * s6;
  float e4 = 4.0f * c.eps;
  float u = e4 * (s12 - s6);
  // U'(r)/r = 4 eps (6 s6 - 12 s12) / r^2
  float gr = e4 * (6.0f * s6 - 12.0f * s12) * inv_r2;
  float hh = 0.f;
  if (SECOND) hh = e4 * (156.0f * s12 - 42.0f * s6) * inv_r2;  // U''(r)
  if (KIND == JMD_LJ && r2 > c.ro2) {
    // S(u) = (rc2-u)^2 (rc2+2u-3ro2) / den ; dS/dr / r = 12 (rc2-u)(ro2-u)/den
    float a = c.rc2 - r2;
    float bq = c.rc2 + 2.0f * r2 - 3.0f * c.ro2;
    float S = a * a * bq * c.inv_den;
    float dSr = 12.0f * a * (c.ro2 - r2) * c.inv_den;
    if (SECOND) {
      // d2S/dr2 = 4 r^2 S_uu + 2 S_u,  S_u = 6(rc2-u)(ro2-u)/den,
      // S_uu = 6(2u - rc2 - ro2)/den
      float Su = 6.0f * a * (c.ro2 - r2) * c.inv_den;
      float Suu = 6.0f * (2.0f * r2 - c.rc2 - c.ro2) * c.inv_den;
      float d2S = 4.0f * r2 * Suu + 2.0f * Su;
      // U'(r) = gr * r ; (U S)'' = U'' S + 2 U' S' + U S''
      hh = hh * S + 2.0f * (gr * r2) * dSr + u * d2S;  // U' S' = (gr r)(dSr r)
    }
    g = gr * S + u * dSr;
    U = u * S;
  } else {
    g = gr;
    U = u;
  }
  h = hh;
}

// Displacement a - b for atoms inside a periodic box: the plain difference,
// re-done exactly only when a component wraps (see min_image).
template <int DIM>
__device__ __forceinline__ void displacement(const float4& a, const float4& b, const Geo& g,
                                             float& dx, float& dy, float& dz) {
  dx = a.x - b.x;
  dy = a.y - b.y;
  dz = DIM == 3 ? a.z - b.z : 0.f;
  if (g.periodic) {
    bool wrapped = fabsf(dx) > g.halfL[0] || fabsf(dy) > g.halfL[1];
    if (DIM == 3) wrapped = wrapped || fabsf(dz) > g.halfL[2];
    if (wrapped) {
      dx = min_image(a.x, b.x, g.L[0], g.halfL[0]);
      dy = min_image(a.y, b.y, g.L[1], g.halfL[1]);
      if (DIM == 3) dz = min_image(a.z, b.z, g.L[2], g.halfL[2]);
    }
    // general cell: the unit-cube image mapped into the cell (space.py:430-431)
    if (g.general) cell_apply<DIM>(g.T, dx, dy, dz);
  }
}

}  // namespace jmd

namespace jmd {
// Reverse Verlet step of the engine (adjoint.cu): pack (x, q) records, with
// q = pbar + (dt/m) xbar when `kick` (pbar <- q), and the skin test of x when
// `skin`; then xbar += weight * (dF/dR)^T q over the system's Dense list and,
// when grad_params is given, weight * d(q . F)/d theta into its 130 bins.
int adjoint_pack(const jmd_nve_system& s, const float* x, float* xbar, float* pbar, float* rec,
                 bool kick, bool skin, cudaStream_t st);
int adjoint_vjp_step(const jmd_nve_system& s, float* xbar, const float* rec, float weight,
                     double* grad_params, cudaStream_t st);
}  // namespace jmd

namespace jmd {
// CUDA graph helpers of the engine (engine.cu): append "IF (*flag) { body }"
// to the capture on st (body recorded on body_st); record enq(capture,
// body stream) once per key as a graph and launch it on st.
int graph_conditional(const int32_t* flag, const std::function<int(cudaStream_t)>& body,
                      cudaStream_t st, cudaStream_t body_st);
int graph_launch_cached(const std::string& key,
                        const std::function<int(cudaStream_t, cudaStream_t)>& enq,
                        cudaStream_t st);
}  // namespace jmd

namespace jmd {
// Tiled Dense build reusing the bins of a jmd_sort_by_cell just run on the
// same positions and workspace (nlist.cu).
int build_tiled_after_sort(const jmd_nlist* nl, const float* position, int64_t n, int32_t* tidx,
                           int64_t depth, int32_t* nbr_count, int64_t* occupancy,
                           uint8_t* error_code, float* reference_position, int32_t* rebuild_flag,
                           void* workspace, size_t workspace_bytes, cudaStream_t st);
}  // namespace jmd

namespace jmd {
// Segment-local engine list (segment.cuh, nlist.cu, segment.cu): cell starts
// of the last jmd_sort_by_cell in its workspace; the build right after that
// sort; and the force (mode 0), fused step (2) and force + kick (3) kernels.
const int32_t* sort_cell_starts(const jmd_nlist* nl, int64_t n, void* workspace,
                                size_t workspace_bytes);
int build_segment_after_sort(const jmd_nlist* nl, const SegGrid& sg, const float* position,
                             int64_t n, uint8_t* list, int32_t* nbr_count, int64_t* occupancy,
                             uint8_t* error_code, float* reference_position, int32_t* seg_status,
                             int32_t* rebuild_flag, void* workspace, size_t workspace_bytes,
                             cudaStream_t st);
int seg_step(int mode, const jmd_pair& pp, const jmd_space& space, const SegGrid& g,
             const float* x, const int32_t* start, const uint8_t* list, float* f, float* p,
             float* x_next, float m0, float dt, const float* ref, float thr2, int32_t* flag,
             int32_t* status, bool species, cudaStream_t st, int64_t n_atoms = 0);
}  // namespace jmd
