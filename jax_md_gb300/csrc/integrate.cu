// Integrator kernels: velocity Verlet pieces, kinetic energy, Nose-Hoover chain.
//
// Reference: jax_md/simulate.py
//   momentum_step / position_step  :168-188
//   velocity_verlet                :227-243
//   nose_hoover_chain              :384-517  (substep :444-490, half step :492-507)
// and jax_md/quantity.py:124-159 (kinetic_energy, f64 sum).
#include <mutex>

#include "common.cuh"
#include "nhc.cuh"
#include "rng.cuh"

namespace jmd {
namespace {

template <int DIM, bool V4P, bool V4F>
__global__ void k_momentum(float* p, int64_t ps, const float* f, int64_t fs, int n, float dt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 a = load_row_rw<DIM, V4P>(p, ps, i);
  float4 b = load_row<DIM, V4F>(f, fs, i);
  a.x = fmaf(dt, b.x, a.x);
  a.y = fmaf(dt, b.y, a.y);
  a.z = fmaf(dt, b.z, a.z);
  store_row<DIM, V4P>(p, ps, i, a);
}

template <int DIM, bool V4X, bool V4P>
__global__ void k_position(float* x, int64_t xs, const float* p, int64_t ps, const float* mass,
                           float m0, int n, Geo g, float dt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 r = load_row_rw<DIM, V4X>(x, xs, i);
  float4 q = load_row<DIM, V4P>(p, ps, i);
  float m = mass ? mass[i] : m0;
  // shift_fn(R, dt * p / m)  (simulate.py:184)
  float dx = dt * q.x / m, dy = dt * q.y / m, dz = dt * q.z / m;
  if (g.general) cell_apply<DIM>(g.Ti, dx, dy, dz);  // dR lives in the cell (space.py:456)
  if (g.periodic) {
    r.x = wrap(r.x + dx, g.L[0]);
    r.y = wrap(r.y + dy, g.L[1]);
    if (DIM == 3) r.z = wrap(r.z + dz, g.L[2]);
  } else {
    r.x += dx;
    r.y += dy;
    r.z += dz;
  }
  store_row<DIM, V4X>(x, xs, i, r);
}

struct KickDriftArgs {
  float* x;
  int64_t xs;
  float* p;
  int64_t ps;
  const float* f;
  int64_t fs;
  const float* mass;
  float m0;
  int n;
  Geo g;
  float dt;
  const double* p_scale;
  const float* ref;
  int64_t rs;
  float thr2;
  int32_t* flag;
};

template <int DIM, bool V4>
__global__ void k_kick_drift(KickDriftArgs a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (i < a.n) {
    float4 q = load_row_rw<DIM, V4>(a.p, a.ps, i);
    float4 f = load_row<DIM, V4>(a.f, a.fs, i);
    float4 r = load_row_rw<DIM, V4>(a.x, a.xs, i);
    const float h = 0.5f * a.dt;
    if (a.p_scale) {
      float s = (float)(*a.p_scale);
      q.x *= s;
      q.y *= s;
      q.z *= s;
    }
    q.x = fmaf(h, f.x, q.x);
    q.y = fmaf(h, f.y, q.y);
    q.z = fmaf(h, f.z, q.z);
    float m = a.mass ? a.mass[i] : a.m0;
    float dx = a.dt * q.x / m, dy = a.dt * q.y / m, dz = a.dt * q.z / m;
    if (a.g.general) cell_apply<DIM>(a.g.Ti, dx, dy, dz);
    if (a.g.periodic) {
      r.x = wrap(r.x + dx, a.g.L[0]);
      r.y = wrap(r.y + dy, a.g.L[1]);
      if (DIM == 3) r.z = wrap(r.z + dz, a.g.L[2]);
    } else {
      r.x += dx;
      r.y += dy;
      r.z += dz;
    }
    store_row<DIM, V4>(a.p, a.ps, i, q);
    store_row<DIM, V4>(a.x, a.xs, i, r);
    if (a.ref) {
      float4 c = load_row<DIM, false>(a.ref, a.rs, i);
      float ex = a.g.periodic ? min_image(r.x, c.x, a.g.L[0], a.g.halfL[0]) : r.x - c.x;
      float ey = a.g.periodic ? min_image(r.y, c.y, a.g.L[1], a.g.halfL[1]) : r.y - c.y;
      float ez = 0.f;
      if (DIM == 3) ez = a.g.periodic ? min_image(r.z, c.z, a.g.L[2], a.g.halfL[2]) : r.z - c.z;
      if (a.g.general) cell_apply<DIM>(a.g.T, ex, ey, ez);
      over = ex * ex + ey * ey + ez * ez > a.thr2;
    }
  }
  if (a.flag && __any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(a.flag, 1);
}

// Grid-stride: each thread sums its atoms' p^2 / 2m in fp32 (a few terms;
// the FP64 pipe is narrow on this part), the threads' partial sums are then
// reduced in f64 in a fixed order.
template <int DIM>
__global__ void k_ke(const float* p, int64_t ps, const float* mass, float m0, int n,
                     double* partials, unsigned int* counter, double* out) {
  float acc = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 q = load_row<DIM, false>(p, ps, i);
    float m = mass ? mass[i] : m0;
    float s = q.x * q.x + q.y * q.y + (DIM == 3 ? q.z * q.z : 0.f);
    acc += 0.5f * s / m;
  }
  double v[1] = {(double)acc};
  grid_reduce<1>(v, partials, counter, out, false);
}

// Blocks of a grid-stride reduction over n atoms: 256 threads, 8 atoms per
// thread at most, so 2048 atoms per block.
constexpr int64_t kKeAtomsPerBlock = 256 * 8;
inline unsigned ke_blocks(int64_t n) {
  return (unsigned)std::max<int64_t>(1, ceil_div(n, kKeAtomsPerBlock));
}

template <int DIM>
__global__ void k_scale(float* p, int64_t ps, int n, const double* scale) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = (float)(*scale);
  float* r = p + i * ps;
  r[0] *= s;
  r[1] *= s;
  if (DIM == 3) r[2] *= s;
}

// Langevin O step (simulate.py:1102-1110): p <- c1 p + c2 sqrt(m) xi, xi
// drawn from (seed, step, atom) (rng.cuh); the draws are optionally written
// out (float4 rows) so a run can be replayed.
template <int DIM>
__global__ void k_langevin_o(float* p, int64_t ps, int n, const float* mass, float m0, float c1,
                             float c2, uint64_t seed, uint64_t step, float4* noise) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float z[4];
  langevin_normals(seed, step, (uint32_t)i, z);
  const float s = c2 * sqrtf(mass ? mass[i] : m0);
  float* r = p + i * ps;
  r[0] = fmaf(c1, r[0], s * z[0]);
  r[1] = fmaf(c1, r[1], s * z[1]);
  if (DIM == 3) r[2] = fmaf(c1, r[2], s * z[2]);
  if (noise) noise[i] = make_float4(z[0], z[1], z[2], z[3]);
}

// ------------------------------------------------------- Nose-Hoover -------
// One chain, one thread (the chain code is in nhc.cuh).
__global__ void k_nhc_half_vjp(NhcArgs a, const double* chain, const double* ke,
                               const double* cot_pxi, const double* cot_scale, double* out_pxi,
                               double* out_ke) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  nhc_half_chain_vjp(a, chain, (float)*ke, (float)a.dof, cot_pxi, *cot_scale, out_pxi, out_ke);
}

__global__ void k_nhc_half(NhcArgs a, double* chain, const double* ke_in, double* p_scale) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const float KE = (float)(ke_in ? *ke_in : chain[64]);
  *p_scale = nhc_half_chain(a, chain, KE, (float)a.dof);
}

// ------------------------------------------------------------- FIRE ------
// FIRE state on the device (float32 like the reference's scalars):
//   [0] dt  [1] alpha  [2] n_pos (as float)  [3] keep (F.P >= 0)
//   [4] alpha used for this step's mixing  [5] |P| / |F|
struct FireParams {
  float dt_max, n_min, f_inc, f_dec, alpha_start, f_alpha;
};

// simulate.npt_nose_hoover's exp(iL1) (mode 0: positions) and exp(iL2)
// (mode 1: momenta) with caller-computed coefficients (jmd_npt_map).
template <int DIM>
__global__ void k_npt_map(int mode, float4* x, float4* p, const float4* f, const float* mass,
                          float m0, int n, Geo g, float c0, float c1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 q = p[i];
  if (mode == 1) {
    const float4 ff = f[i];
    q.x = fmaf(c1, ff.x, c0 * q.x);
    q.y = fmaf(c1, ff.y, c0 * q.y);
    if (DIM == 3) q.z = fmaf(c1, ff.z, c0 * q.z);
    p[i] = q;
    return;
  }
  float4 r = x[i];
  const float m = mass ? mass[i] : m0;
  float dx = fmaf(c1, q.x / m, c0 * r.x), dy = fmaf(c1, q.y / m, c0 * r.y);
  float dz = DIM == 3 ? fmaf(c1, q.z / m, c0 * r.z) : 0.f;
  if (g.general) cell_apply<DIM>(g.Ti, dx, dy, dz);
  if (g.periodic) {
    r.x = wrap(r.x + dx, g.L[0]);
    r.y = wrap(r.y + dy, g.L[1]);
    if (DIM == 3) r.z = wrap(r.z + dz, g.L[2]);
  } else {
    r.x += dx;
    r.y += dy;
    if (DIM == 3) r.z += dz;
  }
  x[i] = r;
}

template <int DIM>
__global__ void k_fire_kick_drift(float4* x, float4* p, const float4* f, const float* mass,
                                  float m0, int n, Geo g, const float* fs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float dt = fs[0];
  const float h = dt * 0.5f;
  float4 q = p[i];
  const float4 ff = f[i];
  float4 r = x[i];
  q.x = fmaf(h, ff.x, q.x);
  q.y = fmaf(h, ff.y, q.y);
  q.z = fmaf(h, ff.z, q.z);
  const float m = mass ? mass[i] : m0;
  float dx = dt * q.x / m, dy = dt * q.y / m, dz = dt * q.z / m;
  if (g.general) cell_apply<DIM>(g.Ti, dx, dy, dz);
  if (g.periodic) {
    r.x = wrap(r.x + dx, g.L[0]);
    r.y = wrap(r.y + dy, g.L[1]);
    if (DIM == 3) r.z = wrap(r.z + dz, g.L[2]);
  } else {
    r.x += dx;
    r.y += dy;
    if (DIM == 3) r.z += dz;
  }
  p[i] = q;
  x[i] = r;
}

// Closing half kick, then the three FIRE reductions (|F|^2, |P|^2, F.P) in
// f64; k_fire_scalar then runs the scalar update of minimize.py:190-224.
template <int DIM>
__global__ void k_fire_finish(float4* p, const float4* f, int n, const float* fs,
                              double* partials, unsigned int* counter, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v[3] = {0.0, 0.0, 0.0};
  if (i < n) {
    const float h = fs[0] * 0.5f;
    float4 q = p[i];
    const float4 ff = f[i];
    q.x = fmaf(h, ff.x, q.x);
    q.y = fmaf(h, ff.y, q.y);
    q.z = fmaf(h, ff.z, q.z);
    p[i] = q;
    v[0] = (double)ff.x * ff.x + (double)ff.y * ff.y + (DIM == 3 ? (double)ff.z * ff.z : 0.0);
    v[1] = (double)q.x * q.x + (double)q.y * q.y + (DIM == 3 ? (double)q.z * q.z : 0.0);
    v[2] = (double)ff.x * q.x + (double)ff.y * q.y + (DIM == 3 ? (double)ff.z * q.z : 0.0);
  }
  grid_reduce<3>(v, partials, counter, out, false);
}

__global__ void k_fire_scalar(float* fs, FireParams fp, const double* red) {
  if (threadIdx.x != 0) return;
  const float F_norm = (float)sqrt(red[0] + 1e-6);
  const float P_norm = (float)sqrt(red[1]);
  const float F_dot_P = (float)red[2];
  float dt = fs[0], alpha = fs[1], n_pos = fs[2];
  fs[4] = alpha;                          // mixing uses the current alpha
  fs[5] = P_norm / F_norm;
  n_pos = F_dot_P >= 0.f ? n_pos + 1.f : 0.f;
  if (F_dot_P > 0.f && n_pos > fp.n_min) {
    dt = fminf(dt * fp.f_inc, fp.dt_max);
    alpha = alpha * fp.f_alpha;
  }
  if (F_dot_P < 0.f) {
    dt = dt * fp.f_dec;
    alpha = fp.alpha_start;
  }
  fs[0] = dt;
  fs[1] = alpha;
  fs[2] = n_pos;
  fs[3] = F_dot_P >= 0.f ? 1.f : 0.f;
}

__global__ void k_fire_mix(float4* p, const float4* f, int n, const float* fs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float alpha = fs[4], ratio = fs[5], keep = fs[3];
  float4 q = p[i];
  const float4 ff = f[i];
  q.x = keep * (q.x + alpha * (ff.x * ratio - q.x));
  q.y = keep * (q.y + alpha * (ff.y * ratio - q.y));
  q.z = keep * (q.z + alpha * (ff.z * ratio - q.z));
  p[i] = q;
}

struct ReduceWs {
  double* partials;
  unsigned int* counter;
};

constexpr int64_t kMaxReduceBlocks = 1 << 18;

}  // namespace
}  // namespace jmd

using namespace jmd;

extern "C" {

int jmd_momentum_step(float* momentum, int64_t p_stride, const float* force, int64_t f_stride,
                      int64_t n, int32_t dim, float dt, void* stream) {
  JMD_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
  if (n <= 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  unsigned gr = (unsigned)ceil_div(n, 256);
  const bool v4 = is_vec4(momentum, p_stride) && is_vec4(force, f_stride);
  if (dim == 3) {
    if (v4) k_momentum<3, true, true><<<gr, 256, 0, st>>>(momentum, p_stride, force, f_stride, (int)n, dt);
    else k_momentum<3, false, false><<<gr, 256, 0, st>>>(momentum, p_stride, force, f_stride, (int)n, dt);
  } else {
    k_momentum<2, false, false><<<gr, 256, 0, st>>>(momentum, p_stride, force, f_stride, (int)n, dt);
  }
  return check_launch("jmd_momentum_step");
}

int jmd_position_step(float* position, int64_t x_stride, const float* momentum, int64_t p_stride,
                      const float* mass, float mass_scalar, int64_t n, const jmd_space* space,
                      float dt, void* stream) {
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  if (n <= 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  unsigned gr = (unsigned)ceil_div(n, 256);
  Geo g = make_geo(*space);
  const bool v4 = is_vec4(position, x_stride) && is_vec4(momentum, p_stride);
  if (space->dim == 3) {
    if (v4) k_position<3, true, true><<<gr, 256, 0, st>>>(position, x_stride, momentum, p_stride, mass, mass_scalar, (int)n, g, dt);
    else k_position<3, false, false><<<gr, 256, 0, st>>>(position, x_stride, momentum, p_stride, mass, mass_scalar, (int)n, g, dt);
  } else {
    k_position<2, false, false><<<gr, 256, 0, st>>>(position, x_stride, momentum, p_stride, mass, mass_scalar, (int)n, g, dt);
  }
  return check_launch("jmd_position_step");
}

int jmd_verlet_kick_drift(float* position, int64_t x_stride, float* momentum, int64_t p_stride,
                          const float* force, int64_t f_stride, const float* mass,
                          float mass_scalar, int64_t n, const jmd_space* space, float dt,
                          const double* p_scale, const float* reference_position,
                          int64_t ref_stride, float threshold_sq, int32_t* rebuild_flag,
                          void* stream) {
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(reference_position == nullptr || rebuild_flag != nullptr,
              "skin test needs a rebuild flag");
  if (n <= 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  KickDriftArgs a{position, x_stride, momentum, p_stride, force, f_stride, mass, mass_scalar,
                  (int)n, make_geo(*space), dt, p_scale, reference_position, ref_stride,
                  threshold_sq, rebuild_flag};
  unsigned gr = (unsigned)ceil_div(n, 256);
  const bool v4 = is_vec4(position, x_stride) && is_vec4(momentum, p_stride) &&
                  is_vec4(force, f_stride);
  if (space->dim == 3) {
    if (v4) k_kick_drift<3, true><<<gr, 256, 0, st>>>(a);
    else k_kick_drift<3, false><<<gr, 256, 0, st>>>(a);
  } else {
    k_kick_drift<2, false><<<gr, 256, 0, st>>>(a);
  }
  return check_launch("jmd_verlet_kick_drift");
}

size_t jmd_reduce_workspace_bytes(int64_t n) {
  (void)n;
  Carver cv(nullptr, 0);
  cv.take<double>(kMaxReduceBlocks);
  cv.take<unsigned int>(1);
  return cv.used + 256;
}

int jmd_kinetic_energy(const float* momentum, int64_t p_stride, const float* mass,
                       float mass_scalar, int64_t n, int32_t dim, double* out, void* workspace,
                       size_t workspace_bytes, void* stream) {
  JMD_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
  JMD_REQUIRE(out != nullptr, "out is null");
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  ReduceWs w;
  w.partials = cv.take<double>(kMaxReduceBlocks);
  w.counter = cv.take<unsigned int>(1);
  if (!cv.ok()) return fail(JMD_ERR_WORKSPACE, "reduce workspace too small");
  if (n <= 0) {
    JMD_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st));
    return JMD_OK;
  }
  const int64_t gr = ke_blocks(n);
  if (gr > kMaxReduceBlocks) return fail(JMD_ERR_UNSUPPORTED, "system too large");
  JMD_CUDA(cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), st));
  if (dim == 3) k_ke<3><<<(unsigned)gr, 256, 0, st>>>(momentum, p_stride, mass, mass_scalar, (int)n, w.partials, w.counter, out);
  else k_ke<2><<<(unsigned)gr, 256, 0, st>>>(momentum, p_stride, mass, mass_scalar, (int)n, w.partials, w.counter, out);
  return check_launch("jmd_kinetic_energy");
}

int jmd_nhc_half_step(const jmd_nhc* c, double* chain, const double* kinetic_energy,
                      int32_t update_mass, double* p_scale, void* stream) {
  JMD_REQUIRE(c != nullptr && chain != nullptr && p_scale != nullptr, "null argument");
  JMD_REQUIRE(c->chain_length >= 2 && c->chain_length <= 16, "chain_length must be in [2, 16]");
  JMD_REQUIRE(c->chain_steps >= 1, "chain_steps must be >= 1");
  JMD_REQUIRE(c->sy_steps == 1 || c->sy_steps == 3 || c->sy_steps == 5 || c->sy_steps == 7,
              "sy_steps must be 1, 3, 5 or 7");
  const NhcArgs a = nhc_args(*c, update_mass);
  k_nhc_half<<<1, 32, 0, as_stream(stream)>>>(a, chain, kinetic_energy, p_scale);
  return check_launch("jmd_nhc_half_step");
}

int jmd_nhc_half_step_vjp(const jmd_nhc* c, const double* chain, const double* kinetic_energy,
                          int32_t update_mass, const double* cot_p_xi, const double* cot_scale,
                          double* grad_p_xi, double* grad_kinetic_energy, void* stream) {
  JMD_REQUIRE(c != nullptr && chain && kinetic_energy && cot_p_xi && cot_scale && grad_p_xi &&
                  grad_kinetic_energy,
              "null argument");
  JMD_REQUIRE(c->chain_length >= 2 && c->chain_length <= 7,
              "the chain VJP supports chain_length 2..7");
  JMD_REQUIRE(c->chain_steps >= 1, "chain_steps must be >= 1");
  JMD_REQUIRE(c->sy_steps == 1 || c->sy_steps == 3 || c->sy_steps == 5 || c->sy_steps == 7,
              "sy_steps must be 1, 3, 5 or 7");
  const NhcArgs a = nhc_args(*c, update_mass);
  k_nhc_half_vjp<<<1, 32, 0, as_stream(stream)>>>(a, chain, kinetic_energy, cot_p_xi, cot_scale,
                                                  grad_p_xi, grad_kinetic_energy);
  return check_launch("jmd_nhc_half_step_vjp");
}

int jmd_scale_momentum(float* momentum, int64_t p_stride, int64_t n, int32_t dim,
                       const double* scale, void* stream) {
  JMD_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
  if (n <= 0) return JMD_OK;
  unsigned gr = (unsigned)ceil_div(n, 256);
  if (dim == 3) k_scale<3><<<gr, 256, 0, as_stream(stream)>>>(momentum, p_stride, (int)n, scale);
  else k_scale<2><<<gr, 256, 0, as_stream(stream)>>>(momentum, p_stride, (int)n, scale);
  return check_launch("jmd_scale_momentum");
}

int jmd_npt_map(int32_t mode, float* position, float* momentum, const float* force,
                const float* mass, float mass_scalar, int64_t n, const jmd_space* space,
                float c0, float c1, void* stream) {
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(mode == 0 || mode == 1, "mode must be 0 (positions) or 1 (momenta)");
  JMD_REQUIRE(n >= 0 && n < INT32_MAX, "atom count out of range");
  JMD_REQUIRE(momentum && is_vec4(momentum, 4), "momenta must be 16-byte aligned float4 rows");
  JMD_REQUIRE(mode == 1 || (position && is_vec4(position, 4)),
              "positions must be 16-byte aligned float4 rows");
  JMD_REQUIRE(mode == 0 || (force && is_vec4(force, 4)), "forces must be 16-byte aligned float4 rows");
  if (n == 0) return JMD_OK;
  const unsigned gr = (unsigned)ceil_div(n, 256);
  const Geo g = make_geo(*space);
  auto* x = reinterpret_cast<float4*>(position);
  auto* p = reinterpret_cast<float4*>(momentum);
  auto* f = reinterpret_cast<const float4*>(force);
  if (space->dim == 3)
    k_npt_map<3><<<gr, 256, 0, as_stream(stream)>>>(mode, x, p, f, mass, mass_scalar, (int)n, g, c0, c1);
  else
    k_npt_map<2><<<gr, 256, 0, as_stream(stream)>>>(mode, x, p, f, mass, mass_scalar, (int)n, g, c0, c1);
  return check_launch("jmd_npt_map");
}

int jmd_langevin_o_step(float* momentum, int64_t p_stride, int64_t n, int32_t dim,
                        const float* mass, float mass_scalar, float c1, float c2, uint64_t seed,
                        uint64_t step, float* noise_out, void* stream) {
  JMD_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
  JMD_REQUIRE(n >= 0 && n < INT32_MAX, "atom count out of range");
  JMD_REQUIRE(momentum != nullptr || n == 0, "momentum is null");
  JMD_REQUIRE(p_stride >= dim, "momentum rows are narrower than dim");
  JMD_REQUIRE(c1 >= 0.f && c1 <= 1.f && c2 >= 0.f, "need 0 <= c1 <= 1 and c2 >= 0");
  JMD_REQUIRE(noise_out == nullptr || (reinterpret_cast<uintptr_t>(noise_out) % 16) == 0,
              "noise rows must be 16-byte aligned");
  if (n == 0) return JMD_OK;
  const unsigned gr = (unsigned)ceil_div(n, 256);
  float4* z = reinterpret_cast<float4*>(noise_out);
  if (dim == 3)
    k_langevin_o<3><<<gr, 256, 0, as_stream(stream)>>>(momentum, p_stride, (int)n, mass,
                                                       mass_scalar, c1, c2, seed, step, z);
  else
    k_langevin_o<2><<<gr, 256, 0, as_stream(stream)>>>(momentum, p_stride, (int)n, mass,
                                                       mass_scalar, c1, c2, seed, step, z);
  return check_launch("jmd_langevin_o_step");
}

int jmd_fire_kick_drift(float* position, float* momentum, const float* force, const float* mass,
                        float mass_scalar, int64_t n, const jmd_space* space,
                        const float* fire_state, void* stream) {
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(is_vec4(position, 4) && is_vec4(momentum, 4) && is_vec4(force, 4),
              "FIRE needs 16-byte aligned float4 rows");
  if (n <= 0) return JMD_OK;
  const unsigned gr = (unsigned)ceil_div(n, 256);
  Geo g = make_geo(*space);
  auto* x4 = reinterpret_cast<float4*>(position);
  auto* p4 = reinterpret_cast<float4*>(momentum);
  auto* f4 = reinterpret_cast<const float4*>(force);
  if (space->dim == 3)
    k_fire_kick_drift<3><<<gr, 256, 0, as_stream(stream)>>>(x4, p4, f4, mass, mass_scalar, (int)n, g, fire_state);
  else
    k_fire_kick_drift<2><<<gr, 256, 0, as_stream(stream)>>>(x4, p4, f4, mass, mass_scalar, (int)n, g, fire_state);
  return check_launch("jmd_fire_kick_drift");
}

int jmd_fire_update(float* momentum, const float* force, int64_t n, int32_t dim,
                    float* fire_state, float dt_max, float n_min, float f_inc, float f_dec,
                    float alpha_start, float f_alpha, void* workspace, size_t workspace_bytes,
                    void* stream) {
  JMD_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
  JMD_REQUIRE(is_vec4(momentum, 4) && is_vec4(force, 4), "FIRE needs 16-byte aligned float4 rows");
  cudaStream_t st = as_stream(stream);
  Carver cv(workspace, workspace_bytes);
  double* partials = cv.take<double>(kMaxReduceBlocks * 3);
  unsigned int* counter = cv.take<unsigned int>(1);
  double* red = cv.take<double>(4);
  if (!cv.ok()) return fail(JMD_ERR_WORKSPACE, "FIRE workspace too small");
  if (n <= 0) return JMD_OK;
  const int64_t gr = ceil_div(n, 256);
  if (gr > kMaxReduceBlocks) return fail(JMD_ERR_UNSUPPORTED, "system too large");
  FireParams fp{dt_max, n_min, f_inc, f_dec, alpha_start, f_alpha};
  JMD_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), st));
  auto* p4 = reinterpret_cast<float4*>(momentum);
  auto* f4 = reinterpret_cast<const float4*>(force);
  if (dim == 3)
    k_fire_finish<3><<<(unsigned)gr, 256, 0, st>>>(p4, f4, (int)n, fire_state, partials, counter, red);
  else
    k_fire_finish<2><<<(unsigned)gr, 256, 0, st>>>(p4, f4, (int)n, fire_state, partials, counter, red);
  k_fire_scalar<<<1, 32, 0, st>>>(fire_state, fp, red);
  k_fire_mix<<<(unsigned)gr, 256, 0, st>>>(p4, f4, (int)n, fire_state);
  return check_launch("jmd_fire_update");
}

size_t jmd_fire_workspace_bytes(int64_t n) {
  (void)n;
  Carver cv(nullptr, 0);
  cv.take<double>(kMaxReduceBlocks * 3);
  cv.take<unsigned int>(1);
  cv.take<double>(4);
  return cv.used + 256;
}

}  // extern "C"

// ------------------------------------------- kinetic energy, static scratch --
// A variant of jmd_kinetic_energy for callers that cannot hand the library a
// workspace: its block partials and completion counter live in a fixed
// device array compiled into this library, so a call allocates nothing.
namespace jmd {
namespace {

// The documented limit, and the blocks ke_blocks launches for it (2048 atoms
// per block: 2048 blocks).  The array holds one f64 partial per block.
constexpr int64_t kStaticMaxAtoms = 4194304;
constexpr int64_t kStaticReduceBlocks = (kStaticMaxAtoms + kKeAtomsPerBlock - 1) / kKeAtomsPerBlock;
static_assert(kStaticReduceBlocks * kKeAtomsPerBlock >= kStaticMaxAtoms,
              "the static partials must cover every block ke_blocks launches at the limit");
constexpr size_t kStaticCounterOffset = sizeof(double) * kStaticReduceBlocks;
// 16 KiB of partials + one counter (256 bytes keep the counter aligned).
static __device__ __align__(256) unsigned char g_reduce_scratch[kStaticCounterOffset + 256];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_reduce_scratch on the current device, looked up once
// per device (the first call on that device) and cached.
int static_reduce_scratch(void** out) {
  int dev = 0;
  JMD_CUDA(cudaGetDevice(&dev));
  JMD_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal beyond the static scratch table");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_reduce_scratch);
    if (e != cudaSuccess)
      return fail(JMD_ERR_CUDA, std::string("cudaGetSymbolAddress(static reduce scratch): ") +
                                    cudaGetErrorString(e));
    g_scratch_ptr[dev] = ptr;
  }
  *out = g_scratch_ptr[dev];
  return JMD_OK;
}

}  // namespace
}  // namespace jmd

extern "C" {

int jmd_kinetic_energy_static_scratch(const float* momentum, int64_t p_stride, const float* mass,
                                      float mass_scalar, int64_t n, int32_t dim, double* out,
                                      void* stream) {
  JMD_REQUIRE(dim == 2 || dim == 3, "dim must be 2 or 3");
  JMD_REQUIRE(out != nullptr, "out is null");
  JMD_REQUIRE(n <= kStaticMaxAtoms,
              "n exceeds the static-scratch limit of 4194304 atoms; use jmd_kinetic_energy with "
              "a workspace");
  void* base = nullptr;
  int rc = static_reduce_scratch(&base);
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  if (n <= 0) {
    JMD_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st));
    return JMD_OK;
  }
  double* partials = static_cast<double*>(base);
  unsigned int* counter =
      reinterpret_cast<unsigned int*>(static_cast<char*>(base) + kStaticCounterOffset);
  // the completion counter must start at zero; the partials are overwritten
  JMD_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), st));
  const unsigned gr = ke_blocks(n);
  JMD_REQUIRE(gr <= kStaticReduceBlocks, "static scratch smaller than the reduction's block count");
  if (dim == 3)
    k_ke<3><<<gr, 256, 0, st>>>(momentum, p_stride, mass, mass_scalar, (int)n, partials, counter, out);
  else
    k_ke<2><<<gr, 256, 0, st>>>(momentum, p_stride, mass, mass_scalar, (int)n, partials, counter, out);
  return check_launch("jmd_kinetic_energy_static_scratch");
}

}  // extern "C"
