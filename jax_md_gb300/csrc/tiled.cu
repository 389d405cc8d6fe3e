// Thread-per-atom pair kernels on the engine's tiled neighbour layout.
//
// Reference: jax_md/smap.py:922-979 (pair energy over a neighbour list),
// quantity.py:58-60 (force), simulate.py:227-243 (velocity_verlet),
// partition.py:1146-1154 (skin test).
//
// Tiled layout (engine-private, atoms in cell order): atoms are grouped in
// tiles of 32; tile t stores entry k of its atoms contiguously,
//   tidx[t][k][lane]  (t = i / 32, lane = i % 32),
// so a warp reading entry k of its 32 atoms issues one 128-byte load.  The
// count array bounds each atom's column; nothing is padded.
//
// One thread owns one atom: it loads four column entries, issues their four
// position gathers back to back (evict-last), and evaluates them as two packed
// FP32x2 pairs.  No cross-lane reduction is needed.  The kernel is capped
// at 56 registers (9 CTAs of 128 threads per SM): it is bound by gather
// latency, so resident warps matter more than prefetched epilogue rows.
#include "dense.cuh"

namespace jmd {
namespace {

enum { T_FORCE = 0, T_STEP = 2, T_KICK = 3 };

struct TArgs {
  const float4* x;
  const int32_t* species;
  int n;
  const int32_t* tidx;
  int64_t depth;     // entries per atom column (row capacity of the tile)
  int width;         // max_occupancy
  const int32_t* cnt;
  float4* f;
  Geo geo;
  float margin;
  float4* p;
  float4* x_next;
  float m0;
  float dt;
  const float4* ref;
  float thr2;
  int32_t* flag;
};

__device__ __forceinline__ int spc2(int s, int nsp) { return s < 0 ? 0 : (s >= nsp ? nsp - 1 : s); }

template <int DIM, int KIND, bool SPECIES, int MODE>
__global__ void __launch_bounds__(128, 9)
k_tiled(TArgs a, const __grid_constant__ PairTable tab) {
  __shared__ PairCoef sc[SPECIES ? JMD_MAX_SPECIES * JMD_MAX_SPECIES : 1];
  if (SPECIES) {
    for (int k = threadIdx.x; k < JMD_MAX_SPECIES * JMD_MAX_SPECIES; k += blockDim.x) sc[k] = tab.c[k];
    __syncthreads();
  }
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4 xi = __ldg(a.x + i);
  float4 q = make_float4(0.f, 0.f, 0.f, 0.f), rf = q;
  const int c = min(__ldg(a.cnt + i), a.width);
  const int32_t* col = a.tidx + (int64_t)(i >> 5) * a.depth * 32 + (i & 31);
  const int si = SPECIES ? spc2(__ldg(a.species + i), tab.nsp) : 0;
  const bool inner = interior<DIM>(xi, a.geo, a.margin);
  const float2 xx = f2s(xi.x), xy = f2s(xi.y), xz = f2s(xi.z);
  const float rc2m = tab.rc2_max;
  const Coef2 c0 = coef2(tab.c[0]);
  const uint64_t pol = policy_keep();
  float2 ax = f2s(0.f), ay = f2s(0.f), az = f2s(0.f);

  auto pair2 = [&](int j0, int j1, const float4& b0, const float4& b1) {
    float2 dx = sub2(xx, f2(b0.x, b1.x));
    float2 dy = sub2(xy, f2(b0.y, b1.y));
    float2 dz = DIM == 3 ? sub2(xz, f2(b0.z, b1.z)) : f2s(0.f);
    if (!inner) {
      float ex, ey, ez;
      displacement<DIM>(xi, b0, a.geo, ex, ey, ez);
      dx.x = ex; dy.x = ey; dz.x = ez;
      displacement<DIM>(xi, b1, a.geo, ex, ey, ez);
      dx.y = ex; dy.y = ey; dz.y = ez;
    }
    float2 r2 = mul2(dx, dx);
    r2 = fma2(dy, dy, r2);
    if (DIM == 3) r2 = fma2(dz, dz, r2);
    Coef2 cc;
    if (SPECIES)
      cc = coef2(sc[si * JMD_MAX_SPECIES + spc2(__ldg(a.species + j0), tab.nsp)],
                 sc[si * JMD_MAX_SPECIES + spc2(__ldg(a.species + j1), tab.nsp)]);
    else
      cc = c0;
    const float rc0 = SPECIES ? cc.rc2.x : rc2m, rc1 = SPECIES ? cc.rc2.y : rc2m;
    const bool m0 = r2.x < rc0 && r2.x > 0.f;
    const bool m1 = r2.y < rc1 && r2.y > 0.f;
    // masked pairs (beyond the cutoff, or the atom itself at r2 = 0) may give
    // inf/NaN here; the selects below discard them
    float2 U, g;
    pair_eval2<KIND, false>(r2, cc, U, g);
    g.x = m0 ? g.x : 0.f;
    g.y = m1 ? g.y : 0.f;
    ax = fma2(g, dx, ax);
    ay = fma2(g, dy, ay);
    if (DIM == 3) az = fma2(g, dz, az);
  };

  // Entries past the count point at the atom itself (distance 0: masked).
  // The column indices of the next four entries are loaded while the current
  // four positions are gathered, so each iteration waits on one memory
  // latency (the gathers) instead of two.
  int jn[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) jn[u] = (u < c) ? __ldcs(col + u * 32) : i;
  for (int k0 = 0; k0 < c; k0 += 4) {
    int j[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) j[u] = jn[u];
    float4 b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) b[u] = ldg_keep(a.x + j[u], pol);
#pragma unroll
    for (int u = 0; u < 4; ++u) jn[u] = (k0 + 4 + u < c) ? __ldcs(col + (k0 + 4 + u) * 32) : i;
    pair2(j[0], j[1], b[0], b[1]);
    if (k0 + 2 < c) pair2(j[2], j[3], b[2], b[3]);
  }
  const float fx = -(ax.x + ax.y), fy = -(ay.x + ay.y), fz = DIM == 3 ? -(az.x + az.y) : 0.f;
  // epilogue rows are loaded after the loop: keeping them live through it
  // would cost the registers of a ninth resident CTA
  if (MODE == T_STEP || MODE == T_KICK) q = a.p[i];
  if (MODE == T_STEP && a.ref) rf = __ldg(a.ref + i);
  if (MODE == T_FORCE || MODE == T_KICK) a.f[i] = make_float4(fx, fy, fz, 0.f);
  const float h = 0.5f * a.dt;
  if (MODE == T_KICK) {
    q.x = fmaf(h, fx, q.x);
    q.y = fmaf(h, fy, q.y);
    q.z = fmaf(h, fz, q.z);
    a.p[i] = q;
  }
  if (MODE == T_STEP) {
    q.x = fmaf(h, fx, q.x);
    q.y = fmaf(h, fy, q.y);
    q.z = fmaf(h, fz, q.z);
    q.x = fmaf(h, fx, q.x);
    q.y = fmaf(h, fy, q.y);
    q.z = fmaf(h, fz, q.z);
    float4 r = xi;
    const float ddx = a.dt * q.x / a.m0, ddy = a.dt * q.y / a.m0, ddz = a.dt * q.z / a.m0;
    if (a.geo.periodic) {
      r.x = wrap(r.x + ddx, a.geo.L[0]);
      r.y = wrap(r.y + ddy, a.geo.L[1]);
      if (DIM == 3) r.z = wrap(r.z + ddz, a.geo.L[2]);
    } else {
      r.x += ddx;
      r.y += ddy;
      if (DIM == 3) r.z += ddz;
    }
    a.p[i] = q;
    a.x_next[i] = r;
    if (a.ref) {
      float ex, ey, ez;
      displacement<DIM>(r, rf, a.geo, ex, ey, ez);
      if (ex * ex + ey * ey + ez * ez > a.thr2) atomicOr(a.flag, 1);
    }
  }
}

template <int DIM, int KIND, int MODE>
void tl_sp(bool sp, const TArgs& a, const PairTable& t, cudaStream_t st) {
  const unsigned grid = (unsigned)std::max<int64_t>(1, ceil_div(a.n, 128));
  if (sp) k_tiled<DIM, KIND, true, MODE><<<grid, 128, 0, st>>>(a, t);
  else k_tiled<DIM, KIND, false, MODE><<<grid, 128, 0, st>>>(a, t);
}

template <int MODE>
void tl_launch(int dim, int kind, bool sp, const TArgs& a, const PairTable& t, cudaStream_t st) {
  if (dim == 3) {
    if (kind == JMD_LJ) tl_sp<3, JMD_LJ, MODE>(sp, a, t, st);
    else if (kind == JMD_LJ_TRUNCATED) tl_sp<3, JMD_LJ_TRUNCATED, MODE>(sp, a, t, st);
    else if (kind == JMD_MORSE) tl_sp<3, JMD_MORSE, MODE>(sp, a, t, st);
    else tl_sp<3, JMD_SOFT_SPHERE, MODE>(sp, a, t, st);
  } else {
    if (kind == JMD_LJ) tl_sp<2, JMD_LJ, MODE>(sp, a, t, st);
    else if (kind == JMD_LJ_TRUNCATED) tl_sp<2, JMD_LJ_TRUNCATED, MODE>(sp, a, t, st);
    else if (kind == JMD_MORSE) tl_sp<2, JMD_MORSE, MODE>(sp, a, t, st);
    else tl_sp<2, JMD_SOFT_SPHERE, MODE>(sp, a, t, st);
  }
}

int tl_validate(const jmd_pair* pp, const jmd_space* space, const float* x, const int32_t* tidx,
                const int32_t* cnt) {
  int e = validate_pair(pp);
  if (e) return e;
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(space->periodic != JMD_GENERAL_CELL, "the tiled kernels take orthorhombic boxes");
  JMD_REQUIRE(is_vec4(x, 4), "positions must be 16-byte aligned float4 rows");
  JMD_REQUIRE(tidx != nullptr && cnt != nullptr, "tiled list and counts are required");
  return JMD_OK;
}

TArgs tl_args(const jmd_pair* pp, const jmd_space* space, const float* x, const int32_t* species,
              int64_t n, const int32_t* tidx, int64_t depth, int64_t width, const int32_t* cnt,
              const PairTable& t) {
  TArgs a{};
  a.x = reinterpret_cast<const float4*>(x);
  a.species = species;
  a.n = (int)n;
  a.tidx = tidx;
  a.depth = depth;
  a.width = (int)std::min<int64_t>(width, depth);
  a.cnt = cnt;
  a.geo = make_geo(*space);
  a.margin = sqrtf(t.rc2_max);
  (void)pp;
  return a;
}

}  // namespace
}  // namespace jmd

using namespace jmd;

extern "C" {

int jmd_pair_forces_tiled(const jmd_pair* pp, const jmd_space* space, const float* position,
                          const int32_t* species, int64_t n, const int32_t* tidx, int64_t depth,
                          int64_t width, const int32_t* nbr_count, float* force, void* stream) {
  int e = tl_validate(pp, space, position, tidx, nbr_count);
  if (e) return e;
  JMD_REQUIRE(is_vec4(force, 4), "forces must be 16-byte aligned float4 rows");
  if (n <= 0) return JMD_OK;
  PairTable t = make_pair_table(*pp);
  TArgs a = tl_args(pp, space, position, species, n, tidx, depth, width, nbr_count, t);
  a.f = reinterpret_cast<float4*>(force);
  tl_launch<T_FORCE>(space->dim, pp->kind, pp->n_species > 0, a, t, as_stream(stream));
  return check_launch("jmd_pair_forces_tiled");
}

int jmd_nve_fused_step_tiled(const jmd_pair* pp, const jmd_space* space, const float* position,
                             float* position_next, float* momentum, float mass_scalar,
                             const int32_t* species, int64_t n, const int32_t* tidx, int64_t depth,
                             int64_t width, const int32_t* nbr_count, float dt,
                             const float* reference_position, float threshold_sq,
                             int32_t* rebuild_flag, void* stream) {
  int e = tl_validate(pp, space, position, tidx, nbr_count);
  if (e) return e;
  JMD_REQUIRE(position != position_next, "position and position_next must differ");
  JMD_REQUIRE(is_vec4(position_next, 4) && is_vec4(momentum, 4) &&
                  (reference_position == nullptr || is_vec4(reference_position, 4)),
              "float4 rows must be 16-byte aligned");
  JMD_REQUIRE(reference_position == nullptr || rebuild_flag != nullptr, "skin test needs a flag");
  if (n <= 0) return JMD_OK;
  PairTable t = make_pair_table(*pp);
  TArgs a = tl_args(pp, space, position, species, n, tidx, depth, width, nbr_count, t);
  a.p = reinterpret_cast<float4*>(momentum);
  a.x_next = reinterpret_cast<float4*>(position_next);
  a.m0 = mass_scalar;
  a.dt = dt;
  a.ref = reinterpret_cast<const float4*>(reference_position);
  a.thr2 = threshold_sq;
  a.flag = rebuild_flag;
  tl_launch<T_STEP>(space->dim, pp->kind, pp->n_species > 0, a, t, as_stream(stream));
  return check_launch("jmd_nve_fused_step_tiled");
}

int jmd_force_kick_tiled(const jmd_pair* pp, const jmd_space* space, const float* position,
                         float* force, float* momentum, const int32_t* species, int64_t n,
                         const int32_t* tidx, int64_t depth, int64_t width,
                         const int32_t* nbr_count, float dt, void* stream) {
  int e = tl_validate(pp, space, position, tidx, nbr_count);
  if (e) return e;
  JMD_REQUIRE(is_vec4(force, 4) && is_vec4(momentum, 4), "float4 rows must be 16-byte aligned");
  if (n <= 0) return JMD_OK;
  PairTable t = make_pair_table(*pp);
  TArgs a = tl_args(pp, space, position, species, n, tidx, depth, width, nbr_count, t);
  a.f = reinterpret_cast<float4*>(force);
  a.p = reinterpret_cast<float4*>(momentum);
  a.dt = dt;
  tl_launch<T_KICK>(space->dim, pp->kind, pp->n_species > 0, a, t, as_stream(stream));
  return check_launch("jmd_force_kick_tiled");
}

}  // extern "C"
