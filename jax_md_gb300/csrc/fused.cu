// Dense-list pair kernels on float4 rows with packed FP32x2 arithmetic, and
// the fused velocity-Verlet step built on them.
//
// Reference: jax_md/smap.py:922-979 (pair_neighbor_list), quantity.py:58-60
// (force = -grad E), simulate.py:227-243 (velocity_verlet),
// partition.py:1146-1154 (skin test).
//
// Layout: positions, momenta and forces are float4 rows ([N,4] storage, the
// fourth float is carried unchanged); Dense rows are int32 with an even row
// stride so each lane loads two consecutive entries as one 8-byte load.
//
// Work split: TPA lanes per atom, each lane two entries per iteration.  The
// pair arithmetic runs on float2 (FFMA2/FMUL2/FADD2), i.e. two pairs per
// issued instruction, which halves the FP32 issue pressure that bounds this
// gather-heavy kernel.  Atoms farther than the interaction cutoff from every
// periodic face ("interior") skip the wrap logic entirely: for them the plain
// difference equals the minimum image for every pair that can interact.
//
// Modes
//   FORCE : f_i = -dE/dR_i
//   EV    : + energy, per-atom energy, virial (deterministic f64 reduction)
//   STEP  : fused NVE step from the half-kicked state (p' = p + dt/2 f_old):
//           f = F(x); p += dt/2 f; p += dt/2 f; x_next = shift(x, dt p / m);
//           skin test of x_next against the reference positions -> flag.
//           The force is not stored (the next launch recomputes it).
//   KICK  : f = F(x) stored; p += dt/2 f (the closing half kick).
#include "dense.cuh"

namespace jmd {
namespace {

enum { MODE_FORCE = 0, MODE_EV = 1, MODE_STEP = 2, MODE_KICK = 3 };

struct D2Args {
  const float4* x;
  const int32_t* species;
  int n;
  const int32_t* idx;
  int64_t ld;
  int64_t width;
  const int32_t* cnt;
  float4* f;
  float* e_atom;
  double* partials;
  unsigned int* counter;
  double* totals;
  Geo geo;
  float margin;        // interaction cutoff (interior test)
  // STEP / KICK
  float4* p;
  float4* x_next;
  const float* mass;
  float m0;
  float dt;
  const float4* ref;
  float thr2;
  int32_t* flag;
};

template <int TPA, typename T>
__device__ __forceinline__ T gsum(T v) {
#pragma unroll
  for (int o = TPA / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int spc(int s, int nsp) { return s < 0 ? 0 : (s >= nsp ? nsp - 1 : s); }

template <int DIM, int TPA, int KIND, bool SPECIES, int MODE, bool CNT>
__global__ void __launch_bounds__(256)
k_dense2(D2Args a, const __grid_constant__ PairTable tab) {
  constexpr bool EV = MODE == MODE_EV;
  __shared__ PairCoef sc[SPECIES ? JMD_MAX_SPECIES * JMD_MAX_SPECIES : 1];
  if (SPECIES) {
    for (int k = threadIdx.x; k < JMD_MAX_SPECIES * JMD_MAX_SPECIES; k += blockDim.x) sc[k] = tab.c[k];
    __syncthreads();
  }
  const int atom = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / TPA);
  const int sub = threadIdx.x & (TPA - 1);
  const bool active = atom < a.n;
  float2 ax = f2s(0.f), ay = f2s(0.f), az = f2s(0.f), ae = f2s(0.f);
  float2 w0 = f2s(0.f), w1 = f2s(0.f), w2 = f2s(0.f), w3 = f2s(0.f), w4 = f2s(0.f), w5 = f2s(0.f);
  float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
  // rows the epilogue needs, loaded now so their latency overlaps the loop
  float4 q = xi, rf = xi;
  if (active && sub == 0) {
    if (MODE == MODE_STEP || MODE == MODE_KICK) q = a.p[atom];
    if (MODE == MODE_STEP && a.ref) rf = __ldg(a.ref + atom);
  }
  if (active) {
    xi = __ldg(a.x + atom);
    const int si = SPECIES ? spc(__ldg(a.species + atom), tab.nsp) : 0;
    const int32_t* row = a.idx + (int64_t)atom * a.ld;
    int end = (int)a.width;
    if (CNT) end = min(__ldg(a.cnt + atom), end);
    const float2 xx = f2s(xi.x), xy = f2s(xi.y), xz = f2s(xi.z);
    const bool inner = interior<DIM>(xi, a.geo, a.margin);
    const float rc2m = tab.rc2_max;
    const Coef2 c0 = coef2(tab.c[0]);
    const uint64_t pol = policy_keep();
    // One packed step over the entries k, k+1 whose ids and positions are loaded.
    auto body = [&](int2 jj, int k, const float4& b0, const float4& b1) {
      const bool v1 = k + 1 < end;
      bool ok0 = true, ok1 = v1;
      int j0 = jj.x, j1 = jj.y;
      if (!CNT) {
        ok0 = (unsigned)j0 < (unsigned)a.n;
        ok1 = ok1 && (unsigned)j1 < (unsigned)a.n;
      }
      float2 dx = sub2(xx, f2(b0.x, b1.x));
      float2 dy = sub2(xy, f2(b0.y, b1.y));
      float2 dz = DIM == 3 ? sub2(xz, f2(b0.z, b1.z)) : f2s(0.f);
      if (!inner) {
        // exact minimum image, element by element (atoms near a periodic face)
        float ex, ey, ez;
        displacement<DIM>(xi, b0, a.geo, ex, ey, ez);
        dx.x = ex; dy.x = ey; dz.x = ez;
        displacement<DIM>(xi, b1, a.geo, ex, ey, ez);
        dx.y = ex; dy.y = ey; dz.y = ez;
      }
      float2 r2 = mul2(dx, dx);
      r2 = fma2(dy, dy, r2);
      if (DIM == 3) r2 = fma2(dz, dz, r2);
      Coef2 c;
      if (SPECIES) {
        const int sj0 = ok0 ? spc(__ldg(a.species + j0), tab.nsp) : 0;
        const int sj1 = ok1 ? spc(__ldg(a.species + j1), tab.nsp) : 0;
        c = coef2(sc[si * JMD_MAX_SPECIES + sj0], sc[si * JMD_MAX_SPECIES + sj1]);
      } else {
        c = c0;
      }
      const float rc0 = SPECIES ? c.rc2.x : rc2m, rc1 = SPECIES ? c.rc2.y : rc2m;
      const bool m0 = ok0 && r2.x < rc0 && r2.x > 0.f;
      const bool m1 = ok1 && r2.y < rc1 && r2.y > 0.f;
      if (!(m0 || m1)) return;
      const float2 r2s = f2(m0 ? r2.x : 1.f, m1 ? r2.y : 1.f);
      float2 U, g;
      pair_eval2<KIND, EV>(r2s, c, U, g);
      g.x = m0 ? g.x : 0.f;
      g.y = m1 ? g.y : 0.f;
      // accumulate +g d; the force is its negative
      ax = fma2(g, dx, ax);
      ay = fma2(g, dy, ay);
      if (DIM == 3) az = fma2(g, dz, az);
      if (EV) {
        U.x = m0 ? U.x : 0.f;
        U.y = m1 ? U.y : 0.f;
        ae = add2(ae, U);
        const float2 gx = mul2(g, dx), gy = mul2(g, dy);
        w0 = fma2(gx, dx, w0);
        w1 = fma2(gy, dy, w1);
        if (DIM == 3) {
          const float2 gz = mul2(g, dz);
          w2 = fma2(gz, dz, w2);
          w3 = fma2(gx, dy, w3);
          w4 = fma2(gx, dz, w4);
          w5 = fma2(gy, dz, w5);
        } else {
          w3 = fma2(gx, dy, w3);
        }
      }
    };
    // Ids that cannot be gathered (padding, sentinels) are replaced by the atom
    // itself: its position is at distance 0 and the pair is masked.
    auto fix = [&](int2 jj, int k) -> int2 {
      if (!(k + 1 < end)) jj.y = atom;
      if (!CNT) {
        if ((unsigned)jj.x >= (unsigned)a.n) jj.x = atom;
        if ((unsigned)jj.y >= (unsigned)a.n) jj.y = atom;
      }
      return jj;
    };
    // Software pipeline: every id of this lane's slice (up to IT pairs) is
    // loaded up front, and the neighbour positions of slot t+1 are in flight
    // while slot t is evaluated.
    constexpr int IT = TPA == 4 ? 16 : (TPA == 8 ? 8 : 4);
    int2 ids[IT];
#pragma unroll
    for (int t = 0; t < IT; ++t) {
      const int k = 2 * sub + t * 2 * TPA;
      ids[t] = k < end ? fix(__ldcs(reinterpret_cast<const int2*>(row + k)), k)
                       : make_int2(atom, atom);
    }
    float4 c0p = make_float4(0.f, 0.f, 0.f, 0.f), c1p = c0p;
    if (2 * sub < end) {
      c0p = ldg_keep(a.x + ids[0].x, pol);
      c1p = ldg_keep(a.x + ids[0].y, pol);
    }
#pragma unroll
    for (int t = 0; t < IT; ++t) {
      const int k = 2 * sub + t * 2 * TPA;
      if (k >= end) break;
      float4 n0 = c0p, n1 = c1p;
      if (t + 1 < IT && k + 2 * TPA < end) {
        n0 = ldg_keep(a.x + ids[t + 1].x, pol);
        n1 = ldg_keep(a.x + ids[t + 1].y, pol);
      }
      body(ids[t], k, c0p, c1p);
      c0p = n0;
      c1p = n1;
    }
    // rows longer than the prefetched slice
    for (int k = 2 * sub + IT * 2 * TPA; k < end; k += 2 * TPA) {
      const int2 jj = fix(__ldcs(reinterpret_cast<const int2*>(row + k)), k);
      const float4 b0 = ldg_keep(a.x + jj.x, pol);
      const float4 b1 = ldg_keep(a.x + jj.y, pol);
      body(jj, k, b0, b1);
    }
  }
  float fx = -gsum<TPA>(ax.x + ax.y);
  float fy = -gsum<TPA>(ay.x + ay.y);
  float fz = DIM == 3 ? -gsum<TPA>(az.x + az.y) : 0.f;
  const bool leader = active && sub == 0;
  if (MODE == MODE_FORCE || MODE == MODE_EV || MODE == MODE_KICK) {
    if (leader && a.f) a.f[atom] = make_float4(fx, fy, fz, 0.f);
  }
  if (MODE == MODE_KICK && leader) {
    const float h = 0.5f * a.dt;
    q.x = fmaf(h, fx, q.x);
    q.y = fmaf(h, fy, q.y);
    q.z = fmaf(h, fz, q.z);
    a.p[atom] = q;
  }
  if (MODE == MODE_STEP) {
    bool over = false;
    if (leader) {
      const float h = 0.5f * a.dt;
      // closing half kick of the previous step, opening half kick of this one
      q.x = fmaf(h, fx, q.x);
      q.y = fmaf(h, fy, q.y);
      q.z = fmaf(h, fz, q.z);
      q.x = fmaf(h, fx, q.x);
      q.y = fmaf(h, fy, q.y);
      q.z = fmaf(h, fz, q.z);
      const float m = a.mass ? a.mass[atom] : a.m0;
      float4 r = xi;
      const float ddx = a.dt * q.x / m, ddy = a.dt * q.y / m, ddz = a.dt * q.z / m;
      if (a.geo.periodic) {
        r.x = wrap(r.x + ddx, a.geo.L[0]);
        r.y = wrap(r.y + ddy, a.geo.L[1]);
        if (DIM == 3) r.z = wrap(r.z + ddz, a.geo.L[2]);
      } else {
        r.x += ddx;
        r.y += ddy;
        if (DIM == 3) r.z += ddz;
      }
      a.p[atom] = q;
      a.x_next[atom] = r;
      if (a.ref) {
        float ex, ey, ez;
        displacement<DIM>(r, rf, a.geo, ex, ey, ez);
        over = ex * ex + ey * ey + ez * ez > a.thr2;
      }
    }
    if (a.flag && __any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(a.flag, 1);
  }
  if (EV) {
    const float e = gsum<TPA>(ae.x + ae.y);
    float wv[6];
    wv[0] = gsum<TPA>(w0.x + w0.y);
    wv[1] = gsum<TPA>(w1.x + w1.y);
    wv[2] = gsum<TPA>(w2.x + w2.y);
    wv[3] = gsum<TPA>(w3.x + w3.y);
    wv[4] = gsum<TPA>(w4.x + w4.y);
    wv[5] = gsum<TPA>(w5.x + w5.y);
    if (leader && a.e_atom) a.e_atom[atom] = 0.5f * e;
    double v[7];
    v[0] = leader ? 0.5 * (double)e : 0.0;
    for (int k = 0; k < 6; ++k) v[1 + k] = leader ? 0.5 * (double)wv[k] : 0.0;
    grid_reduce<7>(v, a.partials, a.counter, a.totals, false);
  }
}

template <int DIM, int TPA, int KIND, bool SPECIES, int MODE>
void launch2(bool cnt, const D2Args& a, const PairTable& t, cudaStream_t st) {
  const int64_t threads = (int64_t)a.n * TPA;
  const unsigned grid = (unsigned)std::max<int64_t>(1, ceil_div(threads, 256));
  if (cnt) k_dense2<DIM, TPA, KIND, SPECIES, MODE, true><<<grid, 256, 0, st>>>(a, t);
  else k_dense2<DIM, TPA, KIND, SPECIES, MODE, false><<<grid, 256, 0, st>>>(a, t);
}

template <int DIM, int TPA, int KIND, int MODE>
void launch_sp(bool sp, bool cnt, const D2Args& a, const PairTable& t, cudaStream_t st) {
  if (sp) launch2<DIM, TPA, KIND, true, MODE>(cnt, a, t, st);
  else launch2<DIM, TPA, KIND, false, MODE>(cnt, a, t, st);
}

template <int DIM, int TPA, int MODE>
void launch_kind(int kind, bool sp, bool cnt, const D2Args& a, const PairTable& t, cudaStream_t st) {
  if (kind == JMD_LJ) launch_sp<DIM, TPA, JMD_LJ, MODE>(sp, cnt, a, t, st);
  else if (kind == JMD_LJ_TRUNCATED) launch_sp<DIM, TPA, JMD_LJ_TRUNCATED, MODE>(sp, cnt, a, t, st);
  else if (kind == JMD_MORSE) {
    if constexpr (TPA == 8) launch_sp<DIM, 8, JMD_MORSE, MODE>(sp, cnt, a, t, st);
  } else launch_sp<DIM, TPA, JMD_SOFT_SPHERE, MODE>(sp, cnt, a, t, st);
}

template <int DIM, int MODE>
void launch_tpa(int tpa, int kind, bool sp, bool cnt, const D2Args& a, const PairTable& t,
                cudaStream_t st) {
  // Morse runs at 8 lanes per atom only: its two exponentials per pair make
  // the lane width matter little, and one width keeps the build small
  if (kind == JMD_MORSE) tpa = 8;
  switch (tpa) {
    case 4: launch_kind<DIM, 4, MODE>(kind, sp, cnt, a, t, st); break;
    case 16: launch_kind<DIM, 16, MODE>(kind, sp, cnt, a, t, st); break;
    default: launch_kind<DIM, 8, MODE>(kind, sp, cnt, a, t, st); break;
  }
}

template <int MODE>
void launch_mode(int dim, int tpa, int kind, bool sp, bool cnt, const D2Args& a,
                 const PairTable& t, cudaStream_t st) {
  if (dim == 3) launch_tpa<3, MODE>(tpa, kind, sp, cnt, a, t, st);
  else launch_tpa<2, MODE>(tpa, kind, sp, cnt, a, t, st);
}

int g_tpa2 = 8;

}  // namespace

int dense_tpa() { return g_tpa2; }

// Shared with pair.cu: true when the float4 / packed path applies.
bool dense2_applicable(const float* x, int64_t xs, const int32_t* idx, int64_t ld, const float* f,
                       int64_t fs) {
  const bool idx_ok = (reinterpret_cast<uintptr_t>(idx) % 8) == 0 && (ld % 2) == 0;
  return is_vec4(x, xs) && (f == nullptr || is_vec4(f, fs)) && idx_ok;
}

int dense2_forces(const jmd_pair* pp, const jmd_space* space, const float* x, const int32_t* species,
                  int64_t n, const int32_t* idx, int64_t ld, int64_t width, const int32_t* cnt,
                  float* f, double* energy, float* e_atom, double* virial, double* partials,
                  unsigned int* counter, double* totals, cudaStream_t st) {
  PairTable t = make_pair_table(*pp);
  D2Args a{};
  a.x = reinterpret_cast<const float4*>(x);
  a.species = species;
  a.n = (int)n;
  a.idx = idx;
  a.ld = ld;
  a.width = width;
  a.cnt = cnt;
  a.f = reinterpret_cast<float4*>(f);
  a.e_atom = e_atom;
  a.partials = partials;
  a.counter = counter;
  a.totals = totals;
  a.geo = make_geo(*space);
  a.margin = sqrtf(t.rc2_max);
  const bool ev = energy || e_atom || virial;
  const bool sp = pp->n_species > 0;
  if (n > 0) {
    if (ev) launch_mode<MODE_EV>(space->dim, g_tpa2, pp->kind, sp, cnt != nullptr, a, t, st);
    else launch_mode<MODE_FORCE>(space->dim, g_tpa2, pp->kind, sp, cnt != nullptr, a, t, st);
  }
  return JMD_OK;
}

}  // namespace jmd

using namespace jmd;

extern "C" {

int jmd_set_dense_threads_per_atom(int tpa) {
  JMD_REQUIRE(tpa == 4 || tpa == 8 || tpa == 16, "threads per atom must be 4, 8 or 16");
  g_tpa2 = tpa;
  return JMD_OK;
}

int jmd_nve_fused_step(const jmd_pair* pp, const jmd_space* space, const float* position,
                       float* position_next, float* momentum, const float* mass,
                       float mass_scalar, const int32_t* species, int64_t n, const int32_t* idx,
                       int64_t idx_ld, int64_t idx_width, const int32_t* nbr_count, float dt,
                       const float* reference_position, float threshold_sq,
                       int32_t* rebuild_flag, void* stream) {
  int e = validate_pair(pp);
  if (e) return e;
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(space->periodic != JMD_GENERAL_CELL,
              "the fused kernels take orthorhombic boxes (general cells: jmd_pair_forces)");
  JMD_REQUIRE(position != position_next, "position and position_next must differ");
  JMD_REQUIRE(dense2_applicable(position, 4, idx, idx_ld, position_next, 4) &&
                  is_vec4(momentum, 4) && (reference_position == nullptr || is_vec4(reference_position, 4)),
              "fused step needs 16-byte aligned float4 rows and an even, 8-byte aligned idx");
  JMD_REQUIRE(reference_position == nullptr || rebuild_flag != nullptr, "skin test needs a flag");
  if (n <= 0) return JMD_OK;
  PairTable t = make_pair_table(*pp);
  D2Args a{};
  a.x = reinterpret_cast<const float4*>(position);
  a.species = species;
  a.n = (int)n;
  a.idx = idx;
  a.ld = idx_ld;
  a.width = idx_width;
  a.cnt = nbr_count;
  a.geo = make_geo(*space);
  a.margin = sqrtf(t.rc2_max);
  a.p = reinterpret_cast<float4*>(momentum);
  a.x_next = reinterpret_cast<float4*>(position_next);
  a.mass = mass;
  a.m0 = mass_scalar;
  a.dt = dt;
  a.ref = reinterpret_cast<const float4*>(reference_position);
  a.thr2 = threshold_sq;
  a.flag = rebuild_flag;
  launch_mode<MODE_STEP>(space->dim, g_tpa2, pp->kind, pp->n_species > 0, nbr_count != nullptr, a,
                         t, as_stream(stream));
  return check_launch("jmd_nve_fused_step");
}

int jmd_force_kick(const jmd_pair* pp, const jmd_space* space, const float* position,
                   float* force, float* momentum, const int32_t* species, int64_t n,
                   const int32_t* idx, int64_t idx_ld, int64_t idx_width,
                   const int32_t* nbr_count, float dt, void* stream) {
  int e = validate_pair(pp);
  if (e) return e;
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(space->periodic != JMD_GENERAL_CELL,
              "the fused kernels take orthorhombic boxes (general cells: jmd_pair_forces)");
  JMD_REQUIRE(dense2_applicable(position, 4, idx, idx_ld, force, 4) && is_vec4(momentum, 4),
              "force_kick needs 16-byte aligned float4 rows and an even, 8-byte aligned idx");
  if (n <= 0) return JMD_OK;
  PairTable t = make_pair_table(*pp);
  D2Args a{};
  a.x = reinterpret_cast<const float4*>(position);
  a.species = species;
  a.n = (int)n;
  a.idx = idx;
  a.ld = idx_ld;
  a.width = idx_width;
  a.cnt = nbr_count;
  a.f = reinterpret_cast<float4*>(force);
  a.geo = make_geo(*space);
  a.margin = sqrtf(t.rc2_max);
  a.p = reinterpret_cast<float4*>(momentum);
  a.dt = dt;
  launch_mode<MODE_KICK>(space->dim, g_tpa2, pp->kind, pp->n_species > 0, nbr_count != nullptr, a,
                         t, as_stream(stream));
  return check_launch("jmd_force_kick");
}

}  // extern "C"
