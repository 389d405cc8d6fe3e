// Neighbour-list pair energy / force / virial kernels.
//
// Reference: jax_md/smap.py:922-979 (pair_neighbor_list fn_mapped) with the
// force taken as grad(-E) (jax_md/quantity.py:58-60) and the virial as
// dU/d(strain) (jax_md/quantity.py:238-282).
//
// Dense lists: TPA lanes cooperate on one atom.  Each lane streams a slice of
// the atom's index row (evict-first loads: the row is read once per step),
// gathers neighbour positions as float4 from L2, evaluates the pair and
// accumulates the force in registers; the group reduces with xor shuffles and
// one lane writes the row.  Because the full list holds every pair twice, the
// force on atom i is sum_j -U'(r)/r (R_i - R_j) from its own row alone:
// no atomics, deterministic.  Energies and the virial go through a
// deterministic f64 grid reduction.
//
// Sparse / OrderedSparse lists: one thread per stored pair, forces scattered
// with float4 atomics (sm_90+), as the gradient of sum_pairs U / norm.
#include "pair.cuh"

namespace jmd {

PairTable make_pair_table(const jmd_pair& pp) {
  PairTable t;
  memset(&t, 0, sizeof(t));
  t.kind = pp.kind;
  t.nsp = pp.n_species;
  int S = pp.n_species > 0 ? pp.n_species : 1;
  float maxs = 0.f;
  for (int a = 0; a < S; ++a)
    for (int b = 0; b < S; ++b) maxs = std::max(maxs, pp.sigma[a][b]);
  t.rc2_max = 0.f;
  for (int a = 0; a < S; ++a) {
    for (int b = 0; b < S; ++b) {
      PairCoef& c = t.c[a * JMD_MAX_SPECIES + b];
      float sig = pp.sigma[a][b];
      c.sig2 = sig * sig;
      c.eps = pp.epsilon[a][b];
      c.alpha = pp.alpha[a][b];
      c.inv_sig = 1.0f / sig;
      c.pad = sig;
      if (pp.kind == JMD_SOFT_SPHERE) {
        c.rc2 = sig * sig;
        c.ro2 = c.rc2;
        c.inv_den = 0.f;
      } else {
        float ro = pp.r_onset, rc = pp.r_cutoff;
        if (pp.per_pair_cutoff && maxs > 0.f) {
          ro = pp.r_onset * sig / maxs;
          rc = pp.r_cutoff * sig / maxs;
        }
        c.ro2 = ro * ro;
        c.rc2 = rc * rc;
        double den = (double)c.rc2 - (double)c.ro2;
        c.inv_den = den > 0 ? (float)(1.0 / (den * den * den)) : 0.f;
        if (pp.kind == JMD_LJ_TRUNCATED) c.ro2 = c.rc2;
      }
      t.rc2_max = std::max(t.rc2_max, c.rc2);
    }
  }
  t.psig = pp.particle_sigma;
  t.peps = pp.particle_epsilon;
  t.per_pair_cutoff = pp.per_pair_cutoff;
  t.maxs = maxs;
  t.r_onset = pp.r_onset;
  t.r_cutoff = pp.r_cutoff;
  return t;
}

namespace {

struct DenseArgs {
  const float* x;
  int64_t xs;
  const int32_t* species;
  int n;
  const int32_t* idx;
  int64_t ld;
  int64_t width;
  const int32_t* cnt;
  float* f;
  int64_t fs;
  float* e_atom;
  double* energy;
  double* virial;
  double* partials;
  unsigned int* counter;
  double* totals;
  Geo geo;
};

// Species index clamped into the table (JAX clamps out-of-range gathers too).
__device__ __forceinline__ int sp_clamp(int s, int nsp) {
  return s < 0 ? 0 : (s >= nsp ? nsp - 1 : s);
}

template <int TPA, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = TPA / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// EV: also energy, per-atom energy and virial.
template <int DIM, int TPA, int KIND, bool SPECIES, bool EV, bool VEC4>
__global__ void __launch_bounds__(256) k_pair_dense(DenseArgs a, const __grid_constant__ PairTable tab) {
  __shared__ PairCoef sc[SPECIES ? JMD_MAX_SPECIES * JMD_MAX_SPECIES : 1];
  if (SPECIES) {
    for (int k = threadIdx.x; k < JMD_MAX_SPECIES * JMD_MAX_SPECIES; k += blockDim.x) sc[k] = tab.c[k];
    __syncthreads();
  }
  const int64_t gt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t atom = gt / TPA;
  const int sub = threadIdx.x & (TPA - 1);
  const bool active = atom < a.n;
  float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
  float w0 = 0.f, w1 = 0.f, w2 = 0.f, w3 = 0.f, w4 = 0.f, w5 = 0.f;
  if (active) {
    const float4 xi = load_row<DIM, VEC4>(a.x, a.xs, atom);
    const int si = SPECIES ? sp_clamp(__ldg(a.species + atom), tab.nsp) : 0;
    const int32_t* row = a.idx + atom * a.ld;
    int64_t end = a.width;
    if (a.cnt) end = min((int64_t)__ldg(a.cnt + atom), a.width);
    const float rc2m = tab.rc2_max;
    for (int64_t k = sub; k < end; k += TPA) {
      const int j = __ldcs(row + k);
      if ((unsigned)j >= (unsigned)a.n) continue;
      const float4 xj = load_row<DIM, VEC4>(a.x, a.xs, j);
      float dx, dy, dz;
      displacement<DIM>(xi, xj, a.geo, dx, dy, dz);  // R_i - R_j
      float r2 = dx * dx;
      r2 = fmaf(dy, dy, r2);
      if (DIM == 3) r2 = fmaf(dz, dz, r2);
      if (!(r2 < rc2m) || r2 == 0.f) continue;
      const bool part = !SPECIES && (tab.psig != nullptr || tab.peps != nullptr);
      const PairCoef c = SPECIES ? sc[si * JMD_MAX_SPECIES + sp_clamp(__ldg(a.species + j), tab.nsp)]
                                 : (part ? particle_coef(tab, (int)atom, j) : tab.c[0]);
      if ((SPECIES || part) && !(r2 < c.rc2)) continue;
      float U, g, h;
      pair_eval<KIND, false>(r2, c, U, g, h);
      // F_i = -U'(r)/r (R_i - R_j)
      fx = fmaf(-g, dx, fx);
      fy = fmaf(-g, dy, fy);
      if (DIM == 3) fz = fmaf(-g, dz, fz);
      if (EV) {
        e += U;
        w0 = fmaf(g * dx, dx, w0);
        w1 = fmaf(g * dy, dy, w1);
        if (DIM == 3) {
          w2 = fmaf(g * dz, dz, w2);
          w3 = fmaf(g * dx, dy, w3);
          w4 = fmaf(g * dx, dz, w4);
          w5 = fmaf(g * dy, dz, w5);
        } else {
          w3 = fmaf(g * dx, dy, w3);
        }
      }
    }
  }
  fx = group_sum<TPA>(fx);
  fy = group_sum<TPA>(fy);
  if (DIM == 3) fz = group_sum<TPA>(fz);
  if (EV) {
    e = group_sum<TPA>(e);
    w0 = group_sum<TPA>(w0);
    w1 = group_sum<TPA>(w1);
    w2 = group_sum<TPA>(w2);
    w3 = group_sum<TPA>(w3);
    w4 = group_sum<TPA>(w4);
    w5 = group_sum<TPA>(w5);
  }
  const bool leader = active && sub == 0;
  if (leader && a.f) store_row_full<DIM, VEC4>(a.f, a.fs, atom, make_float4(fx, fy, fz, 0.f));
  if (EV) {
    if (leader && a.e_atom) a.e_atom[atom] = 0.5f * e;
    double v[7];
    v[0] = leader ? 0.5 * (double)e : 0.0;
    v[1] = leader ? 0.5 * (double)w0 : 0.0;
    v[2] = leader ? 0.5 * (double)w1 : 0.0;
    v[3] = leader ? 0.5 * (double)w2 : 0.0;
    v[4] = leader ? 0.5 * (double)w3 : 0.0;
    v[5] = leader ? 0.5 * (double)w4 : 0.0;
    v[6] = leader ? 0.5 * (double)w5 : 0.0;
    grid_reduce<7>(v, a.partials, a.counter, a.totals, false);
  }
}

// Copies grid-reduced totals to the caller's energy / virial slots.
__global__ void k_emit_totals(const double* totals, double* energy, double* virial, int dim) {
  if (threadIdx.x != 0) return;
  if (energy) *energy = totals[0];
  if (virial) {
    if (dim == 3) {
      for (int k = 0; k < 6; ++k) virial[k] = totals[1 + k];
    } else {
      virial[0] = totals[1];
      virial[1] = totals[2];
      virial[2] = totals[4];
    }
  }
}

template <int DIM, bool VEC4>
__global__ void k_zero_rows(float* f, int64_t fs, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) store_row_full<DIM, VEC4>(f, fs, i, make_float4(0.f, 0.f, 0.f, 0.f));
}

__global__ void k_zero_f(float* p, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.f;
}

template <int DIM, bool VEC4>
__device__ __forceinline__ void add_row(float* f, int64_t fs, int i, float x, float y, float z) {
  if (VEC4) {
    atomicAdd(reinterpret_cast<float4*>(f) + i, make_float4(x, y, z, 0.f));
  } else {
    atomicAdd(f + i * fs, x);
    atomicAdd(f + i * fs + 1, y);
    if (DIM == 3) atomicAdd(f + i * fs + 2, z);
  }
}

struct SparseArgs {
  const float* x;
  int64_t xs;
  const int32_t* species;
  int n;
  const int32_t* idx;  // [2, ld]: row 0 receivers, row 1 senders
  int64_t ld;
  int64_t width;
  float inv_norm;      // 1/2 Sparse, 1 OrderedSparse
  float* f;
  int64_t fs;
  float* e_atom;
  double* partials;
  unsigned int* counter;
  double* totals;
  Geo geo;
};

template <int DIM, int KIND, bool SPECIES, bool EV, bool VEC4, bool FVEC4>
__global__ void __launch_bounds__(256) k_pair_sparse(SparseArgs a, const __grid_constant__ PairTable tab) {
  __shared__ PairCoef sc[SPECIES ? JMD_MAX_SPECIES * JMD_MAX_SPECIES : 1];
  if (SPECIES) {
    for (int k = threadIdx.x; k < JMD_MAX_SPECIES * JMD_MAX_SPECIES; k += blockDim.x) sc[k] = tab.c[k];
    __syncthreads();
  }
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float e = 0.f, w0 = 0.f, w1 = 0.f, w2 = 0.f, w3 = 0.f, w4 = 0.f, w5 = 0.f;
  if (p < a.width) {
    const int j = __ldg(a.idx + p);
    const int i = __ldg(a.idx + a.ld + p);
    if ((unsigned)j < (unsigned)a.n && (unsigned)i < (unsigned)a.n) {
      const float4 xj = load_row<DIM, VEC4>(a.x, a.xs, j);
      const float4 xi = load_row<DIM, VEC4>(a.x, a.xs, i);
      float dx, dy, dz;
      displacement<DIM>(xj, xi, a.geo, dx, dy, dz);  // R_j - R_i (smap.py:937)
      float r2 = dx * dx;
      r2 = fmaf(dy, dy, r2);
      if (DIM == 3) r2 = fmaf(dz, dz, r2);
      const bool part = !SPECIES && (tab.psig != nullptr || tab.peps != nullptr);
      const PairCoef c = SPECIES ? sc[sp_clamp(__ldg(a.species + i), tab.nsp) * JMD_MAX_SPECIES +
                                      sp_clamp(__ldg(a.species + j), tab.nsp)]
                                 : (part ? particle_coef(tab, i, j) : tab.c[0]);
      if (r2 < c.rc2 && r2 > 0.f) {
        float U, g, h;
        pair_eval<KIND, false>(r2, c, U, g, h);
        g *= a.inv_norm;
        if (a.f) {
          add_row<DIM, FVEC4>(a.f, a.fs, j, -g * dx, -g * dy, -g * dz);
          add_row<DIM, FVEC4>(a.f, a.fs, i, g * dx, g * dy, g * dz);
        }
        if (EV) {
          e = U * a.inv_norm;
          if (a.e_atom) atomicAdd(a.e_atom + j, e);
          w0 = g * dx * dx;
          w1 = g * dy * dy;
          w2 = g * dz * dz;
          w3 = g * dx * dy;
          w4 = g * dx * dz;
          w5 = g * dy * dz;
        }
      }
    }
  }
  if (EV) {
    double v[7] = {e, w0, w1, w2, w3, w4, w5};
    grid_reduce<7>(v, a.partials, a.counter, a.totals, false);
  }
}

struct PairWs {
  double* partials;
  unsigned int* counter;
  double* totals;
};

constexpr int64_t kMaxPairBlocks = 1 << 20;

size_t pair_ws_bytes(int64_t n) {
  (void)n;
  Carver cv(nullptr, 0);
  cv.take<double>(kMaxPairBlocks * 7);
  cv.take<unsigned int>(1);
  cv.take<double>(8);
  return cv.used + 256;
}

template <int DIM, int TPA, int KIND, bool SPECIES, bool EV, bool VEC4>
void launch_dense(const DenseArgs& a, const PairTable& t, cudaStream_t st) {
  int64_t threads = (int64_t)a.n * TPA;
  unsigned grid = (unsigned)std::max<int64_t>(1, ceil_div(threads, 256));
  k_pair_dense<DIM, TPA, KIND, SPECIES, EV, VEC4><<<grid, 256, 0, st>>>(a, t);
}

template <int DIM, int TPA, int KIND, bool SPECIES, bool VEC4>
void dispatch_ev(bool ev, const DenseArgs& a, const PairTable& t, cudaStream_t st) {
  if (ev) launch_dense<DIM, TPA, KIND, SPECIES, true, VEC4>(a, t, st);
  else launch_dense<DIM, TPA, KIND, SPECIES, false, VEC4>(a, t, st);
}

template <int DIM, int TPA, int KIND, bool VEC4>
void dispatch_sp(bool species, bool ev, const DenseArgs& a, const PairTable& t, cudaStream_t st) {
  if (species) dispatch_ev<DIM, TPA, KIND, true, VEC4>(ev, a, t, st);
  else dispatch_ev<DIM, TPA, KIND, false, VEC4>(ev, a, t, st);
}

template <int DIM, int TPA, bool VEC4>
void dispatch_kind(int kind, bool species, bool ev, const DenseArgs& a, const PairTable& t,
                   cudaStream_t st) {
  if (kind == JMD_LJ) dispatch_sp<DIM, TPA, JMD_LJ, VEC4>(species, ev, a, t, st);
  else if (kind == JMD_LJ_TRUNCATED) dispatch_sp<DIM, TPA, JMD_LJ_TRUNCATED, VEC4>(species, ev, a, t, st);
  else if (kind == JMD_MORSE) dispatch_sp<DIM, TPA, JMD_MORSE, VEC4>(species, ev, a, t, st);
  else dispatch_sp<DIM, TPA, JMD_SOFT_SPHERE, VEC4>(species, ev, a, t, st);
}

template <int DIM, bool VEC4>
void dispatch_tpa(int tpa, int kind, bool species, bool ev, const DenseArgs& a, const PairTable& t,
                  cudaStream_t st) {
  switch (tpa) {
    case 4: dispatch_kind<DIM, 4, VEC4>(kind, species, ev, a, t, st); break;
    case 8: dispatch_kind<DIM, 8, VEC4>(kind, species, ev, a, t, st); break;
    case 16: dispatch_kind<DIM, 16, VEC4>(kind, species, ev, a, t, st); break;
    default: dispatch_kind<DIM, 32, VEC4>(kind, species, ev, a, t, st); break;
  }
}

template <int DIM, int KIND, bool SPECIES, bool EV>
void launch_sparse(bool v4, bool fv4, const SparseArgs& a, const PairTable& t, cudaStream_t st) {
  unsigned grid = (unsigned)std::max<int64_t>(1, ceil_div(a.width, 256));
  if (v4 && fv4) k_pair_sparse<DIM, KIND, SPECIES, EV, true, true><<<grid, 256, 0, st>>>(a, t);
  else if (v4) k_pair_sparse<DIM, KIND, SPECIES, EV, true, false><<<grid, 256, 0, st>>>(a, t);
  else if (fv4) k_pair_sparse<DIM, KIND, SPECIES, EV, false, true><<<grid, 256, 0, st>>>(a, t);
  else k_pair_sparse<DIM, KIND, SPECIES, EV, false, false><<<grid, 256, 0, st>>>(a, t);
}

template <int DIM, int KIND>
void sparse_sp(bool species, bool ev, bool v4, bool fv4, const SparseArgs& a, const PairTable& t,
               cudaStream_t st) {
  if (species) {
    if (ev) launch_sparse<DIM, KIND, true, true>(v4, fv4, a, t, st);
    else launch_sparse<DIM, KIND, true, false>(v4, fv4, a, t, st);
  } else {
    if (ev) launch_sparse<DIM, KIND, false, true>(v4, fv4, a, t, st);
    else launch_sparse<DIM, KIND, false, false>(v4, fv4, a, t, st);
  }
}

template <int DIM>
void sparse_kind(int kind, bool species, bool ev, bool v4, bool fv4, const SparseArgs& a,
                 const PairTable& t, cudaStream_t st) {
  if (kind == JMD_LJ) sparse_sp<DIM, JMD_LJ>(species, ev, v4, fv4, a, t, st);
  else if (kind == JMD_LJ_TRUNCATED) sparse_sp<DIM, JMD_LJ_TRUNCATED>(species, ev, v4, fv4, a, t, st);
  else if (kind == JMD_MORSE) sparse_sp<DIM, JMD_MORSE>(species, ev, v4, fv4, a, t, st);
  else sparse_sp<DIM, JMD_SOFT_SPHERE>(species, ev, v4, fv4, a, t, st);
}

int g_default_tpa = 8;
bool g_force_generic = false;

}  // namespace

int validate_pair(const jmd_pair* pp, bool allow_particle) {
  JMD_REQUIRE(pp != nullptr, "pair parameters are null");
  const bool particle = pp->particle_sigma != nullptr || pp->particle_epsilon != nullptr;
  JMD_REQUIRE(allow_particle || !particle,
              "per-particle parameters run on jmd_pair_forces (the generic pair kernels) only");
  JMD_REQUIRE(!particle || pp->n_species == 0, "per-particle parameters exclude species matrices");
  JMD_REQUIRE(pp->kind >= 0 && pp->kind <= 3, "unknown pair potential");
  JMD_REQUIRE(pp->n_species >= 0 && pp->n_species <= JMD_MAX_SPECIES, "n_species out of range");
  int S = pp->n_species > 0 ? pp->n_species : 1;
  for (int a = 0; a < S; ++a)
    for (int b = 0; b < S; ++b) JMD_REQUIRE(pp->sigma[a][b] > 0.f, "sigma must be positive");
  if (pp->kind != JMD_SOFT_SPHERE)
    JMD_REQUIRE(pp->r_cutoff > 0.f && pp->r_onset <= pp->r_cutoff, "need 0 < r_onset <= r_cutoff");
  JMD_REQUIRE(pp->kind != JMD_MORSE || !pp->per_pair_cutoff,
              "Morse radii are absolute (per_pair_cutoff must be 0)");
  return JMD_OK;
}

}  // namespace jmd

using namespace jmd;

extern "C" {

size_t jmd_pair_workspace_bytes(int64_t n) { return pair_ws_bytes(n); }

int jmd_set_pair_generic(int generic) {
  g_force_generic = generic != 0;
  return JMD_OK;
}

int jmd_set_pair_threads_per_atom(int tpa) {
  JMD_REQUIRE(tpa == 4 || tpa == 8 || tpa == 16 || tpa == 32, "threads per atom must be 4, 8, 16 or 32");
  g_default_tpa = tpa;
  return JMD_OK;
}

int jmd_pair_forces(const jmd_pair* pp, const jmd_space* space, int32_t format,
                    const float* position, int64_t pos_stride, const int32_t* species, int64_t n,
                    const int32_t* idx, int64_t idx_ld, int64_t idx_width,
                    const int32_t* nbr_count, float* force, int64_t force_stride, double* energy,
                    float* per_atom_energy, double* virial, void* workspace,
                    size_t workspace_bytes, void* stream) {
  int e = validate_pair(pp, true);
  if (e) return e;
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(n >= 0 && n < INT32_MAX, "atom count out of range");
  JMD_REQUIRE(format >= 0 && format <= 2, "unknown format");
  const bool particle = pp->particle_sigma != nullptr || pp->particle_epsilon != nullptr;
  JMD_REQUIRE(!(format == JMD_ORDERED_SPARSE && per_atom_energy),
              "per-particle energies are not defined for OrderedSparse lists");
  JMD_REQUIRE(idx_width >= 0 && idx_ld >= idx_width, "idx_ld must be >= idx_width");
  JMD_REQUIRE(pp->n_species == 0 || species != nullptr, "species matrices need a species array");
  cudaStream_t st = as_stream(stream);
  const bool ev = energy || per_atom_energy || virial;
  Carver cv(workspace, workspace_bytes);
  PairWs w;
  w.partials = cv.take<double>(kMaxPairBlocks * 7);
  w.counter = cv.take<unsigned int>(1);
  w.totals = cv.take<double>(8);
  if (ev && !cv.ok()) return fail(JMD_ERR_WORKSPACE, "pair workspace too small");
  // the grid reduction needs a zero block counter; the workspace may hold
  // anything (callers pass uninitialised scratch)
  if (ev) JMD_CUDA(cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), st));
  PairTable t = make_pair_table(*pp);
  const bool sp = pp->n_species > 0;
  const int dim = space->dim;
  const bool v4 = is_vec4(position, pos_stride);
  Geo geo = make_geo(*space);
  if (format == JMD_DENSE) {
    DenseArgs a;
    a.x = position;
    a.xs = pos_stride;
    a.species = species;
    a.n = (int)n;
    a.idx = idx;
    a.ld = idx_ld;
    a.width = idx_width;
    a.cnt = nbr_count;
    a.f = force;
    a.fs = force_stride;
    a.e_atom = per_atom_energy;
    a.energy = energy;
    a.virial = virial;
    a.partials = w.partials;
    a.counter = w.counter;
    a.totals = w.totals;
    a.geo = geo;
    const bool fast = !g_force_generic && !particle && !geo.general &&
                      dense2_applicable(position, pos_stride, idx, idx_ld, force, force_stride);
    // lanes per atom of the kernel that will run (the packed path uses its
    // own width, 8 for Morse): one partial per block must fit the workspace
    const int tpa = !fast ? g_default_tpa : (pp->kind == JMD_MORSE ? 8 : dense_tpa());
    if (ev && ceil_div(n * tpa, 256) > kMaxPairBlocks)
      return fail(JMD_ERR_UNSUPPORTED, "system too large for the energy reduction");
    if (fast) {
      int rc = dense2_forces(pp, space, position, species, n, idx, idx_ld, idx_width, nbr_count,
                             force, energy, per_atom_energy, virial, w.partials, w.counter,
                             w.totals, st);
      if (rc) return rc;
    } else if (n > 0) {
      const bool fv4 = force == nullptr || is_vec4(force, force_stride);
      if (dim == 3) {
        if (v4 && fv4) dispatch_tpa<3, true>(tpa, pp->kind, sp, ev, a, t, st);
        else dispatch_tpa<3, false>(tpa, pp->kind, sp, ev, a, t, st);
      } else {
        if (v4 && fv4) dispatch_tpa<2, true>(tpa, pp->kind, sp, ev, a, t, st);
        else dispatch_tpa<2, false>(tpa, pp->kind, sp, ev, a, t, st);
      }
    }
    if (ev) {
      if (n == 0) {
        // no atoms: totals are zero
        JMD_CUDA(cudaMemsetAsync(w.totals, 0, 8 * sizeof(double), st));
      }
      k_emit_totals<<<1, 32, 0, st>>>(w.totals, energy, virial, dim);
    }
  } else {
    SparseArgs a;
    a.x = position;
    a.xs = pos_stride;
    a.species = species;
    a.n = (int)n;
    a.idx = idx;
    a.ld = idx_ld;
    a.width = idx_width;
    a.inv_norm = format == JMD_ORDERED_SPARSE ? 1.0f : 0.5f;
    a.f = force;
    a.fs = force_stride;
    a.e_atom = per_atom_energy;
    a.partials = w.partials;
    a.counter = w.counter;
    a.totals = w.totals;
    a.geo = geo;
    if (ev && ceil_div(idx_width, 256) > kMaxPairBlocks)
      return fail(JMD_ERR_UNSUPPORTED, "pair list too large for the energy reduction");
    const bool fv4 = force != nullptr && is_vec4(force, force_stride);
    if (n > 0) {
      unsigned gr = (unsigned)ceil_div(n, 256);
      if (force) {
        if (dim == 3) {
          if (fv4) k_zero_rows<3, true><<<gr, 256, 0, st>>>(force, force_stride, (int)n);
          else k_zero_rows<3, false><<<gr, 256, 0, st>>>(force, force_stride, (int)n);
        } else {
          if (fv4) k_zero_rows<2, true><<<gr, 256, 0, st>>>(force, force_stride, (int)n);
          else k_zero_rows<2, false><<<gr, 256, 0, st>>>(force, force_stride, (int)n);
        }
      }
      if (per_atom_energy) k_zero_f<<<gr, 256, 0, st>>>(per_atom_energy, (int)n);
    }
    if (idx_width > 0) {
      if (dim == 3) sparse_kind<3>(pp->kind, sp, ev, v4, fv4, a, t, st);
      else sparse_kind<2>(pp->kind, sp, ev, v4, fv4, a, t, st);
    } else if (ev) {
      JMD_CUDA(cudaMemsetAsync(w.totals, 0, 8 * sizeof(double), st));
    }
    if (ev) k_emit_totals<<<1, 32, 0, st>>>(w.totals, energy, virial, dim);
  }
  return check_launch("jmd_pair_forces");
}

}  // extern "C"
