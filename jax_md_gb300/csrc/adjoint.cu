// Adjoint of the pair force and of velocity Verlet.
//
// Reference: the forces of jax_md/smap.py:922-979 + quantity.py:58-60 and
// their derivatives as jax.grad would take them, including the dependence of
// the LJ cutoff radii on sigma (energy.py:319-320: r_onset = 2 max(sigma),
// r_cutoff = 2.5 max(sigma)); velocity Verlet of simulate.py:227-243.
//
// With d = R_k - R_j, g = U'(r)/r, the force is F_k = -sum_j g d and its
// Jacobian blocks are J = g I + ((U'' - g)/r^2) d d^T.  For a symmetric
// (Dense, full) list the VJP with cotangent lam is
//   gR_k = sum_{j in N(k)} J_kj (lam_j - lam_k)
// (each atom sums its own row, no atomics on positions).  A Dense entry (k, j)
// carries half of the pair energy with the parameters of (s_k, s_j), so the
// parameter gradient of L = lam . F per entry is
//   dL/d theta[s_k][s_j] += 1/2 (dg/d theta) (lam_j - lam_k) . d.
#include "adjoint.cuh"

namespace jmd {
namespace {

// ------------------------------------------------- generic-stride VJP kernel --
struct VjpArgs {
  const float* x;
  int64_t xs;
  const int32_t* species;
  int n;
  const int32_t* idx;
  int64_t ld;
  int64_t width;
  const int32_t* cnt;
  const float* lam;
  int64_t ls;
  float* gx;
  int64_t gs;
  float weight;
  double* gp;      // [kBins] dL/dtheta (accumulated, times weight)
  double* ge;      // [kBins] dE/dtheta (accumulated), optional
  Geo geo;
  int per_pair;    // cutoff scales with sigma_ij
};

// One thread per atom over a row-major Dense list of any stride.
template <int DIM, int KIND, bool SPECIES, bool EGRAD>
__global__ void __launch_bounds__(128) k_force_vjp(VjpArgs a, const __grid_constant__ PairTable tab,
                                                  const __grid_constant__ PairTable sig) {
  constexpr int NB = SPECIES ? JMD_MAX_SPECIES : 1;
  __shared__ float bins[kBins];
  __shared__ float ebins[EGRAD ? kBins : 1];
  zero_bins(bins);
  if (EGRAD) zero_bins(ebins);
  __syncthreads();
  BinAcc<NB> acc, eacc;
  acc.zero();
  eacc.zero();
  const bool per_pair = a.per_pair != 0;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  int sk = 0;
  if (k < a.n) {
    const float4 xk = load_row<DIM, false>(a.x, a.xs, k);
    const float4 lk = load_row<DIM, false>(a.lam, a.ls, k);
    sk = SPECIES ? min(max(__ldg(a.species + k), 0), tab.nsp - 1) : 0;
    const int32_t* row = a.idx + (int64_t)k * a.ld;
    int end = (int)a.width;
    if (a.cnt) end = min(__ldg(a.cnt + k), end);
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int e = 0; e < end; ++e) {
      const int j = __ldg(row + e);
      if ((unsigned)j >= (unsigned)a.n) continue;
      const float4 xj = load_row<DIM, false>(a.x, a.xs, j);
      float dx, dy, dz;
      displacement<DIM>(xk, xj, a.geo, dx, dy, dz);
      const float r2 = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f);
      const int sj = SPECIES ? min(max(__ldg(a.species + j), 0), tab.nsp - 1) : 0;
      const int bin = sk * JMD_MAX_SPECIES + sj;
      const PairCoef& c = tab.c[SPECIES ? bin : 0];
      if (!(r2 < c.rc2) || r2 == 0.f) continue;
      const float sigma = sig.c[SPECIES ? bin : 0].pad;   // sigma_ij
      const float kappa = per_pair ? sigma : sig.pad;     // cutoff scale
      const PairD q = pair_derivs<KIND>(r2, c, sigma, kappa);
      const float4 lj = load_row<DIM, false>(a.lam, a.ls, j);
      const float ex = lj.x - lk.x, ey = lj.y - lk.y, ez = DIM == 3 ? lj.z - lk.z : 0.f;
      const float t = dx * ex + dy * ey + dz * ez;     // (lam_j - lam_k) . d
      const float cdd = (q.hh - q.g) / r2 * t;
      gx += q.g * ex + cdd * dx;
      gy += q.g * ey + cdd * dy;
      if (DIM == 3) gz += q.g * ez + cdd * dz;
      const float ht = 0.5f * t;
      acc.add(sj, q.dg_s * ht, q.dg_e * ht, KIND == JMD_LJ ? q.dg_k * ht : 0.f, per_pair);
      if (EGRAD)
        eacc.add(sj, 0.5f * q.dU_s, 0.5f * q.dU_e, KIND == JMD_LJ ? 0.5f * q.dU_k : 0.f, per_pair);
    }
    if (a.gx) {
      float* o = a.gx + (int64_t)k * a.gs;
      o[0] += a.weight * gx;
      o[1] += a.weight * gy;
      if (DIM == 3) o[2] += a.weight * gz;
    }
  }
  const int ncol = SPECIES ? tab.nsp : 1;
  if (!SPECIES) {
    acc.group_sum(kWarp, 1);
    if (EGRAD) eacc.group_sum(kWarp, 1);
  }
  if (SPECIES || (threadIdx.x & (kWarp - 1)) == 0) {
    acc.flush(bins, sk, ncol);
    if (EGRAD) eacc.flush(ebins, sk, ncol);
  }
  __syncthreads();
  publish_bins(bins, a.gp, (double)a.weight);
  if (EGRAD) publish_bins(ebins, a.ge, 1.0);
}

template <int DIM, int KIND>
void vjp_launch(bool sp, bool eg, const VjpArgs& a, const PairTable& t, const PairTable& s,
                cudaStream_t st) {
  const unsigned grid = (unsigned)std::max<int64_t>(1, ceil_div(a.n, 128));
  if (sp) {
    if (eg) k_force_vjp<DIM, KIND, true, true><<<grid, 128, 0, st>>>(a, t, s);
    else k_force_vjp<DIM, KIND, true, false><<<grid, 128, 0, st>>>(a, t, s);
  } else {
    if (eg) k_force_vjp<DIM, KIND, false, true><<<grid, 128, 0, st>>>(a, t, s);
    else k_force_vjp<DIM, KIND, false, false><<<grid, 128, 0, st>>>(a, t, s);
  }
}

// ----------------------------------------------- engine reverse-step kernels --
// A reverse Verlet step at x_s takes two kernels:
//   pack:  q = pbar + (dt/m) xbar  (pbar <- q), record[i] = (x_i, q_i) in 32
//          bytes, and the skin test of x_s against the list's reference;
//   step:  xbar_k += w sum_j J_kj (q_j - q_k) over k's Dense row, TPA lanes
//          per atom, each neighbour one 32-byte record gather.
// The closing half kick at the end of a run is a pack without the kick
// (q = pbar) followed by a step with w = dt/2.

template <int DIM>
__global__ void __launch_bounds__(256) k_adj_pack(int n, const float4* __restrict__ x,
                                                  float4* __restrict__ xbar, float4* __restrict__ pbar,
                                                  const float* __restrict__ mass, float mass_scalar,
                                                  float dt, int kick, float4* __restrict__ rec,
                                                  const float4* __restrict__ ref, float thr2,
                                                  int32_t* flag, Geo geo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (i < n) {
    const float4 xi = __ldg(x + i);
    float4 q = pbar[i];
    if (kick) {
      const float4 xb = xbar[i];
      const float c = dt / (mass ? __ldg(mass + i) : mass_scalar);
      q.x = fmaf(c, xb.x, q.x);
      q.y = fmaf(c, xb.y, q.y);
      if (DIM == 3) q.z = fmaf(c, xb.z, q.z);
      pbar[i] = q;
    }
    rec[2 * i] = make_float4(xi.x, xi.y, DIM == 3 ? xi.z : 0.f, q.x);
    rec[2 * i + 1] = make_float4(q.y, DIM == 3 ? q.z : 0.f, 0.f, 0.f);
    if (ref) {
      float dx, dy, dz;
      displacement<DIM>(xi, __ldg(ref + i), geo, dx, dy, dz);
      over = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f) > thr2;
    }
  }
  if (ref && __any_sync(0xffffffffu, over) && (threadIdx.x & (kWarp - 1)) == 0) atomicOr(flag, 1);
}

struct StepArgs {
  int n;
  const float4* rec;
  float4* xbar;
  const int32_t* species;
  const int32_t* idx;
  int64_t ld;
  int width;
  const int32_t* cnt;
  float weight;
  double* gp;
  Geo geo;
  int per_pair;
};

template <int DIM, int KIND, bool SPECIES, bool PARAMS, int TPA>
__global__ void __launch_bounds__(256) k_adj_step(StepArgs a, const __grid_constant__ PairTable tab,
                                                  const __grid_constant__ PairTable sig) {
  constexpr int NB = SPECIES ? JMD_MAX_SPECIES : 1;
  __shared__ float bins[PARAMS ? kBins : 1];
  if (PARAMS) {
    zero_bins(bins);
    __syncthreads();
  }
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int k = (int)(t / TPA);
  const int lane = (int)(t % TPA);
  const bool active = k < a.n;
  const bool per_pair = a.per_pair != 0;
  BinAcc<NB> acc;
  acc.zero();
  float gx = 0.f, gy = 0.f, gz = 0.f;
  int sk = 0;
  if (active) {
    const float4 r0 = __ldg(a.rec + 2 * k);
    const float4 r1 = __ldg(a.rec + 2 * k + 1);
    const float qx = r0.w, qy = r1.x, qz = r1.y;
    sk = SPECIES ? min(max(__ldg(a.species + k), 0), tab.nsp - 1) : 0;
    const int32_t* row = a.idx + (int64_t)k * a.ld;
    int end = a.width;
    if (a.cnt) end = min(__ldg(a.cnt + k), end);
    for (int e = lane; e < end; e += TPA) {
      const int j = __ldg(row + e);
      if ((unsigned)j >= (unsigned)a.n) continue;
      const float4 j0 = __ldg(a.rec + 2 * j);
      const float4 j1 = __ldg(a.rec + 2 * j + 1);
      float dx, dy, dz;
      displacement<DIM>(r0, j0, a.geo, dx, dy, dz);
      const float r2 = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f);
      const int sj = SPECIES ? min(max(__ldg(a.species + j), 0), tab.nsp - 1) : 0;
      const int bin = sk * JMD_MAX_SPECIES + sj;
      const PairCoef& c = tab.c[SPECIES ? bin : 0];
      if (!(r2 < c.rc2) || r2 == 0.f) continue;
      float g, hh;
      PairD q;
      if (PARAMS) {
        const float sigma = sig.c[SPECIES ? bin : 0].pad;
        q = pair_derivs<KIND>(r2, c, sigma, per_pair ? sigma : sig.pad);
        g = q.g;
        hh = q.hh;
      } else {
        float U;
        pair_eval<KIND, true>(r2, c, U, g, hh);
      }
      const float ex = j0.w - qx, ey = j1.x - qy, ez = DIM == 3 ? j1.y - qz : 0.f;
      const float tt = dx * ex + dy * ey + dz * ez;    // (q_j - q_k) . d
      const float cdd = (hh - g) * rcp_nr(r2) * tt;
      gx = fmaf(g, ex, fmaf(cdd, dx, gx));
      gy = fmaf(g, ey, fmaf(cdd, dy, gy));
      if (DIM == 3) gz = fmaf(g, ez, fmaf(cdd, dz, gz));
      if (PARAMS) {
        const float ht = 0.5f * tt;
        acc.add(sj, q.dg_s * ht, q.dg_e * ht, KIND == JMD_LJ ? q.dg_k * ht : 0.f, per_pair);
      }
    }
  }
#pragma unroll
  for (int o = TPA / 2; o > 0; o >>= 1) {
    gx += __shfl_xor_sync(0xffffffffu, gx, o, TPA);
    gy += __shfl_xor_sync(0xffffffffu, gy, o, TPA);
    if (DIM == 3) gz += __shfl_xor_sync(0xffffffffu, gz, o, TPA);
  }
  if (active && lane == 0) {
    float4 b = a.xbar[k];
    b.x = fmaf(a.weight, gx, b.x);
    b.y = fmaf(a.weight, gy, b.y);
    if (DIM == 3) b.z = fmaf(a.weight, gz, b.z);
    a.xbar[k] = b;
  }
  if (PARAMS) {
    const int ncol = SPECIES ? tab.nsp : 1;
    if (SPECIES) {
      acc.group_sum(TPA, ncol);
      if (active && lane == 0) acc.flush(bins, sk, ncol);
    } else {
      acc.group_sum(kWarp, 1);
      if ((threadIdx.x & (kWarp - 1)) == 0) acc.flush(bins, 0, 1);
    }
    __syncthreads();
    publish_bins(bins, a.gp, (double)a.weight);
  }
}

template <int DIM, int KIND, bool SPECIES, bool PARAMS>
void step_launch_tpa(int tpa, const StepArgs& a, const PairTable& t, const PairTable& s,
                     cudaStream_t st) {
  const unsigned grid = (unsigned)std::max<int64_t>(1, ceil_div((int64_t)a.n * tpa, 256));
  if (tpa == 4) k_adj_step<DIM, KIND, SPECIES, PARAMS, 4><<<grid, 256, 0, st>>>(a, t, s);
  else if (tpa == 16) k_adj_step<DIM, KIND, SPECIES, PARAMS, 16><<<grid, 256, 0, st>>>(a, t, s);
  else k_adj_step<DIM, KIND, SPECIES, PARAMS, 8><<<grid, 256, 0, st>>>(a, t, s);
}

template <int DIM, int KIND>
void step_launch(int tpa, bool sp, bool params, const StepArgs& a, const PairTable& t,
                 const PairTable& s, cudaStream_t st) {
  if (sp) {
    if (params) step_launch_tpa<DIM, KIND, true, true>(tpa, a, t, s, st);
    else step_launch_tpa<DIM, KIND, true, false>(tpa, a, t, s, st);
  } else {
    if (params) step_launch_tpa<DIM, KIND, false, true>(tpa, a, t, s, st);
    else step_launch_tpa<DIM, KIND, false, false>(tpa, a, t, s, st);
  }
}

// ------------------------------------------------------ Sparse-list VJP --
// One thread per entry of a Sparse / OrderedSparse list (idx[0] receivers j,
// idx[1] senders i, smap.py:967-977): the entry carries c = 1/2 (Sparse) or
// 1 (OrderedSparse) of the pair energy with the parameters of (s_i, s_j), so
//   gR_i += c J (lam_j - lam_i),  gR_j -= c J (lam_j - lam_i)   (atomics)
//   dL/d theta[s_i][s_j] += c (dg/d theta) (lam_j - lam_i) . (R_i - R_j).
struct SparseVjpArgs {
  const float* x;
  int64_t xs;
  const int32_t* species;
  int n;
  const int32_t* idx;
  int64_t ld;
  int64_t width;
  const float* lam;
  int64_t ls;
  float* gx;
  int64_t gs;
  float weight;
  float c;
  double* gp;
  double* ge;
  Geo geo;
  int per_pair;
};

template <int DIM, int KIND, bool SPECIES, bool EGRAD>
__global__ void __launch_bounds__(256) k_force_vjp_sparse(SparseVjpArgs a,
                                                          const __grid_constant__ PairTable tab,
                                                          const __grid_constant__ PairTable sig) {
  constexpr int NB = SPECIES ? JMD_MAX_SPECIES : 1;
  __shared__ float bins[kBins];
  __shared__ float ebins[EGRAD ? kBins : 1];
  zero_bins(bins);
  if (EGRAD) zero_bins(ebins);
  __syncthreads();
  BinAcc<NB> acc, eacc;
  acc.zero();
  eacc.zero();
  const bool per_pair = a.per_pair != 0;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int si = 0;
  if (e < a.width) {
    const int j = __ldg(a.idx + e);
    const int i = __ldg(a.idx + a.ld + e);
    if ((unsigned)j < (unsigned)a.n && (unsigned)i < (unsigned)a.n) {
      const float4 xi = load_row<DIM, false>(a.x, a.xs, i);
      const float4 xj = load_row<DIM, false>(a.x, a.xs, j);
      float dx, dy, dz;
      displacement<DIM>(xi, xj, a.geo, dx, dy, dz);   // R_i - R_j
      const float r2 = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f);
      si = SPECIES ? min(max(__ldg(a.species + i), 0), tab.nsp - 1) : 0;
      const int sj = SPECIES ? min(max(__ldg(a.species + j), 0), tab.nsp - 1) : 0;
      const int bin = si * JMD_MAX_SPECIES + sj;
      const PairCoef& c = tab.c[SPECIES ? bin : 0];
      if (r2 < c.rc2 && r2 > 0.f) {
        const float sigma = sig.c[SPECIES ? bin : 0].pad;
        const PairD q = pair_derivs<KIND>(r2, c, sigma, per_pair ? sigma : sig.pad);
        const float4 li = load_row<DIM, false>(a.lam, a.ls, i);
        const float4 lj = load_row<DIM, false>(a.lam, a.ls, j);
        const float ex = lj.x - li.x, ey = lj.y - li.y, ez = DIM == 3 ? lj.z - li.z : 0.f;
        const float t = dx * ex + dy * ey + dz * ez;
        const float cdd = (q.hh - q.g) / r2 * t;
        if (a.gx) {
          const float w = a.weight * a.c;
          const float gx = w * (q.g * ex + cdd * dx), gy = w * (q.g * ey + cdd * dy);
          const float gz = DIM == 3 ? w * (q.g * ez + cdd * dz) : 0.f;
          float* oi = a.gx + (int64_t)i * a.gs;
          float* oj = a.gx + (int64_t)j * a.gs;
          atomicAdd(oi, gx);
          atomicAdd(oi + 1, gy);
          atomicAdd(oj, -gx);
          atomicAdd(oj + 1, -gy);
          if (DIM == 3) {
            atomicAdd(oi + 2, gz);
            atomicAdd(oj + 2, -gz);
          }
        }
        const float ct = a.c * t;
        acc.add(sj, q.dg_s * ct, q.dg_e * ct, KIND == JMD_LJ ? q.dg_k * ct : 0.f, per_pair);
        if (EGRAD)
          eacc.add(sj, a.c * q.dU_s, a.c * q.dU_e, KIND == JMD_LJ ? a.c * q.dU_k : 0.f, per_pair);
      }
    }
  }
  const int ncol = SPECIES ? tab.nsp : 1;
  if (!SPECIES) {
    acc.group_sum(kWarp, 1);
    if (EGRAD) eacc.group_sum(kWarp, 1);
  }
  if (SPECIES || (threadIdx.x & (kWarp - 1)) == 0) {
    acc.flush(bins, si, ncol);
    if (EGRAD) eacc.flush(ebins, si, ncol);
  }
  __syncthreads();
  publish_bins(bins, a.gp, (double)a.weight);
  if (EGRAD) publish_bins(ebins, a.ge, 1.0);
}

template <int DIM, int KIND>
void svjp_launch(bool sp, bool eg, const SparseVjpArgs& a, const PairTable& t,
                 const PairTable& s, cudaStream_t st) {
  const unsigned grid = (unsigned)std::max<int64_t>(1, ceil_div(a.width, 256));
  if (sp) {
    if (eg) k_force_vjp_sparse<DIM, KIND, true, true><<<grid, 256, 0, st>>>(a, t, s);
    else k_force_vjp_sparse<DIM, KIND, true, false><<<grid, 256, 0, st>>>(a, t, s);
  } else {
    if (eg) k_force_vjp_sparse<DIM, KIND, false, true><<<grid, 256, 0, st>>>(a, t, s);
    else k_force_vjp_sparse<DIM, KIND, false, false><<<grid, 256, 0, st>>>(a, t, s);
  }
}

}  // namespace

// Host side of the engine's reverse step (declared in pair.cuh).
int adjoint_pack(const jmd_nve_system& s, const float* x, float* xbar, float* pbar, float* rec,
                 bool kick, bool skin, cudaStream_t st) {
  const int n = (int)s.n;
  const unsigned grid = (unsigned)ceil_div(n, 256);
  const float4* ref = skin ? reinterpret_cast<const float4*>(s.reference_position) : nullptr;
  const Geo g = make_geo(s.space);
  if (s.space.dim == 3)
    k_adj_pack<3><<<grid, 256, 0, st>>>(n, reinterpret_cast<const float4*>(x),
                                        reinterpret_cast<float4*>(xbar), reinterpret_cast<float4*>(pbar),
                                        s.mass, s.mass_scalar, s.dt, kick ? 1 : 0,
                                        reinterpret_cast<float4*>(rec), ref, s.threshold_sq,
                                        s.rebuild_flag, g);
  else
    k_adj_pack<2><<<grid, 256, 0, st>>>(n, reinterpret_cast<const float4*>(x),
                                        reinterpret_cast<float4*>(xbar), reinterpret_cast<float4*>(pbar),
                                        s.mass, s.mass_scalar, s.dt, kick ? 1 : 0,
                                        reinterpret_cast<float4*>(rec), ref, s.threshold_sq,
                                        s.rebuild_flag, g);
  JMD_CUDA(cudaGetLastError());
  return JMD_OK;
}

int adjoint_vjp_step(const jmd_nve_system& s, float* xbar, const float* rec, float weight,
                     double* grad_params, cudaStream_t st) {
  const PairTable t = make_pair_table(s.pair);
  const PairTable sg = sigma_table(s.pair);
  StepArgs a{};
  a.n = (int)s.n;
  a.rec = reinterpret_cast<const float4*>(rec);
  a.xbar = reinterpret_cast<float4*>(xbar);
  a.species = s.species;
  a.idx = s.idx;
  a.ld = s.idx_ld;
  a.width = (int)s.nlist.max_occupancy;
  a.cnt = s.nbr_count;
  a.weight = weight;
  a.gp = grad_params;
  a.geo = make_geo(s.space);
  a.per_pair = s.pair.per_pair_cutoff;
  const int tpa = dense_tpa();
  const bool sp = s.pair.n_species > 0 && s.species != nullptr, pr = grad_params != nullptr;
  if (s.space.dim == 3) {
    if (s.pair.kind == JMD_LJ) step_launch<3, JMD_LJ>(tpa, sp, pr, a, t, sg, st);
    else if (s.pair.kind == JMD_LJ_TRUNCATED) step_launch<3, JMD_LJ_TRUNCATED>(tpa, sp, pr, a, t, sg, st);
    else if (s.pair.kind == JMD_MORSE) step_launch<3, JMD_MORSE>(tpa, sp, pr, a, t, sg, st);
    else step_launch<3, JMD_SOFT_SPHERE>(tpa, sp, pr, a, t, sg, st);
  } else {
    if (s.pair.kind == JMD_LJ) step_launch<2, JMD_LJ>(tpa, sp, pr, a, t, sg, st);
    else if (s.pair.kind == JMD_LJ_TRUNCATED) step_launch<2, JMD_LJ_TRUNCATED>(tpa, sp, pr, a, t, sg, st);
    else if (s.pair.kind == JMD_MORSE) step_launch<2, JMD_MORSE>(tpa, sp, pr, a, t, sg, st);
    else step_launch<2, JMD_SOFT_SPHERE>(tpa, sp, pr, a, t, sg, st);
  }
  JMD_CUDA(cudaGetLastError());
  return JMD_OK;
}

}  // namespace jmd

using namespace jmd;

extern "C" {

int jmd_pair_force_vjp(const jmd_pair* pp, const jmd_space* space, const float* position,
                       int64_t pos_stride, const int32_t* species, int64_t n, const int32_t* idx,
                       int64_t idx_ld, int64_t idx_width, const int32_t* nbr_count,
                       const float* cotangent, int64_t cot_stride, float weight,
                       float* grad_position, int64_t grad_stride, double* grad_params,
                       double* grad_energy_params, void* stream) {
  int e = validate_pair(pp);
  if (e) return e;
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(n >= 0 && n < INT32_MAX, "atom count out of range");
  JMD_REQUIRE(idx_ld >= idx_width, "idx_ld must be >= idx_width");
  JMD_REQUIRE(cotangent != nullptr, "cotangent is null");
  JMD_REQUIRE(pp->n_species == 0 || species != nullptr, "species matrices need a species array");
  if (n <= 0) return JMD_OK;
  const PairTable t = make_pair_table(*pp);
  const PairTable sg = sigma_table(*pp);
  VjpArgs a{};
  a.x = position;
  a.xs = pos_stride;
  a.species = species;
  a.n = (int)n;
  a.idx = idx;
  a.ld = idx_ld;
  a.width = idx_width;
  a.cnt = nbr_count;
  a.lam = cotangent;
  a.ls = cot_stride;
  a.gx = grad_position;
  a.gs = grad_stride;
  a.weight = weight;
  a.gp = grad_params;
  a.ge = grad_energy_params;
  a.geo = make_geo(*space);
  a.per_pair = pp->per_pair_cutoff;
  const bool sp = pp->n_species > 0, eg = grad_energy_params != nullptr;
  cudaStream_t st = as_stream(stream);
  if (space->dim == 3) {
    if (pp->kind == JMD_LJ) vjp_launch<3, JMD_LJ>(sp, eg, a, t, sg, st);
    else if (pp->kind == JMD_LJ_TRUNCATED) vjp_launch<3, JMD_LJ_TRUNCATED>(sp, eg, a, t, sg, st);
    else if (pp->kind == JMD_MORSE) vjp_launch<3, JMD_MORSE>(sp, eg, a, t, sg, st);
    else vjp_launch<3, JMD_SOFT_SPHERE>(sp, eg, a, t, sg, st);
  } else {
    if (pp->kind == JMD_LJ) vjp_launch<2, JMD_LJ>(sp, eg, a, t, sg, st);
    else if (pp->kind == JMD_LJ_TRUNCATED) vjp_launch<2, JMD_LJ_TRUNCATED>(sp, eg, a, t, sg, st);
    else if (pp->kind == JMD_MORSE) vjp_launch<2, JMD_MORSE>(sp, eg, a, t, sg, st);
    else vjp_launch<2, JMD_SOFT_SPHERE>(sp, eg, a, t, sg, st);
  }
  return check_launch("jmd_pair_force_vjp");
}

int jmd_pair_force_vjp_sparse(const jmd_pair* pp, const jmd_space* space, int32_t format,
                              const float* position, int64_t pos_stride, const int32_t* species,
                              int64_t n, const int32_t* idx, int64_t idx_ld, int64_t idx_width,
                              const float* cotangent, int64_t cot_stride, float weight,
                              float* grad_position, int64_t grad_stride, double* grad_params,
                              double* grad_energy_params, void* stream) {
  int e = validate_pair(pp);
  if (e) return e;
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(format == JMD_SPARSE || format == JMD_ORDERED_SPARSE, "format must be Sparse or OrderedSparse");
  JMD_REQUIRE(n >= 0 && n < INT32_MAX, "atom count out of range");
  JMD_REQUIRE(idx_ld >= idx_width, "idx_ld must be >= idx_width");
  JMD_REQUIRE(cotangent != nullptr, "cotangent is null");
  JMD_REQUIRE(pp->n_species == 0 || species != nullptr, "species matrices need a species array");
  if (n <= 0 || idx_width <= 0) return JMD_OK;
  const PairTable t = make_pair_table(*pp);
  const PairTable sg = sigma_table(*pp);
  SparseVjpArgs a{};
  a.x = position;
  a.xs = pos_stride;
  a.species = species;
  a.n = (int)n;
  a.idx = idx;
  a.ld = idx_ld;
  a.width = idx_width;
  a.lam = cotangent;
  a.ls = cot_stride;
  a.gx = grad_position;
  a.gs = grad_stride;
  a.weight = weight;
  a.c = format == JMD_ORDERED_SPARSE ? 1.f : 0.5f;
  a.gp = grad_params;
  a.ge = grad_energy_params;
  a.geo = make_geo(*space);
  a.per_pair = pp->per_pair_cutoff;
  const bool sp = pp->n_species > 0, eg = grad_energy_params != nullptr;
  cudaStream_t st = as_stream(stream);
  if (space->dim == 3) {
    if (pp->kind == JMD_LJ) svjp_launch<3, JMD_LJ>(sp, eg, a, t, sg, st);
    else if (pp->kind == JMD_LJ_TRUNCATED) svjp_launch<3, JMD_LJ_TRUNCATED>(sp, eg, a, t, sg, st);
    else if (pp->kind == JMD_MORSE) svjp_launch<3, JMD_MORSE>(sp, eg, a, t, sg, st);
    else svjp_launch<3, JMD_SOFT_SPHERE>(sp, eg, a, t, sg, st);
  } else {
    if (pp->kind == JMD_LJ) svjp_launch<2, JMD_LJ>(sp, eg, a, t, sg, st);
    else if (pp->kind == JMD_LJ_TRUNCATED) svjp_launch<2, JMD_LJ_TRUNCATED>(sp, eg, a, t, sg, st);
    else if (pp->kind == JMD_MORSE) svjp_launch<2, JMD_MORSE>(sp, eg, a, t, sg, st);
    else svjp_launch<2, JMD_SOFT_SPHERE>(sp, eg, a, t, sg, st);
  }
  return check_launch("jmd_pair_force_vjp_sparse");
}

}  // extern "C"
