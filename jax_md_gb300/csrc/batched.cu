// Batched systems: many independent periodic systems of uneven size, each
// phase of a step one launch over all of them.
//
// Reference (per system): partition.neighbor_list's cell-list build
// (partition.py:296-488, 1034-1121), smap.pair_neighbor_list (smap.py:922-979)
// with energy.soft_sphere / lennard_jones (energy.py:125-343), velocity Verlet
// (simulate.py:227-243) and FIRE (minimize.py:124-226).  jax.vmap batches only
// equal-size systems; here each atom carries its system id and every kernel
// looks up that system's box and cell grid.
//
// Build of the lists (one launch each):
//   k_bbin    one CTA per system: shared-memory histogram over the system's
//             cells, block scan, scatter of atom ids into cell order, then a
//             per-cell insertion sort of the ids (a deterministic order) and
//             the cell-ordered position copy;
//   k_bsearch one thread per atom in cell order: the 3^d cells around it in
//             its own grid (periodic), distance test with its own box, writes
//             its row of the tiled Dense list;
//   k_bfinal  error bits and occupancy, clears the rebuild flag.
#include <algorithm>
#include <cstring>
#include <functional>
#include <string>
#include <type_traits>

#include "adjoint.cuh"
#include "nhc.cuh"

namespace jmd {
namespace {

constexpr int kBinThreads = 512;
constexpr int kMaxBatchCellsShared = 24576;   // 2 x 96 KiB of int32 per system

struct BatchView {
  int dim, nsys, total_cells, max_cells;
  int n;
  const int32_t* sys_offset;
  const int32_t* atom_sys;
  const float* box;
  const int32_t* cell_offset;
  const int32_t* cps;
  const float* cs;
};

BatchView view_of(const jmd_batch& b) {
  BatchView v;
  v.dim = b.dim;
  v.nsys = b.n_systems;
  v.total_cells = b.total_cells;
  v.max_cells = b.max_cells;
  v.n = (int)b.n_atoms;
  v.sys_offset = b.sys_offset;
  v.atom_sys = b.atom_sys;
  v.box = b.box;
  v.cell_offset = b.cell_offset;
  v.cps = b.cells_per_side;
  v.cs = b.cell_size;
  return v;
}

// Workspace: cell starts and counts [total_cells], atom ids in cell order [N],
// positions in cell order [N] float4, local cell of each atom [N], scalars.
struct BWs {
  int32_t* cstart;
  int32_t* ccount;
  int32_t* sid;
  float4* xs;
  int32_t* cellof;
  unsigned int* sc;   // [0] error bits, [1] max row length
};

BWs carve(const jmd_batch& b, void* base, size_t bytes, bool* ok) {
  Carver cv(base, bytes);
  BWs w;
  w.cstart = cv.take<int32_t>(std::max<int64_t>(b.total_cells, 1));
  w.ccount = cv.take<int32_t>(std::max<int64_t>(b.total_cells, 1));
  w.sid = cv.take<int32_t>(std::max<int64_t>(b.n_atoms, 1));
  w.xs = cv.take<float4>(std::max<int64_t>(b.n_atoms, 1));
  w.cellof = cv.take<int32_t>(std::max<int64_t>(b.n_atoms, 1));
  w.sc = cv.take<unsigned int>(4);
  if (ok) *ok = base != nullptr && cv.ok();
  return w;
}

struct SysGeo {
  float L[3], halfL[3];
};

__device__ __forceinline__ SysGeo sys_geo(const BatchView& v, int b) {
  SysGeo g;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    g.L[d] = d < v.dim ? __ldg(v.box + 3 * b + d) : 1.f;
    g.halfL[d] = 0.5f * g.L[d];
  }
  return g;
}

// Minimum-image displacement a - b inside one system's box.
template <int DIM>
__device__ __forceinline__ void bdisp(const float4& a, const float4& c, const SysGeo& g, float& dx,
                                      float& dy, float& dz) {
  dx = a.x - c.x;
  dy = a.y - c.y;
  dz = DIM == 3 ? a.z - c.z : 0.f;
  bool wrapped = fabsf(dx) > g.halfL[0] || fabsf(dy) > g.halfL[1];
  if (DIM == 3) wrapped = wrapped || fabsf(dz) > g.halfL[2];
  if (wrapped) {
    dx = min_image(a.x, c.x, g.L[0], g.halfL[0]);
    dy = min_image(a.y, c.y, g.L[1], g.halfL[1]);
    if (DIM == 3) dz = min_image(a.z, c.z, g.L[2], g.halfL[2]);
  }
}

// Cell coordinates of a position in its system's grid (floor(x / cell_size),
// clamped to the grid as positions at the upper edge round there).
template <int DIM>
__device__ __forceinline__ void cell_coords(const BatchView& v, int b, const float4& x, int c[3]) {
  const float xx[3] = {x.x, x.y, x.z};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (d < DIM) {
      const int n = __ldg(v.cps + 3 * b + d);
      int k = (int)floorf(xx[d] / __ldg(v.cs + 3 * b + d));
      c[d] = min(max(k, 0), n - 1);
    } else {
      c[d] = 0;
    }
  }
}

template <int DIM>
__device__ __forceinline__ int cell_hash(const BatchView& v, int b, const int c[3]) {
  const int nx = __ldg(v.cps + 3 * b), ny = __ldg(v.cps + 3 * b + 1);
  return DIM == 3 ? c[0] + nx * (c[1] + ny * c[2]) : c[0] + nx * c[1];
}

__device__ __forceinline__ bool gated_off(const int32_t* flag) { return flag && *flag == 0; }

template <int DIM>
__global__ void __launch_bounds__(kBinThreads) k_bbin(BatchView v, BWs w, const float4* __restrict__ x,
                                                      const int32_t* flag) {
  if (gated_off(flag)) return;
  extern __shared__ int32_t sm[];
  const int b = blockIdx.x;
  const int a0 = __ldg(v.sys_offset + b), a1 = __ldg(v.sys_offset + b + 1);
  const int c0 = __ldg(v.cell_offset + b);
  const int nc = __ldg(v.cell_offset + b + 1) - c0;
  int32_t* cnt = sm;        // [nc] counts, then scatter cursors
  int32_t* start = sm + nc; // [nc] exclusive scan
  if (b == 0 && threadIdx.x < 4) w.sc[threadIdx.x] = 0u;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) cnt[c] = 0;
  __syncthreads();
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    int cc[3];
    cell_coords<DIM>(v, b, __ldg(x + i), cc);
    const int lc = cell_hash<DIM>(v, b, cc);
    w.cellof[i] = lc;
    atomicAdd(&cnt[lc], 1);
  }
  __syncthreads();
  // exclusive scan: each thread a contiguous chunk, then a scan of chunk sums
  __shared__ int32_t tsum[kBinThreads];
  const int per = (nc + blockDim.x - 1) / blockDim.x;
  const int lo = min(nc, threadIdx.x * per), hi = min(nc, lo + per);
  int s = 0;
  for (int c = lo; c < hi; ++c) s += cnt[c];
  tsum[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      const int q = tsum[t];
      tsum[t] = run;
      run += q;
    }
  }
  __syncthreads();
  int run = tsum[threadIdx.x];
  for (int c = lo; c < hi; ++c) {
    start[c] = run;
    w.cstart[c0 + c] = a0 + run;
    w.ccount[c0 + c] = cnt[c];
    run += cnt[c];
    cnt[c] = start[c];   // becomes the scatter cursor
  }
  __syncthreads();
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    const int slot = atomicAdd(&cnt[w.cellof[i]], 1);
    w.sid[a0 + slot] = i;
  }
  __syncthreads();
  // deterministic order inside each cell: ascending atom id
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    int32_t* ids = w.sid + a0 + start[c];
    const int m = cnt[c] - start[c];
    for (int p = 1; p < m; ++p) {
      const int key = ids[p];
      int q = p - 1;
      while (q >= 0 && ids[q] > key) {
        ids[q + 1] = ids[q];
        --q;
      }
      ids[q + 1] = key;
    }
    for (int p = 0; p < m; ++p) w.xs[a0 + start[c] + p] = __ldg(x + ids[p]);
  }
}

struct SearchArgs {
  float cutoff_sq;
  int width, ld, mask_self;
  int32_t* idx;
  int32_t* count;
  float4* ref;
};

__device__ __forceinline__ int64_t tile_at(int i, int k, int ld) {
  return (int64_t)(i >> 5) * ld * 32 + (int64_t)k * 32 + (i & 31);
}

template <int DIM>
__global__ void __launch_bounds__(128) k_bsearch(BatchView v, BWs w, SearchArgs a,
                                                 const int32_t* flag) {
  if (gated_off(flag)) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= v.n) return;
  const int i = w.sid[k];
  const float4 xi = w.xs[k];
  const int b = __ldg(v.atom_sys + i);
  const SysGeo g = sys_geo(v, b);
  const int c0 = __ldg(v.cell_offset + b);
  int cc[3];
  cell_coords<DIM>(v, b, xi, cc);
  const int nx = __ldg(v.cps + 3 * b), ny = __ldg(v.cps + 3 * b + 1);
  const int nz = DIM == 3 ? __ldg(v.cps + 3 * b + 2) : 1;
  int cnt = 0;
  // neighbour cells along an axis: -1..1 with >= 3 cells, the two cells with
  // 2, the one cell with 1 (each distinct cell visited once; the minimum
  // image then gives the pair set of an all-pairs search)
  const int lz = DIM == 3 ? (nz >= 3 ? -1 : 0) : 0, hz = DIM == 3 ? (nz >= 2 ? 1 : 0) : 0;
  const int ly = ny >= 3 ? -1 : 0, hy = ny >= 2 ? 1 : 0;
  const int lx = nx >= 3 ? -1 : 0, hx = nx >= 2 ? 1 : 0;
  for (int oz = lz; oz <= hz; ++oz) {
    const int z = DIM == 3 ? (cc[2] + oz + nz) % nz : 0;
    for (int oy = ly; oy <= hy; ++oy) {
      const int y = (cc[1] + oy + ny) % ny;
      for (int ox = lx; ox <= hx; ++ox) {
        const int xcell = (cc[0] + ox + nx) % nx;
        const int gc = c0 + xcell + nx * (y + ny * z);
        const int s = w.cstart[gc], e = s + w.ccount[gc];
        for (int m = s; m < e; ++m) {
          const int j = w.sid[m];
          if (a.mask_self && j == i) continue;
          float dx, dy, dz;
          bdisp<DIM>(xi, w.xs[m], g, dx, dy, dz);
          const float d2 = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f);
          if (d2 < a.cutoff_sq) {
            if (cnt < a.width) a.idx[tile_at(i, cnt, a.ld)] = j;
            ++cnt;
          }
        }
      }
    }
  }
  a.count[i] = min(cnt, a.width);
  a.ref[i] = xi;
  if (cnt > a.width) atomicOr(&w.sc[0], (unsigned)JMD_NEIGHBOR_LIST_OVERFLOW);
  atomicMax(&w.sc[1], (unsigned)cnt);
}

__global__ void k_bfinal(BWs w, int32_t* occupancy, uint8_t* error_code, int32_t* flag) {
  if (gated_off(flag)) return;
  if (occupancy) *occupancy = (int32_t)w.sc[1];
  if (error_code) *error_code = (uint8_t)(*error_code | w.sc[0]);
  if (flag) *flag = 0;
}

template <int DIM>
__global__ void k_bskin(BatchView v, const float4* __restrict__ x, const float4* __restrict__ ref,
                        float thr2, int32_t* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (i < v.n) {
    const SysGeo g = sys_geo(v, __ldg(v.atom_sys + i));
    float dx, dy, dz;
    bdisp<DIM>(__ldg(x + i), __ldg(ref + i), g, dx, dy, dz);
    over = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f) > thr2;
  }
  if (__any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// ------------------------------------------------------------- forces ----
enum BMode { B_FORCE = 0, B_KICK = 1, B_FIRE = 2 };

struct BForceArgs {
  const float4* x;
  float4* f;
  float4* p;
  const int32_t* species;
  const int32_t* idx;
  const int32_t* count;
  int ld;
  float h;                  // B_KICK: p += h F
  const int32_t* done;      // B_FIRE: frozen systems are skipped
};

// One thread per atom over the tiled list; each atom uses its system's box.
template <int DIM, int KIND, bool SPECIES, int MODE>
__global__ void __launch_bounds__(256) k_bforce(BatchView v, BForceArgs a,
                                                const __grid_constant__ PairTable tab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n) return;
  const int b = __ldg(v.atom_sys + i);
  if (MODE == B_FIRE && __ldg(a.done + b)) return;
  const SysGeo g = sys_geo(v, b);
  const float4 xi = __ldg(a.x + i);
  const int si = SPECIES ? min(max(__ldg(a.species + i), 0), tab.nsp - 1) : 0;
  const int m = __ldg(a.count + i);
  const int32_t* col = a.idx + (int64_t)(i >> 5) * a.ld * 32 + (i & 31);
  float fx = 0.f, fy = 0.f, fz = 0.f;
  for (int e = 0; e < m; ++e) {
    const int j = __ldcs(col + (int64_t)e * 32);
    const float4 xj = __ldg(a.x + j);
    float dx, dy, dz;
    bdisp<DIM>(xi, xj, g, dx, dy, dz);
    const float r2 = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f);
    const int sj = SPECIES ? min(max(__ldg(a.species + j), 0), tab.nsp - 1) : 0;
    const PairCoef& c = tab.c[SPECIES ? si * JMD_MAX_SPECIES + sj : 0];
    if (!(r2 < c.rc2) || r2 == 0.f) continue;
    float U, gr, hh;
    pair_eval<KIND, false>(r2, c, U, gr, hh);
    // F_i = -sum_j U'(r)/r (R_i - R_j)
    fx = fmaf(-gr, dx, fx);
    fy = fmaf(-gr, dy, fy);
    if (DIM == 3) fz = fmaf(-gr, dz, fz);
  }
  a.f[i] = make_float4(fx, fy, fz, 0.f);
  if (MODE == B_KICK) {
    float4 q = a.p[i];
    q.x = fmaf(a.h, fx, q.x);
    q.y = fmaf(a.h, fy, q.y);
    if (DIM == 3) q.z = fmaf(a.h, fz, q.z);
    a.p[i] = q;
  }
}

// Block sum of a double (all threads), result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double part[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) part[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)((blockDim.x + 31) >> 5); ++k) s += part[k];
  return s;
}

__device__ __forceinline__ float block_max(float v) {
  __shared__ float part[32];
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) part[wid] = v;
  __syncthreads();
  float s = 0.f;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)((blockDim.x + 31) >> 5); ++k) s = fmaxf(s, part[k]);
  return s;
}

// Per-system potential energy (Dense rows, each entry half the pair energy),
// one CTA per system, f64 sums in a fixed order.
template <int DIM, int KIND, bool SPECIES>
__global__ void __launch_bounds__(256) k_bsys_energy(BatchView v, BForceArgs a,
                                                     const __grid_constant__ PairTable tab,
                                                     double* energy) {
  const int b = blockIdx.x;
  const int a0 = __ldg(v.sys_offset + b), a1 = __ldg(v.sys_offset + b + 1);
  const SysGeo g = sys_geo(v, b);
  double acc = 0.0;
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    const float4 xi = __ldg(a.x + i);
    const int si = SPECIES ? min(max(__ldg(a.species + i), 0), tab.nsp - 1) : 0;
    const int m = __ldg(a.count + i);
    const int32_t* col = a.idx + (int64_t)(i >> 5) * a.ld * 32 + (i & 31);
    float e_i = 0.f;
    for (int e = 0; e < m; ++e) {
      const int j = __ldg(col + (int64_t)e * 32);
      float dx, dy, dz;
      bdisp<DIM>(xi, __ldg(a.x + j), g, dx, dy, dz);
      const float r2 = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f);
      const int sj = SPECIES ? min(max(__ldg(a.species + j), 0), tab.nsp - 1) : 0;
      const PairCoef& c = tab.c[SPECIES ? si * JMD_MAX_SPECIES + sj : 0];
      if (!(r2 < c.rc2) || r2 == 0.f) continue;
      float U, gr, hh;
      pair_eval<KIND, false>(r2, c, U, gr, hh);
      e_i += U;
    }
    acc += 0.5 * (double)e_i;
  }
  const double s = block_sum(acc);
  if (threadIdx.x == 0) energy[b] = s;
}

// Per-system kinetic energy and largest atom force norm.
template <int DIM>
__global__ void __launch_bounds__(256) k_bke(BatchView v, const float4* __restrict__ p,
                                             const float4* __restrict__ f, const float* mass,
                                             float m0, double* ke, float* fmax) {
  const int b = blockIdx.x;
  const int a0 = __ldg(v.sys_offset + b), a1 = __ldg(v.sys_offset + b + 1);
  double acc = 0.0;
  float mf = 0.f;
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    if (ke) {
      const float4 q = __ldg(p + i);
      const float m = mass ? __ldg(mass + i) : m0;
      acc += 0.5 * ((double)q.x * q.x + (double)q.y * q.y + (DIM == 3 ? (double)q.z * q.z : 0.0)) / m;
    }
    if (fmax) {
      const float4 ff = __ldg(f + i);
      mf = fmaxf(mf, ff.x * ff.x + ff.y * ff.y + (DIM == 3 ? ff.z * ff.z : 0.f));
    }
  }
  const double s = block_sum(acc);
  const float mx = block_max(mf);
  if (threadIdx.x == 0) {
    if (ke) ke[b] = s;
    if (fmax) fmax[b] = sqrtf(mx);
  }
}

// ------------------------------------------ Nose-Hoover adjoint helpers ----
// The per-atom algebra of one reverse Nose-Hoover step of the batched
// trajectory adjoint (batch.BatchNvtTrajectory), fused: per-system dot
// products in f64 (CTA per system, no contended atomics) and the elementwise
// cotangent updates.  Rows are [n, stride] float; `dim` components are used.
template <int DIM>
__global__ void __launch_bounds__(256) k_bdot(BatchView v, const float* __restrict__ a, int64_t as,
                                              const float* __restrict__ c, int64_t cs,
                                              double* out) {
  const int b = blockIdx.x;
  const int a0 = __ldg(v.sys_offset + b), a1 = __ldg(v.sys_offset + b + 1);
  double acc = 0.0;
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    float d = a[i * as] * c[i * cs];
    d = fmaf(a[i * as + 1], c[i * cs + 1], d);
    if (DIM == 3) d = fmaf(a[i * as + 2], c[i * cs + 2], d);
    acc += (double)d;
  }
  const double s = block_sum(acc);
  if (threadIdx.x == 0) out[b] = s;
}

// rbar = pbar s2[sys] + kebar[sys] r / m ;  lam = h (rbar + pending)
template <int DIM>
__global__ void k_bnvt_pre(BatchView v, const float* pbar, const float* r, int64_t rs,
                           const double* s2, const double* kebar, float inv_m, float h,
                           const float* pending, float* rbar, float* lam4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n) return;
  const int b = __ldg(v.atom_sys + i);
  const float sc = (float)s2[b], kb = (float)kebar[b];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const float rb = fmaf(kb * r[i * rs + d], inv_m, pbar[i * DIM + d] * sc);
    rbar[i * DIM + d] = rb;
    lam4[i * 4 + d] = h * (pending ? rb + pending[i * DIM + d] : rb);
  }
}

// qbar = rbar + (dt / m) xbar ;  sbar1[sys] = sum qbar . p_k
template <int DIM>
__global__ void __launch_bounds__(256) k_bnvt_post(BatchView v, const float* rbar,
                                                   const float* xbar4, float dt_inv_m,
                                                   const float* pk, int64_t ps, float* qbar,
                                                   double* sbar1) {
  const int b = blockIdx.x;
  const int a0 = __ldg(v.sys_offset + b), a1 = __ldg(v.sys_offset + b + 1);
  double acc = 0.0;
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    float d = 0.f;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const float q = fmaf(dt_inv_m, xbar4[i * 4 + k], rbar[i * DIM + k]);
      qbar[i * DIM + k] = q;
      d = fmaf(q, pk[i * ps + k], d);
    }
    acc += (double)d;
  }
  const double s = block_sum(acc);
  if (threadIdx.x == 0) sbar1[b] = s;
}

// pbar = qbar s1[sys] + kebar[sys] p_k / m
template <int DIM>
__global__ void k_bnvt_pbar(BatchView v, const float* qbar, const double* s1, const double* kebar,
                            const float* pk, int64_t ps, float inv_m, float* pbar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n) return;
  const int b = __ldg(v.atom_sys + i);
  const float sc = (float)s1[b], kb = (float)kebar[b];
#pragma unroll
  for (int d = 0; d < DIM; ++d)
    pbar[i * DIM + d] = fmaf(kb * pk[i * ps + d], inv_m, qbar[i * DIM + d] * sc);
}

// --------------------------------------------------------- integration ----
// Kick + drift with the skin test of the drifted positions.  FIRE: the time
// step is the system's own (fire_state[8b]) and frozen systems are skipped.
template <int DIM, bool FIRE>
__global__ void __launch_bounds__(256) k_bkick_drift(BatchView v, float4* x, float4* p,
                                                     const float4* __restrict__ f,
                                                     const float* mass, float m0, float dt,
                                                     const float* fs, const int32_t* done,
                                                     const float4* ref, float thr2, int32_t* flag,
                                                     const double* pscale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (i < v.n) {
    const int b = __ldg(v.atom_sys + i);
    if (!(FIRE && done[b])) {
      const float dts = FIRE ? fs[8 * b] : dt;
      const float h = 0.5f * dts;
      const SysGeo g = sys_geo(v, b);
      float4 q = p[i];
      if (pscale) {  // the Nose-Hoover chain's momentum rescale before the kick
        const float sc = (float)__ldg(pscale + b);
        q.x *= sc;
        q.y *= sc;
        q.z *= sc;
      }
      const float4 ff = __ldg(f + i);
      q.x = fmaf(h, ff.x, q.x);
      q.y = fmaf(h, ff.y, q.y);
      if (DIM == 3) q.z = fmaf(h, ff.z, q.z);
      const float m = mass ? __ldg(mass + i) : m0;
      float4 r = x[i];
      r.x = wrap(r.x + dts * q.x / m, g.L[0]);
      r.y = wrap(r.y + dts * q.y / m, g.L[1]);
      if (DIM == 3) r.z = wrap(r.z + dts * q.z / m, g.L[2]);
      p[i] = q;
      x[i] = r;
      if (ref) {
        float dx, dy, dz;
        bdisp<DIM>(r, __ldg(ref + i), g, dx, dy, dz);
        over = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f) > thr2;
      }
    }
  }
  if (ref && __any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// Nose-Hoover chain half step of every system, one CTA per system
// (simulate.py:492-517 with update_mass :509-515; the chain of system b is
// chain[66 b ..], its degrees of freedom n_b * DIM as quantity.count_dof).
// MEASURE: the kinetic energy is summed from p (FP32 per thread, f64 across
// threads) and written to the chain first, else the chain's stored one is
// used.  With p, the system's momenta are multiplied by its scale.
template <int DIM>
__global__ void __launch_bounds__(256) k_bnhc(BatchView v, NhcArgs a, double* chain, float4* p,
                                              const float* mass, float m0, int measure,
                                              double* scale_out, double* ke_out) {
  const int b = blockIdx.x;
  const int a0 = __ldg(v.sys_offset + b), a1 = __ldg(v.sys_offset + b + 1);
  __shared__ float s_scale;
  double ke = 0.0;
  if (measure) {
    float acc = 0.f;
    for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
      const float4 q = p[i];
      const float m = mass ? __ldg(mass + i) : m0;
      acc += (q.x * q.x + q.y * q.y + (DIM == 3 ? q.z * q.z : 0.f)) / m;
    }
    ke = 0.5 * block_sum((double)acc);
  }
  if (threadIdx.x == 0) {
    double* c = chain + 66 * (size_t)b;
    if (measure) c[64] = ke;
    else ke = c[64];
    if (ke_out) ke_out[b] = ke;
    const float sc = nhc_half_chain(a, c, (float)ke, (float)((a1 - a0) * DIM));
    if (scale_out) scale_out[b] = sc;
    s_scale = sc;
  }
  __syncthreads();
  if (p) {
    const float sc = s_scale;
    for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
      float4 q = p[i];
      q.x *= sc;
      q.y *= sc;
      if (DIM == 3) q.z *= sc;
      p[i] = q;
    }
  }
}

// Reverse of k_bnhc's chain half step, one thread per system: chain[66 b ..]
// the state before it, ke[b] the kinetic energy it used, cot_pxi[16 b ..] and
// cot_scale[b] the cotangents of its outputs; writes grad_pxi[16 b ..] and
// grad_ke[b].
__global__ void k_bnhc_vjp(NhcArgs a, int nsys, const int32_t* sys_offset, int dim,
                           const double* chain, const double* ke, const double* cot_pxi,
                           const double* cot_scale, double* grad_pxi, double* grad_ke) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nsys) return;
  const float dof = (float)((sys_offset[b + 1] - sys_offset[b]) * dim);
  nhc_half_chain_vjp(a, chain + 66 * (size_t)b, (float)ke[b], dof, cot_pxi + 16 * (size_t)b,
                     cot_scale[b], grad_pxi + 16 * (size_t)b, grad_ke + b);
}

// (x, lambda) records of the batched force VJP (the layout k_badj_step reads).
template <int DIM>
__global__ void __launch_bounds__(256) k_bvjp_pack(int n, const float4* __restrict__ x,
                                                   const float4* __restrict__ lam, float4* rec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = __ldg(x + i), q = __ldg(lam + i);
  rec[2 * i] = make_float4(xi.x, xi.y, DIM == 3 ? xi.z : 0.f, q.x);
  rec[2 * i + 1] = make_float4(q.y, DIM == 3 ? q.z : 0.f, 0.f, 0.f);
}

// FIRE after the force: closing half kick, the three f64 reductions, the
// scalar update of minimize.py:190-224, the mixing, and the convergence test
// on the largest atom force norm.  One CTA per system.
constexpr int kFireThreads = 1024;  // upper bound; the launch uses g_fire_threads

// Launch shapes chosen by the batch autotuner (jmd_batch_set_launch).
int g_force_block = 128;
int g_fire_threads = 1024;

template <int DIM>
__global__ void __launch_bounds__(kFireThreads) k_bfire_update(BatchView v, float4* p, const float4* __restrict__ f,
                                                      float* fs, int32_t* done, int32_t* n_done,
                                                      jmd_fire_params fp) {
  const int b = blockIdx.x;
  if (done[b]) return;
  const int a0 = __ldg(v.sys_offset + b), a1 = __ldg(v.sys_offset + b + 1);
  float* s = fs + 8 * b;
  const float h = 0.5f * s[0];
  // each thread sums its few atoms in fp32 (the FP64 pipe is narrow); the
  // block reduction of the partial sums runs in f64
  float ff = 0.f, pp = 0.f, fpd = 0.f;
  float mf = 0.f;
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    float4 q = p[i];
    const float4 fi = __ldg(f + i);
    q.x = fmaf(h, fi.x, q.x);
    q.y = fmaf(h, fi.y, q.y);
    if (DIM == 3) q.z = fmaf(h, fi.z, q.z);
    p[i] = q;
    const float f2 = fi.x * fi.x + fi.y * fi.y + (DIM == 3 ? fi.z * fi.z : 0.f);
    ff += f2;
    pp += q.x * q.x + q.y * q.y + (DIM == 3 ? q.z * q.z : 0.f);
    fpd += fi.x * q.x + fi.y * q.y + (DIM == 3 ? fi.z * q.z : 0.f);
    mf = fmaxf(mf, f2);
  }
  const double sff = block_sum((double)ff);
  const double spp = block_sum((double)pp);
  const double sfp = block_sum((double)fpd);
  const float smf = block_max(mf);
  __shared__ float mix[3];
  if (threadIdx.x == 0) {
    const float F_norm = (float)sqrt(sff + 1e-6);
    const float P_norm = (float)sqrt(spp);
    const float F_dot_P = (float)sfp;
    float dt = s[0], alpha = s[1], n_pos = s[2];
    mix[0] = alpha;
    mix[1] = P_norm / F_norm;
    mix[2] = F_dot_P >= 0.f ? 1.f : 0.f;
    n_pos = F_dot_P >= 0.f ? n_pos + 1.f : 0.f;
    if (F_dot_P > 0.f && n_pos > fp.n_min) {
      dt = fminf(dt * fp.f_inc, fp.dt_max);
      alpha = alpha * fp.f_alpha;
    }
    if (F_dot_P < 0.f) {
      dt = dt * fp.f_dec;
      alpha = fp.alpha_start;
    }
    s[0] = dt;
    s[1] = alpha;
    s[2] = n_pos;
    s[3] = mix[2];
    s[4] = mix[0];
    s[5] = mix[1];
    s[6] = sqrtf(smf);
  }
  __syncthreads();
  const float alpha = mix[0], ratio = mix[1], keep = mix[2];
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
    float4 q = p[i];
    const float4 fi = __ldg(f + i);
    q.x = keep * (q.x + alpha * (fi.x * ratio - q.x));
    q.y = keep * (q.y + alpha * (fi.y * ratio - q.y));
    if (DIM == 3) q.z = keep * (q.z + alpha * (fi.z * ratio - q.z));
    p[i] = q;
  }
  if (threadIdx.x == 0 && sqrtf(smf) < fp.f_tol) {
    done[b] = 1;
    atomicAdd(n_done, 1);
  }
}

__global__ void k_bfire_init(int nsys, float* fs, int32_t* done, int32_t* n_done, float dt0,
                             float alpha0) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b == 0) *n_done = 0;
  if (b >= nsys) return;
  float* s = fs + 8 * b;
  s[0] = dt0;
  s[1] = alpha0;
  for (int k = 2; k < 8; ++k) s[k] = 0.f;
  done[b] = 0;
}

// ------------------------------------------------------------ adjoint ----
// Reverse velocity Verlet over a batch (the single-system form is in
// adjoint.cu): pack writes (x, q) records with q = pbar + (dt/m) xbar and runs
// the skin test with each atom's own box; the step accumulates
// xbar_k += w sum_j J_kj (q_j - q_k) over k's tiled row and, with PARAMS, the
// shared sigma / epsilon / cutoff-scale bins summed over every system.
template <int DIM>
__global__ void __launch_bounds__(256) k_badj_pack(BatchView v, const float4* __restrict__ x,
                                                   float4* xbar, float4* pbar, const float* mass,
                                                   float m0, float dt, int kick, float4* rec,
                                                   const float4* ref, float thr2, int32_t* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (i < v.n) {
    const float4 xi = __ldg(x + i);
    float4 q = pbar[i];
    if (kick) {
      const float4 xb = xbar[i];
      const float c = dt / (mass ? __ldg(mass + i) : m0);
      q.x = fmaf(c, xb.x, q.x);
      q.y = fmaf(c, xb.y, q.y);
      if (DIM == 3) q.z = fmaf(c, xb.z, q.z);
      pbar[i] = q;
    }
    rec[2 * i] = make_float4(xi.x, xi.y, DIM == 3 ? xi.z : 0.f, q.x);
    rec[2 * i + 1] = make_float4(q.y, DIM == 3 ? q.z : 0.f, 0.f, 0.f);
    if (ref) {
      const SysGeo g = sys_geo(v, __ldg(v.atom_sys + i));
      float dx, dy, dz;
      bdisp<DIM>(xi, __ldg(ref + i), g, dx, dy, dz);
      over = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f) > thr2;
    }
  }
  if (ref && __any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

struct BAdjArgs {
  const float4* rec;        // step: (x, q) records; energy mode: positions in rec[i] (float4 rows)
  float4* xbar;
  const int32_t* species;
  const int32_t* idx;
  const int32_t* count;
  int ld;
  float weight;
  const double* sys_weight; // energy mode: per-system weight of dE_b/dtheta
  double* gp;
  int per_pair;
};

// MODE 0: reverse step (records, xbar, optional bins); MODE 1: bins of
// sum_b sys_weight[b] dE_b/dtheta only.
template <int DIM, int KIND, bool SPECIES, bool PARAMS, int MODE>
__global__ void __launch_bounds__(128) k_badj_step(BatchView v, BAdjArgs a,
                                                   const __grid_constant__ PairTable tab,
                                                   const __grid_constant__ PairTable sig) {
  constexpr int NB = SPECIES ? JMD_MAX_SPECIES : 1;
  __shared__ float bins[PARAMS ? kBins : 1];
  if (PARAMS) {
    zero_bins(bins);
    __syncthreads();
  }
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < v.n;
  const bool per_pair = a.per_pair != 0;
  BinAcc<NB> acc;
  acc.zero();
  int si = 0;
  if (active) {
    const int b = __ldg(v.atom_sys + i);
    const SysGeo g = sys_geo(v, b);
    const float ew = MODE == 1 ? (float)__ldg(a.sys_weight + b) : 1.f;
    const float4 r0 = MODE == 0 ? __ldg(a.rec + 2 * i) : __ldg(a.rec + i);
    const float4 r1 = MODE == 0 ? __ldg(a.rec + 2 * i + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float qx = r0.w, qy = r1.x, qz = r1.y;
    si = SPECIES ? min(max(__ldg(a.species + i), 0), tab.nsp - 1) : 0;
    const int m = __ldg(a.count + i);
    const int32_t* col = a.idx + (int64_t)(i >> 5) * a.ld * 32 + (i & 31);
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int e = 0; e < m; ++e) {
      const int j = __ldcs(col + (int64_t)e * 32);
      const float4 j0 = MODE == 0 ? __ldg(a.rec + 2 * j) : __ldg(a.rec + j);
      float dx, dy, dz;
      bdisp<DIM>(r0, j0, g, dx, dy, dz);
      const float r2 = dx * dx + dy * dy + (DIM == 3 ? dz * dz : 0.f);
      const int sj = SPECIES ? min(max(__ldg(a.species + j), 0), tab.nsp - 1) : 0;
      const int bin = si * JMD_MAX_SPECIES + sj;
      const PairCoef& c = tab.c[SPECIES ? bin : 0];
      if (!(r2 < c.rc2) || r2 == 0.f) continue;
      if (MODE == 1) {
        const float sigma = sig.c[SPECIES ? bin : 0].pad;
        const PairD q = pair_derivs<KIND>(r2, c, sigma, per_pair ? sigma : sig.pad);
        const float h = 0.5f * ew;
        acc.add(sj, h * q.dU_s, h * q.dU_e, KIND == JMD_LJ ? h * q.dU_k : 0.f, per_pair);
        continue;
      }
      const float4 j1 = __ldg(a.rec + 2 * j + 1);
      float gg, hh;
      PairD q;
      if (PARAMS) {
        const float sigma = sig.c[SPECIES ? bin : 0].pad;
        q = pair_derivs<KIND>(r2, c, sigma, per_pair ? sigma : sig.pad);
        gg = q.g;
        hh = q.hh;
      } else {
        float U;
        pair_eval<KIND, true>(r2, c, U, gg, hh);
      }
      const float ex = j0.w - qx, ey = j1.x - qy, ez = DIM == 3 ? j1.y - qz : 0.f;
      const float tt = dx * ex + dy * ey + dz * ez;
      const float cdd = (hh - gg) * rcp_nr(r2) * tt;
      gx = fmaf(gg, ex, fmaf(cdd, dx, gx));
      gy = fmaf(gg, ey, fmaf(cdd, dy, gy));
      if (DIM == 3) gz = fmaf(gg, ez, fmaf(cdd, dz, gz));
      if (PARAMS) {
        const float ht = 0.5f * tt;
        acc.add(sj, q.dg_s * ht, q.dg_e * ht, KIND == JMD_LJ ? q.dg_k * ht : 0.f, per_pair);
      }
    }
    if (MODE == 0) {
      float4 xb = a.xbar[i];
      xb.x = fmaf(a.weight, gx, xb.x);
      xb.y = fmaf(a.weight, gy, xb.y);
      if (DIM == 3) xb.z = fmaf(a.weight, gz, xb.z);
      a.xbar[i] = xb;
    }
  }
  if (PARAMS) {
    const int ncol = SPECIES ? tab.nsp : 1;
    if (SPECIES) {
      if (active) acc.flush(bins, si, ncol);
    } else {
      acc.group_sum(kWarp, 1);
      if ((threadIdx.x & (kWarp - 1)) == 0) acc.flush(bins, 0, 1);
    }
    __syncthreads();
    publish_bins(bins, a.gp, MODE == 0 ? (double)a.weight : 1.0);
  }
}

template <int DIM, int KIND, bool SP>
void badj_launch3(int mode, bool params, const BatchView& v, const BAdjArgs& a,
                  const PairTable& t, const PairTable& s, cudaStream_t st) {
  const unsigned gr = (unsigned)std::max<int64_t>(1, ceil_div(v.n, 128));
  if (mode == 1) k_badj_step<DIM, KIND, SP, true, 1><<<gr, 128, 0, st>>>(v, a, t, s);
  else if (params) k_badj_step<DIM, KIND, SP, true, 0><<<gr, 128, 0, st>>>(v, a, t, s);
  else k_badj_step<DIM, KIND, SP, false, 0><<<gr, 128, 0, st>>>(v, a, t, s);
}

int badj_launch(int mode, const jmd_pair& pp, const jmd_batch& bt, const jmd_batch_nlist& nl,
                const float* rec, float* xbar, const int32_t* species, float weight,
                const double* sys_weight, double* gp, cudaStream_t st) {
  if (bt.n_atoms <= 0) return JMD_OK;
  const PairTable t = make_pair_table(pp);
  const PairTable sg = sigma_table(pp);
  const BatchView v = view_of(bt);
  BAdjArgs a{reinterpret_cast<const float4*>(rec), reinterpret_cast<float4*>(xbar), species,
             nl.idx, nl.count, nl.ld, weight, sys_weight, gp, pp.per_pair_cutoff};
  const bool sp = pp.n_species > 0 && species != nullptr, pr = gp != nullptr;
  auto go = [&](auto dimc, auto kindc) {
    constexpr int D = decltype(dimc)::value, K = decltype(kindc)::value;
    if (sp) badj_launch3<D, K, true>(mode, pr, v, a, t, sg, st);
    else badj_launch3<D, K, false>(mode, pr, v, a, t, sg, st);
  };
  using I3 = std::integral_constant<int, 3>;
  using I2 = std::integral_constant<int, 2>;
  using KL = std::integral_constant<int, JMD_LJ>;
  using KT = std::integral_constant<int, JMD_LJ_TRUNCATED>;
  using KS = std::integral_constant<int, JMD_SOFT_SPHERE>;
  using KM = std::integral_constant<int, JMD_MORSE>;
  if (bt.dim == 3) {
    if (pp.kind == JMD_LJ) go(I3{}, KL{});
    else if (pp.kind == JMD_LJ_TRUNCATED) go(I3{}, KT{});
    else if (pp.kind == JMD_MORSE) go(I3{}, KM{});
    else go(I3{}, KS{});
  } else {
    if (pp.kind == JMD_LJ) go(I2{}, KL{});
    else if (pp.kind == JMD_LJ_TRUNCATED) go(I2{}, KT{});
    else if (pp.kind == JMD_MORSE) go(I2{}, KM{});
    else go(I2{}, KS{});
  }
  JMD_CUDA(cudaGetLastError());
  return JMD_OK;
}

// ----------------------------------------------------------------- host ----
int validate_batch(const jmd_batch* b) {
  JMD_REQUIRE(b != nullptr, "batch is null");
  JMD_REQUIRE(b->dim == 2 || b->dim == 3, "dim must be 2 or 3");
  JMD_REQUIRE(b->n_systems >= 1, "a batch needs at least one system");
  JMD_REQUIRE(b->n_atoms >= 0 && b->n_atoms < INT32_MAX, "atom count out of range");
  JMD_REQUIRE(b->sys_offset && b->atom_sys && b->box && b->cell_offset && b->cells_per_side &&
                  b->cell_size,
              "null array in jmd_batch");
  JMD_REQUIRE(b->max_cells >= 1 && b->max_cells <= kMaxBatchCellsShared,
              "a system of the batch has more than 24576 cells (binning runs in shared memory)");
  return JMD_OK;
}

int validate_nl(const jmd_batch_nlist* nl, int64_t n) {
  JMD_REQUIRE(nl != nullptr, "nlist is null");
  JMD_REQUIRE(nl->max_occupancy >= 1 && nl->ld >= nl->max_occupancy, "ld must be >= max_occupancy >= 1");
  JMD_REQUIRE(nl->idx && nl->count && nl->reference_position && nl->occupancy && nl->error_code,
              "null buffer in jmd_batch_nlist");
  JMD_REQUIRE((reinterpret_cast<uintptr_t>(nl->reference_position) % 16) == 0,
              "reference_position must be float4 rows");
  (void)n;
  return JMD_OK;
}

int build_impl(const jmd_batch& b, const jmd_batch_nlist& nl, const float* x, int32_t* flag,
               cudaStream_t st) {
  bool ok = false;
  BWs w = carve(b, nl.workspace, nl.workspace_bytes, &ok);
  if (!ok) return fail(JMD_ERR_WORKSPACE, "batch neighbour-list workspace too small");
  const BatchView v = view_of(b);
  const float4* x4 = reinterpret_cast<const float4*>(x);
  const size_t smem = sizeof(int32_t) * 2 * (size_t)b.max_cells;
  if (b.dim == 3) {
    JMD_CUDA(cudaFuncSetAttribute(k_bbin<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_bbin<3><<<b.n_systems, kBinThreads, smem, st>>>(v, w, x4, flag);
  } else {
    JMD_CUDA(cudaFuncSetAttribute(k_bbin<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_bbin<2><<<b.n_systems, kBinThreads, smem, st>>>(v, w, x4, flag);
  }
  JMD_CUDA(cudaGetLastError());
  SearchArgs a{nl.cutoff_sq, nl.max_occupancy, nl.ld, nl.mask_self, nl.idx, nl.count,
               reinterpret_cast<float4*>(nl.reference_position)};
  const unsigned gr = (unsigned)std::max<int64_t>(1, ceil_div(b.n_atoms, 128));
  if (b.n_atoms > 0) {
    if (b.dim == 3) k_bsearch<3><<<gr, 128, 0, st>>>(v, w, a, flag);
    else k_bsearch<2><<<gr, 128, 0, st>>>(v, w, a, flag);
    JMD_CUDA(cudaGetLastError());
  }
  k_bfinal<<<1, 1, 0, st>>>(w, nl.occupancy, nl.error_code, flag);
  JMD_CUDA(cudaGetLastError());
  return JMD_OK;
}

int skin_impl(const jmd_batch& b, const jmd_batch_nlist& nl, const float* x, float thr2,
              cudaStream_t st) {
  if (b.n_atoms <= 0) return JMD_OK;
  const BatchView v = view_of(b);
  const unsigned gr = (unsigned)ceil_div(b.n_atoms, 256);
  const float4* x4 = reinterpret_cast<const float4*>(x);
  const float4* r4 = reinterpret_cast<const float4*>(nl.reference_position);
  if (b.dim == 3) k_bskin<3><<<gr, 256, 0, st>>>(v, x4, r4, thr2, nl.rebuild_flag);
  else k_bskin<2><<<gr, 256, 0, st>>>(v, x4, r4, thr2, nl.rebuild_flag);
  JMD_CUDA(cudaGetLastError());
  return JMD_OK;
}

template <int DIM, int KIND, bool SP>
void force_launch3(int mode, const BatchView& v, const BForceArgs& a, const PairTable& t,
                   unsigned gr, cudaStream_t st) {
  const int bs = g_force_block;
  if (mode == B_KICK) k_bforce<DIM, KIND, SP, B_KICK><<<gr, bs, 0, st>>>(v, a, t);
  else if (mode == B_FIRE) k_bforce<DIM, KIND, SP, B_FIRE><<<gr, bs, 0, st>>>(v, a, t);
  else k_bforce<DIM, KIND, SP, B_FORCE><<<gr, bs, 0, st>>>(v, a, t);
}

template <int DIM, int KIND>
void force_launch2(int mode, bool sp, const BatchView& v, const BForceArgs& a, const PairTable& t,
                   unsigned gr, double* energy, int nsys, cudaStream_t st) {
  if (sp) force_launch3<DIM, KIND, true>(mode, v, a, t, gr, st);
  else force_launch3<DIM, KIND, false>(mode, v, a, t, gr, st);
  if (energy) {
    if (sp) k_bsys_energy<DIM, KIND, true><<<nsys, 256, 0, st>>>(v, a, t, energy);
    else k_bsys_energy<DIM, KIND, false><<<nsys, 256, 0, st>>>(v, a, t, energy);
  }
}

int force_impl(const jmd_pair& pp, const jmd_batch& b, const jmd_batch_nlist& nl, const float* x,
               const int32_t* species, float* f, float* p, float h, const int32_t* done, int mode,
               double* energy, cudaStream_t st) {
  if (b.n_atoms <= 0) return JMD_OK;
  const PairTable t = make_pair_table(pp);
  const BatchView v = view_of(b);
  BForceArgs a{reinterpret_cast<const float4*>(x), reinterpret_cast<float4*>(f),
               reinterpret_cast<float4*>(p), species, nl.idx, nl.count, nl.ld, h, done};
  const bool sp = pp.n_species > 0 && species != nullptr;
  const unsigned gr = (unsigned)ceil_div(b.n_atoms, g_force_block);
  const int ns = b.n_systems;
  if (b.dim == 3) {
    if (pp.kind == JMD_LJ) force_launch2<3, JMD_LJ>(mode, sp, v, a, t, gr, energy, ns, st);
    else if (pp.kind == JMD_LJ_TRUNCATED) force_launch2<3, JMD_LJ_TRUNCATED>(mode, sp, v, a, t, gr, energy, ns, st);
    else if (pp.kind == JMD_MORSE) force_launch2<3, JMD_MORSE>(mode, sp, v, a, t, gr, energy, ns, st);
    else force_launch2<3, JMD_SOFT_SPHERE>(mode, sp, v, a, t, gr, energy, ns, st);
  } else {
    if (pp.kind == JMD_LJ) force_launch2<2, JMD_LJ>(mode, sp, v, a, t, gr, energy, ns, st);
    else if (pp.kind == JMD_LJ_TRUNCATED) force_launch2<2, JMD_LJ_TRUNCATED>(mode, sp, v, a, t, gr, energy, ns, st);
    else if (pp.kind == JMD_MORSE) force_launch2<2, JMD_MORSE>(mode, sp, v, a, t, gr, energy, ns, st);
    else force_launch2<2, JMD_SOFT_SPHERE>(mode, sp, v, a, t, gr, energy, ns, st);
  }
  JMD_CUDA(cudaGetLastError());
  return JMD_OK;
}

int validate_system(const jmd_batch_system* s, bool fire) {
  JMD_REQUIRE(s != nullptr, "system is null");
  int e = validate_batch(&s->batch);
  if (e) return e;
  e = validate_nl(&s->nlist, s->batch.n_atoms);
  if (e) return e;
  e = validate_pair(&s->pair);
  if (e) return e;
  JMD_REQUIRE(s->position && s->momentum && s->force && s->nlist.rebuild_flag,
              "null buffer in jmd_batch_system");
  for (const void* q : {(const void*)s->position, (const void*)s->momentum, (const void*)s->force})
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(q) % 16) == 0, "float4 rows must be 16-byte aligned");
  JMD_REQUIRE(s->pair.n_species == 0 || s->species != nullptr, "species matrices need species");
  if (fire) JMD_REQUIRE(s->fire_state && s->done && s->n_done, "FIRE needs fire_state, done, n_done");
  return JMD_OK;
}

// One step: kick + drift (+ skin test) -> conditional rebuild -> force (+ the
// closing half kick for NVE, the FIRE update for FIRE).
int enqueue_batch_run(const jmd_batch_system& s, const jmd_fire_params* fp, int64_t steps,
                      bool graphed, cudaStream_t st, cudaStream_t body_st, float* traj = nullptr,
                      bool force_rebuild = false, const jmd_batch_nvt* nvt = nullptr) {
  const jmd_batch& b = s.batch;
  const BatchView v = view_of(b);
  const bool always = s.threshold_sq < 0.f;
  const bool fire = fp != nullptr;
  float4* x = reinterpret_cast<float4*>(s.position);
  float4* p = reinterpret_cast<float4*>(s.momentum);
  float4* f = reinterpret_cast<float4*>(s.force);
  const float4* ref = always ? nullptr : reinterpret_cast<const float4*>(s.nlist.reference_position);
  const unsigned gr = (unsigned)std::max<int64_t>(1, ceil_div(b.n_atoms, 256));
  auto gate = [&]() -> int {
    if (always) return build_impl(b, s.nlist, s.position, nullptr, st);
    if (graphed)
      return graph_conditional(s.nlist.rebuild_flag, [&](cudaStream_t q) {
        return build_impl(b, s.nlist, s.position, s.nlist.rebuild_flag, q);
      }, st, body_st);
    return build_impl(b, s.nlist, s.position, s.nlist.rebuild_flag, st);
  };
  const size_t rows = sizeof(float4) * (size_t)b.n_atoms;
  auto slot = [&](int64_t k) { return traj + (size_t)k * 4 * (size_t)b.n_atoms; };
  if (traj) JMD_CUDA(cudaMemcpyAsync(slot(0), s.position, rows, cudaMemcpyDeviceToDevice, st));
  if (force_rebuild) {
    if (!always) JMD_CUDA(cudaMemsetAsync(s.nlist.rebuild_flag, 1, sizeof(int32_t), st));
    int rc0 = gate();
    if (rc0) return rc0;
  }
  // Nose-Hoover (simulate.py:649-667): chain half step with update_mass on the
  // stored kinetic energy (its scale applied inside the kick) -> velocity
  // Verlet -> chain half step on the measured kinetic energy + rescale.
  const NhcArgs na1 = nvt ? nhc_args(nvt->chain, 1) : NhcArgs{};
  const NhcArgs na0 = nvt ? nhc_args(nvt->chain, 0) : NhcArgs{};
  const double* pscale = nvt ? nvt->p_scale : nullptr;
  auto chain_half = [&](const NhcArgs& na, bool second) {
    if (b.dim == 3)
      k_bnhc<3><<<b.n_systems, second ? 256 : 32, 0, st>>>(
          v, na, nvt->chain_state, second ? p : nullptr, s.mass, s.mass_scalar, second ? 1 : 0,
          nvt->p_scale + (second ? b.n_systems : 0), nullptr);
    else
      k_bnhc<2><<<b.n_systems, second ? 256 : 32, 0, st>>>(
          v, na, nvt->chain_state, second ? p : nullptr, s.mass, s.mass_scalar, second ? 1 : 0,
          nvt->p_scale + (second ? b.n_systems : 0), nullptr);
    return cudaGetLastError();
  };
  for (int64_t k = 0; k < steps; ++k) {
    if (nvt) JMD_CUDA(chain_half(na1, false));
    if (b.dim == 3) {
      if (fire)
        k_bkick_drift<3, true><<<gr, 256, 0, st>>>(v, x, p, f, s.mass, s.mass_scalar, s.dt, s.fire_state,
                                                   s.done, ref, s.threshold_sq, s.nlist.rebuild_flag, nullptr);
      else
        k_bkick_drift<3, false><<<gr, 256, 0, st>>>(v, x, p, f, s.mass, s.mass_scalar, s.dt, nullptr,
                                                    nullptr, ref, s.threshold_sq, s.nlist.rebuild_flag, pscale);
    } else {
      if (fire)
        k_bkick_drift<2, true><<<gr, 256, 0, st>>>(v, x, p, f, s.mass, s.mass_scalar, s.dt, s.fire_state,
                                                   s.done, ref, s.threshold_sq, s.nlist.rebuild_flag, nullptr);
      else
        k_bkick_drift<2, false><<<gr, 256, 0, st>>>(v, x, p, f, s.mass, s.mass_scalar, s.dt, nullptr,
                                                    nullptr, ref, s.threshold_sq, s.nlist.rebuild_flag, pscale);
    }
    JMD_CUDA(cudaGetLastError());
    int rc = gate();
    if (rc) return rc;
    rc = force_impl(s.pair, b, s.nlist, s.position, s.species, s.force, s.momentum, 0.5f * s.dt,
                    s.done, fire ? B_FIRE : B_KICK, nullptr, st);
    if (rc) return rc;
    if (fire) {
      if (b.dim == 3)
        k_bfire_update<3><<<b.n_systems, g_fire_threads, 0, st>>>(v, p, f, s.fire_state, s.done, s.n_done, *fp);
      else
        k_bfire_update<2><<<b.n_systems, g_fire_threads, 0, st>>>(v, p, f, s.fire_state, s.done, s.n_done, *fp);
      JMD_CUDA(cudaGetLastError());
    }
    if (nvt) JMD_CUDA(chain_half(na0, true));
    if (traj) JMD_CUDA(cudaMemcpyAsync(slot(k + 1), s.position, rows, cudaMemcpyDeviceToDevice, st));
  }
  return JMD_OK;
}

// Reverse pass over a recorded segment (slots 0..steps of traj), as
// enqueue_adjoint of the single-system engine.
int enqueue_batch_adjoint(const jmd_batch_system& s, const float* traj, int64_t steps,
                          bool closing, bool opening, float* xbar, float* pbar, float* rec,
                          double* gp, bool graphed, cudaStream_t st, cudaStream_t body_st) {
  const jmd_batch& b = s.batch;
  const BatchView v = view_of(b);
  const bool always = s.threshold_sq < 0.f;
  auto slot = [&](int64_t k) { return traj + (size_t)k * 4 * (size_t)b.n_atoms; };
  auto gate = [&](const float* x) -> int {
    if (always) return build_impl(b, s.nlist, x, nullptr, st);
    if (graphed)
      return graph_conditional(s.nlist.rebuild_flag, [&](cudaStream_t q) {
        return build_impl(b, s.nlist, x, s.nlist.rebuild_flag, q);
      }, st, body_st);
    return build_impl(b, s.nlist, x, s.nlist.rebuild_flag, st);
  };
  const unsigned gr = (unsigned)std::max<int64_t>(1, ceil_div(b.n_atoms, 256));
  const float4* ref = always ? nullptr : reinterpret_cast<const float4*>(s.nlist.reference_position);
  auto rstep = [&](int64_t k, bool kick, float w) -> int {
    const float4* x = reinterpret_cast<const float4*>(slot(k));
    if (b.dim == 3)
      k_badj_pack<3><<<gr, 256, 0, st>>>(v, x, reinterpret_cast<float4*>(xbar),
                                         reinterpret_cast<float4*>(pbar), s.mass, s.mass_scalar,
                                         s.dt, kick ? 1 : 0, reinterpret_cast<float4*>(rec), ref,
                                         s.threshold_sq, s.nlist.rebuild_flag);
    else
      k_badj_pack<2><<<gr, 256, 0, st>>>(v, x, reinterpret_cast<float4*>(xbar),
                                         reinterpret_cast<float4*>(pbar), s.mass, s.mass_scalar,
                                         s.dt, kick ? 1 : 0, reinterpret_cast<float4*>(rec), ref,
                                         s.threshold_sq, s.nlist.rebuild_flag);
    JMD_CUDA(cudaGetLastError());
    int rc = gate(slot(k));
    if (rc) return rc;
    return badj_launch(0, s.pair, b, s.nlist, rec, xbar, s.species, w, nullptr, gp, st);
  };
  if (!always) JMD_CUDA(cudaMemsetAsync(s.nlist.rebuild_flag, 1, sizeof(int32_t), st));
  const float h = 0.5f * s.dt;
  int rc;
  if (closing && (rc = rstep(steps, false, h))) return rc;
  for (int64_t k = steps - 1; k >= 0; --k)
    if ((rc = rstep(k, true, (opening && k == 0) ? h : s.dt))) return rc;
  return JMD_OK;
}

int run_impl(const jmd_batch_system* sys, const jmd_fire_params* fp, int64_t n_steps,
             int32_t use_graph, void* stream, const char* what,
             const jmd_batch_nvt* nvt = nullptr) {
  int e = validate_system(sys, fp != nullptr);
  if (e) return e;
  JMD_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (n_steps == 0 || sys->batch.n_atoms == 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus cap;
  JMD_CUDA(cudaStreamIsCapturing(st, &cap));
  if (!use_graph || cap != cudaStreamCaptureStatusNone) {
    int rc = enqueue_batch_run(*sys, fp, n_steps, false, st, nullptr, nullptr, false, nvt);
    return rc ? rc : check_launch(what);
  }
  int device;
  JMD_CUDA(cudaGetDevice(&device));
  std::string key(what);
  key.append(reinterpret_cast<const char*>(sys), sizeof(*sys));
  const int shape[2] = {g_force_block, g_fire_threads};   // baked into the graph
  key.append(reinterpret_cast<const char*>(shape), sizeof(shape));
  if (fp) key.append(reinterpret_cast<const char*>(fp), sizeof(*fp));
  if (nvt) key.append(reinterpret_cast<const char*>(nvt), sizeof(*nvt));
  key.append(reinterpret_cast<const char*>(&n_steps), sizeof(n_steps));
  key.append(reinterpret_cast<const char*>(&device), sizeof(device));
  return graph_launch_cached(key, [&](cudaStream_t cs, cudaStream_t bs) {
    return enqueue_batch_run(*sys, fp, n_steps, true, cs, bs, nullptr, false, nvt);
  }, st);
}

int graph_or_direct(const std::string& key, const std::function<int(cudaStream_t, cudaStream_t, bool)>& enq,
                    int32_t use_graph, void* stream, const char* what) {
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus cap;
  JMD_CUDA(cudaStreamIsCapturing(st, &cap));
  if (!use_graph || cap != cudaStreamCaptureStatusNone) {
    int rc = enq(st, nullptr, false);
    return rc ? rc : check_launch(what);
  }
  int device;
  JMD_CUDA(cudaGetDevice(&device));
  std::string k = key;
  k.append(reinterpret_cast<const char*>(&device), sizeof(device));
  const int shape[2] = {g_force_block, g_fire_threads};
  k.append(reinterpret_cast<const char*>(shape), sizeof(shape));
  return graph_launch_cached(k, [&](cudaStream_t cs, cudaStream_t bs) { return enq(cs, bs, true); },
                             st);
}

int validate_chain(const jmd_nhc& c, int max_length) {
  JMD_REQUIRE(c.chain_length >= 2 && c.chain_length <= max_length,
              max_length == 16 ? "chain_length must be in 2..16" : "the chain VJP supports chain_length 2..7");
  JMD_REQUIRE(c.chain_steps >= 1, "chain_steps must be >= 1");
  JMD_REQUIRE(c.sy_steps == 1 || c.sy_steps == 3 || c.sy_steps == 5 || c.sy_steps == 7,
              "sy_steps must be 1, 3, 5 or 7");
  return JMD_OK;
}

}  // namespace
}  // namespace jmd

using namespace jmd;

extern "C" {

int jmd_batch_set_launch(int force_block, int fire_threads) {
  JMD_REQUIRE(force_block == 64 || force_block == 128 || force_block == 256,
              "force_block must be 64, 128 or 256");
  JMD_REQUIRE(fire_threads == 256 || fire_threads == 512 || fire_threads == 1024,
              "fire_threads must be 256, 512 or 1024");
  g_force_block = force_block;
  g_fire_threads = fire_threads;
  return JMD_OK;
}

int jmd_batch_nve_run_recorded(const jmd_batch_system* sys, float* trajectory, int64_t n_steps,
                               int32_t force_rebuild, int32_t use_graph, void* stream) {
  int e = validate_system(sys, false);
  if (e) return e;
  JMD_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  JMD_REQUIRE(trajectory == nullptr || (reinterpret_cast<uintptr_t>(trajectory) % 16) == 0,
              "trajectory must be 16-byte aligned float4 rows");
  if (sys->batch.n_atoms == 0) return JMD_OK;
  std::string key("brec");
  key.append(reinterpret_cast<const char*>(sys), sizeof(*sys));
  key.append(reinterpret_cast<const char*>(&trajectory), sizeof(trajectory));
  key.append(reinterpret_cast<const char*>(&n_steps), sizeof(n_steps));
  key.push_back(force_rebuild ? 'f' : '-');
  return graph_or_direct(key, [&](cudaStream_t cs, cudaStream_t bs, bool g) {
    return enqueue_batch_run(*sys, nullptr, n_steps, g, cs, bs, trajectory, force_rebuild != 0);
  }, use_graph, stream, "jmd_batch_nve_run_recorded");
}

int jmd_batch_nve_adjoint_segment(const jmd_batch_system* sys, const float* trajectory,
                                  int64_t n_steps, int32_t closing, int32_t opening, float* xbar,
                                  float* pbar, float* record_scratch, double* grad_params,
                                  int32_t use_graph, void* stream) {
  int e = validate_system(sys, false);
  if (e) return e;
  JMD_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  JMD_REQUIRE(trajectory && xbar && pbar && record_scratch, "null buffer");
  for (const void* q : {(const void*)trajectory, (const void*)xbar, (const void*)pbar,
                        (const void*)record_scratch})
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(q) % 16) == 0, "float4 rows must be 16-byte aligned");
  if (sys->batch.n_atoms == 0 || (n_steps == 0 && !closing)) return JMD_OK;
  std::string key("badj");
  key.append(reinterpret_cast<const char*>(sys), sizeof(*sys));
  for (const void* q : {(const void*)trajectory, (const void*)xbar, (const void*)pbar,
                        (const void*)record_scratch, (const void*)grad_params})
    key.append(reinterpret_cast<const char*>(&q), sizeof(q));
  key.append(reinterpret_cast<const char*>(&n_steps), sizeof(n_steps));
  key.push_back(closing ? 'c' : '-');
  key.push_back(opening ? 'o' : '-');
  return graph_or_direct(key, [&](cudaStream_t cs, cudaStream_t bs, bool g) {
    return enqueue_batch_adjoint(*sys, trajectory, n_steps, closing != 0, opening != 0, xbar,
                                 pbar, record_scratch, grad_params, g, cs, bs);
  }, use_graph, stream, "jmd_batch_nve_adjoint_segment");
}

int jmd_batch_energy_param_grad(const jmd_pair* pair, const jmd_batch* batch,
                                const jmd_batch_nlist* nl, const float* position,
                                const int32_t* species, const double* system_weight,
                                double* grad_params, void* stream) {
  int e = validate_pair(pair);
  if (e) return e;
  if ((e = validate_batch(batch))) return e;
  if ((e = validate_nl(nl, batch->n_atoms))) return e;
  JMD_REQUIRE(position && system_weight && grad_params, "null buffer");
  JMD_REQUIRE((reinterpret_cast<uintptr_t>(position) % 16) == 0, "float4 rows must be 16-byte aligned");
  JMD_REQUIRE(pair->n_species == 0 || species != nullptr, "species matrices need species");
  int rc = badj_launch(1, *pair, *batch, *nl, position, nullptr, species, 1.f, system_weight,
                       grad_params, as_stream(stream));
  return rc ? rc : check_launch("jmd_batch_energy_param_grad");
}

size_t jmd_batch_nlist_workspace_bytes(const jmd_batch* batch) {
  if (!batch) return 0;
  Carver cv(nullptr, 0);
  cv.take<int32_t>(std::max<int64_t>(batch->total_cells, 1));
  cv.take<int32_t>(std::max<int64_t>(batch->total_cells, 1));
  cv.take<int32_t>(std::max<int64_t>(batch->n_atoms, 1));
  cv.take<float4>(std::max<int64_t>(batch->n_atoms, 1));
  cv.take<int32_t>(std::max<int64_t>(batch->n_atoms, 1));
  cv.take<unsigned int>(4);
  return cv.used + 256;
}

int jmd_batch_neighbor_list_build(const jmd_batch* batch, const jmd_batch_nlist* nl,
                                  const float* position, int32_t gated, void* stream) {
  int e = validate_batch(batch);
  if (e) return e;
  e = validate_nl(nl, batch->n_atoms);
  if (e) return e;
  JMD_REQUIRE(position && (reinterpret_cast<uintptr_t>(position) % 16) == 0,
              "position must be float4 rows");
  JMD_REQUIRE(!gated || nl->rebuild_flag, "a gated build needs rebuild_flag");
  int rc = build_impl(*batch, *nl, position, gated ? nl->rebuild_flag : nullptr, as_stream(stream));
  return rc ? rc : check_launch("jmd_batch_neighbor_list_build");
}

int jmd_batch_skin_check(const jmd_batch* batch, const jmd_batch_nlist* nl, const float* position,
                         float threshold_sq, void* stream) {
  int e = validate_batch(batch);
  if (e) return e;
  e = validate_nl(nl, batch->n_atoms);
  if (e) return e;
  JMD_REQUIRE(nl->rebuild_flag != nullptr, "skin check needs rebuild_flag");
  int rc = skin_impl(*batch, *nl, position, threshold_sq, as_stream(stream));
  return rc ? rc : check_launch("jmd_batch_skin_check");
}

int jmd_batch_pair_forces(const jmd_pair* pair, const jmd_batch* batch, const jmd_batch_nlist* nl,
                          const float* position, const int32_t* species, float* force,
                          double* energy, void* stream) {
  int e = validate_pair(pair);
  if (e) return e;
  e = validate_batch(batch);
  if (e) return e;
  e = validate_nl(nl, batch->n_atoms);
  if (e) return e;
  JMD_REQUIRE(position && force, "null buffer");
  JMD_REQUIRE(pair->n_species == 0 || species != nullptr, "species matrices need species");
  for (const void* q : {(const void*)position, (const void*)force})
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(q) % 16) == 0, "float4 rows must be 16-byte aligned");
  int rc = force_impl(*pair, *batch, *nl, position, species, force, nullptr, 0.f, nullptr, B_FORCE,
                      energy, as_stream(stream));
  return rc ? rc : check_launch("jmd_batch_pair_forces");
}

int jmd_batch_dot_per_system(const jmd_batch* batch, const float* a, int64_t a_stride,
                             const float* c, int64_t c_stride, double* out, void* stream) {
  int e = validate_batch(batch);
  if (e) return e;
  JMD_REQUIRE(a && c && out, "null buffer");
  const BatchView v = view_of(*batch);
  cudaStream_t st = as_stream(stream);
  if (batch->dim == 3) k_bdot<3><<<batch->n_systems, 256, 0, st>>>(v, a, a_stride, c, c_stride, out);
  else k_bdot<2><<<batch->n_systems, 256, 0, st>>>(v, a, a_stride, c, c_stride, out);
  return check_launch("jmd_batch_dot_per_system");
}

int jmd_batch_nvt_adjoint_update(const jmd_batch* batch, int32_t stage, const float* in_a,
                                 const float* in_b, int64_t b_stride, const double* scale,
                                 const double* kebar, float inv_m, float coef,
                                 const float* pending, float* out_a, float* out_b,
                                 double* sums, void* stream) {
  int e = validate_batch(batch);
  if (e) return e;
  JMD_REQUIRE(stage >= 0 && stage <= 2, "stage must be 0, 1 or 2");
  const BatchView v = view_of(*batch);
  cudaStream_t st = as_stream(stream);
  const unsigned gr = (unsigned)std::max<int64_t>(1, ceil_div(v.n, 256));
  const bool d3 = batch->dim == 3;
  if (stage == 0) {  // rbar, lam4 from pbar (in_a), r (in_b)
    JMD_REQUIRE(in_a && in_b && scale && kebar && out_a && out_b, "null buffer");
    if (d3) k_bnvt_pre<3><<<gr, 256, 0, st>>>(v, in_a, in_b, b_stride, scale, kebar, inv_m, coef, pending, out_a, out_b);
    else k_bnvt_pre<2><<<gr, 256, 0, st>>>(v, in_a, in_b, b_stride, scale, kebar, inv_m, coef, pending, out_a, out_b);
  } else if (stage == 1) {  // qbar (out_a) and sums from rbar (in_a), xbar4 (pending), p_k (in_b)
    JMD_REQUIRE(in_a && in_b && pending && out_a && sums, "null buffer");
    if (d3) k_bnvt_post<3><<<batch->n_systems, 256, 0, st>>>(v, in_a, pending, coef, in_b, b_stride, out_a, sums);
    else k_bnvt_post<2><<<batch->n_systems, 256, 0, st>>>(v, in_a, pending, coef, in_b, b_stride, out_a, sums);
  } else {  // pbar (out_a) from qbar (in_a), p_k (in_b)
    JMD_REQUIRE(in_a && in_b && scale && kebar && out_a, "null buffer");
    if (d3) k_bnvt_pbar<3><<<gr, 256, 0, st>>>(v, in_a, scale, kebar, in_b, b_stride, inv_m, out_a);
    else k_bnvt_pbar<2><<<gr, 256, 0, st>>>(v, in_a, scale, kebar, in_b, b_stride, inv_m, out_a);
  }
  return check_launch("jmd_batch_nvt_adjoint_update");
}

int jmd_batch_kinetic_energy(const jmd_batch* batch, const float* momentum, const float* force,
                             const float* mass, float mass_scalar, double* ke, float* fmax,
                             void* stream) {
  int e = validate_batch(batch);
  if (e) return e;
  JMD_REQUIRE(!ke || momentum, "ke needs momentum");
  JMD_REQUIRE(!fmax || force, "fmax needs force");
  const BatchView v = view_of(*batch);
  cudaStream_t st = as_stream(stream);
  const float4* p4 = reinterpret_cast<const float4*>(momentum);
  const float4* f4 = reinterpret_cast<const float4*>(force);
  if (batch->dim == 3) k_bke<3><<<batch->n_systems, 256, 0, st>>>(v, p4, f4, mass, mass_scalar, ke, fmax);
  else k_bke<2><<<batch->n_systems, 256, 0, st>>>(v, p4, f4, mass, mass_scalar, ke, fmax);
  return check_launch("jmd_batch_kinetic_energy");
}

int jmd_batch_fire_init(const jmd_batch_system* sys, const jmd_fire_params* fp, void* stream) {
  int e = validate_system(sys, true);
  if (e) return e;
  JMD_REQUIRE(fp != nullptr, "fire params are null");
  const int ns = sys->batch.n_systems;
  k_bfire_init<<<(unsigned)ceil_div(ns, 128), 128, 0, as_stream(stream)>>>(
      ns, sys->fire_state, sys->done, sys->n_done, fp->dt_start, fp->alpha_start);
  return check_launch("jmd_batch_fire_init");
}

int jmd_batch_nve_run(const jmd_batch_system* sys, int64_t n_steps, int32_t use_graph,
                      void* stream) {
  return run_impl(sys, nullptr, n_steps, use_graph, stream, "jmd_batch_nve_run");
}

int jmd_batch_fire_run(const jmd_batch_system* sys, const jmd_fire_params* fp, int64_t n_steps,
                       int32_t use_graph, void* stream) {
  JMD_REQUIRE(fp != nullptr, "fire params are null");
  return run_impl(sys, fp, n_steps, use_graph, stream, "jmd_batch_fire_run");
}

int jmd_batch_nvt_run(const jmd_batch_system* sys, const jmd_batch_nvt* nvt, int64_t n_steps,
                      int32_t use_graph, void* stream) {
  JMD_REQUIRE(nvt != nullptr && nvt->chain_state && nvt->p_scale, "null chain buffer");
  int e = validate_chain(nvt->chain, 16);
  if (e) return e;
  return run_impl(sys, nullptr, n_steps, use_graph, stream, "jmd_batch_nvt_run", nvt);
}

int jmd_batch_nhc_half_step(const jmd_batch* batch, const jmd_batch_nvt* nvt, float* momentum,
                            const float* mass, float mass_scalar, int32_t update_mass,
                            int32_t measure_ke, double* scale_out, double* ke_out, void* stream) {
  int e = validate_batch(batch);
  if (e) return e;
  JMD_REQUIRE(nvt != nullptr && nvt->chain_state, "null chain buffer");
  e = validate_chain(nvt->chain, 16);
  if (e) return e;
  JMD_REQUIRE(!measure_ke || momentum, "measuring the kinetic energy needs the momenta");
  JMD_REQUIRE(!momentum || (reinterpret_cast<uintptr_t>(momentum) % 16) == 0,
              "float4 rows must be 16-byte aligned");
  const BatchView v = view_of(*batch);
  const NhcArgs a = nhc_args(nvt->chain, update_mass);
  float4* p = reinterpret_cast<float4*>(momentum);
  const unsigned th = (p || measure_ke) ? 256 : 32;
  if (batch->dim == 3)
    k_bnhc<3><<<batch->n_systems, th, 0, as_stream(stream)>>>(v, a, nvt->chain_state, p, mass,
                                                             mass_scalar, measure_ke ? 1 : 0,
                                                             scale_out, ke_out);
  else
    k_bnhc<2><<<batch->n_systems, th, 0, as_stream(stream)>>>(v, a, nvt->chain_state, p, mass,
                                                             mass_scalar, measure_ke ? 1 : 0,
                                                             scale_out, ke_out);
  return check_launch("jmd_batch_nhc_half_step");
}

int jmd_batch_nhc_half_step_vjp(const jmd_batch* batch, const jmd_nhc* c, const double* chain,
                                const double* kinetic_energy, int32_t update_mass,
                                const double* cot_p_xi, const double* cot_scale,
                                double* grad_p_xi, double* grad_kinetic_energy, void* stream) {
  int e = validate_batch(batch);
  if (e) return e;
  JMD_REQUIRE(c != nullptr, "chain constants are null");
  e = validate_chain(*c, 7);
  if (e) return e;
  JMD_REQUIRE(chain && kinetic_energy && cot_p_xi && cot_scale && grad_p_xi && grad_kinetic_energy,
              "null buffer");
  const NhcArgs a = nhc_args(*c, update_mass);
  const int ns = batch->n_systems;
  k_bnhc_vjp<<<(unsigned)ceil_div(ns, 64), 64, 0, as_stream(stream)>>>(
      a, ns, batch->sys_offset, batch->dim, chain, kinetic_energy, cot_p_xi, cot_scale, grad_p_xi,
      grad_kinetic_energy);
  return check_launch("jmd_batch_nhc_half_step_vjp");
}

int jmd_batch_pair_force_vjp(const jmd_pair* pair, const jmd_batch* batch,
                             const jmd_batch_nlist* nl, const float* position,
                             const float* cotangent, const int32_t* species, float weight,
                             float* grad_position, double* grad_params, float* record_scratch,
                             void* stream) {
  JMD_REQUIRE(pair != nullptr, "pair is null");
  int e = validate_batch(batch);
  if (e) return e;
  e = validate_nl(nl, batch->n_atoms);
  if (e) return e;
  e = validate_pair(pair);
  if (e) return e;
  JMD_REQUIRE(position && cotangent && grad_position && record_scratch, "null buffer");
  for (const void* q : {(const void*)position, (const void*)cotangent, (const void*)grad_position,
                        (const void*)record_scratch})
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(q) % 16) == 0, "float4 rows must be 16-byte aligned");
  JMD_REQUIRE(pair->n_species == 0 || species != nullptr, "species matrices need species");
  if (batch->n_atoms == 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  const int n = (int)batch->n_atoms;
  const unsigned gr = (unsigned)ceil_div(n, 256);
  const float4* x = reinterpret_cast<const float4*>(position);
  const float4* lam = reinterpret_cast<const float4*>(cotangent);
  float4* rec = reinterpret_cast<float4*>(record_scratch);
  if (batch->dim == 3) k_bvjp_pack<3><<<gr, 256, 0, st>>>(n, x, lam, rec);
  else k_bvjp_pack<2><<<gr, 256, 0, st>>>(n, x, lam, rec);
  JMD_CUDA(cudaGetLastError());
  int rc = badj_launch(0, *pair, *batch, *nl, record_scratch, grad_position, species, weight,
                       nullptr, grad_params, st);
  return rc ? rc : check_launch("jmd_batch_pair_force_vjp");
}

}  // extern "C"
