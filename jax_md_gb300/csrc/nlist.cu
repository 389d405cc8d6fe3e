// Cell binning (counting sort) and neighbour-list construction.
//
// Reference: jax_md/partition.py
//   cell hashing            :212-224, 421-423
//   cell slot rule          :438-447  slot = hash*cap + (sorted_rank mod cap)
//   candidate order         :911-951  3^d shifted cells (first axis slowest),
//                                     slots 0..cap-1 within each cell
//   self mask / prune       :953-1032 strict d^2 < cutoff^2, stable compaction
//   capacity / overflow     :1090-1117
//   skin test               :1146-1154
//
// GB300 design.  Binning is a counting sort: a histogram (atomics), one
// exclusive scan, a scatter, and a per-cell rank pass that restores the
// stable (ascending id) order of the reference's argsort; atoms end up
// reordered by cell in `sorted_pos` (float4) so that the neighbour search
// reads every candidate cell as one contiguous, coalesced range.  The search
// runs one warp per atom, visits candidates in the reference's order
// (including the slot rotation that the reference's `rank mod cap` slot rule
// implies), and compacts hits with a warp ballot straight into the atom's
// row, so the Dense list is bit-identical to the reference's, order included.
#include "dense.cuh"
#include "segment.cuh"

namespace jmd {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // per thread per tile
constexpr int kScanTile = kScanThreads * kScanItems;

// Internal scalars kept in the workspace.
struct Scalars {
  unsigned int max_fill;
  unsigned int flags;
  unsigned long long occupancy;  // Dense: max row count; Sparse: total
  unsigned int sparse_total_hi;  // unused padding
  unsigned int counter;
};

struct Bins {
  int32_t* cell_of;    // [N]
  int32_t* count;      // [C]
  int32_t* start;      // [C+1]
  int32_t* cursor;     // [C]
  int32_t* tmp_id;     // [N]
  int32_t* sorted_id;  // [N]
  float4* sorted_pos;  // [N]
  int32_t* blocksum;   // [ceil(C/tile)] (also used for atom scans)
  int32_t* atom_off;   // [N+1] sparse row offsets
  Scalars* sc;
};

struct Grid {
  int dim;
  int cps[3];
  float cs[3];
  int mult[3];
  int64_t count;
};

inline Grid make_grid(const jmd_nlist& nl) {
  Grid g;
  g.dim = nl.space.dim;
  g.count = 1;
  for (int d = 0; d < 3; ++d) {
    g.cps[d] = d < g.dim ? nl.cells_per_side[d] : 1;
    g.cs[d] = d < g.dim ? nl.cell_size[d] : 1.f;
  }
  g.mult[0] = 1;
  g.mult[1] = g.cps[0];
  g.mult[2] = g.cps[0] * g.cps[1];
  for (int d = 0; d < g.dim; ++d) g.count *= g.cps[d];
  return g;
}

int64_t grid_count(const jmd_nlist& nl) {
  if (!nl.use_cell_list) return 1;
  return make_grid(nl).count;
}

size_t bins_bytes(int64_t n, int64_t c) {
  Carver cv(nullptr, 0);
  cv.take<int32_t>(n);
  cv.take<int32_t>(c);
  cv.take<int32_t>(c + 1);
  cv.take<int32_t>(c);
  cv.take<int32_t>(n);
  cv.take<int32_t>(n);
  cv.take<float4>(n);
  cv.take<int32_t>(ceil_div(std::max(c, n + 1), kScanTile) + 1);
  cv.take<int32_t>(n + 1);
  cv.take<Scalars>(1);
  return cv.used + 256;
}

Bins carve_bins(void* ws, size_t bytes, int64_t n, int64_t c, bool* ok) {
  Carver cv(ws, bytes);
  Bins b;
  b.cell_of = cv.take<int32_t>(n);
  b.count = cv.take<int32_t>(c);
  b.start = cv.take<int32_t>(c + 1);
  b.cursor = cv.take<int32_t>(c);
  b.tmp_id = cv.take<int32_t>(n);
  b.sorted_id = cv.take<int32_t>(n);
  b.sorted_pos = cv.take<float4>(n);
  b.blocksum = cv.take<int32_t>(ceil_div(std::max(c, n + 1), kScanTile) + 1);
  b.atom_off = cv.take<int32_t>(n + 1);
  b.sc = cv.take<Scalars>(1);
  *ok = cv.ok();
  return b;
}

__device__ __forceinline__ bool skip(const int32_t* flag) { return flag != nullptr && *flag == 0; }

// int(x / cell_size) mod cells_per_side, float32 division as the reference.
__device__ __forceinline__ int cell_coord(float x, float cs, int cps) {
  int q = __float2int_rz(__fdiv_rn(x, cs));
  int m = q % cps;
  return m < 0 ? m + cps : m;
}

template <int DIM>
__device__ __forceinline__ int cell_hash(float4 x, const Grid& g, int* c3) {
  c3[0] = cell_coord(x.x, g.cs[0], g.cps[0]);
  c3[1] = cell_coord(x.y, g.cs[1], g.cps[1]);
  c3[2] = DIM == 3 ? cell_coord(x.z, g.cs[2], g.cps[2]) : 0;
  return c3[0] + c3[1] * g.mult[1] + (DIM == 3 ? c3[2] * g.mult[2] : 0);
}

// ----------------------------------------------------------- binning -------
__global__ void k_zero(int32_t* count, int64_t c, Scalars* sc, const int32_t* flag) {
  if (skip(flag)) return;
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int64_t k = t; k < c; k += (int64_t)gridDim.x * blockDim.x) count[k] = 0;
  if (t == 0) {
    sc->max_fill = 0;
    sc->flags = 0;
    sc->occupancy = 0;
    sc->counter = 0;
  }
}

template <int DIM, bool VEC4>
__global__ void k_bin(const float* __restrict__ x, int64_t stride, int n, Grid g, Bins b,
                      int32_t* particle_cell_id, const int32_t* flag) {
  if (skip(flag)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 r = load_row<DIM, VEC4>(x, stride, i);
  int c3[3];
  int h = cell_hash<DIM>(r, g, c3);
  b.cell_of[i] = h;
  atomicAdd(b.count + h, 1);
  if (particle_cell_id) {
    for (int d = 0; d < DIM; ++d) particle_cell_id[(int64_t)i * DIM + d] = c3[d];
  }
}

// Exclusive scan of `in[0..len)` into out[0..len] (out[len] = total), also
// copying the result into `copy` (cursor) when given and taking the max of
// the inputs into *max_out.  One block walks the array tile by tile.
__global__ void __launch_bounds__(kScanThreads)
k_scan_single(const int32_t* __restrict__ in, int64_t len, int32_t* out, int32_t* copy,
              unsigned int* max_out, const int32_t* flag) {
  if (skip(flag)) return;
  __shared__ int32_t warp_tot[32];
  __shared__ int32_t carry_s;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  int32_t carry = 0;
  int32_t vmax = 0;
  for (int64_t base = 0; base < len; base += kScanTile) {
    int32_t v[kScanItems];
    int32_t tsum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      int64_t idx = base + (int64_t)t * kScanItems + k;
      v[k] = idx < len ? in[idx] : 0;
      vmax = max(vmax, v[k]);
      tsum += v[k];
    }
    // inclusive warp scan of thread sums
    int32_t incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      int32_t w = warp_tot[lane];
      int32_t wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += y;
      }
      warp_tot[lane] = wi - w;  // exclusive warp offsets
      if (lane == 31) carry_s = wi;
    }
    __syncthreads();
    int32_t run = carry + warp_tot[warp] + incl - tsum;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      int64_t idx = base + (int64_t)t * kScanItems + k;
      if (idx < len) {
        out[idx] = run;
        if (copy) copy[idx] = run;
      }
      run += v[k];
    }
    carry += carry_s;
    __syncthreads();
  }
  if (t == 0) out[len] = carry;
  // block max
  for (int o = 16; o > 0; o >>= 1) vmax = max(vmax, __shfl_down_sync(0xffffffffu, vmax, o));
  if (lane == 0 && max_out) atomicMax(max_out, (unsigned int)vmax);
}

__global__ void k_scatter(int n, Bins b, const int32_t* flag) {
  if (skip(flag)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int pos = atomicAdd(b.cursor + b.cell_of[i], 1);
  b.tmp_id[pos] = i;
}

// One warp per cell: rank every member by id (stable argsort order of the
// reference) and write the cell-sorted id and position arrays.
template <int DIM, bool VEC4>
__global__ void k_cell_rank(const float* __restrict__ x, int64_t stride, int64_t ncell, Bins b,
                            const int32_t* flag) {
  if (skip(flag)) return;
  int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (c >= ncell) return;
  int beg = b.start[c], end = b.start[c + 1];
  int k = end - beg;
  for (int base = 0; base < k; base += 32) {
    const int a = base + lane;
    int mine = a < k ? b.tmp_id[beg + a] : INT32_MAX;
    int rank = 0;
    for (int q = 0; q < k; q += 32) {
      int other = (q + lane) < k ? b.tmp_id[beg + q + lane] : INT32_MAX;
#pragma unroll 8
      for (int s = 0; s < 32; ++s) {
        int o = __shfl_sync(0xffffffffu, other, s);
        rank += (o < mine);
      }
    }
    if (a < k) {
      b.sorted_id[beg + rank] = mine;
      // the fourth float travels with the atom (the engine keeps species ids
      // there; plain rows have w = 0 and strided rows load it as 0)
      b.sorted_pos[beg + rank] = load_row<DIM, VEC4>(x, stride, mine);
    }
  }
}

// Reference layout of the cell list (partition.py:425-452).
template <int DIM>
__global__ void k_fill_cell_buffers(int64_t ncell, int cap, int n, int32_t* id_buffer,
                                    float* position_buffer) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t total = ncell * cap;
  for (int64_t s = t; s < total; s += (int64_t)gridDim.x * blockDim.x) {
    id_buffer[s] = n;
    if (position_buffer)
      for (int d = 0; d < DIM; ++d) position_buffer[s * DIM + d] = 0.f;
  }
}

template <int DIM>
__global__ void k_emplace(int n, int cap, Grid g, Bins b, int32_t* id_buffer,
                          float* position_buffer) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int i = b.sorted_id[s];
  int h = b.cell_of[i];
  int64_t slot = (int64_t)h * cap + (s % cap);
  id_buffer[slot] = i;
  if (position_buffer) {
    float4 r = b.sorted_pos[s];
    position_buffer[slot * DIM + 0] = r.x;
    position_buffer[slot * DIM + 1] = r.y;
    if (DIM == 3) position_buffer[slot * DIM + 2] = r.z;
  }
}

// ---------------------------------------------------- neighbour search -----
struct SearchArgs {
  Geo geo;
  Grid grid;
  float cut2;
  int mask_self;
  int ordered;   // OrderedSparse: keep j < i
  int cap;       // cell capacity (slot rotation)
  int n;
  int64_t width; // Dense row width (max_occupancy)
};

template <int DIM>
__device__ __forceinline__ float dist2(const float4& a, const float4& b, const Geo& g) {
  float dx, dy, dz = 0.f;
  if (g.periodic) {
    dx = min_image(a.x, b.x, g.L[0], g.halfL[0]);
    dy = min_image(a.y, b.y, g.L[1], g.halfL[1]);
    if (DIM == 3) dz = min_image(a.z, b.z, g.L[2], g.halfL[2]);
    if (g.general) cell_apply<DIM>(g.T, dx, dy, dz);
  } else {
    dx = a.x - b.x;
    dy = a.y - b.y;
    if (DIM == 3) dz = a.z - b.z;
  }
  float d2 = dx * dx;
  d2 = fmaf(dy, dy, d2);
  if (DIM == 3) d2 = fmaf(dz, dz, d2);
  return d2;
}

// Visits candidates sid/spos[beg, end) in order; appends hits to `row`
// (entries at positions >= row_cap are dropped but still counted).
// Sparse rows also write the sender id into `row2`.
template <int DIM>
__device__ __forceinline__ void visit(int beg, int end, const int32_t* __restrict__ sid,
                                      const float4* __restrict__ spos, float4 xi, int i,
                                      const SearchArgs& a, int lane, int& count, int32_t* row,
                                      int32_t* row2, int64_t row_cap) {
  const unsigned lt = (1u << lane) - 1u;
  for (int base = beg; base < end; base += 32) {
    int s = base + lane;
    bool ok = false;
    int j = 0;
    if (s < end) {
      j = sid ? __ldg(sid + s) : s;
      float4 xj = __ldg(spos + s);
      float d2 = dist2<DIM>(xi, xj, a.geo);
      ok = d2 < a.cut2;
      if (a.mask_self) ok = ok && (j != i);
      if (a.ordered) ok = ok && (j < i);
    }
    unsigned m = __ballot_sync(0xffffffffu, ok);
    if (ok && row) {
      int64_t p = (int64_t)count + __popc(m & lt);
      if (p < row_cap) {
        row[p] = j;
        if (row2) row2[p] = i;
      }
    }
    count += __popc(m);
  }
}

// All candidates of atom i in the reference's order.  Cell-list path: 3^d
// shifted cells, first axis slowest (partition.py:232-240), each cell's
// members in slot order 0..cap-1; the slot of member r of a cell starting at
// sorted position b is (b + r) mod cap, i.e. the members with r >= cap - o
// (o = b mod cap) come first.
template <int DIM, bool CELLS>
__device__ __forceinline__ void search(const Bins& b, const float4* __restrict__ allpos,
                                       float4 xi, int i, const SearchArgs& a, int lane,
                                       int& count, int32_t* row, int32_t* row2, int64_t row_cap) {
  if (!CELLS) {
    visit<DIM>(0, a.n, nullptr, allpos, xi, i, a, lane, count, row, row2, row_cap);
    return;
  }
  int c3[3];
  cell_hash<DIM>(xi, a.grid, c3);
  const int ns = DIM == 3 ? 27 : 9;
  for (int k = 0; k < ns; ++k) {
    int sh0, sh1, sh2;
    if (DIM == 3) {
      sh0 = k / 9 - 1;
      sh1 = (k / 3) % 3 - 1;
      sh2 = k % 3 - 1;
    } else {
      sh0 = k / 3 - 1;
      sh1 = k % 3 - 1;
      sh2 = 0;
    }
    int q0 = c3[0] + sh0, q1 = c3[1] + sh1, q2 = c3[2] + sh2;
    q0 = q0 < 0 ? q0 + a.grid.cps[0] : (q0 >= a.grid.cps[0] ? q0 - a.grid.cps[0] : q0);
    q1 = q1 < 0 ? q1 + a.grid.cps[1] : (q1 >= a.grid.cps[1] ? q1 - a.grid.cps[1] : q1);
    if (DIM == 3)
      q2 = q2 < 0 ? q2 + a.grid.cps[2] : (q2 >= a.grid.cps[2] ? q2 - a.grid.cps[2] : q2);
    int h = q0 + q1 * a.grid.mult[1] + (DIM == 3 ? q2 * a.grid.mult[2] : 0);
    int beg = __ldg(b.start + h), end = __ldg(b.start + h + 1);
    int kk = end - beg;
    int split = a.cap - (beg % a.cap);
    if (kk <= split) {
      visit<DIM>(beg, end, b.sorted_id, b.sorted_pos, xi, i, a, lane, count, row, row2, row_cap);
    } else {
      visit<DIM>(beg + split, end, b.sorted_id, b.sorted_pos, xi, i, a, lane, count, row, row2,
                 row_cap);
      visit<DIM>(beg, beg + split, b.sorted_id, b.sorted_pos, xi, i, a, lane, count, row, row2,
                 row_cap);
    }
  }
}

// Mode: 0 = Dense write, 1 = count only (per atom into atom_off), 2 = Sparse write.
template <int DIM, bool CELLS, bool VEC4, int MODE>
__global__ void __launch_bounds__(256)
k_search(const float* __restrict__ x, int64_t stride, Bins b, SearchArgs a, int32_t* idx,
         int64_t ld, int32_t* nbr_count, float* ref, int64_t ref_stride, const int32_t* flag,
         const float4* __restrict__ allpos) {
  if (skip(flag)) return;
  int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= a.n) return;
  int i;
  float4 xi;
  if (CELLS) {
    i = b.sorted_id[w];
    xi = b.sorted_pos[w];
  } else {
    i = (int)w;
    xi = allpos[w];
  }
  int count = 0;
  int32_t* row = nullptr;
  int32_t* row2 = nullptr;
  int64_t row_cap = 0;
  if (MODE == 0 && idx) {
    row = idx + (int64_t)i * ld;
    row_cap = a.width;
  } else if (MODE == 2) {
    int64_t off = b.atom_off[i];
    row = idx + off;
    row2 = idx + ld + off;
    row_cap = a.width - off;  // entries past the capacity are dropped
  }
  search<DIM, CELLS>(b, allpos, xi, i, a, lane, count, row, row2, row_cap);
  if (MODE == 0) {
    if (row) {
      for (int64_t p = min((int64_t)count, a.width) + lane; p < a.width; p += 32) row[p] = a.n;
    }
    if (lane == 0) {
      if (nbr_count) nbr_count[i] = count;
      atomicMax(&b.sc->occupancy, (unsigned long long)count);
      if (count > a.width) atomicOr(&b.sc->flags, (unsigned)JMD_NEIGHBOR_LIST_OVERFLOW);
    }
  } else if (MODE == 1) {
    if (lane == 0) b.atom_off[i] = count;
  }
  if (ref && lane == 0) {
    float4 r = load_row<DIM, VEC4>(x, stride, i);
    store_row_full<DIM, false>(ref, ref_stride, i, r);
  }
}

// Cell-staged Dense search: one CTA per cell.  The CTA stages the members
// of the 3^d neighbour cells into shared memory in the reference's candidate
// order (shift order, slot rotation within each cell), then every warp takes
// one atom of the centre cell and scans the whole candidate stream in chunks
// of 64 (two candidates per lane), so lanes stay busy across cell borders and
// each candidate position is read from global memory once per cell rather
// than once per atom.  Cells whose stream exceeds the shared-memory budget read
// the same stream from global memory instead.
constexpr int kStageMax = 1024;

template <int DIM>
struct CellStream {
  int beg[27], cnt[27], split[27], off[28];
};

template <int DIM>
__device__ __forceinline__ int stream_index(const CellStream<DIM>& cs, int ns, int t) {
  // largest k with off[k] <= t
  int lo = 0, hi = ns - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (cs.off[mid] <= t) lo = mid; else hi = mid - 1;
  }
  const int k = lo;
  const int r = t - cs.off[k];
  const int c = cs.cnt[k], sp = cs.split[k];
  int m;
  if (c <= sp) {
    m = r;
  } else {
    const int l1 = c - sp;
    m = r < l1 ? sp + r : r - l1;
  }
  return cs.beg[k] + m;
}

// Search geometry of one CTA.
//   PLAIN : free space, raw differences.
//   FRAME : periodic with >= 4 cells per side.  Every staged coordinate is
//           moved into the centre cell's frame by subtracting 0 or L (exact,
//           Sterbenz: only coordinates >= L/2 are shifted), after folding a
//           coordinate equal to L back to 0; plain differences of the moved
//           coordinates are then the minimum image with a single rounding.
//   EXACT : periodic with 3 cells on some side: exact minimum image per test.
enum { S_PLAIN = 0, S_FRAME = 1, S_EXACT = 2 };

template <int DIM, int GEOM>
__device__ __forceinline__ void test2(const float4& xa, const float4& xb, const float4& c,
                                      const SearchArgs& a, float& d0, float& d1) {
  if (GEOM == S_EXACT) {
    d0 = dist2<DIM>(xa, c, a.geo);
    d1 = dist2<DIM>(xb, c, a.geo);
    return;
  }
  float2 dx = __ffma2_rn(make_float2(c.x, c.x), make_float2(-1.f, -1.f), make_float2(xa.x, xb.x));
  float2 dy = __ffma2_rn(make_float2(c.y, c.y), make_float2(-1.f, -1.f), make_float2(xa.y, xb.y));
  float2 r2 = __fmul2_rn(dx, dx);
  r2 = __ffma2_rn(dy, dy, r2);
  if (DIM == 3) {
    float2 dz = __ffma2_rn(make_float2(c.z, c.z), make_float2(-1.f, -1.f), make_float2(xa.z, xb.z));
    r2 = __ffma2_rn(dz, dz, r2);
  }
  d0 = r2.x;
  d1 = r2.y;
}

// Scans the cell's candidate stream for the centre atoms ia / ib (ib < 0: none)
// and appends hits to their rows in stream order.  Lanes own candidates.
template <int DIM, int GEOM, bool MASK_SELF>
__device__ __forceinline__ void scan_pair(const CellStream<DIM>& cs, int ns, int total,
                                          bool staged, const float4* __restrict__ spos,
                                          const Bins& b, int ia, float4 xa, int ib, float4 xb,
                                          const SearchArgs& a, int lane, int& ca, int& cb,
                                          int32_t* ra, int32_t* rb, int row_cap, int rs) {
  const unsigned lt = (1u << lane) - 1u;
  for (int base = 0; base < total; base += 32) {
    const int t = base + lane;
    bool oka = false, okb = false;
    int j = 0;
    if (t < total) {
      float4 c;
      if (staged) {
        c = spos[t];
      } else {
        const int s = stream_index<DIM>(cs, ns, t);
        c = __ldg(b.sorted_pos + s);
        c.w = __int_as_float(__ldg(b.sorted_id + s));
      }
      j = __float_as_int(c.w);
      float d0, d1;
      test2<DIM, GEOM>(xa, xb, c, a, d0, d1);
      oka = d0 < a.cut2;
      okb = d1 < a.cut2 && ib >= 0;
      if (MASK_SELF) {
        oka = oka && j != ia;
        okb = okb && j != ib;
      }
    }
    const unsigned ma = __ballot_sync(0xffffffffu, oka);
    const unsigned mb = __ballot_sync(0xffffffffu, okb);
    const int pa = ca + __popc(ma & lt);
    const int pb = cb + __popc(mb & lt);
    if (oka && pa < row_cap) ra[pa * rs] = j;
    if (okb && pb < row_cap) rb[pb * rs] = j;
    ca += __popc(ma);
    cb += __popc(mb);
  }
}

// TILED: rows go to the engine's tiled layout (entry k of atom i at
// idx[(i/32)*ld*32 + k*32 + i%32]) without padding; otherwise row-major
// [n, ld] padded with n up to max_occupancy.
template <int DIM, bool TILED>
__global__ void __launch_bounds__(128)
k_search_cells(const float* __restrict__ x, int64_t stride, Bins b, SearchArgs a, int32_t* idx,
               int64_t ld, int32_t* nbr_count, float* ref, int64_t ref_stride,
               const int32_t* flag) {
  if (skip(flag)) return;
  extern __shared__ float4 spos[];  // kStageMax candidates: xyz + id (as the w bits)
  __shared__ CellStream<DIM> cs;
  __shared__ float soff[27][3];     // per neighbour cell: amount subtracted (FRAME)
  __shared__ float coff[3];         // for the centre cell's atoms
  const int c = blockIdx.x;
  const int ns = DIM == 3 ? 27 : 9;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int cc[3];
  cc[0] = c % a.grid.cps[0];
  cc[1] = (c / a.grid.cps[0]) % a.grid.cps[1];
  cc[2] = DIM == 3 ? c / (a.grid.cps[0] * a.grid.cps[1]) : 0;
  // the shifted frame is a plain difference in box units; a general cell
  // maps the unit-cube image through T, so it takes the exact path
  bool frame = a.geo.periodic != 0 && !a.geo.general;
#pragma unroll
  for (int d = 0; d < DIM; ++d) frame = frame && a.grid.cps[d] >= 4;
  const int geom = !a.geo.periodic ? S_PLAIN : (frame ? S_FRAME : S_EXACT);
  if (threadIdx.x < ns) {
    const int k = threadIdx.x;
    int sh[3];
    if (DIM == 3) { sh[0] = k / 9 - 1; sh[1] = (k / 3) % 3 - 1; sh[2] = k % 3 - 1; }
    else { sh[0] = k / 3 - 1; sh[1] = k % 3 - 1; sh[2] = 0; }
    int q[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      int v = cc[d] + sh[d];
      v = v < 0 ? v + a.grid.cps[d] : (v >= a.grid.cps[d] ? v - a.grid.cps[d] : v);
      q[d] = v;
      // FRAME: shift by L the coordinates that lie in the upper half of the box
      // as seen from the centre cell: a wrapped lower neighbour of a centre at
      // the low face, or every non-wrapped cell of a centre at the high face.
      float o = 0.f;
      if (cc[d] == 0 && sh[d] == -1) o = a.geo.L[d];
      if (cc[d] == a.grid.cps[d] - 1 && sh[d] != 1) o = a.geo.L[d];
      soff[k][d] = o;
    }
    const int h = q[0] + q[1] * a.grid.mult[1] + (DIM == 3 ? q[2] * a.grid.mult[2] : 0);
    const int beg = b.start[h], end = b.start[h + 1];
    cs.beg[k] = beg;
    cs.cnt[k] = end - beg;
    cs.split[k] = a.cap - (beg % a.cap);
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      coff[d] = (d < DIM && cc[d] == a.grid.cps[d] - 1) ? a.geo.L[d] : 0.f;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int o = 0;
    for (int k = 0; k < ns; ++k) { cs.off[k] = o; o += cs.cnt[k]; }
    cs.off[ns] = o;
  }
  __syncthreads();
  const int total = cs.off[ns];
  // the shifted frame is applied only to staged streams
  const bool staged = total <= kStageMax;
  const int g2 = (geom == S_FRAME && !staged) ? S_EXACT : geom;
  if (staged) {
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int s = stream_index<DIM>(cs, ns, t);
      float4 v = b.sorted_pos[s];
      if (g2 == S_FRAME) {
        int lo = 0, hi = ns - 1;  // cell of stream position t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (cs.off[mid] <= t) lo = mid; else hi = mid - 1;
        }
        v.x = (v.x >= a.geo.L[0] ? v.x - a.geo.L[0] : v.x) - soff[lo][0];
        v.y = (v.y >= a.geo.L[1] ? v.y - a.geo.L[1] : v.y) - soff[lo][1];
        if (DIM == 3) v.z = (v.z >= a.geo.L[2] ? v.z - a.geo.L[2] : v.z) - soff[lo][2];
      }
      v.w = __int_as_float(b.sorted_id[s]);
      spos[t] = v;
    }
  }
  __syncthreads();
  auto centre = [&](float4 v) -> float4 {
    if (g2 == S_FRAME) {
      v.x = (v.x >= a.geo.L[0] ? v.x - a.geo.L[0] : v.x) - coff[0];
      v.y = (v.y >= a.geo.L[1] ? v.y - a.geo.L[1] : v.y) - coff[1];
      if (DIM == 3) v.z = (v.z >= a.geo.L[2] ? v.z - a.geo.L[2] : v.z) - coff[2];
    }
    return v;
  };
  const int cb0 = b.start[c], cn = b.start[c + 1] - cb0;
  const int row_cap = (int)min(a.width, (int64_t)INT32_MAX);
  const int rs = TILED ? 32 : 1;
  for (int qa = 2 * warp; qa < cn; qa += 2 * nw) {
    const int ia = b.sorted_id[cb0 + qa];
    const float4 pa = b.sorted_pos[cb0 + qa];
    const bool two = qa + 1 < cn;
    const int ib = two ? b.sorted_id[cb0 + qa + 1] : -1;
    const float4 pb = two ? b.sorted_pos[cb0 + qa + 1] : pa;
    const float4 xa = centre(pa), xb = centre(pb);
    auto row_of = [&](int atom) -> int32_t* {
      if (!idx || atom < 0) return nullptr;
      if (TILED) return idx + (int64_t)(atom >> 5) * ld * 32 + (atom & 31);
      return idx + (int64_t)atom * ld;
    };
    int32_t* ra = row_of(ia);
    int32_t* rb = row_of(ib);
    // no rows (count pass): capacity 0 suppresses every write; a missing
    // second atom never matches (ib < 0), so rb is never written
    const int cap = idx ? row_cap : 0;
    int na = 0, nb = 0;
    if (a.mask_self) {
      if (g2 == S_FRAME)
        scan_pair<DIM, S_FRAME, true>(cs, ns, total, staged, spos, b, ia, xa, ib, xb, a, lane, na, nb, ra, rb, cap, rs);
      else if (g2 == S_EXACT)
        scan_pair<DIM, S_EXACT, true>(cs, ns, total, staged, spos, b, ia, xa, ib, xb, a, lane, na, nb, ra, rb, cap, rs);
      else
        scan_pair<DIM, S_PLAIN, true>(cs, ns, total, staged, spos, b, ia, xa, ib, xb, a, lane, na, nb, ra, rb, cap, rs);
    } else {
      if (g2 == S_FRAME)
        scan_pair<DIM, S_FRAME, false>(cs, ns, total, staged, spos, b, ia, xa, ib, xb, a, lane, na, nb, ra, rb, cap, rs);
      else if (g2 == S_EXACT)
        scan_pair<DIM, S_EXACT, false>(cs, ns, total, staged, spos, b, ia, xa, ib, xb, a, lane, na, nb, ra, rb, cap, rs);
      else
        scan_pair<DIM, S_PLAIN, false>(cs, ns, total, staged, spos, b, ia, xa, ib, xb, a, lane, na, nb, ra, rb, cap, rs);
    }
    if (!TILED) {
      if (ra) for (int64_t p = min((int64_t)na, a.width) + lane; p < a.width; p += 32) ra[p] = a.n;
      if (rb) for (int64_t p = min((int64_t)nb, a.width) + lane; p < a.width; p += 32) rb[p] = a.n;
    }
    if (lane == 0) {
      if (nbr_count) nbr_count[ia] = na;
      atomicMax(&b.sc->occupancy, (unsigned long long)na);
      if (na > a.width) atomicOr(&b.sc->flags, (unsigned)JMD_NEIGHBOR_LIST_OVERFLOW);
      if (ref) store_row_full<DIM, false>(ref, ref_stride, ia, pa);
      if (two) {
        if (nbr_count) nbr_count[ib] = nb;
        atomicMax(&b.sc->occupancy, (unsigned long long)nb);
        if (nb > a.width) atomicOr(&b.sc->flags, (unsigned)JMD_NEIGHBOR_LIST_OVERFLOW);
        if (ref) store_row_full<DIM, false>(ref, ref_stride, ib, pb);
      }
    }
  }
}

// Copies the raw positions as float4 rows for the all-pairs path.
template <int DIM, bool VEC4>
__global__ void k_pack(const float* __restrict__ x, int64_t stride, int n, float4* out,
                       const int32_t* flag) {
  if (skip(flag)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 r = load_row<DIM, VEC4>(x, stride, i);
  r.w = 0.f;
  out[i] = r;
}

__global__ void k_sparse_pad(int32_t* idx, int64_t ld, int64_t width, const int32_t* total_ptr,
                             int n, const int32_t* flag) {
  if (skip(flag)) return;
  int64_t total = *total_ptr;
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int64_t p = min(total, width) + t; p < width; p += (int64_t)gridDim.x * blockDim.x) {
    idx[p] = n;
    idx[ld + p] = n;
  }
}


// ------------------------------------------------------- spatial sort -------
// Gathers every per-atom array into cell order after a binning pass:
// new position s takes old atom sorted_id[s].  Positions come from the
// binning's sorted copy; the rest are gathered into scratch and copied back
// by k_sort_copy_back (both gated by the rebuild flag when one is given).
__global__ void k_sort_gather(int n, Bins b, const float4* p, const float4* f,
                              const int32_t* species, const int32_t* perm, float4* tp, float4* tf,
                              int32_t* tsp, int32_t* tperm, const int32_t* flag) {
  if (skip(flag)) return;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int i = b.sorted_id[s];
  tp[s] = p[i];
  if (f) tf[s] = f[i];
  if (species) tsp[s] = species[i];
  tperm[s] = perm[i];
}

__global__ void k_sort_copy_back(int n, Bins b, float4* x, float4* p, float4* f, int32_t* species,
                                 int32_t* perm, const float4* tp, const float4* tf,
                                 const int32_t* tsp, const int32_t* tperm, const int32_t* flag) {
  if (skip(flag)) return;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  x[s] = b.sorted_pos[s];
  b.sorted_id[s] = s;  // the bins now describe the reordered atoms
  p[s] = tp[s];
  if (f) f[s] = tf[s];
  if (species) species[s] = tsp[s];
  perm[s] = tperm[s];
}

// Host-side constants carried into the finalize kernel.
struct FinalizeArgs {
  int format;
  int64_t width;
  int use_cells;
  int cap;
  int n;
};

__global__ void k_finalize(Bins b, FinalizeArgs f, int64_t* occupancy, uint8_t* error_code,
                           int32_t* flag) {
  if (skip(flag)) return;
  unsigned flags = b.sc->flags;
  if (f.use_cells && (int)b.sc->max_fill > f.cap) flags |= JMD_CELL_LIST_OVERFLOW;
  unsigned long long occ = b.sc->occupancy;
  if (f.format != JMD_DENSE) {
    occ = (unsigned long long)b.atom_off[f.n];  // total written by the atom scan
    if ((int64_t)occ > f.width) flags |= JMD_NEIGHBOR_LIST_OVERFLOW;
  }
  if (occupancy) *occupancy = (int64_t)occ;
  if (error_code) *error_code = (uint8_t)(*error_code | flags);
  if (flag) *flag = 0;
}

template <int DIM>
__global__ void k_skin(const float* __restrict__ x, int64_t xs, const float* __restrict__ ref,
                       int64_t rs, int n, Geo g, float thr2, int32_t* flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (i < n) {
    float4 a = load_row<DIM, false>(x, xs, i);
    float4 c = load_row<DIM, false>(ref, rs, i);
    over = dist2<DIM>(a, c, g) > thr2;
  }
  if (__any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// ------------------------------------------------------------ host side ----
int validate(const jmd_nlist* nl, int64_t n, int min_cells = 3) {
  JMD_REQUIRE(nl != nullptr, "nlist descriptor is null");
  JMD_REQUIRE(nl->space.dim == 2 || nl->space.dim == 3, "dim must be 2 or 3");
  JMD_REQUIRE(n >= 0 && n < (int64_t)INT32_MAX, "atom count out of range");
  JMD_REQUIRE(nl->format >= 0 && nl->format <= 2, "unknown neighbour list format");
  if (nl->use_cell_list) {
    for (int d = 0; d < nl->space.dim; ++d) {
      JMD_REQUIRE(nl->cells_per_side[d] >= min_cells,
                  min_cells == 3 ? "the neighbour search needs >= 3 cells per side"
                                 : "cells_per_side must be >= 1");
      JMD_REQUIRE(nl->cell_size[d] > 0.f, "cell size must be positive");
    }
    JMD_REQUIRE(nl->cell_capacity >= 1, "cell capacity must be >= 1");
  }
  return JMD_OK;
}

// Runs the binning stage (zero, histogram, scan, scatter, rank).
template <int DIM, bool VEC4>
void run_binning(const float* x, int64_t stride, int n, const Grid& g, const Bins& b,
                 int32_t* particle_cell_id, const int32_t* flag, cudaStream_t st) {
  int64_t c = g.count;
  k_zero<<<(unsigned)std::min<int64_t>(ceil_div(c, 256), 1024), 256, 0, st>>>(b.count, c, b.sc,
                                                                             flag);
  if (n > 0) k_bin<DIM, VEC4><<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(x, stride, n, g, b,
                                                                          particle_cell_id, flag);
  k_scan_single<<<1, kScanThreads, 0, st>>>(b.count, c, b.start, b.cursor, &b.sc->max_fill, flag);
  if (n > 0) {
    k_scatter<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(n, b, flag);
    k_cell_rank<DIM, VEC4><<<(unsigned)ceil_div(c * 32, 256), 256, 0, st>>>(x, stride, c, b, flag);
  }
}

template <int DIM, bool VEC4>
int build_impl(const jmd_nlist* nl, const float* x, int64_t stride, int64_t n64, int32_t* idx,
               int64_t ld, int32_t* nbr_count, int64_t* occupancy, uint8_t* error_code,
               float* ref, int64_t ref_stride, int32_t* flag, void* ws, size_t ws_bytes,
               cudaStream_t st, bool tiled = false, bool bins_ready = false) {
  const int n = (int)n64;
  const bool cells = nl->use_cell_list != 0;
  Grid g = cells ? make_grid(*nl) : Grid{};
  int64_t c = cells ? g.count : 1;
  bool ok;
  Bins b = carve_bins(ws, ws_bytes, n, c, &ok);
  if (!ok) return fail(JMD_ERR_WORKSPACE, "neighbour-list workspace too small");
  SearchArgs a;
  a.geo = make_geo(nl->space);
  a.grid = g;
  a.cut2 = nl->cutoff_sq;
  a.mask_self = nl->mask_self;
  a.ordered = nl->format == JMD_ORDERED_SPARSE;
  a.cap = cells ? nl->cell_capacity : 1;
  a.n = n;
  a.width = nl->max_occupancy;
  if (cells) {
    if (!bins_ready) run_binning<DIM, VEC4>(x, stride, n, g, b, nullptr, flag, st);
  } else {
    k_zero<<<1, 256, 0, st>>>(b.count, 1, b.sc, flag);
    if (n > 0) k_pack<DIM, VEC4><<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(x, stride, n,
                                                                             b.sorted_pos, flag);
  }
  const float4* allpos = b.sorted_pos;
  const unsigned sgrid = (unsigned)std::max<int64_t>(1, ceil_div((int64_t)n * 32, 256));
  FinalizeArgs f{nl->format, nl->max_occupancy, cells ? 1 : 0, a.cap, n};
  if (nl->format == JMD_DENSE) {
    if (n > 0) {
      if (cells && tiled)
        k_search_cells<DIM, true><<<(unsigned)c, 128, kStageMax * sizeof(float4), st>>>(
            x, stride, b, a, idx, ld, nbr_count, ref, ref_stride, flag);
      else if (cells)
        k_search_cells<DIM, false><<<(unsigned)c, 128, kStageMax * sizeof(float4), st>>>(
            x, stride, b, a, idx, ld, nbr_count, ref, ref_stride, flag);
      else
        k_search<DIM, false, VEC4, 0><<<sgrid, 256, 0, st>>>(x, stride, b, a, idx, ld, nbr_count,
                                                             ref, ref_stride, flag, allpos);
    }
  } else {
    // count pass -> exclusive scan over atoms -> write pass -> pad
    if (n > 0) {
      if (cells)
        k_search<DIM, true, VEC4, 1><<<sgrid, 256, 0, st>>>(x, stride, b, a, nullptr, ld, nullptr,
                                                            nullptr, 0, flag, allpos);
      else
        k_search<DIM, false, VEC4, 1><<<sgrid, 256, 0, st>>>(x, stride, b, a, nullptr, ld,
                                                             nullptr, nullptr, 0, flag, allpos);
    }
    // scan atom counts in place: atom_off[0..n) -> offsets, atom_off[n] = total
    k_scan_single<<<1, kScanThreads, 0, st>>>(b.atom_off, n, b.atom_off, nullptr, nullptr, flag);
    if (idx && n > 0) {
      if (cells)
        k_search<DIM, true, VEC4, 2><<<sgrid, 256, 0, st>>>(x, stride, b, a, idx, ld, nullptr, ref,
                                                            ref_stride, flag, allpos);
      else
        k_search<DIM, false, VEC4, 2><<<sgrid, 256, 0, st>>>(x, stride, b, a, idx, ld, nullptr,
                                                             ref, ref_stride, flag, allpos);
    }
    if (idx && nl->max_occupancy > 0)
      k_sparse_pad<<<(unsigned)std::min<int64_t>(ceil_div(nl->max_occupancy, 256), 4096), 256, 0,
                     st>>>(idx, ld, nl->max_occupancy, b.atom_off + n, n, flag);
  }
  k_finalize<<<1, 1, 0, st>>>(b, f, occupancy, error_code, flag);
  return check_launch("jmd_neighbor_list_build");
}

}  // namespace

namespace {
// ------------------------------------------------ segment-local search ----
// The engine's private list on the segment layout (segment.cuh): one CTA per
// segment stages the neighbourhood with bulk copies, then each thread takes
// one own atom and tests the 3^(d-1) staged runs of cells x-1 .. x+1 around
// it (about 27 cells x occupancy candidates, read from shared memory; the
// threads of one cell read the same candidate at the same time, so the reads
// broadcast).  Hits are kept as 16-bit staged slots, 8 per 16-byte store.
// Entry order inside a row is the staged order (not the reference's); the
// forces do not depend on it.  Pairs are compared in float32 as
// d^2 < cutoff^2 with the minimum image taken only for atoms within the list
// cutoff of a face, so a pair within an ulp of the list cutoff may be kept
// where the reference drops it (or the reverse): such pairs lie beyond the
// interaction cutoff and change no force.
// HALF: half lists (Newton's third law).  A warp walks the forward half of
// the stencil (segment.cuh): in the centre row its own cell (atoms after
// the lane's atom) and the next cell, then the forward rows.  Each pair is
// listed once; every atom's full neighbour count (list length + the times
// it is listed by others) is accumulated in `count` (zeroed by
// k_seg_zero_counts) for the occupancy and overflow of the Dense contract.
template <int DIM, bool FRAME, bool HALF>
__global__ void __launch_bounds__(kSegMaxThreads)
k_seg_search(SegGrid sg, const float4* __restrict__ x, Bins b, Geo geo, float cut2, float margin,
             int mask_self, uint8_t* __restrict__ blocks, int32_t* __restrict__ nck_table,
             SegRecord* __restrict__ recs, int width, int32_t* __restrict__ count,
             float4* __restrict__ ref, int32_t* status, const int32_t* flag) {
  if (skip(flag)) return;
  extern __shared__ float4 spos[];
  __shared__ SegShared sh;
  __shared__ unsigned cta_max;
  __shared__ int cta_nck;
  if (threadIdx.x == 0) {
    cta_max = 0u;
    cta_nck = 0;
  }
  SegRecord* rec = recs + blockIdx.x;
  if (!seg_stage<DIM>(sg, x, b.start, spos, sh, status, rec)) {
    if (threadIdx.x == 0) {
      atomicOr(&b.sc->flags, (unsigned)JMD_CELL_LIST_OVERFLOW);
      nck_table[blockIdx.x] = 0;
      rec->nck = 0;
      rec->total = -1;
    }
    return;
  }
  // half lists: full-count contributions of each staged atom
  int* hcnt = reinterpret_cast<int*>(spos + sg.cap + 1);
  if (HALF) {
    for (int t = threadIdx.x; t < sh.total; t += blockDim.x) hcnt[t] = 0;
  }
  const int fmask = FRAME ? seg_frame<DIM>(sg, sh, spos, geo.L) : 0;
  if (HALF && !FRAME) __syncthreads();  // seg_frame ends with one
  const int W = sh.W;
  const int rows = sh.rows;
  const uint64_t far = (uint64_t)sg.cap;  // the far slot: pads chunks and rows past width
  const int nch = sg.nch;
  const int P = seg_pad(sh.own_cnt);
  uint8_t* blk = blocks + (int64_t)blockIdx.x * sg.stride;
  // a segment with more own atoms than a block holds only occurs with a cell
  // over capacity (flagged by the binning); its list is not written
  const bool fits = P <= sg.pmax;
  if (!fits && threadIdx.x == 0) atomicOr(&b.sc->flags, (unsigned)JMD_CELL_LIST_OVERFLOW);
  unsigned my_max = 0u;
  int my_nck = 0;
  // one warp per own cell (u = 1..nx of the centre row): the cell's atoms are
  // the lanes (32 at a time), and every lane walks the same candidate runs
  // (cells u-1..u+1 of each staged row), so trip counts are uniform and
  // each candidate read is a shared-memory broadcast
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int cr = seg_centre_row<DIM>(HALF ? 1 : 0) * W;
  for (int task = warp; ; task += nwarps) {
    // task -> (own cell u, group of 32 of its atoms)
    int u = 1, t = task;
    while (u <= sh.nx) {
      const int groups = (sh.coff[cr + u + 1] - sh.coff[cr + u] + 31) >> 5;
      if (t < groups) break;
      t -= groups;
      ++u;
    }
    if (u > sh.nx) break;
    const int cb = sh.coff[cr + u], ce = sh.coff[cr + u + 1];
    const int is = cb + 32 * t + lane;
    const bool active = is < ce;
    const int ia = is - sh.own_sm;  // own index of the lane's atom
    const int s = sh.own_beg + ia;
    const float4 xi = spos[active ? is : cb];
    const bool inner = FRAME || interior<DIM>(xi, geo, margin);
    int cnt = 0;
    // the chunk being filled: entries 0-3 in `lo`, 4-7 in `acc` (16 bits each)
    uint64_t lo = 0, acc = 0;
    auto put = [&](uint64_t j, int p) {  // entry j at position p of the chunk
      acc |= j << (16 * (p & 3));
      if ((p & 3) == 3) {
        if (p == 3) {
          lo = acc;
        } else if ((cnt >> 3) < nch && fits) {
          *reinterpret_cast<uint4*>(blk + seg_chunk_off(P, cnt >> 3, ia)) =
              make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)acc, (uint32_t)(acc >> 32));
        }
        acc = 0;
      }
    };
    const float2 xx = f2s(xi.x), xy = f2s(xi.y), xz = f2s(xi.z);
    for (int r = 0; r < rows; ++r) {
      // half: the centre row from the own cell on (later atoms only)
      const int j0 = sh.coff[r * W + u - ((HALF && r == 0) ? 0 : 1)], j1 = sh.coff[r * W + u + 2];
      for (int jb = j0; jb < j1; jb += 32) {
        // distance tests of up to 32 candidates into a hit mask; j + 1 may
        // read one slot past the run (still inside the staged block or the
        // far slot) and its bit is masked below
        const int nb = min(32, j1 - jb);
        uint32_t hits = 0u;
        auto test2 = [&](int k) {  // candidates jb + k, jb + k + 1 -> bits k, k + 1
          const int j = jb + k;
          const float4 b0 = spos[j];
          const float4 b1 = spos[j + 1];
          float2 dx = sub2(xx, f2(b0.x, b1.x));
          float2 dy = sub2(xy, f2(b0.y, b1.y));
          float2 dz = DIM == 3 ? sub2(xz, f2(b0.z, b1.z)) : f2s(0.f);
          if (!inner) {
            dx.x = min_image(xi.x, b0.x, geo.L[0], geo.halfL[0]);
            dx.y = min_image(xi.x, b1.x, geo.L[0], geo.halfL[0]);
            dy.x = min_image(xi.y, b0.y, geo.L[1], geo.halfL[1]);
            dy.y = min_image(xi.y, b1.y, geo.L[1], geo.halfL[1]);
            if (DIM == 3) {
              dz.x = min_image(xi.z, b0.z, geo.L[2], geo.halfL[2]);
              dz.y = min_image(xi.z, b1.z, geo.L[2], geo.halfL[2]);
            }
          }
          float2 r2 = mul2(dx, dx);
          r2 = fma2(dy, dy, r2);
          if (DIM == 3) r2 = fma2(dz, dz, r2);
          hits |= ((r2.x < cut2 ? 1u : 0u) | (r2.y < cut2 ? 2u : 0u)) << k;
        };
        if (nb == 32) {
          // a full batch: unrolled, the bit positions are constants
#pragma unroll
          for (int k = 0; k < 32; k += 2) test2(k);
        } else {
          for (int k = 0; k < nb; k += 2) test2(k);
          hits &= (1u << nb) - 1u;
        }
        if (HALF && r == 0) {
          // keep j > is: bits of candidates at or before the lane's atom go
          const int cut_bits = is + 1 - jb;
          if (cut_bits >= 32) hits = 0u;
          else if (cut_bits > 0) hits &= ~((1u << cut_bits) - 1u);
        } else if (mask_self && is >= jb && is < jb + nb) {
          hits &= ~(1u << (is - jb));
        }
        if (!active) hits = 0u;
        // append the hits in candidate order; rows past `width` keep the far
        // slot so the chunk stays valid
        while (hits) {
          const int bit = __ffs(hits) - 1;
          hits &= hits - 1;
          if (HALF) atomicAdd(hcnt + jb + bit, 1);
          put(cnt < width ? (uint64_t)(jb + bit) : far, cnt & 7);
          ++cnt;
        }
      }
    }
    if (active) {
      // pad the last chunk with the far slot
      if (cnt & 7)
        for (int p = cnt & 7; p < 8; ++p) put(far, p);
      if (HALF)  // the atom's own entries (and itself without mask_self); others add theirs below
        atomicAdd(count + s, cnt + (mask_self ? 0 : 1));
      else
        count[s] = cnt;
      const int kept = min(cnt, width);
      if (fits) reinterpret_cast<uint16_t*>(blk + 16)[ia] = (uint16_t)kept;
      my_nck = max(my_nck, (kept + 7) >> 3);
      float4 rr = xi;
      if (FRAME && fmask) {
        if ((fmask & 1) && rr.x < 0.f) rr.x += geo.L[0];
        if ((fmask & 2) && rr.y < 0.f) rr.y += geo.L[1];
        if (DIM == 3 && (fmask & 4) && rr.z < 0.f) rr.z += geo.L[2];
      }
      rr.w = 0.f;
      ref[s] = rr;
      my_max = max(my_max, (unsigned)cnt);
    }
  }
  if (HALF) {
    // the times each staged atom was listed here, to its full count
    __syncthreads();
    for (int c = warp; c < rows * W; c += nwarps) {
      const int cb = sh.coff[c], ce = sh.coff[c + 1];
      for (int t = cb + lane; t < ce; t += 32)
        if (hcnt[t]) atomicAdd(count + sh.gbeg[c] + (t - cb), hcnt[t]);
    }
  }
  my_max = __reduce_max_sync(0xffffffffu, my_max);
  my_nck = __reduce_max_sync(0xffffffffu, (unsigned)my_nck);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&cta_max, my_max);
    atomicMax(&cta_nck, my_nck);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!HALF) {
      // half lists: occupancy and overflow come from the full counts
      // (k_seg_occupancy)
      atomicMax(&b.sc->occupancy, (unsigned long long)cta_max);
      if ((int)cta_max > width) atomicOr(&b.sc->flags, (unsigned)JMD_NEIGHBOR_LIST_OVERFLOW);
    }
    const int nck = fits ? min(cta_nck, nch) : 0;
    reinterpret_cast<int32_t*>(blk)[0] = nck;
    reinterpret_cast<int32_t*>(blk)[1] = sh.own_cnt;
    nck_table[blockIdx.x] = nck;
    rec->nck = nck;
  }
}

// Half lists: zero the full counts before the search (gated like the rest of
// the rebuild chain).
__global__ void k_seg_zero_counts(int32_t* count, int n, const int32_t* flag) {
  if (skip(flag)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    count[i] = 0;
}

// Half lists: occupancy (largest full count) and the overflow bit.
__global__ void k_seg_occupancy(const int32_t* count, int n, int width, Bins b,
                                const int32_t* flag) {
  if (skip(flag)) return;
  __shared__ unsigned wmax[32];
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = max(m, count[i]);
  m = __reduce_max_sync(0xffffffffu, (unsigned)m);
  // one atomic per block (thousands of warps on one address serialise)
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = (unsigned)m;
  __syncthreads();
  if (threadIdx.x < 32) {
    const unsigned v = threadIdx.x < (blockDim.x >> 5) ? wmax[threadIdx.x] : 0u;
    const unsigned bm = __reduce_max_sync(0xffffffffu, v);
    if (threadIdx.x == 0 && bm > 0) {
      atomicMax(&b.sc->occupancy, (unsigned long long)bm);
      if ((int)bm > width) atomicOr(&b.sc->flags, (unsigned)JMD_NEIGHBOR_LIST_OVERFLOW);
    }
  }
}

}  // namespace

// Dynamic shared memory above the default 48 KB needs an opt-in per kernel.
template <typename K>
int seg_smem_optin(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return JMD_OK;
  JMD_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return JMD_OK;
}

const int32_t* sort_cell_starts(const jmd_nlist* nl, int64_t n, void* workspace,
                                size_t workspace_bytes) {
  bool ok;
  Bins b = carve_bins(workspace, workspace_bytes, n, make_grid(*nl).count, &ok);
  return ok ? b.start : nullptr;
}

int build_segment_after_sort(const jmd_nlist* nl, const SegGrid& sg, const float* position,
                             int64_t n, uint8_t* list, int32_t* nbr_count, int64_t* occupancy,
                             uint8_t* error_code, float* reference_position, int32_t* seg_status,
                             int32_t* rebuild_flag, void* workspace, size_t workspace_bytes,
                             cudaStream_t st) {
  int e = validate(nl, n);
  if (e) return e;
  JMD_REQUIRE(nl->format == JMD_DENSE && nl->use_cell_list, "segment lists are Dense with a cell grid");
  JMD_REQUIRE(list && nbr_count && (int64_t)sg.nch * 8 >= nl->max_occupancy,
              "segment list needs 8 * nch >= max_occupancy");
  JMD_REQUIRE((reinterpret_cast<uintptr_t>(list) % 16) == 0, "segment list must be 16-byte aligned");
  JMD_REQUIRE(is_vec4(position, 4) && is_vec4(reference_position, 4), "float4 rows must be 16-byte aligned");
  JMD_REQUIRE(nl->max_occupancy < INT32_MAX, "max_occupancy out of range");
  Grid g = make_grid(*nl);
  bool ok;
  Bins b = carve_bins(workspace, workspace_bytes, n, g.count, &ok);
  if (!ok) return fail(JMD_ERR_WORKSPACE, "neighbour-list workspace too small");
  const Geo geo = make_geo(nl->space);
  const float margin = sqrtf(nl->cutoff_sq);
  // staged positions + far slot (+ the half search's per-slot counts)
  const size_t smem = (size_t)(sg.cap + 1) * (sizeof(float4) + (sg.half ? sizeof(int) : 0));
  const float4* x = reinterpret_cast<const float4*>(position);
  float4* ref = reinterpret_cast<float4*>(reference_position);
  const int width = (int)nl->max_occupancy;
  const unsigned zgrid = (unsigned)std::min<int64_t>(std::max<int64_t>(1, ceil_div(n, 256)), 4096);
  if (sg.half && n > 0) k_seg_zero_counts<<<zgrid, 256, 0, st>>>(nbr_count, (int)n, rebuild_flag);
  auto go = [&](auto kernel) -> int {
    int rc = seg_smem_optin(kernel, smem);
    if (rc) return rc;
    // one warp per own cell of a segment (at most 8 warps)
    const unsigned threads = (unsigned)(32 * std::min(sg.K, kSegMaxThreads / 32));
    int32_t* table = reinterpret_cast<int32_t*>(list);
    SegRecord* recs = reinterpret_cast<SegRecord*>(list + seg_table_bytes(sg.nseg));
    uint8_t* blocks = list + seg_table_bytes(sg.nseg) + seg_records_bytes(sg.nseg);
    kernel<<<(unsigned)sg.nseg, threads, smem, st>>>(
        sg, x, b, geo, nl->cutoff_sq, margin, nl->mask_self, blocks, table, recs, width, nbr_count,
        ref, seg_status, rebuild_flag);
    return JMD_OK;
  };
  if (n > 0) {
    if (nl->space.dim == 3) {
      if (sg.half) e = sg.frame ? go(k_seg_search<3, true, true>) : go(k_seg_search<3, false, true>);
      else e = sg.frame ? go(k_seg_search<3, true, false>) : go(k_seg_search<3, false, false>);
    } else {
      if (sg.half) e = sg.frame ? go(k_seg_search<2, true, true>) : go(k_seg_search<2, false, true>);
      else e = sg.frame ? go(k_seg_search<2, true, false>) : go(k_seg_search<2, false, false>);
    }
    if (e) return e;
    if (sg.half)
      // grid-stride: four blocks per SM of the 152-SM part cover any n
      k_seg_occupancy<<<(unsigned)std::min<int64_t>(zgrid, 4 * 152), 256, 0, st>>>(
          nbr_count, (int)n, width, b, rebuild_flag);
  }
  FinalizeArgs f{JMD_DENSE, nl->max_occupancy, 1, nl->cell_capacity, (int)n};
  k_finalize<<<1, 1, 0, st>>>(b, f, occupancy, error_code, rebuild_flag);
  return check_launch("jmd segment list build");
}

// The tiled build right after jmd_sort_by_cell on the same positions and
// workspace: the sort's bins already describe the reordered atoms (its
// copy-back sets sorted_id to the identity), so the binning is not repeated.
int build_tiled_after_sort(const jmd_nlist* nl, const float* position, int64_t n, int32_t* tidx,
                           int64_t depth, int32_t* nbr_count, int64_t* occupancy,
                           uint8_t* error_code, float* reference_position, int32_t* rebuild_flag,
                           void* workspace, size_t workspace_bytes, cudaStream_t st) {
  int e = validate(nl, n);
  if (e) return e;
  JMD_REQUIRE(nl->format == JMD_DENSE && nl->use_cell_list, "tiled lists are Dense with a cell grid");
  JMD_REQUIRE(tidx && nbr_count && depth >= nl->max_occupancy, "tiled list needs depth >= max_occupancy");
  if (nl->space.dim == 3)
    return build_impl<3, true>(nl, position, 4, n, tidx, depth, nbr_count, occupancy, error_code,
                               reference_position, 4, rebuild_flag, workspace, workspace_bytes, st,
                               true, true);
  return build_impl<2, true>(nl, position, 4, n, tidx, depth, nbr_count, occupancy, error_code,
                             reference_position, 4, rebuild_flag, workspace, workspace_bytes, st,
                             true, true);
}

}  // namespace jmd

using namespace jmd;

extern "C" {

size_t jmd_cell_workspace_bytes(int64_t n_atoms, int64_t cell_count) {
  return bins_bytes(n_atoms, cell_count);
}

size_t jmd_neighbor_list_workspace_bytes(const jmd_nlist* nl, int64_t n) {
  if (!nl) return 0;
  return bins_bytes(n, grid_count(*nl));
}

int jmd_cell_max_filling(const float* position, int64_t pos_stride, int64_t n,
                         const jmd_nlist* nl, int32_t* max_filling, void* workspace,
                         size_t workspace_bytes, void* stream) {
  int e = validate(nl, n, 1);
  if (e) return e;
  JMD_REQUIRE(nl->use_cell_list, "cell grid required");
  JMD_REQUIRE(max_filling != nullptr, "max_filling is null");
  cudaStream_t st = as_stream(stream);
  Grid g = make_grid(*nl);
  bool ok;
  Bins b = carve_bins(workspace, workspace_bytes, n, g.count, &ok);
  if (!ok) return fail(JMD_ERR_WORKSPACE, "cell workspace too small");
  const int dim = nl->space.dim;
  const bool v4 = is_vec4(position, pos_stride);
  k_zero<<<(unsigned)std::min<int64_t>(ceil_div(g.count, 256), 1024), 256, 0, st>>>(
      b.count, g.count, b.sc, nullptr);
  if (n > 0) {
    unsigned gr = (unsigned)ceil_div(n, 256);
    if (dim == 3 && v4) k_bin<3, true><<<gr, 256, 0, st>>>(position, pos_stride, (int)n, g, b, nullptr, nullptr);
    else if (dim == 3) k_bin<3, false><<<gr, 256, 0, st>>>(position, pos_stride, (int)n, g, b, nullptr, nullptr);
    else if (v4) k_bin<2, true><<<gr, 256, 0, st>>>(position, pos_stride, (int)n, g, b, nullptr, nullptr);
    else k_bin<2, false><<<gr, 256, 0, st>>>(position, pos_stride, (int)n, g, b, nullptr, nullptr);
  }
  k_scan_single<<<1, kScanThreads, 0, st>>>(b.count, g.count, b.start, nullptr, &b.sc->max_fill,
                                            nullptr);
  JMD_CUDA(cudaMemcpyAsync(max_filling, &b.sc->max_fill, sizeof(int32_t),
                           cudaMemcpyDeviceToDevice, st));
  return check_launch("jmd_cell_max_filling");
}

int jmd_cell_list_build(const float* position, int64_t pos_stride, int64_t n, const jmd_nlist* nl,
                        int32_t* id_buffer, float* position_buffer, int32_t* particle_cell_id,
                        uint8_t* error_code, void* workspace, size_t workspace_bytes,
                        void* stream) {
  int e = validate(nl, n, 1);
  if (e) return e;
  JMD_REQUIRE(nl->use_cell_list, "cell grid required");
  JMD_REQUIRE(id_buffer != nullptr, "id_buffer is null");
  cudaStream_t st = as_stream(stream);
  Grid g = make_grid(*nl);
  bool ok;
  Bins b = carve_bins(workspace, workspace_bytes, n, g.count, &ok);
  if (!ok) return fail(JMD_ERR_WORKSPACE, "cell workspace too small");
  const int dim = nl->space.dim;
  const bool v4 = is_vec4(position, pos_stride);
  const int cap = nl->cell_capacity;
  if (dim == 3 && v4) run_binning<3, true>(position, pos_stride, (int)n, g, b, particle_cell_id, nullptr, st);
  else if (dim == 3) run_binning<3, false>(position, pos_stride, (int)n, g, b, particle_cell_id, nullptr, st);
  else if (v4) run_binning<2, true>(position, pos_stride, (int)n, g, b, particle_cell_id, nullptr, st);
  else run_binning<2, false>(position, pos_stride, (int)n, g, b, particle_cell_id, nullptr, st);
  int64_t total = g.count * cap;
  unsigned fg = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(total, 256), 8192));
  if (dim == 3) k_fill_cell_buffers<3><<<fg, 256, 0, st>>>(g.count, cap, (int)n, id_buffer, position_buffer);
  else k_fill_cell_buffers<2><<<fg, 256, 0, st>>>(g.count, cap, (int)n, id_buffer, position_buffer);
  if (n > 0) {
    unsigned gr = (unsigned)ceil_div(n, 256);
    if (dim == 3) k_emplace<3><<<gr, 256, 0, st>>>((int)n, cap, g, b, id_buffer, position_buffer);
    else k_emplace<2><<<gr, 256, 0, st>>>((int)n, cap, g, b, id_buffer, position_buffer);
  }
  FinalizeArgs f{JMD_DENSE, INT64_MAX, 1, cap, (int)n};
  k_finalize<<<1, 1, 0, st>>>(b, f, nullptr, error_code, nullptr);
  return check_launch("jmd_cell_list_build");
}

int jmd_neighbor_list_build(const jmd_nlist* nl, const float* position, int64_t pos_stride,
                            int64_t n, int32_t* idx, int64_t idx_ld, int32_t* nbr_count,
                            int64_t* occupancy, uint8_t* error_code, float* reference_position,
                            int64_t ref_stride, int32_t* rebuild_flag, void* workspace,
                            size_t workspace_bytes, void* stream) {
  int e = validate(nl, n);
  if (e) return e;
  JMD_REQUIRE(position != nullptr || n == 0, "position is null");
  JMD_REQUIRE(nl->max_occupancy >= 0, "max_occupancy must be >= 0");
  if (idx) {
    if (nl->format == JMD_DENSE)
      JMD_REQUIRE(idx_ld >= nl->max_occupancy, "idx leading dimension < max_occupancy");
    else
      JMD_REQUIRE(idx_ld >= nl->max_occupancy, "sparse idx row stride < capacity");
  }
  cudaStream_t st = as_stream(stream);
  const bool v4 = is_vec4(position, pos_stride);
  if (nl->space.dim == 3) {
    return v4 ? build_impl<3, true>(nl, position, pos_stride, n, idx, idx_ld, nbr_count, occupancy,
                                    error_code, reference_position, ref_stride, rebuild_flag,
                                    workspace, workspace_bytes, st)
              : build_impl<3, false>(nl, position, pos_stride, n, idx, idx_ld, nbr_count,
                                     occupancy, error_code, reference_position, ref_stride,
                                     rebuild_flag, workspace, workspace_bytes, st);
  }
  return v4 ? build_impl<2, true>(nl, position, pos_stride, n, idx, idx_ld, nbr_count, occupancy,
                                  error_code, reference_position, ref_stride, rebuild_flag,
                                  workspace, workspace_bytes, st)
            : build_impl<2, false>(nl, position, pos_stride, n, idx, idx_ld, nbr_count, occupancy,
                                   error_code, reference_position, ref_stride, rebuild_flag,
                                   workspace, workspace_bytes, st);
}

int jmd_neighbor_list_build_tiled(const jmd_nlist* nl, const float* position, int64_t n,
                                  int32_t* tidx, int64_t depth, int32_t* nbr_count,
                                  int64_t* occupancy, uint8_t* error_code,
                                  float* reference_position, int32_t* rebuild_flag,
                                  void* workspace, size_t workspace_bytes, void* stream) {
  int e = validate(nl, n);
  if (e) return e;
  JMD_REQUIRE(nl->format == JMD_DENSE && nl->use_cell_list, "tiled lists are Dense with a cell grid");
  JMD_REQUIRE(tidx && nbr_count && depth >= nl->max_occupancy, "tiled list needs depth >= max_occupancy");
  JMD_REQUIRE(is_vec4(position, 4), "positions must be 16-byte aligned float4 rows");
  cudaStream_t st = as_stream(stream);
  if (nl->space.dim == 3)
    return build_impl<3, true>(nl, position, 4, n, tidx, depth, nbr_count, occupancy, error_code,
                               reference_position, 4, rebuild_flag, workspace, workspace_bytes, st,
                               true);
  return build_impl<2, true>(nl, position, 4, n, tidx, depth, nbr_count, occupancy, error_code,
                             reference_position, 4, rebuild_flag, workspace, workspace_bytes, st, true);
}

int jmd_skin_check(const float* position, int64_t pos_stride, const float* reference_position,
                   int64_t ref_stride, int64_t n, const jmd_space* space, float threshold_sq,
                   int32_t* rebuild_flag, void* stream) {
  JMD_REQUIRE(space && (space->dim == 2 || space->dim == 3), "bad space");
  JMD_REQUIRE(rebuild_flag != nullptr, "rebuild_flag is null");
  if (n <= 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  Geo g = make_geo(*space);
  unsigned gr = (unsigned)ceil_div(n, 256);
  if (space->dim == 3)
    k_skin<3><<<gr, 256, 0, st>>>(position, pos_stride, reference_position, ref_stride, (int)n, g,
                                  threshold_sq, rebuild_flag);
  else
    k_skin<2><<<gr, 256, 0, st>>>(position, pos_stride, reference_position, ref_stride, (int)n, g,
                                  threshold_sq, rebuild_flag);
  return check_launch("jmd_skin_check");
}

int jmd_sort_by_cell(const jmd_nlist* nl, float* position, float* momentum, float* force,
                     int32_t* species, int32_t* perm, int64_t n, float* scratch4a,
                     float* scratch4b, int32_t* scratch_i_a, int32_t* scratch_i_b,
                     int32_t* rebuild_flag, void* workspace, size_t workspace_bytes,
                     void* stream) {
  int e = validate(nl, n, 1);
  if (e) return e;
  JMD_REQUIRE(nl->use_cell_list, "sorting needs a cell grid");
  JMD_REQUIRE(position && momentum && perm && scratch4a && scratch_i_b, "null buffer");
  JMD_REQUIRE(!force || scratch4b, "force needs scratch4b");
  JMD_REQUIRE(!species || scratch_i_a, "species needs scratch_i_a");
  for (const void* q : {(const void*)position, (const void*)momentum, (const void*)scratch4a})
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(q) % 16) == 0, "float4 rows must be 16-byte aligned");
  if (n <= 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  Grid g = make_grid(*nl);
  bool ok;
  Bins b = carve_bins(workspace, workspace_bytes, n, g.count, &ok);
  if (!ok) return fail(JMD_ERR_WORKSPACE, "sort workspace too small");
  if (nl->space.dim == 3) run_binning<3, true>(position, 4, (int)n, g, b, nullptr, rebuild_flag, st);
  else run_binning<2, true>(position, 4, (int)n, g, b, nullptr, rebuild_flag, st);
  const unsigned gr = (unsigned)ceil_div(n, 256);
  k_sort_gather<<<gr, 256, 0, st>>>((int)n, b, reinterpret_cast<const float4*>(momentum),
                                    reinterpret_cast<const float4*>(force), species, perm,
                                    reinterpret_cast<float4*>(scratch4a),
                                    reinterpret_cast<float4*>(scratch4b), scratch_i_a, scratch_i_b,
                                    rebuild_flag);
  k_sort_copy_back<<<gr, 256, 0, st>>>((int)n, b, reinterpret_cast<float4*>(position),
                                       reinterpret_cast<float4*>(momentum),
                                       reinterpret_cast<float4*>(force), species, perm,
                                       reinterpret_cast<const float4*>(scratch4a),
                                       reinterpret_cast<const float4*>(scratch4b), scratch_i_a,
                                       scratch_i_b, rebuild_flag);
  return check_launch("jmd_sort_by_cell");
}

}  // extern "C"

