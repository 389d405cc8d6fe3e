// Segment staging for the engine's cell-sorted kernels.
//
// The engine keeps its atoms in cell order (cells hashed x-fastest, as
// partition.py:212-224 hashes them) and rebuilds its private neighbour list
// from that order.  A *segment* is K consecutive cells along x inside one row
// (fixed y, z) of the cell grid; one CTA owns one segment.  Every neighbour of
// an atom of the segment lies in the segment's neighbourhood: the 3^(d-1) rows
// around it (y +- 1, z +- 1, periodic), each over the cells x0-1 .. x0+K
// (periodic).  Those rows are contiguous runs of sorted atoms (one or two runs
// per row, two where the row wraps), so the CTA stages the neighbourhood's
// float4 positions into shared memory with a handful of bulk (TMA) copies that
// complete on one mbarrier, and the private list stores each neighbour as a
// 16-bit slot of that staged block.  The layout of the block depends only on
// the cell starts of the last rebuild, so every step between two rebuilds
// stages the same slots (the atoms move, their slots do not).
//
// Requirements (checked on the host): at least 3 cells per side in every
// dimension, so the staged rows and cells are distinct; K <= cells_x - 2.
#pragma once

#include "common.cuh"

namespace jmd {

constexpr int kSegMaxW = 16;                   // staged cells per row: K + 2 <= 16
constexpr int kSegMaxCells = 9 * kSegMaxW;     // staged cells per CTA
constexpr int kSegMaxStaged = 65535;           // 16-bit slots
// Status bits of the segment kernels (a device int32 owned by the engine).
constexpr int kSegStatusOverflow = 1;  // a neighbourhood exceeded the staging capacity
constexpr int kSegStatusTimeout = 2;   // a bulk copy did not complete within the wait limit

struct SegGrid {
  int cps[3];   // cells per side (1 beyond dim)
  int mult1;    // cps[0]
  int mult2;    // cps[0] * cps[1]
  int K;        // cells per segment along x
  int spr;      // segments per row, ceil(cps[0] / K)
  int nseg;     // segments (= CTAs)
  int cap;      // staged atoms one CTA can hold (dynamic shared memory / 16)
  int threads;  // threads per CTA (a multiple of 32, at most kSegMaxThreads)
};

constexpr int kSegMaxThreads = 256;

// Host: the segment grid of a cell grid, or false when it does not apply.
inline bool make_seg_grid(const jmd_nlist& nl, int K, int cap, SegGrid* out) {
  const int dim = nl.space.dim;
  if (!nl.use_cell_list || (dim != 2 && dim != 3)) return false;
  SegGrid g{};
  for (int d = 0; d < 3; ++d) g.cps[d] = d < dim ? nl.cells_per_side[d] : 1;
  for (int d = 0; d < dim; ++d)
    if (g.cps[d] < 3) return false;
  if (K < 1) return false;
  K = K > g.cps[0] - 2 ? g.cps[0] - 2 : K;
  if (K + 2 > kSegMaxW) return false;
  g.mult1 = g.cps[0];
  g.mult2 = g.cps[0] * g.cps[1];
  g.K = K;
  g.spr = (g.cps[0] + K - 1) / K;
  const int64_t nseg = (int64_t)g.spr * g.cps[1] * g.cps[2];
  if (nseg >= INT32_MAX) return false;
  g.nseg = (int)nseg;
  g.cap = cap;
  g.threads = 128;
  *out = g;
  return true;
}

// ------------------------------------------------ mbarrier / bulk copy ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Global -> shared bulk copy (16-byte aligned addresses, size a multiple of
// 16) completing `bytes` of the mbarrier's transaction count.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Waits for phase 0 of the barrier, at most ~`limit_ns` nanoseconds.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint64_t limit_ns) {
  if (mbar_test_wait(bar, 0)) return true;
  const uint64_t t0 = global_ns();
  unsigned spins = 0;
  while (!mbar_test_wait(bar, 0)) {
    if ((++spins & 63u) == 0 && global_ns() - t0 > limit_ns) return false;
    __nanosleep(64);
  }
  return true;
}

constexpr uint64_t kSegWaitNs = 1000000000ull;  // 1 s: a staged copy takes microseconds

// Per-CTA description of the staged neighbourhood.
struct SegShared {
  uint64_t bar;
  int nx;        // own cells (K, or fewer in a row's last segment)
  int W;         // staged cells per row, nx + 2
  int rows;      // staged rows, 3^(dim-1)
  int own_beg;   // first own atom (sorted slot)
  int own_cnt;   // own atoms
  int own_sm;    // staged slot of the first own atom
  int total;     // staged atoms
  int ok;        // 0: the CTA must not use the staged block
  int coff[kSegMaxCells + 1];  // staged slot of each staged cell's first atom
  int gbeg[kSegMaxCells];      // sorted slot of each staged cell's first atom
};

// Staged cells of a CTA: row r (dz = r / 3 - 1, dy = r % 3 - 1), column u
// (x = x0 - 1 + u), at index r * W + u; the centre row is r = rows / 2.
template <int DIM>
__device__ __forceinline__ int seg_centre_row() {
  return DIM == 3 ? 4 : 1;
}

// Stages segment blockIdx.x's neighbourhood of `x` into `spos` (dynamic shared
// memory of g.cap float4) and fills `sh`.  Every thread of the CTA must call
// it; afterwards sh.ok says whether the block is usable (false: the
// neighbourhood exceeded g.cap, or a copy timed out; the status bit is set).
template <int DIM>
__device__ void seg_stage(const SegGrid& g, const float4* __restrict__ x,
                          const int32_t* __restrict__ start, float4* spos, SegShared& sh,
                          int32_t* status) {
  const int tid = threadIdx.x;
  const int seg = blockIdx.x;
  const int row = seg / g.spr, sx = seg - row * g.spr;
  const int x0 = sx * g.K;
  const int nx = min(g.K, g.cps[0] - x0);
  const int W = nx + 2;
  const int rows = DIM == 3 ? 9 : 3;
  const int ncell = rows * W;
  const int cy = row % g.cps[1];
  const int cz = DIM == 3 ? row / g.cps[1] : 0;
  if (tid == 0) mbar_init(&sh.bar, 1);
  for (int t = tid; t < ncell; t += blockDim.x) {
    const int r = t / W, u = t - r * W;
    int y = cy + (r % 3) - 1, z = DIM == 3 ? cz + r / 3 - 1 : 0;
    int xx = x0 - 1 + u;
    y = y < 0 ? y + g.cps[1] : (y >= g.cps[1] ? y - g.cps[1] : y);
    if (DIM == 3) z = z < 0 ? z + g.cps[2] : (z >= g.cps[2] ? z - g.cps[2] : z);
    xx = xx < 0 ? xx + g.cps[0] : (xx >= g.cps[0] ? xx - g.cps[0] : xx);
    const int h = xx + y * g.mult1 + z * g.mult2;
    const int b = __ldg(start + h), e = __ldg(start + h + 1);
    sh.gbeg[t] = b;
    sh.coff[t] = e - b;  // counts first; the scan below turns them into offsets
  }
  __syncthreads();
  if (tid < 32) {
    const int lane = tid;
    const int per = (ncell + 31) >> 5;
    const int lo = min(lane * per, ncell), hi = min(lo + per, ncell);
    int cnt[(kSegMaxCells + 31) / 32];
    int s = 0;
#pragma unroll
    for (int k = 0; k < (kSegMaxCells + 31) / 32; ++k) {
      cnt[k] = (lo + k < hi) ? sh.coff[lo + k] : 0;
      s += cnt[k];
    }
    int incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    int run = incl - s;
    __syncwarp();
#pragma unroll
    for (int k = 0; k < (kSegMaxCells + 31) / 32; ++k) {
      if (lo + k < hi) {
        sh.coff[lo + k] = run;
        run += cnt[k];
      }
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (lane == 0) {
      sh.coff[ncell] = total;
      sh.total = total;
      sh.nx = nx;
      sh.W = W;
      sh.rows = rows;
    }
    __syncwarp();
    const int cr = seg_centre_row<DIM>() * W;
    if (lane == 0) {
      sh.own_sm = sh.coff[cr + 1];
      sh.own_cnt = sh.coff[cr + nx + 1] - sh.coff[cr + 1];
      sh.own_beg = sh.gbeg[cr + 1];
      sh.ok = total <= g.cap;
      if (total > g.cap) atomicOr(status, kSegStatusOverflow);
    }
    __syncwarp();
    if (total <= g.cap) {
      if (lane == 0) mbar_arrive_expect_tx(&sh.bar, (uint32_t)total * 16u);
      __syncwarp();
      // one lane per row: merge the row's cells into runs contiguous in memory
      if (lane < rows) {
        int u0 = 0;
        while (u0 < W) {
          const int t0 = lane * W + u0;
          int u1 = u0 + 1;
          while (u1 < W && sh.gbeg[lane * W + u1] == sh.gbeg[t0] + (sh.coff[lane * W + u1] - sh.coff[t0]))
            ++u1;
          const int n_at = sh.coff[lane * W + u1] - sh.coff[t0];
          if (n_at > 0) bulk_g2s(spos + sh.coff[t0], x + sh.gbeg[t0], (uint32_t)n_at * 16u, &sh.bar);
          u0 = u1;
        }
      }
    }
  }
  __syncthreads();
  if (sh.ok) {
    if (!mbar_wait_bounded(&sh.bar, kSegWaitNs)) {
      atomicOr(status, kSegStatusTimeout);
      // give the copies in flight a second bounded chance before the block
      // is released; the results of this CTA are discarded either way
      mbar_wait_bounded(&sh.bar, kSegWaitNs);
      sh.ok = 0;
    }
  }
  __syncthreads();
}

// Own cell (column u in 1..nx of the centre row) of the staged slot `is`.
template <int DIM>
__device__ __forceinline__ int seg_own_cell(const SegShared& sh, int is) {
  const int cr = seg_centre_row<DIM>() * sh.W;
  int u = 1;
  while (u < sh.nx && sh.coff[cr + u + 1] <= is) ++u;
  return u;
}

// Private list layout: 16-bit staged slots, entry k of sorted atom s at
//   list[((s / 32) * nch + k / 8) * 256 + (s % 32) * 8 + k % 8]
// (nch = depth / 8 chunks): a thread reads its next 8 entries as one 16-byte
// load, a warp's 32 threads one 512-byte line run.
__device__ __forceinline__ int64_t seg_list_base(int s, int64_t nch) {
  return ((int64_t)(s >> 5) * nch) * 256 + (int64_t)(s & 31) * 8;
}

}  // namespace jmd
