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
  int cap;      // staged atoms one CTA can hold (dynamic shared memory / 16 - 1)
  int threads;  // threads per CTA (a multiple of 32, at most kSegMaxThreads)
  int frame;    // 1: staged coordinates are put in the CTA's periodic frame (below)
  int pmax;     // own atoms a segment block holds, rounded to 8 (K x cell capacity)
  int nch;      // 8-entry chunks per atom at most (8 nch >= max_occupancy)
  int64_t stride;  // bytes per segment block
  int lcap;     // shared-memory bytes for a staged segment block (0: never staged)
  int half;     // 1: half lists (Newton's third law): only the forward half
                //    of the neighbourhood is staged and searched
};

// Segment-block list layout.  The private list of segment g is one block of
// `stride` bytes at blocks + g * stride (the int32 table nck[nseg] of each
// block's chunk count comes first in the buffer, padded to 16 bytes):
//   [0, 16)           header: int32 chunks of the longest own row, int32 own atoms
//   [16, 16 + 2P)     uint16 entry count of each own atom (P = own atoms rounded to 8)
//   [16 + 2P, ...)    chunk k (8 16-bit staged slots) of own atom a at
//                     16 + 2P + (k P + a) 16
// so the used part of a block (header, counts, chunks of its longest row) is
// one contiguous range that a single bulk copy stages with the positions.
__host__ __device__ inline int seg_pad(int own) { return (own + 7) & ~7; }
__host__ __device__ inline int64_t seg_chunk_off(int P, int k, int a) {
  return 16 + 2 * (int64_t)P + ((int64_t)k * P + a) * 16;
}
__host__ __device__ inline int64_t seg_block_used(int P, int nck) {
  return 16 + 2 * (int64_t)P + (int64_t)nck * P * 16;
}
inline int64_t seg_table_bytes(int64_t nseg) { return (4 * nseg + 15) / 16 * 16; }
// buffer: the chunk-count table, the per-segment records, the blocks
inline int64_t seg_list_bytes(const SegGrid& g) {
  return seg_table_bytes(g.nseg) + (int64_t)g.nseg * 256 + (int64_t)g.nseg * g.stride;
}

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
  // The periodic frame (seg_frame) needs the staged cells of a CTA that
  // touches a face to lie within half a box of that face, with a cell of
  // room for the drift since the rebuild (< skin / 2 < one cell):
  // 2 K + 3 < cells_x, and >= 6 cells along y (and z).
  g.frame = nl.space.periodic && 2 * K + 3 < g.cps[0] && g.cps[1] >= 6 && (dim < 3 || g.cps[2] >= 6);
  g.pmax = seg_pad(K * (nl.cell_capacity > 0 ? nl.cell_capacity : 1));
  g.nch = (int)((nl.max_occupancy + 7) / 8);
  if (g.nch < 1) g.nch = 1;
  g.stride = seg_block_used(g.pmax, g.nch);
  g.lcap = 0;
  g.half = 0;
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

// Fire-and-forget prefetch of [src, src + bytes) into L2 (16-byte aligned,
// a multiple of 16 bytes).
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
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

// Staged slot `cap` holds a point far outside the box: list entries past an
// atom's count point at it, so every entry of a 16-byte chunk is a valid
// slot and lies beyond every cutoff.
__device__ __forceinline__ float4 seg_far_point() {
  return make_float4(1e15f, 1e15f, 1e15f, 0.f);
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
  int list_sm;   // 1: the segment's list block was staged with the positions
  int nck;       // chunks of the block's longest row
  int coff[kSegMaxCells + 1];  // staged slot of each staged cell's first atom
  int gbeg[kSegMaxCells];      // sorted slot of each staged cell's first atom
};

// What the rebuild's search learned about a segment's staging, so that the
// per-step kernel can stage without reading the cell starts: the own range,
// the staged total, the chunk count of the list block, and up to two bulk
// copies per staged row (global slot, staged slot, atoms; 0 atoms = unused).
constexpr int kSegMaxPieces = 18;
struct SegRecord {
  int32_t own_beg, own_cnt, own_sm, total, nck, pad[3];
  int32_t pg[kSegMaxPieces], ps[kSegMaxPieces], pn[kSegMaxPieces];
  int32_t tail[2];
};
static_assert(sizeof(SegRecord) == 256, "segment record is 256 bytes");
inline int64_t seg_records_bytes(int64_t nseg) { return nseg * (int64_t)sizeof(SegRecord); }

// Staged cells of a CTA: staged row r, column u (x = x0 - 1 + u), at index
// r * W + u.  Full stencil: rows r = 0 .. 3^(d-1) - 1 with dy = r % 3 - 1,
// dz = r / 3 - 1 (the centre row is r = 4 in 3-D, 1 in 2-D).  Half stencil
// (g.half): the forward rows only -- full rows from the centre row on (the
// centre row, then dy = +1, then the dz = +1 rows) -- and in the centre row
// only the own cells and the one to their right (column 0 is left empty).
// Every pair of atoms within a cutoff is then seen from exactly one side:
// cells ahead of an atom's cell in (dz, dy, dx) order, and atoms after it in
// its own cell.
__host__ __device__ inline int seg_rows(int dim, int half) {
  return half ? (dim == 3 ? 5 : 2) : (dim == 3 ? 9 : 3);
}
__host__ __device__ inline int seg_full_row(int dim, int half, int r) {
  return half ? r + (dim == 3 ? 4 : 1) : r;
}
template <int DIM>
__device__ __forceinline__ int seg_centre_row(int half) {
  return half ? 0 : (DIM == 3 ? 4 : 1);
}

// The segment of CTA blockIdx.x: its row, first cell and own cell count.
struct SegPos {
  int row, x0, nx, cy, cz;
};

template <int DIM>
__device__ __forceinline__ SegPos seg_pos(const SegGrid& g) {
  SegPos p;
  p.row = blockIdx.x / g.spr;
  p.x0 = (blockIdx.x - p.row * g.spr) * g.K;
  p.nx = min(g.K, g.cps[0] - p.x0);
  p.cy = p.row % g.cps[1];
  p.cz = DIM == 3 ? p.row / g.cps[1] : 0;
  return p;
}

// Own atoms of the CTA's segment, [beg, beg + cnt) in sorted slots: two
// loads of the cell starts, which every thread can make for itself before
// the staged block is ready.
struct SegOwn {
  int beg, cnt;
};

template <int DIM>
__device__ __forceinline__ SegOwn seg_own_range(const SegGrid& g, const int32_t* __restrict__ start) {
  const SegPos p = seg_pos<DIM>(g);
  const int h0 = p.x0 + p.cy * g.mult1 + p.cz * g.mult2;
  SegOwn o;
  o.beg = __ldg(start + h0);
  o.cnt = __ldg(start + h0 + p.nx) - o.beg;
  return o;
}

// Starts staging segment blockIdx.x's neighbourhood of `x` into `spos`
// (dynamic shared memory of g.cap + 1 float4) and fills `sh`.  Warp 0 alone
// reads the cell starts, scans the cell counts into staged offsets and issues
// one bulk copy per contiguous run of a row; the other warps only meet it at
// the closing barrier.  Every thread of the CTA must call it.
template <int DIM>
__device__ __forceinline__ void seg_stage_issue(const SegGrid& g, const float4* __restrict__ x,
                                                const int32_t* __restrict__ start, float4* spos,
                                                SegShared& sh, int32_t* status,
                                                const uint8_t* gblock = nullptr,
                                                const int32_t* nck_table = nullptr,
                                                uint8_t* slist = nullptr,
                                                SegRecord* rec_out = nullptr) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const SegPos sp = seg_pos<DIM>(g);
    const int W = sp.nx + 2;
    const int rows = seg_rows(DIM, g.half);
    const int ncell = rows * W;
    if (lane == 0) {
      mbar_init(&sh.bar, 1);
      spos[g.cap] = seg_far_point();
    }
    constexpr int kPer = (kSegMaxCells + 31) / 32;
    const int per = (ncell + 31) >> 5;
    const int lo = min(lane * per, ncell), hi = min(lo + per, ncell);
    int cnt[kPer], beg[kPer];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      cnt[k] = 0;
      beg[k] = 0;
      const int t = lo + k;
      if (t < hi) {
        const int r = t / W, u = t - r * W;
        const int fr = seg_full_row(DIM, g.half, r);
        int y = sp.cy + (fr % 3) - 1, z = DIM == 3 ? sp.cz + fr / 3 - 1 : 0;
        // the half stencil's centre row starts at the own cells: column 0
        // is empty, placed at the first own cell's start so the row stays
        // one contiguous run
        const bool skip0 = g.half && r == 0 && u == 0;
        int xx = sp.x0 - 1 + (skip0 ? 1 : u);
        y = y < 0 ? y + g.cps[1] : (y >= g.cps[1] ? y - g.cps[1] : y);
        if (DIM == 3) z = z < 0 ? z + g.cps[2] : (z >= g.cps[2] ? z - g.cps[2] : z);
        xx = xx < 0 ? xx + g.cps[0] : (xx >= g.cps[0] ? xx - g.cps[0] : xx);
        const int h = xx + y * g.mult1 + z * g.mult2;
        beg[k] = __ldg(start + h);
        cnt[k] = skip0 ? 0 : __ldg(start + h + 1) - beg[k];
      }
      sum += cnt[k];
    }
    // the list block's chunk count, read with the cell starts
    const int nck = (gblock && lane == 0) ? __ldg(nck_table + blockIdx.x) : 0;
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    int run = incl - sum;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      if (lo + k < hi) {
        sh.coff[lo + k] = run;
        sh.gbeg[lo + k] = beg[k];
        run += cnt[k];
      }
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const bool fits = total <= g.cap;
    if (lane == 0) {
      sh.coff[ncell] = total;
      sh.total = total;
      sh.nx = sp.nx;
      sh.W = W;
      sh.rows = rows;
      sh.ok = fits;
      if (!fits) atomicOr(status, kSegStatusOverflow);
    }
    __syncwarp();
    int64_t lbytes = 0;
    if (lane == 0) {
      const int cr = seg_centre_row<DIM>(g.half) * W;
      sh.own_sm = sh.coff[cr + 1];
      sh.own_cnt = sh.coff[cr + sp.nx + 1] - sh.coff[cr + 1];
      sh.own_beg = sh.gbeg[cr + 1];
      sh.nck = nck;
      const int P = seg_pad(sh.own_cnt);
      lbytes = seg_block_used(P, nck);
      sh.list_sm = (gblock != nullptr && slist != nullptr && P <= g.pmax && lbytes <= g.lcap) ? 1 : 0;
      if (!sh.list_sm) lbytes = 0;
    }
    if (rec_out && lane == 0) {
      rec_out->own_beg = sh.own_beg;
      rec_out->own_cnt = sh.own_cnt;
      rec_out->own_sm = sh.own_sm;
      rec_out->total = fits ? total : -1;
    }
    if (fits) {
      if (lane == 0) {
        mbar_arrive_expect_tx(&sh.bar, (uint32_t)total * 16u + (uint32_t)lbytes);
        if (lbytes > 0) bulk_g2s(slist, gblock, (uint32_t)lbytes, &sh.bar);
      }
      __syncwarp();
      // one lane per row: the row's cells as runs contiguous in memory (one,
      // or two where the row wraps around the box)
      if (lane < rows) {
        int u0 = 0, piece = 0;
        while (u0 < W) {
          const int t0 = lane * W + u0;
          int u1 = u0 + 1;
          while (u1 < W && sh.gbeg[lane * W + u1] == sh.gbeg[t0] + (sh.coff[lane * W + u1] - sh.coff[t0]))
            ++u1;
          const int n_at = sh.coff[lane * W + u1] - sh.coff[t0];
          if (n_at > 0) bulk_g2s(spos + sh.coff[t0], x + sh.gbeg[t0], (uint32_t)n_at * 16u, &sh.bar);
          if (rec_out && piece < 2) {
            rec_out->pg[2 * lane + piece] = sh.gbeg[t0];
            rec_out->ps[2 * lane + piece] = sh.coff[t0];
            rec_out->pn[2 * lane + piece] = n_at;
          }
          ++piece;
          u0 = u1;
        }
        for (; rec_out && piece < 2; ++piece) rec_out->pn[2 * lane + piece] = 0;
      }
      if (rec_out && lane >= rows && 2 * lane + 1 < kSegMaxPieces) {
        rec_out->pn[2 * lane] = 0;
        rec_out->pn[2 * lane + 1] = 0;
      }
    }
  }
  __syncthreads();
}

// Staging from the segment's record (written by the rebuild's search): the
// neighbourhood pieces and, when it fits in `slist`, the list block, on one
// mbarrier.  Every thread reads the record header itself (one line); one
// barrier publishes the mbarrier's initialisation, and the copies are then
// issued by warp 0 while the other warps go on.  Returns the header.
struct SegHead {
  int own_beg, own_cnt, own_sm, total, nck, list_sm;
};

template <int DIM>
__device__ __forceinline__ SegHead seg_stage_record(const SegGrid& g, const float4* __restrict__ x,
                                                    const SegRecord* __restrict__ rec, float4* spos,
                                                    SegShared& sh, int32_t* status,
                                                    const uint8_t* gblock, uint8_t* slist) {
  if (threadIdx.x == 0) {
    mbar_init(&sh.bar, 1);
    spos[g.cap] = seg_far_point();
  }
  SegHead h;
  const int4 r0 = __ldg(reinterpret_cast<const int4*>(rec));
  const int4 r1 = __ldg(reinterpret_cast<const int4*>(rec) + 1);
  h.own_beg = r0.x;
  h.own_cnt = r0.y;
  h.own_sm = r0.z;
  h.total = r0.w;
  h.nck = r1.x;
  const bool fits = h.total >= 0 && h.total <= g.cap;
  const int P = seg_pad(h.own_cnt);
  const int64_t lbytes = seg_block_used(P, h.nck);
  h.list_sm = (fits && slist != nullptr && P <= g.pmax && lbytes <= g.lcap) ? 1 : 0;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    if (!fits) {
      if (lane == 0) atomicOr(status, kSegStatusOverflow);
    } else {
      if (lane == 0) {
        mbar_arrive_expect_tx(&sh.bar, (uint32_t)h.total * 16u + (h.list_sm ? (uint32_t)lbytes : 0u));
        if (h.list_sm) bulk_g2s(slist, gblock, (uint32_t)lbytes, &sh.bar);
      }
      __syncwarp();
      if (lane < kSegMaxPieces) {
        const int n_at = __ldg(rec->pn + lane);
        if (n_at > 0)
          bulk_g2s(spos + __ldg(rec->ps + lane), x + __ldg(rec->pg + lane), (uint32_t)n_at * 16u,
                   &sh.bar);
      }
    }
  }
  if (!fits) h.total = -1;
  return h;
}

// Bounded wait of one thread for the staged block (no barrier).
__device__ __forceinline__ bool seg_wait_one(SegShared& sh, int32_t* status) {
  if (!mbar_wait_bounded(&sh.bar, kSegWaitNs)) {
    atomicOr(status, kSegStatusTimeout);
    mbar_wait_bounded(&sh.bar, kSegWaitNs);
    return false;
  }
  return true;
}

// Waits (bounded) for the staged block; afterwards sh.ok says whether it is
// usable (false: the neighbourhood exceeded g.cap, or a copy timed out; the
// status bit is set).  Every thread of the CTA must call it.
__device__ __forceinline__ bool seg_stage_wait(SegShared& sh, int32_t* status) {
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
  return sh.ok != 0;
}

template <int DIM>
__device__ __forceinline__ bool seg_stage(const SegGrid& g, const float4* __restrict__ x,
                                          const int32_t* __restrict__ start, float4* spos,
                                          SegShared& sh, int32_t* status,
                                          SegRecord* rec_out = nullptr) {
  seg_stage_issue<DIM>(g, x, start, spos, sh, status, nullptr, nullptr, nullptr, rec_out);
  return seg_stage_wait(sh, status);
}

// The CTA's periodic frame.  Along every dimension in which the CTA's staged
// cells include cell 0 or the last cell (it touches a face of the box),
// coordinates v >= L/2 become v - L, which is exact (Sterbenz: v is in
// [L/2, L)); along the others the staged cells do not wrap and coordinates
// stay.  With SegGrid::frame set (the staged cells of a face-touching CTA lie
// within half a box of the face) every pair of staged atoms within a cutoff
// is then separated by its minimum image as a plain difference, so the pair
// loops need no periodic test.  Returns the bit mask of shifted dimensions
// (bit d), so a kernel can restore a coordinate exactly: v' < 0 -> v' + L.
template <int DIM>
__device__ int seg_frame(const SegGrid& g, const SegShared& sh, float4* spos, const float L[3]) {
  const SegPos p = seg_pos<DIM>(g);
  int mask = 0;
  if (p.x0 == 0 || p.x0 + p.nx >= g.cps[0]) mask |= 1;
  if (p.cy == 0 || p.cy == g.cps[1] - 1) mask |= 2;
  if (DIM == 3 && (p.cz == 0 || p.cz == g.cps[2] - 1)) mask |= 4;
  if (mask) {
    const float h0 = 0.5f * L[0], h1 = 0.5f * L[1], h2 = 0.5f * L[2];
    for (int t = threadIdx.x; t < sh.total; t += blockDim.x) {
      float4 v = spos[t];
      if ((mask & 1) && v.x >= h0) v.x -= L[0];
      if ((mask & 2) && v.y >= h1) v.y -= L[1];
      if (DIM == 3 && (mask & 4) && v.z >= h2) v.z -= L[2];
      spos[t] = v;
    }
  }
  __syncthreads();
  return mask;
}

// Own cell (column u in 1..nx of the centre row) of the staged slot `is`.
template <int DIM>
__device__ __forceinline__ int seg_own_cell(const SegShared& sh, int is, int half) {
  const int cr = seg_centre_row<DIM>(half) * sh.W;
  int u = 1;
  while (u < sh.nx && sh.coff[cr + u + 1] <= is) ++u;
  return u;
}



}  // namespace jmd
