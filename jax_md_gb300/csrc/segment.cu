// Pair forces and the fused NVE step on the engine's segment-local list.
//
// Reference: jax_md/smap.py:922-979 (pair energy over a neighbour list),
// quantity.py:58-60 (force), simulate.py:227-243 (velocity_verlet),
// partition.py:1146-1154 (skin test).
//
// One CTA per segment (segment.cuh): the neighbourhood's positions are
// staged in shared memory by bulk copies on one mbarrier, each thread takes an
// own atom and walks its private list of 16-bit staged slots, 8 entries per
// 16-byte load (the next 8 loaded while the current 8 are evaluated), and
// evaluates pairs two at a time with packed FP32x2 arithmetic.  Neighbour
// positions come from shared memory, so a step reads from HBM only the list
// (2 bytes per entry) and the per-atom rows; the staged positions (13.8 MB
// for 864,000 atoms) are L2 traffic.  Species ids, when present, ride in the
// fourth float of the engine's private position rows.
#include "dense.cuh"
#include "segment.cuh"

namespace jmd {
namespace {

enum { S_FORCE = 0, S_STEP = 2, S_KICK = 3 };

struct SegStepArgs {
  const float4* x;
  const SegRecord* recs;     // per-segment staging records of the last rebuild
  const uint8_t* blocks;     // segment blocks (segment.cuh)
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
  int32_t* status;
  float fix_max;             // half lists: largest reaction component kept in fixed point
};

__device__ __forceinline__ int sclamp(int s, int nsp) { return s < 0 ? 0 : (s >= nsp ? nsp - 1 : s); }

// FRAME: the staged block is in the CTA's periodic frame (seg_frame), pair
// displacements are plain differences; otherwise atoms within the cutoff of
// a face take the minimum image per pair.
template <int DIM, int KIND, bool SPECIES, int MODE, bool FRAME>
__global__ void __maxnreg__(72)
k_seg_step(SegGrid sg, SegStepArgs a, const __grid_constant__ PairTable tab) {
  extern __shared__ float4 spos[];
  __shared__ SegShared sh;
  __shared__ PairCoef sc[SPECIES ? JMD_MAX_SPECIES * JMD_MAX_SPECIES : 1];
  if (SPECIES)
    for (int k = threadIdx.x; k < JMD_MAX_SPECIES * JMD_MAX_SPECIES; k += blockDim.x) sc[k] = tab.c[k];
  // staging from the segment's record: the positions (and the list block
  // when it fits in shared memory) arrive on one mbarrier; each thread's
  // first list chunks are requested meanwhile when the block stays in global
  // memory
  uint8_t* slist = reinterpret_cast<uint8_t*>(spos + sg.cap + 1);
  const uint8_t* gblk = a.blocks + (int64_t)blockIdx.x * sg.stride;
  const SegHead hd = seg_stage_record<DIM>(sg, a.x, a.recs + blockIdx.x, spos, sh, a.status, gblk,
                                           sg.lcap > 0 ? slist : nullptr);
  if (hd.total < 0) return;  // neighbourhood over capacity (flagged at the rebuild)
  const int P = seg_pad(hd.own_cnt);
  // more own atoms than a block holds (a cell over capacity, flagged at the
  // rebuild): the block was not written and is not read
  const bool blk_ok = P <= sg.pmax;
  const int nck_seg = blk_ok ? hd.nck : 0;
  const uint8_t* blk = hd.list_sm ? slist : gblk;
  const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
  const int o0 = threadIdx.x;
  int c_pre = 0;
  uint4 n1_pre = z4, n2_pre = z4;
  if (!hd.list_sm && blk_ok && o0 < hd.own_cnt) {
    const uint4* lp = reinterpret_cast<const uint4*>(gblk + seg_chunk_off(P, 0, o0));
    c_pre = min((int)reinterpret_cast<const uint16_t*>(gblk + 16)[o0], 8 * nck_seg);
    if (nck_seg > 0) n1_pre = lp[0];
    if (nck_seg > 1) n2_pre = lp[P];
  }
  bool ok = seg_wait_one(sh, a.status);
  int fmask = 0;
  if (FRAME) {
    const SegPos sp = seg_pos<DIM>(sg);
    if (sp.x0 == 0 || sp.x0 + sp.nx >= sg.cps[0]) fmask |= 1;
    if (sp.cy == 0 || sp.cy == sg.cps[1] - 1) fmask |= 2;
    if (DIM == 3 && (sp.cz == 0 || sp.cz == sg.cps[2] - 1)) fmask |= 4;
    if (fmask) {
      // face segments: all threads agree on the staged block, then shift it
      if (!__syncthreads_and(ok)) return;
      const float h0 = 0.5f * a.geo.L[0], h1 = 0.5f * a.geo.L[1], h2 = 0.5f * a.geo.L[2];
      for (int t = threadIdx.x; t < hd.total; t += blockDim.x) {
        float4 v = spos[t];
        if ((fmask & 1) && v.x >= h0) v.x -= a.geo.L[0];
        if ((fmask & 2) && v.y >= h1) v.y -= a.geo.L[1];
        if (DIM == 3 && (fmask & 4) && v.z >= h2) v.z -= a.geo.L[2];
        spos[t] = v;
      }
      __syncthreads();
    }
  }
  if (!ok) return;
  const float rc2m = tab.rc2_max;
  const Coef2 c0 = coef2(tab.c[0]);
  for (int o = threadIdx.x; o < hd.own_cnt; o += blockDim.x) {
    const int is = hd.own_sm + o, s = hd.own_beg + o;
    float4 xi = spos[is];
    const bool first = o == o0 && !hd.list_sm;
    // a block written for fewer chunks is read no further than it was written
    const int c = !blk_ok ? 0 : (first ? c_pre : min((int)reinterpret_cast<const uint16_t*>(blk + 16)[o], 8 * nck_seg));
    const uint4* lp = reinterpret_cast<const uint4*>(blk + seg_chunk_off(P, 0, o));
    const bool inner = FRAME || interior<DIM>(xi, a.geo, a.margin);
    const int si = SPECIES ? sclamp(__float_as_int(xi.w), tab.nsp) : 0;
    const float2 xx = f2s(xi.x), xy = f2s(xi.y), xz = f2s(xi.z);
    float2 ax = f2s(0.f), ay = f2s(0.f), az = f2s(0.f);

    auto pair2 = [&](int j0, int j1) {
      const float4 b0 = spos[j0], b1 = spos[j1];
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
        cc = coef2(sc[si * JMD_MAX_SPECIES + sclamp(__float_as_int(b0.w), tab.nsp)],
                   sc[si * JMD_MAX_SPECIES + sclamp(__float_as_int(b1.w), tab.nsp)]);
      else
        cc = c0;
      const float rc0 = SPECIES ? cc.rc2.x : rc2m, rc1 = SPECIES ? cc.rc2.y : rc2m;
      const bool m0 = r2.x < rc0 && r2.x > 0.f;
      const bool m1 = r2.y < rc1 && r2.y > 0.f;
      // masked pairs (beyond the cutoff, or the atom itself at r2 = 0) may
      // give inf/NaN here; the selects below discard them
      float2 U, g;
      pair_eval2<KIND, false>(r2, cc, U, g);
      g.x = m0 ? g.x : 0.f;
      g.y = m1 ? g.y : 0.f;
      ax = fma2(g, dx, ax);
      ay = fma2(g, dy, ay);
      if (DIM == 3) az = fma2(g, dz, az);
    };

    // entries past the count (to the end of the last chunk) point at the
    // far slot, beyond every cutoff
    // chunk k of this atom at lp + k P; two chunks in flight ahead (the
    // block is in shared memory, or in global memory when it did not fit)
    const int nck = (c + 7) >> 3;
    uint4 n1 = first ? n1_pre : (nck > 0 ? lp[0] : z4);
    uint4 n2 = first ? n2_pre : (nck > 1 ? lp[P] : z4);
    for (int kc = 0; kc < nck; ++kc) {
      const uint4 cur = n1;
      n1 = n2;
      if (kc + 2 < nck) n2 = lp[(int64_t)(kc + 2) * P];
      pair2((int)(cur.x & 0xFFFFu), (int)(cur.x >> 16));
      pair2((int)(cur.y & 0xFFFFu), (int)(cur.y >> 16));
      pair2((int)(cur.z & 0xFFFFu), (int)(cur.z >> 16));
      pair2((int)(cur.w & 0xFFFFu), (int)(cur.w >> 16));
    }
    const float fx = -(ax.x + ax.y), fy = -(ay.x + ay.y), fz = DIM == 3 ? -(az.x + az.y) : 0.f;
    if (FRAME && fmask) {
      // back to the box's coordinates, exactly (the frame subtracted L)
      if ((fmask & 1) && xi.x < 0.f) xi.x += a.geo.L[0];
      if ((fmask & 2) && xi.y < 0.f) xi.y += a.geo.L[1];
      if (DIM == 3 && (fmask & 4) && xi.z < 0.f) xi.z += a.geo.L[2];
    }
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f), rf = q;
    if (MODE == S_STEP || MODE == S_KICK) q = a.p[s];
    if (MODE == S_STEP && a.ref) rf = __ldg(a.ref + s);
    if (MODE == S_FORCE || MODE == S_KICK) a.f[s] = make_float4(fx, fy, fz, 0.f);
    const float h = 0.5f * a.dt;
    if (MODE == S_KICK) {
      q.x = fmaf(h, fx, q.x);
      q.y = fmaf(h, fy, q.y);
      q.z = fmaf(h, fz, q.z);
      a.p[s] = q;
    }
    if (MODE == S_STEP) {
      // closing half kick of step k, opening half kick of step k + 1, drift
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
      a.p[s] = q;
      a.x_next[s] = r;
      if (a.ref) {
        float ex, ey, ez;
        displacement<DIM>(r, rf, a.geo, ex, ey, ez);
        if (ex * ex + ey * ey + ez * ez > a.thr2) atomicOr(a.flag, 1);
      }
    }
  }
}

// Reaction accumulators of the half-list kernel are fixed point: 32-bit
// integer reductions in shared memory measured several times faster than
// float (and 64-bit) ones on this part.  A force component v with |v| <
// fix_max is added as round(v 2^19) (resolution 1.9e-6).  A staged atom takes
// at most (list width + 16) contributions within one CTA (as a partner of
// the segment's own atoms, plus its own chunk sums), so fix_max =
// min(64, 2^31 / (2^19 (width + 16))) keeps every slot's sum inside 32 bits;
// larger components (close contacts) go to global memory as float
// reductions.
constexpr float kFixScale = 524288.0f;  // 2^19
constexpr float kFixInv = 1.0f / 524288.0f;
constexpr float kFixMaxCap = 64.0f;

// (two's complement: an unsigned 32-bit add is the signed one)
__device__ __forceinline__ void red_shared_s32(int* p, int v) {
  asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(smem_u32(p)), "r"((unsigned)v) : "memory");
}

__device__ __forceinline__ void red_global_v4(float4* dst, float x, float y, float z) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(x), "f"(y), "f"(z),
               "f"(0.f)
               : "memory");
}

// Half lists (Newton's third law): each pair once, from the atom whose
// forward stencil holds the other.  The own atom keeps its force in
// registers and adds it to `f` once; the partner's reaction goes to a
// fixed-point shared-memory accumulator per staged atom, which the CTA then
// adds to `f` in global memory with one vector reduction per staged atom
// (f is zero before the kernel; k_seg_integrate consumes and clears it).
// cpre[0..n) = exclusive prefix of f(o) over o < n, cpre[n] = the total;
// every thread of the block calls it (warp shuffles + one value per warp).
template <typename F>
__device__ void seg_chunk_prefix(int n, int* cpre, F f) {
  __shared__ int wsum[kSegMaxThreads / 32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += blockDim.x) {
    const int o = base + threadIdx.x;
    const int v = o < n ? f(o) : 0;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = lane < nw ? wsum[lane] : 0;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, d);
        if (lane >= d) t += y;
      }
      if (lane < nw) wsum[lane] = t;
    }
    __syncthreads();
    const int excl = carry + (w ? wsum[w - 1] : 0) + x - v;
    if (o < n) cpre[o] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) cpre[n] = carry;
  __syncthreads();
}

template <int DIM, int KIND, bool SPECIES, bool FRAME>
__global__ void __maxnreg__(72)
k_seg_half(SegGrid sg, SegStepArgs a, const __grid_constant__ PairTable tab) {
  extern __shared__ float4 spos[];
  __shared__ SegShared sh;
  __shared__ PairCoef sc[SPECIES ? JMD_MAX_SPECIES * JMD_MAX_SPECIES : 1];
  if (SPECIES)
    for (int k = threadIdx.x; k < JMD_MAX_SPECIES * JMD_MAX_SPECIES; k += blockDim.x) sc[k] = tab.c[k];
  int* fx = reinterpret_cast<int*>(spos + sg.cap + 1);
  int* fy = fx + (sg.cap + 1);
  int* fz = fy + (sg.cap + 1);
  int* cpre = fz + (sg.cap + 1);  // [pmax + 1] chunk prefix
  const SegRecord* rec = a.recs + blockIdx.x;
  const uint8_t* gblk = a.blocks + (int64_t)blockIdx.x * sg.stride;
  const SegHead hd = seg_stage_record<DIM>(sg, a.x, rec, spos, sh, a.status, gblk, nullptr);
  if (hd.total < 0) return;  // neighbourhood over capacity (flagged at the rebuild)
  for (int t = threadIdx.x; t < hd.total; t += blockDim.x) {
    fx[t] = 0;
    fy[t] = 0;
    if (DIM == 3) fz[t] = 0;
  }
  const int P = seg_pad(hd.own_cnt);
  const bool blk_ok = P <= sg.pmax;
  const int nck_seg = blk_ok ? hd.nck : 0;
  bool ok = seg_wait_one(sh, a.status);
  // every thread meets this barrier: the accumulators are zero and, for a
  // face segment, the staged block is about to be shifted
  if (!__syncthreads_and(ok)) return;
  if (FRAME) {
    const SegPos sp = seg_pos<DIM>(sg);
    int fmask = 0;
    if (sp.x0 == 0 || sp.x0 + sp.nx >= sg.cps[0]) fmask |= 1;
    if (sp.cy == 0 || sp.cy == sg.cps[1] - 1) fmask |= 2;
    if (DIM == 3 && (sp.cz == 0 || sp.cz == sg.cps[2] - 1)) fmask |= 4;
    if (fmask) {
      const float h0 = 0.5f * a.geo.L[0], h1 = 0.5f * a.geo.L[1], h2 = 0.5f * a.geo.L[2];
      for (int t = threadIdx.x; t < hd.total; t += blockDim.x) {
        float4 v = spos[t];
        if ((fmask & 1) && v.x >= h0) v.x -= a.geo.L[0];
        if ((fmask & 2) && v.y >= h1) v.y -= a.geo.L[1];
        if (DIM == 3 && (fmask & 4) && v.z >= h2) v.z -= a.geo.L[2];
        spos[t] = v;
      }
      __syncthreads();
    }
  }
  const float rc2m = tab.rc2_max;
  const Coef2 c0 = coef2(tab.c[0]);
  // chunk-balanced work: the threads take the segment's 8-entry list chunks
  // in atom order (cpre = exclusive prefix of the atoms' chunk counts), so
  // a row's length decides how many threads share it rather than how long
  // one thread runs
  const uint16_t* cnts = reinterpret_cast<const uint16_t*>(gblk + 16);
  const int nown = blk_ok ? hd.own_cnt : 0;  // cpre holds pmax + 1 entries
  seg_chunk_prefix(nown, cpre, [&](int o) {
    const int c = min((int)cnts[o], 8 * nck_seg);
    return (c + 7) >> 3;
  });
  const int nchunks = cpre[nown];
  // chunk u -> (own atom o, its chunk kc), and that chunk's list entries
  auto locate = [&](int u, int& o, int& kc) {
    int lo = 0, hi = nown - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (cpre[mid] <= u) lo = mid; else hi = mid - 1;
    }
    o = lo;
    kc = u - cpre[lo];
  };
  int o_next = 0, kc_next = 0;
  uint4 next = make_uint4(0u, 0u, 0u, 0u);
  if (threadIdx.x < nchunks) {
    locate(threadIdx.x, o_next, kc_next);
    next = *reinterpret_cast<const uint4*>(gblk + seg_chunk_off(P, kc_next, o_next));
  }
  for (int u = threadIdx.x; u < nchunks; u += blockDim.x) {
    const int o = o_next, kc = kc_next;
    const uint4 cur = next;
    // the next chunk's entries are in flight while this one is evaluated
    if (u + (int)blockDim.x < nchunks) {
      locate(u + blockDim.x, o_next, kc_next);
      next = *reinterpret_cast<const uint4*>(gblk + seg_chunk_off(P, kc_next, o_next));
    }
    (void)kc;
    const int is = hd.own_sm + o;
    const float4 xi = spos[is];
    const bool inner = FRAME || interior<DIM>(xi, a.geo, a.margin);
    const int si = SPECIES ? sclamp(__float_as_int(xi.w), tab.nsp) : 0;
    const float2 xx = f2s(xi.x), xy = f2s(xi.y), xz = f2s(xi.z);
    float2 ax = f2s(0.f), ay = f2s(0.f), az = f2s(0.f);
    // a force into a staged slot: 32-bit fixed point in shared memory, or a
    // close contact straight to the atom's sorted slot (the pieces partition
    // the staged slots; a slot outside them is skipped rather than written)
    auto deposit = [&](int j, float vx, float vy, float vz) {
      if (fabsf(vx) < a.fix_max && fabsf(vy) < a.fix_max && fabsf(vz) < a.fix_max) {
        red_shared_s32(fx + j, __float2int_rn(vx * kFixScale));
        red_shared_s32(fy + j, __float2int_rn(vy * kFixScale));
        if (DIM == 3) red_shared_s32(fz + j, __float2int_rn(vz * kFixScale));
      } else {
        for (int q = 0; q < kSegMaxPieces; ++q) {
          const int ps = __ldg(rec->ps + q), pn = __ldg(rec->pn + q);
          if (pn > 0 && j >= ps && j < ps + pn) {
            red_global_v4(a.f + __ldg(rec->pg + q) + (j - ps), vx, vy, vz);
            break;
          }
        }
      }
    };
    auto pair2 = [&](int j0, int j1) {
      const float4 b0 = spos[j0], b1 = spos[j1];
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
        cc = coef2(sc[si * JMD_MAX_SPECIES + sclamp(__float_as_int(b0.w), tab.nsp)],
                   sc[si * JMD_MAX_SPECIES + sclamp(__float_as_int(b1.w), tab.nsp)]);
      else
        cc = c0;
      const float rc0 = SPECIES ? cc.rc2.x : rc2m, rc1 = SPECIES ? cc.rc2.y : rc2m;
      const bool m0 = r2.x < rc0 && r2.x > 0.f;
      const bool m1 = r2.y < rc1 && r2.y > 0.f;
      float2 U, g;
      pair_eval2<KIND, false>(r2, cc, U, g);
      g.x = m0 ? g.x : 0.f;
      g.y = m1 ? g.y : 0.f;
      const float2 gx = mul2(g, dx), gy = mul2(g, dy);
      ax = add2(ax, gx);
      ay = add2(ay, gy);
      float2 gz = f2s(0.f);
      if (DIM == 3) {
        gz = mul2(g, dz);
        az = add2(az, gz);
      }
      // reactions (masked pairs, the far slot included, add nothing).  One
      // packed test of both pair forces' squared magnitudes, g^2 r^2 <
      // fix_max^2, clears both for the fixed-point path (each component is
      // at most the magnitude); otherwise each pair goes through deposit's
      // per-component test
      const float2 f2m = mul2(mul2(g, g), r2);
      const float fix2 = a.fix_max * a.fix_max;
      if (f2m.x < fix2 && f2m.y < fix2) {
        if (m0) {
          red_shared_s32(fx + j0, __float2int_rn(gx.x * kFixScale));
          red_shared_s32(fy + j0, __float2int_rn(gy.x * kFixScale));
          if (DIM == 3) red_shared_s32(fz + j0, __float2int_rn(gz.x * kFixScale));
        }
        if (m1) {
          red_shared_s32(fx + j1, __float2int_rn(gx.y * kFixScale));
          red_shared_s32(fy + j1, __float2int_rn(gy.y * kFixScale));
          if (DIM == 3) red_shared_s32(fz + j1, __float2int_rn(gz.y * kFixScale));
        }
      } else {
        if (m0) deposit(j0, gx.x, gy.x, DIM == 3 ? gz.x : 0.f);
        if (m1) deposit(j1, gx.y, gy.y, DIM == 3 ? gz.y : 0.f);
      }
    };
    pair2((int)(cur.x & 0xFFFFu), (int)(cur.x >> 16));
    pair2((int)(cur.y & 0xFFFFu), (int)(cur.y >> 16));
    pair2((int)(cur.z & 0xFFFFu), (int)(cur.z >> 16));
    pair2((int)(cur.w & 0xFFFFu), (int)(cur.w >> 16));
    // this chunk's share of the own atom's force, F_i = -sum g d (the
    // reactions were +g d), into the own atom's staged slot
    deposit(is, -(ax.x + ax.y), -(ay.x + ay.y), DIM == 3 ? -(az.x + az.y) : 0.f);
  }
  __syncthreads();
  // flush: every staged atom's accumulated force to its sorted slot
  const int npieces = kSegMaxPieces;
  for (int p = 0; p < npieces; ++p) {
    const int n_at = __ldg(rec->pn + p);
    if (n_at <= 0) continue;
    const int ps = __ldg(rec->ps + p), pg = __ldg(rec->pg + p);
    for (int t = threadIdx.x; t < n_at; t += blockDim.x) {
      const int ix = fx[ps + t], iy = fy[ps + t], iz = DIM == 3 ? fz[ps + t] : 0;
      if (ix | iy | iz)
        red_global_v4(a.f + pg + t, (float)ix * kFixInv, (float)iy * kFixInv,
                      (float)iz * kFixInv);
    }
  }
}

// Consumes the half-list forces: mode 2 (step) p += dt f, x' = x + dt p / m
// (the closing half kick of step k, the opening one of k + 1, the drift),
// skin test, f cleared; mode 3 (kick) p += dt/2 f, f kept.
template <int DIM, int MODE>
__global__ void k_seg_integrate(int n, float4* f, float4* p, const float4* x, float4* x_next,
                                const float4* ref, float m0, float dt, float thr2, int32_t* flag,
                                Geo geo) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (s < n) {
    const float4 fs = f[s];
    float4 q = p[s];
    const float h = 0.5f * dt;
    q.x = fmaf(h, fs.x, q.x);
    q.y = fmaf(h, fs.y, q.y);
    if (DIM == 3) q.z = fmaf(h, fs.z, q.z);
    if (MODE == S_STEP) {
      q.x = fmaf(h, fs.x, q.x);
      q.y = fmaf(h, fs.y, q.y);
      if (DIM == 3) q.z = fmaf(h, fs.z, q.z);
      float4 r = x[s];
      const float ddx = dt * q.x / m0, ddy = dt * q.y / m0, ddz = dt * q.z / m0;
      if (geo.periodic) {
        r.x = wrap(r.x + ddx, geo.L[0]);
        r.y = wrap(r.y + ddy, geo.L[1]);
        if (DIM == 3) r.z = wrap(r.z + ddz, geo.L[2]);
      } else {
        r.x += ddx;
        r.y += ddy;
        if (DIM == 3) r.z += ddz;
      }
      x_next[s] = r;
      f[s] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (ref) {
        float ex, ey, ez;
        displacement<DIM>(r, __ldg(ref + s), geo, ex, ey, ez);
        over = ex * ex + ey * ey + ez * ez > thr2;
      }
    }
    p[s] = q;
  }
  if (MODE == S_STEP && flag && __any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0)
    atomicOr(flag, 1);
}

template <int DIM, int KIND, bool SP, bool FRAME>
int seg_half_go(const SegGrid& g, const SegStepArgs& a, const PairTable& t, cudaStream_t st) {
  const size_t smem = (size_t)(g.cap + 1) * (sizeof(float4) + 3 * sizeof(int)) +
                      (size_t)(g.pmax + 1) * sizeof(int);
  auto k = k_seg_half<DIM, KIND, SP, FRAME>;
  if (smem > 48 * 1024)
    JMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k<<<(unsigned)g.nseg, (unsigned)g.threads, smem, st>>>(g, a, t);
  return JMD_OK;
}

template <int DIM, int KIND>
int seg_half_sp(bool sp, const SegGrid& g, const SegStepArgs& a, const PairTable& t, cudaStream_t st) {
  if (g.frame)
    return sp ? seg_half_go<DIM, KIND, true, true>(g, a, t, st)
              : seg_half_go<DIM, KIND, false, true>(g, a, t, st);
  return sp ? seg_half_go<DIM, KIND, true, false>(g, a, t, st)
            : seg_half_go<DIM, KIND, false, false>(g, a, t, st);
}

int seg_half_launch(int dim, int kind, bool sp, const SegGrid& g, const SegStepArgs& a,
                    const PairTable& t, cudaStream_t st) {
  if (dim == 3) {
    if (kind == JMD_LJ) return seg_half_sp<3, JMD_LJ>(sp, g, a, t, st);
    if (kind == JMD_LJ_TRUNCATED) return seg_half_sp<3, JMD_LJ_TRUNCATED>(sp, g, a, t, st);
    if (kind == JMD_MORSE) return seg_half_sp<3, JMD_MORSE>(sp, g, a, t, st);
    return seg_half_sp<3, JMD_SOFT_SPHERE>(sp, g, a, t, st);
  }
  if (kind == JMD_LJ) return seg_half_sp<2, JMD_LJ>(sp, g, a, t, st);
  if (kind == JMD_LJ_TRUNCATED) return seg_half_sp<2, JMD_LJ_TRUNCATED>(sp, g, a, t, st);
  if (kind == JMD_MORSE) return seg_half_sp<2, JMD_MORSE>(sp, g, a, t, st);
  return seg_half_sp<2, JMD_SOFT_SPHERE>(sp, g, a, t, st);
}

template <int DIM, int KIND, bool SP, int MODE, bool FRAME>
int seg_go(const SegGrid& g, const SegStepArgs& a, const PairTable& t, cudaStream_t st) {
  const size_t smem = (size_t)(g.cap + 1) * sizeof(float4) + (size_t)g.lcap;
  auto k = k_seg_step<DIM, KIND, SP, MODE, FRAME>;
  if (smem > 48 * 1024)
    JMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k<<<(unsigned)g.nseg, (unsigned)g.threads, smem, st>>>(g, a, t);
  return JMD_OK;
}

template <int DIM, int KIND, int MODE>
int seg_sp(bool sp, const SegGrid& g, const SegStepArgs& a, const PairTable& t, cudaStream_t st) {
  if (g.frame)
    return sp ? seg_go<DIM, KIND, true, MODE, true>(g, a, t, st)
              : seg_go<DIM, KIND, false, MODE, true>(g, a, t, st);
  return sp ? seg_go<DIM, KIND, true, MODE, false>(g, a, t, st)
            : seg_go<DIM, KIND, false, MODE, false>(g, a, t, st);
}

template <int MODE>
int seg_launch(int dim, int kind, bool sp, const SegGrid& g, const SegStepArgs& a,
               const PairTable& t, cudaStream_t st) {
  if (dim == 3) {
    if (kind == JMD_LJ) return seg_sp<3, JMD_LJ, MODE>(sp, g, a, t, st);
    if (kind == JMD_LJ_TRUNCATED) return seg_sp<3, JMD_LJ_TRUNCATED, MODE>(sp, g, a, t, st);
    if (kind == JMD_MORSE) return seg_sp<3, JMD_MORSE, MODE>(sp, g, a, t, st);
    return seg_sp<3, JMD_SOFT_SPHERE, MODE>(sp, g, a, t, st);
  }
  if (kind == JMD_LJ) return seg_sp<2, JMD_LJ, MODE>(sp, g, a, t, st);
  if (kind == JMD_LJ_TRUNCATED) return seg_sp<2, JMD_LJ_TRUNCATED, MODE>(sp, g, a, t, st);
  if (kind == JMD_MORSE) return seg_sp<2, JMD_MORSE, MODE>(sp, g, a, t, st);
  return seg_sp<2, JMD_SOFT_SPHERE, MODE>(sp, g, a, t, st);
}

}  // namespace

// Engine entry (declared in pair.cuh): mode 0 forces, 2 fused NVE step, 3
// force + closing half kick.
int seg_step(int mode, const jmd_pair& pp, const jmd_space& space, const SegGrid& g,
             const float* x, const int32_t* start, const uint8_t* list, float* f, float* p,
             float* x_next, float m0, float dt, const float* ref, float thr2, int32_t* flag,
             int32_t* status, bool species, cudaStream_t st, int64_t n_atoms) {
  int e = validate_pair(&pp);
  if (e) return e;
  PairTable t = make_pair_table(pp);
  SegStepArgs a{};
  a.x = reinterpret_cast<const float4*>(x);
  a.recs = reinterpret_cast<const SegRecord*>(list + seg_table_bytes(g.nseg));
  a.blocks = list + seg_table_bytes(g.nseg) + seg_records_bytes(g.nseg);
  (void)start;
  a.f = reinterpret_cast<float4*>(f);
  a.geo = make_geo(space);
  a.margin = sqrtf(t.rc2_max);
  a.p = reinterpret_cast<float4*>(p);
  a.x_next = reinterpret_cast<float4*>(x_next);
  a.m0 = m0;
  a.dt = dt;
  a.ref = reinterpret_cast<const float4*>(ref);
  a.thr2 = thr2;
  a.flag = flag;
  a.status = status;
  // rows hold at most 8 nch entries
  a.fix_max = fminf(kFixMaxCap, 2147483648.0f / (kFixScale * (float)(8 * g.nch + 16)));
  if (g.half) {
    // forces into f (zero on entry), then the integration
    a.f = reinterpret_cast<float4*>(f);
    e = seg_half_launch(space.dim, pp.kind, species, g, a, t, st);
    if (e) return e;
    if (mode == S_FORCE) return check_launch("jmd segment half forces");
    const unsigned gr = (unsigned)std::max<int64_t>(1, ceil_div(n_atoms, 256));
    float4* f4 = reinterpret_cast<float4*>(f);
    float4* p4 = reinterpret_cast<float4*>(p);
    const float4* x4 = reinterpret_cast<const float4*>(x);
    float4* xn4 = reinterpret_cast<float4*>(x_next);
    const float4* r4 = reinterpret_cast<const float4*>(ref);
    if (space.dim == 3) {
      if (mode == S_STEP)
        k_seg_integrate<3, S_STEP><<<gr, 256, 0, st>>>((int)n_atoms, f4, p4, x4, xn4, r4, m0, dt, thr2, flag, a.geo);
      else
        k_seg_integrate<3, S_KICK><<<gr, 256, 0, st>>>((int)n_atoms, f4, p4, x4, xn4, r4, m0, dt, thr2, flag, a.geo);
    } else {
      if (mode == S_STEP)
        k_seg_integrate<2, S_STEP><<<gr, 256, 0, st>>>((int)n_atoms, f4, p4, x4, xn4, r4, m0, dt, thr2, flag, a.geo);
      else
        k_seg_integrate<2, S_KICK><<<gr, 256, 0, st>>>((int)n_atoms, f4, p4, x4, xn4, r4, m0, dt, thr2, flag, a.geo);
    }
    return check_launch("jmd segment half step");
  }
  if (mode == S_STEP) e = seg_launch<S_STEP>(space.dim, pp.kind, species, g, a, t, st);
  else if (mode == S_KICK) e = seg_launch<S_KICK>(space.dim, pp.kind, species, g, a, t, st);
  else e = seg_launch<S_FORCE>(space.dim, pp.kind, species, g, a, t, st);
  if (e) return e;
  return check_launch("jmd segment step");
}

}  // namespace jmd
