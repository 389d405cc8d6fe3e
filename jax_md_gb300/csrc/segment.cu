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
  const int32_t* start;
  const uint16_t* list;
  int64_t nch;
  int width;
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
  int32_t* status;
};

__device__ __forceinline__ int sclamp(int s, int nsp) { return s < 0 ? 0 : (s >= nsp ? nsp - 1 : s); }

template <int DIM, int KIND, bool SPECIES, int MODE>
__global__ void __launch_bounds__(kSegMaxThreads)
k_seg_step(SegGrid sg, SegStepArgs a, const __grid_constant__ PairTable tab) {
  extern __shared__ float4 spos[];
  __shared__ SegShared sh;
  __shared__ PairCoef sc[SPECIES ? JMD_MAX_SPECIES * JMD_MAX_SPECIES : 1];
  if (SPECIES)
    for (int k = threadIdx.x; k < JMD_MAX_SPECIES * JMD_MAX_SPECIES; k += blockDim.x) sc[k] = tab.c[k];
  seg_stage<DIM>(sg, a.x, a.start, spos, sh, a.status);
  if (!sh.ok) return;
  const float rc2m = tab.rc2_max;
  const Coef2 c0 = coef2(tab.c[0]);
  for (int o = threadIdx.x; o < sh.own_cnt; o += blockDim.x) {
    const int is = sh.own_sm + o, s = sh.own_beg + o;
    const float4 xi = spos[is];
    const int c = min(__ldg(a.cnt + s), a.width);
    const uint4* lp = reinterpret_cast<const uint4*>(a.list + seg_list_base(s, a.nch));
    const bool inner = interior<DIM>(xi, a.geo, a.margin);
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

    // entries past the count point at the atom itself (distance 0: masked)
    const int nck = (c + 7) >> 3;
    uint4 nxt = nck > 0 ? __ldcs(lp) : make_uint4(0u, 0u, 0u, 0u);
    for (int kc = 0; kc < nck; ++kc) {
      const uint4 cur = nxt;
      if (kc + 1 < nck) nxt = __ldcs(lp + (int64_t)(kc + 1) * 32);
      const int k0 = kc * 8;
      const uint32_t wv[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int j0 = (k0 + 2 * m < c) ? (int)(wv[m] & 0xFFFFu) : is;
        const int j1 = (k0 + 2 * m + 1 < c) ? (int)(wv[m] >> 16) : is;
        pair2(j0, j1);
      }
    }
    const float fx = -(ax.x + ax.y), fy = -(ay.x + ay.y), fz = DIM == 3 ? -(az.x + az.y) : 0.f;
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

template <int DIM, int KIND, int MODE>
int seg_sp(bool sp, const SegGrid& g, const SegStepArgs& a, const PairTable& t, cudaStream_t st) {
  const size_t smem = (size_t)g.cap * sizeof(float4);
  if (sp) {
    auto k = k_seg_step<DIM, KIND, true, MODE>;
    if (smem > 48 * 1024)
      JMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<(unsigned)g.nseg, (unsigned)g.threads, smem, st>>>(g, a, t);
  } else {
    auto k = k_seg_step<DIM, KIND, false, MODE>;
    if (smem > 48 * 1024)
      JMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<(unsigned)g.nseg, (unsigned)g.threads, smem, st>>>(g, a, t);
  }
  return JMD_OK;
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
             const float* x, const int32_t* start, const uint16_t* list, int64_t nch, int64_t width,
             const int32_t* cnt, float* f, float* p, float* x_next, float m0, float dt,
             const float* ref, float thr2, int32_t* flag, int32_t* status, bool species,
             cudaStream_t st) {
  int e = validate_pair(&pp);
  if (e) return e;
  PairTable t = make_pair_table(pp);
  SegStepArgs a{};
  a.x = reinterpret_cast<const float4*>(x);
  a.start = start;
  a.list = list;
  a.nch = nch;
  a.width = (int)std::min<int64_t>(width, nch * 8);
  a.cnt = cnt;
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
  if (mode == S_STEP) e = seg_launch<S_STEP>(space.dim, pp.kind, species, g, a, t, st);
  else if (mode == S_KICK) e = seg_launch<S_KICK>(space.dim, pp.kind, species, g, a, t, st);
  else e = seg_launch<S_FORCE>(space.dim, pp.kind, species, g, a, t, st);
  if (e) return e;
  return check_launch("jmd segment step");
}

}  // namespace jmd
