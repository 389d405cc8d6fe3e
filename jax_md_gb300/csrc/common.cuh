// Shared device helpers for the GB300 short-range MD kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/jax_md_gb300.h"

namespace jmd {

// ----------------------------------------------------------------- errors --
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int check_launch(const char* what);

#define JMD_REQUIRE(cond, msg)                                   \
  do {                                                           \
    if (!(cond)) return ::jmd::fail(JMD_ERR_INVALID_ARGUMENT, msg); \
  } while (0)

#define JMD_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      return ::jmd::fail(JMD_ERR_CUDA, std::string(#call) + ": " +            \
                                           cudaGetErrorString(e_));           \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

constexpr int kWarp = 32;

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Carves aligned sub-buffers out of a caller workspace.
struct Carver {
  char* base;
  size_t used = 0;
  size_t cap;
  Carver(void* b, size_t c) : base(static_cast<char*>(b)), cap(c) {}
  template <typename T>
  T* take(int64_t count) {
    used = align_up(used, 256);
    T* p = reinterpret_cast<T*>(base ? base + used : nullptr);
    used += sizeof(T) * static_cast<size_t>(count);
    return p;
  }
  bool ok() const { return base != nullptr && used <= cap; }
};

// ------------------------------------------------------------- geometry ----
struct Geo {
  int dim;
  int periodic;  // nonzero: minimum image over L (the unit cube for a general cell)
  int general;   // space.periodic_general, fractional coordinates
  float L[3];
  float halfL[3];
  float T[6];    // upper-triangular cell: xx xy xz yy yz zz
  float Ti[6];   // its inverse, same layout
};

inline Geo make_geo(const jmd_space& s) {
  Geo g;
  g.dim = s.dim;
  g.periodic = s.periodic;
  g.general = s.periodic == JMD_GENERAL_CELL;
  for (int d = 0; d < 3; ++d) {
    g.L[d] = g.general ? 1.f : s.box[d];
    g.halfL[d] = 0.5f * g.L[d];
  }
  const int up[6] = {0, 1, 2, 4, 5, 8};
  for (int k = 0; k < 6; ++k) {
    g.T[k] = g.general ? s.cell[up[k]] : 0.f;
    g.Ti[k] = g.general ? s.inv_cell[up[k]] : 0.f;
  }
  return g;
}

// v <- M v for an upper-triangular M in the Geo layout (space.transform,
// space.py:125-148, x = T u).  In 2D only xx, xy, yy enter.
template <int DIM>
__device__ __forceinline__ void cell_apply(const float* m, float& x, float& y, float& z) {
  if (DIM == 3) {
    x = fmaf(m[0], x, fmaf(m[1], y, m[2] * z));
    y = fmaf(m[3], y, m[4] * z);
    z = m[5] * z;
  } else {
    x = fmaf(m[0], x, m[1] * y);
    y = m[3] * y;
  }
}

// Minimum-image displacement a - b along one axis for coordinates inside the
// box.  The wrapped branches subtract L from the coordinate that lies in the
// upper half first, which is exact (Sterbenz), so the result carries a single
// rounding; and d(a, b) == -d(b, a) bit for bit.  JAX MD computes
// mod(a - b + L/2, L) - L/2 (space.py:213-224); for coordinates in [0, L) both
// give the same minimum image, this form with smaller rounding error.
__device__ __forceinline__ float min_image(float a, float b, float L, float halfL) {
  float d = a - b;
  if (d > halfL) {
    d = (a - L) - b;
  } else if (d < -halfL) {
    d = a - (b - L);
  }
  return d;
}

// Floored mod for |x| < 2L as space.periodic_shift (space.py:250-252):
// mod(y, L) with y = x + dx; fmod is exact, so y - L / y + L reproduce it.
__device__ __forceinline__ float wrap(float y, float L) {
  if (y >= L) {
    y -= L;
    if (y >= L) y = fmodf(y, L);
  } else if (y < 0.f) {
    float r = fmodf(y, L);
    y = (r < 0.f) ? r + L : r;
  }
  return y;
}

// Position row loaders.  VEC4: rows are float4 (stride 4, 16-byte aligned).
template <int DIM, bool VEC4>
__device__ __forceinline__ float4 load_row(const float* __restrict__ x, int64_t stride, int64_t i) {
  if (VEC4) {
    return __ldg(reinterpret_cast<const float4*>(x) + i);
  } else {
    const float* p = x + i * stride;
    float4 r;
    r.x = __ldg(p);
    r.y = __ldg(p + 1);
    r.z = (DIM == 3) ? __ldg(p + 2) : 0.f;
    r.w = 0.f;
    return r;
  }
}

template <int DIM, bool VEC4>
__device__ __forceinline__ float4 load_row_rw(const float* x, int64_t stride, int64_t i) {
  if (VEC4) {
    return reinterpret_cast<const float4*>(x)[i];
  } else {
    const float* p = x + i * stride;
    float4 r;
    r.x = p[0];
    r.y = p[1];
    r.z = (DIM == 3) ? p[2] : 0.f;
    r.w = 0.f;
    return r;
  }
}

// Stores x/y/z of v; the fourth float of a float4 row is preserved.
template <int DIM, bool VEC4>
__device__ __forceinline__ void store_row(float* x, int64_t stride, int64_t i, float4 v) {
  if (VEC4) {
    float4* p = reinterpret_cast<float4*>(x) + i;
    v.w = p->w;
    *p = v;
  } else {
    float* p = x + i * stride;
    p[0] = v.x;
    p[1] = v.y;
    if (DIM == 3) p[2] = v.z;
  }
}

// Overwrites the whole float4 row (w = 0) when VEC4.
template <int DIM, bool VEC4>
__device__ __forceinline__ void store_row_full(float* x, int64_t stride, int64_t i, float4 v) {
  if (VEC4) {
    v.w = 0.f;
    reinterpret_cast<float4*>(x)[i] = v;
  } else {
    float* p = x + i * stride;
    p[0] = v.x;
    p[1] = v.y;
    if (DIM == 3) p[2] = v.z;
  }
}

inline bool is_vec4(const void* p, int64_t stride) {
  return stride == 4 && (reinterpret_cast<uintptr_t>(p) % 16) == 0;
}

// ------------------------------------------------------------ reductions ---
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic grid reduction of NV doubles: block sums go to `partials`
// [gridDim.x * NV]; the last block to finish adds them in a fixed order and
// writes (or accumulates into) out[NV], then resets *counter to zero.  The
// result depends only on the grid size, not on block scheduling.
template <int NV>
__device__ void grid_reduce(double (&v)[NV], double* partials, unsigned int* counter,
                            double* out, bool accumulate) {
  __shared__ double sm[NV][32];
  __shared__ bool is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = warp_sum(v[k]);
    if (lane == 0) sm[k][warp] = s;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < nwarps ? sm[k][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0) partials[(size_t)blockIdx.x * NV + k] = s;
    }
  }
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned int t = atomicAdd(counter, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] += __ldcg(partials + (size_t)b * NV + k);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = warp_sum(acc[k]);
    if (lane == 0) sm[k][warp] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int w = 0; w < nwarps; ++w) s += sm[k][w];
      out[k] = accumulate ? out[k] + s : s;
    }
    *counter = 0u;
  }
}

}  // namespace jmd
