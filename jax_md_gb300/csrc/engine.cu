// Device-resident NVE runner: the reference's simulation loop
//   for s in range(n): nbrs = nbrs.update(x); state = apply_fn(state, neighbor=nbrs)
// (jax_md/partition.py:841-854, jax_md/simulate.py:279-317) with the host
// taken out of the loop.
//
// Per run of n steps:
//   skin test (x0)          -> conditional rebuild
//   kick + drift            (p' = p + dt/2 f, x1)        + skin test (x1)
//   n-1 times:              conditional rebuild;  fused step  x_s -> x_{s+1}
//                           (F(x_s), both half kicks, drift, skin test)
//   conditional rebuild;    force + closing half kick at x_n
// Positions ping-pong between `position` and `position_alt`; the final
// positions are copied back into `position` when the run ends in the other
// buffer.
//
// Graph mode records this sequence once per (system, n) into a CUDA graph.
// Each "conditional rebuild" is a one-thread kernel that copies the device
// rebuild flag into a graph conditional handle (cudaGraphSetConditional) and
// an IF node whose body is the rebuild chain, so a step without a rebuild
// costs nothing for the rebuild kernels; the flag itself is cleared by the
// rebuild's last kernel.  Direct mode launches the same kernels with the
// rebuild chain gated by the device flag inside each kernel.
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "pair.cuh"

namespace jmd {
namespace {

__global__ void k_set_cond(cudaGraphConditionalHandle h, const int32_t* flag) {
  cudaGraphSetConditional(h, *flag != 0 ? 1u : 0u);
}

__global__ void k_set_flag(int32_t* flag) { *flag = 1; }

struct GraphPlan {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

std::mutex g_mu;
std::map<std::string, GraphPlan> g_cache;

int validate_sys(const jmd_nve_system& s) {
  JMD_REQUIRE(s.n > 0 && s.n < INT32_MAX, "atom count out of range");
  JMD_REQUIRE(s.pair.particle_sigma == nullptr && s.pair.particle_epsilon == nullptr,
              "the engine's kernels take scalar or species parameters (per-particle parameters "
              "run on jmd_pair_forces)");
  JMD_REQUIRE(s.space.dim == 2 || s.space.dim == 3, "dim must be 2 or 3");
  JMD_REQUIRE(s.space.periodic != JMD_GENERAL_CELL && s.nlist.space.periodic != JMD_GENERAL_CELL,
              "the engine runs space.periodic / space.free systems (general cells run step by "
              "step on jmd_pair_forces and the integrator kernels)");
  JMD_REQUIRE(s.nlist.format == JMD_DENSE, "the engine runs Dense neighbour lists");
  JMD_REQUIRE(s.position && s.position_alt && s.momentum && s.force && s.idx &&
                  s.reference_position && s.error_code && s.occupancy && s.rebuild_flag,
              "null buffer in jmd_nve_system");
  JMD_REQUIRE(s.position != s.position_alt, "position_alt must be a separate buffer");
  for (const void* p : {(const void*)s.position, (const void*)s.position_alt,
                        (const void*)s.momentum, (const void*)s.force,
                        (const void*)s.reference_position})
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(p) % 16) == 0, "float4 rows must be 16-byte aligned");
  JMD_REQUIRE(s.idx_ld >= s.nlist.max_occupancy && s.idx_ld % 2 == 0, "idx_ld must be even and >= max_occupancy");
  return JMD_OK;
}

// One rebuild of the Dense list at positions x (gated by the device flag).
int rebuild(const jmd_nve_system& s, const float* x, bool gated, cudaStream_t st) {
  return jmd_neighbor_list_build(&s.nlist, x, 4, s.n, s.idx, s.idx_ld, s.nbr_count, s.occupancy,
                                 s.error_code, s.reference_position, 4,
                                 gated ? s.rebuild_flag : nullptr, s.nl_workspace,
                                 s.nl_workspace_bytes, st);
}

// Appends "set conditional from flag; IF { body(body_st) }" to the capture on st.
template <typename Body>
int conditional(const int32_t* rebuild_flag, Body body, cudaStream_t st, cudaStream_t body_st) {
  cudaStreamCaptureStatus status;
  cudaGraph_t graph;
  JMD_CUDA(cudaStreamGetCaptureInfo(st, &status, nullptr, &graph, nullptr, nullptr, nullptr));
  if (status != cudaStreamCaptureStatusActive) return fail(JMD_ERR_CUDA, "stream is not capturing");
  cudaGraphConditionalHandle h;
  JMD_CUDA(cudaGraphConditionalHandleCreate(&h, graph, 0, cudaGraphCondAssignDefault));
  k_set_cond<<<1, 1, 0, st>>>(h, rebuild_flag);
  JMD_CUDA(cudaGetLastError());
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  JMD_CUDA(cudaStreamGetCaptureInfo(st, &status, nullptr, &graph, &deps, nullptr, &ndeps));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  JMD_CUDA(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp));
  cudaGraph_t body_graph = cp.conditional.phGraph_out[0];
  JMD_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  JMD_CUDA(cudaStreamBeginCaptureToGraph(body_st, body_graph, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal));
  int rc = body(body_st);
  cudaGraph_t out;
  cudaError_t e = cudaStreamEndCapture(body_st, &out);
  if (rc) return rc;
  JMD_CUDA(e);
  return JMD_OK;
}

// Enqueues the whole run; `graphed` selects conditional nodes vs gated kernels.
// With `traj`, positions step through its slots (slot k = x_k, slot 0 a copy
// of the start) instead of ping-ponging; `force_rebuild` rebuilds at x_0
// whatever the skin test says.
int enqueue_run(const jmd_nve_system& s, int64_t steps, bool graphed, cudaStream_t st,
                cudaStream_t body_st, float* traj = nullptr, bool force_rebuild = false) {
  const bool always = s.threshold_sq < 0.f;
  auto gate = [&](const float* x) -> int {
    if (always) return rebuild(s, x, false, st);
    if (graphed)
      return conditional(s.rebuild_flag, [&](cudaStream_t b) { return rebuild(s, x, true, b); }, st,
                         body_st);
    return rebuild(s, x, true, st);
  };
  auto slot = [&](int64_t k) { return traj + (size_t)k * 4 * (size_t)s.n; };
  const size_t rows = sizeof(float4) * (size_t)s.n;
  int rc;
  if (traj) {
    JMD_CUDA(cudaMemcpyAsync(slot(0), s.position, rows, cudaMemcpyDeviceToDevice, st));
    JMD_CUDA(cudaMemcpyAsync(slot(1), s.position, rows, cudaMemcpyDeviceToDevice, st));
  }
  // update at x0
  if (force_rebuild && !always) {
    k_set_flag<<<1, 1, 0, st>>>(s.rebuild_flag);
    JMD_CUDA(cudaGetLastError());
  } else if (!always) {
    rc = jmd_skin_check(s.position, 4, s.reference_position, 4, s.n, &s.space, s.threshold_sq,
                        s.rebuild_flag, st);
    if (rc) return rc;
  }
  if ((rc = gate(s.position))) return rc;
  // first half of step 0: kick + drift + skin test of x1
  float* cur = traj ? slot(1) : s.position;
  float* nxt = traj ? (steps >= 2 ? slot(2) : nullptr) : s.position_alt;
  rc = jmd_verlet_kick_drift(cur, 4, s.momentum, 4, s.force, 4, s.mass, s.mass_scalar,
                             s.n, &s.space, s.dt, nullptr,
                             always ? nullptr : s.reference_position, 4,
                             s.threshold_sq, always ? nullptr : s.rebuild_flag, st);
  if (rc) return rc;
  const int64_t width = s.nlist.max_occupancy;
  for (int64_t k = 1; k < steps; ++k) {
    if ((rc = gate(cur))) return rc;
    rc = jmd_nve_fused_step(&s.pair, &s.space, cur, nxt, s.momentum, s.mass, s.mass_scalar,
                            s.species, s.n, s.idx, s.idx_ld, width, s.nbr_count, s.dt,
                            always ? nullptr : s.reference_position, s.threshold_sq,
                            always ? nullptr : s.rebuild_flag, st);
    if (rc) return rc;
    if (traj) {
      cur = slot(k + 1);
      nxt = k + 2 <= steps ? slot(k + 2) : nullptr;
    } else {
      std::swap(cur, nxt);
    }
  }
  if ((rc = gate(cur))) return rc;
  rc = jmd_force_kick(&s.pair, &s.space, cur, s.force, s.momentum, s.species, s.n, s.idx,
                      s.idx_ld, width, s.nbr_count, s.dt, st);
  if (rc) return rc;
  if (cur != s.position) {
    JMD_CUDA(cudaMemcpyAsync(s.position, cur, sizeof(float4) * (size_t)s.n,
                             cudaMemcpyDeviceToDevice, st));
  }
  return JMD_OK;
}

// One NVT step on float4 rows x (in place), momentum p, force f:
// chain half step (update_mass) -> kick + drift scaled by the chain ->
// gate(x) -> force + kick -> kinetic energy -> chain half step -> scale.
template <typename Gate, typename ForceKick>
int nvt_step(const jmd_nve_system& s, const jmd_nvt& v, float* x, float* p, float* f,
             const float* mass, float* ref, int32_t* flag, bool always, Gate gate,
             ForceKick force_kick, cudaStream_t st) {
  int rc = jmd_nhc_half_step(&v.chain, v.chain_state, nullptr, 1, v.p_scale, st);
  if (rc) return rc;
  rc = jmd_verlet_kick_drift(x, 4, p, 4, f, 4, mass, s.mass_scalar, s.n, &s.space, s.dt, v.p_scale,
                             always ? nullptr : ref, 4, s.threshold_sq, always ? nullptr : flag, st);
  if (rc) return rc;
  if ((rc = gate(x))) return rc;
  if ((rc = force_kick(x))) return rc;
  rc = jmd_kinetic_energy(p, 4, mass, s.mass_scalar, s.n, s.space.dim, v.chain_state + 64,
                          v.reduce_workspace, v.reduce_workspace_bytes, st);
  if (rc) return rc;
  rc = jmd_nhc_half_step(&v.chain, v.chain_state, nullptr, 0, v.p_scale, st);
  if (rc) return rc;
  return jmd_scale_momentum(p, 4, s.n, s.space.dim, v.p_scale, st);
}

int enqueue_nvt(const jmd_nve_system& s, const jmd_nvt& v, int64_t steps, bool graphed,
                cudaStream_t st, cudaStream_t body_st) {
  const bool always = s.threshold_sq < 0.f;
  auto gate = [&](const float* x) -> int {
    if (always) return rebuild(s, x, false, st);
    if (graphed)
      return conditional(s.rebuild_flag, [&](cudaStream_t b) { return rebuild(s, x, true, b); }, st,
                         body_st);
    return rebuild(s, x, true, st);
  };
  int rc;
  if (!always) {
    rc = jmd_skin_check(s.position, 4, s.reference_position, 4, s.n, &s.space, s.threshold_sq,
                        s.rebuild_flag, st);
    if (rc) return rc;
  }
  if ((rc = gate(s.position))) return rc;
  const int64_t width = s.nlist.max_occupancy;
  auto force_kick = [&](const float* x) -> int {
    return jmd_force_kick(&s.pair, &s.space, x, s.force, s.momentum, s.species, s.n, s.idx,
                          s.idx_ld, width, s.nbr_count, s.dt, st);
  };
  for (int64_t k = 0; k < steps; ++k) {
    rc = nvt_step(s, v, s.position, s.momentum, s.force, s.mass, s.reference_position,
                  s.rebuild_flag, always, gate, force_kick, st);
    if (rc) return rc;
  }
  return JMD_OK;
}

// Reverse pass of velocity Verlet over positions recorded by enqueue_run's
// trajectory slots 0..steps (see jmd_nve_adjoint_segment).  The list is
// rebuilt at the first position visited and then maintained by the skin test
// as the pass walks back in time.
int enqueue_adjoint(const jmd_nve_system& s, const float* traj, int64_t steps, bool closing,
                    bool opening, float* xbar, float* pbar, float* rec, double* gp, bool graphed,
                    cudaStream_t st, cudaStream_t body_st) {
  const bool always = s.threshold_sq < 0.f;
  auto gate = [&](const float* x) -> int {
    if (always) return rebuild(s, x, false, st);
    if (graphed)
      return conditional(s.rebuild_flag, [&](cudaStream_t b) { return rebuild(s, x, true, b); }, st,
                         body_st);
    return rebuild(s, x, true, st);
  };
  auto slot = [&](int64_t k) { return traj + (size_t)k * 4 * (size_t)s.n; };
  auto rstep = [&](int64_t k, bool kick, float w) -> int {
    int rc = adjoint_pack(s, slot(k), xbar, pbar, rec, kick, !always, st);
    if (rc) return rc;
    if ((rc = gate(slot(k)))) return rc;
    return adjoint_vjp_step(s, xbar, rec, w, gp, st);
  };
  if (!always) {
    k_set_flag<<<1, 1, 0, st>>>(s.rebuild_flag);
    JMD_CUDA(cudaGetLastError());
  }
  const float h = 0.5f * s.dt;
  int rc;
  if (closing && (rc = rstep(steps, false, h))) return rc;
  for (int64_t k = steps - 1; k >= 0; --k)
    if ((rc = rstep(k, true, (opening && k == 0) ? h : s.dt))) return rc;
  return JMD_OK;
}

// ---------------------------------------------------------- sorted run ----
// Copies the caller's state into the private buffers.  With species_in_w the
// species id rides in the fourth float of the private position rows (the
// segment kernels read it from the staged positions).
__global__ void k_load_user(int n, const float4* x, const float4* p, const float4* f,
                            const int32_t* species, float4* xs, float4* ps, float4* fs,
                            int32_t* ss, int32_t* perm, uint8_t* err, int32_t* seg_status,
                            bool species_in_w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    *err = 0;
    if (seg_status) *seg_status = 0;
  }
  if (i >= n) return;
  float4 r = x[i];
  r.w = (species_in_w && species) ? __int_as_float(species[i]) : 0.f;
  xs[i] = r;
  ps[i] = p[i];
  fs[i] = f[i];
  if (species) ss[i] = species[i];
  perm[i] = i;
}

// Warm start: the caller's state into the private cell order of the previous
// run (slot s takes atom perm[s]); a rebuild is forced when the previous run
// left an error bit or a staging status.
__global__ void k_load_user_warm(int n, const float4* x, const float4* p, const float4* f,
                                 const int32_t* species, float4* xs, float4* ps, float4* fs,
                                 int32_t* ss, const int32_t* perm, uint8_t* err,
                                 int32_t* seg_status, bool species_in_w, int32_t* rebuild_flag) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) {
    if (*err || (seg_status && *seg_status)) *rebuild_flag = 1;
    *err = 0;
    if (seg_status) *seg_status = 0;
  }
  if (s >= n) return;
  const int i = perm[s];
  float4 r = x[i];
  r.w = (species_in_w && species) ? __int_as_float(species[i]) : 0.f;
  xs[s] = r;
  ps[s] = p[i];
  fs[s] = f[i];
  if (species) ss[s] = species[i];
}

__global__ void k_store_user(int n, const int32_t* perm, const float4* xs, const float4* ps,
                             const float4* fs, const float4* rs, float4* x, float4* p, float4* f,
                             float4* ref) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int i = perm[s];
  float4 r = xs[s];
  r.w = x[i].w;
  x[i] = r;
  p[i] = ps[s];
  f[i] = fs[s];
  ref[i] = rs[s];
}

__global__ void k_or_error(uint8_t* dst, const uint8_t* src) { *dst = (uint8_t)(*dst | *src); }

// Segment grid of a run, from the cell grid and the caller's K; false when
// the segment layout does not apply (the host planned it with jmd_segment_plan).
bool run_seg_grid(const jmd_nve_system& s, const jmd_sorted_state& z, SegGrid* g) {
  if (!z.seg_list) return false;
  if (!make_seg_grid(s.nlist, z.seg_cells, 1, g)) return false;
  const int rows = s.space.dim == 3 ? 9 : 3;
  g->cap = rows * (g->K + 2) * s.nlist.cell_capacity;
  g->threads = z.seg_threads;
  g->half = z.seg_half ? 1 : 0;
  // half lists read their blocks from global memory (shared memory holds
  // the reaction accumulators instead)
  g->lcap = g->half ? 0 : std::max(0, z.seg_list_smem) / 16 * 16;
  if (g->half) g->cap = seg_rows(s.space.dim, 1) * (g->K + 2) * s.nlist.cell_capacity;
  return true;
}

// Shared memory of a segment step CTA: staged positions + far slot + the
// list block capacity; checked against what a CTA may opt into.
int seg_check_smem(const SegGrid& g) {
  int dev = 0, optin = 227 * 1024;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    optin = 227 * 1024;
  }
  const int64_t per_slot = 16 + (g.half ? 12 : 0);  // + reaction accumulators
  const int64_t need = (int64_t)(g.cap + 1) * per_slot + g.lcap + (int64_t)sizeof(SegShared) +
                       64 * (int64_t)sizeof(PairCoef) + 64 +
                       (g.half ? 4 * (int64_t)(g.pmax + 1) + 4 * (kSegMaxThreads / 32 + 1) : 0);
  JMD_REQUIRE(need <= optin, "segment staging (positions + list block) exceeds a CTA's shared memory");
  return JMD_OK;
}

int validate_sorted(const jmd_nve_system& s, const jmd_sorted_state& z) {
  JMD_REQUIRE(s.mass == nullptr, "the sorted run needs a scalar mass");
  JMD_REQUIRE(s.nlist.use_cell_list, "the sorted run needs a cell grid");
  JMD_REQUIRE(z.position_a && z.position_b && z.momentum && z.force && z.reference_position &&
                  z.scratch4a && z.scratch4b && z.perm && z.scratch_i_a && z.scratch_i_b &&
                  (z.idx || z.seg_list) && z.nbr_count && z.error_code && z.occupancy &&
                  z.rebuild_flag,
              "null buffer in jmd_sorted_state");
  JMD_REQUIRE(!s.species || z.species, "sorted species buffer required");
  if (z.seg_list) {
    SegGrid g;
    JMD_REQUIRE(run_seg_grid(s, z, &g), "the segment layout does not apply to this cell grid");
    JMD_REQUIRE(g.cap < kSegMaxStaged, "segment staging capacity beyond 16-bit slots");
    JMD_REQUIRE(s.nlist.max_occupancy < 65536, "the segment list stores counts in 16 bits");
    JMD_REQUIRE(z.seg_list_bytes >= seg_list_bytes(g), "seg_list smaller than the plan's list_bytes");
    int e = seg_check_smem(g);
    if (e) return e;
    JMD_REQUIRE(z.seg_status != nullptr, "seg_status is required with seg_list");
    JMD_REQUIRE(z.seg_threads >= 32 && z.seg_threads <= kSegMaxThreads && z.seg_threads % 32 == 0,
                "seg_threads must be a multiple of 32 in [32, 256]");
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(z.seg_list) % 16) == 0, "seg_list must be 16-byte aligned");
  } else {
    JMD_REQUIRE(z.idx_ld >= s.nlist.max_occupancy, "tile depth (idx_ld) < max_occupancy");
  }
  for (const void* p : {(const void*)z.position_a, (const void*)z.position_b,
                        (const void*)z.momentum, (const void*)z.force,
                        (const void*)z.reference_position, (const void*)z.scratch4a,
                        (const void*)z.scratch4b})
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(p) % 16) == 0, "float4 rows must be 16-byte aligned");
  return JMD_OK;
}

int enqueue_run_sorted(const jmd_nve_system& s, const jmd_sorted_state& z, int64_t steps,
                       bool graphed, cudaStream_t st, cudaStream_t body_st,
                       const jmd_nvt* nvt = nullptr) {
  const bool always = s.threshold_sq < 0.f;
  const int n = (int)s.n;
  const unsigned gr = (unsigned)ceil_div(n, 256);
  SegGrid sg{};
  const bool seg = run_seg_grid(s, z, &sg);
  const int32_t* starts = seg ? sort_cell_starts(&s.nlist, s.n, z.workspace, z.workspace_bytes) : nullptr;
  if (seg && !starts) return fail(JMD_ERR_WORKSPACE, "sorted-run workspace too small");
  // sort + build on the private copy; gated by the flag unless `force_now`
  auto rebuild_at = [&](float* x, bool gated, bool with_force, cudaStream_t q) -> int {
    int32_t* flag = gated ? z.rebuild_flag : nullptr;
    int rc = jmd_sort_by_cell(&s.nlist, x, z.momentum, with_force ? z.force : nullptr, z.species,
                              z.perm, s.n, z.scratch4a, z.scratch4b, z.scratch_i_a, z.scratch_i_b,
                              flag, z.workspace, z.workspace_bytes, q);
    if (rc) return rc;
    if (seg)
      return build_segment_after_sort(&s.nlist, sg, x, s.n, z.seg_list, z.nbr_count, z.occupancy,
                                      z.error_code, z.reference_position, z.seg_status, flag,
                                      z.workspace, z.workspace_bytes, q);
    return build_tiled_after_sort(&s.nlist, x, s.n, z.idx, z.idx_ld, z.nbr_count, z.occupancy,
                                  z.error_code, z.reference_position, flag, z.workspace,
                                  z.workspace_bytes, q);
  };
  const bool sp = s.species != nullptr;
  const size_t frows = sizeof(float4) * (size_t)s.n;
  auto force_kick_at = [&](const float* x, cudaStream_t q) -> int {
    if (seg && sg.half) {
      // the half-list forces accumulate into a cleared force buffer
      JMD_CUDA(cudaMemsetAsync(z.force, 0, frows, q));
      return seg_step(3, s.pair, s.space, sg, x, starts, z.seg_list, z.force, z.momentum, nullptr,
                      s.mass_scalar, s.dt, nullptr, 0.f, nullptr, z.seg_status, sp, q, s.n);
    }
    if (seg)
      return seg_step(3, s.pair, s.space, sg, x, starts, z.seg_list, z.force, z.momentum, nullptr,
                      s.mass_scalar, s.dt, nullptr, 0.f, nullptr, z.seg_status, sp, q);
    return jmd_force_kick_tiled(&s.pair, &s.space, x, z.force, z.momentum, z.species, s.n, z.idx,
                                z.idx_ld, s.nlist.max_occupancy, z.nbr_count, s.dt, q);
  };
  auto gate = [&](float* x) -> int {
    if (always) return rebuild_at(x, false, false, st);
    if (graphed)
      return conditional(z.rebuild_flag, [&](cudaStream_t b) { return rebuild_at(x, true, false, b); },
                         st, body_st);
    return rebuild_at(x, true, false, st);
  };
  int rc;
  const bool warm = (z.flags & JMD_RUN_WARM_START) != 0 && !always;
  if (warm) {
    k_load_user_warm<<<gr, 256, 0, st>>>(n, reinterpret_cast<const float4*>(s.position),
                                         reinterpret_cast<const float4*>(s.momentum),
                                         reinterpret_cast<const float4*>(s.force), s.species,
                                         reinterpret_cast<float4*>(z.position_a),
                                         reinterpret_cast<float4*>(z.momentum),
                                         reinterpret_cast<float4*>(z.force), z.species, z.perm,
                                         z.error_code, seg ? z.seg_status : nullptr, seg,
                                         z.rebuild_flag);
    JMD_CUDA(cudaGetLastError());
    if ((rc = jmd_skin_check(z.position_a, 4, z.reference_position, 4, s.n, &s.space,
                             s.threshold_sq, z.rebuild_flag, st)))
      return rc;
    // the first rebuild (with the forces, which the sort permutes) only when
    // the flag asks for it
    if (graphed)
      rc = conditional(z.rebuild_flag,
                       [&](cudaStream_t b) { return rebuild_at(z.position_a, true, true, b); },
                       st, body_st);
    else
      rc = rebuild_at(z.position_a, true, true, st);
    if (rc) return rc;
  } else {
    k_load_user<<<gr, 256, 0, st>>>(n, reinterpret_cast<const float4*>(s.position),
                                    reinterpret_cast<const float4*>(s.momentum),
                                    reinterpret_cast<const float4*>(s.force), s.species,
                                    reinterpret_cast<float4*>(z.position_a),
                                    reinterpret_cast<float4*>(z.momentum),
                                    reinterpret_cast<float4*>(z.force), z.species, z.perm,
                                    z.error_code, seg ? z.seg_status : nullptr, seg);
    JMD_CUDA(cudaGetLastError());
    if ((rc = rebuild_at(z.position_a, false, true, st))) return rc;
  }
  float* cur = z.position_a;
  float* nxt = z.position_b;
  const int64_t width = s.nlist.max_occupancy;
  if (nvt) {
    auto force_kick = [&](const float* x) -> int { return force_kick_at(x, st); };
    for (int64_t k = 0; k < steps; ++k) {
      rc = nvt_step(s, *nvt, cur, z.momentum, z.force, nullptr, z.reference_position,
                    z.rebuild_flag, always, gate, force_kick, st);
      if (rc) return rc;
    }
  } else {
    rc = jmd_verlet_kick_drift(z.position_a, 4, z.momentum, 4, z.force, 4, nullptr, s.mass_scalar,
                               s.n, &s.space, s.dt, nullptr,
                               always ? nullptr : z.reference_position, 4, s.threshold_sq,
                               always ? nullptr : z.rebuild_flag, st);
    if (rc) return rc;
    // half lists: the force buffer is an accumulator, zero between steps
    // (the integration clears it after use)
    if (seg && sg.half && steps > 1) JMD_CUDA(cudaMemsetAsync(z.force, 0, frows, st));
    for (int64_t k = 1; k < steps; ++k) {
      if ((rc = gate(cur))) return rc;
      if (seg && sg.half)
        rc = seg_step(2, s.pair, s.space, sg, cur, starts, z.seg_list, z.force, z.momentum, nxt,
                      s.mass_scalar, s.dt, always ? nullptr : z.reference_position,
                      s.threshold_sq, always ? nullptr : z.rebuild_flag, z.seg_status, sp, st, s.n);
      else if (seg)
        rc = seg_step(2, s.pair, s.space, sg, cur, starts, z.seg_list, nullptr, z.momentum, nxt,
                      s.mass_scalar, s.dt, always ? nullptr : z.reference_position,
                      s.threshold_sq, always ? nullptr : z.rebuild_flag, z.seg_status, sp, st);
      else
        rc = jmd_nve_fused_step_tiled(&s.pair, &s.space, cur, nxt, z.momentum, s.mass_scalar,
                                      z.species, s.n, z.idx, z.idx_ld, width, z.nbr_count, s.dt,
                                      always ? nullptr : z.reference_position, s.threshold_sq,
                                      always ? nullptr : z.rebuild_flag, st);
      if (rc) return rc;
      std::swap(cur, nxt);
    }
    if ((rc = gate(cur))) return rc;
    if ((rc = force_kick_at(cur, st))) return rc;
  }
  k_store_user<<<gr, 256, 0, st>>>(n, z.perm, reinterpret_cast<const float4*>(cur),
                                   reinterpret_cast<const float4*>(z.momentum),
                                   reinterpret_cast<const float4*>(z.force),
                                   reinterpret_cast<const float4*>(z.reference_position),
                                   reinterpret_cast<float4*>(s.position),
                                   reinterpret_cast<float4*>(s.momentum),
                                   reinterpret_cast<float4*>(s.force),
                                   reinterpret_cast<float4*>(s.reference_position));
  JMD_CUDA(cudaGetLastError());
  // the caller's list, in the reference's order, at the last rebuild's
  // positions (unless the caller builds it when it is read)
  if (!(z.flags & JMD_RUN_SKIP_EXIT_LIST)) {
    rc = jmd_neighbor_list_build(&s.nlist, s.reference_position, 4, s.n, s.idx, s.idx_ld,
                                 s.nbr_count, s.occupancy, s.error_code, s.reference_position, 4,
                                 nullptr, s.nl_workspace, s.nl_workspace_bytes, st);
    if (rc) return rc;
  }
  k_or_error<<<1, 1, 0, st>>>(s.error_code, z.error_code);
  JMD_CUDA(cudaGetLastError());
  return JMD_OK;
}

std::string plan_key(const jmd_nve_system& s, int64_t steps, int device) {
  std::string k(reinterpret_cast<const char*>(&s), sizeof(s));
  k.append(reinterpret_cast<const char*>(&steps), sizeof(steps));
  k.append(reinterpret_cast<const char*>(&device), sizeof(device));
  const int tpa = dense_tpa();  // the launch shape is baked into the graph
  k.append(reinterpret_cast<const char*>(&tpa), sizeof(tpa));
  return k;
}

}  // namespace
}  // namespace jmd

using namespace jmd;

extern "C" {

}  // extern "C"

namespace jmd {
namespace {

// Records `enq(capture_stream, body_stream)` once per key as a CUDA graph and
// launches it on st.
template <typename Enq>
int launch_graphed(const std::string& key, Enq enq, cudaStream_t st) {
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_cache.find(key);
  if (it == g_cache.end()) {
    cudaStream_t cs, bs;
    JMD_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    JMD_CUDA(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
    GraphPlan plan;
    cudaError_t ce = cudaGraphCreate(&plan.graph, 0);
    int rc = JMD_OK;
    if (ce == cudaSuccess)
      ce = cudaStreamBeginCaptureToGraph(cs, plan.graph, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      rc = enq(cs, bs);
      cudaGraph_t out;
      cudaError_t ee = cudaStreamEndCapture(cs, &out);
      if (!rc && ee != cudaSuccess) ce = ee;
    }
    if (!rc && ce == cudaSuccess) ce = cudaGraphInstantiate(&plan.exec, plan.graph, 0);
    cudaStreamDestroy(cs);
    cudaStreamDestroy(bs);
    if (rc || ce != cudaSuccess) {
      if (plan.exec) cudaGraphExecDestroy(plan.exec);
      if (plan.graph) cudaGraphDestroy(plan.graph);
      cudaGetLastError();
      if (rc) return rc;
      return fail(JMD_ERR_CUDA, std::string("engine graph build: ") + cudaGetErrorString(ce));
    }
    it = g_cache.emplace(key, plan).first;
  }
  JMD_CUDA(cudaGraphLaunch(it->second.exec, st));
  return JMD_OK;
}

}  // namespace

// Shared with the batched runner (declared in pair.cuh).
int graph_conditional(const int32_t* flag, const std::function<int(cudaStream_t)>& body,
                      cudaStream_t st, cudaStream_t body_st) {
  return conditional(flag, body, st, body_st);
}

int graph_launch_cached(const std::string& key,
                        const std::function<int(cudaStream_t, cudaStream_t)>& enq,
                        cudaStream_t st) {
  return launch_graphed(key, enq, st);
}

}  // namespace jmd

extern "C" {

int jmd_nve_run_sorted(const jmd_nve_system* sys, const jmd_sorted_state* sorted, int64_t n_steps,
                       int32_t use_graph, void* stream) {
  JMD_REQUIRE(sys != nullptr && sorted != nullptr, "null argument");
  int e = validate_sys(*sys);
  if (e) return e;
  e = validate_sorted(*sys, *sorted);
  if (e) return e;
  JMD_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (n_steps == 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus cap;
  JMD_CUDA(cudaStreamIsCapturing(st, &cap));
  if (!use_graph || cap != cudaStreamCaptureStatusNone) {
    int rc = enqueue_run_sorted(*sys, *sorted, n_steps, false, st, nullptr);
    return rc ? rc : check_launch("jmd_nve_run_sorted");
  }
  int device;
  JMD_CUDA(cudaGetDevice(&device));
  std::string key = "sorted" + plan_key(*sys, n_steps, device);
  key.append(reinterpret_cast<const char*>(sorted), sizeof(*sorted));
  return launch_graphed(key, [&](cudaStream_t cs, cudaStream_t bs) {
    return enqueue_run_sorted(*sys, *sorted, n_steps, true, cs, bs);
  }, st);
}

int jmd_nve_run(const jmd_nve_system* sys, int64_t n_steps, int32_t use_graph, void* stream) {
  JMD_REQUIRE(sys != nullptr, "system is null");
  int e = validate_sys(*sys);
  if (e) return e;
  JMD_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (n_steps == 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus cap;
  JMD_CUDA(cudaStreamIsCapturing(st, &cap));
  if (!use_graph || cap != cudaStreamCaptureStatusNone) {
    int rc = enqueue_run(*sys, n_steps, false, st, nullptr);
    return rc ? rc : check_launch("jmd_nve_run");
  }
  int device;
  JMD_CUDA(cudaGetDevice(&device));
  const std::string key = plan_key(*sys, n_steps, device);
  return launch_graphed(key, [&](cudaStream_t cs, cudaStream_t bs) {
    return enqueue_run(*sys, n_steps, true, cs, bs);
  }, st);
}

int jmd_nve_run_recorded(const jmd_nve_system* sys, float* trajectory, int64_t n_steps,
                         int32_t force_rebuild, int32_t use_graph, void* stream) {
  JMD_REQUIRE(sys != nullptr, "system is null");
  int e = validate_sys(*sys);
  if (e) return e;
  JMD_REQUIRE(n_steps >= 1, "n_steps must be >= 1");
  JMD_REQUIRE(trajectory == nullptr || (reinterpret_cast<uintptr_t>(trajectory) % 16) == 0,
              "trajectory must be 16-byte aligned float4 rows");
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus cap;
  JMD_CUDA(cudaStreamIsCapturing(st, &cap));
  if (!use_graph || cap != cudaStreamCaptureStatusNone) {
    int rc = enqueue_run(*sys, n_steps, false, st, nullptr, trajectory, force_rebuild != 0);
    return rc ? rc : check_launch("jmd_nve_run_recorded");
  }
  int device;
  JMD_CUDA(cudaGetDevice(&device));
  std::string key = "rec" + plan_key(*sys, n_steps, device);
  key.append(reinterpret_cast<const char*>(&trajectory), sizeof(trajectory));
  key.push_back(force_rebuild ? 'f' : 'g');
  return launch_graphed(key, [&](cudaStream_t cs, cudaStream_t bs) {
    return enqueue_run(*sys, n_steps, true, cs, bs, trajectory, force_rebuild != 0);
  }, st);
}

int jmd_nve_adjoint_segment(const jmd_nve_system* sys, const float* trajectory, int64_t n_steps,
                            int32_t closing, int32_t opening, float* xbar, float* pbar,
                            float* record_scratch, double* grad_params, int32_t use_graph,
                            void* stream) {
  JMD_REQUIRE(sys != nullptr, "system is null");
  int e = validate_sys(*sys);
  if (e) return e;
  JMD_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  JMD_REQUIRE(trajectory && xbar && pbar && record_scratch, "null buffer");
  for (const void* p : {(const void*)trajectory, (const void*)xbar, (const void*)pbar,
                        (const void*)record_scratch})
    JMD_REQUIRE((reinterpret_cast<uintptr_t>(p) % 16) == 0, "float4 rows must be 16-byte aligned");
  if (n_steps == 0 && !closing) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus cap;
  JMD_CUDA(cudaStreamIsCapturing(st, &cap));
  if (!use_graph || cap != cudaStreamCaptureStatusNone) {
    int rc = enqueue_adjoint(*sys, trajectory, n_steps, closing != 0, opening != 0, xbar, pbar,
                             record_scratch, grad_params, false, st, nullptr);
    return rc ? rc : check_launch("jmd_nve_adjoint_segment");
  }
  int device;
  JMD_CUDA(cudaGetDevice(&device));
  std::string key = "adj" + plan_key(*sys, n_steps, device);
  for (const void* p : {(const void*)trajectory, (const void*)xbar, (const void*)pbar,
                        (const void*)record_scratch, (const void*)grad_params})
    key.append(reinterpret_cast<const char*>(&p), sizeof(p));
  key.push_back(closing ? 'c' : '-');
  key.push_back(opening ? 'o' : '-');
  return launch_graphed(key, [&](cudaStream_t cs, cudaStream_t bs) {
    return enqueue_adjoint(*sys, trajectory, n_steps, closing != 0, opening != 0, xbar, pbar,
                           record_scratch, grad_params, true, cs, bs);
  }, st);
}

int validate_nvt(const jmd_nvt* v) {
  JMD_REQUIRE(v != nullptr, "nvt is null");
  JMD_REQUIRE(v->chain_state && v->p_scale && v->reduce_workspace, "null buffer in jmd_nvt");
  JMD_REQUIRE(v->reduce_workspace_bytes >= jmd_reduce_workspace_bytes(0),
              "reduce workspace too small");
  return JMD_OK;
}

int jmd_nvt_run(const jmd_nve_system* sys, const jmd_nvt* nvt, int64_t n_steps, int32_t use_graph,
                void* stream) {
  JMD_REQUIRE(sys != nullptr, "system is null");
  int e = validate_sys(*sys);
  if (e) return e;
  if ((e = validate_nvt(nvt))) return e;
  JMD_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (n_steps == 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus cap;
  JMD_CUDA(cudaStreamIsCapturing(st, &cap));
  if (!use_graph || cap != cudaStreamCaptureStatusNone) {
    int rc = enqueue_nvt(*sys, *nvt, n_steps, false, st, nullptr);
    return rc ? rc : check_launch("jmd_nvt_run");
  }
  int device;
  JMD_CUDA(cudaGetDevice(&device));
  std::string key = "nvt" + plan_key(*sys, n_steps, device);
  key.append(reinterpret_cast<const char*>(nvt), sizeof(*nvt));
  return launch_graphed(key, [&](cudaStream_t cs, cudaStream_t bs) {
    return enqueue_nvt(*sys, *nvt, n_steps, true, cs, bs);
  }, st);
}

int jmd_nvt_run_sorted(const jmd_nve_system* sys, const jmd_sorted_state* sorted,
                       const jmd_nvt* nvt, int64_t n_steps, int32_t use_graph, void* stream) {
  JMD_REQUIRE(sys != nullptr && sorted != nullptr, "null argument");
  int e = validate_sys(*sys);
  if (e) return e;
  if ((e = validate_sorted(*sys, *sorted))) return e;
  if ((e = validate_nvt(nvt))) return e;
  JMD_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (n_steps == 0) return JMD_OK;
  cudaStream_t st = as_stream(stream);
  cudaStreamCaptureStatus cap;
  JMD_CUDA(cudaStreamIsCapturing(st, &cap));
  if (!use_graph || cap != cudaStreamCaptureStatusNone) {
    int rc = enqueue_run_sorted(*sys, *sorted, n_steps, false, st, nullptr, nvt);
    return rc ? rc : check_launch("jmd_nvt_run_sorted");
  }
  int device;
  JMD_CUDA(cudaGetDevice(&device));
  std::string key = "nvtsorted" + plan_key(*sys, n_steps, device);
  key.append(reinterpret_cast<const char*>(sorted), sizeof(*sorted));
  key.append(reinterpret_cast<const char*>(nvt), sizeof(*nvt));
  return launch_graphed(key, [&](cudaStream_t cs, cudaStream_t bs) {
    return enqueue_run_sorted(*sys, *sorted, n_steps, true, cs, bs, nvt);
  }, st);
}

int jmd_segment_plan(const jmd_nlist* nl, int32_t cells, int32_t* n_segments,
                     int32_t* capacity_atoms, int64_t* smem_bytes, int32_t* cells_used,
                     int64_t* list_bytes) {
  JMD_REQUIRE(nl != nullptr, "nlist descriptor is null");
  SegGrid g;
  if (!make_seg_grid(*nl, cells, 1, &g))
    return fail(JMD_ERR_INVALID_ARGUMENT,
                "the segment layout needs a cell grid with >= 3 cells per side and 1 <= K <= 14");
  const int rows = nl->space.dim == 3 ? 9 : 3;
  const int64_t cap = (int64_t)rows * (g.K + 2) * std::max(1, nl->cell_capacity);
  // the shared memory a CTA may opt into (227 KB on this part); without a
  // device (host-only use) assume that figure
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    optin = 227 * 1024;
  }
  const int64_t smem = (cap + 1) * (int64_t)sizeof(float4);  // + the far slot
  const int64_t static_smem = (int64_t)sizeof(SegShared) + 64 * (int64_t)sizeof(PairCoef) + 64;
  if (cap >= kSegMaxStaged || smem + static_smem > optin || nl->max_occupancy >= 65536)
    return fail(JMD_ERR_INVALID_ARGUMENT, "segment staging exceeds a CTA's shared memory");
  if (n_segments) *n_segments = g.nseg;
  if (capacity_atoms) *capacity_atoms = (int32_t)cap;
  if (smem_bytes) *smem_bytes = smem;
  if (cells_used) *cells_used = g.K;
  if (list_bytes) *list_bytes = seg_list_bytes(g);
  return JMD_OK;
}

int jmd_nve_fused_step_segment(const jmd_pair* pair, const jmd_space* space, const jmd_nlist* nl,
                               int32_t cells, int32_t threads, int32_t list_smem, int32_t half,
                               const float* position, float* position_next, float* momentum,
                               float* force, float mass_scalar, int64_t n, int32_t species_in_w,
                               const uint8_t* seg_list, int64_t seg_list_bytes_, float dt,
                               const float* reference_position, float threshold_sq,
                               int32_t* rebuild_flag, void* workspace, size_t workspace_bytes,
                               int32_t* seg_status, void* stream) {
  JMD_REQUIRE(pair && space && nl, "null descriptor");
  JMD_REQUIRE(space->periodic != JMD_GENERAL_CELL, "the segment kernels take orthorhombic boxes");
  JMD_REQUIRE(n > 0 && n < INT32_MAX, "atom count out of range");
  JMD_REQUIRE(position && position_next && momentum && seg_list && seg_status, "null buffer");
  JMD_REQUIRE(position != position_next, "position and position_next must differ");
  JMD_REQUIRE(reference_position == nullptr || rebuild_flag != nullptr, "skin test needs a flag");
  JMD_REQUIRE(threads >= 32 && threads <= kSegMaxThreads && threads % 32 == 0,
              "threads must be a multiple of 32 in [32, 256]");
  SegGrid g;
  JMD_REQUIRE(make_seg_grid(*nl, cells, 1, &g), "the segment layout does not apply to this cell grid");
  g.half = half ? 1 : 0;
  JMD_REQUIRE(!g.half || force != nullptr, "half lists accumulate forces: force is required");
  g.cap = seg_rows(nl->space.dim, g.half) * (g.K + 2) * nl->cell_capacity;
  g.threads = threads;
  g.lcap = g.half ? 0 : std::max(0, list_smem) / 16 * 16;
  JMD_REQUIRE(g.cap < kSegMaxStaged, "segment staging capacity beyond 16-bit slots");
  JMD_REQUIRE(seg_list_bytes_ >= seg_list_bytes(g), "seg_list smaller than the plan's list_bytes");
  int e = seg_check_smem(g);
  if (e) return e;
  const int32_t* starts = sort_cell_starts(nl, n, workspace, workspace_bytes);
  if (!starts) return fail(JMD_ERR_WORKSPACE, "workspace too small for the cell starts");
  return seg_step(2, *pair, *space, g, position, starts, seg_list, g.half ? force : nullptr,
                  momentum, position_next, mass_scalar, dt, reference_position, threshold_sq,
                  rebuild_flag, seg_status, species_in_w != 0, as_stream(stream), n);
}

int jmd_engine_clear_cache(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  for (auto& kv : g_cache) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
  }
  g_cache.clear();
  return JMD_OK;
}

}  // extern "C"
