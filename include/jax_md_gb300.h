/*
 * jax_md_gb300.h — C ABI of the GB300-native short-range MD path.
 *
 * Every entry point is `extern "C"`, takes plain device pointers, element
 * strides and sizes, and a CUDA stream (`cudaStream_t`, passed here as
 * `void*` so this header needs no CUDA include).  All buffers are owned by the
 * caller.  Functions that need scratch memory take a caller-provided workspace
 * and a `*_workspace_bytes` query; its contents need not be initialised, and
 * calls that share one workspace must not overlap on the GPU.  Nothing here synchronises the stream, so
 * every call is stream-ordered and may be captured into a CUDA graph.
 *
 * Return value: JMD_OK (0) or a JMD_ERR_* code for argument / launch errors;
 * `jmd_last_error()` gives a message (per thread).  Data-dependent conditions
 * (neighbour-list overflow, cell-list overflow, cell size too small, malformed
 * box) are NOT errors: they are OR-ed into a device-side uint8 `error_code`
 * with the bit values of JAX MD's PartitionErrorCode
 * (jax_md/partition.py:494-520), which keeps `did_buffer_overflow` semantics.
 *
 * Positions, momenta and forces are float32 rows of `dim` (2 or 3) components
 * with a row stride given in floats; a stride of 4 (float4 rows) is the fast
 * layout.  Neighbour indices are int32 with sentinel N (jax_md/partition.py:972).
 */
#ifndef JAX_MD_GB300_H_
#define JAX_MD_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JMD_OK 0
#define JMD_ERR_INVALID_ARGUMENT 1
#define JMD_ERR_CUDA 2
#define JMD_ERR_WORKSPACE 3
#define JMD_ERR_UNSUPPORTED 4

/* PartitionErrorCode bits, jax_md/partition.py:494-520. */
#define JMD_NEIGHBOR_LIST_OVERFLOW 1
#define JMD_CELL_LIST_OVERFLOW 2
#define JMD_CELL_SIZE_TOO_SMALL 4
#define JMD_MALFORMED_BOX 8

/* NeighborListFormat, jax_md/partition.py:641-657. */
#define JMD_DENSE 0
#define JMD_SPARSE 1
#define JMD_ORDERED_SPARSE 2

/* Pair potentials. */
#define JMD_LJ 0            /* energy.lennard_jones x multiplicative_isotropic_cutoff (energy.py:246-272,534-580) */
#define JMD_LJ_TRUNCATED 1  /* energy.lennard_jones, hard truncation at r_cutoff */
#define JMD_SOFT_SPHERE 2   /* energy.soft_sphere (energy.py:125-173) */
#define JMD_MORSE 3         /* energy.morse (energy.py:346-371), times the multiplicative cutoff
                               between r_onset and r_cutoff when r_onset < r_cutoff
                               (energy.py:374-440); sigma = position of the minimum */

#define JMD_MAX_SPECIES 8

/* Geometry: space.periodic (jax_md/space.py:275-329), space.free (:258-272)
 * or space.periodic_general with fractional coordinates (:332-468). */
typedef struct {
  int32_t dim;       /* 2 or 3 */
  int32_t periodic;  /* 1: minimum-image displacement and wrapped shift; 0: free;
                        JMD_GENERAL_CELL: positions u in the unit cube, displacement
                        T d_U(u, v) and shift mod(u + T^-1 dR, 1) */
  float box[3];      /* side lengths; box[2] unused for dim 2; 1 for a general cell */
  float cell[9];     /* JMD_GENERAL_CELL: T, row-major 3x3 (upper triangular, the
                        reference's is_box_valid, partition.py:676-681) */
  float inv_cell[9]; /* JMD_GENERAL_CELL: T^-1, row-major */
} jmd_space;

#define JMD_GENERAL_CELL 2

/* Static description of a neighbour list, the C mirror of the static fields
 * of jax_md's NeighborList (partition.py:684-737) plus the cell grid from
 * _cell_dimensions (partition.py:146-188). */
typedef struct {
  jmd_space space;
  float cutoff_sq;            /* (r_cutoff + dr_threshold)^2, partition.py:882-883 */
  int32_t use_cell_list;      /* 0: all-pairs candidates (partition.py:893-898) */
  int32_t cells_per_side[3];  /* floor(L / cutoff) per dimension */
  float cell_size[3];         /* L / cells_per_side, float32 as the reference bins */
  int32_t cell_capacity;      /* cell-list capacity (slot rule, overflow test) */
  int32_t format;             /* JMD_DENSE / JMD_SPARSE / JMD_ORDERED_SPARSE */
  int32_t mask_self;          /* partition.py:953-958 */
  int64_t max_occupancy;      /* Dense: row width; Sparse: pair capacity */
} jmd_nlist;

/* Pair potential parameters.  n_species == 0 means scalar parameters stored
 * at [0][0]; otherwise species matrices [S][S] (smap.py:778-823). */
typedef struct {
  int32_t kind;            /* JMD_LJ / JMD_LJ_TRUNCATED / JMD_SOFT_SPHERE / JMD_MORSE */
  int32_t n_species;
  int32_t per_pair_cutoff; /* 1: r_onset/r_cutoff scale with sigma_ij instead of max sigma */
  int32_t pad_;
  float r_onset;           /* absolute onset radius (LJ, Morse), energy.py:319 */
  float r_cutoff;          /* absolute cutoff radius (LJ, Morse), energy.py:320 */
  float sigma[JMD_MAX_SPECIES][JMD_MAX_SPECIES];
  float epsilon[JMD_MAX_SPECIES][JMD_MAX_SPECIES];
  float alpha[JMD_MAX_SPECIES][JMD_MAX_SPECIES];  /* soft-sphere exponent / Morse range */
  /* Per-particle parameters (smap.py:697-846 with the default combinator
   * 0.5 (p_i + p_j), smap.py:704-713): device float arrays [n] or NULL.
   * When set, sigma[0][0] holds max sigma (the cutoff scale) and n_species
   * must be 0; only jmd_pair_forces (the generic kernels) accepts them. */
  const float* particle_sigma;
  const float* particle_epsilon;
} jmd_pair;

const char* jmd_last_error(void);
int jmd_version(void);

/* ---------------------------------------------------------------- cells -- */

/* Workspace for the binning stage shared by cell-list and neighbour builds. */
size_t jmd_cell_workspace_bytes(int64_t n_atoms, int64_t cell_count);

/* Maximum number of atoms in any cell; the device half of
 * _estimate_cell_capacity (partition.py:191-209, 243-250).  Writes one int32
 * to `max_filling` (device). */
int jmd_cell_max_filling(const float* position, int64_t pos_stride, int64_t n,
                         const jmd_nlist* nl, int32_t* max_filling,
                         void* workspace, size_t workspace_bytes, void* stream);

/* partition.cell_list update (partition.py:349-471): fills the reference
 * layout buffers id_buffer [cell_count*cap] (empty = N) and position_buffer
 * [cell_count*cap*dim] (empty = 0) with the reference slot rule
 * slot = hash*cap + (sorted_rank mod cap), particle_cell_id [N*dim], and ORs
 * JMD_CELL_LIST_OVERFLOW into error_code when a cell holds more than cap. */
int jmd_cell_list_build(const float* position, int64_t pos_stride, int64_t n,
                        const jmd_nlist* nl, int32_t* id_buffer,
                        float* position_buffer, int32_t* particle_cell_id,
                        uint8_t* error_code, void* workspace,
                        size_t workspace_bytes, void* stream);

/* ------------------------------------------------------- neighbour lists -- */

size_t jmd_neighbor_list_workspace_bytes(const jmd_nlist* nl, int64_t n);

/* Builds the neighbour list of partition.neighbor_list's neighbor_fn
 * (partition.py:1034-1121): candidates from the 3^d cells in the reference's
 * order, self mask, strict d^2 < cutoff^2, stable compaction.
 *   Dense:  idx is [n, idx_ld], rows hold max_occupancy entries padded with n.
 *   Sparse: idx is [2, idx_ld]: row 0 receivers (neighbour j), row 1 senders
 *           (atom i), ordered by sender then candidate order; OrderedSparse
 *           keeps j < i only (partition.py:997-998).
 * idx == NULL computes only `occupancy` (count pass of allocate).
 * occupancy (device int64): Dense max row count / Sparse total pair count.
 * nbr_count (device [n], optional): per-atom counts (Dense only).
 * Sets JMD_NEIGHBOR_LIST_OVERFLOW when occupancy > max_occupancy and
 * JMD_CELL_LIST_OVERFLOW when a cell holds more than cell_capacity.
 * reference_position (optional, row stride ref_stride) receives a copy of
 * `position` (NeighborList.reference_position).
 * rebuild_flag (optional device int32): when given, the build runs only if
 * *rebuild_flag != 0 and clears it; this is the lax.cond of
 * partition.py:1146-1154 kept on the device. */
int jmd_neighbor_list_build(const jmd_nlist* nl, const float* position,
                            int64_t pos_stride, int64_t n, int32_t* idx,
                            int64_t idx_ld, int32_t* nbr_count,
                            int64_t* occupancy, uint8_t* error_code,
                            float* reference_position, int64_t ref_stride,
                            int32_t* rebuild_flag, void* workspace,
                            size_t workspace_bytes, void* stream);

/* Skin test of partition.py:1146-1154: ORs 1 into *rebuild_flag when any
 * |d(position_i, reference_i)|^2 > threshold_sq. */
int jmd_skin_check(const float* position, int64_t pos_stride,
                   const float* reference_position, int64_t ref_stride,
                   int64_t n, const jmd_space* space, float threshold_sq,
                   int32_t* rebuild_flag, void* stream);

/* --------------------------------------------------------- pair kernels -- */

size_t jmd_pair_workspace_bytes(int64_t n);

/* smap.pair_neighbor_list energy (smap.py:922-979) and its gradient for the
 * potential in `pp`, over a neighbour list of `format`:
 *   force  [n, force_stride] (optional): -dE/dR;
 *   energy (optional device double): total energy, sum over pairs / 2
 *          (Dense, Sparse) or / 1 (OrderedSparse), f64 reduction;
 *   per_atom_energy [n] (optional, Dense/Sparse): reduce_axis=(1,);
 *   virial [6] (optional device double): dU/d(strain) = sum_pairs
 *          U'(r)/r dR_a dR_b, order xx yy zz xy xz yz (2D: xx yy xy).
 * species (optional [n] int32) selects rows of the species matrices.
 * nbr_count (optional, Dense) bounds each row; otherwise rows end at the
 * first sentinel.  The Dense path assumes a symmetric list (every list this
 * library builds without overflow is). */
int jmd_pair_forces(const jmd_pair* pp, const jmd_space* space, int32_t format,
                    const float* position, int64_t pos_stride,
                    const int32_t* species, int64_t n, const int32_t* idx,
                    int64_t idx_ld, int64_t idx_width,
                    const int32_t* nbr_count, float* force,
                    int64_t force_stride, double* energy,
                    float* per_atom_energy, double* virial, void* workspace,
                    size_t workspace_bytes, void* stream);

/* --------------------------------------------------------------- adjoint -- */

/* Vector-Jacobian product of the Dense-list pair force F(R; sigma, eps) with a
 * cotangent lam [n, cot_stride] (the reverse-mode derivative jax.grad takes
 * through smap.pair_neighbor_list + quantity.force; the LJ cutoff radii follow
 * sigma as in energy.py:319-320).  Accumulates, scaled by `weight`:
 *   grad_position [n, grad_stride] += weight * (dF/dR)^T lam   (optional)
 *   grad_params[130] += weight * d(lam . F)/d theta             (optional)
 * and, unscaled, grad_energy_params[130] += dE/d theta           (optional),
 * with bins [a*8+b] = sigma[a][b], [64+a*8+b] = epsilon[a][b] and [128] = the
 * global cutoff scale max(sigma) (to be credited to the largest sigma entry;
 * per-pair cutoffs credit sigma[a][b] directly).  Scalar parameters use bin 0
 * and 64.  Assumes a symmetric list, as built by jmd_neighbor_list_build. */
int jmd_pair_force_vjp(const jmd_pair* pp, const jmd_space* space,
                       const float* position, int64_t pos_stride,
                       const int32_t* species, int64_t n, const int32_t* idx,
                       int64_t idx_ld, int64_t idx_width,
                       const int32_t* nbr_count, const float* cotangent,
                       int64_t cot_stride, float weight, float* grad_position,
                       int64_t grad_stride, double* grad_params,
                       double* grad_energy_params, void* stream);

/* ---------------------------------------------------------- integrators -- */

/* momentum_step (simulate.py:168-173): p += dt * f. */
int jmd_momentum_step(float* momentum, int64_t p_stride, const float* force,
                      int64_t f_stride, int64_t n, int32_t dim, float dt,
                      void* stream);

/* position_step with shift_fn (simulate.py:176-188, space.py:250-252):
 * x = shift(x, dt * p / m).  mass (optional [n]) else mass_scalar. */
int jmd_position_step(float* position, int64_t x_stride, const float* momentum,
                      int64_t p_stride, const float* mass, float mass_scalar,
                      int64_t n, const jmd_space* space, float dt,
                      void* stream);

/* The first half of velocity_verlet (simulate.py:235-239) fused:
 *   p = p_scale * p + dt/2 * f ; x = shift(x, dt * p / m)
 * p_scale (optional device double, else 1) applies a pending Nose-Hoover
 * rescale.  When reference_position is given it also runs the skin test on
 * the new x and ORs 1 into *rebuild_flag. */
int jmd_verlet_kick_drift(float* position, int64_t x_stride, float* momentum,
                          int64_t p_stride, const float* force,
                          int64_t f_stride, const float* mass,
                          float mass_scalar, int64_t n,
                          const jmd_space* space, float dt,
                          const double* p_scale,
                          const float* reference_position, int64_t ref_stride,
                          float threshold_sq, int32_t* rebuild_flag,
                          void* stream);

/* Kinetic energy 0.5 sum p^2/m in f64 (quantity.py:124-159). */
size_t jmd_reduce_workspace_bytes(int64_t n);
int jmd_kinetic_energy(const float* momentum, int64_t p_stride,
                       const float* mass, float mass_scalar, int64_t n,
                       int32_t dim, double* out, void* workspace,
                       size_t workspace_bytes, void* stream);

/* jmd_kinetic_energy without a workspace: the same kernel and result, with
 * its scratch (block partials and a completion counter) in a fixed device
 * array built into this library, so the call allocates nothing.  It serves
 * callers that have no device buffer to lend and may not allocate one at the
 * point of the call: a host MD code or plugin that measures the temperature
 * inside its time-step loop, where cudaMalloc/cudaFree would synchronise the
 * device and break its stream pipelining, or a foreign runtime that hands out
 * no scratch.  No counterpart in the reference (JAX allocates the reduction's
 * scratch itself).
 *   - n <= 4,194,304 atoms; larger n returns JMD_ERR_INVALID_ARGUMENT.
 *   - The first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress, with that device current) and caches it; make
 *     that first call before any stream capture.
 *   - Every call on a device shares the one array, so calls that overlap on
 *     the GPU (other streams, other host threads) race: issue them in order
 *     on one stream.  The counter is cleared by each call. */
int jmd_kinetic_energy_static_scratch(const float* momentum, int64_t p_stride,
                                      const float* mass, float mass_scalar,
                                      int64_t n, int32_t dim, double* out,
                                      void* stream);

/* Nose-Hoover chain state on the device, f64 (simulate.py:350-374). */
typedef struct {
  int32_t chain_length;  /* M + 1 <= 16 */
  int32_t chain_steps;
  int32_t sy_steps;      /* 1, 3, 5, 7 */
  int32_t dof;
  double dt;
  double tau;
} jmd_nhc;

/* chain [4*16 + 2] doubles: xi[16], p_xi[16], Q[16], spare[16], KE, kT.
 * Runs update_mass (simulate.py:509-515) when update_mass != 0, then
 * half_step (simulate.py:492-507) with the kinetic energy stored in the chain
 * (or *kinetic_energy when given), and writes the total momentum scale to
 * *p_scale (the caller applies it, e.g. through jmd_verlet_kick_drift or
 * jmd_scale_momentum). */
int jmd_nhc_half_step(const jmd_nhc* c, double* chain,
                      const double* kinetic_energy, int32_t update_mass,
                      double* p_scale, void* stream);

/* Reverse of jmd_nhc_half_step (the adjoint of simulate.nvt_nose_hoover's
 * chain, simulate.py:444-507): from the chain state before the half step
 * (chain, 66 doubles, unchanged), the kinetic energy it used and the
 * cotangents of its outputs (cot_p_xi [chain_length] of the chain momenta
 * after it, cot_scale of the momentum scale), writes grad_p_xi
 * [chain_length] and grad_kinetic_energy.  Forward-mode dual numbers in one
 * thread; chain_length <= 7. */
int jmd_nhc_half_step_vjp(const jmd_nhc* c, const double* chain,
                          const double* kinetic_energy, int32_t update_mass,
                          const double* cot_p_xi, const double* cot_scale,
                          double* grad_p_xi, double* grad_kinetic_energy, void* stream);

/* FIRE (minimize.fire_descent, minimize.py:124-226) on float4 rows with the
 * minimiser's scalars kept on the device: fire_state[6] floats
 * {dt, alpha, n_pos, keep, alpha_mix, |P|/|F|}, initialised by the caller to
 * {dt_start, alpha_start, 0, 1, 0, 0}.  One FIRE step is
 *   jmd_fire_kick_drift (p += dt/2 f; x = shift(x, dt p / m)),
 *   the force of the new positions (any pair entry point),
 *   jmd_fire_update (p += dt/2 f; f64 |F|, |P|, F.P; the scalar update of
 *   dt / alpha / n_pos; P mixing and the reset when F.P < 0). */
int jmd_fire_kick_drift(float* position, float* momentum, const float* force,
                        const float* mass, float mass_scalar, int64_t n,
                        const jmd_space* space, const float* fire_state,
                        void* stream);
size_t jmd_fire_workspace_bytes(int64_t n);
int jmd_fire_update(float* momentum, const float* force, int64_t n, int32_t dim,
                    float* fire_state, float dt_max, float n_min, float f_inc,
                    float f_dec, float alpha_start, float f_alpha,
                    void* workspace, size_t workspace_bytes, void* stream);

/* p *= *scale. */
int jmd_scale_momentum(float* momentum, int64_t p_stride, int64_t n,
                       int32_t dim, const double* scale, void* stream);

/* The exp(iL) maps of simulate.npt_nose_hoover's inner step
 * (simulate.py:925-940), on float4 rows:
 *   mode 0 (exp_iL1): R <- shift(R, c0 R + c1 P / m), the shift of `space`
 *          (a general cell: u <- mod(u + T^-1 dR, 1));
 *          c0 = exp(x) - 1, c1 = dt exp(x / 2) sinh(x / 2) / (x / 2), x = v_box dt;
 *   mode 1 (exp_iL2): P <- c0 P + c1 F,
 *          c0 = exp(-x), c1 = (dt / 2) exp(-x / 2) sinh(x / 2) / (x / 2),
 *          x = (1 + 1/N) v_box dt / 2.
 * The coefficients are computed by the caller (the box variables are host
 * scalars). */
int jmd_npt_map(int32_t mode, float* position, float* momentum, const float* force,
                const float* mass, float mass_scalar, int64_t n, const jmd_space* space,
                float c0, float c1, void* stream);

/* The O step of simulate.nvt_langevin's BAOAB step (stochastic_step,
 * simulate.py:1102-1110): p <- c1 p + c2 sqrt(m) xi with c1 = exp(-gamma dt),
 * c2 = sqrt(kT (1 - c1^2)).  xi is standard normal, drawn per atom from
 * Philox4x32-10 (Salmon et al., SC'11) on counter (atom, 0, step) and key
 * seed, then Box-Muller: the same (seed, step) gives the same draws.  The
 * reference draws from jax.random instead, so runs agree in distribution,
 * not draw for draw.  noise_out (float4 rows, may be NULL) receives the four
 * normals of each atom (the first dim are used). */
int jmd_langevin_o_step(float* momentum, int64_t p_stride, int64_t n, int32_t dim,
                        const float* mass, float mass_scalar, float c1, float c2, uint64_t seed,
                        uint64_t step, float* noise_out, void* stream);

/* ------------------------------------------------------- fused kernels -- */

/* Threads per atom of the float4 Dense pair kernels (4, 8 or 16; default 8;
 * JMD_MORSE always runs at 8). */
int jmd_set_dense_threads_per_atom(int tpa);
/* Threads per atom of the generic-stride Dense pair kernel (4, 8, 16, 32). */
int jmd_set_pair_threads_per_atom(int tpa);
/* 1: route Dense pair calls through the generic-stride kernel (testing). */
int jmd_set_pair_generic(int generic);

/* One fused velocity-Verlet step on float4 rows, starting from the
 * half-kicked state p' = p + dt/2 f_old (simulate.py:227-243):
 *   f = F(position); p' += dt/2 f; p' += dt/2 f;
 *   position_next = shift(position, dt p' / m);
 * and the skin test of position_next against reference_position (ORs 1 into
 * *rebuild_flag).  The force is not stored.  Dense lists only. */
int jmd_nve_fused_step(const jmd_pair* pp, const jmd_space* space,
                       const float* position, float* position_next,
                       float* momentum, const float* mass, float mass_scalar,
                       const int32_t* species, int64_t n, const int32_t* idx,
                       int64_t idx_ld, int64_t idx_width,
                       const int32_t* nbr_count, float dt,
                       const float* reference_position, float threshold_sq,
                       int32_t* rebuild_flag, void* stream);

/* Closing half of velocity_verlet on float4 rows: force = F(position),
 * momentum += dt/2 force. */
int jmd_force_kick(const jmd_pair* pp, const jmd_space* space,
                   const float* position, float* force, float* momentum,
                   const int32_t* species, int64_t n, const int32_t* idx,
                   int64_t idx_ld, int64_t idx_width, const int32_t* nbr_count,
                   float dt, void* stream);

/* Tiled Dense layout used inside the engine (atoms in cell order): entry k
 * of atom i lives at tidx[(i / 32) * depth * 32 + k * 32 + i % 32], columns
 * are bounded by nbr_count and not padded.  Same pairs and the same entry
 * order per atom as jmd_neighbor_list_build. */
int jmd_neighbor_list_build_tiled(const jmd_nlist* nl, const float* position,
                                  int64_t n, int32_t* tidx, int64_t depth,
                                  int32_t* nbr_count, int64_t* occupancy,
                                  uint8_t* error_code, float* reference_position,
                                  int32_t* rebuild_flag, void* workspace,
                                  size_t workspace_bytes, void* stream);

/* Forces over a tiled list, one thread per atom (float4 rows). */
int jmd_pair_forces_tiled(const jmd_pair* pp, const jmd_space* space,
                          const float* position, const int32_t* species,
                          int64_t n, const int32_t* tidx, int64_t depth,
                          int64_t width, const int32_t* nbr_count, float* force,
                          void* stream);

/* jmd_nve_fused_step over a tiled list (scalar mass). */
int jmd_nve_fused_step_tiled(const jmd_pair* pp, const jmd_space* space,
                             const float* position, float* position_next,
                             float* momentum, float mass_scalar,
                             const int32_t* species, int64_t n,
                             const int32_t* tidx, int64_t depth, int64_t width,
                             const int32_t* nbr_count, float dt,
                             const float* reference_position, float threshold_sq,
                             int32_t* rebuild_flag, void* stream);

/* jmd_force_kick over a tiled list. */
int jmd_force_kick_tiled(const jmd_pair* pp, const jmd_space* space,
                         const float* position, float* force, float* momentum,
                         const int32_t* species, int64_t n, const int32_t* tidx,
                         int64_t depth, int64_t width, const int32_t* nbr_count,
                         float dt, void* stream);

/* ------------------------------------------------------------- engine ---- */

/* A device-resident NVE system with its Dense neighbour list: the state of
 * the reference's simulation loop body
 *   nbrs = nbrs.update(state.position); state = apply_fn(state, neighbor=nbrs)
 * (partition.py:841-854, simulate.py:279-317).  All buffers are float4 rows
 * (16-byte aligned) owned by the caller; position_alt is scratch of the same
 * size used to ping-pong positions between fused steps. */
typedef struct {
  int64_t n;
  jmd_space space;
  float* position;
  float* position_alt;
  float* momentum;
  float* force;
  const float* mass;          /* [n] or NULL (mass_scalar) */
  float mass_scalar;
  const int32_t* species;     /* [n] or NULL */
  jmd_pair pair;
  jmd_nlist nlist;            /* format must be JMD_DENSE */
  int32_t* idx;
  int64_t idx_ld;
  int32_t* nbr_count;
  float* reference_position;
  uint8_t* error_code;
  int64_t* occupancy;
  int32_t* rebuild_flag;      /* device int32, 0 between calls */
  void* nl_workspace;
  size_t nl_workspace_bytes;
  float dt;
  float threshold_sq;         /* (dr_threshold / 2)^2; < 0: rebuild every step */
} jmd_nve_system;

/* Runs n_steps NVE steps.  use_graph != 0 records the whole run once per
 * (system, n_steps) as a CUDA graph in which each step's rebuild chain sits
 * in a device-side conditional (IF) node set by the skin test, and replays it
 * on `stream`; use_graph == 0 launches the kernels directly with the rebuild
 * kernels gated by the device flag.  Neighbour-list overflow is reported in
 * error_code exactly as jmd_neighbor_list_build does. */
int jmd_nve_run(const jmd_nve_system* sys, int64_t n_steps, int32_t use_graph,
                void* stream);

/* Spatial sort (cell order) of float4 per-atom state, the reordering that
 * keeps neighbour gathers coalesced.  Bins `position` on nl's grid (stable
 * counting sort, the order of partition.py:425-447) and permutes position,
 * momentum, optional force and species, and `perm` (which maps sorted index to
 * the caller's atom id) in place, through the scratch buffers (float4
 * scratch4a/b, int32 scratch_i_a/b, each [n]).  rebuild_flag gates it like
 * jmd_neighbor_list_build (and is not cleared). */
int jmd_sort_by_cell(const jmd_nlist* nl, float* position, float* momentum,
                     float* force, int32_t* species, int32_t* perm, int64_t n,
                     float* scratch4a, float* scratch4b, int32_t* scratch_i_a,
                     int32_t* scratch_i_b, int32_t* rebuild_flag,
                     void* workspace, size_t workspace_bytes, void* stream);

/* Engine-private state of a spatially sorted run: the system's atoms held in
 * cell order (re-sorted at every rebuild) with their own Dense list in sorted
 * ids.  Every buffer is [n] rows (float4 or int32) owned by the caller. */
typedef struct {
  float* position_a;
  float* position_b;
  float* momentum;
  float* force;
  float* reference_position;
  float* scratch4a;
  float* scratch4b;
  int32_t* species;           /* NULL when the system has no species */
  int32_t* perm;              /* sorted index -> caller atom id */
  int32_t* scratch_i_a;
  int32_t* scratch_i_b;
  int32_t* idx;               /* tiled Dense list in sorted ids, ceil(n/32)*32*idx_ld */
  int64_t idx_ld;             /* tile depth >= max_occupancy */
  int32_t* nbr_count;
  uint8_t* error_code;
  int64_t* occupancy;
  int32_t* rebuild_flag;
  void* workspace;
  size_t workspace_bytes;
  /* Segment-local list (see jmd_segment_plan); seg_list == NULL runs the
   * tiled int32 list above instead.  With seg_list set, idx may be NULL. */
  uint8_t* seg_list;          /* segment blocks, 16-byte aligned */
  int64_t seg_list_bytes;     /* >= the list_bytes jmd_segment_plan reports */
  int32_t seg_cells;          /* cells per segment along x (K) */
  int32_t seg_threads;        /* threads per segment CTA: a multiple of 32 in [32, 256] */
  int32_t seg_list_smem;      /* shared-memory bytes for staging a segment's list block
                                 with its positions (0: lists are read from global) */
  int32_t seg_half;           /* 1: half lists (Newton's third law, forward stencil);
                                 forces are accumulated, then integrated */
  int32_t flags;              /* JMD_RUN_* bits */
  int32_t* seg_status;        /* device int32: staging overflow (1) / copy timeout (2) */
} jmd_sorted_state;

/* jmd_sorted_state.flags: leave the caller's Dense list unbuilt on exit (the
 * caller builds it at reference_position when it is read). */
#define JMD_RUN_SKIP_EXIT_LIST 1
/* jmd_sorted_state.flags: the private copy holds the cell order, list and
 * reference positions a previous run of the same system left.  The caller's
 * state is loaded in that order and the run's first rebuild is taken only
 * when it is needed: a rebuild pending from the previous run, an error or
 * staging status left by it, or an atom of the loaded state farther than
 * the skin threshold from its reference position (partition.py:1146-1154). */
#define JMD_RUN_WARM_START 2

/* Segment-local engine list of a cell grid (no reference counterpart: the
 * engine's private layout).  A segment is `cells` consecutive cells along x
 * of one row of the grid; one CTA per segment stages the positions of the
 * segment's neighbourhood (3^(d-1) rows x (cells + 2) cells) in shared memory
 * and the list holds 16-bit slots of that staged block.  Writes the number of
 * segments, the staging capacity in atoms (3^(d-1) (K + 2) cell_capacity) and
 * its shared-memory bytes, and the K actually used (at most cells_x - 2).
 * Returns JMD_OK when the layout applies to nl (a cell grid with >= 3 cells
 * per side, a capacity within 16-bit slots and the shared memory of a CTA),
 * JMD_ERR_INVALID_ARGUMENT otherwise. */
int jmd_segment_plan(const jmd_nlist* nl, int32_t cells, int32_t* n_segments,
                     int32_t* capacity_atoms, int64_t* smem_bytes, int32_t* cells_used,
                     int64_t* list_bytes);

/* One fused NVE step (jmd_nve_fused_step's arithmetic: force, both half
 * kicks, drift, skin test) on the segment-local list of the last sorted
 * rebuild: positions in cell order as float4 rows, `workspace` the sort's
 * workspace (its cell starts place the segments), seg_list as the engine's
 * build wrote it, species ids (when species_in_w) in the fourth float of the
 * position rows; list_smem and half as jmd_sorted_state.seg_list_smem and
 * seg_half.  With half lists the step is two kernels (forces accumulated
 * into `force`, which must be zero on entry, then the integration, which
 * clears it again); otherwise `force` is not used.  The engine's per-step kernel, exposed
 * so it can be timed and tested alone; no reference counterpart (it replaces
 * the force evaluation inside simulate.py:227-243 for the engine's private
 * layout). */
int jmd_nve_fused_step_segment(const jmd_pair* pair, const jmd_space* space, const jmd_nlist* nl,
                               int32_t cells, int32_t threads, int32_t list_smem, int32_t half,
                               const float* position, float* position_next, float* momentum,
                               float* force, float mass_scalar, int64_t n, int32_t species_in_w,
                               const uint8_t* seg_list, int64_t seg_list_bytes, float dt,
                               const float* reference_position, float threshold_sq,
                               int32_t* rebuild_flag, void* workspace, size_t workspace_bytes,
                               int32_t* seg_status, void* stream);

/* jmd_nve_run with the atoms kept in cell order inside the run: on entry the
 * caller's state is copied in and sorted, the steps run on the sorted copy
 * (each rebuild re-sorts it), and on exit positions, momenta, forces and the
 * reference positions go back to the caller's order and the caller's Dense
 * list is rebuilt there (in the reference's entry order).  Requires a scalar
 * mass.  Overflow bits of the private list are OR-ed into the caller's
 * error_code. */
int jmd_nve_run_sorted(const jmd_nve_system* sys, const jmd_sorted_state* sorted,
                       int64_t n_steps, int32_t use_graph, void* stream);

/* Drops every cached graph of the engine. */
int jmd_engine_clear_cache(void);

/* Nose-Hoover chain of an NVT run: the chain constants, its device state
 * (66 doubles, as jmd_nhc_half_step), one double of scratch for the momentum
 * scale and a reduction workspace of jmd_reduce_workspace_bytes(n) bytes. */
typedef struct {
  jmd_nhc chain;
  double* chain_state;
  double* p_scale;
  void* reduce_workspace;
  size_t reduce_workspace_bytes;
} jmd_nvt;

/* n_steps of simulate.nvt_nose_hoover's apply_fn (simulate.py:639-669) on the
 * device, each step: chain half step (with update_mass) -> kick + drift with
 * the chain's momentum scale -> skin-gated rebuild -> force + kick -> kinetic
 * energy -> chain half step -> momentum scale.  As jmd_nve_run /
 * jmd_nve_run_sorted otherwise (the sorted form needs a scalar mass). */
int jmd_nvt_run(const jmd_nve_system* sys, const jmd_nvt* nvt, int64_t n_steps,
                int32_t use_graph, void* stream);
int jmd_nvt_run_sorted(const jmd_nve_system* sys, const jmd_sorted_state* sorted,
                       const jmd_nvt* nvt, int64_t n_steps, int32_t use_graph, void* stream);

/* jmd_pair_force_vjp for Sparse / OrderedSparse lists (idx [2, idx_ld]:
 * row 0 receivers, row 1 senders; padding entries >= n are skipped).  Same
 * outputs and bins; grad_position is accumulated with atomics. */
int jmd_pair_force_vjp_sparse(const jmd_pair* pp, const jmd_space* space, int32_t format,
                              const float* position, int64_t pos_stride,
                              const int32_t* species, int64_t n, const int32_t* idx,
                              int64_t idx_ld, int64_t idx_width, const float* cotangent,
                              int64_t cot_stride, float weight, float* grad_position,
                              int64_t grad_stride, double* grad_params,
                              double* grad_energy_params, void* stream);

/* ------------------------------------------------------ engine adjoint -- */

/* jmd_nve_run with the positions recorded: `trajectory` (optional) holds
 * n_steps + 1 blocks of n float4 rows; block k receives x_k (block 0 a copy
 * of the starting position), and the final position is also left in
 * sys->position.  force_rebuild != 0 rebuilds the list at x_0 whatever the
 * skin test says, so a run restarted from the same (position, momentum,
 * force) repeats bit for bit (every kernel on the path is deterministic).
 * The reverse-mode derivative of the reference's simulation loop
 * (simulate.py:227-243 under jax.grad) keeps its trajectory in the same way;
 * the recording replaces that tape. */
int jmd_nve_run_recorded(const jmd_nve_system* sys, float* trajectory, int64_t n_steps,
                         int32_t force_rebuild, int32_t use_graph, void* stream);

/* Reverse pass of velocity Verlet over a recorded segment x_0..x_{n_steps}
 * (trajectory as written by jmd_nve_run_recorded).  With cotangents
 * xbar = dL/dx, pbar = dL/dp of the segment's end state (float4 rows, updated
 * in place to those of its start state):
 *   closing != 0:  xbar += dt/2 (dF/dR)^T(x_n) pbar    (the closing half kick
 *                  of the run's last step; set on the last segment only)
 *   for k = n_steps-1 .. 0:
 *       q = pbar + (dt/m) xbar;  xbar += w_k (dF/dR)^T(x_k) q;  pbar = q
 *   with w_k = dt, except dt/2 for k = 0 when opening != 0 (the first segment
 *   of the run, whose initial force is F(x_0)).
 * grad_params (optional, [130] doubles) accumulates the matching
 * d/d(sigma, epsilon, cutoff scale) in the bins of jmd_pair_force_vjp.
 * The system's list buffers are used (and left valid for some x_k);
 * record_scratch is 2n float4 rows.  use_graph as for jmd_nve_run. */
int jmd_nve_adjoint_segment(const jmd_nve_system* sys, const float* trajectory,
                            int64_t n_steps, int32_t closing, int32_t opening, float* xbar,
                            float* pbar, float* record_scratch, double* grad_params,
                            int32_t use_graph, void* stream);

/* ---------------------------------------------------------------- batch -- */
/* Many independent periodic systems of uneven size packed end to end: atoms
 * of system b are rows sys_offset[b] .. sys_offset[b+1]-1 of every per-atom
 * array, its cells are global cells cell_offset[b] .. cell_offset[b+1]-1 of
 * its own grid.  Each phase of a step (binning, search, forces, integration)
 * is one launch over all systems.  The reference runs one system per call
 * (jax.vmap needs equal N); a batch gives each system exactly the results of
 * its own single-system call: the neighbour sets of partition.neighbor_list
 * (partition.py:1034-1121) with the system's box and cell grid, the forces of
 * smap.pair_neighbor_list, and the updates of simulate.nve / minimize.fire_descent.
 * Every array named here is a device array. */
typedef struct {
  int32_t dim;                   /* 2 or 3 */
  int32_t n_systems;             /* B */
  int64_t n_atoms;               /* sys_offset[B] */
  int32_t total_cells;           /* cell_offset[B] */
  int32_t max_cells;             /* largest cell count of one system */
  const int32_t* sys_offset;     /* [B+1] */
  const int32_t* atom_sys;       /* [N] system of each atom */
  const float* box;              /* [B*3] periodic box side per system and axis */
  const int32_t* cell_offset;    /* [B+1] */
  const int32_t* cells_per_side; /* [B*3], each >= 1 (1 or 2: every cell is searched once) */
  const float* cell_size;        /* [B*3] box / cells_per_side (float32, as partition.py:99-132) */
} jmd_batch;

/* Dense list of a batch in the engine's tiled layout: the entries of atom i
 * are idx[(i/32)*ld*32 + k*32 + i%32], k < count[i]; entries are global atom
 * ids (system-local id = id - sys_offset[b]).  Rows hold at most
 * max_occupancy entries (ld >= max_occupancy); a longer row sets
 * JMD_NEIGHBOR_LIST_OVERFLOW in error_code, and occupancy[0] receives the
 * largest row length found (int32). */
typedef struct {
  float cutoff_sq;               /* (r_cutoff + dr_threshold)^2, all systems */
  int32_t max_occupancy;
  int32_t ld;
  int32_t mask_self;
  int32_t* idx;                  /* ((N + 31) / 32) * 32 * ld */
  int32_t* count;                /* [N] */
  float* reference_position;     /* [N] float4 rows, positions of the last build */
  int32_t* occupancy;            /* [1] */
  uint8_t* error_code;           /* [1] sticky PartitionErrorCode bits */
  int32_t* rebuild_flag;         /* [1] gate of a conditional build, cleared by it */
  void* workspace;
  size_t workspace_bytes;
} jmd_batch_nlist;

size_t jmd_batch_nlist_workspace_bytes(const jmd_batch* batch);

/* Builds the batch's lists at `position` (float4 rows).  gated != 0: only if
 * *rebuild_flag != 0 (then clears it). */
int jmd_batch_neighbor_list_build(const jmd_batch* batch, const jmd_batch_nlist* nl,
                                  const float* position, int32_t gated, void* stream);

/* Sets *rebuild_flag when any atom moved more than sqrt(threshold_sq) from
 * its reference position (partition.py:1146-1154, per system box). */
int jmd_batch_skin_check(const jmd_batch* batch, const jmd_batch_nlist* nl,
                         const float* position, float threshold_sq, void* stream);

/* Forces of every system (float4 rows) and, optionally, per-system f64
 * potential energies energy[B] (smap.pair_neighbor_list, Dense /2). */
int jmd_batch_pair_forces(const jmd_pair* pair, const jmd_batch* batch,
                          const jmd_batch_nlist* nl, const float* position,
                          const int32_t* species, float* force, double* energy,
                          void* stream);

/* Per-system dot products out[b] = sum over system b's atoms of a_i . c_i
 * (dim components of rows of the given strides), f64 sums of fp32 products.
 * The reductions of the batched Nose-Hoover adjoint (sum_i pbar_i . r_i):
 * the derivative of the loss with respect to each system's momentum scale
 * (simulate.py:639-669 differentiated).  No reference counterpart. */
int jmd_batch_dot_per_system(const jmd_batch* batch, const float* a, int64_t a_stride,
                             const float* c, int64_t c_stride, double* out, void* stream);

/* One fused stage of the batched Nose-Hoover reverse step (the cotangent
 * algebra around the force VJP and the chain VJPs; no reference
 * counterpart, it is what jax.grad evaluates through simulate.py:639-669).
 * Rows of [n, dim] floats unless noted; scale / kebar / sums are [B] f64.
 *   stage 0: rbar = in_a s[sys] + kebar[sys] in_b / m -> out_a;
 *            coef (rbar + pending) -> out_b ([n, 4] rows; pending may be NULL)
 *   stage 1: qbar = in_a + coef pending ([n, 4] rows) -> out_a;
 *            sums[b] = sum qbar . in_b
 *   stage 2: out_a = in_a s[sys] + kebar[sys] in_b / m
 * in_b rows have stride b_stride; inv_m = 1 / mass. */
int jmd_batch_nvt_adjoint_update(const jmd_batch* batch, int32_t stage, const float* in_a,
                                 const float* in_b, int64_t b_stride, const double* scale,
                                 const double* kebar, float inv_m, float coef,
                                 const float* pending, float* out_a, float* out_b,
                                 double* sums, void* stream);

/* Per-system f64 kinetic energy ke[B] (quantity.kinetic_energy) and
 * largest atom force norm fmax[B] (either may be NULL). */
int jmd_batch_kinetic_energy(const jmd_batch* batch, const float* momentum,
                             const float* force, const float* mass, float mass_scalar,
                             double* ke, float* fmax, void* stream);

/* FIRE constants (minimize.fire_descent, minimize.py:124-226) plus the
 * convergence tolerance on the largest atom force norm of a system. */
typedef struct {
  float dt_start, dt_max, n_min, f_inc, f_dec, alpha_start, f_alpha, f_tol;
} jmd_fire_params;

/* State of a batched run.  fire_state holds 8 floats per system:
 * [dt, alpha, n_pos, keep, alpha_mix, |P|/|F|, max |F_i|, -].  done[b]
 * becomes 1 once system b's largest force norm is below f_tol after a FIRE
 * step; a done system is frozen (no further updates); n_done[0] counts
 * them. */
typedef struct {
  jmd_batch batch;
  jmd_batch_nlist nlist;
  jmd_pair pair;
  const int32_t* species;        /* [N] or NULL */
  float* position;               /* [N] float4 rows */
  float* momentum;
  float* force;
  const float* mass;             /* [N] or NULL: mass_scalar */
  float mass_scalar;
  float dt;                      /* NVE time step */
  float threshold_sq;            /* (dr_threshold / 2)^2; < 0: rebuild every step */
  float* fire_state;             /* [B * 8] */
  int32_t* done;                 /* [B] */
  int32_t* n_done;               /* [1] */
} jmd_batch_system;

/* Sets every system's FIRE scalars to (dt_start, alpha_start, 0, ...) and
 * clears done / n_done. */
int jmd_batch_fire_init(const jmd_batch_system* sys, const jmd_fire_params* fp, void* stream);

/* n_steps of batched NVE (velocity Verlet, simulate.py:227-243) or FIRE
 * (minimize.py:171-226) with the skin-gated list rebuild before every force
 * evaluation.  The force array must hold F(position) on entry (from
 * jmd_batch_pair_forces after a build).  use_graph != 0 records the whole run
 * once per (system, n_steps) as one CUDA graph, each rebuild in a device-side
 * conditional node, and replays it. */
int jmd_batch_nve_run(const jmd_batch_system* sys, int64_t n_steps, int32_t use_graph,
                      void* stream);
int jmd_batch_fire_run(const jmd_batch_system* sys, const jmd_fire_params* fp,
                       int64_t n_steps, int32_t use_graph, void* stream);

/* Launch shapes of the batched kernels (the batch autotuner's choice):
 * threads per CTA of the force kernels (64, 128, 256; default 128) and
 * threads per system of the FIRE update (256, 512, 1024; default 1024).
 * Library-wide; cached graphs are keyed by them. */
int jmd_batch_set_launch(int force_block, int fire_threads);

/* Adjoint of a batched NVE run: the batched forms of jmd_nve_run_recorded and
 * jmd_nve_adjoint_segment (same slot layout, same recurrences; each atom
 * uses its system's box; grad_params bins are summed over all systems, the
 * gradient with respect to parameters shared by every system). */
int jmd_batch_nve_run_recorded(const jmd_batch_system* sys, float* trajectory,
                               int64_t n_steps, int32_t force_rebuild, int32_t use_graph,
                               void* stream);
int jmd_batch_nve_adjoint_segment(const jmd_batch_system* sys, const float* trajectory,
                                  int64_t n_steps, int32_t closing, int32_t opening,
                                  float* xbar, float* pbar, float* record_scratch,
                                  double* grad_params, int32_t use_graph, void* stream);

/* grad_params[130] += sum_b system_weight[b] dE_b/d(sigma, epsilon, cutoff
 * scale), E_b the potential energy of system b (bins of jmd_pair_force_vjp). */
int jmd_batch_energy_param_grad(const jmd_pair* pair, const jmd_batch* batch,
                                const jmd_batch_nlist* nl, const float* position,
                                const int32_t* species, const double* system_weight,
                                double* grad_params, void* stream);

/* Nose-Hoover chains of a batch, one per system (simulate.nvt_nose_hoover,
 * simulate.py:565-669, run on every system with its own chain).  The chain
 * constants are shared; chain.dof is not used: system b has
 * (sys_offset[b+1] - sys_offset[b]) * dim degrees of freedom
 * (quantity.count_dof).  chain_state holds 66 doubles per system in the
 * layout of jmd_nhc_half_step (kT per system at [65]); p_scale [2 B]
 * receives the two momentum scales of each system's last step (first half
 * step at [b], second at [B + b]). */
typedef struct {
  jmd_nhc chain;
  double* chain_state;
  double* p_scale;
} jmd_batch_nvt;

/* n_steps of batched Nose-Hoover NVT, each step: chain half step with
 * update_mass on the stored kinetic energy -> kick (after the chain's
 * momentum scale) + drift -> skin-gated rebuild -> force + kick -> kinetic
 * energy -> chain half step -> momentum scale (simulate.py:649-667 per
 * system).  Graphs and forces as jmd_batch_nve_run.  chain_length 2..16. */
int jmd_batch_nvt_run(const jmd_batch_system* sys, const jmd_batch_nvt* nvt, int64_t n_steps,
                      int32_t use_graph, void* stream);

/* One chain half step of every system (update_mass first when update_mass
 * != 0).  measure_ke != 0: the kinetic energy is summed from momentum (f64)
 * and stored in the chain first, else the chain's stored one is used.
 * momentum != NULL: each system's momenta are multiplied by its scale.
 * scale_out[B] / ke_out[B] (either may be NULL) receive each system's scale
 * and the kinetic energy the step used. */
int jmd_batch_nhc_half_step(const jmd_batch* batch, const jmd_batch_nvt* nvt, float* momentum,
                            const float* mass, float mass_scalar, int32_t update_mass,
                            int32_t measure_ke, double* scale_out, double* ke_out, void* stream);

/* Batched jmd_nhc_half_step_vjp, one thread per system: chain [66 B] the
 * states before the half step, kinetic_energy [B] the energies they used,
 * cot_p_xi [16 B] / cot_scale [B] the cotangents of the outputs; writes
 * grad_p_xi [16 B] and grad_kinetic_energy [B].  chain_length 2..7. */
int jmd_batch_nhc_half_step_vjp(const jmd_batch* batch, const jmd_nhc* c, const double* chain,
                                const double* kinetic_energy, int32_t update_mass,
                                const double* cot_p_xi, const double* cot_scale,
                                double* grad_p_xi, double* grad_kinetic_energy, void* stream);

/* Force VJP of a batch (the batched jmd_pair_force_vjp, Dense tiled list
 * built at `position`): grad_position += weight (dF/dR)^T cotangent and,
 * when grad_params is given, grad_params[130] += weight d(cotangent . F)/d
 * (sigma, epsilon, cutoff scale) summed over systems.  position, cotangent
 * and grad_position are float4 rows; record_scratch holds 2 N float4. */
int jmd_batch_pair_force_vjp(const jmd_pair* pair, const jmd_batch* batch,
                             const jmd_batch_nlist* nl, const float* position,
                             const float* cotangent, const int32_t* species, float weight,
                             float* grad_position, double* grad_params, float* record_scratch,
                             void* stream);

#ifdef __cplusplus
}
#endif

#endif  /* JAX_MD_GB300_H_ */
