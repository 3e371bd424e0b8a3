/*
 * apple_gb300 -- C ABI of the GB300-native FEM elasticity / PNCG hot path.
 *
 * Drop-in boundary for the reference's per-energy surface
 *   WarpPotential.{fun,grad,hess_diag,hess_prod,hess_quad}(u[, p], output)
 *     -- liblaf/apple src/liblaf/apple/warp/model/_potential.py:9-32,
 *        implemented per material by warp/fem/_base.py:151-194 --
 * the zero-then-accumulate model sum (warp/model/_model.py:13-36), the DOF
 * map (forward/dof_map/_dof_map.py:30-49), the external force
 * (warp/potential/_ext_force.py:17-90) and the PNCG solve entry
 * (forward/_forward.py:52-56, Optimizer.minimize).
 *
 * Conventions
 *  - Every entry point returns an int status: AGB_OK (0) or a negative
 *    AGB_E_* code; agb_last_error() gives a message for the calling thread.
 *  - Vector arguments are (n_points, 3) row-major arrays in the caller's
 *    vertex order, of the potential's precision (float for AGB_F32 handles,
 *    double for AGB_F64), in DEVICE memory unless a function says "host".
 *    Scalar outputs (energy, p^T H p) are device doubles.
 *  - Outputs are ACCUMULATED into (never zeroed), as in the reference.
 *  - `stream` is a cudaStream_t passed as void*; NULL is the legacy stream.
 *  - No torch or other library types cross this boundary.
 */
#ifndef APPLE_GB300_H
#define APPLE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AGB_OK 0
#define AGB_E_INVALID (-1)    /* bad argument (null pointer, size, enum) */
#define AGB_E_CUDA (-2)       /* a CUDA runtime call failed */
#define AGB_E_MESH (-3)       /* mesh rejected (index out of range, dV <= 0 where checked) */
#define AGB_E_STATE (-4)      /* call not valid in the object's state */
#define AGB_E_DEVICE (-5)     /* a kernel reported a device-side error status */

/* precision of element arithmetic and vector storage */
#define AGB_F32 0
#define AGB_F64 1

/* materials: warp/fem/_arap.py, warp/fem/_stable_neo_hookean.py */
#define AGB_ARAP 0
#define AGB_STABLE_NEO_HOOKEAN 1
/* stable Neo-Hookean with an activation prestrain G = F A, A = I + sym(a) per
 * cell (warp/fem/_stable_neo_hookean_muscle.py:18-114); a = 0 until
 * agb_fem_set_activation */
#define AGB_STABLE_NEO_HOOKEAN_MUSCLE 2

/* flags of agb_fem_eval */
#define AGB_FUN 1u
#define AGB_GRAD 2u
#define AGB_HESS_DIAG 4u
#define AGB_HESS_PROD 8u
#define AGB_HESS_QUAD 16u

typedef struct agb_space agb_space;
typedef struct agb_fem agb_fem;
typedef struct agb_model agb_model;
typedef struct agb_solver agb_solver;
typedef struct agb_batch agb_batch;

const char* agb_last_error(void);
const char* agb_version(void);

/* ---------------------------------------------------------------------------
 * Vertex space: the global point set (ModelBuilder.add_vertices,
 * forward/dof_map/_builder.py:41-50).  `points` (host, n_points x 3) fixes
 * the device vertex order (Morton order of the rest positions); NULL keeps
 * the caller's order.
 * ------------------------------------------------------------------------- */
int agb_space_create(int32_t n_points, const double* points, agb_space** out);
int agb_space_destroy(agb_space* space);
/* internal position of each caller vertex (host out, n_points int32) */
int agb_space_order(const agb_space* space, int32_t* internal_of_user);

/* Region.compute_grad (jax/fem/region/_region.py:84-108) on host arrays:
 * dhdX (n_cells x 4 x 3, row a = grad of shape function a) and
 * dV (n_cells) = det(Dm) / 6 * fraction (fraction may be NULL).  Returns
 * AGB_OK; *n_nonpositive (may be NULL) counts cells with dV <= 0, which the
 * reference only warns about (region/_region.py:98-99). */
int agb_region_compute(int32_t n_cells, const int32_t* cells, int32_t n_points,
                       const double* points, const double* fraction, double* dhdX, double* dV,
                       int32_t* n_nonpositive);

/* ---------------------------------------------------------------------------
 * FEM potential over tetrahedra (WarpPotentialFem.from_region,
 * warp/fem/_base.py:78-111).  All inputs are HOST arrays, copied.
 *   cells     n_cells x 4, global point ids (GlobalPointId-mapped)
 *   points    n_points x 3 rest positions; used when dhdX/dV are NULL to
 *             compute them (jax/fem/region/_region.py:84-108)
 *   dhdX      n_cells x 4 x 3 shape-function gradients, or NULL
 *   dV        n_cells, or NULL (det(Dm)/6)
 *   fraction  n_cells volume fraction scaling dV (utils/_material.py:19-23), or NULL
 *   mu        n_cells Lame mu (cell data "mu")
 *   lambda    n_cells Lame lambda (cell data "lambda"); ignored for ARAP
 * Options: tile_elems (max elements per tile, 0 = default 1024).
 * ------------------------------------------------------------------------- */
int agb_fem_create(agb_space* space, int material, int precision, int32_t n_cells,
                   const int32_t* cells, const double* points, const double* dhdX,
                   const double* dV, const double* fraction, const double* mu,
                   const double* lambda, int32_t tile_elems, agb_fem** out);
int agb_fem_destroy(agb_fem* fem);
/* tile statistics: n_tiles, n_tile_vertices (host out; any may be NULL) */
int agb_fem_info(const agb_fem* fem, int32_t* n_tiles, int32_t* n_tile_vertices);
/* Host only (no device work): the tile and warp-group plan that a potential
 * over these cells builds -- vertices in Morton order of `points`, elements
 * in Morton order of their centroids, tiles of <= tile_elems (0: 1024)
 * elements and <= 256 vertices, warp groups of <= 32 elements in which every
 * corner slot holds 32 distinct vertices (the colouring that lets a warp
 * accumulate without atomics).  Outputs per caller cell (may be NULL): its
 * tile, its group, and its four corners in stored slot order (caller point
 * ids).  For inspection and tests of the plan. */
int agb_plan_tiles(int32_t n_points, int32_t n_cells, const int32_t* cells, const double* points,
                   int32_t tile_elems, int32_t* n_tiles, int32_t* n_groups, int32_t* tile_of_cell,
                   int32_t* group_of_cell, int32_t* slot_cells);

/* Connectivity as stored after the Morton reorder, tiling and warp-group
 * colouring: cells_out[4 c + a] = caller point id of stored corner a of the
 * caller's cell c (the colouring permutes a cell's corners, with the element
 * gradients permuted alike; the corner set is kept, the orientation of the
 * stored order may be odd).  tile_color_hash (may be NULL) receives a
 * hash of the whole tile / group / corner-slot plan, for bit-exactness checks
 * across builds and machines.  Host only; no reference counterpart. */
int agb_fem_cells(const agb_fem* fem, int32_t* cells_out, uint32_t* tile_color_hash);
/* Muscle potentials: set the per-cell activation a (host, n_cells x 6, the
 * caller's cell order; cell data `activation`, common/attr_name.py:40-44,
 * utils/_material.py:15-16).  The element records are rebuilt in place
 * (synchronous copies on the default stream), so a solver whose model has this
 * as its only FEM potential sees the new activation at its next launch; a
 * solver over several potentials copied the records at creation.  Call it
 * while no launch that reads this potential is in flight. */
int agb_fem_set_activation(agb_fem* fem, const double* activation);

/* WarpPotential methods (warp/fem/_base.py:151-194); accumulate into output.
 *   fun:       output[0] += sum_e Psi_e dV_e                       (_base.py:243-263)
 *   grad:      output    += element gradients scattered            (_base.py:265-291)
 *   hess_diag: output    += max(dV diag(H_e), 0) scattered         (_base.py:293-324)
 *   hess_prod: output    += dV H_e p_e scattered                   (_base.py:326-351)
 *   hess_quad: output[0] += sum_e max(dV p_e^T H_e p_e, 0)         (_base.py:353-383)
 * ARAP hess_prod implements the intended H p (the reference's
 * _arap.py:55-56 passes the operands of h4_prod/h5_prod in swapped order). */
int agb_fem_fun(agb_fem* fem, const void* u, double* output, void* stream);
int agb_fem_grad(agb_fem* fem, const void* u, void* output, void* stream);
int agb_fem_hess_diag(agb_fem* fem, const void* u, void* output, void* stream);
int agb_fem_hess_prod(agb_fem* fem, const void* u, const void* p, void* output, void* stream);
int agb_fem_hess_quad(agb_fem* fem, const void* u, const void* p, double* output, void* stream);
/* Allocation-free variant of agb_fem_fun (no counterpart in the reference).
 * For callers that must not allocate device memory themselves, such as an
 * XLA/JAX FFI handler running under XLA's allocator (which reserves most of
 * the device up front) or a loop with a fixed memory budget: u is read in
 * the caller's order and the per-block partial sums and completion counter
 * live in one file-scope device array of 512 KiB + 256 B, which holds meshes
 * of at most 65,536 tiles (larger meshes: AGB_E_INVALID).  Every call looks
 * up the array's device address (cudaGetSymbolAddress) with the caller's
 * device current, so the address stays valid across cudaDeviceReset; the
 * first call on a device may load the module, so make that first call
 * before any stream capture.  Muscle potentials: AGB_E_INVALID.  All calls on a device
 * share the array; calls that overlap on the GPU race on it.  Accumulates
 * into output[0] like agb_fem_fun. */
int agb_fem_fun_noalloc(agb_fem* fem, const void* u, double* output, void* stream);
/* fused: any subset of AGB_* flags in one pass over the mesh; NULL outputs
 * for unset flags.  p is needed for HESS_PROD and HESS_QUAD. */
int agb_fem_eval(agb_fem* fem, unsigned flags, const void* u, const void* p, double* energy,
                 void* grad, void* hess_diag, void* hess_prod, double* hess_quad, void* stream);

/* ---------------------------------------------------------------------------
 * Model = potentials + fixed DOFs + external force over one space
 * (ModelBuilder.finalize, forward/_builder.py:27-40).  Host inputs, copied.
 *   fixed_mask    n_points x 3 (nonzero = fixed component), or NULL
 *   fixed_values  n_points x 3 displacement of fixed components, or NULL
 *   force_index / force  n_force point ids and forces (ExternalForce), or 0/NULL
 * The potentials (n_potentials >= 0) must share `space` and `precision`; they
 * stay owned by the caller and must outlive the model.
 * ------------------------------------------------------------------------- */
int agb_model_create(agb_space* space, int precision, int32_t n_potentials, agb_fem* const* potentials,
                     const uint8_t* fixed_mask, const double* fixed_values, int32_t n_force,
                     const int32_t* force_index, const double* force, agb_model** out);
int agb_model_destroy(agb_model* model);
/* WarpModel.*: zero then accumulate all potentials and the external force
 * (warp/model/_model.py:13-36, potential/_ext_force.py:17-39). */
int agb_model_eval(agb_model* model, unsigned flags, const void* u, const void* p, double* energy,
                   void* grad, void* hess_diag, void* hess_prod, double* hess_quad, void* stream);

/* Free/fixed DOF maps over the flattened n_points x 3 vector
 * (DofMap.to_free / to_free_grad / to_free_hess_diag / to_full /
 * to_full_grad, forward/dof_map/_dof_map.py:30-50), one kernel each, device
 * pointers of the given precision.
 *   agb_dof_to_free: free_out[i] = full[free_index[i]], i < n_free.
 *   agb_dof_to_full: full_out[j] = slot[j] >= 0 ? free_in[slot[j]]
 *                    : (fill ? fill[j] : 0), j < n_full; slot[j] is DOF j's
 *                    free index or -1 for a fixed DOF.  fill = the fixed
 *                    values scattered into a full-length vector gives
 *                    to_full (:39-43); fill = NULL gives to_full_grad (:45-50).
 * The indices are not checked on the device: free_index[i] < n_full and
 * slot[j] < n_free are the caller's to keep (the Python DofMap builds both
 * from one mask). */
int agb_dof_to_free(int32_t precision, int64_t n_free, const int64_t* free_index, const void* full,
                    void* free_out, void* stream);
int agb_dof_to_full(int32_t precision, int64_t n_full, const int32_t* slot, const void* free_in,
                    const void* fill, void* full_out, void* stream);

/* ---------------------------------------------------------------------------
 * PNCG (liblaf-peach PNCG as used by forward/_forward.py:22-30; iteration as
 * benches/bench_pncg_branching_backends.py:254-456,606-679).
 * ------------------------------------------------------------------------- */
typedef struct agb_pncg_params {
  int32_t max_steps;           /* ConvergenceCriteria.max_steps (default 1500) */
  double rtol;                 /* converged: ||g|| <= max(atol, rtol ||g_0||) */
  double atol;
  int32_t max_backtracking;    /* Armijo halvings after the first trial (8) */
  double armijo_c;             /* 1e-4 */
  double overstep;             /* alpha_0 = overstep * (-g.p / p.Hp); 1 */
  double beta_max;             /* |beta| above this resets to steepest descent (10) */
  double refresh_ratio;        /* FP32 stable Neo-Hookean: reference-state correction, refreshing
                                  the FP64 reference gradient whenever ||g|| has dropped by this
                                  factor; 0: off; < 0 (default): 1e-1 when rtol < 1e-5 asks for
                                  more than FP32 element forces resolve, else off */
} agb_pncg_params;

#define AGB_PRIMARY_SUCCESS 0
#define AGB_MAX_STEPS_REACHED 1
#define AGB_LINE_SEARCH_FAILED 2
#define AGB_NAN_ENCOUNTERED 3
#define AGB_RUNNING 4

typedef struct agb_pncg_stats {
  int32_t result;              /* AGB_PRIMARY_SUCCESS ... AGB_RUNNING */
  int32_t n_steps;
  double grad_norm;            /* ||g|| over free DOFs at the returned u */
  double grad_norm_first;
  double energy;               /* total energy at the returned u */
  double alpha;                /* last accepted step length (0 if rejected) */
  double beta;                 /* last beta */
  int32_t line_search_steps;   /* halvings in the last line search */
  int32_t line_search_ok;
  double hess_diag_mean;       /* mean of the positive free Hessian-diagonal entries at the
                                  returned u: the preconditioner's fill for zero entries
                                  (1 when there are none) */
} agb_pncg_stats;

void agb_pncg_default_params(agb_pncg_params* params);

/* A PNCG solver over the model (Forward.step / Optimizer.minimize,
 * forward/_forward.py:52-56).  The model's FEM potentials must be all ARAP, or
 * all stable Neo-Hookean and muscle (mixed ones run as muscle cells, the
 * stable Neo-Hookean ones with zero activation), with at least one cell
 * among them (AGB_E_INVALID otherwise).  A single FEM potential's element
 * records are used in place; several are copied and concatenated. */
int agb_solver_create(agb_model* model, const agb_pncg_params* params, agb_solver** out);
int agb_solver_destroy(agb_solver* solver);
/* load u (device, full vector; fixed components are overwritten by the
 * model's fixed values) and evaluate g_0, hess_diag_0. */
int agb_solver_reset(agb_solver* solver, const void* u, void* stream);
/* run up to n_steps iterations (fewer if the solve terminates); the loop
 * runs on the device as one CUDA graph launch (conditional while node; with
 * the FP32 correction on, the two refresh passes sit in an outer while loop
 * and run only when a refresh is due). */
int agb_solver_iterate(agb_solver* solver, int32_t n_steps, void* stream);
/* exactly one iteration as one graph launch (benchmark building block); with
 * the FP32 correction on, the two refresh passes follow and return at once
 * unless a refresh is due */
int agb_solver_step(agb_solver* solver, void* stream);
/* number of kernels one iteration of agb_solver_step launches (the three
 * passes, plus the two refresh passes when the FP32 correction is on) */
int agb_solver_step_kernels(agb_solver* solver, int32_t* n_kernels);
/* copy u out (device, caller order) and the stats (host); synchronises stream */
int agb_solver_read(agb_solver* solver, void* u_out, agb_pncg_stats* stats, void* stream);
/* the search direction p of the last iteration (the step taken was
 * alpha * p; zero after agb_solver_reset and on fixed components), copied to
 * HOST memory in caller order, n_points x 3 of the solver precision
 * (PNCG state `direction`, exp/2026/05/06/toy/src/
 * 20-ext-force-stable-neo-hookean-collision.py:211-224).  Synchronises the
 * stream; AGB_E_INVALID before the first agb_solver_reset / agb_solver_load. */
int agb_solver_read_direction(agb_solver* solver, void* p_host, void* stream);
/* The stored free gradient g and clamped Hessian diagonal d of the current
 * iterate (zero on fixed components; PNCG state `grad` / `hess_diag`),
 * copied to HOST memory in caller order, n_points x 3 of the solver
 * precision each; either pointer may be NULL.  Synchronises the stream;
 * AGB_E_INVALID before the first agb_solver_reset / agb_solver_load. */
int agb_solver_read_gradient(agb_solver* solver, void* g_host, void* d_host, void* stream);
/* The scalars the last iteration's reductions produced (FP64, from FP32
 * per-thread sums and float-float trees in the FP32 build): out[0] = p^T H p
 * of the last direction at its base point (the clamped per-element sum that
 * sets alpha_0), out[1] = g . p_next = -g^T P g + beta p.g of the next
 * direction, out[2] = ||g|| over the free DOFs, out[3] = the preconditioner's
 * fill 1 / mean(|d| > 0), out[4] = beta.  Synchronises the stream. */
int agb_solver_read_reductions(agb_solver* solver, double* out5, void* stream);

/* Checkpoint / resume of a solve (the reference has none; its experiments
 * restart from saved .vtu states).  A checkpoint is the solver's whole PNCG
 * state -- positions as float-float pairs, gradient, Hessian diagonal, both
 * search directions, the reference state of the FP32 correction and the
 * scalar state -- in a host buffer of agb_solver_checkpoint_size bytes.
 * The header carries a fingerprint of the model and parameters (each
 * potential's tiles, corner ids, element geometry and Lame parameters, the
 * fixed mask and values, the external force, every agb_pncg_params field;
 * muscle activations are not part of it).  agb_solver_load takes the
 * buffer's length and accepts only a checkpoint of exactly that size whose
 * precision, vertex count, correction setting and fingerprint match this
 * solver's (AGB_E_INVALID otherwise, before anything is copied); the next
 * agb_solver_iterate continues the solve exactly where it was saved.  Both
 * synchronise the stream. */
int agb_solver_checkpoint_size(agb_solver* solver, size_t* bytes);
int agb_solver_save(agb_solver* solver, void* host, void* stream);
int agb_solver_load(agb_solver* solver, const void* host, size_t bytes, void* stream);
/* Diagnostics: time each pass of an iteration on its own with CUDA events on
 * `stream`, `reps` launches each (direction, gradient, vertex pass), writing
 * `flush_bytes` of the device buffer `flush` (may be NULL) before every launch
 * to evict L2.  ms[3] receives the mean launch times.  Mutates the solver
 * state (the vertex pass advances x): call agb_solver_reset before solving. */
int agb_solver_time_passes(agb_solver* solver, int32_t reps, void* flush, size_t flush_bytes,
                           float* ms, void* stream);
/* Optimizer.minimize(problem, state, free) with HOST buffers: copies u_host
 * in, solves to termination, copies the result back into u_host. */
int agb_pncg_minimize_host(agb_solver* solver, void* u_host, agb_pncg_stats* stats, void* stream);

/* ---------------------------------------------------------------------------
 * Batched PNCG: independent models (each its own space, potentials of one
 * precision with at least one cell, fixed DOFs, external force) solved
 * together.  The models' FEM potentials are all ARAP, or all stable
 * Neo-Hookean and muscle (AGB_E_INVALID otherwise, as for one solver).
 * Every model runs the PNCG iteration above with its own beta, step and
 * termination; an iteration of all running models is one set of launches
 * (one CUDA graph).  No reference counterpart: the reference steps one
 * Forward (forward/_forward.py:52-56) per model.  Vectors are the models'
 * caller-order displacements concatenated (n_points_total x 3, device);
 * chunk_verts (0: 512) is the vertex-pass block size.
 * ------------------------------------------------------------------------- */
int agb_batch_create(int32_t n_models, agb_model* const* models, const agb_pncg_params* params,
                     int32_t chunk_verts, agb_batch** out);
int agb_batch_destroy(agb_batch* batch);
/* totals: concatenated vertices and tets */
int agb_batch_info(agb_batch* batch, int32_t* n_points, int32_t* n_cells);
int agb_batch_reset(agb_batch* batch, const void* u, void* stream);
/* up to n_steps iterations of every running model (one graph launch) */
int agb_batch_iterate(agb_batch* batch, int32_t n_steps, void* stream);
/* exactly one iteration as a plain graph */
int agb_batch_step(agb_batch* batch, void* stream);
/* u out (device, concatenated caller order; may be NULL) and stats[n_models]
 * (host); synchronises stream */
int agb_batch_read(agb_batch* batch, void* u_out, agb_pncg_stats* stats, void* stream);

/* ---------------------------------------------------------------------------
 * Differentiation of the converged equilibrium g(u*, theta) = 0 (the inverse
 * experiments' adjoint, exp/2025/09/24/inverse-grin/src/32-inverse.py:223-300):
 * dL/dtheta = -lam^T dg/dtheta with H(u*) lam = dL/du on the free DOFs.
 * ------------------------------------------------------------------------- */
typedef struct agb_cg_params {
  int32_t max_iter;            /* 10000 */
  double rtol;                 /* ||r|| <= max(atol, rtol ||r_0||); 1e-6 */
  double atol;                 /* 0 */
} agb_cg_params;

typedef struct agb_cg_stats {
  int32_t result;              /* AGB_PRIMARY_SUCCESS, AGB_MAX_STEPS_REACHED, AGB_NAN_ENCOUNTERED,
                                  AGB_LINE_SEARCH_FAILED (p^T H p <= 0: H not positive definite) */
  int32_t n_iter;
  double residual;             /* ||r|| at the end (free DOFs) */
  double residual_first;       /* ||r_0|| = ||rhs|| on the free DOFs */
} agb_cg_stats;

void agb_cg_default_params(agb_cg_params* params);

/* Solve H(x) lam = rhs on the free DOFs at the solver's current x (after
 * agb_solver_iterate: the converged u*) with Jacobi-preconditioned CG
 * (jax.scipy.sparse.linalg.cg with M = 1/hess_diag in the reference recipe;
 * M from the Hessian diagonal at x, zero entries replaced by the mean of the
 * positive ones as in the PNCG preconditioner).  H is the sum of the model's
 * hess_prod (warp/fem/_base.py:326-351); fixed components of lam are 0.
 * rhs and lam: device, caller order, n_points x 3 of the solver precision.
 * The CG loop runs on the device as one CUDA graph launch; stats on the host.
 * The solver's PNCG state is not modified.  Only for models whose potentials
 * share one material (the solver's element passes). */
int agb_solver_adjoint(agb_solver* solver, const void* rhs, void* lam, const agb_cg_params* params,
                       agb_cg_stats* stats, void* stream);

/* Backward of the gradient on the cell materials (the Warp tape over the
 * arrays marked requires_grad, warp/fem/_base.py:80-117,
 * utils/_material.py:34-38): for a vector field w (device, caller order,
 * n_points x 3) and displacement u,
 *   out_mu[c]     += d(w . grad(u))/d mu_c
 *   out_lambda[c] += d(w . grad(u))/d lambda_c   (stable Neo-Hookean and its muscle; may be NULL)
 * with cells in the caller's order (device arrays of the fem's precision). */
int agb_fem_grad_param_vjp(agb_fem* fem, const void* u, const void* w, void* out_mu, void* out_lambda,
                           void* stream);
/* Muscle potentials: out_activation[6 c + k] += d(w . grad(u))/d a_{c,k}
 * (device, the fem's precision, caller's cell order), the backward of the
 * gradient on the activation array that the reference's inverse experiments
 * optimise (requires_grad=("activation",)). */
int agb_fem_grad_activation_vjp(agb_fem* fem, const void* u, const void* w, void* out_activation,
                                void* stream);

#ifdef __cplusplus
}
#endif
#endif /* APPLE_GB300_H */
