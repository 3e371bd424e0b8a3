// Device-resident PNCG state and the solver handle.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "agb_internal.h"

namespace agb {

// Scalars of the PNCG iteration, kept in device memory and updated only by
// the last block of a pass (thread 0), so that an iteration runs without a
// host round trip.  Layout is plain-old-data for cudaMemcpy.
struct SolverState {
  // current direction coefficients: p = -P g + beta p_prev, P from d and inv_mean
  double beta;
  double inv_mean;
  double gd;        // g . p for the current p (<0 for a descent direction)
  double t;         // accepted step of the current iteration (0 if rejected)
  double alpha0;    // first trial step (ARAP trial passes)
  double hq;        // clamped p^T H p
  double gnorm;     // ||g|| over free DOFs at x
  double gnorm0;
  double energy;    // total energy at x (summed on demand, see solver_energy)
  double ext_energy;  // external-force work term at x
  double delta_e;   // predicted energy change of the accepted step
  // parameters
  double rtol, atol, armijo_c, overstep, beta_max;
  int32_t max_steps;
  int32_t max_bt;
  // iteration bookkeeping
  int32_t iter;
  int32_t iter_limit;
  int32_t done;
  int32_t result;
  int32_t init;        // next vertex pass is the initial one (beta = 0, record ||g_0||)
  int32_t reset_beta;  // the last line search was rejected: restart with steepest descent
  int32_t ls_fail;     // rejected along steepest descent: terminate
  int32_t ls_steps;
  int32_t ls_ok;
  int32_t decided;     // ARAP: a trial pass has decided the step
  int32_t error;       // device-side status (nonzero = a guard tripped)
  int32_t pbuf;        // p[pbuf] holds p_prev; the direction pass writes p into p[pbuf ^ 1]
  // reference-state correction (FP32 stable Neo-Hookean): refresh x_ref and
  // g(x_ref) once ||g|| has dropped by ref_ratio since the last refresh
  int32_t refresh;     // the refresh passes run after this iteration's vertex pass
  double gnorm_ref;    // ||g|| at the last refresh
  double ref_ratio;    // 0: off
  // ARAP: svd[sbuf] holds each element's SVD at x; the gradient passes write
  // svd[sbuf ^ 1] and the vertex pass that moves x flips sbuf.  spec_ok: the
  // speculative gradient pass at alpha_0 passed the Armijo test, so its
  // gradient is the iteration's and the fallback passes return at once.
  int32_t sbuf;
  int32_t spec_ok;
};

// Everything a solver kernel needs, by value.
struct SolveArgs {
  FemView fv;
  int n_points;
  int precision;
  // Vertex state, per internal vertex v (V4<R> = 4 lanes of R):
  //   xa[2v] = (x_hi, fixed-mask bits), xa[2v+1] = (x_lo, 0); x = hi + lo
  //   gd[2v] = (g, 0) free gradient, gd[2v+1] = (d, 0) Hessian diagonal
  //   p0[v], p1[v]: search directions; p[pbuf] = p_prev, p[pbuf ^ 1] = p
  void* xa;
  void* gd;
  void* p0;
  void* p1;
  // reference state (delta != 0): xref[v] = (x_ref, 0) and gref[v] = the
  // gradient at x_ref computed in FP64 (external force folded in), rounded
  // once to R; the gradient pass then evaluates only f_e(x) - f_e(x_ref),
  // which FP32 resolves to its own relative precision
  void* xref;
  void* gref;
  int delta;
  const void* force;  // V4<R> external force per vertex or null
  const int32_t* slot_of_tv;
  const int32_t* off;  // CSR over slots (n_points + 1)
  void* slots;         // V4<R> [n_slots][2]: (gradient, 0), (diagonal, 0)
  int32_t n_slots;
  SolverState* st;
  void* part_a;        // direction-pass partials (n_tiles x 6) and group partials
  void* gpart_a;
  void* part_b;        // energy partials of the on-demand energy pass (n_tiles x 1)
  void* part_v;        // vertex-pass partials (vblocks x 12) and group partials
  void* gpart_v;
  void* part_t;        // ARAP trial partials (n_tiles x 3) and group partials
  void* gpart_t;
  unsigned* cnt_a;     // ceil(n_tiles/32) + 1 completion counters
  unsigned* cnt_v;     // ceil(vblocks/32) + 1
  unsigned* cnt_t;     // ceil(n_tiles/32) + 1
  int vblocks;
  int max_bt;               // Armijo halvings (ARAP trial passes launched)
  unsigned long long cond;  // cudaGraphConditionalHandle or 0
  // Gating of the two reference-state refresh passes in agb_solver_iterate's
  // graph: with refresh_exits the vertex pass also ends the WHILE loop `cond`
  // when a refresh is due, and the refresh vertex pass, which follows that
  // loop inside an outer WHILE loop `cond_outer`, re-arms `cond` and decides
  // whether the outer loop continues.
  unsigned long long cond_outer;
  int refresh_exits;
  // second iteration of an unrolled loop body: its passes return at once
  // (with no effect) when the first one ended the solve, reached the
  // iteration limit or asked for a refresh
  int guard;
  // ARAP: two per-element SVD caches, each V4<R>[3][n_cells] (U and V as
  // quaternions (w x y z), then (sigma - 1, 0)); null for other materials
  void* svd;
};

cudaError_t launch_solver_init(const SolveArgs& a, const void* u_user, const void* fixed,
                               const int32_t* user_of_internal, cudaStream_t s);
cudaError_t launch_solver_set_limit(const SolveArgs& a, int n_steps, cudaStream_t s);
// one PNCG iteration: direction pass, [ARAP trial passes], gradient pass, vertex pass
cudaError_t launch_solver_iteration(const SolveArgs& a, bool use_cond, cudaStream_t s);
// gradient + vertex pass at t = 0 (initial g_0, diag_0)
cudaError_t launch_solver_first(const SolveArgs& a, cudaStream_t s);
cudaError_t launch_solver_unpack_x(const SolveArgs& a, const void* fixed_unused,
                                   const int32_t* user_of_internal, void* u_user, cudaStream_t s);
int solver_vertex_blocks(int n_points);
// set kernel attributes (dynamic shared memory of the gradient pass); call
// once before launching or capturing solver kernels
cudaError_t solver_prepare_kernels(int precision);
// energy at x into st->energy: an element pass (per-tile partials) and their
// sum plus the external work of the last vertex pass
cudaError_t launch_solver_energy(const SolveArgs& a, cudaStream_t s);
size_t solver_grad_smem(int precision);
// one pass of an iteration on its own: 0 direction, 1 gradient, 2 vertex
cudaError_t launch_solver_pass(const SolveArgs& a, int which, cudaStream_t s);
// the refresh of the reference state (element pass in FP64, vertex pass);
// both return at once unless st->refresh is set.  pdl: launch them as
// programmatic dependents of the kernel before them in the stream.
cudaError_t launch_solver_refresh(const SolveArgs& a, cudaStream_t s, bool pdl = true);
// set st->refresh (the next refresh passes run unconditionally)
cudaError_t launch_solver_force_refresh(const SolveArgs& a, cudaStream_t s);

// Adjoint CG (adjoint.cu): scalars of H lam = rhs on the free DOFs at the
// solver's current x, kept on the device like SolverState.
struct CgState {
  double alpha, beta;
  double rz;   // r . M^-1 r
  double rr;   // r . r
  double rr0;  // r . r at the start
  double rtol, atol;
  int32_t max_iter;
  int32_t iter;
  int32_t iter_limit;
  int32_t done;
  int32_t result;
  int32_t pbuf;  // p[pbuf] = p_prev, p[pbuf ^ 1] = p
};

struct CgArgs {
  SolveArgs a;  // mesh, tiles, slots, positions x = hi + lo (read only)
  void* lam;    // V4<R> solution
  void* res;    // V4<R> residual
  void* q;      // V4<R> H p
  void* minv;   // V4<R> Jacobi M^-1 (0 on fixed components)
  void* p0;
  void* p1;
  void* part;   // reduction partials (vblocks x 2)
  unsigned* cnt;
  CgState* cs;
  int vblocks;
  unsigned long long cond;
};

// Batched PNCG (batch.cu): independent meshes concatenated into one vertex
// and tile set; every mesh has its own SolverState and its own reductions.
struct BatchState {
  int32_t iter;        // iterations of the batch loop
  int32_t iter_limit;
  uint32_t n_active;   // meshes still running after this iteration (vertex tail)
  uint32_t arrived;    // vertex-tail CTAs finished (last one sets the condition)
};

struct BatchArgs {
  SolveArgs a;                 // concatenated meshes (a.st unused)
  int n_meshes;
  int n_chunks;
  const int32_t* tile_mesh;    // n_tiles
  const int32_t* mesh_tile0;   // n_meshes + 1
  const int32_t* chunk_v0;     // n_chunks + 1 vertex ranges, each inside one mesh
  const int32_t* chunk_mesh;   // n_chunks
  const int32_t* mesh_chunk0;  // n_meshes + 1
  SolverState* st;             // n_meshes
  BatchState* bs;
  void* part_dir;              // n_tiles x 6
  void* part_grad;             // n_tiles energy partials (on demand)
  void* part_vert;             // n_chunks x 12
  unsigned long long cond;
};

cudaError_t batch_prepare_kernels(int precision);
cudaError_t launch_batch_init(const BatchArgs& b, const void* u_user, const void* fixed,
                              const int32_t* user_of_internal, const SolverState& proto, cudaStream_t s);
// one iteration of every running mesh: direction pass + tail, gradient pass,
// vertex pass + tail
cudaError_t launch_batch_iteration(const BatchArgs& b, cudaStream_t s);
// gradient + vertex pass at t = 0 (g_0, diag_0 of every mesh)
cudaError_t launch_batch_first(const BatchArgs& b, cudaStream_t s);
cudaError_t launch_batch_set_limit(const BatchArgs& b, int n, cudaStream_t s);
cudaError_t launch_batch_energy(const BatchArgs& b, cudaStream_t s);

cudaError_t cg_prepare_kernels(int precision);
size_t cg_smem(int precision);
cudaError_t launch_cg_init(const CgArgs& c, const void* rhs_user, const int32_t* user_of_internal,
                           cudaStream_t s);
// one CG iteration: element pass (H p), two vertex passes
cudaError_t launch_cg_iteration(const CgArgs& c, cudaStream_t s);
cudaError_t launch_cg_set_limit(const CgArgs& c, int n, cudaStream_t s);
cudaError_t launch_cg_unpack(const CgArgs& c, const int32_t* user_of_internal, void* out_user,
                             cudaStream_t s);
// muscle: out_act[6 c + k] += d(w . grad)/d a_{c,k}, cells in the caller's order
cudaError_t launch_activation_vjp(const FemView& fv, int precision, const void* u_int, const void* w_int,
                                  const int32_t* elem_user, void* out_act, cudaStream_t s);
// out_mu[c] += d(w . grad)/d mu_c (and lambda), cells in the caller's order
cudaError_t launch_param_vjp(const FemView& fv, int precision, const void* u_int, const void* w_int,
                             const void* vol, const int32_t* elem_user, void* out_mu, void* out_lam,
                             cudaStream_t s);

}  // namespace agb

struct agb_solver {
  agb_model* model = nullptr;
  agb_pncg_params params{};
  int precision = 0;
  agb::FemView fv{};
  // combined element data of all potentials (same material)
  agb::TilePlan plan;
  int32_t* d_tile_estart = nullptr;
  int32_t* d_tile_vstart = nullptr;
  int32_t* d_tile_gstart = nullptr;
  int32_t* d_group_estart = nullptr;
  int32_t* d_tv_vid = nullptr;
  int32_t* d_slot_of_tv = nullptr;
  void* d_rec = nullptr;
  uint32_t* d_ids = nullptr;
  // vertex state
  void* d_xa = nullptr;
  void* d_gd = nullptr;
  void* d_p0 = nullptr;
  void* d_p1 = nullptr;
  void* d_xref = nullptr;  // reference state (FP32 stable Neo-Hookean)
  void* d_gref = nullptr;
  void* d_svd = nullptr;   // ARAP: two per-element SVD caches (SolveArgs::svd)
  void* d_slots = nullptr;
  void* d_part = nullptr;
  unsigned* d_cnt = nullptr;
  agb::SolverState* d_state = nullptr;
  agb::SolverState* h_state = nullptr;  // pinned
  void* d_act = nullptr;                // several potentials: concatenated activation stream (muscle)
  void* d_u_tmp = nullptr;              // caller-order staging for host I/O
  agb::SolveArgs args{};
  // adjoint CG (allocated on first use)
  void* d_cg = nullptr;            // lam, res, q, minv, p0, p1: 6 x V4<R> x n_points
  void* d_cg_part = nullptr;
  unsigned* d_cg_cnt = nullptr;
  agb::CgState* d_cg_state = nullptr;
  agb::CgState* h_cg_state = nullptr;  // pinned
  agb::CgArgs cg{};
  cudaGraphExec_t cg_exec = nullptr;
  // graphs
  cudaGraphExec_t loop_exec = nullptr;
  cudaGraphExec_t step_exec = nullptr;
  int step_kernels = 0;  // kernel nodes of one iteration
  cudaStream_t capture_stream = nullptr;
  bool has_state = false;  // vertex state written (reset or checkpoint load)
  uint64_t fingerprint = 0;  // of the model and parameters, checked by agb_solver_load
};

struct agb_batch {
  std::vector<agb_model*> models;
  agb_pncg_params params{};
  int precision = 0;
  int chunk_verts = 0;
  std::vector<int32_t> vert_off;  // per model, n_models + 1 (concatenated vertex ids)
  agb::TilePlan plan;             // concatenated tiles (tv_vid in concatenated ids)
  int32_t n_slots = 0;
  // device
  int32_t* d_tile_estart = nullptr;
  int32_t* d_tile_vstart = nullptr;
  int32_t* d_tile_gstart = nullptr;
  int32_t* d_group_estart = nullptr;
  int32_t* d_tv_vid = nullptr;
  void* d_act = nullptr;           // muscle activation stream (any muscle potential), else null
  void* d_rec = nullptr;
  uint32_t* d_ids = nullptr;
  int32_t* d_slot_of_tv = nullptr;
  int32_t* d_off = nullptr;
  int32_t* d_uoi = nullptr;        // concatenated user_of_internal
  void* d_fixed = nullptr;         // V4<R>, w = mask bits
  void* d_force = nullptr;         // V4<R> or null
  int32_t* d_tile_mesh = nullptr;
  int32_t* d_mesh_tile0 = nullptr;
  int32_t* d_chunk_v0 = nullptr;
  int32_t* d_chunk_mesh = nullptr;
  int32_t* d_mesh_chunk0 = nullptr;
  void* d_xa = nullptr;
  void* d_gd = nullptr;
  void* d_p0 = nullptr;
  void* d_p1 = nullptr;
  void* d_xref = nullptr;  // reference state (FP32)
  void* d_gref = nullptr;
  void* d_slots = nullptr;
  void* d_svd = nullptr;   // ARAP: the two per-element SVD caches
  void* d_part = nullptr;
  agb::SolverState* d_state = nullptr;
  agb::SolverState* h_state = nullptr;  // pinned, n_meshes
  agb::BatchState* d_bstate = nullptr;
  agb::BatchArgs args{};
  cudaGraphExec_t loop_exec = nullptr;
  cudaGraphExec_t step_exec = nullptr;
  cudaStream_t capture_stream = nullptr;
};
