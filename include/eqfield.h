/*
 * eqfield — GB300-native quorum-sensing field step (C ABI).
 *
 * One handle = one batch of independent traps (HSL layers); a single trap is a
 * batch of one.  Each trap carries one species on a structured "right"
 * triangulation of [0, W] x [0, H] and is stepped by backward Euler:
 *
 *   ((1 + dt*g) M + dt*D*K + dt*C(v)) c^{n+1} = M c^n + F,  c = 0 on Dirichlet walls
 *
 * with F = dt * sum_i s_i phi(x_i) from point cells (sources) and/or values added
 * to the nodal field before a step (the reference's deposit into u0).
 *
 * This replaces the reference's FEniCS/PETSc layer solver, the plugin
 * eQ::diffusionSolver (src/eQ.h:302-330) as implemented by fenicsInterface
 * (src/fHSL.h:333-449, src/fHSL.cpp), together with the controller-side
 * deposit/gather lambdas writeHSL/readHSL (src/abm/eQabm.cpp:326-359).  Each
 * entry point names the reference interface it replaces.
 *
 * Conventions: every call returns EQF_OK (0) or a negative EQF_ERR_* code and
 * records a message readable with eqf_last_error().  Nodal vectors are in grid
 * order k = j + i*(nx+1) (eQ::data::index_from_ij, src/eQ.h:131-134); the DOLFIN
 * DOF map of the reference is the identity here.  The library owns all device
 * memory; host buffers are read or written only during the call.  A handle is
 * not thread-safe: use one handle per host thread or lock externally.
 */
#ifndef EQFIELD_H
#define EQFIELD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EQF_OK 0
#define EQF_ERR_INVALID (-1)        /* bad argument or size */
#define EQF_ERR_CUDA (-2)           /* CUDA runtime error (message has the detail) */
#define EQF_ERR_NOT_CONVERGED (-3)  /* a trap missed its tolerance within the schedule */
#define EQF_ERR_NO_DEVICE (-4)      /* no CUDA device visible */
#define EQF_ERR_NOMEM (-5)          /* device allocation failed */
#define EQF_ERR_TOO_LARGE (-6)      /* input beyond the fixed maximum of an allocation-free call */

/* Dirichlet walls (c = 0); unset walls are zero-flux.  The reference's trap types
 * (src/fHSL.h:456-504, decoded at src/fHSL.cpp:557-569) map to:
 * THREEWALLED = BOTTOM, TWOWALLED = BOTTOM|TOP, ONEWALLED = BOTTOM|LEFT|RIGHT,
 * NOWALLED = all four. */
#define EQF_WALL_BOTTOM 1u
#define EQF_WALL_TOP 2u
#define EQF_WALL_LEFT 4u
#define EQF_WALL_RIGHT 8u

/* Arithmetic of the solve. */
#define EQF_PREC_FP64 0    /* plain form: FP64 operator, multigrid and Krylov */
#define EQF_PREC_FP32_IR 1 /* FP32 operator/multigrid/Krylov inside FP64 refinement */

/* Per-trap parameters.  Replaces eQ::diffusionSolver::params (src/eQ.h:305-321):
 * trapWidthMicrons/trapHeightMicrons -> width/height, nodesPerMicron -> nx, ny
 * (the reference uses nx = ceil(W*npm), ny = ceil(H*npm), src/fHSL.cpp:242-243),
 * D_HSL -> D, dt -> dt.  decay and the advection velocity are extensions. */
typedef struct eqf_trap_params {
  double width, height; /* trap size W, H */
  int32_t nx, ny;       /* squares along x, y (nodes: (nx+1)*(ny+1)) */
  double D;             /* diffusion constant */
  double dt;            /* time step */
  double decay;         /* first-order decay g (0 in the reference form) */
  double adv_u;         /* advection v = (0, -adv_u * y / adv_len); 0 = none */
  double adv_len;
  uint32_t walls;       /* EQF_WALL_* bits */
} eqf_trap_params;

/* Krylov method of the inner solve (eqf_solver_opts.krylov). */
#define EQF_KRYLOV_AUTO 0
#define EQF_KRYLOV_CG 1
#define EQF_KRYLOV_BICGSTAB 2

/* Solver options shared by a batch. */
typedef struct eqf_solver_opts {
  int32_t precision;  /* EQF_PREC_* */
  double rtol;        /* |b - A c| <= rtol |b| per trap and step (FP64 residual) */
  int32_t max_sweeps; /* refinement sweeps per step (FP64 form: Krylov restarts) */
  int32_t max_iters;  /* preconditioned Krylov iterations per sweep */
  double inner_tol;   /* FP32 inner solve: relative residual reduction per sweep */
  int32_t cheb_pre, cheb_post, cheb_coarse; /* Chebyshev degrees */
  double cheb_ratio;  /* smoothing interval [lmax/ratio, lmax] */
  int32_t use_graph;  /* capture steps as CUDA graphs */
  int32_t adaptive;   /* after each step check convergence and add refinement sweeps
                       * (up to 8) for the traps that missed rtol: with use_graph on
                       * the device, as a conditional loop inside the step's graph (the
                       * step does not wait; a trap still failing is reported by the
                       * next eqf_sync or readout), else on the host after each step */
  int32_t tile_nodes; /* target nodes per row tile of the finest level (0: default) */
  int32_t krylov;     /* EQF_KRYLOV_*: AUTO = BiCGSTAB iff some trap has advection */
  int32_t fuse_levels; /* 0: step-by-step V-cycle kernels; 1 (default): temporally
                        * blocked V(2,2) level kernels where they fit; 2: also the levels
                        * from the first whose grids fit one CTA's shared memory down to
                        * the coarsest in one kernel, one CTA per trap (bit-identical to
                        * 1; slower on large uneven batches, where the largest trap's
                        * CTA sets the time) */
  int32_t residual64;  /* FP32 form: 0 (default) evaluates the refinement's right-hand
                        * side b = F + M c^n and residual b - A c in float-pair arithmetic
                        * on the FP32 pipe (~47 significant bits); 1 evaluates them in FP64
                        * with the plain form's kernels (the FP64 pipe is ~1/64 of the
                        * FP32 rate on this part).  Ignored by the FP64 form. */
  int32_t tile_cols;   /* columns of the fused level kernels' 2-D tiles (a multiple of 4
                        * in [16, 512]; 0: the default 128); their rows follow from the
                        * tile node target */
} eqf_solver_opts;

typedef struct eqf_batch eqf_batch;

/* Fills opts with the defaults for a precision. */
int eqf_default_opts(int32_t precision, eqf_solver_opts* opts);

/* Creates a batch of n_traps traps on the current CUDA device.
 * Replaces fenicsInterface::initDiffusion (src/fHSL.cpp:37-53) -> fenicsClassInit
 * (src/fHSL.cpp:195-328: mesh, forms, boundary conditions, solver). */
int eqf_create(int32_t n_traps, const eqf_trap_params* traps, const eqf_solver_opts* opts,
               eqf_batch** out);

/* Autotuning (no reference counterpart).  A tuning table maps trap size buckets
 * (node count <= max_nodes, ascending; the last bucket takes the rest) to the tile
 * node target, the 2-D tile width of the fused level kernels and the pre/post
 * Chebyshev degrees that were fastest for traps of that size (DOF-steps/s at the
 * solver tolerance, measured by eqf_autotune), and the Krylov schedule (inner
 * iterations per refinement sweep, scheduled sweeps) that was fastest with them.
 * eqf_create_tuned creates a batch whose traps take the tile target and width of
 * their bucket and whose smoother degrees and schedule are those of the bucket that
 * holds most of its nodes. */
#define EQF_TUNE_MAX_BUCKETS 8
typedef struct eqf_tune_bucket {
  int64_t max_nodes;
  int32_t tile_nodes, cheb_pre, cheb_post;
  int32_t tile_cols;      /* 2-D tile columns of the fused level kernels (0: default) */
  double dof_steps_per_s; /* measured rate of the chosen configuration */
  int32_t max_iters, max_sweeps; /* Krylov schedule (0: the caller's eqf_solver_opts) */
} eqf_tune_bucket;
typedef struct eqf_tune_table {
  int32_t n;
  eqf_tune_bucket b[EQF_TUNE_MAX_BUCKETS];
} eqf_tune_table;

int eqf_create_tuned(int32_t n_traps, const eqf_trap_params* traps, const eqf_solver_opts* opts,
                     const eqf_tune_table* table, eqf_batch** out);

/* Measures, for each size bucket, candidate Chebyshev degrees, then tile node
 * targets x 2-D tile widths at the best degrees, then Krylov schedules (inner
 * iterations x scheduled refinement sweeps: the caller's, 2 x 4 and 3 x 3) at the best
 * of those, on a batch of the given traps that fall into the bucket (replicated up to
 * a GPU-filling node count), with random point cells, and writes the fastest into
 * *table.  Buckets: <= 32k, <= 128k, <= 512k nodes, and larger.  Takes about budget_s
 * seconds of GPU time at most (unexplored candidates keep the defaults).  When log is
 * not NULL, one line per measured candidate ("bucket tile_nodes tile_cols cheb_pre
 * cheb_post max_iters max_sweeps dof_steps_per_s") is written into it, at most
 * log_size bytes including the terminating zero. */
int eqf_autotune(int32_t n_traps, const eqf_trap_params* traps, const eqf_solver_opts* opts,
                 double budget_s, eqf_tune_table* table);
int eqf_autotune_log(int32_t n_traps, const eqf_trap_params* traps, const eqf_solver_opts* opts,
                     double budget_s, eqf_tune_table* table, char* log, int64_t log_size);

/* Releases all device memory.  Replaces fenicsInterface::finalize / destructor
 * (src/fHSL.cpp:655-661). */
int eqf_destroy(eqf_batch* b);

/* Message of the last failed call on this handle (or of the last eqf_create). */
const char* eqf_last_error(const eqf_batch* b);

/* Node count of a trap. */
int eqf_num_nodes(const eqf_batch* b, int32_t trap, int64_t* n_nodes);
/* The parameters a trap was created with (walls as set by eqf_set_boundaries). */
int eqf_trap_info(const eqf_batch* b, int32_t trap, eqf_trap_params* out);

/* Point cells of trap `trap`: positions xy[2*n] (x, y interleaved) and source
 * rates s[n].  The load dt * sum s_i phi(x_i) is deposited deterministically
 * onto the containing triangles and applied every step until replaced.
 * Replaces the deposit writeHSL (src/abm/eQabm.cpp:338-359) for point cells. */
int eqf_set_cells(eqf_batch* b, int32_t trap, int64_t n, const double* xy, const double* s);

/* Couples trap2 to trap1 as the sender/receiver quorum-sensing pair: species 1
 * lives on trap1, species 2 on trap2 (same mesh).  The cells are those set on
 * trap1 by eqf_set_cells (their rates s are the senders' production of species 1);
 * trap2 gets the same positions.  sender[i] (1 = sender, 0 = receiver) for each
 * of trap1's cells.  Every step, from the concentrations c1, c2 gathered at the
 * cell centres at the start of the step, the point sources
 *   s1_i = sender_i * s_i - uptake * c1_i
 *   s2_i = (1 - sender_i) * vmax * c1_i / (K + c1_i) - uptake * c2_i
 * are deposited for the two species (explicit in time).  No reference counterpart:
 * a config extension whose per-cell exchange is evaluated like the membrane term
 * of the reference's strains (src/Strain.h:312-313).  The cells of both traps must
 * not be replaced afterwards. */
int eqf_couple_species(eqf_batch* b, int32_t trap1, int32_t trap2, const int32_t* sender,
                       double vmax, double K, double uptake);

/* Replaces the source rates of the cells set by eqf_set_cells (same order),
 * keeping their positions and sort order. */
int eqf_set_cell_rates(eqf_batch* b, int32_t trap, int64_t n, const double* s);

/* Sets the nodal field (grid order).  Replaces the controller's write of
 * solution_vector before stepDiffusion (src/simulation.cpp:455-463, 500-505;
 * src/fHSL.cpp:104). */
int eqf_set_nodal(eqf_batch* b, int32_t trap, const double* c);

/* Adds increments to nodes (grid-order indices): the reference deposit that
 * adds dHSL into u0 (src/abm/eQabm.cpp:347-358). */
int eqf_add_nodal(eqf_batch* b, int32_t trap, int64_t n, const int64_t* node,
                  const double* delta);

/* Advances every trap of the batch by n_steps backward-Euler steps.
 * Replaces fenicsInterface::stepDiffusion (src/fHSL.cpp:98-161). */
int eqf_step(eqf_batch* b, int32_t n_steps);

/* Reads the nodal field (grid order).  Replaces reading solution_vector after
 * stepDiffusion (src/fHSL.cpp:108; src/simulation.cpp:491-492). */
int eqf_read_nodal(eqf_batch* b, int32_t trap, double* c);

/* The nodal field in a caller's DOF order: dof_from_vertex[v] is the DOF index of
 * vertex v = j + i*(nx+1) (grid order), a permutation of 0 .. n-1 (checked), such as
 * DOLFIN's vertex_to_dof_map that fenicsShell::getVertexMappings exports
 * (src/fHSL.h:82-87) and Simulation::create_HSLgrid turns into its lookup table
 * (src/simulation.cpp:363-386).  eqf_read_nodal_dof writes c[dof_from_vertex[v]] =
 * field(v) (solution_vector after stepDiffusion, src/fHSL.cpp:108); eqf_set_nodal_dof
 * sets field(v) = c[dof_from_vertex[v]] (u0 before the solve, src/fHSL.cpp:104), as
 * eqf_set_nodal does. */
int eqf_read_nodal_dof(eqf_batch* b, int32_t trap, const int32_t* dof_from_vertex, double* c);
int eqf_set_nodal_dof(eqf_batch* b, int32_t trap, const int32_t* dof_from_vertex,
                      const double* c);

/* Concentration at the cells set by eqf_set_cells, sampled on their triangles.
 * Replaces the gather readHSL (src/abm/eQabm.cpp:326-337) for point cells. */
int eqf_read_cells(eqf_batch* b, int32_t trap, int64_t n, double* c);

/* D * dt * (-int grad c . n ds): the reference's totalBoundaryFlux
 * (fenics/boundary.ufl:9-12, src/fHSL.cpp:156-160, read by getBoundaryFlux). */
int eqf_boundary_flux(eqf_batch* b, int32_t trap, double* flux);

/* Total amount 1^T M c (FP64), for the mass-balance check. */
int eqf_total_mass(eqf_batch* b, int32_t trap, double* mass);

/* FP64 total-HSL mass balance of every step (no reference counterpart: the
 * reference keeps only the facet flux functional of the new field,
 * fenics/boundary.ufl:9-12, src/fHSL.cpp:156-160, and the boundary well built on it,
 * src/simulation.cpp:581-604).  While enabled, every step ends with an FP64
 * reduction over each trap (one extra pass over the old and new fields and the load)
 * that closes the step's discrete balance
 *   mass - mass_prev = load - decay - operator_loss - wall_outflow + drift
 * where mass = 1^T M c^{n+1}; mass_prev = 1^T M c^n, the field the step started from
 * (after any deposit into it); load = the sum of the step's load F (point cells,
 * Robin walls); decay = dt*g*mass; operator_loss = 1^T (dt C + R) c^{n+1} (advective
 * and Robin outflow); wall_outflow = the consistent flux through the Dirichlet walls
 * (minus the full operator's residual summed over the Dirichlet rows); drift = the
 * solver's residual summed over the free rows, zero up to the step's tolerance.
 * Enabling (again) zeroes the sums; eqf_read_balance returns the last step's terms
 * and the sums since then. */
typedef struct eqf_balance {
  double mass, mass_prev, load, decay, operator_loss, wall_outflow, drift;
  double drift_sum;     /* sum of drift over the steps since enabled */
  double drift_abs_sum; /* sum of |drift| */
  double load_sum;      /* sum of load */
  double drift_rel_max; /* max over steps of |drift| / max(|mass|, |mass_prev|, |load|,
                           |wall_outflow|) */
  int64_t steps;        /* steps since enabled (frozen traps' steps not counted) */
} eqf_balance;
int eqf_mass_balance(eqf_batch* b, int32_t enable);
int eqf_read_balance(eqf_batch* b, int32_t trap, eqf_balance* out);

/* Solver statistics of a trap since creation: steps, refinement sweeps and
 * Krylov iterations, and the last step's relative FP64 residual. */
int eqf_stats(eqf_batch* b, int32_t trap, int64_t* steps, int64_t* sweeps, int64_t* iters,
              double* last_rel_residual);

/* Waits for queued device work and reports deferred errors (convergence). */
int eqf_sync(eqf_batch* b);

/* Asynchronous use (no reference counterpart; the serving loop of eqserve.h is
 * built on these).  With opts.adaptive = 0, or adaptive with use_graph, eqf_step
 * only queues the steps on the batch's stream and returns.  eqf_poll sets *idle to 1 once all queued work has
 * finished (and then reports deferred errors, as eqf_sync), else 0, without
 * waiting.  eqf_read_cells_async / eqf_read_nodal_async queue the readout of a
 * trap's current state into host memory (pinned for the copy to overlap), valid
 * once eqf_poll reports idle or after eqf_sync; a second asynchronous cell readout
 * of the same trap before then overwrites the first's device staging.
 * eqf_set_active(b, t, 0) freezes trap t: the following steps skip it entirely
 * and its field stays as it is; eqf_set_active(b, t, 1) resumes it (with a fresh
 * initial-guess history).  Frozen traps keep their device memory. */
int eqf_poll(eqf_batch* b, int32_t* idle);
/* Slot reuse (no reference counterpart; the serving loop admits requests into the
 * slots of finished ones with it): trap t becomes the trap *p, whose grid must fit
 * t's slot at every multigrid level (eqf_slot_fits tells; a smaller nx and ny is not
 * enough, as a level halves an axis only while it has at least 4 cells), with no more
 * levels than the batch and, if advective, in a batch that solves with BiCGSTAB.
 * The new trap starts from a zero field with no cells, couplings, tensor or well and
 * with the Dirichlet walls of p->walls; it is active.  The other traps keep their
 * state and give the same bits as without the replacement.  Operators, tile lists and
 * the geometry are rebuilt before the call returns (it waits for the batch's own
 * queued work), the cell index and the captured step at the next step.  A trap that
 * carries rod cells or a flow channel cannot be replaced (EQF_ERR_INVALID). */
int eqf_replace_trap(eqf_batch* b, int32_t trap, const eqf_trap_params* p);
/* The same for n slots at once (one rebuild): traps[k] becomes p[k]; every entry is
 * checked before any slot changes. */
int eqf_replace_traps(eqf_batch* b, int32_t n, const int32_t* traps, const eqf_trap_params* p);
/* *fits = 1 if eqf_replace_trap(b, trap, p) would accept p, else 0 (host-side check). */
int eqf_slot_fits(const eqf_batch* b, int32_t trap, const eqf_trap_params* p, int32_t* fits);
int eqf_read_cells_async(eqf_batch* b, int32_t trap, int64_t n, double* c);
int eqf_read_nodal_async(eqf_batch* b, int32_t trap, double* c);
int eqf_set_active(eqf_batch* b, int32_t trap, int32_t active);
/* Queues a copy of the batch's count of trap-steps that missed rtol so far into
 * *count (host memory), valid like the asynchronous readouts above. */
int eqf_fail_count_async(eqf_batch* b, int32_t* count);

/* Device bytes a batch of these traps with n_cells cells in total would hold
 * (including the transient of the first cell upload), for admission control.
 * Needs no device. */
int eqf_footprint_estimate(int32_t n_traps, const eqf_trap_params* traps,
                           const eqf_solver_opts* opts, int64_t n_cells, int64_t* bytes);

/* Batch-wide cell I/O for the per-step host exchange (one copy each way): rates
 * and concentrations of every trap's cells, concatenated in trap order (the
 * order of the eqf_set_cells calls within a trap).  Replaces the controller's
 * per-layer vector exchange of src/simulation.cpp:425-463 / 491-505. */
int eqf_set_cell_rates_all(eqf_batch* b, int64_t n, const double* s);
int eqf_read_cells_all(eqf_batch* b, int64_t n, double* c);

/* ---------------------------------------------------------------------------
 * Wall conditions and flow channels: the reference's MICROFLUIDIC_TRAP boundary
 * mode (fenicsInterface::createHSL, src/fHSL.cpp:446-540; setRobinBoundaryConditions,
 * 331-364; the channels' stepping in stepDiffusion, 54-152).
 *
 * Each wall of a trap is Neumann (zero flux), Dirichlet (c = value), Robin (the
 * hslD terms dt*r*(c - s)*v on ds, fenics/hslD.ufl:31-42) or, for the bottom and top
 * walls, Dirichlet to a flow channel: a 1D advection-diffusion layer of nx+1 nodes on
 * [0, W] (fenics/AdvectionDiffusion.ufl: Crank-Nicolson, flow velocity v, Robin rates
 * at its two ends, fenicsChannel, src/fHSL.h:240-330).  Every step: the trap solve
 * takes the channels' current values on those walls, then each channel receives the
 * flux h*(dt*D*grad_j)/well_scaling of every column j (grad from the wall row and the
 * row next to it, computeBoundaryFlux, src/fHSL.cpp:54-95) spread over `substeps`
 * Crank-Nicolson sub-steps of dt/substeps.  Where walls meet, the bottom and top
 * walls' conditions win (the reference applies them last).
 */
#define EQF_SIDE_BOTTOM 0
#define EQF_SIDE_TOP 1
#define EQF_SIDE_LEFT 2
#define EQF_SIDE_RIGHT 3
#define EQF_BC_NEUMANN 0
#define EQF_BC_DIRICHLET 1 /* c = value */
#define EQF_BC_ROBIN 2     /* dt*rate*(c - value) on the wall */
#define EQF_BC_CHANNEL 3   /* c = the flow channel's concentration (bottom, top) */
#define EQF_BC_WELL 4      /* c = the trap's boundary-well concentration (the reference's
                              DIRICHLET_UPDATE walls, src/fHSL.cpp:545-554) */
typedef struct eqf_wall {
  int32_t kind; /* EQF_BC_* */
  double value; /* Dirichlet value / Robin external concentration s */
  double rate;  /* Robin rate r */
} eqf_wall;
typedef struct eqf_boundaries {
  eqf_wall wall[4];         /* indexed by EQF_SIDE_* */
  double channel_velocity;  /* flow velocity v (parameters["simulationFlowRate"]) */
  double channel_D;         /* channel diffusion constant (the layer's D_HSL) */
  double channel_rate[2];   /* Robin rates at the channel's x = 0 and x = W ends (s = 0) */
  int32_t channel_substeps; /* parameters["channelSolverNumberIterations"] (>= 1) */
  double well_scaling;      /* wellScaling of src/fHSL.cpp:47 */
} eqf_boundaries;

/* Sets the wall conditions of a trap (replacing the walls bitfield of its
 * eqf_trap_params: a set bit there means EQF_BC_DIRICHLET with value 0).  Channel
 * walls need a square lattice (W/nx = H/ny).  Rebuilds the batch's operators. */
int eqf_set_boundaries(eqf_batch* b, int32_t trap, const eqf_boundaries* bc);
/* The trap's bottom and top channel concentrations (nx+1 values each, x = j*W/nx);
 * either pointer may be NULL.  Channels start at 0. */
int eqf_read_channels(eqf_batch* b, int32_t trap, double* bottom, double* top);
int eqf_set_channels(eqf_batch* b, int32_t trap, const double* bottom, const double* top);

/* Anisotropic diffusion tensor of a trap: per node (grid order) the D11, D22, D12 of
 * hslD's A = D*[[D11, D12], [D12, D22]] (fenics/hslD.ufl:31), the reference's
 * D11/D22/D12 vectors (src/fHSL.h:418), filled per cell by setDiffusionTensor
 * (src/abm/eQabm.cpp:306-325) and sampled by AnisotropicDiffusionTensor
 * (src/Expressions.h:95-124).  The fields are P1: each triangle's stiffness uses the
 * mean of its three vertex tensors.  All three NULL restores the isotropic tensor
 * (1, 1, 0).  The tensor must be symmetric positive definite at every node.  Such
 * traps take the per-node stencil path; their multigrid levels take the tensor by
 * injection.  Rebuilds the batch's operators. */
int eqf_set_tensor(eqf_batch* b, int32_t trap, const double* D11, const double* D22,
                   const double* D12);

/* Boundary well of a trap (Simulation::computeBoundaryWell, src/simulation.cpp:581-604):
 * after every step, with the step's totalBoundaryFlux F = D*dt*(-int grad c . n ds),
 *   w += F / well_scaling;  w -= dt * decay_rate * w;  w < 0 -> w = 0 (an underflow)
 * well_scaling = 2*10*(15/lengthScaling)*(W + H) and decay_rate = flow rate / W in the
 * reference (initBoundaryWell, setBoundaryRate: src/simulation.cpp:605-627).  Walls of
 * kind EQF_BC_WELL take w as their value in the next step.  well_scaling = 0 switches
 * the well off; it starts at 0. */
int eqf_set_well(eqf_batch* b, int32_t trap, double well_scaling, double decay_rate);
int eqf_read_well(eqf_batch* b, int32_t trap, double* concentration, int64_t* underflows);
/* Sets the well concentration w that EQF_BC_WELL walls take as their value in the
 * next step: fenicsInterface::setBoundaryValues (src/fHSL.cpp:601-604), called by
 * Simulation::computeBoundaryWell with the host's own well model under
 * DIRICHLET_UPDATE (src/simulation.cpp:581-604).  With the device's well model off
 * (well_scaling 0) the value stays until set again. */
int eqf_set_well_concentration(eqf_batch* b, int32_t trap, double concentration);

/* ---------------------------------------------------------------------------
 * Output in the reference's formats (host-side writers; the reads from a batch are
 * ordinary synchronous readouts).
 *
 * JSON recording: jsonRecording (src/main.cpp:81-192), "jsonSimVersion" v00_02.  The
 * file is one object with the keys in sorted order, as the reference's JSON library
 * writes them: cellDataFormat, frames, jsonSimVersion, nodeID, parameters, simNumber,
 * timeSinceEpoch.  A frame is {"cells", "divisions", "externalHSL", "simTime"}: cells
 * as [[id, strainType], [x, y, angle, length, spring, HSL (nM) ...]], divisions as
 * [time, parent id, parent length, daughter id, daughter length]
 * (eQabm::recordDivisionEvent, src/abm/eQabm.cpp:458-480) and externalHSL as one array
 * per layer in grid order.  Frames stream to the file as they are recorded.
 */
typedef struct eqf_json eqf_json;
int eqf_json_open(const char* path, int64_t time_since_epoch, int32_t node_id,
                  int32_t sim_number, eqf_json** out);
/* One frame with the layers' fields read from the batch: n_div divisions (5 values
 * each), n_cells cells with ids[2*i] = id, ids[2*i+1] = strain type and n_data values
 * each in data. */
int eqf_json_frame(eqf_json* j, eqf_batch* b, int32_t n_layers, const int32_t* layers,
                   double sim_time, int64_t n_div, const double* divisions, int64_t n_cells,
                   const int64_t* ids, int32_t n_data, const double* data);
/* The same with the fields in host memory: n_layers grids of n_nodes values each. */
int eqf_json_frame_host(eqf_json* j, int32_t n_layers, int64_t n_nodes, const double* fields,
                        double sim_time, int64_t n_div, const double* divisions,
                        int64_t n_cells, const int64_t* ids, int32_t n_data, const double* data);
/* Finishes and closes the file; parameters_json is the "parameters" object as JSON text
 * (NULL: {}). */
int eqf_json_close(eqf_json* j, const char* parameters_json);

/* VTK snapshots: what fenicsInterface::writeDiffusionFiles writes through DOLFIN's File
 * (src/fHSL.cpp:606-632): a .pvd collection (rewritten at every snapshot) and one .vtu
 * per snapshot (<stem>NNNNNN.vtu beside it) with the mesh and the nodal field "u".
 * A trap is its "right" triangulation; a channel the nx+1 nodes of its wall as line
 * cells. */
typedef struct eqf_vtk eqf_vtk;
int eqf_vtk_open(const char* pvd_path, eqf_vtk** out);
int eqf_vtk_write(eqf_vtk* v, eqf_batch* b, int32_t trap, double time);
int eqf_vtk_write_channel(eqf_vtk* v, eqf_batch* b, int32_t trap, int32_t side, double time);
/* A field in host memory: ny > 0 a trap of nx x ny squares on [0, W] x [0, H]; ny = 0 a
 * channel of nx cells on [0, W]. */
int eqf_vtk_write_host(eqf_vtk* v, double width, double height, int32_t nx, int32_t ny,
                       const double* field, double time);
int eqf_vtk_close(eqf_vtk* v);

/* ---------------------------------------------------------------------------
 * Rod cells of the agent-based model, coupled the reference's way.
 *
 * Replaces the per-cell loop of eQabm::updateCells (src/abm/eQabm.cpp:234-390):
 * the interior-node search findInteriorPoints (268-304) with
 * cpmEcoli::pointIsInCell (src/abm/cpmEcoli.cpp:313-328), the interior-mean
 * gather readHSL (326-337), the strain's membrane exchange
 * (Strain::computeConcentrations / pushConcentrations, src/Strain.h:281-345, and
 * sendRecvStrain::computeProteins, src/Strain.cpp:10-73) and the equal-split
 * deposit writeHSL into u0 (338-359), with the unit conversions of eQ::Cell
 * (src/eQcell.h:42-97).  The cells are processed in array order with the
 * reference's sequential semantics: a cell reads the deposits of every earlier
 * cell whose footprint shares a node with its own.  Every eqf_step runs the
 * exchange for all rod cells at the start of each step, before the solve.
 *
 * One rod set belongs to one simulation: its layers are traps of the batch with
 * the same mesh, a lattice of nodes_per_micron nodes per micron in both directions
 * (W*npm = nx and H*npm = ny exactly, eQabm's nodesWide - 1 and nodesHigh - 1,
 * src/abm/eQabm.cpp:30-31).  A trap belongs to at most one rod set.
 */
#define EQF_MAX_ROD_LAYERS 4
/* per cell and layer: how the cell's circuit treats that HSL species */
#define EQF_ROD_HELD 0    /* exchange deposited; intracellular HSL only converted
                             nM <-> molecules (a species the strain does not update) */
#define EQF_ROD_CIRCUIT 1 /* iHSL += dt*production - exchange (sender: production =
                             hslProductionRate; receiver: 0), clamped at 0 */
#define EQF_ROD_INERT 2   /* no exchange (a strain without an HSL circuit) */

/* One rod cell as the agent-based model holds it.  All lengths in microns. */
typedef struct eqf_rod {
  double center[2];   /* Ecoli::getCenter_x/y: the fallback node when no lattice
                         node lies inside (src/abm/eQabm.cpp:299-303) */
  double pole_a[2];   /* Ecoli::polePositionA/B, clamped to the trap as
                         Ecoli::updatePoleCenters does (src/abm/Ecoli.cpp:36-60): */
  double pole_b[2];   /*   they bound the node search */
  double body_pos[2]; /* position of the cell's first half (cpBodyGetPosition(bodyA)) */
  double body_rot[2]; /* its rotation (cos, sin) (cpBodyGetRotation(bodyA)) */
  double verts[8];    /* cpmEcoli::vertsA[0..3], that half's box in its own frame,
                         clockwise (x, y pairs) */
  double length;      /* Ecoli::getLengthMicrons */
  double reserved;    /* 0 */
} eqf_rod;

typedef struct eqf_rod_law {
  double nodes_per_micron; /* parameters["nodesPerMicronSignaling"] */
  double dt;               /* cell-model time step (the strain's params.dt) */
  double membrane_rate[EQF_MAX_ROD_LAYERS]; /* parameters["membraneDiffusionRates"] */
} eqf_rod_law;

/* Sets (replaces) the rod cells of the simulation whose layers are
 * layers[0..n_layers-1], with their state: ihsl[c*n_layers + l] intracellular
 * HSL (molecules, as Strain stores iHSL), production[c*n_layers + l] (nM/min) and
 * mode[c*n_layers + l] (EQF_ROD_*).  n_cells = 0 removes the set. */
int eqf_set_rods(eqf_batch* b, int32_t n_layers, const int32_t* layers, const eqf_rod_law* law,
                 int64_t n_cells, const eqf_rod* rods, const double* ihsl,
                 const double* production, const uint8_t* mode);
/* Moves the cells of the set whose first layer is layer0 (same count and order);
 * their intracellular state stays on the device.  production may be NULL (kept). */
int eqf_update_rods(eqf_batch* b, int32_t layer0, int64_t n_cells, const eqf_rod* rods,
                    const double* production);
/* Reads, per cell and layer, the intracellular HSL (molecules) and the mean field
 * value over the cell's footprint gathered by the last exchange (readHSL; 0 before
 * the first), and per cell the number of footprint nodes.  Any pointer may be NULL. */
int eqf_read_rods(eqf_batch* b, int32_t layer0, int64_t n_cells, double* ihsl, double* ehsl,
                  int32_t* points);
/* eqf_update_rods and eqf_read_rods for every rod set of the batch in one call (no
 * reference counterpart: a controller driving several simulations on one GPU).  The
 * sets are taken in increasing order of their first layer; rods, production, ihsl,
 * ehsl and points hold each set's block in turn, laid out as for the per-set calls;
 * n_total is the number of cells of all sets.  The result is the same as one per-set
 * call per set, with a few host round trips for the whole batch instead of several
 * per set. */
int eqf_update_rods_all(eqf_batch* b, int64_t n_total, const eqf_rod* rods,
                        const double* production);
int eqf_read_rods_all(eqf_batch* b, int64_t n_total, double* ihsl, double* ehsl,
                      int32_t* points);
/* Runs the exchange once now, without a solve (the reference's updateCells alone). */
int eqf_exchange_rods(eqf_batch* b);
/* Number of sequential waves the exchange of the current rod cells takes (1 when
 * no two cells share a footprint node). */
int eqf_rod_waves(eqf_batch* b, int32_t* waves);
/* Passes the last wave analysis of any rod set took to settle (0 when no set has a
 * shared node).  The analysis relaxes every footprint entry once per pass in one CTA,
 * so its device time grows with the entries times this count (the longest chain of
 * cells sharing nodes, plus one). */
int eqf_rod_relax_passes(eqf_batch* b, int32_t* passes);

/* Built-in profiler (no counterpart in the reference, which only keeps MPI_Wtime
 * accumulators, src/simulation.h:512-521).  While enabled, steps run without CUDA
 * graphs and every kernel launch is bracketed by CUDA events on the batch's
 * stream and counts the nodes it processed.  eqf_profile(b, 1) resets and starts,
 * eqf_profile(b, 0) stops.  eqf_profile_read returns per kernel class the summed
 * launch time (ms), launches, processed nodes and algorithmic bytes.  Classes, in
 * order: finest-level operator smoothing step, finest-level first smoothing step,
 * finest-level residual, restriction from the finest level, prolongation to the
 * finest level, coarser levels, CG direction (q = A p), CG update, refinement
 * residual (first of a step), refinement residual, refinement update, per-trap
 * scalar phases, finest-level fused pre-smoothing + residual, finest-level fused
 * prolongation + post-smoothing, rod-cell exchange (eqf_set_rods), mass balance
 * (eqf_mass_balance). */
/* The CUDA stream (cudaStream_t) all work of the batch is queued on, for callers
 * that time the batch with their own CUDA events or order their own work. */
int eqf_stream(eqf_batch* b, void** stream);

#define EQF_PROF_CLASSES 17
int eqf_profile(eqf_batch* b, int32_t enable);
int eqf_profile_read(eqf_batch* b, int32_t n_classes, double* ms, int64_t* launches,
                     int64_t* nodes, double* bytes);

/* Allocation-free field integral.  No counterpart in the reference: this is an
 * extra entry point for callers that may not allocate device memory when they
 * need a figure (a simulation running under its own device-memory budget or
 * allocator, or code that must not trigger the device-wide synchronisation a
 * cudaMalloc/cudaFree can cause).  It computes, for a nodal field d_field in the
 * caller's device memory (grid order, nx x ny squares on [0, width] x [0, height]):
 *   what 0: the total amount 1^T M c            (as eqf_total_mass)
 *   what 1: -int grad c . n ds over the boundary (as eqf_boundary_flux / (D*dt))
 * multiplied by `scale`, into *out (host), on `stream` (a cudaStream_t, NULL for
 * the default stream), and waits for the result.  It calls no cudaMalloc,
 * cudaFree or allocating library routine: its scratch is a fixed device array in
 * the library (about 32 KB per GPU, held until exit), sized for at most
 * EQF_NOALLOC_MAX_NODES nodes; larger fields return EQF_ERR_TOO_LARGE.  The first
 * call on each device looks up the array's device address (cudaGetSymbolAddress);
 * make that first call before any stream capture.  Every call waits on `stream` for
 * its result (cudaStreamSynchronize) and copies it into *out.  All calls share the
 * array: calls that overlap on the GPU race, so serialise them. */
#define EQF_NOALLOC_MAX_NODES 8388608
int eqf_field_integral_noalloc(const double* d_field, int32_t nx, int32_t ny, double width,
                               double height, int32_t what, double scale, void* stream,
                               double* out);

#ifdef __cplusplus
}
#endif

#endif /* EQFIELD_H */
