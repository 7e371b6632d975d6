/*
 * lvgpu.h — C ABI of the GB300 implementation of the Lagrangian Voronoi
 * per-timestep path (LagrangianVoronoi.jl).
 *
 * One opaque context (`lv_ctx`) holds one VoronoiGrid: the domain, the cell
 * list, the particle state in device memory (SoA, FP64) and the pressure
 * solver.  Every call is ordered on the context's CUDA stream.  Calls that
 * return host data, or that are documented as synchronising, wait for the
 * stream; the others return as soon as their kernels are queued, and their
 * failures (NaN velocity, destroyed mesh, ...) are reported by the next
 * synchronising call or by lv_status().
 *
 * Return values: 0 on success, otherwise one of the LV_ERR_* codes;
 * lv_last_error() gives a message.  Particle indices are 0-based; boundary
 * labels keep the reference's values (BDARY_UP=-1, RIGHT=-2, DOWN=-3,
 * LEFT=-4, src/polygon.jl:4-7).
 *
 * Threading: one context per host thread; calls on one context are not
 * reentrant.  Host pointers are borrowed only for the duration of a call.
 */
#ifndef LVGPU_H
#define LVGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define LV_OK 0
#define LV_ERR_NAN_VELOCITY 1      /* move.jl:24-26 "Velocity field invalidated." */
#define LV_ERR_MESH_DESTROYED 2    /* voronoigrid.jl:63-65 "The Voronoi Mesh has been destroyed." */
#define LV_ERR_EDGE_OVERFLOW 3     /* a polygon needed more than LV_MAX_EDGES edges */
#define LV_ERR_CELL_OVERFLOW 4     /* more cell-list entries than the capacity */
#define LV_ERR_CG_MAXITER 5        /* a pressure solve stopped at itmax (reported in stats) */
#define LV_ERR_BAD_ARGUMENT 6
#define LV_ERR_CUDA 7
#define LV_ERR_NOT_MESHED 8
#define LV_ERR_LEARNED_WORSE 9     /* learned preconditioner fell back to Jacobi */
#define LV_ERR_NONFINITE_POSITION 10
#define LV_ERR_BARRIER_TIMEOUT 11  /* a grid barrier in a persistent kernel gave up */

/* maximum number of edges a Voronoi polygon may have at any time */
#define LV_MAX_EDGES 20

/* boundary labels (src/polygon.jl:4-7) */
#define LV_BDARY_UP (-1)
#define LV_BDARY_RIGHT (-2)
#define LV_BDARY_DOWN (-3)
#define LV_BDARY_LEFT (-4)

/* fields of the polygon state (src/celldefs.jl:7-41, PolygonNS);
 * vector fields are [n][2], D is [n][4] column-major (D11 D21 D12 D22),
 * phase is passed as doubles holding small integers. */
enum lv_field {
  LV_FIELD_X = 0, LV_FIELD_V = 1, LV_FIELD_E = 2, LV_FIELD_P = 3, LV_FIELD_RHO = 4, LV_FIELD_C2 = 5,
  LV_FIELD_DV = 6, LV_FIELD_MASS = 7, LV_FIELD_MOMENTUM = 8, LV_FIELD_ENERGY = 9, LV_FIELD_PHASE = 10,
  LV_FIELD_QUALITY = 11, LV_FIELD_D = 12, LV_FIELD_MU = 13,
  /* PolygonNSF (celldefs.jl:49-56): temperature, heat conductivity k, specific heat cV */
  LV_FIELD_T = 14, LV_FIELD_K = 15, LV_FIELD_CV = 16,
  /* read-only geometry derived by lv_remesh */
  LV_FIELD_AREA = 20, LV_FIELD_CENTROID = 21
};

/* pressure solver methods */
enum lv_method {
  LV_METHOD_JACOBI_PCG = 0,   /* FP64 Jacobi-preconditioned CG (the fallback, and the plain solver the others are measured against) */
  LV_METHOD_MIXED_IR = 1,     /* FP32 CG inner solves inside FP64 iterative refinement */
  LV_METHOD_LEARNED_PCG = 2,  /* mixed IR preconditioned by the learned sparse factor */
  LV_METHOD_MINRES = 3        /* the reference's solve: FP64 MINRES without a preconditioner, stopping at
                                 ||r|| <= tol + tol ||r0|| (Krylov.jl minres!, atol = rtol = tol,
                                 pressure.jl:219), warm-started from P in every sweep */
};

typedef struct lv_params {
  double xmin[2], xmax[2];   /* boundary rectangle (Rectangle, geometry.jl:94-111) */
  double dr;                 /* resolution */
  double h;                  /* cell-list cell size; <= 0 selects the reference default 2dr */
  double r_max;              /* maximum neighbour distance; <= 0 selects the default 10dr */
  int32_t xperiodic, yperiodic;
  int32_t capacity;          /* maximum number of particles */
  int32_t device;            /* CUDA device ordinal */
} lv_params;

typedef struct lv_solve_stats {
  int32_t iterations;        /* CG iterations (inner iterations for mixed IR) */
  int32_t converged;         /* 1 if ||b - A x|| <= tol ||b|| was reached */
  int32_t outer;             /* refinement steps (mixed IR / learned) */
  int32_t method;            /* method actually used */
  double rel_residual;       /* final ||b - A x|| / ||b||, recomputed in FP64 */
} lv_solve_stats;

typedef struct lv_ctx lv_ctx;

/* VoronoiGrid{T}(rect, dr; h, r_max, xperiodic, yperiodic)
 * (src/voronoigrid.jl:14-50).  Returns NULL on failure. */
lv_ctx* lv_create(const lv_params* params);
int lv_destroy(lv_ctx* ctx);
const char* lv_last_error(const lv_ctx* ctx);
/* Pending device status (LV_OK or an LV_ERR_* code); synchronises. */
int lv_status(lv_ctx* ctx);
int lv_synchronize(lv_ctx* ctx);

/* Replaces the particle set: `push!(grid.polygons, T(x = x))` for n seeds
 * (src/populate.jl); x is [n][2].  Other fields are zeroed. */
int lv_set_positions(lv_ctx* ctx, int32_t n, const double* x);
int32_t lv_num_particles(const lv_ctx* ctx);
/* Upload / download one field of all n particles (see lv_field). */
int lv_set_field(lv_ctx* ctx, int32_t field, const double* host);
int lv_get_field(lv_ctx* ctx, int32_t field, double* host);
/* Several fields in one call with one synchronisation (fields[count],
 * host arrays data[count] laid out as for lv_set_field / lv_get_field). */
int lv_set_fields(lv_ctx* ctx, int32_t count, const int32_t* fields, const double* const* data);
int lv_get_fields(lv_ctx* ctx, int32_t count, const int32_t* fields, double* const* data);
/* Device pointer of a field (for zero-copy interop); NULL if unknown. */
void* lv_field_device_ptr(lv_ctx* ctx, int32_t field);

/* remesh!(grid) (src/voronoigrid.jl:89-108): re-bins every seed and rebuilds
 * every Voronoi polygon by half-plane clipping, then orders its edges
 * (sort_edges!, src/IO.jl:35-48).  Synchronises and returns the status. */
int lv_remesh(lv_ctx* ctx);
/* Same, without the final synchronisation (status via lv_status). */
int lv_remesh_async(lv_ctx* ctx);

/* Geometry of the last remesh.  nedges[n]; verts[n][LV_MAX_EDGES][4]
 * (v1x v1y v2x v2y) and labels[n][LV_MAX_EDGES] in the polygon's edge order;
 * any pointer may be NULL. */
int lv_get_geometry(lv_ctx* ctx, int32_t* nedges, double* verts, int32_t* labels);
/* Interior faces in `neighbors(p, grid)` order (src/iterators.jl:23-33):
 * rowptr[n+1]; nbr, lrr = lr_ratio(x-y, e), mid = midpoint(e), y = p.x +
 * get_arrow(q.x, p.x), len = len(e).  Returns the face count through *nfaces
 * when the arrays are NULL. */
int lv_get_faces(lv_ctx* ctx, int64_t* nfaces, int64_t* rowptr, int32_t* nbr, double* lrr, double* mid, double* y,
                 double* len);
/* Cell list: starts[ncells+1] and items (particle indices in insertion order);
 * ncells = n1*n2 (column-major, neighborlist.jl:11-44). */
int lv_get_cell_list(lv_ctx* ctx, int64_t* ncells, int64_t* nitems, int32_t* starts, int32_t* items);

/* Physics steps — names and arguments follow the reference's exports. */
int lv_move(lv_ctx* ctx, double dt);                                   /* move!  (move.jl:9-21), remeshes */
int lv_ideal_eos(lv_ctx* ctx, double gamma, double Pmin);              /* ideal_eos!  (pressure.jl:49-55) */
int lv_stiffened_eos(lv_ctx* ctx, double gamma, double P0);            /* stiffened_eos! (pressure.jl:64-70) */
int lv_find_rho(lv_ctx* ctx);                                          /* find_rho! (pressure.jl:36-40) */
int lv_gravity_step(lv_ctx* ctx, double gx, double gy, double dt);     /* gravity_step! (pressure.jl:77-82) */
int lv_pressure_step(lv_ctx* ctx, double dt);                          /* pressure_step! (pressure.jl:10-25) */
int lv_find_D(lv_ctx* ctx);                                            /* find_D! (diffusion.jl:8-19) */
int lv_viscous_step(lv_ctx* ctx, double dt, int32_t artificial_viscosity); /* viscous_step! (diffusion.jl:39-53) */
/* bdary_friction!(grid, vDirichlet, dt) (diffusion.jl:64-79) with a constant
 * wall velocity per boundary label: vwall[4][2] indexed by -label-1. */
int lv_bdary_friction(lv_ctx* ctx, const double* vwall, double dt);
int lv_find_dv(lv_ctx* ctx, double dt, double alpha);                 /* find_dv! (relaxation.jl:10-25) */
/* viscous_step!(solver::ViscousSolver, dt) (viscous_solver.jl:43-129): the
 * implicit viscous step, (m/dt) v_new - sum_j 0.5 lrr (mu_i + mu_j)(v_j - v_i)
 * = (m/dt) v, both components together solved by MINRES with atol = rtol =
 * 1e-6, itmax = 2000; stats may be NULL (when given, the call synchronises). */
int lv_viscous_solve(lv_ctx* ctx, double dt, lv_solve_stats* stats);
/* Navier-Stokes-Fourier (fourier.jl), on LV_FIELD_T, LV_FIELD_K, LV_FIELD_CV:
 * ideal_temperature!(grid): T = (e - v.v/2) / cV; fourier_step!(grid, dt):
 * e -= dt k_ij / m lrr (T_i - T_j); heat_from_bdary!(grid, dt, T_bc, gamma)
 * with T_bc(midpoint(e), e.label) evaluated per boundary edge by the caller
 * (the order of lv_get_boundary_edges; NaN for an adiabatic edge).  A
 * boundary polygon with cV <= 0 (the reference asserts cV > 0) is reported
 * as LV_ERR_BAD_ARGUMENT by the next synchronising call. */
int lv_ideal_temperature(lv_ctx* ctx);
int lv_fourier_step(lv_ctx* ctx, double dt);
int lv_heat_from_bdary_edges(lv_ctx* ctx, int64_t nb, const double* T_bc, double gamma, double dt);
int lv_relaxation_step(lv_ctx* ctx, double dt, int32_t rusanov);      /* relaxation_step! (relaxation.jl:36-73), remeshes */

/* PressureSolver(grid) options (pressure.jl:142-159): method, tolerance and
 * iteration cap.  The CG methods stop at ||b - A x|| <= tol ||b||; MINRES
 * at the reference's test.  The reference's PressureSolver is
 * LV_METHOD_MINRES, tol 1e-6, itmax 1000, which a new context starts with. */
int lv_set_solver(lv_ctx* ctx, int32_t method, double tol, int32_t itmax);
/* find_pressure!(solver, dt, niter; boundary_velocity) (pressure.jl:215-224).
 * vbc[4][2] (constant boundary velocity per label) may be NULL (zero_vbc).
 * niter <= 31.  stats[niter] may be NULL; when given, the call synchronises. */
int lv_find_pressure(lv_ctx* ctx, double dt, int32_t niter, const double* vbc, lv_solve_stats* stats);
/* Boundary edges of the last remesh, as boundaries(p) yields them
 * (iterators.jl:46-57) over the polygons in index order: *nb, their
 * midpoints mid[nb][2] = midpoint(e) (geometry.jl:145-147) and labels[nb]
 * (-1..-4); with mid and labels NULL only *nb.  Synchronises. */
int lv_get_boundary_edges(lv_ctx* ctx, int64_t* nb, double* mid, int32_t* labels);
/* find_pressure!(solver, dt, niter; boundary_velocity) with the velocity
 * given per boundary edge: vb[nb][2] = boundary_velocity(midpoint(e),
 * e.label) in the order of lv_get_boundary_edges (pressure.jl:182), nb its
 * count.  The host evaluates the reference's closure at those midpoints. */
int lv_find_pressure_edges(lv_ctx* ctx, double dt, int32_t niter, int64_t nb, const double* vb,
                           lv_solve_stats* stats);
/* bdary_friction!(grid, vDirichlet, dt; charfun) per boundary edge
 * (diffusion.jl:64-79): vb[nb][2] = vDirichlet(m) and active[nb] =
 * charfun(m) (NULL: every edge) at the midpoints of lv_get_boundary_edges. */
int lv_bdary_friction_edges(lv_ctx* ctx, int64_t nb, const double* vb, const uint8_t* active, double dt);
/* Pieces of find_pressure! for inspection: PressureOperator refresh!
 * (pressure.jl:104-117) into the device CSR; solver refresh! (pressure.jl:162-203). */
int lv_pressure_operator(lv_ctx* ctx, double dt);
int lv_pressure_rhs(lv_ctx* ctx, double dt, int32_t gp_step, const double* vbc);
/* Export of the assembled system: diag[n] (the reference's diagonal term),
 * rowptr[n+1], col[nnz], w[nnz] (off-diagonal weights w_ij), b[n]; with NULL
 * arrays only *nnz is returned. */
int lv_export_system(lv_ctx* ctx, int64_t* nnz, double* diag, int64_t* rowptr, int32_t* col, double* w, double* b);
/* Solve A x = b on the current operator with the current method; b and x are
 * host arrays of n doubles, x holds the initial guess on entry.  Returns
 * LV_ERR_CG_MAXITER when the solve stopped above the tolerance (x then holds
 * the last iterate). */
int lv_solve(lv_ctx* ctx, const double* b, double* x, lv_solve_stats* stats);
/* y = A x on the current operator (host arrays). */
int lv_operator_apply(lv_ctx* ctx, const double* x, double* y);

/* FP64 Jacobi-PCG on a system the caller already holds in device memory,
 * without allocating anything.  No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc, such as hosts that reserve the
 * whole device memory for their own allocator up front, or time-step loops
 * that must not stall, since cudaMalloc synchronises the device and can take
 * milliseconds.
 * Inputs (device pointers): the reference's operator in the form
 * lv_export_system returns, diag[n], rowptr[n+1] (int32), col[nnz], w[nnz],
 * and b[n]; x[n] holds the initial guess on entry and the solution on return.
 * The solver's scratch is a static device array sized for at most
 * LV_NOALLOC_MAX_ROWS rows (about 24 MiB, held by every GPU that loads the
 * library until exit); larger n returns LV_ERR_BAD_ARGUMENT.  The first call
 * on a device looks up the array's device address, so make that first call
 * before anything that forbids such a lookup.  Every call shares the array,
 * so calls that overlap on the GPU race; run them on one stream.  With
 * iterations and rel_residual both NULL the call only queues work on
 * `stream` (a cudaStream_t, NULL = default stream); otherwise it waits for it
 * and returns LV_OK when ||b - A x|| <= tol ||b||, else LV_ERR_CG_MAXITER. */
#define LV_NOALLOC_MAX_ROWS 524288
int lv_pcg_solve_noalloc(int32_t n, const double* diag, const int32_t* rowptr, const int32_t* col, const double* w,
                         const double* b, double* x, double tol, int32_t itmax, void* stream, int32_t* iterations,
                         double* rel_residual);

/* Learned preconditioner (LV_METHOD_LEARNED_PCG).  A 3-layer message-passing
 * network (hidden width 32, BF16 tensor-core matrix products, FP32
 * accumulation) maps the assembled operator to a sparse factor G on the
 * pattern of its lower triangle; the inner CG of the mixed-precision solver
 * is preconditioned by M^-1 = D^-1/2 (G^T G + eps I) D^-1/2 (SPD).  The
 * network is trained on systems snapshot from the solver itself by
 * hand-written forward/backward kernels and Adam, minimising a stochastic
 * estimate of ||G A~ G^T - I||_F^2 / n (A~ = D^-1/2 A D^-1/2).  A learned
 * solve that needs more iterations than the last Jacobi solve falls back to
 * Jacobi (stats.method reports the method used). */
int lv_learn_init(lv_ctx* ctx, uint64_t seed);                  /* random initialisation */
int32_t lv_learn_num_params(void);
int lv_learn_get_params(lv_ctx* ctx, float* out);
int lv_learn_set_params(lv_ctx* ctx, const float* in);
int lv_learn_add_system(lv_ctx* ctx);                          /* snapshot the assembled operator */
int32_t lv_learn_num_systems(lv_ctx* ctx);
int lv_learn_clear_systems(lv_ctx* ctx);
/* Adam on the snapshot systems (round robin); losses[steps] may be NULL.
 * probes = 0: the exact FSAI (Kaporin) objective (1/n)[tr(Gt At Gt^T) -
 * 2 sum log Gt_ii]; probes = K in 1..8: a Hutchinson estimate of
 * ||Gt At Gt^T - I||_F^2 / n with K Rademacher probes per step. */
int lv_learn_train(lv_ctx* ctx, int32_t steps, float lr, int32_t probes, uint64_t seed, float* losses);
/* Loss and gradient for system `sys` (< 0: the assembled operator): K = 0 the
 * FSAI (Kaporin) objective, K >= 1 the Hutchinson loss with the given
 * probes[K][n] or Rademacher probes from seed; grad[num_params] may be NULL. */
int lv_learn_loss_grad(lv_ctx* ctx, int32_t sys, const float* probes, int32_t K, uint64_t seed, double* loss,
                       float* grad);
/* Pattern of the learned factor: hops = 1, the operator's lower triangle (the
 * default); hops = 2, also the lower neighbours at distance two (their entries
 * Gt_ij = pw_ij sum ro2 H_i H_j with the path weight pw_ij).  The two-hop
 * pattern trains with the FSAI objective only (probes = 0). */
int lv_learn_set_pattern(lv_ctx* ctx, int32_t hops);
int32_t lv_learn_get_pattern(lv_ctx* ctx);
/* Two-hop part of the factor of the assembled operator: rowptr2[n+1],
 * col2[nnz2] (both triangles) and g2[nnz2] (lower entries, zero elsewhere);
 * with NULL arrays only *nnz2 is returned. */
int lv_learn_factor2(lv_ctx* ctx, int64_t* nnz2, int64_t* rowptr2, int32_t* col2, float* g2);
/* Factor of the assembled operator: gdiag[n], glower[nnz] (CSR positions with
 * col < row, zero elsewhere) and the node features[n][16]; any may be NULL. */
int lv_learn_factor(lv_ctx* ctx, float* gdiag, float* glower, float* features);

/* MultiphaseSolver / multiphase_projection! (relaxation.jl:137-206). */
int lv_multiphase_projection(lv_ctx* ctx, double quality_threshold, lv_solve_stats* stats);

/* Post-processing on the current mesh (host arrays in and out).
 * nearest_polygon (voronoigrid.jl:154-178): out[m] = 0-based index of the
 * nearest seed of each points[m][2] (-1 when the cell path meets none). */
int lv_nearest_polygon(lv_ctx* ctx, int32_t m, const double* points, int32_t* out);
/* movingls (movingls.jl:52-86) with gaussian_kernel: Taylor coefficients of
 * the per-polygon values[n] at polygons polys[m] (NULL: all, m = n), order 1
 * linear (2 coefficients), 2 quadratic (5), 3 cubic (9), moving radius h;
 * coeffs[m][2|5|9] in power_vector order (movingls.jl:26-36). */
int lv_movingls(lv_ctx* ctx, int32_t order, int32_t m, const int32_t* polys, const double* values, double h,
                double* coeffs);
/* point_value (movingls.jl:140-146): values[n] interpolated at points[m][2]
 * from the nearest polygon's linear expansion (h = cell size). */
int lv_point_value(lv_ctx* ctx, int32_t m, const double* points, const double* values, double* out);

/* The CUDA stream (cudaStream_t) every call of this context is ordered on;
 * callers may record events or enqueue their own work on it. */
void* lv_stream(lv_ctx* ctx);

/* Kernel families timed by lv_kernel_timing. */
#define LV_KF_BIN 0      /* cell-list re-binning (count, scan, scatter, order) */
#define LV_KF_CLIP 1     /* Voronoi clipping + geometry + faces (k_clip) */
#define LV_KF_PCG 2      /* persistent pressure-solve kernels */
#define LV_KF_RHS 3      /* operator assembly, right-hand side and initial guess of each sweep */
#define LV_KF_OPS 4      /* per-particle physics operators */
#define LV_KF_LEARN 5    /* learned factor of the assembled operator (network forward, M^-1) */
#define LV_KF_COUNT 6
/* When enabled, every launch of every family is bracketed by CUDA events on
 * the context's stream (no synchronisation).  lv_kernel_time synchronises
 * and returns, for one family, the launches and total device ms since the
 * last reset (reset != 0 clears the family). */
int lv_kernel_timing(lv_ctx* ctx, int32_t enable);
int lv_kernel_time(lv_ctx* ctx, int32_t family, int64_t* launches, double* ms, int32_t reset);
/* Cumulative pressure-solver counters since creation: linear solves and CG
 * iterations (inner iterations for the mixed-precision solver); synchronises. */
int lv_solver_counters(lv_ctx* ctx, int64_t* solves, int64_t* iterations);
/* The persistent solvers wait on one another's blocks (grid phases,
 * neighbour exchanges); every such wait gives up after `cycles` GPU clock
 * cycles (<= 0 restores the default, about 2 s), and the call then reports
 * LV_ERR_BARRIER_TIMEOUT, leaving the context usable: the next solve clears
 * the solvers' synchronisation words, and the sweep guess forgets its
 * history.  No counterpart in the reference (its threads never wait on a
 * GPU); a test lowers the limit to make a wait run out. */
int lv_set_wait_limit(lv_ctx* ctx, int64_t cycles);
/* Cumulative count of linear solves (pressure sweeps, lv_solve) that ended
 * with a recursive or true residual above tol ||b|| (itmax reached, or a
 * non-finite residual); synchronises.  lv_find_pressure without stats queues
 * its sweeps and returns at once, so a caller that does not ask for stats
 * reads this count (e.g. once after a run of steps) to learn that every
 * sweep converged.  No counterpart in the reference, whose find_pressure!
 * leaves Krylov's statistics unread (pressure.jl:219-220). */
int lv_solver_unconverged(lv_ctx* ctx, int64_t* solves);
/* Diagnostic of the learned solve for systems that fit one block per SM:
 * the largest halo (rows outside a block that the block's rows reference)
 * over the blocks of the last built factor, or 0 when that solve moves
 * M^-1 r between blocks instead of computing it on the halo (halo mode off
 * through LVGPU_FCG_HALO=0, a halo above 1536 rows, or a larger system);
 * synchronises. */
int lv_solver_halo(lv_ctx* ctx, int32_t* max_rows);
/* The sweeps of lv_find_pressure start from a Galerkin guess that uses the
 * previous call's change of each sweep (LVGPU_SWEEP_GUESS=0 turns the guess
 * off).  lv_solver_forget forgets that history, e.g. after the state was
 * replaced (a restart from a checkpoint): the next call starts like the first. */
int lv_solver_forget(lv_ctx* ctx);
/* Polygons of the last remesh that outgrew the first clipping pass's edge
 * slots and were finished by the second pass (LVGPU_CLIP_SLOTS=5..8 lowers
 * the first pass's slots, so that tests can drive most polygons through the
 * second pass); synchronises. */
int lv_mesh_captures(lv_ctx* ctx, int32_t* count);

/* Per-kernel-family device times in ms accumulated since the last reset:
 * out[0] mesh, [1] operators, [2] pressure solve, [3] other.  Returns the
 * number of entries written. */
int lv_get_timings(lv_ctx* ctx, double* out, int32_t cap);
int lv_reset_timings(lv_ctx* ctx);
/* Number of kernel launches issued by the context since creation. */
int64_t lv_launch_count(const lv_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* LVGPU_H */
