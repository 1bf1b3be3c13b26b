/*
 * wedg.h -- C ABI of libwedg, the GB300 (sm_103a, FP64) right-hand side and
 * RK4 step of the energy-based DG scheme of WesterveltEDG.jl (v0.3.0).
 *
 * The library is a drop-in for the reference's hot path: a GPU workspace
 * replaces `Workspace(pre, N)` (src/rhs.jl:184), and the calls below replace
 * `edg_rhs!` (src/rhs.jl:490-494), `rk4_step!` (src/solver.jl:289-297) and the
 * step loop of `solve` (src/solver.jl:213-217). `pre` stays the reference's
 * own host data (`precompute`, src/solver.jl:428-694): `wedg_create` reads its
 * arrays through host pointers in the reference's (Julia, column-major)
 * layouts and copies what the device needs.
 *
 * Conventions
 *  - All arithmetic is FP64.
 *  - Status codes mirror the reference's exceptions (wedg_status); the exact
 *    message text of the reference is available from wedg_error_message.
 *  - State arrays u (N,N,q_u+1,q_u+1) and v (N,N,q_v+1,q_v+1) use the
 *    reference's state layout (column-major, element index j + N*k fastest).
 *    `where` says whether the pointers are host (WEDG_HOST: the library
 *    copies in and out) or device (WEDG_DEVICE) memory.
 *  - Every call is synchronous, like the reference's, and one workspace must
 *    not be used from two threads at once.
 */
#ifndef WEDG_H
#define WEDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum wedg_status {
  WEDG_OK = 0,
  WEDG_ERR_DIMENSION = 1,          /* DimensionMismatch, src/rhs.jl:500-503 */
  WEDG_ERR_BOUNDARY_WEIGHT = 2,    /* 1 - kβv ≤ 0 at a face point, src/rhs.jl:112-116, 768-776 */
  WEDG_ERR_MASS_NOT_PD = 3,        /* 1 - 2βv_h ≤ 0, src/rhs.jl:916 (Chebyshev), :845 (CG) */
  WEDG_WARN_CG_NOT_CONVERGED = 4,  /* the @warn of src/rhs.jl:855-859; outputs are valid */
  WEDG_ERR_TIMEOUT = 5,            /* a bounded device wait gave up */
  WEDG_ERR_CUDA = 6,               /* CUDA runtime error */
  WEDG_ERR_ARGUMENT = 7,           /* invalid argument (the reference's argument ErrorExceptions) */
  WEDG_ERR_NO_DEVICE = 8           /* no usable GPU */
};

enum wedg_kind { WEDG_ABSORBING_2BETA = 0, WEDG_ABSORBING = 1, WEDG_DIRICHLET = 2, WEDG_WALL = 3 };
enum wedg_where { WEDG_HOST = 0, WEDG_DEVICE = 1 };
enum wedg_mass_solver { WEDG_CHEBYSHEV = 0, WEDG_CG = 1 };
enum wedg_cheb_steps { WEDG_CHEB_PER_ELEMENT = 0, WEDG_CHEB_COMMON_MAX = 1 };

/* Scalars of `pre` (src/solver.jl:665-689) and the per-side boundary table
 * `pre.bc` (src/solver.jl:39-45), sides in the order bot, top, lft, rgt. */
typedef struct wedg_config {
  int32_t N, qu1, qv1, q_high;
  double theta, tau, lambda_u, lambda_v; /* flux parameters, src/solver.jl:16-21 */
  double omega;                          /* 2π √(kx² + ky²) */
  int32_t mms_on, src_on, one_sided;     /* mode flags and the face kernel choice */
  int32_t mass_solver;                   /* wedg_mass_solver */
  double mass_tol;                       /* 1e-14 in the reference */
  double src_omega, src_Ts;              /* GaussianSource ω and Ts of src_time (src/solver.jl:662) */
  int32_t kind[4];                       /* wedg_kind per side */
  double gamma_abc[4], eta_abc[4], sigma[4], kb[4], kappa[4];
  int32_t cheb_steps;                    /* wedg_cheb_steps: per-element count (default) or the
                                            reference's common maximum (src/rhs.jl:911-918) */
  int32_t general_only;                  /* 1: never use the constant-coefficient kernels */
  int32_t point_traces;                  /* 1: keep the traces at the face points; 0: as modal end sums
                                            where every interior face's coefficients are one value along
                                            it (wedg_stats.modal_traces) */
} wedg_config;

/* Host pointers to the arrays of `pre`, each in the reference's layout
 * (src/solver.jl:462-536, 716-770). Ainv_u may be NULL: when every element has
 * constant c² and α the library uses the exact fast diagonalization of the
 * pinned stiffness and never needs it; otherwise wedg_create computes the packed
 * inverses of src/solver.jl:528-535 on the device from Cw (and fails with
 * WEDG_ERR_ARGUMENT if a stiffness matrix is not positive definite).
 * wedg_rhs_noalloc needs Ainv_u for coefficients that vary inside elements. */
typedef struct wedg_pre {
  const double *w, *P_u, *S_u, *Ebl_u, *Ebr_u, *E1bl_u, *E1br_u;
  const double *P_h_v, *W2d_h;
  const double *Cw, *Aw, *Ainv_u;
  const double *hc2, *haf, *hcf, *hbf, *vc2, *vaf, *vcf, *vbf;
  const double *hc2m, *hafm, *vc2m, *vafm, *hJC, *vJC;
  const double *bcB_sp, *bcB_spy, *bcT_sp, *bcT_spy, *bcL_sp, *bcL_spx, *bcR_sp, *bcR_spx;
  const double *PiSP, *PiBSP2, *PiCdiv, *PiDdiv, *src_projE;
  const double *beta_hq;
} wedg_pre;

/* Per-call statistics of the last call. */
typedef struct wedg_stats {
  int32_t cheb_steps_max;      /* largest Chebyshev step count of the last evaluation */
  int32_t cg_not_converged;    /* element systems above the CG tolerance (summed over stages) */
  int32_t finite;              /* after an RK4 step: all entries of u and v finite (`all(ws.fin)`) */
  int32_t fast_path;           /* 1 if the constant-coefficient kernels are in use */
  int64_t steps_done;          /* RK4 steps completed by the last wedg_rk4_steps */
  int64_t kernel_launches;     /* kernels launched by the last call */
  int64_t device_bytes;        /* device memory held by the workspace */
  int64_t cheb_steps_sum;      /* Σ over elements and stages of the Chebyshev step counts */
  int64_t element_stages;      /* elements × stages evaluated by the last call */
  int32_t modal_traces;        /* 1 if the traces are kept as modal end sums and the interior flux
                                  slots projected in that form (every interior face's coefficients
                                  one value along the face; jump terms projected on the face modes
                                  once); the adjoint calls use point traces */
  int32_t reserved;
} wedg_stats;

typedef struct wedg_ws wedg_ws;

/* Workspace(pre, N) of src/rhs.jl:184-220: validates the configuration,
 * copies pre to the device and allocates all scratch. Replaces the CPU
 * workspace; there is no nblocks (the GPU grid replaces the element blocks). */
int wedg_create(const wedg_config *cfg, const wedg_pre *pre, wedg_ws **out);
void wedg_destroy(wedg_ws *ws);

/* The same workspace with `pre`'s large arrays built on the device (no counterpart in the reference,
 * whose precompute, src/solver.jl:428-770, builds them on the host). The caller evaluates the
 * coefficient functions at the point grids and passes those values; the device then forms what
 * precompute forms from them: the element matrices c²W, αW (or the constant-coefficient data) and
 * their packed inverses, the one-sided face values of c, α, β with the reference's jump test
 * (src/solver.jl:371-408, step δ = 2^-40, tolerance 1e-8 plus jump_scale), the face arrays and jump
 * terms of _rhs_data (:698-770), the projections Π and the source projection (:647-662, 762-764),
 * and 2β at the mass points. From `pre` only the 1D operators (w ... W2d_h) and the boundary data
 * (bcB_sp ... bcR_spx) are read. The one-sided face kernel is chosen from the device's jump test
 * (wedg_one_sided reports it). On an error, msg (if not NULL) receives the reason, including the
 * reference's refusal of jumping coefficients in :mms mode (src/solver.jl:745-747). */
typedef struct wedg_face_values {
  const double *at, *lo, *hi; /* the value at each face point and δ below (left of) and above (right of) it,
                                 the reference's array of one face family: horizontal faces (q_u1, N+1, N),
                                 face row jf at y = jf h; vertical faces (q_u1, N, N+1), face column kf
                                 at x = kf h. The values δ outside the domain are not read: pass the
                                 value at the face there, as the reference does. */
  double jump_scale;          /* the family's s = 1e-8 max|value at ±δ| of src/solver.jl:387 */
  double value;               /* with at = NULL: the family is this constant everywhere */
} wedg_face_values;
/* A coefficient given as its values on an m × n grid of cells of the unit square, row-major
 * [row (y)][column (x)]: the value at (x, y) is values[clip(floor(m y), 0, m-1) n + clip(floor(n x), 0, n-1)]
 * (the lookup of piecewise-constant coefficients; the device evaluates it at every point). */
typedef struct wedg_cell_table {
  const double *values;
  int32_t rows, cols;
} wedg_cell_table;
typedef struct wedg_points {
  const double *c_q, *alpha_q;          /* c and α at the u-points, (N, N, q_u1, q_u1): [j, k, r, s] at
                                           (x_s of column k, y_r of row j) */
  const double *beta_h;                 /* β at the high-order points, (N, N, q_high, q_high) */
  double c_value, alpha_value, beta_value; /* a coefficient whose array is NULL is this constant... */
  wedg_cell_table c_cells, alpha_cells, beta_cells; /* ...unless it has a table: then the device looks it
                                           up at every point, faces and their δ-neighbours included */
  const double *xloc, *yloc;            /* (N, q_u1): the u-points of the columns and rows (needed for tables) */
  wedg_face_values hc, ha, hb;          /* c, α, β on the horizontal faces */
  wedg_face_values vc, va, vb;          /* c, α, β on the vertical faces */
  wedg_face_values hg0, vg0;            /* ∂u0/∂y on the horizontal and ∂u0/∂x on the vertical faces
                                           (src/solver.jl:554-568); unused in source mode */
  const double *sp_h, *cdiv_h, *ddiv_h; /* at the high-order points: Φ and the two divergence terms of the
                                           manufactured solution (mms), the c²-term alone (initial value);
                                           unused in source mode */
  const double *xloc_h, *yloc_h;        /* (N, q_high): the high-order points of the columns and rows */
  double src_amp, src_x0, src_y0, src_r0; /* the GaussianSource's profile (source mode) */
} wedg_points;
int wedg_create_points(const wedg_config *cfg, const wedg_pre *pre, const wedg_points *pts, char *msg, size_t msg_len,
                       wedg_ws **out);
/* 1 if the workspace uses the one-sided face kernel (pre.one_sided), 0 if not. */
int wedg_one_sided(const wedg_ws *ws);
/* A device array of the workspace in the reference's layout of the `pre` array of that name (for checks
 * of the device-built arrays): hc2 haf hcf hbf hc2m hafm hJC and the v-face arrays, PiSP PiBSP2 PiCdiv
 * PiDdiv src_projE, beta_hq; Cw, Aw (general kernels); c2e, ae (c² and α per element, constant-coefficient
 * kernels); tr, the traces of the last evaluation in the device layout [((fam 4 + side) q_u1 + i) E + e]
 * (fam du, v, dv; side B, T, L, R; i a face point, or a mode with wedg_stats.modal_traces). count must be
 * the array's size; arrays the workspace does not hold are refused. */
int wedg_export(const wedg_ws *ws, const char *name, double *out, size_t count);

/* edg_rhs!(ws, u, v, t, N, h, pre) of src/rhs.jl:490-550: ut, vt receive the
 * right-hand side. Shapes are checked as src/rhs.jl:500-503 does. */
int wedg_rhs(wedg_ws *ws, const double *u, const double *v, double t, double *ut, double *vt,
             const int64_t u_shape[4], const int64_t v_shape[4], int where);

/* rk4_step!(u, v, t, dt, N, h, pre, ws) of src/solver.jl:289-321: u, v are
 * updated in place; on an error they are left unchanged. `finite` receives
 * all(ws.fin). */
int wedg_rk4_step(wedg_ws *ws, double *u, double *v, double t, double dt, const int64_t u_shape[4],
                  const int64_t v_shape[4], int where, int *finite);

/* The step loop of solve (src/solver.jl:213-217): nsteps RK4 steps from t0,
 * t advancing by repeated addition of dt. Stops at the first failing step
 * (state left as before that step); `steps_done` receives the completed steps.
 * With stop_nonfinite, it also stops after the first step whose result is not
 * finite (the blow-up check of src/solver.jl:940); `finite` receives the flag
 * of the last completed step. */
int wedg_rk4_steps(wedg_ws *ws, double *u, double *v, double t0, double dt, int64_t nsteps,
                   const int64_t u_shape[4], const int64_t v_shape[4], int where, int stop_nonfinite,
                   int64_t *steps_done, int *finite);

/* Message of the last error in the reference's words (src/rhs.jl:114-115,
 * 845, 916; the DimensionMismatch text of :503). Returns the status. */
int wedg_error_message(const wedg_ws *ws, char *buf, size_t len);

/* Key of the last error: the boundary key of src/rhs.jl:732 for
 * WEDG_ERR_BOUNDARY_WEIGHT, the 1-based element for WEDG_ERR_MASS_NOT_PD. */
int64_t wedg_error_key(const wedg_ws *ws);

int wedg_get_stats(const wedg_ws *ws, wedg_stats *out);

/* Stream used by the workspace (a cudaStream_t). wedg_set_stream makes the
 * workspace launch on the caller's stream (NULL: the library's own). */
void *wedg_get_stream(const wedg_ws *ws);
int wedg_set_stream(wedg_ws *ws, void *stream);

/* Asynchronous form for device-resident runs: enqueue nsteps RK4 steps on
 * the workspace stream without copies, synchronization or error checks;
 * wedg_sync_status then waits and reports like wedg_rk4_steps. */
int wedg_rk4_steps_async(wedg_ws *ws, double *u_dev, double *v_dev, double t0, double dt, int64_t nsteps);
int wedg_sync_status(wedg_ws *ws, int64_t *steps_done, int *finite);

/* Kernel timing for benchmarks: with enable != 0, every launch of the three stage
 * kernels (k_prep, k_stage, and the mass solve k_cheb or k_cg) is bracketed by CUDA events on the workspace
 * stream and its duration accumulated; wedg_kernel_times reads (and with reset,
 * clears) the totals in milliseconds and the number of launches of each. */
int wedg_time_kernels(wedg_ws *ws, int enable);
int wedg_kernel_times(wedg_ws *ws, double *prep_ms, int64_t *prep_launches, double *stage_ms,
                      int64_t *stage_launches, double *mass_ms, int64_t *mass_launches, int reset);

/* Source-mode run with its diagnostics on the device: the loop of `_run_source`
 * (src/solver.jl:892-958). It replaces the per-step host work of that loop -- the
 * receiver values after every step, and after every record_every-th step (and the
 * last) the Westervelt energy, max|v_h|, min(1 - 2βv_h) (src/solver.jl:864-888) and
 * the slice of v_h along y = slice_y -- with kernels on the workspace stream, and
 * takes the snapshots of v_h on the (N q_u1)² point grid after the listed steps.
 * The time t advances by t += dt after every step, as in the reference. The run
 * stops at the first step with a non-finite state (the reference's "blow-up"),
 * reported through steps_done and finite; errors of the RHS as wedg_rk4_steps.
 * Receiver and slice positions are given as the element and the Legendre values
 * at the local coordinate, which the host computes as the reference does
 * (`locate`, `vrow`, src/solver.jl:898-899). Outputs are host arrays. */
typedef struct wedg_source_run {
  int64_t nsteps, record_every;
  double t0, dt;
  int nrec;                        /* receivers */
  const int32_t *rec_j, *rec_k;    /* 0-based element row j (y) and column k (x) of each receiver */
  const double *rec_py, *rec_px;   /* nrec × q_v1 (receiver-major): P_d at the local y and at the local x */
  int slice_j;                     /* 0-based element row of the slice */
  const double *slice_py;          /* q_v1: P_d at the slice's local y */
  int nsnap;                       /* snapshots, after these step counts (1-based, increasing) */
  const int64_t *snap_after;
  const double *err_c2, *err_beta; /* c² and β at the u-quadrature points, (N, N, q_u1, q_u1) column-major */
  double *recv;                    /* out: nsteps × nrec, step-major */
  double *energy, *vmax, *ndmin;   /* out: one per record, ceil(nsteps / record_every) records */
  double *slices;                  /* out: records × N q_u1 */
  double *snaps;                   /* out: nsnap × (N q_u1)², each column-major */
} wedg_source_run;
int wedg_run_source(wedg_ws *ws, double *u, double *v, const int64_t u_shape[4], const int64_t v_shape[4],
                    int where, const wedg_source_run *run, int64_t *steps_done, int *finite);

/* Discrete adjoint of edg_rhs! (no counterpart in the reference): at the state (u, v) and time
 * t, gu and gv receive Jᵀ(λ_u, λ_v), the gradient of λ_u·ut + λ_v·vt with respect to u and v,
 * where (ut, vt) is the right-hand side of src/rhs.jl:490-550. Layouts, `where` and errors as
 * wedg_rhs (the forward RHS at the state is evaluated first and checked). */
int wedg_rhs_adjoint(wedg_ws *ws, const double *u, const double *v, double t, const double *lam_u,
                     const double *lam_v, double *gu, double *gv, const int64_t u_shape[4], const int64_t v_shape[4],
                     int where);

/* Discrete adjoint of the RK4 time stepping (no counterpart in the reference): for nsteps RK4
 * steps from (u0, v0) at t0 (t advancing by t += dt, as wedg_rk4_steps), gu and gv receive the
 * gradient with respect to (u0, v0) of λ_u·u(T) + λ_v·v(T), i.e. the adjoint state at t0 for the
 * final-time adjoint (λ_u, λ_v) -- for a misfit J(u(T), v(T)), pass ∂J/∂u(T), ∂J/∂v(T). The
 * forward states are kept every `every` steps (checkpoints); each segment is run again with its
 * RK4 stage states kept, and the steps are reversed through wedg_rhs_adjoint's transposes at the
 * stage states. Device memory: (nsteps / every + 4 every) states besides the workspace.
 * With g_c2, g_alpha, g_beta (E each, or all NULL) it also returns the gradient with respect to
 * each element's c², α and β, for source-mode runs whose coefficients are constant on every
 * element (the constant-coefficient kernels); a parameter constant on a union of elements has
 * the sum of their entries as its gradient. */
int wedg_rk4_adjoint(wedg_ws *ws, const double *u0, const double *v0, double t0, double dt, int64_t nsteps,
                     int64_t every, const double *lam_u, const double *lam_v, double *gu, double *gv,
                     double *g_c2, double *g_alpha, double *g_beta, const int64_t u_shape[4],
                     const int64_t v_shape[4], int where);

/* The two halves of wedg_rk4_adjoint, for a final-time adjoint that depends on the final
 * state (a misfit): wedg_rk4_adjoint_forward runs the nsteps steps from (u0, v0), keeps the
 * checkpoints in the workspace and returns the final state (uT, vT; either may be NULL);
 * wedg_rk4_adjoint_reverse then takes (λ_u, λ_v) at T and returns the gradients as
 * wedg_rk4_adjoint does. A reverse sweep needs a preceding forward run on the same workspace. */
int wedg_rk4_adjoint_forward(wedg_ws *ws, const double *u0, const double *v0, double t0, double dt, int64_t nsteps,
                             int64_t every, double *uT, double *vT, const int64_t u_shape[4],
                             const int64_t v_shape[4], int where);
int wedg_rk4_adjoint_reverse(wedg_ws *ws, const double *lam_u, const double *lam_v, double *gu, double *gv,
                             double *g_c2, double *g_alpha, double *g_beta, int where);

/* The same two halves for n workspaces at once (no counterpart in the reference), e.g. the
 * gradients of one misfit for n parameter fields: the workspaces need the same degrees,
 * coefficient kernels and mass solver (any meshes); the forward runs take the same t0, dt, steps
 * and checkpoint interval. Every RK4 stage and every stage's transpose runs as one
 * multi-instance launch per kernel over all n workspaces, so that problems too small to fill
 * the GPU alone fill it together; each workspace's arithmetic is the one of its own call. The
 * reverse sweeps keep the stage data of one segment of every workspace at once when the sum fits
 * the allowance (the workspaces' wedg_set_adjoint_memory, or by default half of the free device
 * memory); otherwise they run one after the other. Arrays of n pointers, as the single calls;
 * uT, vT and the parameter gradients may be NULL (or hold NULL entries). Returns the first error
 * of a workspace, whose message is read with wedg_error_message. */
int wedg_rk4_adjoint_forward_many(int n, wedg_ws *const *ws, const double *const *u0, const double *const *v0,
                                  double t0, double dt, int64_t nsteps, int64_t every, double *const *uT,
                                  double *const *vT, int where);
int wedg_rk4_adjoint_reverse_many(int n, wedg_ws *const *ws, const double *const *lam_u, const double *const *lam_v,
                                  double *const *gu, double *const *gv, double *const *g_c2, double *const *g_alpha,
                                  double *const *g_beta, int where);

/* Launch shapes (no counterpart in the reference, whose parallel regions are the nblocks
 * element blocks of src/rhs.jl:130-180): threads per block of k_prep (one element per thread)
 * and of the mass solves (a team of threads per element, so the block's warps set its
 * elements): 32, 64, 96 or 128 each, 128 by default. Results do not depend on them (every
 * element's arithmetic is its own); only the time does. */
int wedg_set_launch_shape(wedg_ws *ws, int prep_threads, int mass_threads);
int wedg_get_launch_shape(const wedg_ws *ws, int *prep_threads, int *mass_threads);

/* Autotuner of the launch shapes: times `steps` RK4 steps (after one untimed step) from copies
 * of the device state (u_dev, v_dev; left unchanged) for 32, 64 and 128 threads per block of
 * k_prep, then of the mass solves, and keeps the fastest (a candidate must gain 2 %). Returns
 * the best time per step in *best_ms (may be NULL). */
int wedg_autotune(wedg_ws *ws, const double *u_dev, const double *v_dev, double t0, double dt, int64_t steps,
                  double *best_ms);

/* (No counterpart in the reference, which has no adjoint.) Device memory the reverse sweep may
 * use to keep, for every stage of one checkpoint segment,
 * the stage's forward data (its right-hand side, traces and mass-solve data) while it
 * recomputes the segment: with it the adjoint of a stage needs no second forward evaluation.
 * bytes < 0 (the default): half of the free device memory at the sweep; 0: never keep (each
 * stage's forward evaluation is repeated); > 0: keep when one segment's data fits in bytes.
 * The gradients agree either way up to rounding. */
int wedg_set_adjoint_memory(wedg_ws *ws, int64_t bytes);

/* Batched form: many independent instances -- workspaces made by wedg_create, each with its
 * own N, degrees, flux, boundary kinds and coefficients -- advanced together. No counterpart in
 * the reference, whose batching is the caller's loop over instances (the element blocks of
 * src/rhs.jl:130-180, 227-252 split one instance). The instances are grouped into buckets that
 * run the same kernels (the same degrees, coefficient kernels, mass solver and 1D operators;
 * any mesh sizes). A bucket runs in one of two layouts (wedg_batch_set_shape): its instances'
 * own launches, each instance on its own stream (the default, the faster on the mixed batches
 * measured), or per stage of an RK4 step k_prep, k_stage and its mass solve as one launch each
 * over all of its instances (up to 31 instances per launch; larger buckets take several), whose
 * blocks each take a tile of one instance's elements. Either way an element's arithmetic is the
 * one of a launch of its instance alone. The buckets run side by side on their own streams. One
 * RK4 step of the whole batch, and four steps in which each instance (or merged bucket) goes on
 * to its next step without waiting for the others, are captured once into CUDA graphs and
 * replayed. The stage kernels of a replay take their time factors from per-instance tables that
 * the host refills every WEDG_BATCH_CHUNK steps (the factors are the ones the single-instance
 * calls compute), at the instance's device step counter. The graphs are captured again when the
 * state pointers, the steps dt, stop_nonfinite or a bucket's launch shape change. */
#define WEDG_BATCH_CHUNK 256
typedef struct wedg_batch wedg_batch;
int wedg_batch_create(int n, wedg_ws *const *instances, wedg_batch **out);
void wedg_batch_destroy(wedg_batch *b);
/* nsteps RK4 steps of every instance i, in place on its device state u_dev[i], v_dev[i] (the
 * reference's layout), from t0[i] with step dt[i] (t advancing by t += dt). With
 * stop_nonfinite, an instance stops after its first step with a non-finite state. Per
 * instance: steps_done[i], finite[i] and status[i] (a status of wedg_rk4_steps; the message
 * through wedg_error_message on that instance); any of the three may be NULL. Returns WEDG_OK
 * or the first nonzero instance status. */
int wedg_batch_rk4_steps(wedg_batch *b, double *const *u_dev, double *const *v_dev, const double *t0,
                         const double *dt, int64_t nsteps, int stop_nonfinite, int64_t *steps_done, int *finite,
                         int *status);

/* The buckets of a batch and their launch shapes: the elements per block of k_prep (its threads,
 * one element each) and of the mass solves (threads / 32 warps of teams of threads per
 * element), 32, 64, 96 or 128 threads, and `persist`: 0 launches one block per tile, p > 0 a
 * persistent grid of p times the blocks the SMs hold at once, each block taking tile after
 * tile; -1 (the default) launches the bucket's instances one by one instead (the single-instance
 * kernels, each instance on its own stream). Results do not depend on the shape (every element's
 * arithmetic is its own). */
typedef struct wedg_batch_shape {
  int32_t qu1, qv1, instances, fast;   /* the bucket's degrees + 1, its instances, the kernel family */
  int32_t prep_threads, mass_threads, persist;
} wedg_batch_shape;
int wedg_batch_bucket_count(const wedg_batch *b);
int wedg_batch_get_shape(const wedg_batch *b, int bucket, wedg_batch_shape *out);
int wedg_batch_set_shape(wedg_batch *b, int bucket, int prep_threads, int mass_threads, int persist);

/* Autotuner of the batch's launch shapes (no counterpart in the reference, whose only shape is the
 * nblocks partition of src/rhs.jl:139-142): per bucket, run alone from copies of its instances'
 * states (left unchanged), steps RK4 steps after one untimed step, timed with CUDA events, for the
 * candidates of one coordinate at a time (persist: -1, 0, 1, 2; then k_prep's and the mass
 * solves' threads per block: 32, 64, 128). A candidate replaces the bucket's shape only when it is faster in
 * each of three paired trials against it and faster by more than 2 % in the median. Then the
 * whole batch's step (graph replays over at least 8 steps) with the tuned shapes against the
 * shapes it had before, three paired trials: the tuned shapes stay only if they win every trial
 * and gain more than 2 % in the median, so the batch does not end up slower than before tuning. *best_ms (may be NULL) receives the
 * median milliseconds per step of the shapes kept. */
int wedg_batch_autotune(wedg_batch *b, double *const *u_dev, double *const *v_dev, const double *t0,
                        const double *dt, int64_t steps, double *best_ms);

/* Error norms on the device (src/solver.jl:774-836). With uB = vB = NULL: `_mms_errors`, the
 * L² errors of the state A against the manufactured solution u = cos(ωT)Φ (the solver stores
 * u - Φ, so A is compared with (cos(ωT) - 1)Φ), Φ = cos(2πkx x + px) sin(2πky y + py) at the
 * points (xloc, yloc); otherwise `difference_norms`, the norms of A - B. out = {erru, errv,
 * errgradu, errE}, each (h/2)·sqrt(Σ over elements and points of W2d times the squared
 * difference), errE with ½c²|∇e_u|² + ½e_v². States in the reference's layout, host or device
 * memory (where); the other arrays host memory. */
typedef struct wedg_norm_args {
  int N, qu1, qv1;
  const double *w;                  /* q_u1 weights of the u-quadrature */
  const double *P_u, *S_u;          /* (q_u1, q_u1) column-major: P_u[i + q_u1 d] */
  const double *err_c2;             /* c² at the u-quadrature points, (N, N, q_u1, q_u1) column-major */
  const double *uA, *vA, *uB, *vB;  /* states; uB = vB = NULL for the manufactured-solution errors */
  int where;
  double omega, ctT, stT;           /* ω, cos(ωT), sin(ωT) */
  int kx, ky;
  double px, py;
  const double *xloc, *yloc;        /* (N, q_u1) column-major: x of column k, y of row j at point i */
} wedg_norm_args;
int wedg_norms(const wedg_norm_args *a, double out[4]);

/* Size of the static device array used by wedg_rhs_noalloc (16 MiB). */
#define WEDG_NOALLOC_BYTES ((size_t)16 << 20)

/* One right-hand side evaluation that allocates nothing. It has no counterpart in
 * the reference: it exists for callers that cannot let a library allocate device
 * memory, such as programs whose GPU memory belongs to another runtime's pool
 * allocator or code that must not allocate or free device memory at the point
 * where it needs a right-hand side. It takes cfg and pre as wedg_create does
 * (host memory), u and v as device pointers and writes ut, vt (device pointers,
 * the reference's state layout); no workspace is needed. Its device scratch --
 * the copy of pre in the kernels' layouts, traces, Chebyshev data and the error
 * word -- is one static device array of WEDG_NOALLOC_BYTES, which every GPU that
 * loads the library holds until exit; meshes that need more are rejected with
 * WEDG_ERR_ARGUMENT and a message. It calls no cudaMalloc, cudaFree or other
 * allocating routine. The first call on a device looks up the array's address
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * Every call shares the array: calls that overlap on the GPU race and must be
 * serialised by the caller. `stream` is a cudaStream_t (NULL: the default
 * stream); the call returns after the evaluation has finished. Status and
 * message (into msg, if not NULL) as wedg_rhs. */
int wedg_rhs_noalloc(const wedg_config *cfg, const wedg_pre *pre, const double *u, const double *v, double t,
                     double *ut, double *vt, void *stream, char *msg, size_t msg_len);

const char *wedg_status_string(int status);
/* Library version and the GPU architecture it was built for. */
const char *wedg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* WEDG_H */
