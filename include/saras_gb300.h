/*
 * saras_gb300.h -- C ABI of the GB300 (sm_103a) implementation of SARAS-CC's
 * data-parallel hot path: the cell-centred geometric-multigrid pressure-Poisson
 * solve and the low-storage RK3 sub-step stencils around it.
 *
 * Every entry point takes plain pointers and sizes.  Field pointers address
 * element (0,0,0) of a padded, row-major (i,j,k) array with k fastest -- the
 * layout of a Blitz++ plainsf/field array indexed from -pad -- and `strides`
 * gives the element strides of i, j and k.  Host ("_host" or no suffix) and
 * device ("_dev") variants exist where the reference caller may hold either.
 *
 * Reference interfaces replaced (paths relative to the SARAS-CC source tree):
 *   saras_mg_create   <- multigrid_d3::multigrid_d3 / multigrid_d2::multigrid_d2
 *                        (lib/poisson/poisson.h:168,202; poisson.cc:66-92)
 *   saras_mg_solve    <- void poisson::mgSolve(plainsf &outLHS, const plainsf &inpRHS)
 *                        (lib/poisson/poisson.h:128; poisson.cc:109-189)
 *   saras_rk3_create  <- lsRK3_d3::lsRK3_d3 / lsRK3_d2::lsRK3_d2
 *                        (lib/timestep/lsRK3_d3.cc:58-79; timestep.cc:58-121)
 *   saras_rk3_step    <- lsRK3_d3::timeAdvance(vfield&, sfield&, sfield&) and
 *                        timeAdvance(vfield&, sfield&) (lsRK3_d3.cc:94-177,190-305);
 *                        with integration 1 eulerCN_d3::timeAdvance
 *                        (eulerCN_d3.cc:88-176, 178-268)
 *   saras_grid_metrics<- grid::mgGridMetrics / createTanHypGrid / setVCDepth
 *                        (lib/grid/grid.cc:411-742), as copied by
 *                        poisson::copyDerivs (lib/poisson/poisson.cc:501-622)
 *
 * Errors are returned, never raised: no entry point calls exit().  A handle
 * is used by one host thread at a time; its work is ordered on the CUDA
 * stream given at creation.
 */
#ifndef SARAS_GB300_H
#define SARAS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum saras_status {
    SARAS_OK = 0,
    SARAS_NOT_CONVERGED = 1, /* vcCount / outer-iteration cap reached above tolerance */
    SARAS_BAD_ARG = 2,
    SARAS_OOM = 3,           /* device allocation failed */
    SARAS_BUDGET = 4,        /* serving: request does not fit the HBM budget */
    SARAS_TIMEOUT = 5,       /* a bounded device wait gave up */
    SARAS_CUDA_ERR = 6,
    SARAS_NO_DEVICE = 7,
    SARAS_DIVERGED = 8,      /* CN Jacobi hit maxIterations, or the time-series divergence abort
                              * (the reference exits in both) */
    SARAS_NAN = 9            /* non-finite value met in an input or a residual */
} saras_status;

/* "Mesh Type" characters U/S/D (lib/io/parser.cc:413-452) */
enum { SARAS_MESH_UNIFORM = 0, SARAS_MESH_SINGLE_TANH = 1, SARAS_MESH_DOUBLE_TANH = 2 };

/* Poisson ghost-cell kinds per non-periodic face (lib/poisson/poisson_d3.cc:876-952):
 * NEUMANN        ghost = interior              (allNeumann, the reference default)
 * DIRICHLET      ghost = -interior             (homogeneous Dirichlet branch)
 * DIRICHLET_TEST ghost = 2*wall - interior at the finest level outside the
 *                error equation, -interior otherwise, wall = r^2/6 (3D) or
 *                r^2/4 (2D)                    (TEST_POISSON branch) */
enum { SARAS_BC_NEUMANN = 0, SARAS_BC_DIRICHLET = 1, SARAS_BC_DIRICHLET_TEST = 2 };

/* Arithmetic of the multigrid solve.
 * FP64_EXACT  reference operation order, no FMA contraction, IEEE division:
 *             bitwise equal to the CPU restatement of mgSolve.
 * FP64        FP64 throughout, coefficients pre-folded, FMA allowed.
 * MIXED       FP32 V-cycle (smoothing, restriction, prolongation) inside an
 *             FP64 defect-correction loop; residual, update, null-space
 *             projection and coarsest solve in FP64. */
enum { SARAS_PREC_FP64_EXACT = 0, SARAS_PREC_FP64 = 1, SARAS_PREC_MIXED = 2 };

/* Field boundary kinds of the RK3 fields (lib/boundary/dirichlet.cc, neumann.cc) */
enum { SARAS_FBC_DIRICHLET = 0, SARAS_FBC_NEUMANN = 1 };

typedef struct saras_grid_desc {
    int32_t dims;         /* 3, or 2 for the PLANAR (x,z) build */
    int32_t n[3];         /* "X Size", "Y Size", "Z Size"; n[1] is forced to 1 when dims==2 */
    double  len[3];       /* "X Length", "Y Length", "Z Length" */
    int32_t mesh_type[3]; /* SARAS_MESH_* from "Mesh Type" */
    double  beta[3];      /* "X Beta", "Y Beta", "Z Beta" */
    int32_t periodic[3];  /* "Domain Type": 'P' -> 1, 'N' -> 0 */
    int32_t pad;          /* pad width of caller fields: 1 ("Differentiation Scheme" 1) or 2 */
} saras_grid_desc;

typedef struct saras_mg_params {
    int32_t vc_count;      /* "V-Cycle Count" (mixed form: outer iterations) */
    double  vc_tolerance;  /* "Residual Tolerance" */
    int32_t solve_flag;    /* "Solve Coarsest" */
    double  mg_tolerance;  /* Multigrid "Solve Tolerance" (absolute, coarsest level) */
    double  sor_param;     /* "SOR Parameter" */
    int32_t pre_smooth;    /* "Pre-Smoothing Count" */
    int32_t post_smooth;   /* "Post-Smoothing Count" */
    int32_t res_type;      /* "Residual Type": 0 Linf, 1 L1, 2 L2 (relative to the RHS) */
    int32_t print_residual;/* "Print Residual" */
    int32_t bc_kind[6];    /* SARAS_BC_* for faces x-, x+, y-, y+, z-, z+ */
    int32_t test_poisson;  /* TEST_POISSON build semantics: no early exit */
    int32_t precision;     /* SARAS_PREC_* */
    int32_t levels;        /* 0: reference depth from setVCDepth; >0: that many levels */
    int32_t inner_cycles;  /* MIXED form: FP32 V-cycles per FP64 defect correction (>= 1;
                              1 repeats the FP64 form cycle by cycle); negative: adaptive, at most
                              -inner_cycles per correction and, once the residual is within reach,
                              the V-cycles the last correction's contraction says are left (plus
                              one); ignored by the others */
} saras_mg_params;

typedef struct saras_mg saras_mg;

/* Fills the parameters with the reference defaults of input/parameters.yaml's
 * Multigrid section and Neumann walls. */
void saras_mg_default_params(saras_mg_params *p);

/* Builds the level hierarchy, metric tables and device arrays.  `stream` is
 * a cudaStream_t (NULL: the legacy default stream). */
saras_status saras_mg_create(const saras_grid_desc *grid, const saras_mg_params *prm,
                             void *stream, saras_mg **out);

/* mgSolve with HOST fields: reads the core of rhs and of lhs (initial guess),
 * writes the core plus one ghost layer of lhs.  res_hist (may be NULL)
 * receives the residual after each V-cycle, up to hist_cap entries;
 * *n_cycles the number of V-cycles (outer iterations) run. */
saras_status saras_mg_solve(saras_mg *h, double *lhs, const double *rhs, const int64_t strides[3],
                            double *res_hist, int32_t hist_cap, int32_t *n_cycles);

/* Same with DEVICE pointers (same layout rules); no host copies. */
saras_status saras_mg_solve_dev(saras_mg *h, double *lhs, const double *rhs, const int64_t strides[3],
                                double *res_hist, int32_t hist_cap, int32_t *n_cycles);

saras_status saras_mg_destroy(saras_mg *h);

int32_t saras_mg_num_levels(const saras_mg *h);

/* Bytes of device memory the handle holds. */
int64_t saras_mg_device_bytes(const saras_mg *h);

/* Kernel timing: when enabled, launches of each kernel class are bracketed
 * with CUDA events on the solve stream.  Class ids: 0 smoothing sweep at the
 * finest level, 1 residual+restriction, 2 prolongation+correction,
 * 3 residual norm, 4 coarsest solve; and the copies of saras_mg_solve's host
 * boxes: 5 host->device (two per call), 6 device->host (one per call). */
saras_status saras_mg_set_kernel_timing(saras_mg *h, int32_t enable);
saras_status saras_mg_kernel_stats(saras_mg *h, int32_t kclass, int64_t *launches,
                                   double *total_ms, double *bytes_per_launch);
/* No reference counterpart (fault handling).  Bound, in polls, of the
 * mbarrier waits of the TMA-staged FP32 sweeps (MIXED form, large 3-D
 * levels); 0 restores the default of 2^24 polls.  A wait that runs out ends
 * that sweep: the kernel records the error, stops issuing copies, waits
 * (with the default bound) for the loads and stores it issued and returns;
 * the solve then returns SARAS_TIMEOUT after the V-cycle, and the handle
 * stays usable (the next solve starts with the error cleared).  Setting a
 * new bound re-captures the handle's CUDA graphs on their next use. */
saras_status saras_mg_set_wait_limit(saras_mg *h, int64_t polls);

/* Total kernel launches issued by the last solve. */
int64_t saras_mg_last_launches(const saras_mg *h);

/* No reference counterpart.  V-cycles the last solve ran (the MIXED form:
 * FP32 V-cycles over all its outer iterations). */
int64_t saras_mg_last_vcycles(const saras_mg *h);

/* No reference counterpart (measurement).  The FP64 instruction rate of the
 * current device, the denominator of the FP64 form's arithmetic roofline:
 * full-occupancy kernels of independent dependency chains, timed with CUDA
 * events on `stream`.  *fma_per_s: fused multiply-adds per second;
 * *addmul_per_s: separately rounded adds and multiplies per second. */
saras_status saras_measure_fp64_rate(void *stream, double *fma_per_s, double *addmul_per_s);

/* Host restatement of the per-level grid metrics the multigrid uses:
 * x (cell centres), xixx and xix2 for `axis` at `level`, each over indices
 * -1..n_l (n_l + 2 values).  *n_out receives n_l. */
saras_status saras_grid_metrics(const saras_grid_desc *grid, int32_t levels, int32_t level,
                                int32_t axis, double *x, double *xixx, double *xix2,
                                int32_t *n_out);

/* Number of levels setVCDepth gives for this grid (vcdGlo + 1), or -1. */
int32_t saras_reference_levels(const saras_grid_desc *grid);

/* Left null vector w of the 1-D all-Neumann finest-level operator along
 * `axis` (n values, normalised to max |w| = 1).  The 3-D operator's left null
 * vector is w_x (x) w_y (x) w_z; a right-hand side f is compatible iff
 * sum w f = 0. */
saras_status saras_neumann_null_vector(const saras_grid_desc *grid, int32_t axis, double *w);

/* ---------------------------------------------------------------- RK3 ---- */

typedef struct saras_field_bc {
    int32_t type[6];   /* SARAS_FBC_* for faces x-, x+, y-, y+, z-, z+ */
    double  value[6];
} saras_field_bc;

#define SARAS_STENCIL_EXACT 0
#define SARAS_STENCIL_FAST  1

typedef struct saras_rk3_params {
    double  nu, kappa;      /* from timestep::timestep (see saras_rbc_coefficients) */
    double  dt;             /* "Time-Step" */
    double  cn_tolerance;   /* Solver "Solve Tolerance" */
    int32_t max_iterations; /* 0: int(pow(log(Nx*Ny*Nz), 3)) as timestep.cc:115 */
    double  g_terms[3];     /* buoyancy Fb*g/|g|; all zero for zeroForcing */
    int32_t with_scalar;    /* 1: timeAdvance(V,P,T); 0: timeAdvance(V,P) */
    int32_t nl_scheme;      /* "Non-Linear Term": 1 central, 2 hybrid upwind, 3 Morinishi */
    saras_field_bc bc_vx, bc_vy, bc_vz, bc_t;
    saras_field_bc bc_p;    /* pressure field walls */
    saras_mg_params mg;     /* pressure-correction solve */
    /* Solver "Peclet Limit" and "Central Bias" of the hybrid upwind term
     * (nl_scheme 2; vfield.cc:114-130); the Peclet number uses nu for the
     * velocity and kappa for the temperature (scalar_d3.cc:166-167) */
    double  pe_limit, up_param;
    /* "Integration Scheme": 2 (or 0) low-storage RK3, lsRK3_d3/_d2;
     * 1 Euler/Crank-Nicolson, eulerCN_d3/_d2 (scalar_d3.cc:156-163) */
    int32_t integration;
    /* SARAS_STENCIL_EXACT (0): every value of the right-hand sides and the
     * Crank-Nicolson sweeps in the reference's order with separately
     * rounded FP64 operations (bit parity).  SARAS_STENCIL_FAST (1): the same
     * stencils with folded coefficients, fused multiply-adds and products
     * with reciprocals of the stencil constants; equal to the exact form to
     * rounding, not bit for bit. */
    int32_t stencil_form;
} saras_rk3_params;
/* The Differentiation Scheme follows the grid descriptor's pad: pad 1 is
 * dScheme 1 (second order), pad 2 is dScheme 2 (fourth order in the interior,
 * second order on the first and last core cell of every axis). */

typedef struct saras_rk3 saras_rk3;

/* nu, kappa and buoyancy strength Fb for "RBC Type" 1-4 (timestep.cc:74-99,
 * buoyantForce.cc:45-57). */
saras_status saras_rbc_coefficients(int32_t rbc_type, double ra, double pr,
                                    double *nu, double *kappa, double *fb);

saras_status saras_rk3_create(const saras_grid_desc *grid, const saras_rk3_params *prm,
                              void *stream, saras_rk3 **out);
/* Copies full padded fields (pad from the grid descriptor) host -> device.
 * vy is ignored for dims==2, t when with_scalar==0.  pp is the pressure
 * correction, the multigrid initial guess that persists between calls. */
saras_status saras_rk3_upload(saras_rk3 *h, const double *vx, const double *vy, const double *vz,
                              const double *p, const double *t, const double *pp,
                              const int64_t strides[3]);
saras_status saras_rk3_download(saras_rk3 *h, double *vx, double *vy, double *vz,
                                double *p, double *t, double *pp, const int64_t strides[3]);
/* Runs nsteps calls of timeAdvance.  *mg_cycles (may be NULL) receives the
 * total V-cycles of the pressure solves, *cn_iters the total Jacobi sweeps. */
saras_status saras_rk3_step(saras_rk3 *h, int32_t nsteps, int32_t *mg_cycles, int32_t *cn_iters);
saras_status saras_rk3_destroy(saras_rk3 *h);
int64_t saras_rk3_last_launches(const saras_rk3 *h);

/* ---------------------------------------------------- time loop ---- */
/* The time loop of scalar_d3/hydro_d3::solvePDE (src/solvers/scalar/
 * scalar_d3.cc:184-262) on the device-resident fields: timeAdvance, the CFL
 * time step (vfield::computeTStp, vfield.cc:691-719; capped at the
 * "Time-Step" the handle was created with), time += dt, a time-series row
 * every io_count steps (tseries::writeTSData, tseries.cc:209-488), until
 * |t_max - time| < dt/2.  Probes, solution and restart files are the
 * caller's.  The next step uses the CFL time step, as the reference's
 * integrator holds dt by reference. */
typedef struct saras_run_params {
    double  t_max;        /* "Final Time" */
    double  courant;      /* "Courant Number" */
    int32_t use_cfl;      /* "Use CFL Condition" */
    int32_t io_count;     /* "I/O Count" */
    int32_t prob_type;    /* "Problem Type": 9 (open top) counts one wall in Nu */
    int32_t max_steps;    /* stop after this many steps; 0 = no limit */
    double  g_axis[3];    /* "Gravity Direction": Nusselt along z unless g_axis[2] == 0 */
} saras_run_params;

/* One time-series row.  With temperature (tseries.cc:291-488): Re, Nu at
 * the walls, volume Nu, kinetic and thermal energy per volume; without it
 * (tseries.cc:209-289): kinetic energy and U_rms.  divergence is the
 * maximum |div V| over the core.  The sums run over the core in a
 * different order than the reference's sequential loops, so they agree
 * with it to rounding (the maxima are exact). */
typedef struct saras_tseries_row {
    double time, dt;
    double re, nu_wall, nu_vol;
    double ke, te, urms, divergence;
} saras_tseries_row;

/* The row of the current fields at `time` (no time step). */
saras_status saras_rk3_tseries(saras_rk3 *h, const saras_run_params *rp, double time, saras_tseries_row *row);
/* vfield::computeTStp on the current velocity: courant / max(|u|/dx + |v|/dy
 * + |w|/dz) with the average spacings L/N (exact; not capped). */
saras_status saras_rk3_cfl_dt(saras_rk3 *h, double courant, double *dt);
/* Runs the loop from *time (updated).  Row 0 is the state at the start
 * time.  At most row_cap rows are stored; *n_rows counts the rows produced.
 * SARAS_DIVERGED when the divergence exceeds 1e3 and grows (tseries.cc:
 * 216-222), with the rows and steps up to there. */
saras_status saras_rk3_run(saras_rk3 *h, const saras_run_params *rp, double *time, saras_tseries_row *rows,
                           int32_t row_cap, int32_t *n_rows, int32_t *n_steps);

/* ------------------------------------------------------------ serving ---- */
/*
 * Continuous batching of independent Poisson requests (no counterpart in the
 * reference, which solves one problem per MPI job): every admitted request
 * keeps its MIXED-form hierarchy resident in HBM, and one graph launch runs
 * one outer iteration (FP32 V-cycle + FP64 residual) of ALL admitted
 * requests.  Requests are admitted while case slots and the HBM budget allow
 * and retire when their relative residual (max|r| / max|f|) falls below
 * `tolerance`.  Each request's arithmetic is independent of the others and
 * of the schedule, so its result is the same alone and in any mix, and the
 * same as saras_mg_solve in the MIXED form with the engine's parameters.
 * Walls are Neumann on every non-periodic face.
 */
typedef struct saras_serve_params {
    int64_t hbm_budget_bytes; /* resident hierarchies (pooled ones included) */
    int32_t max_cases;        /* requests admitted at once (1..4096) */
    int32_t max_cycles;       /* outer iterations before NOT_CONVERGED */
    double tolerance;         /* relative residual that retires a request */
    double mg_tolerance;      /* coarsest-level absolute tolerance */
    double sor_param;
    int32_t pre_smooth, post_smooth;
    /* schedule (0 = default): cells per work item, threads per block,
     * blocks per SM of the batched kernels; saras_serve_autotune sets them */
    int32_t cells_per_item, threads, blocks_per_sm;
    int32_t pad_;
} saras_serve_params;

typedef struct saras_serve_stats {
    int64_t bytes_allocated; /* device bytes of resident + pooled hierarchies */
    int64_t batched_cycles;  /* graph launches (outer iterations of the batch) */
    int64_t launches;        /* kernels launched by those graphs */
    int64_t admitted, retired;
    int32_t active, pending, pooled, max_active;
    /* wall-clock seconds inside saras_serve_step: batched iterations (graph
     * launch to its residuals on the host), admissions (uploads, hierarchy
     * set-up), retirements (projection, copy out), and the host-driven parts
     * of time-step requests (right-hand sides, CN sweeps, corrections) */
    double t_batch_s, t_admit_s, t_retire_s, t_steps_s;
} saras_serve_stats;

typedef struct saras_serve saras_serve;

void saras_serve_default_params(saras_serve_params *p);
saras_status saras_serve_create(const saras_serve_params *prm, saras_serve **out);
/* Queues a request.  rhs and lhs are dense padded host boxes of the grid
 * (pad from the descriptor, k fastest) that must stay valid until the
 * request is returned by saras_serve_poll; lhs receives the solution core and
 * its ghost layer. */
saras_status saras_serve_submit(saras_serve *h, int64_t id, const saras_grid_desc *grid,
                                const double *rhs, double *lhs);
/* Queues a time-step request: one timeAdvance (lsRK3 or eulerCN, as
 * prm->integration says) of the padded host fields vx, vy, vz, p, t, pp,
 * which are updated in place when the request is returned by
 * saras_serve_poll (vy is ignored for dims == 2, t when with_scalar == 0).
 * Each pressure solve of the step runs in the engine's batch in the MIXED
 * form with the engine's smoothing, SOR and coarsest tolerance, and stops at
 * the request's own prm->mg.vc_tolerance or after prm->mg.vc_count outer
 * iterations ("Residual Tolerance", "V-Cycle Count": the pressure RHS of a
 * collocated step is not exactly compatible with the Neumann operator, so
 * its residual levels off).  The result equals saras_rk3_step on a handle
 * whose mg is that MIXED form with those two keys.  The reported cycles are
 * the outer iterations of all its pressure solves and the status OK also
 * when a pressure solve stopped at its V-Cycle Count above the tolerance:
 * mgSolve simply returns after vcCount cycles and the step completes
 * (poisson.cc:182-188); the residual polled is the last solve's. */
saras_status saras_serve_submit_step(saras_serve *h, int64_t id, const saras_grid_desc *grid,
                                     const saras_rk3_params *prm, double *vx, double *vy, double *vz,
                                     double *p, double *t, double *pp);
/* Admits what fits, runs one batched outer iteration, retires finished
 * requests.  *active / *pending (may be NULL) receive the counts after it. */
saras_status saras_serve_step(saras_serve *h, int32_t *active, int32_t *pending);
/* Up to cap finished requests, oldest first: id, final relative residual,
 * outer iterations, status (OK, NOT_CONVERGED, NAN, ...) and seconds from
 * submit to retirement.  Any output pointer may be NULL. */
saras_status saras_serve_poll(saras_serve *h, int64_t *ids, double *residuals, int32_t *cycles,
                              int32_t *status, double *latency_s, int32_t cap, int32_t *n);
/* Times `cycles` batched iterations of synthetic requests of the given
 * shapes under each candidate schedule, keeps the fastest (written to
 * *chosen when not NULL) and leaves the hierarchies pooled.  The engine
 * must be idle (nothing active or pending). */
saras_status saras_serve_autotune(saras_serve *h, const saras_grid_desc *grids, int32_t n,
                                  int32_t cycles, saras_serve_params *chosen);
saras_status saras_serve_get_stats(const saras_serve *h, saras_serve_stats *out);
saras_status saras_serve_destroy(saras_serve *h);

/* ----------------------------------------------------- static scratch ---- */
/*
 * No counterpart in the reference.  saras_mg_solve_static runs one mgSolve
 * (FP64 or MIXED form) on device fields without allocating device memory:
 * its working memory is one file-scope __device__ array of
 * SARAS_STATIC_SCRATCH_BYTES (32 MiB) per device, which holds the hierarchy
 * of a 3-D grid up to about 80^3 (a 2-D grid up to about 512^2); a grid that
 * does not fit returns SARAS_BUDGET, naming the bytes it needs, before any
 * device work.  It is for callers that cannot allocate at solve time:
 * cudaMalloc/cudaFree synchronise the whole device, a caching allocator may
 * already hold the free HBM, and a time step must not fail half-way for want
 * of memory.  Every call looks up the scratch's address on the current
 * device, so the entry point stays usable after a cudaDeviceReset; the first
 * lookup on a device loads the library's module there, so make the first
 * call before any stream capture.  Nothing in the scratch has to start at
 * zero.  The call
 * returns once its work on `stream` has finished (it synchronises the
 * stream), so a later call on any stream finds the scratch free.  Every call
 * on a device uses the same scratch, so calls that overlap in time (from
 * different host threads) race; the caller serialises them.
 * Arguments as saras_mg_create (grid, params, stream) plus
 * saras_mg_solve_dev (device fields, strides, residual history).
 */
#define SARAS_STATIC_SCRATCH_BYTES (32u << 20)
saras_status saras_mg_solve_static(const saras_grid_desc *grid, const saras_mg_params *prm, void *stream,
                                   double *lhs, const double *rhs, const int64_t strides[3],
                                   double *res_hist, int32_t hist_cap, int32_t *n_cycles);

/* ------------------------------------------------------------- common ---- */

const char *saras_status_string(saras_status s);
/* Text of the last error on the calling thread ("" if none). */
const char *saras_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SARAS_GB300_H */
