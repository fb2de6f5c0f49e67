/*
 * gradpower_gb300.h — C ABI of the GB300-native batched backward-Euler
 * Newton step of GradPower.jl.
 *
 * The library integrates M independent fault scenarios of one power system
 * on one GPU.  Every scenario follows the reference's CPU semantics
 * (`integrate!`, src/dynamics.jl:502-655, and `newton_step!`,
 * src/numerics.jl:55-176): backward Euler with step dt, a Newton solve per
 * step that stops when the residual infinity norm drops below `newton_tol`,
 * fault events toggled after step k's solve with an extra dt = 0 solve, and
 * the state stored before that re-solve.
 *
 * Conventions
 *  - All indices are 0-based.  z is the per-scenario state vector of length
 *    n_sys = n_diff + n_alg + 2*n_bus, laid out as the reference lays it
 *    after `reorder_state!` (src/clusters.jl:225-319): the states of each
 *    generator cluster contiguously, then (vr, vi) per bus.
 *  - Host arrays of per-scenario data are scenario-major: z[m*n_sys + i].
 *  - Every function returns 0 on success or a negative GP_E* code; the
 *    message of the last error is available from gp_last_error().
 *  - The library owns its device memory.  A layout is used by one host
 *    thread at a time; it runs on its own CUDA stream.
 *
 * Reference interfaces replaced (file:line in GradPower.jl):
 *  - GpuBatchedLayout(dp, ps, M)           ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:466
 *      -> gp_layout_create
 *  - integrate_gpu_schur_cudss!(gbl, ps, tf; dt, newton_tol)
 *                                          ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:3008-3080
 *      -> gp_integrate(..., solver = GP_SOLVER_SCHUR_FP64)
 *  - integrate_gpu_cudss!(gbl, ps, tf; dt, newton_tol)
 *                                          ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2924-2996
 *      -> gp_integrate(..., solver = GP_SOLVER_SCHUR_FP64): the monolithic
 *         LU of J is the same exact Newton step; the library eliminates the
 *         cluster blocks first, which is one elimination order of that LU
 *  - _beuler_all_scenarios_gpu!            ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:1522-1542
 *      -> gp_residual (parity probe)
 */
#ifndef GRADPOWER_GB300_H
#define GRADPOWER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GP_ABI_VERSION 1

/* error codes */
#define GP_OK            0
#define GP_E_INVALID    -1   /* bad argument or inconsistent problem */
#define GP_E_CUDA       -2   /* CUDA runtime error */
#define GP_E_NOMEM      -3   /* allocation failed */
#define GP_E_NUMERIC    -4   /* zero pivot / non-finite values */
#define GP_E_TIMEOUT    -5   /* a device wait ran out its iteration limit */
#define GP_E_INTERNAL   -6   /* an internal consistency check failed */

/* device types, in the reference's DEVICE_REGISTRY order (src/layout.jl) */
enum {
    GP_GENROU = 0,      /* GENROU and GENSAL (src/kernels/genrou.jl)      */
    GP_IEESGO = 1,      /* src/kernels/ieesgo.jl                           */
    GP_TGOV1 = 2,       /* src/kernels/tgov1.jl                            */
    GP_SEXS = 3,        /* src/kernels/sexs.jl                             */
    GP_ESDC1A = 4,      /* src/kernels/esdc1a.jl                           */
    GP_IEEEST = 5,      /* src/kernels/ieeest.jl                           */
    GP_ZIPLOAD = 6,     /* src/kernels/zipload.jl                          */
    GP_STATIC_GEN = 7,  /* src/kernels/static_gen.jl                       */
    GP_NTYPES = 8
};

/*
 * One struct-of-arrays device table (the reference's *Table structs,
 * src/layout.jl:61-179).  Arrays have length n.  Absent pointers are -1.
 *   bus      internal bus index
 *   diff_ptr z index of the first differential state
 *   alg_ptr  z index of the first algebraic state
 *   ctrl_ptr index into u of the first control slot
 *   par_ptr  index into p of the first parameter (fill_pvec! order)
 *   link0    GENROU: z index of the governor's p_m (pm_idx)
 *            IEESGO/TGOV1/IEEEST: z index of the machine speed w (w_idx)
 *            SEXS/ESDC1A: z index of the stabiliser output v_s (vs_idx)
 *            STATIC_GEN: bus type (1 PQ, 2 PV, 3 slack)
 *   link1    GENROU: z index of the exciter's e_fd (efd_idx); else unused
 *   online   0 = device skipped (may be NULL: all online)
 */
typedef struct gp_device_table {
    int32_t n;
    const int32_t *bus;
    const int32_t *diff_ptr;
    const int32_t *alg_ptr;
    const int32_t *ctrl_ptr;
    const int32_t *par_ptr;
    const int32_t *link0;
    const int32_t *link1;
    const uint8_t *online;
} gp_device_table;

/*
 * The problem, shared by all scenarios.  Values that differ per scenario
 * (z0, u0, p) are passed to gp_layout_create separately.
 */
typedef struct gp_problem {
    int32_t n_bus, n_diff, n_alg, n_ctrl, n_par;
    /* complex bus admittance matrix in CSR form (src/network.jl:29-85) */
    int32_t y_nnz;
    const int32_t *y_rowptr;     /* [n_bus+1] */
    const int32_t *y_colidx;     /* [y_nnz]   */
    const double *y_re, *y_im;   /* [y_nnz]   */
    /* bus adjacency without self loops, CSR (src/network.jl:15-27) */
    const int32_t *adj_rowptr;   /* [n_bus+1] */
    const int32_t *adj_colidx;
    gp_device_table dev[GP_NTYPES];
    const uint8_t *is_diff;      /* [n_diff+n_alg]: 1 for differential states */
    /* generator clusters (src/clusters.jl:16-57), in z order */
    int32_t n_clusters;
    const int32_t *cl_w_start, *cl_w_size, *cl_bus;
    const int32_t *cl_gen;       /* GENROU table index, -1 for a static generator */
    const int32_t *cl_sg;        /* STATIC_GEN table index or -1 */
    const int32_t *cl_gov_type;  /* GP_IEESGO, GP_TGOV1 or -1 */
    const int32_t *cl_gov;
    const int32_t *cl_exc_type;  /* GP_SEXS, GP_ESDC1A or -1 */
    const int32_t *cl_exc;
    const int32_t *cl_pss;       /* IEEEST table index or -1 */
} gp_problem;

/* A three-phase bus fault (ContingencyEvent, src/GradPower.jl:117-128).
 * on_step/off_step are round(ton/dt), round(toff/dt) with ties to even. */
typedef struct gp_fault {
    int32_t scenario;            /* -1: every scenario (the reference's global events) */
    int32_t bus;
    double rfault;
    int32_t on_step;
    int32_t off_step;
} gp_fault;

/* A line trip (TripLineEvent, src/GradPower.jl:148-167; its admittance
 * terms as create_trip_line_event computes them, :500-543): at the end of
 * step on_step the line's admittance contributions are removed from Ybus
 * (_apply_trip_line!, :551-564), and at the end of step off_step they are
 * added back (_apply_reclose_line!, :566-574; off_step < 0: never), each
 * followed by the dt = 0 re-solve (src/dynamics.jl:612-646).  Buses are
 * 0-based internal indices.  Every gp_integrate call starts and ends with
 * all lines in service (the reference leaves a permanent trip in
 * ps.network.ybus_real after integrate!). */
typedef struct gp_line_trip {
    int32_t scenario;            /* -1: every scenario */
    int32_t from_bus, to_bus;
    double yff[2], yft[2], ytf[2], ytt[2];   /* (real, imag) */
    int32_t on_step;
    int32_t off_step;
} gp_line_trip;

/* A device disconnection (DisconnectDeviceEvent, src/GradPower.jl:131-146):
 * at the end of step on_step the device's online flag is cleared
 * (_set_device_offline!, :672-698) for the rest of the call, followed by the
 * dt = 0 re-solve (src/dynamics.jl:612-646).  The batch kernels skip an
 * offline device (`table.online[k] || continue` in the device kernels of
 * src/kernels/): its differential states hold (their backward-Euler rows
 * become z - zold) and it injects nothing into the network.  A device that owns algebraic rows
 * (GENROU, IEESGO, TGOV1, IEEEST, a PV or slack static generator) would
 * leave those rows without equations, a singular Jacobian: such events are
 * refused with GP_E_INVALID.  Every gp_integrate call starts and ends
 * with all devices online. */
typedef struct gp_device_disconnect {
    int32_t scenario;            /* -1: every scenario */
    int32_t type;                /* GP_SEXS, GP_ESDC1A, GP_ZIPLOAD or GP_STATIC_GEN (PQ) */
    int32_t index;               /* row in that device table */
    int32_t on_step;
} gp_device_disconnect;

/* GP_SOLVER_SCHUR_FP64: exact Newton, the reference's batched schedule: the
 *   cluster blocks and the reduced network matrix are factored in FP64 at
 *   every iteration.
 * GP_SOLVER_SHARED_WOODBURY: integrate_gpu_shared_multi!
 *   (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2640-2708, Newton step
 *   :2523-2627): the reduced network matrix P of scenario 0 at the initial
 *   state (no fault, the call's dt) is factored once per call and shared by
 *   every scenario, iteration and step; a scenario's fault enters as the
 *   rank-2 Woodbury correction of P at its bus.  The cluster blocks, the
 *   residual and the convergence test are exact at every iteration, so the
 *   result is the same root to the same tolerance, reached by a chord
 *   iteration (linear convergence).  Each scenario may have one fault bus
 *   and rfault (several on/off windows allowed; they must not overlap).
 *   The reference shares ton/toff over the scenarios and stops on the L2
 *   norm over all of them; here every scenario has its own windows and its
 *   own infinity-norm test, as the other solvers.
 * GP_SOLVER_SCHUR_MIXED: the cluster blocks' LU and the reduced-system
 *   factors are kept in FP32 and reused across Newton iterations and steps;
 *   every iteration evaluates the residual in FP64 and corrects with the
 *   kept factors (defect correction / iterative refinement of the nonlinear
 *   system), the convergence test is the same FP64 infinity norm.  A
 *   scenario refreshes its factors (FP64 Jacobian at the current iterate,
 *   stored in FP32) at the first solve and around events, and then by the
 *   policy of gp_set_mixed_policy. */
#define GP_SOLVER_SCHUR_FP64   0
#define GP_SOLVER_SCHUR_MIXED  1
#define GP_SOLVER_SHARED_WOODBURY 2

typedef struct gp_options {
    double dt;
    int32_t n_steps;             /* Int(round(tf/dt)) */
    double newton_tol;           /* infinity-norm tolerance, reference default 1e-10 */
    int32_t itermax;             /* reference batched default 30 */
    int32_t solver;              /* GP_SOLVER_* */
} gp_options;

typedef struct gp_layout gp_layout;

/* Library version and the message of the last failed call (thread-local). */
int32_t gp_abi_version(void);
int32_t gp_last_error(char *buf, int32_t len);

/* Build the device-resident layout for M scenarios: uploads the problem,
 * runs the host-once symbolic analysis of the reduced network matrix and
 * allocates all work buffers.  z0 [M*n_sys], u0 [M*n_ctrl], p [M*n_par].
 * Replaces GpuBatchedLayout(dp, ps, M). */
int32_t gp_layout_create(const gp_problem *prob, int32_t M, const double *z0,
                         const double *u0, const double *p, gp_layout **out);
int32_t gp_layout_destroy(gp_layout *L);

/* Sizes of the host-once symbolic analysis, for reporting:
 * out[0] n_red, out[1] nnz of the reduced matrix, out[2] nnz(L+U) of its
 * supernodal factor, out[3] supernodes, out[4] elimination-tree levels,
 * out[5] factor flops per scenario (rounded), out[6] sum of w_k^2. */
int32_t gp_layout_stats(const gp_layout *L, int64_t out[8]);

/* Copy the current state of all scenarios in or out: z [M*n_sys]. */
int32_t gp_set_state(gp_layout *L, const double *z);
int32_t gp_get_state(const gp_layout *L, double *z);
/* Reset the state to the z0 given to gp_layout_create (device-side copy;
 * reruns a batch without host traffic). */
int32_t gp_restore_initial_state(gp_layout *L);

/* Line trips for the following gp_integrate calls (replaces the previous
 * set; n = 0 clears them).  GP_SOLVER_SCHUR_FP64 and GP_SOLVER_SCHUR_MIXED
 * only: GP_SOLVER_SHARED_WOODBURY and gp_adjoint return GP_E_INVALID while
 * trips are set.  The batched GPU path of the reference has no line trips:
 * this carries integrate!'s to it (per scenario). */
int32_t gp_set_line_trips(gp_layout *L, int32_t n, const gp_line_trip *trips);

/* Device initialisation of every scenario on the GPU from solved power
 * flows: initialize_dynamics! (src/dynamics.jl:123-250), with the GENROU
 * initialisation of src/generators.jl:159-285 (a Newton solve of each
 * machine's steady state) and the controllers' steady states.
 *   v_polar [M][n_bus][2]       bus voltage magnitude and angle (rad)
 *   gen_pq  [M][n GENROU][2]    each machine's active and reactive output
 *   sg_pq   [M][n STATIC_GEN][2] each static generator's totals p0, q0
 *                               (NULL when the problem has none)
 * Every parameter comes from the layout's parameter vectors (as given to
 * gp_layout_create, with each scenario's load powers in the ZIP rows); the
 * derived ones are written back: ZIP v0mag and admittance, static-generator
 * p0/q0, governor pref, exciter vref.  The result becomes the layout's
 * state, initial state (gp_restore_initial_state), controls and
 * parameters; z0 [M*n_sys], u0 [M*n_ctrl] and p [M*n_par] receive copies
 * (each may be NULL).  GP_E_NUMERIC when a machine's initialisation
 * residual stays at or above 1e-9 (the reference's bound,
 * src/dynamics.jl:58); the layout then holds the failed state. */
int32_t gp_initialize(gp_layout *L, const double *v_polar, const double *gen_pq, const double *sg_pq,
                      double *z0, double *u0, double *p);

/* Device disconnections for the following gp_integrate calls (replaces the
 * previous set; n = 0 clears them).  GP_SOLVER_SCHUR_FP64 and
 * GP_SOLVER_SCHUR_MIXED only, like line trips: GP_SOLVER_SHARED_WOODBURY
 * and gp_adjoint return GP_E_INVALID while disconnections are set.  The
 * reference's batched GPU path has none: this carries integrate!'s to it
 * (per scenario). */
int32_t gp_set_device_disconnects(gp_layout *L, int32_t n, const gp_device_disconnect *events);

/* Integrate every scenario for opt->n_steps backward-Euler steps from the
 * current state.  Replaces integrate_gpu_schur_cudss! / integrate_gpu_cudss!.
 *   traj    [M][n_steps+1][n_sys] host output, or NULL
 *   iters   [M][2*n_steps] Newton iterations: slot 2k the step solve of
 *           step k+1, slot 2k+1 its event re-solve (0 if none); or NULL
 *   status  [M] bit flags, 0 = converged everywhere: 1 some solve hit
 *           itermax, 2 non-finite values, 4 a zero pivot in the reduced
 *           matrix, 8 a dataflow wait gave up (the call then returns
 *           GP_E_TIMEOUT, with status still filled); or NULL
 * On return the layout holds the final state. */
int32_t gp_integrate(gp_layout *L, const gp_options *opt, int32_t n_faults,
                     const gp_fault *faults, double *traj, int32_t *iters,
                     int32_t *status);

/* Parity probe: the backward-Euler residual of every scenario at the
 * current state against zold [M*n_sys] (src/dynamics.jl:366-391), with the
 * faults whose flag in fault_on [n_faults] is 1 applied.  f [M*n_sys]. */
int32_t gp_residual(gp_layout *L, const double *zold, double dt, int32_t n_faults,
                    const gp_fault *faults, const uint8_t *fault_on, double *f);

/* Newton loop driver.  Off (the default): each Newton solve is one CUDA
 * graph that runs the whole loop on the device (a WHILE node over solve +
 * evaluation, conditions set by the convergence-check kernel; the mixed
 * solver's factorisation variant is a SWITCH node), so the host does not
 * wait on the GPU between iterations.  On: the host drives the loop, one
 * evaluation graph and one solve graph per iteration, with CUDA events
 * around every phase for gp_last_timing.  Both give the same results.
 * No counterpart in the reference: its Newton loop is host code
 * (src/schur.jl:285, `for iter = 1:itermax`). */
int32_t gp_set_profiling(gp_layout *L, int32_t on);

/* Polls (at about 32 ns each) after which a wait of the dataflow kernels on
 * another task's done flag gives up (default 2^20, about 30 ms): the kernel
 * then raises an error flag, every other wait returns at once, the kernel
 * finishes, the waiting scenario gets status bit 8 and the call returns
 * GP_E_TIMEOUT.  The next call clears the flag and starts afresh.  polls >=
 * 1; GP_E_INVALID otherwise.  No counterpart in the reference (cuDSS has no
 * such wait); a failure-detection hook: a tiny limit makes the waits run
 * out without anything on the GPU hanging. */
int32_t gp_set_wait_limit(gp_layout *L, int32_t polls);

/* Time of the last gp_integrate call split by phase, milliseconds between
 * CUDA events recorded on the library's stream inside the captured graphs
 * (the phases only with profiling on, gp_set_profiling; zero otherwise):
 * out[0] total, out[1] cluster kernel, out[2] network kernel, out[3]
 * factorisation (all levels), out[4] triangular solves, out[5] Newton
 * iterations summed over steps (max over scenarios), out[6] kernel launches,
 * out[7] update kernel, out[8] factorisation launches, out[9] linear
 * solves (batched over scenarios), out[10] mixed solver: scenario FP32
 * factor refreshes, out[11] mixed solver: scenario iterations solved with
 * fresh FP64 factors, out[12] mixed solver: scenario solves redone with
 * exact Newton steps after failing with inexact ones; out[13..15] zero. */
int32_t gp_last_timing(const gp_layout *L, double out[16]);

/* Objective of the adjoint:
 *   J = sum over the stored trajectory points t = 1..n_steps of
 *       dt * ( w_speed * sum over machines of w^2
 *            + w_volt * sum over buses of max(0, v_min - |V|)^2 )
 * where w is the machine speed deviation.  w_speed = 1, w_volt = 0 is the
 * reference's functional (src/dynamics.jl:330-337 with the time weighting of
 * src/nlp.jl:30-46). */
typedef struct gp_objective {
    double w_speed;
    double w_volt;
    double v_min;
} gp_objective;

/* Discrete adjoint of gp_integrate (FP64 Schur path), for every scenario:
 * integrates opt->n_steps steps forward from the current state, keeping the
 * state every checkpoint_every steps, then sweeps backwards, recomputing the
 * steps between checkpoints, with one transposed Newton-Jacobian solve per
 * forward solve (regular steps and dt = 0 event re-solves) at its converged
 * state and fault status.
 *   J        [M] objective value
 *   grad_p   [M][n_par] dJ/dp at the fixed initial state: filled for the
 *            machine inertia H and damping D (GENROU/GENSAL), the exciter
 *            gain (SEXS K, ESDC1A KA) and the governor droop (TGOV1 R,
 *            IEESGO K1); zero for the other parameters.  May be NULL.
 *   grad_z0  [M][n_sys] dJ/dz0 (differential states; the algebraic ones are
 *            determined by the first solve and get zero).  May be NULL.
 *   status   [M] as gp_integrate, for the forward run.  May be NULL.
 * opt->solver must be GP_SOLVER_SCHUR_FP64.  On return the layout holds the
 * final state.  Replaces the reference's GradPower.adjoint(lambda0, dprob,
 * sys, traj, tvec; functional=true) (examples/adjoint.jl:105,
 * test/test_adjoint_event_offset.jl:50-53), whose source is no longer in the
 * reference (src/nlp.jl:50-53). */
int32_t gp_adjoint(gp_layout *L, const gp_options *opt, int32_t n_faults, const gp_fault *faults,
                   const gp_objective *obj, int32_t checkpoint_every, double *J, double *grad_p, double *grad_z0,
                   int32_t *status);

/* Policy of GP_SOLVER_SCHUR_MIXED (no counterpart in the reference, whose
 * solvers refactor every iteration):
 *  - a scenario refreshes its kept FP32 factors at the start of a solve once
 *    they have served max_age solves, and after an iteration that reduced
 *    the residual by less than the factor rho_max; refreshes are taken
 *    together (when one scenario refreshes, every scenario on kept factors
 *    does: the factorisation launch costs the same);
 *  - a scenario still iterating after exact_after iterations of one solve
 *    takes exact Newton steps with fresh FP64 factors until that solve ends
 *    (its kept factors are refreshed at the next solve), so that a system
 *    too ill-conditioned for FP32 factors converges as in
 *    GP_SOLVER_SCHUR_FP64; a solve that still ends at itermax (or on a
 *    non-finite residual) after inexact steps is redone from the step's
 *    starting point with exact Newton steps only, and that outcome is the
 *    one reported;
 *  - predict = p > 0 starts every step from the polynomial extrapolation,
 *    of degree at most p (1 linear, 2 quadratic, 3 cubic), through the
 *    previous states that lie on the current smooth stretch (no event
 *    re-solve in between) instead of from the previous state: the same
 *    backward-Euler equations and convergence test, a closer initial
 *    iterate; predict = 0 starts from the previous state.
 * Defaults: max_age 1, rho_max 0.9, exact_after 8, predict 3. */
int32_t gp_set_mixed_policy(gp_layout *L, int32_t max_age, double rho_max, int32_t exact_after, int32_t predict);

/* gp_residual with no fault applied, computed without allocating anything,
 * for callers that may not call cudaMalloc or cudaFree: a host whose device
 * memory is all handed out by its own pool allocator, or a loop in which the
 * implicit device synchronisation of those calls is not allowed.  Its
 * scratch (zold, residual, cluster and network intermediates) lives in one
 * file-scope 16 MiB device array instead of the layout's buffers.
 * f[M][n_sys] as gp_residual(L, zold, dt, 0, NULL, NULL, f).  Returns
 * GP_E_INVALID when the scratch, 8 M (2 n_sys + 3 (n_diff + n_alg) +
 * 8 machine clusters + n_var + n_red) bytes plus a few small arrays, each
 * rounded up to 256 bytes, exceeds the 16 MiB (n_var: the scenario-varying
 * entries of S, 4 per bus plus 4 or 6 per PV or slack static generator;
 * n_red: 2 per bus plus the static generators' algebraic states).  The first
 * call on a device looks up the array's address: make it before any stream
 * capture.  The array is shared by every layout on the device and keeps
 * the last call's contents, so overlapping calls race.
 * No counterpart in the reference. */
int32_t gp_residual_static(gp_layout *L, const double *zold, double dt, double *f);

/* Host-only check of the reduced-system machinery, needs no GPU: builds the
 * same symbolic analysis and front assembly lists as gp_layout_create, takes
 * the diagonal blocks and static-generator couplings of S from the given
 * CSR matrix (reduced indexing: 2b, 2b+1 for bus b, then static-generator
 * states), factors and solves S x = rhs on the host with the operation order
 * of the device kernels: the level-order solves, and the blocked solves of
 * the triangular-solve kernels with their shared-memory staging indices
 * checked against the block maxima (GP_E_INTERNAL when one falls outside).
 * x receives the blocked solve's solution.  out[0] max |S - (-Ybus)| over
 * off-diagonal blocks, out[1] zero pivots, out[2] nnz(L+U), out[3]
 * elimination-tree levels, out[4] max |x_blocked - x_levels| / max |x|,
 * out[5] solve blocks, out[6] levels of the top region, out[7] most
 * supernodes in one block, out[8] max |S^T y - rhs| / max |y| for S^T
 * factored from the transposed assembly lists of the adjoint, out[9]
 * largest front of the top region (0 when every supernode is in a block),
 * out[10] most vector entries one block stages, out[11] max |difference|
 * between the factors with the large fronts near the root split over
 * several CTAs (the FP64 factorisation's parts, emulated on the host) and
 * without (0: the same bits).
 * No counterpart in the reference: a test hook for the analysis that
 * replaces cuDSS's. */
int32_t gp_reduced_selftest(const gp_problem *prob, const int32_t *s_rowptr, const int32_t *s_colidx,
                            const double *s_val, const double *rhs, double *x, double out[12]);

/* Device check of the reciprocal the FP64 factorisations take of each pivot
 * (the hardware's approximate reciprocal refined by two Newton-Raphson
 * steps, the division for zero, subnormal, very large, infinite and NaN
 * pivots): r[i] = that reciprocal of x[i], i < n, computed on the current
 * device.  No counterpart in the reference: a test hook that bounds the
 * reciprocal against the correctly rounded 1/x. */
int32_t gp_recip_check(int32_t n, const double *x, double *r);

/* Host-only check of the cluster factorisation, needs no GPU: builds the
 * class plans of gp_layout_create from (z, u0, p) of one scenario and runs
 * every non-trivial cluster's program on the host in the device kernel's
 * operation order.  yx[3][n_diff+n_alg] receives A_k^-1 f_k, A_k^-1 B_k(:,vr),
 * A_k^-1 B_k(:,vi) at the cluster's states; clout[n_nontrivial][8] the
 * per-cluster outputs (C A^-1 B as 4 values, C A^-1 f as 2, bus injection
 * as 2); f (may be NULL) the backward-Euler residual of the cluster rows.
 * out[0] max |f| over cluster rows, out[1] classes, out[2] FMAs of all
 * cluster factorisations, out[3] maximum slots of a class.
 * No counterpart in the reference: a test hook for the static-pivot sparse
 * factorisation that replaces the dense per-cluster getrf
 * (src/schur.jl:436-493). */
int32_t gp_cluster_selftest(const gp_problem *prob, const double *z, const double *zold, const double *u0,
                            const double *p, double dt, double *yx, double *clout, double *f, double out[4]);

#ifdef __cplusplus
}
#endif

#endif /* GRADPOWER_GB300_H */
