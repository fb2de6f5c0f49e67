// Internal declarations shared by the host orchestration (gp_api.cu) and
// the device kernels (gp_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gp_devices.cuh"

namespace gp {

// Struct-of-arrays device table on the GPU (see gp_device_table).
struct DTab {
    int n;
    const int *bus, *diff_ptr, *alg_ptr, *ctrl_ptr, *par_ptr, *link0, *link1;
};

// Everything the kernels read about the problem.  All pointers are device
// pointers; per-scenario arrays are scenario-major.
struct DevProblem {
    int n_bus, n_diff, n_alg, n_ctrl, n_par, n_sys, net, n_red;
    int M;
    // complex Ybus, CSR; each entry's (G, B) in one 16-byte pair
    const int *y_rowptr, *y_colidx;
    const double2 *y_val;
    DTab dev[8];
    const uint8_t *is_diff;
    // clusters (non-trivial only are processed by the cluster kernel)
    int n_cl;
    const int *cl_w_start, *cl_w_size, *cl_gen, *cl_gov_type, *cl_gov, *cl_exc_type, *cl_exc, *cl_pss;
    // per bus: non-trivial clusters, ZIP loads, static generators
    const int *bus_cl_ptr, *bus_cl, *bus_zl_ptr, *bus_zl, *bus_sg_ptr, *bus_sg;
    const int *bus_order;  // [n_bus] buses sorted by (static generators, loads, clusters, Ybus row length)
    // static generators in the reduced system
    const int *sg_red;     // [n_sg] reduced index of the first alg state (or -1)
    const int *sg_var;     // [n_sg] first index of its coupling entries in the var block
    int n_var;             // per-scenario variable entries of S: 4*n_bus + sg entries
    // faults expanded per scenario
    const int *fl_ptr;     // [M+1]
    const int *fl_bus;
    const double *fl_yf;   // 1/rfault
    const uint8_t *fl_on;  // current status
    // line trips expanded per scenario (gp_set_line_trips)
    int n_tr;
    const int *tr_ptr;     // [M+1]
    const int *tr_from, *tr_to;
    const double *tr_y;    // [n_tr][8]: yff, yft, ytf, ytt (re, im)
    const uint8_t *tr_on;  // current status (tripped)
    // device disconnections (gp_set_device_disconnects): 1 = offline; null
    // when none are set
    const uint8_t *zl_off;   // [M][n ZIP loads]
    const uint8_t *sg_off;   // [M][n static generators]
    const uint8_t *exc_off;  // [M][n_cl] the exciter of cluster c
    const double *zl_k;      // [M][n ZIP loads][4] (1 - al) P, (1 - al) Q, al g0, al b0 (launch_zip_const)
    // symbolic permutation of the reduced system
    const int *iperm;      // reduced index -> permuted position
};

// Per-scenario work arrays of the Newton iteration.
struct DevWork {
    double *z, *zold, *u0, *p;      // [M][n_sys], [M][n_sys], [M][n_ctrl], [M][n_par]
    double *yx;                     // [M][3][n_da]: A^-1 f, A^-1 B(:,1), A^-1 B(:,2)
    double *clout;                  // [M][n_cl][8]: D (4), C y (2), injection (2)
    double *svar;                   // [M][n_var]: diagonal blocks and static-generator couplings
    double *xperm;                  // [M][n_red]: right-hand side / solution, permuted
    double *f;                      // [M][n_sys] residual (written when want_f)
    unsigned long long *norm;       // [M] residual infinity norm as ordered bits
    uint8_t *active;                // [M] scenario takes part in this iteration
    int *iters;                     // [M] Newton updates in the current solve
    int *status;                    // [M] 0 ok, 1 itermax reached, 2 non-finite, 4 zero pivot
    int *flag;                      // [4] scenarios still iterating; of those, MX_FP32 and MX_EXACT ones;
                                    //     [3] mixed solver: solves to retry (kept across iterations)
    double *dt;                     // [1] time step of the current solve
};

// Symbolic factor layout on the GPU.
struct DevSym {
    int n, nsup, nlevels;
    const int *sup_start, *row_ptr, *rows, *child_ptr, *children, *relmap_ptr, *relmap;
    const int64_t *front_off, *uvec_off;
    int64_t front_total, uvec_total;
    const int *asmc_ptr, *asmc_pos;   // constant entries: front position, value
    const double *asmc_val;
    const int *asmv_ptr, *asmv_pos, *asmv_idx;   // variable entries: front position, svar index
    // line-trip entries of the off-diagonal bus blocks: front position,
    // trip entry (its scenario and status in DevProblem), value added while
    // the line is tripped; null without trips
    const int *asmt_ptr, *asmt_pos, *asmt_tr;
    const double *asmt_val;
    double *fronts;                   // [M][front_total]
    // solve-ordered copies of the factors, written by the factorisation for
    // the triangular solves: supernode s's L panel (mm x ns, leading
    // dimension mm: unit-lower L below the diagonal, the reciprocal pivots
    // on it, U11 above) in lfac and its U rows (ns x mm, leading dimension
    // ns: U11 and U12) in ufac, both at lu_off[s].  The supernodes of a
    // solve block are consecutive; blocks and top supernodes start on a
    // multiple of 4 entries
    const int64_t *lu_off;
    int64_t lu_total;
    double *lfac, *ufac;              // [M][lu_total] FP64 factors
    double *uvec;                     // [M][uvec_total]
    int *ipiv;                        // [M][n] pivot row within the supernode, per column
    // extend-add of the CTA-sized fronts, by entry ("pull"): for supernode s
    // (-1 when a warp factors it), pa_ptr[pa_base[s] + p] .. [.. + p + 1]
    // are the children's update-matrix entries (offsets in a scenario's
    // fronts) that add into front entry p, in child order; pr_* likewise
    // for the right-hand side (offsets in a scenario's update vectors)
    const int *pa_base, *pa_ptr, *pa_src;
    const int *pr_base, *pr_ptr, *pr_src;
};

// Sparse cluster factorisation plan: clusters grouped into classes with
// identical local Jacobian pattern; each class carries a straight-line
// program (backward-Euler scaling, static-pivot LU, three solves).
struct DevClu {
    int n_tasks;                // warp tasks: up to 32 clusters of one class
    const int *task_class, *task_first, *task_count;
    const int *order;           // cluster indices (into the P.cl_* arrays) grouped by class
    const short *slot_of;       // [class][32*32] slot of local entry (r, c); c = 29/30 B, 31 f
    const int *prog_ptr;        // [n_class+1]
    const int *prog_mid;        // [n_class] first op of the factorisation part
    const int *prog_sol;        // [n_class] first op of the solve part (after the factorisation)
    const CluOp *ops;
    const int *rhs_base;        // [n_class] first right-hand-side slot
    const int *nslot;           // [n_class] slots used (values + pivots + 3 W)
    const int *perm_col;        // [class][32] state (local) of solution position j
    const int *pos3;            // [class][3] solution positions of delta, i_q, i_d
    const int *row_pos;         // [class][32] position of local row r in the program
    int max_slots;
    int max_w;                  // widest class
    // adjoint: when set, the cluster kernel also saves its FP64 LU values
    // ([M][n_tasks][n_save][32]) and the coupling rows C ([M][n_cl][6])
    double *save_lu, *save_cc;
    int n_save;
};

// Factor reuse of the mixed-precision solver (GP_SOLVER_SCHUR_MIXED).  The
// cluster blocks' LU values and the reduced-system factors are kept in FP32
// and reused across Newton iterations; every iteration evaluates the
// residual in FP64 and applies the kept factors to it.  Per scenario and
// iteration, refac[m] selects the linear solve:
//   0 (MX_KEEP)    the kept FP32 factors;
//   1 (MX_FP32)    fresh factors (FP64 Jacobian at the current iterate),
//                  stored in FP32 and kept;
//   2 (MX_EXACT)   fresh FP64 factors, used once (exact Newton); a scenario
//                  still iterating after exact_after iterations of one
//                  solve uses these until the solve ends, and refreshes its
//                  kept factors at the next solve.
enum { MX_KEEP = 0, MX_FP32 = 1, MX_EXACT = 2 };
struct DevMixed {
    int on;                // 0: exact Newton with fresh FP64 factors every iteration
    int n_lu;              // LU slots kept per cluster (maximum over classes)
    int max_age;           // Newton solves a factor set may serve before a refresh
    int exact_after;       // iterations of one solve after which a scenario uses FP64 factors
    double rho_max;        // residual contraction above which the factors are refreshed
    uint8_t *refac;        // [M] mode of this iteration (MX_*)
    uint8_t *refac_next;   // [M] mode of the next iteration
    uint8_t *prev_mode;    // [M] mode of the previous iteration (the step just taken)
    int *age;              // [M] Newton solves since the last refresh
    uint8_t *all_exact;    // [M] every iteration of this solve is exact (a retry)
    uint8_t *retry;        // [M] this solve failed with inexact steps: redo it exactly
    double *prev_norm;     // [M] residual norm of the previous iteration
    float *lu;             // [M][n_tasks][n_lu][32] cluster LU values and pivot reciprocals
    float *cc;             // [M][n_cl][6] coupling rows of the network equations
    float *fronts;         // [M][front_total] reduced-system fronts (update matrices for the assembly)
    float *lfac, *ufac;    // [M][lu_total] solve-ordered FP32 factors (DevSym::lu_off)
    double *kc;            // [M][n_tasks][kConstSlots][32] parameter constants of the cluster devices
};

// Dataflow schedule of the multifrontal factorisation and solves
// (gp_dag.cu).  order: supernodes of the small region (every front of the
// subtree at most 32 rows) by level, then the others by level; a topological
// order of the assembly tree.
struct DevDag {
    int nsup, n_small;
    int n_tiny;                   // the first n_tiny ranks: subtrees with fronts of at most dag_tiny_front() rows
    int max_front, max_big_front;
    int max_big_whole;            // largest front of the CTA kernel that is not split (FP64)
    const int *order;       // [nsup]
    const int *rank;        // [nsup] position in order
    const int *parent;      // [nsup] parent supernode or -1
    int *ctr;               // [8] claim counters: small factor, big factor, forward top, backward top,
                            //     forward blocks, backward blocks, forward lower top, tiny factor
    int *epoch;             // [1] current solve
    int *err;               // [1] a wait gave up (sticky until the host clears it)
    int *fdone, *xdone, *bdone;   // [nsup][M] epoch at which the task finished
    // Solves on FP32 factors hand values between tasks as tagged words
    // (value, epoch) instead of done flags: utag mirrors uvec (the forward
    // solve's update vectors), xtag mirrors xperm (the backward solve's
    // entries of the top region).  Zero-filled at creation; epochs start at 1.
    unsigned long long *utag;     // [M][uvec_total]
    unsigned long long *xtag;     // [M][n_red]
    int wait_limit = 1 << 20;     // polls before a wait gives up (gp_set_wait_limit)
    // Split fronts (FP64 factorisations): the large fronts near the root of
    // the assembly tree, where few tasks can run at once, are factored by
    // several CTAs together (gp_dag.cu, factor_part).  The last n_tail ranks of `order`
    // (from rank tail0) form the tail; a tail supernode s has nparts[s]
    // parts (1: one CTA as elsewhere), each part a task of its own, the
    // parts of one (supernode, scenario) claimed one after the other.
    int tail0 = 0, n_tail = 0;
    int big_units = 0;            // tasks of the CTA kernel per scenario: ranks below the tail, tail parts
    const int *tail_units;        // [n_tail+1] cumulative parts of the tail ranks
    const uint8_t *nparts;        // [nsup] parts of each front
    int *pdone;                   // [n_tail][M][kMaxParts] epoch at which each part finished
    int *pflag;                   // [n_tail][M][max_panels] epoch at which each panel was published
    int *ppiv;                    // [n_tail][M][max_split_ns] the panels' pivot rows
    void *pbuf;                   // [M][pb_total] published panels (factor type, sized for double)
    const int64_t *pb_off;        // [n_tail] offset of a supernode's panels in a scenario's pbuf
    int64_t pb_total = 0;
    int max_panels = 1, max_split_ns = 1;
    int max_part_entries = 0;     // factor entries of the largest part's shared memory
    int max_part_ints = 0;        // and its pivot integers
};

// Split fronts: at most kMaxParts parts; panels of kSplitPanel pivot
// columns, owned by the parts in turn (block-cyclic columns).
constexpr int kMaxParts = 8;
constexpr int kSplitPanel = 8;
constexpr int kSplitTailMax = 96;   // ranks of the tail

// Column j of a front split in np parts belongs to part (j / kSplitPanel) %
// np.  A part keeps its columns in increasing order: split_owned_below(j)
// of them lie left of column j, and its local column jl is front column
// split_col(jl).  split_cols_cap(nc, np) bounds a part's columns.
__host__ __device__ inline int split_owner(int j, int np) { return (j / kSplitPanel) % np; }
__host__ __device__ inline int split_owned_below(int j, int part, int np) {
    const int per = kSplitPanel * np, full = j / per, rem = j - full * per;
    const int t = rem - part * kSplitPanel;
    return full * kSplitPanel + (t < 0 ? 0 : (t > kSplitPanel ? kSplitPanel : t));
}
__host__ __device__ inline int split_col(int jl, int part, int np) {
    return ((jl / kSplitPanel) * np + part) * kSplitPanel + jl % kSplitPanel;
}
__host__ __device__ inline int split_cols_cap(int nc, int np) {
    const int per = kSplitPanel * np;
    return (nc + per - 1) / per * kSplitPanel;
}

struct DagGrid {
    int tiny = 0, small = 0, big = 0;                    // resident blocks
    int tiny_bytes = 0, small_bytes = 0, big_bytes = 0;  // dynamic shared memory
};

int dag_configure(const DevDag &D, int fp32, DagGrid &g);
// launch_dag_factor<double> also does the forward solve (the right-hand side
// rides along as an extra front column); launch_dag_factor<float> does not.
int dag_small_front();
int dag_tiny_front();
void launch_dag_begin(const DevDag &D, cudaStream_t st);
// r[i] = the factorisations' reciprocal of x[i] (device arrays), i < n.
void launch_recip_check(const double *x, double *r, int n, cudaStream_t st);
// Factors the scenarios m with mask[m] == want: fronts (update matrices) and
// the solve-ordered copies lfac, ufac ([M][lu_total]); lfac may be null when
// no forward solve will read it (the FP64 factorisation's own forward solve
// is fused).
template <class T>
void launch_dag_factor(const DevProblem &P, const DevWork &W, const DevSym &S, const DevDag &D, const DagGrid &g,
                       T *fronts, T *lfac, T *ufac, const uint8_t *mask, int want, cudaStream_t st);
// Split of the assembly tree for the triangular solves (gp_solve.cu).
// Blocks are subtrees solved by one warp each from shared memory; their
// entries are the block's supernodes, children before parents, the last
// entry of a block being its root:
//   ent0 = {supernode, first column, pivots ns, update rows r}
//   ent1 = {-, vector offset, map offset, pivot offset}
// (offsets within the block's shared-memory staging area; map offsets
// relative to the block's first map entry).  The supernodes above the blocks
// form the top region, solved by a dataflow kernel.
struct DevBlk {
    int nblk;
    int max_n, max_v, max_p, max_map;   // per-block maxima
    const int *blk_ptr;          // [nblk+1]
    const int4 *ent0, *ent1;
    const int *map_ptr;          // [nblk+1]
    const int *map_fwd;          // per update row: parent vector position (forward push)
    const int *map_bwd;          // per update row: vector position of that row's solution
    const int *ext_ptr;          // [nblk+1]
    const int *ext_pos, *ext_row;   // solution entries above the block: vector position, xperm row
    // per block, its pivot columns in member order (entry e is pivot slot
    // e) and each one's position in the block's vector
    const int *pcol_ptr;         // [nblk+1]
    const int *pcol, *pvs;
    int n_top, top_max_front;
    int n_lower_top;             // the first n_lower_top entries of top_order: one warp per forward task
    int top_max_xent;            // most extend-add entries of one top supernode
    const int *top_order;        // [n_top] top supernodes, children before parents
    const int *top_rank;         // [nsup] position in top_order, -1 inside a block
    // forward extend-add of the top region, per top supernode (by rank) and
    // front row: the children's update-vector entries (offsets within a
    // scenario's uvec) that add into the row, in child order
    const int *top_xptr;         // [n_top+1] first row pointer of each top supernode
    const int *top_xrow;         // row pointers into top_xent
    const int *top_xent;
};

// Factors of the triangular solves, per scenario: FP64 when f32 is null or
// the scenario's mode is MX_EXACT, else FP32.  With fused64 set, the forward
// solve skips the FP64 scenarios (their factorisation did it).
struct FrontSel {
    const float *l32, *u32;     // solve-ordered FP32 factors (DevSym::lu_off), null: FP64 only
    const double *l64, *u64;    // solve-ordered FP64 factors
    const uint8_t *mode;
    int fused64;
    int shared;    // every scenario solves with scenario 0's factors (shared-factor Woodbury path)
};

struct SolveGrid {
    int blk_bytes = 0, top_bytes = 0;   // dynamic shared memory per CTA
    int top_fwd = 0, top_bwd = 0;       // resident CTAs of the dataflow kernels
};

int solve_configure(const DevBlk &B, SolveGrid &g);
void launch_solve_fwd(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const DevDag &D,
                      const SolveGrid &g, FrontSel fs, cudaStream_t st);
void launch_solve_bwd(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const DevDag &D,
                      const SolveGrid &g, FrontSel fs, cudaStream_t st);
// Largest front the solves' register path handles in a block (rows).
int solve_block_front_limit();

// launches (gp_kernels.cu)
// Device initialisation of every scenario from solved power flows
// (gp_init.cu): writes W.z, W.u0 and the derived entries of W.p; *bad
// counts machines whose initialisation residual stayed at or above 1e-9.
void launch_initialize(const DevProblem &P, const DevWork &W, const double *vpol, const double *gen_pq,
                       const double *sg_pq, int *bad, cudaStream_t st);
// Device disconnections taking effect at `step`: flags[idx[e]] = 1 and the
// scenario marked active for the dt = 0 re-solve.
void launch_disconnects(const int *on_step, const int *scen, const int *idx, uint8_t *flags, uint8_t *active,
                        int n, int step, cudaStream_t st);
// Parameter products of the ZIP loads for network_kernel; rerun whenever
// the parameter vectors change.
void launch_zip_const(const DevProblem &P, const DevWork &W, double *out, cudaStream_t st);
// Parameter constants of the cluster devices for cluster_keep_kernel.
void launch_cluster_const(const DevProblem &P, const DevWork &W, const DevClu &C, const DevMixed &Mx,
                          cudaStream_t st);
int launch_cluster(const DevProblem &P, const DevWork &W, const DevClu &C, const DevMixed &Mx, int want_f,
                    cudaStream_t st);
// skip_s: the entries of S are not needed (shared-factor Woodbury path)
void launch_network(const DevProblem &P, const DevWork &W, const DevMixed &Mx, int want_f, cudaStream_t st,
                    int skip_s = 0);

// Shared-factor Woodbury path: per scenario, its fault (one bus and
// admittance, possibly several on/off windows) is a rank-2 change of the
// shared reduced matrix P.  wb_unit: xperm[m] = the unit vector at the
// fault bus's vr (col 0) or vi (col 1) row, zero without a fault.
// wb_setup: H = U^T W - I/yf and its inverse per scenario.  wb_correct: the
// Woodbury correction of the solution x = P^-1 rhs of the scenarios whose
// fault is on, x -= W H^-1 U^T x.
void launch_wb_unit(const DevProblem &P, const DevWork &W, int col, cudaStream_t st);
void launch_wb_setup(const DevProblem &P, const double *W1, const double *W2, double *Hinv, cudaStream_t st);
void launch_wb_correct(const DevProblem &P, const DevWork &W, const double *W1, const double *W2,
                       const double *Hinv, double *s, cudaStream_t st);
// Control of a Newton loop run on the device (a CUDA graph whose WHILE node
// repeats solve + evaluation): the check kernel sets the loop condition
// (some scenario still iterating) and, for the mixed solver, the SWITCH
// value that picks the next solve's factorisations (bit 0 FP32 refresh,
// bit 1 FP64), and counts into cnt: [0] evaluations, [1] solves, [2]
// scenario FP32 refreshes, [3] scenario FP64 iterations, [4 + v] solves of
// variant v.  on == 0 for the host-driven loop.
struct LoopCtl {
    cudaGraphConditionalHandle loop, var;
    int *cnt;
    int on, mixed;
};

void launch_check(const DevProblem &P, const DevWork &W, const DevMixed &Mx, double tol, int itermax,
                  const LoopCtl &ctl, cudaStream_t st);
void launch_reset_norm(const DevProblem &P, const DevWork &W, const DevMixed &Mx, cudaStream_t st);
void launch_mixed_start(const DevProblem &P, const DevWork &W, const DevMixed &Mx, int force, cudaStream_t st);
void launch_retry_start(const DevProblem &P, const DevWork &W, const DevMixed &Mx, cudaStream_t st);
// Start of a step of the mixed solver: the first iterate z from the
// polynomial extrapolation of order `order` through zold, zprev, zprev2,
// zprev3 (0 none, 1 linear, 2 quadratic, 3 cubic), then the history shifts:
// zprev3 <- zprev2 <- zprev <- zold.
void launch_predict(double *z, const double *zold, double *zprev, double *zprev2, double *zprev3, size_t n,
                    int order, cudaStream_t st);
void launch_update(const DevProblem &P, const DevWork &W, const DevSym &S, const int *perm, cudaStream_t st);
void launch_events(const DevProblem &P, const DevWork &W, const int *fl_on_step, const int *fl_off_step,
                   const int *fl_scen, uint8_t *fl_on, int n_fl, int step, cudaStream_t st);
void launch_snapshot(const double *z, double *traj, int M, int n_sys, int n_steps, int k, cudaStream_t st);
int cluster_smem_optin(int bytes);

// Discrete adjoint of the backward-Euler step (gp_adjoint.cu).
struct DevAdj {
    double *g;            // [M][n_sys] right-hand side of J^T lambda = g; after a step, E lambda
    double *lam;          // [M][n_sys] lambda of the last backward solve
    double *cadj;         // [M][n_cl][2] (A^-1 B)^T g_w per cluster
    double *grad;         // [M][n_par] dJ/dp
    double *J;            // [M] objective
    const int *gen_w;     // [n_gen] z index of every machine's speed
    int n_gen;
    double w_speed, w_volt, v_min;   // objective weights and the voltage floor
};
void launch_adj_objective(const DevProblem &P, const DevWork &W, const DevAdj &A, double dt, cudaStream_t st);
void launch_adj_rhs(const DevProblem &P, const DevWork &W, const DevClu &C, const DevAdj &A, cudaStream_t st);
void launch_adj_back(const DevProblem &P, const DevWork &W, const DevClu &C, const DevAdj &A, const int *state_maps,
                     cudaStream_t st);
int adj_smem_optin(int bytes);
void launch_set_double(double *dst, double v, cudaStream_t st);
void launch_fault_status(const DevProblem &P, const int *fl_on_step, const int *fl_off_step, uint8_t *fl_on,
                         int n_fl, int upto, cudaStream_t st);

}  // namespace gp
