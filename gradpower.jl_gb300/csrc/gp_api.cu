// C-ABI entry points and host orchestration of the batched backward-Euler
// Newton step (see include/gradpower_gb300.h).
//
// Host side of the reference's GpuBatchedLayout constructor
// (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:466-945) and of the time loops of
// integrate_gpu_schur_cudss! / integrate_gpu_cudss!
// (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2924-3080): everything is
// uploaded once, the symbolic analysis of the reduced network matrix runs
// once, and each Newton iteration is two captured CUDA graphs (evaluate,
// solve) with one 4-byte readback of the number of scenarios still
// iterating.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gradpower_gb300.h"
#include "gp_internal.h"
#include "gp_symbolic.h"
#include "gp_cluster_plan.h"

namespace {

thread_local std::string g_last_error;

struct gp_error : std::runtime_error {
    int code;
    gp_error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw gp_error(code, buf);
}

void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) fail(GP_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Device allocations of one lifetime.  Uploads go through the layout's
// stream `st` and are complete on return: that stream does not wait for the
// legacy default stream (cudaStreamNonBlocking), so a plain cudaMemcpy would
// not be ordered before the kernels launched on it.
struct DeviceArena {
    std::vector<void *> ptrs;
    cudaStream_t st = nullptr;
    template <class T>
    T *alloc(size_t n) {
        void *p = nullptr;
        if (n == 0) n = 1;
        cudaError_t e = cudaMalloc(&p, n * sizeof(T));
        if (e != cudaSuccess) fail(GP_E_NOMEM, "cudaMalloc of %zu bytes: %s", n * sizeof(T), cudaGetErrorString(e));
        ptrs.push_back(p);
        return (T *)p;
    }
    template <class T>
    T *upload(const std::vector<T> &v) {
        return upload(v.data(), v.size());
    }
    template <class T>
    T *upload(const T *v, size_t n) {
        T *p = alloc<T>(n);
        if (n && v) {
            ck(cudaMemcpyAsync(p, v, n * sizeof(T), cudaMemcpyHostToDevice, st), "upload");
            ck(cudaStreamSynchronize(st), "upload");
        }
        return p;
    }
    void release() {
        for (void *p : ptrs) cudaFree(p);
        ptrs.clear();
    }
};

std::vector<int> vec(const int32_t *p, int n) {
    std::vector<int> v(n > 0 ? n : 0);
    if (n > 0 && p) std::copy(p, p + n, v.begin());
    return v;
}

}  // namespace

struct gp_layout {
    int M = 0;
    int device = 0;        // CUDA device the layout lives on (current at gp_layout_create)
    int n_sys = 0, n_da = 0, n_red = 0, n_bus = 0, n_ctrl = 0, n_par = 0;
    gp::DevProblem P{};
    gp::DevWork W{};
    gp::DevSym S{};
    gp::DevSym ST{};   // S^T: the same structure and buffers, transposed assembly lists (adjoint)
    gp::Symbolic sym;
    DeviceArena arena;     // lifetime of the layout
    DeviceArena call;      // lifetime of one gp_integrate call
    cudaStream_t st = nullptr;
    // trajectory snapshots of gp_integrate (kept between calls, grown on
    // demand) and the stream that copies them to a pinned host buffer while
    // the following steps run
    DeviceArena traj_arena;
    double *d_traj = nullptr;
    size_t traj_cap = 0;
    cudaStream_t st_copy = nullptr;
    cudaEvent_t ev_snap = nullptr;
    double *d_zl_k = nullptr;   // DevProblem::zl_k
    int *d_state_maps = nullptr;   // state_bus then red_of
    int *d_gen_w = nullptr;        // z index of every machine's speed deviation
    int n_gen = 0;
    int *h_flag = nullptr;         // pinned
    double *h_dt = nullptr;        // pinned
    // faults of the current call
    int n_fl = 0;
    int *d_fl_on_step = nullptr, *d_fl_off_step = nullptr, *d_fl_scen = nullptr;
    uint8_t *d_fl_on = nullptr;
    std::vector<int> h_fl_on_step, h_fl_off_step, h_fl_scen;
    // graphs
    cudaGraphExec_t g_eval = nullptr, g_solve = nullptr;
    // device-driven Newton loop (profiling off): eval, then WHILE(some
    // scenario iterates) { solve; eval }, the solve picked by a SWITCH node
    // for the mixed solver; counts into d_cnt (gp::LoopCtl)
    cudaGraphExec_t g_loop = nullptr;
    cudaGraphConditionalHandle h_loop = 0, h_var = 0;
    int *d_cnt = nullptr;
    bool profiling = false;      // host-driven loop with phase events (gp_set_profiling)
    // line trips (gp_set_line_trips): expanded per scenario, with their
    // off-diagonal assembly entries; statuses reset at every call
    DeviceArena trip_arena;
    int n_tr = 0;
    uint8_t *d_tr_on = nullptr;
    int *d_tr_on_step = nullptr, *d_tr_off_step = nullptr, *d_tr_scen = nullptr;
    std::vector<int> h_tr_on_step, h_tr_off_step;
    std::vector<int> h_adj_ptr, h_adj;   // bus adjacency (line trips are checked against it)
    // fault table (set_faults; grow-only, see there) and the per-step
    // iteration counts of gp_integrate (grow-only)
    DeviceArena fault_arena;
    int fl_cap = 0;
    int *d_fl_ptr = nullptr, *d_fl_bus = nullptr;
    double *d_fl_yf = nullptr;
    DeviceArena iters_arena;
    int *d_iters_buf = nullptr;
    size_t iters_cap = 0;
    // device disconnections (gp_set_device_disconnects): offline flags of
    // ZIP loads, static generators and cluster exciters per scenario (zeroed
    // at every call), and the events as (flag index, scenario, step)
    DeviceArena dc_arena;
    int n_dc = 0;
    size_t dc_bytes = 0;
    uint8_t *d_dc_flags = nullptr;
    int *d_dc_on_step = nullptr, *d_dc_scen = nullptr, *d_dc_idx = nullptr;
    std::vector<int> h_dc_on_step;
    std::vector<int> h_cl_ext, h_cl_ex, h_sg_type;   // cluster exciters; static generator bus types
    int h_ntab[GP_NTYPES] = {};
    // shared-factor Woodbury path (allocated on first use): W = P^-1 U per
    // scenario (two columns), H^-1 (2x2), the correction's coefficients, and
    // the mask that selects scenario 0 for the factorisation of P
    double *wb_W1 = nullptr, *wb_W2 = nullptr, *wb_Hinv = nullptr, *wb_s = nullptr;
    uint8_t *d_only0 = nullptr;
    int solve_graph_factors = 0;   // factorisation launches of the non-mixed solve graph
    bool no_marks = false;       // capturing into a conditional body: no event nodes
    double graph_tol = -1.0;
    int graph_itermax = -1;
    // timing of the last integrate call
    double t_total_ms = 0.0, iters_total = 0.0, launches = 0.0;
    // phase timing: events recorded as nodes of the captured graphs
    // 0 before cluster, 1 after cluster, 2 after network,
    // 3 before factor, 4 after factor, 5 after forward, 6 after backward, 7 after update
    cudaEvent_t pev[8] = {};
    double ph_ms[8] = {};        // 0 cluster, 1 network, 2 factor, 3 forward, 4 backward, 5 update
    double factor_launches = 0.0, solves = 0.0;
    double *z_init = nullptr;    // z0 as given to gp_layout_create
    int64_t sum_w2 = 0;
    int64_t nnz_s = 0;           // structural nonzeros of the reduced matrix S
    // sparse cluster factorisation
    gp::ClusterPlan cplan;
    gp::DevClu C{};
    // dataflow schedule of the reduced-system factorisation and solves
    gp::DevDag D{};
    gp::DagGrid G64, G32;
    gp::DevBlk B{};
    gp::SolveGrid SG;
    int n_top_levels = 0;
    // mixed-precision solver: kept FP32 factors (allocated on first use)
    gp::DevMixed Mx{};
    bool mixed_ready = false;
    int solver = -1;                          // solver the graphs were captured for
    // mixed: solve graphs by the modes present in an iteration (bit 0: some
    // scenario refreshes its FP32 factors, bit 1: some scenario uses FP64)
    cudaGraphExec_t g_mix[4] = {};
    int solve_graph_launches = 0, mix_launches[4] = {}, mix_factor_launches[4] = {};
    int eval_launches = 4;        // kernels of the evaluation graph
    double refreshes = 0.0;                   // mixed: scenario FP32 factor refreshes in the last call
    double exact_iters = 0.0;                 // mixed: scenario iterations with FP64 factors
    double retries = 0.0;                     // mixed: scenario solves redone exactly
    int mx_max_age = 1, mx_exact_after = 8;   // mixed solver policy (gp_set_mixed_policy)
    double mx_rho_max = 0.9;
    int mx_predict = 3;                       // mixed: extrapolation order of the step's first iterate
    double *zprev = nullptr, *zprev2 = nullptr, *zprev3 = nullptr;   // mixed: states at the start of the last steps
};

namespace {

// Copies and fills issued by the entry points, all on the layout's stream
// (ordered with its kernels and graphs).  to_device and to_host return with
// the copy complete, so the caller's host buffer is free again; fill is
// asynchronous.
void to_device(const gp_layout *L, void *d, const void *h, size_t bytes, const char *what) {
    if (!bytes) return;
    ck(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, L->st), what);
    ck(cudaStreamSynchronize(L->st), what);
}
void to_host(const gp_layout *L, void *h, const void *d, size_t bytes, const char *what) {
    if (!bytes) return;
    ck(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, L->st), what);
    ck(cudaStreamSynchronize(L->st), what);
}
void fill(const gp_layout *L, void *d, int value, size_t bytes) {
    if (bytes) ck(cudaMemsetAsync(d, value, bytes, L->st), "memset");
}

// Makes the layout's device current for the duration of an entry point.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(const gp_layout *L) {
        int cur = 0;
        ck(cudaGetDevice(&cur), "cudaGetDevice");
        if (cur != L->device) {
            ck(cudaSetDevice(L->device), "cudaSetDevice");
            prev = cur;
        }
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

// Host-side plan of a layout: everything derived from the problem before
// any device allocation (validated cluster tables, reduced-system maps,
// symbolic analysis, front assembly lists).  Also used, without a GPU, by
// gp_reduced_selftest.
struct Plan {
    int nb = 0, net = 0, n_sys = 0, n_red = 0, n_var = 0;
    std::vector<int> ws, wsz, gen, gvt, gv, ext, ex, pss, cbus;
    std::vector<int> state_bus, red_of, sg_red, sg_var;
    std::vector<int> var_r, var_c;          // (row, col) of every variable entry of S
    gp::Symbolic sym;
    std::vector<int> acp, acpos, avp, avpos, avidx;
    std::vector<double> acval;
    std::vector<int> t_acp, t_acpos, t_avp, t_avpos, t_avidx;   // the same for S^T
    std::vector<double> t_acval;
    int64_t sum_w2 = 0;
    int64_t nnz_s = 0;       // structural nonzeros of S
};

void check_in_cluster(int c, int w0, int w, int idx, const char *what) {
    if (idx < w0 || idx >= w0 + w)
        fail(GP_E_INVALID, "cluster %d: %s index %d outside the cluster states [%d, %d)", c, what, idx, w0, w0 + w);
}

void make_plan(const gp_problem *pr, Plan &pl) {
    const int nb = pr->n_bus;
    if (nb <= 0 || pr->n_diff < 0 || pr->n_alg < 0 || pr->n_ctrl < 0 || pr->n_par < 0)
        fail(GP_E_INVALID, "bad problem sizes");
    pl.nb = nb;
    pl.net = pr->n_diff + pr->n_alg;
    pl.n_sys = pl.net + 2 * nb;
    const int net = pl.net;
    for (int t = 0; t < GP_NTYPES; t++) {
        const gp_device_table &T = pr->dev[t];
        for (int k = 0; k < T.n; k++) {
            if (T.online && !T.online[k]) fail(GP_E_INVALID, "offline devices are not supported (type %d, row %d)", t, k);
            if (T.bus[k] < 0 || T.bus[k] >= nb) fail(GP_E_INVALID, "type %d row %d: bus out of range", t, k);
            // every parameter a kernel reads lies inside the parameter vector
            static const int par_size[GP_NTYPES] = {14, 12, 8, 7, 10, 19, 9, 4};
            if (T.par_ptr[k] < 0 || T.par_ptr[k] + par_size[t] > pr->n_par)
                fail(GP_E_INVALID, "type %d row %d: par_ptr out of range", t, k);
        }
    }
    for (int q = 0; q < pr->y_nnz; q++)
        if (pr->y_colidx[q] < 0 || pr->y_colidx[q] >= nb) fail(GP_E_INVALID, "Ybus column out of range");
    // ---- clusters: non-trivial ones go to the cluster kernel ----
    pl.state_bus.assign(net, -2);
    pl.red_of.assign(net, -1);
    const gp_device_table &G = pr->dev[GP_GENROU];
    for (int c = 0; c < pr->n_clusters; c++) {
        const int w0 = pr->cl_w_start[c], w = pr->cl_w_size[c];
        if (w0 < 0 || w < 0 || w0 + w > net) fail(GP_E_INVALID, "cluster %d outside the state vector", c);
        if (pr->cl_gen[c] < 0) continue;   // static generator: reduced unknowns
        if (w > 29) fail(GP_E_INVALID, "cluster %d has %d states; at most 29 are supported", c, w);
        const int g = pr->cl_gen[c];
        if (g >= G.n) fail(GP_E_INVALID, "cluster %d: generator index out of range", c);
        if (G.bus[g] != pr->cl_bus[c]) fail(GP_E_INVALID, "cluster %d: bus differs from its machine's", c);
        check_in_cluster(c, w0, w, G.diff_ptr[g], "GENROU diff");
        check_in_cluster(c, w0, w, G.diff_ptr[g] + 5, "GENROU diff");
        check_in_cluster(c, w0, w, G.alg_ptr[g], "GENROU alg");
        check_in_cluster(c, w0, w, G.alg_ptr[g] + 3, "GENROU alg");
        if (G.link0[g] >= 0) check_in_cluster(c, w0, w, G.link0[g], "GENROU p_m");
        else if (G.ctrl_ptr[g] < 0 || G.ctrl_ptr[g] + 1 >= pr->n_ctrl) fail(GP_E_INVALID, "cluster %d: GENROU ctrl_ptr", c);
        if (G.link1 && G.link1[g] >= 0) check_in_cluster(c, w0, w, G.link1[g], "GENROU e_fd");
        else if (G.ctrl_ptr[g] < 0 || G.ctrl_ptr[g] >= pr->n_ctrl) fail(GP_E_INVALID, "cluster %d: GENROU ctrl_ptr", c);
        const int gt = pr->cl_gov_type[c], gi = pr->cl_gov[c];
        if (gt == GP_IEESGO || gt == GP_TGOV1) {
            const gp_device_table &T = pr->dev[gt];
            if (gi < 0 || gi >= T.n) fail(GP_E_INVALID, "cluster %d: governor index", c);
            const int nd = gt == GP_IEESGO ? 5 : 2;
            check_in_cluster(c, w0, w, T.diff_ptr[gi], "governor diff");
            check_in_cluster(c, w0, w, T.diff_ptr[gi] + nd - 1, "governor diff");
            check_in_cluster(c, w0, w, T.alg_ptr[gi], "governor alg");
            if (T.link0[gi] >= 0) check_in_cluster(c, w0, w, T.link0[gi], "governor w");
        } else if (gt != -1) fail(GP_E_INVALID, "cluster %d: bad governor type", c);
        const int et = pr->cl_exc_type[c], ei = pr->cl_exc[c];
        if (et == GP_SEXS || et == GP_ESDC1A) {
            const gp_device_table &T = pr->dev[et];
            if (ei < 0 || ei >= T.n) fail(GP_E_INVALID, "cluster %d: exciter index", c);
            const int nd = et == GP_SEXS ? 2 : 3;
            check_in_cluster(c, w0, w, T.diff_ptr[ei], "exciter diff");
            check_in_cluster(c, w0, w, T.diff_ptr[ei] + nd - 1, "exciter diff");
            if (T.link0[ei] >= 0) check_in_cluster(c, w0, w, T.link0[ei], "exciter v_s");
            if (T.bus[ei] != pr->cl_bus[c]) fail(GP_E_INVALID, "cluster %d: exciter on another bus", c);
        } else if (et != -1) fail(GP_E_INVALID, "cluster %d: bad exciter type", c);
        const int si = pr->cl_pss[c];
        if (si >= 0) {
            const gp_device_table &T = pr->dev[GP_IEEEST];
            if (si >= T.n) fail(GP_E_INVALID, "cluster %d: stabiliser index", c);
            check_in_cluster(c, w0, w, T.diff_ptr[si], "stabiliser diff");
            check_in_cluster(c, w0, w, T.diff_ptr[si] + 6, "stabiliser diff");
            check_in_cluster(c, w0, w, T.alg_ptr[si], "stabiliser alg");
            if (T.link0[si] >= 0) check_in_cluster(c, w0, w, T.link0[si], "stabiliser w");
        }
        pl.ws.push_back(w0);
        pl.wsz.push_back(w);
        pl.gen.push_back(g);
        pl.gvt.push_back(gt);
        pl.gv.push_back(gi);
        pl.ext.push_back(et);
        pl.ex.push_back(ei);
        pl.pss.push_back(si);
        pl.cbus.push_back(pr->cl_bus[c]);
        for (int j = 0; j < w; j++) pl.state_bus[w0 + j] = pr->cl_bus[c];
        pl.sum_w2 += (int64_t)w * w;
    }
    // ---- reduced system: bus voltages then static-generator states ----
    const gp_device_table &SG = pr->dev[GP_STATIC_GEN];
    pl.sg_red.assign(SG.n, -1);
    pl.sg_var.assign(SG.n, 0);
    int n_red = 2 * nb, n_var = 4 * nb;
    pl.var_r.clear();
    pl.var_c.clear();
    for (int b = 0; b < nb; b++)
        for (int q = 0; q < 4; q++) {
            pl.var_r.push_back(2 * b + q / 2);
            pl.var_c.push_back(2 * b + q % 2);
        }
    for (int k = 0; k < SG.n; k++) {
        const int bt = SG.link0[k];
        const int na = bt == 2 ? 1 : (bt == 3 ? 2 : 0);
        if (na) {
            pl.sg_red[k] = n_red;
            for (int j = 0; j < na; j++) {
                const int zi = SG.alg_ptr[k] + j;
                if (zi < 0 || zi >= net) fail(GP_E_INVALID, "static generator %d state outside the state vector", k);
                pl.state_bus[zi] = -1;
                pl.red_of[zi] = n_red + j;
            }
        }
        pl.sg_var[k] = n_var;
        const int vr = 2 * SG.bus[k], vi = vr + 1, a0 = n_red;
        if (bt == 2) {
            const int rr[4] = {a0, a0, vr, vi}, cc[4] = {vr, vi, a0, a0};
            for (int q = 0; q < 4; q++) { pl.var_r.push_back(rr[q]); pl.var_c.push_back(cc[q]); }
            n_var += 4;
        } else if (bt == 3) {
            const int rr[6] = {a0, a0 + 1, vr, vi, vr, vi}, cc[6] = {vr, vi, a0, a0, a0 + 1, a0 + 1};
            for (int q = 0; q < 6; q++) { pl.var_r.push_back(rr[q]); pl.var_c.push_back(cc[q]); }
            n_var += 6;
        }
        n_red += na;
    }
    for (int i = 0; i < net; i++)
        if (pl.state_bus[i] == -2) fail(GP_E_INVALID, "state %d belongs to no cluster", i);
    pl.n_red = n_red;
    pl.n_var = n_var;

    // ---- pattern of S and symbolic analysis ----
    struct Ent { int r, c; int kind; double val; int idx; };   // kind 0 const, 1 var
    std::vector<Ent> ents;
    for (int v = 0; v < n_var; v++) ents.push_back({pl.var_r[v], pl.var_c[v], 1, 0.0, v});
    for (int b = 0; b < nb; b++) {
        for (int q = pr->y_rowptr[b]; q < pr->y_rowptr[b + 1]; q++) {
            const int j = pr->y_colidx[q];
            if (j == b) continue;
            const double g = pr->y_re[q], bb = pr->y_im[q];
            ents.push_back({2 * b, 2 * j, 0, -g, 0});
            ents.push_back({2 * b, 2 * j + 1, 0, bb, 0});
            ents.push_back({2 * b + 1, 2 * j, 0, -bb, 0});
            ents.push_back({2 * b + 1, 2 * j + 1, 0, -g, 0});
        }
        for (int q = pr->adj_rowptr[b]; q < pr->adj_rowptr[b + 1]; q++) {
            const int j = pr->adj_colidx[q];
            if (j < 0 || j >= nb) fail(GP_E_INVALID, "adjacency out of range");
            for (int t = 0; t < 4; t++) ents.push_back({2 * b + t / 2, 2 * j + t % 2, 0, 0.0, 0});
        }
    }
    for (int k = 0; k < SG.n; k++) {
        const int a0 = pl.sg_red[k];
        if (a0 < 0) continue;
        const int na = SG.link0[k] == 2 ? 1 : 2;
        for (int i = 0; i < na; i++)
            for (int j = 0; j < na; j++) ents.push_back({a0 + i, a0 + j, 0, 0.0, 0});
    }
    std::vector<std::vector<int>> adjr(n_red);
    for (const Ent &e : ents) {
        adjr[e.r].push_back(e.c);
        adjr[e.c].push_back(e.r);
    }
    std::vector<int> rp(n_red + 1, 0), ci;
    for (int i = 0; i < n_red; i++) {
        std::sort(adjr[i].begin(), adjr[i].end());
        adjr[i].erase(std::unique(adjr[i].begin(), adjr[i].end()), adjr[i].end());
        rp[i + 1] = rp[i] + (int)adjr[i].size();
        ci.insert(ci.end(), adjr[i].begin(), adjr[i].end());
    }
    std::vector<int> group(n_red);
    for (int i = 0; i < 2 * nb; i++) group[i] = i / 2;
    for (int k = 0; k < SG.n; k++) {
        const int a0 = pl.sg_red[k];
        if (a0 < 0) continue;
        const int na = SG.link0[k] == 2 ? 1 : 2;
        for (int j = 0; j < na; j++) group[a0 + j] = SG.bus[k];
    }
    pl.nnz_s = (int64_t)ci.size();
    gp::Symbolic &sym = pl.sym;
    gp::analyse(n_red, rp, ci, group, nb, sym);
    // ---- assembly lists ----
    auto fpos = [&](int s, int k) -> int {
        const int st0 = sym.sup_start[s], en = sym.sup_start[s + 1];
        if (k >= st0 && k < en) return k - st0;
        auto b = sym.rows.begin() + sym.row_ptr[s], e = sym.rows.begin() + sym.row_ptr[s + 1];
        auto it = std::lower_bound(b, e, k);
        if (it == e || *it != k) fail(GP_E_INVALID, "entry outside the symbolic structure");
        return (en - st0) + (int)(it - b);
    };
    // the lists for S, and for S^T (same pattern, entry (r, c) at front
    // position (c, r)): the adjoint factors S^T with the same kernels
    auto build_lists = [&](bool tr, std::vector<int> &acp, std::vector<int> &acpos, std::vector<double> &acval,
                           std::vector<int> &avp, std::vector<int> &avpos, std::vector<int> &avidx) {
        std::vector<std::vector<std::pair<int, double>>> ac(sym.nsup);
        std::vector<std::vector<std::pair<int, int>>> av(sym.nsup);
        for (const Ent &e : ents) {
            if (e.kind == 0 && e.val == 0.0) continue;
            const int pi = sym.iperm[tr ? e.c : e.r], pj = sym.iperm[tr ? e.r : e.c];
            const int s = sym.sup_of[std::min(pi, pj)];
            const int m = sym.front_m(s);
            const int lin = fpos(s, pi) + fpos(s, pj) * m;
            if (lin < 0 || lin >= m * m) fail(GP_E_INVALID, "assembly position outside its front");
            if (e.kind == 0) ac[s].push_back({lin, e.val});
            else av[s].push_back({lin, e.idx});
        }
        // merge duplicate constant positions (parallel branches share a Ybus entry)
        acp.assign(sym.nsup + 1, 0);
        avp.assign(sym.nsup + 1, 0);
        acpos.clear();
        acval.clear();
        avpos.clear();
        avidx.clear();
        for (int s = 0; s < sym.nsup; s++) {
            std::sort(ac[s].begin(), ac[s].end());
            for (size_t q = 0; q < ac[s].size(); q++) {
                if (q > 0 && ac[s][q].first == ac[s][q - 1].first) acval.back() += ac[s][q].second;
                else { acpos.push_back(ac[s][q].first); acval.push_back(ac[s][q].second); }
            }
            acp[s + 1] = (int)acpos.size();
            std::sort(av[s].begin(), av[s].end());
            for (size_t q = 0; q < av[s].size(); q++) {
                if (q > 0 && av[s][q].first == av[s][q - 1].first) fail(GP_E_INVALID, "duplicate variable entry of S");
                avpos.push_back(av[s][q].first);
                avidx.push_back(av[s][q].second);
            }
            avp[s + 1] = (int)avpos.size();
        }
    };
    build_lists(false, pl.acp, pl.acpos, pl.acval, pl.avp, pl.avpos, pl.avidx);
    build_lists(true, pl.t_acp, pl.t_acpos, pl.t_acval, pl.t_avp, pl.t_avpos, pl.t_avidx);
}

// Split of the assembly tree for the triangular solves (gp_solve.cu), on
// the host: blocks are the largest subtrees within the per-warp budget
// (factor entries, vector rows, supernodes, and no front beyond the
// register path of the solve kernels); the supernodes above them form the
// top region, listed children before parents.
struct HostBlk {
    int nblk = 0;
    int max_n = 1, max_v = 1, max_p = 1, max_map = 1, max_ext = 1;
    std::vector<int> blk_ptr{0}, map_ptr{0}, ext_ptr{0}, map_fwd, map_bwd, ext_pos, ext_row;
    // the block's pivot columns in member order (entry e of a block is its
    // pivot slot e) and each one's position in the block's vector
    std::vector<int> pcol_ptr{0}, pcol, pvs;
    std::vector<int4> ent0, ent1;
    int n_top_levels = 0, top_max_front = 1, top_max_xent = 1;
    // the first n_lower_top entries of top_order (whole levels, each front
    // of at most solve_block_front_limit() rows) are forward-solved by one
    // warp per task, the rest (and the whole backward pass) by one CTA per
    // task
    int n_lower_top = 0;
    std::vector<int> top_order, top_rank;
    std::vector<int> top_xptr, top_xrow, top_xent;   // extend-add lists of the top region
    // solve-ordered factor copies: supernode s's L panel (mm x ns, leading
    // dimension mm) and U rows (ns x mm, leading dimension ns) both start at
    // lu_off[s]; the supernodes of a block follow one another in the block's
    // order, every block and every top supernode starts on a multiple of
    // kLuAlign entries
    std::vector<int64_t> lu_off;
    int64_t lu_total = 0;
    int max_seg = 1;   // entries of the largest block (aligned)
};

constexpr int kLuAlign = 4;   // 16 bytes of FP32, 32 of FP64

int64_t lu_align(int64_t x) { return (x + kLuAlign - 1) / kLuAlign * kLuAlign; }

void make_blocks(const gp::Symbolic &sym, HostBlk &B) {
    constexpr long kLimSlices = 2048, kLimRows = 512, kLimSups = 64;
    const long kLimFront = gp::solve_block_front_limit();
    const int ns = sym.nsup;
    std::vector<long> sl(ns, 0), sv(ns, 0), sn(ns, 0), sm(ns, 0);
    for (int l = 0; l < sym.nlevels; l++)
        for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; q++) {
            const int s = sym.level_sups[q];
            const long m = sym.front_m(s), n = sym.front_n(s), r = sym.front_r(s);
            sl[s] = m * n + n * r;
            sv[s] = m;
            sn[s] = 1;
            sm[s] = m;
            for (int c = sym.child_ptr[s]; c < sym.child_ptr[s + 1]; c++) {
                const int ch = sym.children[c];
                sl[s] += sl[ch];
                sv[s] += sv[ch];
                sn[s] += sn[ch];
                sm[s] = std::max(sm[s], sm[ch]);
            }
        }
    auto fits = [&](int s) {
        return sl[s] <= kLimSlices && sv[s] <= kLimRows && sn[s] <= kLimSups && sm[s] <= kLimFront;
    };
    // levels run from the leaves (0) to the roots, so parents are visited
    // before their children here
    std::vector<int> blk_of(ns, -1);
    int nblk = 0;
    for (int l = sym.nlevels - 1; l >= 0; l--)
        for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; q++) {
            const int s = sym.level_sups[q], p = sym.parent[s];
            if (fits(s) && (p < 0 || !fits(p))) blk_of[s] = nblk++;
            else if (p >= 0 && blk_of[p] >= 0) blk_of[s] = blk_of[p];
        }
    // members by level: children before parents, the block's root last
    std::vector<std::vector<int>> members(nblk);
    for (int l = 0; l < sym.nlevels; l++)
        for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; q++) {
            const int s = sym.level_sups[q];
            if (blk_of[s] >= 0) members[blk_of[s]].push_back(s);
        }
    // blocks are emitted (and claimed by the solve kernels) longest first:
    // one warp runs a block's supernodes one after the other, so the block
    // phase ends with its slowest blocks, which should start first.  The
    // estimate per supernode: a fixed cost, one step per pivot column, one
    // per 32 factor entries
    std::vector<double> cost(nblk, 0.0);
    for (int b = 0; b < nblk; b++)
        for (int s : members[b]) {
            const double m = sym.front_m(s), n = sym.front_n(s);
            cost[b] += 8.0 + n + m * n / 32.0;
        }
    std::vector<int> emit(nblk);
    for (int b = 0; b < nblk; b++) emit[b] = b;
    std::stable_sort(emit.begin(), emit.end(), [&](int a, int c) { return cost[a] > cost[c]; });
    std::vector<int> voff_of(ns, -1);
    for (int b : emit) {
        int vo = 0, mo = 0, po = 0;
        for (int s : members[b]) {
            const int m = sym.front_m(s), n = sym.front_n(s), r = sym.front_r(s);
            B.ent0.push_back(make_int4(s, sym.sup_start[s], n, r));
            B.ent1.push_back(make_int4(0, vo, mo, po));
            for (int i = 0; i < n; i++) {
                B.pcol.push_back(sym.sup_start[s] + i);
                B.pvs.push_back(vo + i);
            }
            voff_of[s] = vo;
            vo += m;
            mo += r;
            po += n;
        }
        std::map<int, int> ext;
        for (int s : members[b]) {
            const int r = sym.front_r(s), p = sym.parent[s];
            const bool root = s == members[b].back();
            for (int a = 0; a < r; a++) {
                B.map_fwd.push_back(root ? -1 : voff_of[p] + sym.relmap[sym.relmap_ptr[s] + a]);
                const int g = sym.rows[sym.row_ptr[s] + a], owner = sym.sup_of[g];
                if (blk_of[owner] == b) {
                    B.map_bwd.push_back(voff_of[owner] + (g - sym.sup_start[owner]));
                } else {
                    auto it = ext.find(g);
                    if (it == ext.end()) it = ext.emplace(g, vo + (int)ext.size()).first;
                    B.map_bwd.push_back(it->second);
                }
            }
        }
        for (auto &kv : ext) {
            B.ext_pos.push_back(kv.second);
            B.ext_row.push_back(kv.first);
        }
        B.max_n = std::max(B.max_n, (int)members[b].size());
        B.max_v = std::max(B.max_v, vo + (int)ext.size());
        B.max_p = std::max(B.max_p, po);
        B.max_map = std::max(B.max_map, mo);
        B.max_ext = std::max(B.max_ext, (int)ext.size());
        B.blk_ptr.push_back((int)B.ent0.size());
        B.map_ptr.push_back((int)B.map_fwd.size());
        B.ext_ptr.push_back((int)B.ext_pos.size());
        B.pcol_ptr.push_back((int)B.pcol.size());
    }
    B.nblk = nblk;
    // top region by level (leaves of the region first)
    std::vector<int> tlev(ns, -1);
    int ntl = 0;
    for (int l = 0; l < sym.nlevels; l++)
        for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; q++) {
            const int s = sym.level_sups[q];
            if (blk_of[s] >= 0) continue;
            int d = 0;
            for (int c = sym.child_ptr[s]; c < sym.child_ptr[s + 1]; c++)
                if (blk_of[sym.children[c]] < 0) d = std::max(d, tlev[sym.children[c]] + 1);
            tlev[s] = d;
            ntl = std::max(ntl, d + 1);
            B.top_max_front = std::max(B.top_max_front, sym.front_m(s));
        }
    B.top_order.clear();
    B.top_rank.assign(ns, -1);
    for (int d = 0; d < ntl; d++)
        for (int s = 0; s < ns; s++)
            if (tlev[s] == d) {
                B.top_rank[s] = (int)B.top_order.size();
                B.top_order.push_back(s);
            }
    B.n_top_levels = ntl;
    {
        int lv = 0;   // the lower region: the levels below the first with a front too large for a warp
        while (lv < ntl) {
            bool fits_warp = true;
            for (int s = 0; s < ns; s++)
                if (tlev[s] == lv && sym.front_m(s) > kLimFront) fits_warp = false;
            if (!fits_warp) break;
            lv++;
        }
        B.n_lower_top = 0;
        for (int s : B.top_order)
            if (tlev[s] < lv) B.n_lower_top++;
    }
    // solve-ordered factor copies: the blocks in the order they are claimed,
    // then the top supernodes
    B.lu_off.assign(ns, -1);
    int64_t lo = 0;
    for (int b : emit) {
        const int64_t b0 = lo;
        for (int s : members[b]) {
            B.lu_off[s] = lo;
            lo += (int64_t)sym.front_m(s) * sym.front_n(s);
        }
        lo = lu_align(lo);
        B.max_seg = (int)std::max<int64_t>(B.max_seg, lo - b0);
    }
    for (int s : B.top_order) {
        B.lu_off[s] = lo;
        lo = lu_align(lo + (int64_t)sym.front_m(s) * sym.front_n(s));
    }
    B.lu_total = std::max<int64_t>(lo, kLuAlign);
    // extend-add lists: for every front row of a top supernode, the
    // children's update-vector entries that add into it, in child order
    B.top_xptr.assign(1, 0);
    B.top_xrow.clear();
    B.top_xent.clear();
    for (int s : B.top_order) {
        const int mm = sym.front_m(s);
        std::vector<std::vector<int>> per(mm);
        for (int q = sym.child_ptr[s]; q < sym.child_ptr[s + 1]; q++) {
            const int c = sym.children[q];
            for (int a = 0; a < sym.front_r(c); a++)
                per[sym.relmap[sym.relmap_ptr[c] + a]].push_back((int)sym.uvec_off[c] + a);
        }
        for (int i = 0; i < mm; i++) {
            B.top_xrow.push_back((int)B.top_xent.size());
            B.top_xent.insert(B.top_xent.end(), per[i].begin(), per[i].end());
        }
        B.top_xrow.push_back((int)B.top_xent.size());
        B.top_xptr.push_back((int)B.top_xrow.size());
        B.top_max_xent = std::max(B.top_max_xent, B.top_xrow.back() - B.top_xrow[B.top_xptr[B.top_xptr.size() - 2]]);
    }
}

// Host emulation of the device factorisation (gp_dag.cu): the same front
// layout, assembly order and pivot rule, supernodes by level; the diagonal
// keeps the reciprocal of each pivot and ipiv the composed row permutation
// of each supernode (pivot row i = assembled row ipiv[start + i]), as on the
// device.  Returns the number of zero pivots.
// Host emulation of factor_part (gp_dag.cu) on an assembled front of mm
// rows and ns pivots split in np parts (no right-hand side): each part's
// columns in its own storage (gp::split_col / split_owned_below, every
// mapping checked), each panel factored by its part and copied out, every
// part applying the panel's interchanges, U rows and rank-nb update to its
// own columns; the factored front goes back into F, the pivot rows to piv.
void host_split_eliminate(double *F, int ns, int mm, int np, std::vector<int> &piv) {
    const int nc = mm, B = gp::kSplitPanel;
    std::vector<std::vector<double>> Fl(np);
    std::vector<int> ncl(np);
    int total = 0;
    for (int part = 0; part < np; part++) {
        ncl[part] = gp::split_owned_below(nc, part, np);
        if (ncl[part] > gp::split_cols_cap(nc, np)) fail(GP_E_INTERNAL, "split front: part above its column bound");
        Fl[part].assign((size_t)mm * ncl[part], 0.0);
        for (int jl = 0; jl < ncl[part]; jl++) {
            const int j = gp::split_col(jl, part, np);
            if (j >= nc || gp::split_owner(j, np) != part || gp::split_owned_below(j, part, np) != jl)
                fail(GP_E_INTERNAL, "split front: column map of part %d", part);
            std::copy(F + (size_t)j * mm, F + (size_t)(j + 1) * mm, Fl[part].begin() + (size_t)jl * mm);
        }
        total += ncl[part];
    }
    if (total != nc) fail(GP_E_INTERNAL, "split front: %d of %d columns dealt", total, nc);
    piv.assign(ns, 0);
    std::vector<double> Pn((size_t)mm * B);
    for (int kb = 0; kb < ns; kb += B) {
        const int ke = std::min(ns, kb + B), nb = ke - kb, o = gp::split_owner(kb, np);
        double *Fo = Fl[o].data() + (size_t)gp::split_owned_below(kb, o, np) * mm;
        for (int k = kb; k < ke; k++) {
            double *col = Fo + (size_t)(k - kb) * mm;
            double best = -1.0;
            int bi = k;
            for (int i = k; i < ns; i++)
                if (std::fabs(col[i]) > best) { best = std::fabs(col[i]); bi = i; }
            piv[k] = bi;
            if (bi != k)
                for (int c = 0; c < nb; c++) std::swap(Fo[k + (size_t)c * mm], Fo[bi + (size_t)c * mm]);
            const double inv = 1.0 / col[k];
            for (int i = k + 1; i < mm; i++) col[i] *= inv;
            col[k] = inv;
            for (int c = k - kb + 1; c < nb; c++)
                for (int i = k + 1; i < mm; i++) Fo[i + (size_t)c * mm] -= col[i] * Fo[k + (size_t)c * mm];
        }
        std::copy(Fo, Fo + (size_t)mm * nb, Pn.begin());
        for (int part = 0; part < np; part++) {
            double *Fp = Fl[part].data();
            const int jlp = gp::split_owned_below(kb, part, np);
            for (int jl = 0; jl < ncl[part]; jl++) {
                if (part == o && jl >= jlp && jl < jlp + nb) continue;
                for (int k = kb; k < ke; k++)
                    if (piv[k] != k) std::swap(Fp[k + (size_t)jl * mm], Fp[piv[k] + (size_t)jl * mm]);
            }
            for (int jl = gp::split_owned_below(ke, part, np); jl < ncl[part]; jl++) {
                double *cj = Fp + (size_t)jl * mm;
                for (int q = 0; q < nb; q++)
                    for (int p = q + 1; p < nb; p++) cj[kb + p] -= Pn[kb + p + (size_t)q * mm] * cj[kb + q];
                for (int i = ke; i < mm; i++) {
                    double acc = cj[i];
                    for (int q = 0; q < nb; q++) acc -= Pn[i + (size_t)q * mm] * cj[kb + q];
                    cj[i] = acc;
                }
            }
        }
    }
    for (int part = 0; part < np; part++)
        for (int jl = 0; jl < ncl[part]; jl++)
            std::copy(Fl[part].begin() + (size_t)jl * mm, Fl[part].begin() + (size_t)(jl + 1) * mm,
                      F + (size_t)gp::split_col(jl, part, np) * mm);
}

// split: parts per supernode (DagPlan::nparts); a front with more than one
// is eliminated by host_split_eliminate.
int host_factor(const Plan &pl, const std::vector<double> &svar, std::vector<double> &fronts, std::vector<int> &ipiv,
                bool transpose = false, const std::vector<uint8_t> *split = nullptr) {
    const std::vector<int> &acp = transpose ? pl.t_acp : pl.acp, &acpos = transpose ? pl.t_acpos : pl.acpos;
    const std::vector<double> &acval = transpose ? pl.t_acval : pl.acval;
    const std::vector<int> &avp = transpose ? pl.t_avp : pl.avp, &avpos = transpose ? pl.t_avpos : pl.avpos;
    const std::vector<int> &avidx = transpose ? pl.t_avidx : pl.avidx;
    const gp::Symbolic &S = pl.sym;
    fronts.assign(S.front_off[S.nsup], 0.0);
    ipiv.assign(S.n, 0);
    int zero_pivots = 0;
    for (int l = 0; l < S.nlevels; l++)
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
            const int s = S.level_sups[q];
            const int ns = S.front_n(s), mm = S.front_m(s), start = S.sup_start[s];
            double *F = fronts.data() + S.front_off[s];
            for (int e = acp[s]; e < acp[s + 1]; e++) F[acpos[e]] += acval[e];
            for (int e = avp[s]; e < avp[s + 1]; e++) F[avpos[e]] += svar[avidx[e]];
            for (int cq = S.child_ptr[s]; cq < S.child_ptr[s + 1]; cq++) {
                const int c = S.children[cq];
                const int nc = S.front_n(c), rc = S.front_r(c), mc = S.front_m(c);
                const int *rel = S.relmap.data() + S.relmap_ptr[c];
                const double *Fc = fronts.data() + S.front_off[c];
                for (int b = 0; b < rc; b++)
                    for (int a = 0; a < rc; a++) F[rel[a] + rel[b] * mm] += Fc[(nc + a) + (size_t)(nc + b) * mc];
            }
            std::vector<int> perm(ns);
            for (int i = 0; i < ns; i++) perm[i] = i;
            if (split && (*split)[s] > 1) {
                std::vector<int> pv;
                host_split_eliminate(F, ns, mm, (*split)[s], pv);
                for (int k = 0; k < ns; k++) {
                    if (F[k + k * mm] == 0.0 || !std::isfinite(F[k + k * mm])) zero_pivots++;
                    std::swap(perm[k], perm[pv[k]]);
                }
                for (int i = 0; i < ns; i++) ipiv[start + i] = perm[i];
                continue;
            }
            for (int k = 0; k < ns; k++) {
                double best = -1.0;
                int bi = k;
                for (int i = k; i < ns; i++) {
                    const double v = std::fabs(F[i + k * mm]);
                    if (v > best) { best = v; bi = i; }
                }
                if (best == 0.0) zero_pivots++;
                std::swap(perm[k], perm[bi]);
                if (bi != k)
                    for (int j = 0; j < mm; j++) std::swap(F[k + j * mm], F[bi + j * mm]);
                const double inv = 1.0 / F[k + k * mm];
                for (int i = k + 1; i < mm; i++) F[i + k * mm] *= inv;
                for (int j = k + 1; j < mm; j++)
                    for (int i = k + 1; i < mm; i++) F[i + j * mm] -= F[i + k * mm] * F[k + j * mm];
                F[k + k * mm] = inv;
            }
            for (int i = 0; i < ns; i++) ipiv[start + i] = perm[i];
        }
    return zero_pivots;
}

// Level-order forward and backward solves with the factors of host_factor.
// x: right-hand side in permuted order on entry, solution on exit.
void host_level_solve(const gp::Symbolic &S, const std::vector<double> &fronts, const std::vector<int> &ipiv,
                      std::vector<double> &x) {
    std::vector<double> uvec(std::max<int64_t>(1, S.uvec_off[S.nsup]));
    for (int l = 0; l < S.nlevels; l++)
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
            const int s = S.level_sups[q];
            const int ns = S.front_n(s), r = S.front_r(s), mm = S.front_m(s), start = S.sup_start[s];
            std::vector<double> a(x.begin() + start, x.begin() + start + ns), u(r, 0.0);
            for (int cq = S.child_ptr[s]; cq < S.child_ptr[s + 1]; cq++) {
                const int c = S.children[cq];
                const int *rel = S.relmap.data() + S.relmap_ptr[c];
                const double *uc = uvec.data() + S.uvec_off[c];
                for (int e = 0; e < S.front_r(c); e++) {
                    if (rel[e] < ns) a[rel[e]] += uc[e];
                    else u[rel[e] - ns] += uc[e];
                }
            }
            const double *F = fronts.data() + S.front_off[s];
            std::vector<double> t(ns);
            for (int i = 0; i < ns; i++) t[i] = a[ipiv[start + i]];
            for (int k = 0; k < ns; k++)
                for (int i = k + 1; i < ns; i++) t[i] -= F[i + k * mm] * t[k];
            for (int i = 0; i < r; i++) {
                double acc = 0.0;
                for (int k = 0; k < ns; k++) acc += F[(ns + i) + (size_t)k * mm] * t[k];
                u[i] -= acc;
            }
            std::copy(t.begin(), t.end(), x.begin() + start);
            std::copy(u.begin(), u.end(), uvec.begin() + S.uvec_off[s]);
        }
    for (int l = S.nlevels - 1; l >= 0; l--)
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
            const int s = S.level_sups[q];
            const int ns = S.front_n(s), r = S.front_r(s), mm = S.front_m(s), start = S.sup_start[s];
            const double *F = fronts.data() + S.front_off[s];
            const int *rows = S.rows.data() + S.row_ptr[s];
            std::vector<double> t(ns);
            for (int i = 0; i < ns; i++) {
                double acc = 0.0;
                for (int a = 0; a < r; a++) acc += F[i + (size_t)(ns + a) * mm] * x[rows[a]];
                t[i] = x[start + i] - acc;
            }
            for (int k = ns - 1; k >= 0; k--) {
                t[k] *= F[k + k * mm];
                for (int i = 0; i < k; i++) t[i] -= F[i + k * mm] * t[k];
            }
            std::copy(t.begin(), t.end(), x.begin() + start);
        }
}

// Bounds-checked stand-in for one warp's shared-memory arrays.
struct Staged {
    std::vector<double> v;
    const char *what;
    Staged(size_t n, const char *w) : v(n, 0.0), what(w) {}
    double &operator[](long i) {
        if (i < 0 || i >= (long)v.size()) fail(GP_E_INTERNAL, "block solve: %s index %ld outside [0, %zu)", what, i, v.size());
        return v[(size_t)i];
    }
};

// One front's forward elimination and backward substitution on a staged
// vector v (offset o), in the device kernels' order (gp_solve.cu).
void host_fwd_front(const double *F, const int *perm, int ns, int mm, Staged &v, long o) {
    std::vector<double> t(ns);
    for (int i = 0; i < ns; i++) {
        if (perm[i] < 0 || perm[i] >= ns) fail(GP_E_INTERNAL, "block solve: permutation entry %d outside [0, %d)", perm[i], ns);
        t[i] = v[o + perm[i]];
    }
    for (int i = 0; i < ns; i++) v[o + i] = t[i];
    for (int k = 0; k < ns; k++) {
        const double vk = v[o + k];
        for (int i = k + 1; i < mm; i++) v[o + i] -= F[i + (size_t)k * mm] * vk;
    }
}

// U: the front's U rows (ns x mm, leading dimension ns).
void host_bwd_front(const double *U, int ns, int mm, Staged &v, long o) {
    for (int i = 0; i < ns; i++) {
        double acc = 0.0;
        for (int a = 0; a < mm - ns; a++) acc += U[i + (size_t)(ns + a) * ns] * v[o + ns + a];
        v[o + i] -= acc;
    }
    for (int k = ns - 1; k >= 0; k--) {
        const double tk = v[o + k] * U[k + (size_t)k * ns];
        v[o + k] = tk;
        for (int i = 0; i < k; i++) v[o + i] -= U[i + (size_t)k * ns] * tk;
    }
}

// The factorisation's solve-ordered copies (gp_dag.cu, store): L panel and
// U rows of every supernode at B.lu_off, each range checked against the
// arrays, each block's supernodes consecutive and aligned as the solve
// kernels' prefetch of a block's range assumes.
void host_solve_copies(const gp::Symbolic &S, const HostBlk &B, const std::vector<double> &fronts,
                       std::vector<double> &lf, std::vector<double> &uf) {
    lf.assign(B.lu_total, 0.0);
    uf.assign(B.lu_total, 0.0);
    std::vector<int> seen(B.lu_total, 0);
    for (int s = 0; s < S.nsup; s++) {
        const int64_t o = B.lu_off[s];
        const int ns = S.front_n(s), mm = S.front_m(s);
        if (o < 0 || o + (int64_t)mm * ns > B.lu_total || o % kLuAlign && B.top_rank[s] >= 0)
            fail(GP_E_INTERNAL, "solve copies: supernode %d at %lld", s, (long long)o);
        const double *F = fronts.data() + S.front_off[s];
        for (int k = 0; k < ns; k++)
            for (int i = 0; i < mm; i++) {
                if (seen[o + i + (int64_t)k * mm]++) fail(GP_E_INTERNAL, "solve copies: overlap at supernode %d", s);
                lf[o + i + (int64_t)k * mm] = F[i + (size_t)k * mm];
            }
        for (int c = 0; c < mm; c++)
            for (int i = 0; i < ns; i++) uf[o + i + (int64_t)c * ns] = F[i + (size_t)c * mm];
    }
    for (int blk = 0; blk < B.nblk; blk++) {
        const int e0 = B.blk_ptr[blk], n = B.blk_ptr[blk + 1] - e0;
        int64_t at = B.lu_off[B.ent0[e0].x];
        if (at % kLuAlign) fail(GP_E_INTERNAL, "solve copies: block %d not aligned", blk);
        const int64_t b0 = at;
        for (int q = 0; q < n; q++) {
            const int4 a = B.ent0[e0 + q];
            if (B.lu_off[a.x] != at) fail(GP_E_INTERNAL, "solve copies: block %d not contiguous", blk);
            at += (int64_t)(a.z + a.w) * a.z;
        }
        if (lu_align(at) - b0 > B.max_seg) fail(GP_E_INTERNAL, "solve copies: block %d above max_seg", blk);
    }
}

// Host emulation of the blocked triangular solves (gp_solve.cu) with the
// same staged vectors, maps and permutations, sized by the block maxima,
// every staged index checked against them: blocks forward, top region
// forward in its task order, top region backward, blocks backward.
void host_block_solve(const gp::Symbolic &S, const HostBlk &B, const std::vector<double> &fronts,
                      const std::vector<int> &ipiv, std::vector<double> &x) {
    std::vector<double> uvec(std::max<int64_t>(1, S.uvec_off[S.nsup]), 0.0);
    std::vector<double> lf, uf;
    host_solve_copies(S, B, fronts, lf, uf);
    auto ent = [&](int e, int4 &a, int4 &b) {
        a = B.ent0[e];
        b = B.ent1[e];
        if (a.z != S.front_n(a.x) || a.w != S.front_r(a.x) || a.y != S.sup_start[a.x])
            fail(GP_E_INTERNAL, "block solve: entry %d does not describe supernode %d", e, a.x);
        if (S.front_m(a.x) > gp::solve_block_front_limit())
            fail(GP_E_INTERNAL, "block solve: front of %d rows in a block", S.front_m(a.x));
    };
    for (int blk = 0; blk < B.nblk; blk++) {
        Staged vs(B.max_v, "vector"), pv(B.max_p, "pivot"), mp(B.max_map, "map");
        const int e0 = B.blk_ptr[blk], n = B.blk_ptr[blk + 1] - e0;
        if (n > B.max_n) fail(GP_E_INTERNAL, "block solve: %d entries above max_n", n);
        const int mb = B.map_ptr[blk], nmap = B.map_ptr[blk + 1] - mb;
        for (int i = 0; i < nmap; i++) mp[i] = B.map_fwd[mb + i];
        // the device stages pivots and right-hand side through the block's
        // flat pivot list: entry b.w + i is column a.y + i at vector b.y + i
        const int p0 = B.pcol_ptr[blk];
        if (B.pcol_ptr[blk + 1] - p0 > B.max_p) fail(GP_E_INTERNAL, "block solve: pivot list above max_p");
        for (int q = 0; q < n; q++) {
            int4 a, b;
            ent(e0 + q, a, b);
            for (int i = 0; i < a.z; i++) {
                if (B.pcol[p0 + b.w + i] != a.y + i || B.pvs[p0 + b.w + i] != b.y + i)
                    fail(GP_E_INTERNAL, "block solve: pivot list of block %d", blk);
                pv[b.w + i] = ipiv[B.pcol[p0 + b.w + i]];
            }
            for (int i = 0; i < a.z + a.w; i++) vs[b.y + i] = i < a.z ? x[a.y + i] : 0.0;
        }
        for (int q = 0; q < n; q++) {
            int4 a, b;
            ent(e0 + q, a, b);
            const int s = a.x, ns = a.z, r = a.w;
            std::vector<int> perm(ns);
            for (int i = 0; i < ns; i++) perm[i] = (int)pv[b.w + i];
            host_fwd_front(lf.data() + B.lu_off[s], perm.data(), ns, ns + r, vs, b.y);
            for (int i = 0; i < ns; i++) x[a.y + i] = vs[b.y + i];
            if (q < n - 1)
                for (int i = 0; i < r; i++) vs[(long)mp[b.z + i]] += vs[b.y + ns + i];
            else
                for (int i = 0; i < r; i++) uvec[S.uvec_off[s] + i] = vs[b.y + ns + i];
        }
    }
    const int ntop = (int)B.top_order.size();
    for (int t = 0; t < ntop; t++) {
        const int s = B.top_order[t];
        for (int cq = S.child_ptr[s]; cq < S.child_ptr[s + 1]; cq++) {
            const int c = S.children[cq];
            if (B.top_rank[c] >= t) fail(GP_E_INTERNAL, "top order: child %d after parent %d", c, s);
        }
        const int start = S.sup_start[s], ns = S.front_n(s), r = S.front_r(s), mm = ns + r;
        Staged tv(B.top_max_front, "top vector");
        const int *xr = B.top_xrow.data() + B.top_xptr[t];
        if (B.top_xptr[t + 1] - B.top_xptr[t] != mm + 1) fail(GP_E_INTERNAL, "top extend-add rows of %d", s);
        for (int i = 0; i < mm; i++) {
            double acc = i < ns ? x[start + i] : 0.0;
            for (int e = xr[i]; e < xr[i + 1]; e++) acc += uvec[B.top_xent[e]];
            tv[i] = acc;
        }
        host_fwd_front(lf.data() + B.lu_off[s], ipiv.data() + start, ns, mm, tv, 0);
        for (int i = 0; i < ns; i++) x[start + i] = tv[i];
        for (int a = 0; a < r; a++) uvec[S.uvec_off[s] + a] = tv[ns + a];
    }
    for (int t = ntop - 1; t >= 0; t--) {
        const int s = B.top_order[t];
        const int start = S.sup_start[s], ns = S.front_n(s), r = S.front_r(s), mm = ns + r;
        Staged tv(B.top_max_front, "top vector");
        const int *rows = S.rows.data() + S.row_ptr[s];
        for (int i = 0; i < mm; i++) tv[i] = i < ns ? x[start + i] : x[rows[i - ns]];
        host_bwd_front(uf.data() + B.lu_off[s], ns, mm, tv, 0);
        for (int i = 0; i < ns; i++) x[start + i] = tv[i];
    }
    for (int blk = 0; blk < B.nblk; blk++) {
        Staged vs(B.max_v, "vector"), mp(B.max_map, "map");
        const int e0 = B.blk_ptr[blk], n = B.blk_ptr[blk + 1] - e0;
        const int mb = B.map_ptr[blk], nmap = B.map_ptr[blk + 1] - mb;
        for (int i = 0; i < nmap; i++) mp[i] = B.map_bwd[mb + i];
        const int xb = B.ext_ptr[blk], next = B.ext_ptr[blk + 1] - xb;
        if (next > B.max_ext) fail(GP_E_INTERNAL, "block solve: %d external rows above max_ext", next);
        for (int q = 0; q < n; q++) {
            int4 a, b;
            ent(e0 + q, a, b);
            for (int i = 0; i < a.z; i++) vs[b.y + i] = x[a.y + i];
        }
        for (int k = 0; k < next; k++) vs[B.ext_pos[xb + k]] = x[B.ext_row[xb + k]];
        for (int q = n - 1; q >= 0; q--) {
            int4 a, b;
            ent(e0 + q, a, b);
            const int ns = a.z, r = a.w;
            for (int c = 0; c < r; c++) {
                const long g = (long)mp[b.z + c];
                if (g >= b.y && g < b.y + ns + r) fail(GP_E_INTERNAL, "block solve: map into the front's own rows");
                vs[b.y + ns + c] = vs[g];
            }
            host_bwd_front(uf.data() + B.lu_off[a.x], ns, ns + r, vs, b.y);
            for (int i = 0; i < ns; i++) x[a.y + i] = vs[b.y + i];
        }
    }
}

// Task order of the dataflow kernels: supernodes whose whole subtree has
// fronts of at most dag_small_front() rows first (by level), then the rest
// (by level).  Both parts list children before parents.
// The dataflow schedule (host side): the topological order of the
// factorisation tasks (the tiny region, subtrees whose fronts have at most
// dag_tiny_front() rows, by level; the rest of the small region, at most
// dag_small_front() rows; then the rest by level) and the split of the
// tail's large FP64 fronts into parts.
struct DagPlan {
    std::vector<int> order, rank, submax;
    int n_tiny = 0, n_small = 0, max_big = 0, max_big_whole = 0;
    int tail0 = 0;
    std::vector<uint8_t> nparts;
    std::vector<int> tail_units{0};
    std::vector<int64_t> pb_off;
    int64_t pb_total = 0;
    int max_panels = 1, max_split_ns = 1, max_part_entries = 0, max_part_ints = 0;
};

void make_dag_plan(const gp::Symbolic &sym, DagPlan &dp) {
    const int ns = sym.nsup;
    dp.submax.assign(ns, 0);
    for (int l = 0; l < sym.nlevels; l++)
        for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; q++) {
            const int s = sym.level_sups[q];
            int mx = sym.front_m(s);
            for (int c = sym.child_ptr[s]; c < sym.child_ptr[s + 1]; c++) mx = std::max(mx, dp.submax[sym.children[c]]);
            dp.submax[s] = mx;
        }
    const int lim = gp::dag_small_front(), tiny = gp::dag_tiny_front();
    dp.order.clear();
    dp.rank.assign(ns, 0);
    auto region = [&](int s) { return dp.submax[s] <= tiny ? 0 : (dp.submax[s] <= lim ? 1 : 2); };
    for (int pass = 0; pass < 3; pass++)
        for (int l = 0; l < sym.nlevels; l++)
            for (int q = sym.level_ptr[l]; q < sym.level_ptr[l + 1]; q++) {
                const int s = sym.level_sups[q];
                if (region(s) != pass) continue;
                dp.rank[s] = (int)dp.order.size();
                dp.order.push_back(s);
                if (pass == 2) dp.max_big = std::max(dp.max_big, sym.front_m(s));
            }
    dp.n_tiny = dp.n_small = 0;
    for (int s = 0; s < ns; s++) {
        dp.n_tiny += region(s) == 0;
        dp.n_small += region(s) <= 1;
    }
    // split fronts (FP64): in the last kSplitTail ranks of the order (the
    // narrow top of the tree), a front of at least kSplitMin rows is factored
    // by about one part per 24 columns, at most kMaxParts
    constexpr int kSplitTail = gp::kSplitTailMax, kSplitMin = 48, kColsPerPart = 24;
    dp.tail0 = std::max(dp.n_small, ns - kSplitTail);
    dp.nparts.assign(ns, 1);
    for (int r = dp.tail0; r < ns; r++) {
        const int s = dp.order[r], mm = sym.front_m(s), n = sym.front_n(s);
        const int np =
            mm >= kSplitMin ? std::min(gp::kMaxParts, std::max(2, (mm + kColsPerPart) / kColsPerPart)) : 1;
        dp.nparts[s] = (uint8_t)np;
        dp.tail_units.push_back(dp.tail_units.back() + np);
        dp.pb_off.push_back(dp.pb_total);
        if (np > 1) {
            const int npan = (n + gp::kSplitPanel - 1) / gp::kSplitPanel;
            dp.pb_total += (int64_t)npan * mm * gp::kSplitPanel;
            dp.max_panels = std::max(dp.max_panels, npan);
            dp.max_split_ns = std::max(dp.max_split_ns, n);
            // a part's columns: whole panels of the nc = mm + 1 columns (the
            // FP64 right-hand side included), dealt in turn
            dp.max_part_entries = std::max(dp.max_part_entries, mm * (gp::split_cols_cap(mm + 1, np) + gp::kSplitPanel));
            dp.max_part_ints = std::max(dp.max_part_ints, 2 * mm);
        }
    }
    for (int r = dp.n_small; r < ns; r++)
        if (dp.nparts[dp.order[r]] == 1) dp.max_big_whole = std::max(dp.max_big_whole, sym.front_m(dp.order[r]));
}

void build_dag(gp_layout *L, const gp::Symbolic &sym) {
    DeviceArena &A = L->arena;
    const int ns = sym.nsup;
    DagPlan dp;
    make_dag_plan(sym, dp);
    const std::vector<int> &order = dp.order, &rank = dp.rank, &submax = dp.submax;
    const int lim = gp::dag_small_front();
    const int n_small = dp.n_small;
    gp::DevDag &D = L->D;
    D.nsup = ns;
    D.n_small = n_small;
    D.n_tiny = dp.n_tiny;
    D.max_front = sym.max_front;
    D.order = A.upload(order);
    D.rank = A.upload(rank);
    D.parent = A.upload(sym.parent);
    {
        const size_t M = L->M;
        D.tail0 = dp.tail0;
        D.n_tail = ns - dp.tail0;
        D.big_units = (D.tail0 - n_small) + dp.tail_units.back();
        D.max_panels = dp.max_panels;
        D.max_split_ns = dp.max_split_ns;
        D.max_part_entries = dp.max_part_entries;
        D.max_part_ints = dp.max_part_ints;
        D.max_big_whole = dp.max_big_whole;
        D.nparts = A.upload(dp.nparts);
        D.tail_units = A.upload(dp.tail_units);
        D.pb_off = A.upload(dp.pb_off);
        D.pb_total = std::max<int64_t>(dp.pb_total, 1);
        const size_t nt = std::max(1, D.n_tail);
        D.pdone = A.alloc<int>(nt * M * gp::kMaxParts);
        D.pflag = A.alloc<int>(nt * M * D.max_panels);
        D.ppiv = A.alloc<int>(nt * M * D.max_split_ns);
        D.pbuf = A.alloc<double>(M * D.pb_total);
        fill(L, D.pdone, 0, nt * M * gp::kMaxParts * sizeof(int));
        fill(L, D.pflag, 0, nt * M * D.max_panels * sizeof(int));
    }
    D.max_big_front = dp.max_big;
    // extend-add lists of the fronts the CTA kernel factors: per front entry
    // (and right-hand-side row) its children's contributions, in child order
    {
        if (sym.front_off[ns] > INT32_MAX || sym.uvec_off[ns] > INT32_MAX)
            fail(GP_E_INVALID, "fronts too large for 32-bit assembly offsets");
        std::vector<int> pa_base(ns, -1), pr_base(ns, -1), pa_ptr, pa_src, pr_ptr, pr_src;
        for (int s = 0; s < ns; s++) {
            if (submax[s] <= lim) continue;
            const int mm = sym.front_m(s);
            std::vector<std::vector<int>> per((size_t)mm * mm), perr(mm);
            for (int q = sym.child_ptr[s]; q < sym.child_ptr[s + 1]; q++) {
                const int c = sym.children[q];
                const int ncc = sym.front_n(c), rc = sym.front_r(c), mc = ncc + rc;
                const int *rel = sym.relmap.data() + sym.relmap_ptr[c];
                for (int b = 0; b < rc; b++)
                    for (int a = 0; a < rc; a++)
                        per[(size_t)rel[a] + (size_t)rel[b] * mm].push_back(
                            (int)(sym.front_off[c] + (ncc + a) + (int64_t)(ncc + b) * mc));
                for (int a = 0; a < rc; a++) perr[rel[a]].push_back((int)sym.uvec_off[c] + a);
            }
            pa_base[s] = (int)pa_ptr.size();
            for (size_t p = 0; p < per.size(); p++) {
                pa_ptr.push_back((int)pa_src.size());
                pa_src.insert(pa_src.end(), per[p].begin(), per[p].end());
            }
            pa_ptr.push_back((int)pa_src.size());
            pr_base[s] = (int)pr_ptr.size();
            for (int i = 0; i < mm; i++) {
                pr_ptr.push_back((int)pr_src.size());
                pr_src.insert(pr_src.end(), perr[i].begin(), perr[i].end());
            }
            pr_ptr.push_back((int)pr_src.size());
        }
        gp::DevSym &S = L->S;
        S.pa_base = A.upload(pa_base);
        S.pa_ptr = A.upload(pa_ptr);
        S.pa_src = A.upload(pa_src);
        S.pr_base = A.upload(pr_base);
        S.pr_ptr = A.upload(pr_ptr);
        S.pr_src = A.upload(pr_src);
        L->ST.pa_base = S.pa_base;
        L->ST.pa_ptr = S.pa_ptr;
        L->ST.pa_src = S.pa_src;
        L->ST.pr_base = S.pr_base;
        L->ST.pr_ptr = S.pr_ptr;
        L->ST.pr_src = S.pr_src;
    }
    if (gp::dag_configure(D, 0, L->G64) != 0) fail(GP_E_CUDA, "could not configure the dataflow kernels");
}

void build_blocks(gp_layout *L, const gp::Symbolic &sym) {
    HostBlk H;
    make_blocks(sym, H);
    DeviceArena &A = L->arena;
    gp::DevBlk &B = L->B;
    B.nblk = H.nblk;
    B.max_n = H.max_n;
    B.max_v = H.max_v;
    B.max_p = H.max_p;
    B.max_map = H.max_map;
    B.blk_ptr = A.upload(H.blk_ptr);
    B.ent0 = A.upload(H.ent0);
    B.ent1 = A.upload(H.ent1);
    B.map_ptr = A.upload(H.map_ptr);
    B.map_fwd = A.upload(H.map_fwd);
    B.map_bwd = A.upload(H.map_bwd);
    B.ext_ptr = A.upload(H.ext_ptr);
    B.ext_pos = A.upload(H.ext_pos);
    B.ext_row = A.upload(H.ext_row);
    B.pcol_ptr = A.upload(H.pcol_ptr);
    B.pcol = A.upload(H.pcol);
    B.pvs = A.upload(H.pvs);
    B.n_top = (int)H.top_order.size();
    B.n_lower_top = H.n_lower_top;
    B.top_max_front = H.top_max_front;
    B.top_max_xent = H.top_max_xent;
    B.top_order = A.upload(H.top_order);
    B.top_rank = A.upload(H.top_rank);
    B.top_xptr = A.upload(H.top_xptr);
    B.top_xrow = A.upload(H.top_xrow);
    B.top_xent = A.upload(H.top_xent);
    L->S.lu_off = A.upload(H.lu_off);
    L->S.lu_total = H.lu_total;
    L->ST.lu_off = L->S.lu_off;
    L->ST.lu_total = L->S.lu_total;
    L->n_top_levels = H.n_top_levels;
    const int sc = gp::solve_configure(B, L->SG);
    if (sc == -2) fail(GP_E_INVALID, "front of %d rows exceeds the solve kernels' staging area", B.top_max_front);
    if (sc != 0) fail(GP_E_CUDA, "could not configure the solve kernels");
}

void build_problem(gp_layout *L, const gp_problem *pr) {
    using namespace gp;
    Plan &pl = *new Plan();
    std::unique_ptr<Plan> own(&pl);
    make_plan(pr, pl);
    DeviceArena &A = L->arena;
    DevProblem &P = L->P;
    const int nb = pl.nb;
    P.n_bus = nb;
    P.n_diff = pr->n_diff;
    P.n_alg = pr->n_alg;
    P.n_ctrl = pr->n_ctrl;
    P.n_par = pr->n_par;
    P.net = pl.net;
    P.n_sys = pl.n_sys;
    P.M = L->M;
    L->n_sys = P.n_sys;
    L->n_da = P.net;
    L->n_bus = nb;
    L->n_ctrl = pr->n_ctrl;
    L->n_par = pr->n_par;
    P.y_rowptr = A.upload(pr->y_rowptr, nb + 1);
    P.y_colidx = A.upload(pr->y_colidx, pr->y_nnz);
    {
        std::vector<double2> yv(std::max(1, pr->y_nnz));
        for (int q = 0; q < pr->y_nnz; q++) yv[q] = make_double2(pr->y_re[q], pr->y_im[q]);
        P.y_val = A.upload(yv);
    }
    for (int t = 0; t < GP_NTYPES; t++) {
        const gp_device_table &T = pr->dev[t];
        DTab &D = P.dev[t];
        D.n = T.n;
        auto up = [&](const int32_t *a) -> const int * {
            if (T.n == 0) return A.alloc<int>(1);
            if (!a) {
                std::vector<int> m1(T.n, -1);
                return A.upload(m1);
            }
            return A.upload(a, T.n);
        };
        D.bus = up(T.bus);
        D.diff_ptr = up(T.diff_ptr);
        D.alg_ptr = up(T.alg_ptr);
        D.ctrl_ptr = up(T.ctrl_ptr);
        D.par_ptr = up(T.par_ptr);
        D.link0 = up(T.link0);
        D.link1 = up(T.link1);
    }
    P.is_diff = A.upload(pr->is_diff, P.net);
    {
        // z index of every machine's speed deviation (objective of the adjoint)
        const gp_device_table &G = pr->dev[GP_GENROU];
        std::vector<int> gw;
        for (int k = 0; k < G.n; k++) gw.push_back(G.diff_ptr[k] + 4);
        L->n_gen = (int)gw.size();
        L->d_gen_w = A.upload(gw);
    }
    L->sum_w2 = pl.sum_w2;
    L->nnz_s = pl.nnz_s;
    P.n_cl = (int)pl.ws.size();
    P.cl_w_start = A.upload(pl.ws);
    P.cl_w_size = A.upload(pl.wsz);
    P.cl_gen = A.upload(pl.gen);
    P.cl_gov_type = A.upload(pl.gvt);
    P.cl_gov = A.upload(pl.gv);
    P.cl_exc_type = A.upload(pl.ext);
    P.cl_exc = A.upload(pl.ex);
    L->h_cl_ext = pl.ext;
    L->h_cl_ex = pl.ex;
    for (int t = 0; t < GP_NTYPES; t++) L->h_ntab[t] = pr->dev[t].n;
    {
        const gp_device_table &SG = pr->dev[GP_STATIC_GEN];
        L->h_sg_type.assign(SG.link0, SG.link0 + SG.n);
    }
    P.cl_pss = A.upload(pl.pss);
    P.n_red = pl.n_red;
    P.n_var = pl.n_var;
    L->n_red = pl.n_red;
    P.sg_red = A.upload(pl.sg_red);
    P.sg_var = A.upload(pl.sg_var);
    {
        std::vector<int> maps(2 * P.net);
        std::copy(pl.state_bus.begin(), pl.state_bus.end(), maps.begin());
        std::copy(pl.red_of.begin(), pl.red_of.end(), maps.begin() + P.net);
        L->d_state_maps = A.upload(maps);
    }
    // ---- per-bus device lists (deterministic summation order) ----
    auto bus_csr = [&](const std::vector<int> &bus_of, const int **ptr, const int **lst) {
        std::vector<int> cnt(nb + 1, 0);
        for (int b : bus_of) cnt[b + 1]++;
        for (int b = 0; b < nb; b++) cnt[b + 1] += cnt[b];
        std::vector<int> l(bus_of.size()), fill(cnt.begin(), cnt.end() - 1);
        for (size_t k = 0; k < bus_of.size(); k++) l[fill[bus_of[k]]++] = (int)k;
        *ptr = A.upload(cnt);
        *lst = A.upload(l);
    };
    bus_csr(pl.cbus, &P.bus_cl_ptr, &P.bus_cl);
    bus_csr(vec(pr->dev[GP_ZIPLOAD].bus, pr->dev[GP_ZIPLOAD].n), &P.bus_zl_ptr, &P.bus_zl);
    bus_csr(vec(pr->dev[GP_STATIC_GEN].bus, pr->dev[GP_STATIC_GEN].n), &P.bus_sg_ptr, &P.bus_sg);
    {
        // the network kernel's bus order: buses with the same device counts
        // and Ybus row length side by side (same loop trip counts per warp)
        std::vector<std::array<int, 5>> key(nb);
        for (int b = 0; b < nb; b++) key[b] = {0, 0, 0, pr->y_rowptr[b + 1] - pr->y_rowptr[b], b};
        for (int k = 0; k < pr->dev[GP_STATIC_GEN].n; k++) key[pr->dev[GP_STATIC_GEN].bus[k]][0]++;
        for (int k = 0; k < pr->dev[GP_ZIPLOAD].n; k++) key[pr->dev[GP_ZIPLOAD].bus[k]][1]++;
        for (int b : pl.cbus) key[b][2]++;
        std::sort(key.begin(), key.end());
        std::vector<int> order(nb);
        for (int i = 0; i < nb; i++) order[i] = key[i][4];
        P.bus_order = A.upload(order);
    }
    const gp::Symbolic &sym = pl.sym;
    P.iperm = A.upload(sym.iperm);
    DevSym &S = L->S;
    S.n = pl.n_red;
    S.nsup = sym.nsup;
    S.nlevels = sym.nlevels;
    S.sup_start = A.upload(sym.sup_start);
    S.row_ptr = A.upload(sym.row_ptr);
    S.rows = A.upload(sym.rows);
    S.child_ptr = A.upload(sym.child_ptr);
    S.children = A.upload(sym.children);
    S.relmap_ptr = A.upload(sym.relmap_ptr);
    S.relmap = A.upload(sym.relmap);
    S.front_off = A.upload(sym.front_off);
    S.uvec_off = A.upload(sym.uvec_off);
    S.front_total = sym.front_off[sym.nsup];
    S.uvec_total = sym.uvec_off[sym.nsup];
    S.asmc_ptr = A.upload(pl.acp);
    S.asmc_pos = A.upload(pl.acpos);
    S.asmc_val = A.upload(pl.acval);
    S.asmv_ptr = A.upload(pl.avp);
    S.asmv_pos = A.upload(pl.avpos);
    S.asmv_idx = A.upload(pl.avidx);
    L->ST = S;
    L->ST.asmc_ptr = A.upload(pl.t_acp);
    L->ST.asmc_pos = A.upload(pl.t_acpos);
    L->ST.asmc_val = A.upload(pl.t_acval);
    L->ST.asmv_ptr = A.upload(pl.t_avp);
    L->ST.asmv_pos = A.upload(pl.t_avpos);
    L->ST.asmv_idx = A.upload(pl.t_avidx);
    L->sym = pl.sym;
    build_dag(L, sym);
    build_blocks(L, sym);
}

void build_work(gp_layout *L, const double *z0, const double *u0, const double *p) {
    using namespace gp;
    DeviceArena &A = L->arena;
    DevProblem &P = L->P;
    DevWork &W = L->W;
    const size_t M = L->M;
    W.z = A.upload(z0, M * P.n_sys);
    W.zold = A.alloc<double>(M * P.n_sys);
    W.u0 = A.upload(u0, M * std::max(1, P.n_ctrl));
    W.p = A.upload(p, M * std::max(1, P.n_par));
    L->d_zl_k = A.alloc<double>(M * 4 * std::max(1, P.dev[6].n));
    P.zl_k = L->d_zl_k;
    W.yx = A.alloc<double>(M * 3 * std::max(1, P.net));
    W.clout = A.alloc<double>(M * 8 * std::max(1, P.n_cl));
    W.svar = A.alloc<double>(M * P.n_var);
    W.xperm = A.alloc<double>(M * P.n_red);
    W.f = A.alloc<double>(M * P.n_sys);
    W.norm = A.alloc<unsigned long long>(M);
    W.active = A.alloc<uint8_t>(M);
    W.iters = A.alloc<int>(M);
    W.status = A.alloc<int>(M);
    W.flag = A.alloc<int>(4);
    W.dt = A.alloc<double>(1);
    DevSym &S = L->S;
    S.fronts = A.alloc<double>(M * S.front_total);
    S.lfac = A.alloc<double>(M * S.lu_total);
    S.ufac = A.alloc<double>(M * S.lu_total);
    fill(L, S.lfac, 0, M * S.lu_total * sizeof(double));
    fill(L, S.ufac, 0, M * S.lu_total * sizeof(double));
    S.uvec = A.alloc<double>(M * std::max<int64_t>(1, S.uvec_total));
    S.ipiv = A.alloc<int>(M * S.n);
    // S^T (the adjoint) factors into the same buffers
    L->ST.fronts = S.fronts;
    L->ST.lfac = S.lfac;
    L->ST.ufac = S.ufac;
    L->ST.uvec = S.uvec;
    L->ST.ipiv = S.ipiv;
    {
        // no row swaps until a factorisation has run: the solves of a
        // scenario whose factors were never computed stay in bounds
        std::vector<int> ident((size_t)M * S.n);
        for (size_t m = 0; m < M; m++)
            for (int s = 0; s < L->sym.nsup; s++)
                for (int c = L->sym.sup_start[s]; c < L->sym.sup_start[s + 1]; c++)
                    ident[m * S.n + c] = c - L->sym.sup_start[s];
        to_device(L, S.ipiv, ident.data(), ident.size() * sizeof(int), "ipiv");
    }
    gp::DevDag &D = L->D;
    D.ctr = A.alloc<int>(8);
    D.epoch = A.alloc<int>(1);
    D.err = A.alloc<int>(1);
    D.fdone = A.alloc<int>(M * D.nsup);
    D.xdone = A.alloc<int>(M * D.nsup);
    D.bdone = A.alloc<int>(M * D.nsup);
    D.utag = A.alloc<unsigned long long>(M * std::max<int64_t>(1, S.uvec_total));
    D.xtag = A.alloc<unsigned long long>(M * std::max(1, P.n_red));
    fill(L, D.utag, 0, M * std::max<int64_t>(1, S.uvec_total) * sizeof(unsigned long long));
    fill(L, D.xtag, 0, M * std::max(1, P.n_red) * sizeof(unsigned long long));
    fill(L, D.ctr, 0, 8 * sizeof(int));
    fill(L, D.epoch, 0, sizeof(int));
    fill(L, D.err, 0, sizeof(int));
    fill(L, D.fdone, 0, M * D.nsup * sizeof(int));
    fill(L, D.xdone, 0, M * D.nsup * sizeof(int));
    fill(L, D.bdone, 0, M * D.nsup * sizeof(int));
    fill(L, W.status, 0, M * sizeof(int));
    ck(cudaMallocHost(&L->h_flag, 4 * sizeof(int)), "cudaMallocHost");
    L->d_cnt = A.alloc<int>(8);
    fill(L, L->d_cnt, 0, 8 * sizeof(int));
    ck(cudaMallocHost(&L->h_dt, sizeof(double)), "cudaMallocHost");
    ck(cudaEventCreateWithFlags(&L->ev_snap, cudaEventDisableTiming), "event");
    for (int i = 0; i < 8; i++) ck(cudaEventCreate(&L->pev[i]), "event");
    gp::launch_zip_const(P, W, L->d_zl_k, L->st);
    ck(cudaStreamSynchronize(L->st), "load constants");
    // keep the initial state for gp_restore_initial_state
    L->z_init = A.alloc<double>(M * P.n_sys);
    ck(cudaMemcpyAsync(L->z_init, W.z, M * P.n_sys * sizeof(double), cudaMemcpyDeviceToDevice, L->st), "z0 copy");
}

// Sparse cluster programs (gp_cluster_plan.cpp), uploaded with the cluster
// indices translated to the compacted non-trivial cluster arrays.
void build_clusters(gp_layout *L, const gp_problem *pr, const double *z0, const double *u0, const double *p) {
    gp::ClusterPlan &cp = L->cplan;
    gp::make_cluster_plan(pr, z0, u0, p, cp);
    std::vector<int> compact(pr->n_clusters, -1);
    int k = 0;
    for (int c = 0; c < pr->n_clusters; c++)
        if (pr->cl_gen[c] >= 0) compact[c] = k++;
    std::vector<int> order(cp.order.size());
    for (size_t q = 0; q < cp.order.size(); q++) order[q] = compact[cp.order[q]];
    DeviceArena &A = L->arena;
    gp::DevClu &C = L->C;
    C.n_tasks = (int)cp.task_class.size();
    C.task_class = A.upload(cp.task_class);
    C.task_first = A.upload(cp.task_first);
    C.task_count = A.upload(cp.task_count);
    C.order = A.upload(order);
    C.slot_of = A.upload(cp.slot_of);
    C.prog_ptr = A.upload(cp.prog_ptr);
    C.prog_mid = A.upload(cp.prog_mid);
    C.prog_sol = A.upload(cp.prog_sol);
    C.ops = A.upload(cp.ops);
    C.rhs_base = A.upload(cp.rhs_base);
    C.nslot = A.upload(cp.nslot);
    C.perm_col = A.upload(cp.perm_col);
    C.pos3 = A.upload(cp.pos3);
    {
        // position of each local row in the class program (the residual
        // placement ops name it): the transposed solves of the adjoint
        // return the row of each position
        std::vector<int> row_pos((size_t)cp.n_class * 32, 0);
        for (int cls = 0; cls < cp.n_class; cls++) {
            const int W = cp.cls_W[cls], rb = cp.rhs_base[cls];
            for (int q = cp.prog_ptr[cls]; q < cp.prog_mid[cls]; q++) {
                const gp::CluOp &o = cp.ops[q];
                if (o.code == gp::OP_BEF || o.code == gp::OP_ROW) row_pos[(size_t)cls * 32 + o.a] = o.d - rb - 2 * W;
            }
        }
        C.row_pos = A.upload(row_pos);
    }
    C.max_slots = cp.max_slots;
    C.max_w = 1;
    for (int w : cp.cls_W) C.max_w = std::max(C.max_w, w);
    const int bytes = cp.max_slots * 32 * (int)sizeof(double);
    if (bytes > 48 * 1024 && (gp::cluster_smem_optin(bytes) < 0 || gp::adj_smem_optin(bytes) < 0))
        fail(GP_E_CUDA, "cluster kernel needs %d bytes of shared memory", bytes);
}

void drop_graphs(gp_layout *L) {
    for (cudaGraphExec_t *g :
         {&L->g_eval, &L->g_solve, &L->g_mix[0], &L->g_mix[1], &L->g_mix[2], &L->g_mix[3], &L->g_loop})
        if (*g) {
            cudaGraphExecDestroy(*g);
            *g = nullptr;
        }
}

void set_faults(gp_layout *L, int n_faults, const gp_fault *faults) {
    using namespace gp;
    L->call.release();
    const int M = L->M;
    std::vector<std::vector<int>> per(M);
    for (int e = 0; e < n_faults; e++) {
        const gp_fault &f = faults[e];
        if (f.bus < 0 || f.bus >= L->n_bus) fail(GP_E_INVALID, "fault %d: bus %d out of range", e, f.bus);
        if (!(f.rfault > 0.0)) fail(GP_E_INVALID, "fault %d: rfault must be positive", e);
        if (f.scenario >= M) fail(GP_E_INVALID, "fault %d: scenario %d out of range", e, f.scenario);
        if (f.scenario < 0)
            for (int m = 0; m < M; m++) per[m].push_back(e);
        else
            per[f.scenario].push_back(e);
    }
    std::vector<int> ptr(M + 1, 0), bus, on, off, scen;
    std::vector<double> yf;
    for (int m = 0; m < M; m++) {
        for (int e : per[m]) {
            bus.push_back(faults[e].bus);
            yf.push_back(1.0 / faults[e].rfault);
            on.push_back(faults[e].on_step);
            off.push_back(faults[e].off_step);
            scen.push_back(m);
        }
        ptr[m + 1] = (int)bus.size();
    }
    L->n_fl = (int)bus.size();
    // the fault table keeps its device addresses while it fits (grow-only):
    // the captured graphs hold those addresses, and stay valid across calls
    const int cap = std::max(1, L->n_fl);
    if (!L->d_fl_ptr || cap > L->fl_cap) {
        L->fault_arena.release();
        DeviceArena &A = L->fault_arena;
        L->d_fl_ptr = A.alloc<int>(M + 1);
        L->d_fl_bus = A.alloc<int>(cap);
        L->d_fl_yf = A.alloc<double>(cap);
        L->d_fl_on = A.alloc<uint8_t>(cap);
        L->d_fl_on_step = A.alloc<int>(cap);
        L->d_fl_off_step = A.alloc<int>(cap);
        L->d_fl_scen = A.alloc<int>(cap);
        L->fl_cap = cap;
        L->P.fl_ptr = L->d_fl_ptr;
        L->P.fl_bus = L->d_fl_bus;
        L->P.fl_yf = L->d_fl_yf;
        L->P.fl_on = L->d_fl_on;
        drop_graphs(L);
    }
    auto put = [&](void *d, const void *h, size_t bytes) {
        if (bytes) to_device(L, d, h, bytes, "fault table");
    };
    put(L->d_fl_ptr, ptr.data(), ptr.size() * sizeof(int));
    put(L->d_fl_bus, bus.data(), bus.size() * sizeof(int));
    put(L->d_fl_yf, yf.data(), yf.size() * sizeof(double));
    put(L->d_fl_on_step, on.data(), on.size() * sizeof(int));
    put(L->d_fl_off_step, off.data(), off.size() * sizeof(int));
    put(L->d_fl_scen, scen.data(), scen.size() * sizeof(int));
    fill(L, L->d_fl_on, 0, cap);
    L->h_fl_on_step = on;
    L->h_fl_off_step = off;
    L->h_fl_scen = scen;
}

void mark(gp_layout *L, int i) {
    if (L->no_marks) return;
    ck(cudaEventRecordWithFlags(L->pev[i], L->st, cudaEventRecordExternal), "event record");
}

// Solve graph; returns its kernel launches and counts its factorisation
// launches in *nfac_out.  FP64 (variant < 0): fresh factorisation with the
// forward solve fused, backward solve, update.  Mixed, variant bits: 1 the
// FP32 factorisation of the MX_FP32 scenarios, 2 the FP64 factorisation
// (forward solve fused) of the MX_EXACT scenarios; then the forward solve of
// the scenarios on FP32 factors, the backward solve of all (each with its
// own factors), and the update.
int enqueue_solve(gp_layout *L, int variant, int *nfac_out) {
    const gp::DevDag &D = L->D;
    // factorisation launches: FP32 the warp and CTA kernels; FP64 also the
    // tiny region's warp launch
    const int nfac = (D.n_small > 0) + (D.nsup > D.n_small);
    const int nfac64 = (D.n_tiny > 0) + (D.n_small > D.n_tiny) + (D.nsup > D.n_small);
    const gp::DevBlk &B = L->B;
    const int nsolve = (B.nblk + B.n_top) > 0;   // one fused kernel per direction
    int launches = 2, facs = 0;   // dag_begin, update
    mark(L, 3);
    gp::launch_dag_begin(D, L->st);
    if (variant == -2) {
        // shared-factor Woodbury: the factors of P (scenario 0's slot), the
        // fault's rank-2 correction, no factorisation
        const gp::FrontSel fs{nullptr, nullptr, L->S.lfac, L->S.ufac, nullptr, 0, 1};
        mark(L, 4);
        gp::launch_solve_fwd(L->P, L->W, L->S, B, D, L->SG, fs, L->st);
        mark(L, 5);
        gp::launch_solve_bwd(L->P, L->W, L->S, B, D, L->SG, fs, L->st);
        gp::launch_wb_correct(L->P, L->W, L->wb_W1, L->wb_W2, L->wb_Hinv, L->wb_s, L->st);
        launches += 2 * nsolve + 2;
    } else if (variant < 0) {
        const gp::FrontSel fs{nullptr, nullptr, L->S.lfac, L->S.ufac, nullptr, 1};
        gp::launch_dag_factor<double>(L->P, L->W, L->S, D, L->G64, L->S.fronts, nullptr, L->S.ufac, L->W.active, 1,
                                      L->st);
        mark(L, 4);   // the FP64 factorisation includes the forward solve
        mark(L, 5);
        gp::launch_solve_bwd(L->P, L->W, L->S, B, D, L->SG, fs, L->st);
        facs = nfac64;
        launches += nfac64 + nsolve;
    } else {
        const gp::FrontSel fs{L->Mx.lfac, L->Mx.ufac, L->S.lfac, L->S.ufac, L->Mx.refac, 1};
        if (variant & 1) {
            gp::launch_dag_factor<float>(L->P, L->W, L->S, D, L->G32, L->Mx.fronts, L->Mx.lfac, L->Mx.ufac,
                                         L->Mx.refac, gp::MX_FP32, L->st);
            facs += nfac;
        }
        if (variant & 2) {
            // the two factorisations share the claim counters and done
            // flags: re-arm them (new epoch) for the second one
            if (variant & 1) {
                gp::launch_dag_begin(D, L->st);
                launches += 1;
            }
            gp::launch_dag_factor<double>(L->P, L->W, L->S, D, L->G64, L->S.fronts, nullptr, L->S.ufac, L->Mx.refac,
                                          gp::MX_EXACT, L->st);
            facs += nfac64;
        }
        mark(L, 4);
        gp::launch_solve_fwd(L->P, L->W, L->S, B, D, L->SG, fs, L->st);
        mark(L, 5);
        gp::launch_solve_bwd(L->P, L->W, L->S, B, D, L->SG, fs, L->st);
        launches += facs + 2 * nsolve;
    }
    mark(L, 6);
    gp::launch_update(L->P, L->W, L->S, L->d_state_maps, L->st);
    mark(L, 7);
    *nfac_out = facs;
    return launches;
}

// Evaluation: residuals, cluster solves, reduced right-hand side, check.
// The host-driven loop copies the flags to the host; the device-driven loop
// (ctl.on) leaves the decision to the check kernel.
void enqueue_eval(gp_layout *L, double tol, int itermax, const gp::LoopCtl &ctl) {
    gp::launch_reset_norm(L->P, L->W, L->Mx, L->st);
    mark(L, 0);
    L->eval_launches = 3 + gp::launch_cluster(L->P, L->W, L->C, L->Mx, 0, L->st);
    mark(L, 1);
    gp::launch_network(L->P, L->W, L->Mx, 0, L->st, L->solver == GP_SOLVER_SHARED_WOODBURY ? 1 : 0);
    mark(L, 2);
    gp::launch_check(L->P, L->W, L->Mx, tol, itermax, ctl, L->st);
    if (!ctl.on)
        ck(cudaMemcpyAsync(L->h_flag, L->W.flag, 4 * sizeof(int), cudaMemcpyDeviceToHost, L->st), "flag copy");
}

template <class F>
cudaGraphExec_t capture(gp_layout *L, F enqueue) {
    cudaGraph_t g;
    ck(cudaStreamBeginCapture(L->st, cudaStreamCaptureModeThreadLocal), "begin capture");
    enqueue();
    ck(cudaStreamEndCapture(L->st, &g), "end capture");
    cudaGraphExec_t ex;
    ck(cudaGraphInstantiate(&ex, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    return ex;
}

// Captures the work of enqueue into the existing graph g after the nodes
// deps; returns the last node captured.
template <class F>
cudaGraphNode_t capture_into(gp_layout *L, cudaGraph_t g, const cudaGraphNode_t *deps, size_t n_deps, F enqueue) {
    ck(cudaStreamBeginCaptureToGraph(L->st, g, deps, nullptr, n_deps, cudaStreamCaptureModeThreadLocal),
       "begin capture");
    enqueue();
    cudaStreamCaptureStatus status;
    const cudaGraphNode_t *tail = nullptr;
    size_t n_tail = 0;
    ck(cudaStreamGetCaptureInfo(L->st, &status, nullptr, nullptr, &tail, nullptr, &n_tail), "capture info");
    const cudaGraphNode_t last = n_tail == 1 ? tail[0] : nullptr;
    cudaGraph_t out;
    ck(cudaStreamEndCapture(L->st, &out), "end capture");
    if (!last) fail(GP_E_INTERNAL, "captured work does not end in one node");
    return last;
}

cudaGraphNode_t add_conditional(cudaGraph_t g, const cudaGraphNode_t *deps, size_t n_deps,
                                cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, unsigned size,
                                cudaGraph_t *bodies) {
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = type;
    np.conditional.size = size;
    cudaGraphNode_t node;
    ck(cudaGraphAddNode(&node, g, deps, nullptr, n_deps, &np), "conditional node");
    for (unsigned b = 0; b < size; b++) bodies[b] = np.conditional.phGraph_out[b];
    return node;
}

int enqueue_solve(gp_layout *L, int variant, int *nfac_out);

// The whole Newton solve as one graph: the first evaluation, then
// WHILE(some scenario iterates) { solve; evaluation }.  The mixed solver's
// solve is a SWITCH over the four factorisation variants, chosen by the
// check kernel; the FP64 solve is always the same.  No event nodes: the
// phase timing needs the host-driven loop.
cudaGraphExec_t build_loop(gp_layout *L, double tol, int itermax, bool mixed, int plain_variant) {
    cudaGraph_t g;
    ck(cudaGraphCreate(&g, 0), "graph create");
    ck(cudaGraphConditionalHandleCreate(&L->h_loop, g, 0, cudaGraphCondAssignDefault), "conditional handle");
    L->h_var = 0;
    if (mixed) ck(cudaGraphConditionalHandleCreate(&L->h_var, g, 0, cudaGraphCondAssignDefault), "conditional handle");
    const gp::LoopCtl ctl{L->h_loop, L->h_var, L->d_cnt, 1, mixed ? 1 : 0};
    L->no_marks = true;
    const cudaGraphNode_t first = capture_into(L, g, nullptr, 0, [&] { enqueue_eval(L, tol, itermax, ctl); });
    cudaGraph_t body;
    add_conditional(g, &first, 1, L->h_loop, cudaGraphCondTypeWhile, 1, &body);
    cudaGraphNode_t solved;
    if (mixed) {
        cudaGraph_t var[4];
        solved = add_conditional(body, nullptr, 0, L->h_var, cudaGraphCondTypeSwitch, 4, var);
        for (int v = 0; v < 4; v++)
            capture_into(L, var[v], nullptr, 0,
                         [&] { L->mix_launches[v] = enqueue_solve(L, v, &L->mix_factor_launches[v]); });
    } else {
        solved = capture_into(L, body, nullptr, 0, [&] {
            L->solve_graph_launches = enqueue_solve(L, plain_variant, &L->solve_graph_factors);
        });
    }
    capture_into(L, body, &solved, 1, [&] { enqueue_eval(L, tol, itermax, ctl); });
    L->no_marks = false;
    cudaGraphExec_t ex;
    ck(cudaGraphInstantiate(&ex, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    return ex;
}

// Folds the device-driven loop's counts into the call's totals.
void harvest_counts(gp_layout *L) {
    int c[8];
    to_host(L, c, L->d_cnt, sizeof(c), "count copy");
    fill(L, L->d_cnt, 0, sizeof(c));
    const bool mixed = L->Mx.on != 0;
    const int nfac = L->solve_graph_factors;
    L->launches += (double)c[0] * L->eval_launches;
    L->solves += c[1];
    L->refreshes += c[2];
    L->exact_iters += c[3];
    for (int v = 0; v < 4; v++) {
        L->launches += (double)c[4 + v] * (mixed ? L->mix_launches[v] : L->solve_graph_launches);
        L->factor_launches += (double)c[4 + v] * (mixed ? L->mix_factor_launches[v] : nfac);
    }
}

// Kept FP32 factors of the mixed solver, allocated on its first use.
void ensure_mixed(gp_layout *L) {
    if (L->mixed_ready) return;
    DeviceArena &A = L->arena;
    const size_t M = L->M;
    gp::DevMixed &X = L->Mx;
    int n_lu = 1;
    for (int v : L->cplan.rhs_base) n_lu = std::max(n_lu, v);
    X.n_lu = n_lu;
    X.max_age = L->mx_max_age;
    X.exact_after = L->mx_exact_after;
    X.rho_max = L->mx_rho_max;
    X.refac = A.alloc<uint8_t>(M);
    X.refac_next = A.alloc<uint8_t>(M);
    X.prev_mode = A.alloc<uint8_t>(M);
    X.age = A.alloc<int>(M);
    X.all_exact = A.alloc<uint8_t>(M);
    X.retry = A.alloc<uint8_t>(M);
    X.prev_norm = A.alloc<double>(M);
    X.lu = A.alloc<float>(M * std::max(1, L->C.n_tasks) * n_lu * 32);
    X.cc = A.alloc<float>(M * std::max(1, L->P.n_cl) * 6);
    X.fronts = A.alloc<float>(M * L->S.front_total);
    X.lfac = A.alloc<float>(M * L->S.lu_total);
    X.ufac = A.alloc<float>(M * L->S.lu_total);
    X.kc = A.alloc<double>(M * std::max(1, L->C.n_tasks) * gp::kConstSlots * 32);
    L->zprev = A.alloc<double>(M * L->n_sys);
    L->zprev2 = A.alloc<double>(M * L->n_sys);
    L->zprev3 = A.alloc<double>(M * L->n_sys);
    fill(L, X.refac, 0, M);
    fill(L, X.refac_next, 0, M);
    fill(L, X.prev_mode, 0, M);
    fill(L, X.age, 0, M * sizeof(int));
    fill(L, X.all_exact, 0, M);
    fill(L, X.retry, 0, M);
    // kept factors start at zero (zero pivot reciprocals give a zero step,
    // which the contraction test turns into a refresh)
    fill(L, X.lu, 0, M * std::max(1, L->C.n_tasks) * n_lu * 32 * sizeof(float));
    fill(L, X.cc, 0, M * std::max(1, L->P.n_cl) * 6 * sizeof(float));
    fill(L, X.fronts, 0, M * L->S.front_total * sizeof(float));
    fill(L, X.lfac, 0, M * L->S.lu_total * sizeof(float));
    fill(L, X.ufac, 0, M * L->S.lu_total * sizeof(float));
    if (gp::dag_configure(L->D, 1, L->G32) != 0) fail(GP_E_CUDA, "could not configure the FP32 dataflow kernels");
    L->mixed_ready = true;
}

// Buffers of the shared-factor Woodbury path, allocated on its first use.
void ensure_woodbury(gp_layout *L) {
    if (L->wb_W1) return;
    DeviceArena &A = L->arena;
    const size_t M = L->M, nr = std::max(1, L->P.n_red);
    L->wb_W1 = A.alloc<double>(M * nr);
    L->wb_W2 = A.alloc<double>(M * nr);
    L->wb_Hinv = A.alloc<double>(M * 4);
    L->wb_s = A.alloc<double>(M * 2);
    std::vector<uint8_t> only0(M, 0);
    only0[0] = 1;
    L->d_only0 = A.upload(only0);
}

// Start of a shared-factor Woodbury integration: P, the reduced matrix of
// scenario 0 at the initial state with the call's dt and no fault, is
// factored once into scenario 0's front slot (_factor_shared_P_gpu!,
// ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2149-2172); then per scenario
// W = P^-1 [e_vr e_vi] at its fault bus and H^-1
// (_precompute_woodbury_multi_gpu!, :2441-2489).
void wb_prepare(gp_layout *L, double dt) {
    const int M = L->M;
    gp::launch_set_double(L->W.dt, dt, L->st);
    ck(cudaMemcpyAsync(L->W.zold, L->W.z, (size_t)M * L->n_sys * sizeof(double), cudaMemcpyDeviceToDevice, L->st),
       "zold");
    ck(cudaMemsetAsync(L->W.active, 1, M, L->st), "memset");
    gp::launch_reset_norm(L->P, L->W, L->Mx, L->st);
    gp::launch_cluster(L->P, L->W, L->C, L->Mx, 0, L->st);
    gp::launch_network(L->P, L->W, L->Mx, 0, L->st);
    gp::launch_dag_begin(L->D, L->st);
    gp::launch_dag_factor<double>(L->P, L->W, L->S, L->D, L->G64, L->S.fronts, L->S.lfac, L->S.ufac, L->d_only0, 1,
                                  L->st);
    const gp::FrontSel fs{nullptr, nullptr, L->S.lfac, L->S.ufac, nullptr, 0, 1};
    double *cols[2] = {L->wb_W1, L->wb_W2};
    for (int c = 0; c < 2; c++) {
        gp::launch_wb_unit(L->P, L->W, c, L->st);
        gp::launch_dag_begin(L->D, L->st);
        gp::launch_solve_fwd(L->P, L->W, L->S, L->B, L->D, L->SG, fs, L->st);
        gp::launch_solve_bwd(L->P, L->W, L->S, L->B, L->D, L->SG, fs, L->st);
        ck(cudaMemcpyAsync(cols[c], L->W.xperm, (size_t)M * L->P.n_red * sizeof(double), cudaMemcpyDeviceToDevice,
                           L->st),
           "woodbury column");
    }
    gp::launch_wb_setup(L->P, L->wb_W1, L->wb_W2, L->wb_Hinv, L->st);
    {
        const gp::DevDag &D = L->D;
        const int nfac64 = (D.n_tiny > 0) + (D.n_small > D.n_tiny) + (D.nsup > D.n_small);
        L->launches += 14 + nfac64;
        L->factor_launches += nfac64;
    }
}

void ensure_graphs(gp_layout *L, double tol, int itermax, int solver) {
    if (L->solver != solver || L->graph_tol != tol || L->graph_itermax != itermax) drop_graphs(L);
    const bool mixed = solver == GP_SOLVER_SCHUR_MIXED;
    if (mixed) ensure_mixed(L);
    L->Mx.on = mixed ? 1 : 0;
    L->graph_tol = tol;
    L->graph_itermax = itermax;
    L->solver = solver;
    const int plain = solver == GP_SOLVER_SHARED_WOODBURY ? -2 : -1;
    if (solver == GP_SOLVER_SHARED_WOODBURY) ensure_woodbury(L);
    if (!L->profiling) {
        if (!L->g_loop) L->g_loop = build_loop(L, tol, itermax, mixed, plain);
        return;
    }
    if (!L->g_eval) L->g_eval = capture(L, [&] { enqueue_eval(L, tol, itermax, gp::LoopCtl{0, 0, nullptr, 0, 0}); });
    if (!mixed && !L->g_solve)
        L->g_solve = capture(L, [&] { L->solve_graph_launches = enqueue_solve(L, plain, &L->solve_graph_factors); });
}

// Solve graph of the mixed solver for the modes present (captured on first use).
cudaGraphExec_t mixed_graph(gp_layout *L, int variant) {
    if (!L->g_mix[variant])
        L->g_mix[variant] = capture(
            L, [&] { L->mix_launches[variant] = enqueue_solve(L, variant, &L->mix_factor_launches[variant]); });
    return L->g_mix[variant];
}

// One Newton solve for the scenarios marked active; returns after every
// scenario converged, diverged or used itermax updates.
float elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, a, b), "event elapsed");
    return ms;
}

void newton(gp_layout *L, double dt, double tol, int itermax, bool force_refresh, bool reset_iters) {
    // dt by value (a kernel argument): the host may run steps ahead of the GPU
    gp::launch_set_double(L->W.dt, dt, L->st);
    L->launches += 1;
    if (reset_iters) ck(cudaMemsetAsync(L->W.iters, 0, L->M * sizeof(int), L->st), "memset");
    const bool mixed = L->Mx.on != 0;
    if (mixed) {
        gp::launch_mixed_start(L->P, L->W, L->Mx, force_refresh ? 1 : 0, L->st);
        L->launches += 1;
    }
    if (!L->profiling) {
        // the whole loop on the device; the mixed solver's retry test reads
        // the flags afterwards
        ck(cudaGraphLaunch(L->g_loop, L->st), "graph launch");
        if (mixed) {
            ck(cudaMemcpyAsync(L->h_flag, L->W.flag, 4 * sizeof(int), cudaMemcpyDeviceToHost, L->st), "flag copy");
            ck(cudaStreamSynchronize(L->st), "newton sync");
        }
        return;
    }
    bool solve_pending = false;
    for (int guard = 0; guard <= itermax + 1; guard++) {
        ck(cudaGraphLaunch(L->g_eval, L->st), "graph launch");
        ck(cudaStreamSynchronize(L->st), "newton sync");
        L->launches += L->eval_launches;
        L->ph_ms[0] += elapsed(L->pev[0], L->pev[1]);
        L->ph_ms[1] += elapsed(L->pev[1], L->pev[2]);
        if (solve_pending) {
            L->ph_ms[2] += elapsed(L->pev[3], L->pev[4]);
            L->ph_ms[3] += elapsed(L->pev[4], L->pev[5]);
            L->ph_ms[4] += elapsed(L->pev[5], L->pev[6]);
            L->ph_ms[5] += elapsed(L->pev[6], L->pev[7]);
            solve_pending = false;
        }
        if (L->h_flag[0] == 0) return;
        if (mixed) {
            const int v = (L->h_flag[1] > 0 ? 1 : 0) | (L->h_flag[2] > 0 ? 2 : 0);
            ck(cudaGraphLaunch(mixed_graph(L, v), L->st), "graph launch");
            L->launches += L->mix_launches[v];
            L->factor_launches += L->mix_factor_launches[v];
            L->refreshes += L->h_flag[1];
            L->exact_iters += L->h_flag[2];
        } else {
            ck(cudaGraphLaunch(L->g_solve, L->st), "graph launch");
            L->launches += L->solve_graph_launches;
            L->factor_launches += L->solve_graph_factors;
        }
        solve_pending = true;
        L->solves += 1;
    }
    fail(GP_E_NUMERIC, "Newton loop did not terminate");
}

// One Newton solve of every scenario.  With the mixed solver, scenarios
// whose solve failed with inexact steps redo it from the step's starting
// point with exact Newton steps (retry_start_kernel), so that the mixed
// solver converges wherever the FP64 one does.
void solve_step(gp_layout *L, double dt, double tol, int itermax, bool force_refresh) {
    ck(cudaMemsetAsync(L->W.flag + 3, 0, sizeof(int), L->st), "memset");
    newton(L, dt, tol, itermax, force_refresh, true);
    if (L->Mx.on && L->h_flag[3] > 0) {
        L->retries += L->h_flag[3];
        gp::launch_retry_start(L->P, L->W, L->Mx, L->st);
        L->launches += 1;
        newton(L, dt, tol, itermax, false, false);
        ck(cudaMemsetAsync(L->Mx.retry, 0, L->M, L->st), "memset");
        ck(cudaMemsetAsync(L->Mx.all_exact, 0, L->M, L->st), "memset");
    }
}

// Event steps of the current fault table, and per step the scenarios whose
// faults toggle there (they take a dt = 0 re-solve after that step).
std::map<int, std::vector<uint8_t>> event_masks(const gp_layout *L) {
    std::map<int, std::vector<uint8_t>> ev;
    for (int e = 0; e < L->n_fl; e++)
        for (int k : {L->h_fl_on_step[e], L->h_fl_off_step[e]}) {
            auto &mk = ev[k];
            if (mk.empty()) mk.assign(L->M, 0);
            mk[L->h_fl_scen[e]] = 1;
        }
    return ev;
}

// One transposed Newton-Jacobian solve of the adjoint for the active
// scenarios at the current state W.z (time step dt, current fault status):
// g holds the right-hand side on entry and E lambda on exit; lambda and the
// parameter partials go to A.
void adj_solve(gp_layout *L, const gp::DevAdj &A, const gp::DevClu &Csave, double dt) {
    using namespace gp;
    const size_t M = L->M, nsys = L->n_sys;
    launch_set_double(L->W.dt, dt, L->st);
    ck(cudaMemcpyAsync(L->W.zold, L->W.z, M * nsys * sizeof(double), cudaMemcpyDeviceToDevice, L->st), "zold");
    const DevMixed exact{};
    launch_cluster(L->P, L->W, Csave, exact, 0, L->st);
    launch_network(L->P, L->W, exact, 0, L->st);
    launch_adj_rhs(L->P, L->W, Csave, A, L->st);
    launch_dag_begin(L->D, L->st);
    launch_dag_factor<double>(L->P, L->W, L->ST, L->D, L->G64, L->ST.fronts, nullptr, L->ST.ufac, L->W.active, 1,
                              L->st);
    launch_solve_bwd(L->P, L->W, L->ST, L->B, L->D, L->SG, FrontSel{nullptr, nullptr, L->ST.lfac, L->ST.ufac, nullptr, 1},
                     L->st);
    launch_adj_back(L->P, L->W, Csave, A, L->d_state_maps, L->st);
    ck(cudaGetLastError(), "adjoint launch");
}

}  // namespace

// ---------------------------------------------------------------------------
// exported API
// ---------------------------------------------------------------------------

namespace {

// Frees everything a layout holds (also a partly built one).
void free_layout(gp_layout *L) {
    if (!L) return;
    drop_graphs(L);
    if (L->st) cudaStreamSynchronize(L->st);
    if (L->st_copy) cudaStreamSynchronize(L->st_copy);
    L->call.release();
    L->traj_arena.release();
    L->fault_arena.release();
    L->iters_arena.release();
    L->dc_arena.release();
    L->trip_arena.release();
    L->arena.release();
    if (L->h_flag) cudaFreeHost(L->h_flag);
    if (L->h_dt) cudaFreeHost(L->h_dt);
    for (int i = 0; i < 8; i++)
        if (L->pev[i]) cudaEventDestroy(L->pev[i]);
    if (L->st) cudaStreamDestroy(L->st);
    if (L->st_copy) cudaStreamDestroy(L->st_copy);
    if (L->ev_snap) cudaEventDestroy(L->ev_snap);
    delete L;
}

}  // namespace

#define API_BEGIN try {
#define API_END                                  \
    }                                            \
    catch (const gp_error &e) {                  \
        g_last_error = e.what();                 \
        return e.code;                           \
    }                                            \
    catch (const std::exception &e) {            \
        g_last_error = e.what();                 \
        return GP_E_INVALID;                     \
    }                                            \
    return GP_OK;

extern "C" {

int32_t gp_abi_version(void) { return GP_ABI_VERSION; }

int32_t gp_last_error(char *buf, int32_t len) {
    if (!buf || len <= 0) return (int32_t)g_last_error.size();
    snprintf(buf, (size_t)len, "%s", g_last_error.c_str());
    return (int32_t)g_last_error.size();
}

int32_t gp_layout_create(const gp_problem *prob, int32_t M, const double *z0, const double *u0, const double *p,
                         gp_layout **out) {
    gp_layout *L = nullptr;
    API_BEGIN
    if (!prob || !out || !z0 || M <= 0) fail(GP_E_INVALID, "gp_layout_create: null argument or M <= 0");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) fail(GP_E_CUDA, "no CUDA device available");
    L = new gp_layout();
    L->M = M;
    ck(cudaGetDevice(&L->device), "cudaGetDevice");
    ck(cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking), "stream");
    ck(cudaStreamCreateWithFlags(&L->st_copy, cudaStreamNonBlocking), "stream");
    for (DeviceArena *a : {&L->arena, &L->call, &L->traj_arena, &L->trip_arena, &L->fault_arena, &L->iters_arena,
                           &L->dc_arena})
        a->st = L->st;
    build_problem(L, prob);
    build_work(L, z0, u0, p);
    build_clusters(L, prob, z0, u0, p);
    L->h_adj_ptr.assign(prob->adj_rowptr, prob->adj_rowptr + prob->n_bus + 1);
    L->h_adj.assign(prob->adj_colidx, prob->adj_colidx + prob->adj_rowptr[prob->n_bus]);
    if (gp_set_line_trips(L, 0, nullptr) != GP_OK) fail(GP_E_CUDA, "%s", g_last_error.c_str());
    ck(cudaDeviceSynchronize(), "layout create");
    *out = L;
    L = nullptr;
    }
    catch (const gp_error &e) {
        g_last_error = e.what();
        free_layout(L);
        return e.code;
    }
    catch (const std::exception &e) {
        g_last_error = e.what();
        free_layout(L);
        return GP_E_INVALID;
    }
    return GP_OK;
}

int32_t gp_layout_destroy(gp_layout *L) {
    API_BEGIN
    if (!L) return GP_OK;
    DeviceScope dev(L);
    free_layout(L);
    API_END
}

int32_t gp_layout_stats(const gp_layout *L, int64_t out[8]) {
    API_BEGIN
    if (!L || !out) fail(GP_E_INVALID, "null argument");
    const gp::Symbolic &s = L->sym;
    out[0] = L->n_red;
    out[1] = L->nnz_s;
    out[2] = s.nnz_lu;
    out[3] = s.nsup;
    out[4] = s.nlevels;
    out[5] = (int64_t)std::llround(s.flops);
    out[6] = L->sum_w2;
    out[7] = s.max_front;
    API_END
}

int32_t gp_set_state(gp_layout *L, const double *z) {
    API_BEGIN
    if (!L || !z) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    to_device(L, L->W.z, z, (size_t)L->M * L->n_sys * sizeof(double), "set state");
    API_END
}

int32_t gp_restore_initial_state(gp_layout *L) {
    API_BEGIN
    if (!L) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    ck(cudaMemcpyAsync(L->W.z, L->z_init, (size_t)L->M * L->n_sys * sizeof(double), cudaMemcpyDeviceToDevice,
                       L->st),
       "restore state");
    ck(cudaStreamSynchronize(L->st), "restore state");
    API_END
}

int32_t gp_get_state(const gp_layout *L, double *z) {
    API_BEGIN
    if (!L || !z) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    to_host(L, z, L->W.z, (size_t)L->M * L->n_sys * sizeof(double), "get state");
    API_END
}

int32_t gp_residual(gp_layout *L, const double *zold, double dt, int32_t n_faults, const gp_fault *faults,
                    const uint8_t *fault_on, double *f) {
    API_BEGIN
    if (!L || !zold || !f) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    set_faults(L, n_faults, faults);
    // expanded fault status from the per-input flags
    {
        std::vector<uint8_t> on;
        for (int m = 0; m < L->M; m++)
            for (int e = 0; e < n_faults; e++)
                if (faults[e].scenario < 0 || faults[e].scenario == m) on.push_back(fault_on ? fault_on[e] : 0);
        if (!on.empty()) to_device(L, L->d_fl_on, on.data(), on.size(), "fault flags");
    }
    const size_t n = (size_t)L->M * L->n_sys;
    to_device(L, L->W.zold, zold, n * sizeof(double), "zold");
    *L->h_dt = dt;
    to_device(L, L->W.dt, L->h_dt, sizeof(double), "dt");
    fill(L, L->W.active, 1, L->M);
    const gp::DevMixed exact{};
    gp::launch_reset_norm(L->P, L->W, exact, L->st);
    gp::launch_cluster(L->P, L->W, L->C, exact, 1, L->st);
    gp::launch_network(L->P, L->W, exact, 1, L->st);
    ck(cudaGetLastError(), "residual launch");
    ck(cudaStreamSynchronize(L->st), "residual");
    to_host(L, f, L->W.f, n * sizeof(double), "residual copy");
    API_END
}

int32_t gp_integrate(gp_layout *L, const gp_options *opt, int32_t n_faults, const gp_fault *faults, double *traj,
                     int32_t *iters, int32_t *status) {
    API_BEGIN
    if (!L || !opt) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    if (opt->n_steps < 0 || !(opt->dt > 0.0) || opt->itermax <= 0) fail(GP_E_INVALID, "bad options");
    if (opt->solver != GP_SOLVER_SCHUR_FP64 && opt->solver != GP_SOLVER_SCHUR_MIXED &&
        opt->solver != GP_SOLVER_SHARED_WOODBURY)
        fail(GP_E_INVALID, "solver %d is not available", opt->solver);
    if (opt->solver == GP_SOLVER_SHARED_WOODBURY && L->n_tr > 0)
        fail(GP_E_INVALID, "the shared-factor Woodbury solver does not take line trips");
    if (opt->solver == GP_SOLVER_SHARED_WOODBURY && L->n_dc > 0)
        fail(GP_E_INVALID, "the shared-factor Woodbury solver does not take device disconnections");
    if (opt->solver == GP_SOLVER_SHARED_WOODBURY) {
        // one fault (bus, rfault) per scenario: its rank-2 correction of P
        std::vector<int> fb(L->M, -1);
        std::vector<double> fr(L->M, 0.0);
        for (int e = 0; e < n_faults; e++)
            for (int m = 0; m < L->M; m++) {
                if (faults[e].scenario >= 0 && faults[e].scenario != m) continue;
                if (fb[m] >= 0 && (fb[m] != faults[e].bus || fr[m] != faults[e].rfault))
                    fail(GP_E_INVALID, "shared-factor Woodbury solver: scenario %d has more than one fault bus", m);
                fb[m] = faults[e].bus;
                fr[m] = faults[e].rfault;
            }
    }
    const int M = L->M, ns = opt->n_steps, nsys = L->n_sys;
    set_faults(L, n_faults, faults);
    ensure_graphs(L, opt->newton_tol, opt->itermax, opt->solver);
    if (L->Mx.on) {
        // the parameters may have changed since the last integration
        gp::launch_cluster_const(L->P, L->W, L->C, L->Mx, L->st);
        L->launches += L->C.n_tasks > 0;
    }
    ck(cudaMemsetAsync(L->W.status, 0, M * sizeof(int), L->st), "memset");
    // event steps
    std::map<int, int> ev_steps;
    for (int e = 0; e < L->n_fl; e++) {
        ev_steps[L->h_fl_on_step[e]] = 1;
        ev_steps[L->h_fl_off_step[e]] = 1;
    }
    for (int e = 0; e < L->n_tr; e++) {
        ev_steps[L->h_tr_on_step[e]] = 1;
        if (L->h_tr_off_step[e] >= 0) ev_steps[L->h_tr_off_step[e]] = 1;
    }
    if (L->n_tr > 0) ck(cudaMemsetAsync(L->d_tr_on, 0, L->n_tr, L->st), "memset");
    for (int e = 0; e < L->n_dc; e++) ev_steps[L->h_dc_on_step[e]] = 1;
    if (L->n_dc > 0) ck(cudaMemsetAsync(L->d_dc_flags, 0, L->dc_bytes, L->st), "memset");
    double *d_traj = nullptr;
    const size_t n_it = (size_t)2 * std::max(ns, 1) * M;
    if (n_it > L->iters_cap) {
        L->iters_arena.release();
        L->d_iters_buf = L->iters_arena.alloc<int>(n_it);
        L->iters_cap = n_it;
    }
    int *d_iters = L->d_iters_buf;
    ck(cudaMemsetAsync(d_iters, 0, (size_t)2 * std::max(ns, 1) * M * sizeof(int), L->st), "memset");
    // a page-locked host trajectory receives each step's snapshot as soon as
    // it is taken (copy stream); any other host buffer, all of them at the end
    bool stream_traj = false;
    const size_t tpitch = (size_t)(ns + 1) * nsys * sizeof(double);
    if (traj) {
        const size_t need = (size_t)M * (ns + 1) * nsys;
        if (need > L->traj_cap) {
            L->traj_arena.release();
            L->d_traj = L->traj_arena.alloc<double>(need);
            L->traj_cap = need;
        }
        d_traj = L->d_traj;
        cudaPointerAttributes pa{};
        stream_traj = cudaPointerGetAttributes(&pa, traj) == cudaSuccess && pa.type == cudaMemoryTypeHost;
        cudaGetLastError();
        ck(cudaMemcpy2DAsync(d_traj, tpitch, L->W.z, nsys * sizeof(double), nsys * sizeof(double), M,
                             cudaMemcpyDeviceToDevice, L->st),
           "snapshot");
    }
    auto send_slice = [&](int k) {
        if (!stream_traj) return;
        ck(cudaEventRecord(L->ev_snap, L->st), "event");
        ck(cudaStreamWaitEvent(L->st_copy, L->ev_snap, 0), "event wait");
        ck(cudaMemcpy2DAsync(traj + (size_t)k * nsys, tpitch, d_traj + (size_t)k * nsys, tpitch,
                             nsys * sizeof(double), M, cudaMemcpyDeviceToHost, L->st_copy),
           "trajectory copy");
    };
    // line trips and device disconnections end with the call, also when it
    // fails part way (the success path resets them before its last sync)
    struct EventReset {
        gp_layout *L;
        bool armed = true;
        ~EventReset() {
            if (!armed) return;
            if (L->n_tr > 0) cudaMemsetAsync(L->d_tr_on, 0, L->n_tr, L->st);
            if (L->n_dc > 0) cudaMemsetAsync(L->d_dc_flags, 0, L->dc_bytes, L->st);
            cudaStreamSynchronize(L->st);
        }
    } reset{L};
    // the copy stream ends before the call returns, on every path
    struct CopyJoin {
        cudaStream_t s;
        bool on;
        ~CopyJoin() {
            if (on) cudaStreamSynchronize(s);
        }
    } join{L->st_copy, stream_traj};
    send_slice(0);
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    ck(cudaEventRecord(e0, L->st), "event");
    L->launches = 0;
    L->factor_launches = 0;
    L->solves = 0;
    L->refreshes = 0;
    L->exact_iters = 0;
    L->retries = 0;
    for (int i = 0; i < 8; i++) L->ph_ms[i] = 0.0;
    ck(cudaMemsetAsync(L->D.err, 0, sizeof(int), L->st), "memset");
    if (opt->solver == GP_SOLVER_SHARED_WOODBURY) wb_prepare(L, opt->dt);
    // the mixed solver refreshes its kept factors at the first solve and
    // around every event (the dt = 0 re-solve and the step after it); with
    // prediction on, it starts every step from the polynomial extrapolation
    // of the previous states on the current smooth stretch (no event in
    // between), of order at most mx_predict
    bool force = true;
    const int predict = opt->solver == GP_SOLVER_SCHUR_MIXED ? L->mx_predict : 0;
    int smooth = 0;   // earlier states on the current smooth stretch
    for (int k = 1; k <= ns; k++) {
        ck(cudaMemcpyAsync(L->W.zold, L->W.z, (size_t)M * nsys * sizeof(double), cudaMemcpyDeviceToDevice, L->st),
           "zold");
        if (predict) {
            gp::launch_predict(L->W.z, L->W.zold, L->zprev, L->zprev2, L->zprev3, (size_t)M * nsys,
                               std::min(predict, smooth), L->st);
            smooth += 1;
        }
        ck(cudaMemsetAsync(L->W.active, 1, M, L->st), "memset");
        solve_step(L, opt->dt, opt->newton_tol, opt->itermax, force);
        force = false;
        ck(cudaMemcpyAsync(d_iters + (size_t)(2 * (k - 1)) * M, L->W.iters, M * sizeof(int),
                           cudaMemcpyDeviceToDevice, L->st),
           "iters");
        if (d_traj) {
            ck(cudaMemcpy2DAsync(d_traj + (size_t)k * nsys, tpitch, L->W.z, nsys * sizeof(double),
                                 nsys * sizeof(double), M, cudaMemcpyDeviceToDevice, L->st),
               "snapshot");
            send_slice(k);
        }
        if (ev_steps.count(k)) {
            ck(cudaMemsetAsync(L->W.active, 0, M, L->st), "memset");
            gp::launch_events(L->P, L->W, L->d_fl_on_step, L->d_fl_off_step, L->d_fl_scen, L->d_fl_on, L->n_fl, k,
                              L->st);
            gp::launch_events(L->P, L->W, L->d_tr_on_step, L->d_tr_off_step, L->d_tr_scen, L->d_tr_on, L->n_tr, k,
                              L->st);
            gp::launch_disconnects(L->d_dc_on_step, L->d_dc_scen, L->d_dc_idx, L->d_dc_flags, L->W.active, L->n_dc,
                                   k, L->st);
            ck(cudaMemcpyAsync(L->W.zold, L->W.z, (size_t)M * nsys * sizeof(double), cudaMemcpyDeviceToDevice,
                               L->st),
               "zold");
            solve_step(L, 0.0, opt->newton_tol, opt->itermax, true);
            force = true;
            smooth = 0;
            ck(cudaMemcpyAsync(d_iters + (size_t)(2 * (k - 1) + 1) * M, L->W.iters, M * sizeof(int),
                               cudaMemcpyDeviceToDevice, L->st),
               "iters");
        }
    }
    ck(cudaEventRecord(e1, L->st), "event");
    // the call's events end with it: lines back in service, devices online
    // (gp_residual and the next call see the intact system)
    if (L->n_tr > 0) ck(cudaMemsetAsync(L->d_tr_on, 0, L->n_tr, L->st), "memset");
    if (L->n_dc > 0) ck(cudaMemsetAsync(L->d_dc_flags, 0, L->dc_bytes, L->st), "memset");
    reset.armed = false;
    ck(cudaStreamSynchronize(L->st), "integrate");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    L->t_total_ms = ms;
    if (!L->profiling) harvest_counts(L);
    {
        int err = 0;
        to_host(L, &err, L->D.err, sizeof(int), "error flag");
        if (err) {
            // the status words still say which scenarios' waits gave up (bit 8)
            if (status) to_host(L, status, L->W.status, M * sizeof(int), "status copy");
            fail(GP_E_TIMEOUT, "a dataflow wait of the reduced-system solve ran out its iteration limit");
        }
    }
    if (stream_traj) {
        join.on = false;
        ck(cudaStreamSynchronize(L->st_copy), "trajectory copy");
    } else if (traj)
        to_host(L, traj, d_traj, (size_t)M * (ns + 1) * nsys * sizeof(double), "trajectory copy");
    std::vector<int> hi((size_t)2 * std::max(ns, 1) * M);
    to_host(L, hi.data(), d_iters, hi.size() * sizeof(int), "iters copy");
    double tot = 0.0;
    for (int m = 0; m < M; m++) {
        double s = 0.0;
        for (int q = 0; q < 2 * ns; q++) {
            const int v = hi[(size_t)q * M + m];
            if (iters) iters[(size_t)m * 2 * ns + q] = v;
            s += v;
        }
        tot = std::max(tot, s);
    }
    L->iters_total = tot;
    if (status) to_host(L, status, L->W.status, M * sizeof(int), "status copy");
    ck(cudaGetLastError(), "integrate");
    API_END
}

int32_t gp_recip_check(int32_t n, const double *x, double *r) {
    API_BEGIN
    if (n < 0 || (n > 0 && (!x || !r))) fail(GP_E_INVALID, "bad arguments");
    if (n == 0) return GP_OK;
    // the buffers and the stream go on every path out
    struct Scope {
        DeviceArena A;
        cudaStream_t st = nullptr;
        ~Scope() {
            if (st) cudaStreamSynchronize(st);
            A.release();
            if (st) cudaStreamDestroy(st);
        }
    } sc;
    ck(cudaStreamCreateWithFlags(&sc.st, cudaStreamNonBlocking), "cudaStreamCreate");
    sc.A.st = sc.st;
    const double *dx = sc.A.upload(x, (size_t)n);
    double *dr = sc.A.alloc<double>((size_t)n);
    gp::launch_recip_check(dx, dr, n, sc.st);
    ck(cudaGetLastError(), "recip check launch");
    ck(cudaMemcpyAsync(r, dr, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, sc.st), "cudaMemcpyAsync");
    ck(cudaStreamSynchronize(sc.st), "recip check");
    API_END
}

int32_t gp_cluster_selftest(const gp_problem *prob, const double *z, const double *zold, const double *u0,
                            const double *p, double dt, double *yx, double *clout, double *f, double out[4]) {
    API_BEGIN
    if (!prob || !z || !zold || !u0 || !p || !yx || !clout || !out) fail(GP_E_INVALID, "null argument");
    Plan pl;
    make_plan(prob, pl);
    gp::ClusterPlan cp;
    gp::make_cluster_plan(prob, z, u0, p, cp);
    const int n_da = prob->n_diff + prob->n_alg;
    double fmax = 0.0;
    int k = 0;
    std::vector<double> buf(96), fl(32);
    for (int c = 0; c < prob->n_clusters; c++) {
        if (prob->cl_gen[c] < 0) continue;
        const int W = prob->cl_w_size[c], ws = prob->cl_w_start[c];
        const double fm = gp::host_cluster_run(prob, cp, c, z, zold, u0, p, dt, buf.data(), clout + 8 * k, fl.data());
        fmax = std::max(fmax, fm);
        for (int j = 0; j < W; j++) {
            yx[ws + j] = buf[j];
            yx[n_da + ws + j] = buf[W + j];
            yx[2 * n_da + ws + j] = buf[2 * W + j];
            if (f) f[ws + j] = fl[j];
        }
        k++;
    }
    out[0] = fmax;
    out[1] = cp.n_class;
    out[2] = (double)cp.lu_flops;
    out[3] = cp.max_slots;
    API_END
}

int32_t gp_reduced_selftest(const gp_problem *prob, const int32_t *s_rowptr, const int32_t *s_colidx,
                            const double *s_val, const double *rhs, double *x, double out[12]) {
    API_BEGIN
    if (!prob || !s_rowptr || !s_colidx || !s_val || !rhs || !x || !out) fail(GP_E_INVALID, "null argument");
    Plan pl;
    make_plan(prob, pl);
    const int n = pl.n_red;
    auto find = [&](int r, int c, bool &hit) -> double {
        const int32_t *b = s_colidx + s_rowptr[r], *e = s_colidx + s_rowptr[r + 1];
        const int32_t *it = std::lower_bound(b, e, c);
        hit = it != e && *it == c;
        return hit ? s_val[s_rowptr[r] + (it - s_colidx - s_rowptr[r])] : 0.0;
    };
    std::vector<double> svar(pl.n_var);
    for (int v = 0; v < pl.n_var; v++) {
        bool hit;
        svar[v] = find(pl.var_r[v], pl.var_c[v], hit);
    }
    // the constant part must reproduce S off the diagonal blocks
    double mism = 0.0;
    for (int b = 0; b < pl.nb; b++)
        for (int q = prob->y_rowptr[b]; q < prob->y_rowptr[b + 1]; q++) {
            const int j = prob->y_colidx[q];
            if (j == b) continue;
            const double g = prob->y_re[q], bb = prob->y_im[q];
            const double want[4] = {-g, bb, -bb, -g};
            for (int t = 0; t < 4; t++) {
                bool hit;
                const double got = find(2 * b + t / 2, 2 * j + t % 2, hit);
                mism = std::max(mism, std::fabs(got - want[t]));
            }
        }
    std::vector<double> xp(n);
    for (int k = 0; k < n; k++) xp[k] = rhs[pl.sym.perm[k]];
    std::vector<double> fronts;
    std::vector<int> ipiv;
    const int zp = host_factor(pl, svar, fronts, ipiv);
    std::vector<double> xl = xp;
    host_level_solve(pl.sym, fronts, ipiv, xl);
    HostBlk hb;
    make_blocks(pl.sym, hb);
    host_block_solve(pl.sym, hb, fronts, ipiv, xp);
    double dmax = 0.0, xmax = 0.0;
    for (int k = 0; k < n; k++) {
        dmax = std::max(dmax, std::fabs(xp[k] - xl[k]));
        xmax = std::max(xmax, std::fabs(xl[k]));
    }
    for (int k = 0; k < n; k++) x[pl.sym.perm[k]] = xp[k];
    // the split fronts' elimination (factor_part, emulated) against the
    // one-front one: the same operations in the same order, so the same bits
    {
        DagPlan dp;
        make_dag_plan(pl.sym, dp);
        std::vector<double> fs;
        std::vector<int> ps;
        host_factor(pl, svar, fs, ps, false, &dp.nparts);
        double d = 0.0;
        for (size_t i = 0; i < fs.size(); i++) d = std::max(d, std::fabs(fs[i] - fronts[i]));
        for (int k = 0; k < n; k++)
            if (ps[k] != ipiv[k]) d = std::max(d, 1.0);
        out[11] = d;
    }
    out[0] = mism;
    out[1] = zp;
    out[2] = (double)pl.sym.nnz_lu;
    out[3] = pl.sym.nlevels;
    out[4] = xmax > 0.0 ? dmax / xmax : dmax;
    out[5] = hb.nblk;
    out[6] = hb.n_top_levels;
    out[7] = hb.max_n;
    out[9] = hb.top_order.empty() ? 0 : hb.top_max_front;
    out[10] = hb.max_v;
    // S^T from the transposed assembly lists (the adjoint's system):
    // relative residual of S^T y = rhs
    {
        std::vector<double> ft;
        std::vector<int> pt;
        host_factor(pl, svar, ft, pt, true);
        std::vector<double> yp(n);
        for (int k = 0; k < n; k++) yp[k] = rhs[pl.sym.perm[k]];
        host_level_solve(pl.sym, ft, pt, yp);
        std::vector<double> y(n), res(n);
        for (int k = 0; k < n; k++) y[pl.sym.perm[k]] = yp[k];
        for (int i = 0; i < n; i++) res[i] = -rhs[i];
        double ymax = 0.0, rmax = 0.0;
        for (int i = 0; i < n; i++)
            for (int q = s_rowptr[i]; q < s_rowptr[i + 1]; q++) res[s_colidx[q]] += s_val[q] * y[i];
        for (int i = 0; i < n; i++) {
            ymax = std::max(ymax, std::fabs(y[i]));
            rmax = std::max(rmax, std::fabs(res[i]));
        }
        out[8] = ymax > 0.0 ? rmax / ymax : rmax;
    }
    API_END
}

int32_t gp_adjoint(gp_layout *L, const gp_options *opt, int32_t n_faults, const gp_fault *faults,
                   const gp_objective *obj, int32_t checkpoint_every, double *J, double *grad_p, double *grad_z0,
                   int32_t *status) {
    API_BEGIN
    if (!L || !opt || !obj) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    using namespace gp;
    if (opt->n_steps < 1 || !(opt->dt > 0.0) || opt->itermax <= 0 || checkpoint_every < 1)
        fail(GP_E_INVALID, "bad options");
    if (opt->solver != GP_SOLVER_SCHUR_FP64) fail(GP_E_INVALID, "the adjoint runs on the FP64 Schur path");
    if (L->n_tr > 0) fail(GP_E_INVALID, "the adjoint does not take line trips");
    if (L->n_dc > 0) fail(GP_E_INVALID, "the adjoint does not take device disconnections");
    const int M = L->M, ns = opt->n_steps, K = checkpoint_every;
    const size_t nsys = L->n_sys, blk = (size_t)M * nsys;
    set_faults(L, n_faults, faults);
    ensure_graphs(L, opt->newton_tol, opt->itermax, GP_SOLVER_SCHUR_FP64);
    ck(cudaMemsetAsync(L->W.status, 0, M * sizeof(int), L->st), "memset");
    ck(cudaMemsetAsync(L->D.err, 0, sizeof(int), L->st), "memset");
    const auto ev = event_masks(L);
    // device copies of the re-solve masks
    std::map<int, uint8_t *> d_mask;
    for (const auto &kv : ev) d_mask[kv.first] = L->call.upload(kv.second);
    DeviceArena &CA = L->call;
    const int nck = (ns + K - 1) / K;                       // checkpoints at steps 0, K, 2K, ...
    double *ckp = CA.alloc<double>(blk * nck);
    double *seg = CA.alloc<double>(blk * 2 * K);           // per step: regular and re-solve states
    double *zfin = CA.alloc<double>(blk);
    L->launches = L->factor_launches = L->solves = 0;
    L->refreshes = L->exact_iters = L->retries = 0;
    for (int i = 0; i < 8; i++) L->ph_ms[i] = 0.0;
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    ck(cudaEventRecord(e0, L->st), "event");
    // one forward step k; after(0) runs after the regular solve, after(1)
    // after the re-solve of the scenarios whose faults toggle at k
    auto step = [&](int k, auto after) {
        ck(cudaMemcpyAsync(L->W.zold, L->W.z, blk * sizeof(double), cudaMemcpyDeviceToDevice, L->st), "zold");
        ck(cudaMemsetAsync(L->W.active, 1, M, L->st), "memset");
        solve_step(L, opt->dt, opt->newton_tol, opt->itermax, false);
        after(0);
        if (ev.count(k)) {
            ck(cudaMemsetAsync(L->W.active, 0, M, L->st), "memset");
            launch_events(L->P, L->W, L->d_fl_on_step, L->d_fl_off_step, L->d_fl_scen, L->d_fl_on, L->n_fl, k,
                          L->st);
            ck(cudaMemcpyAsync(L->W.zold, L->W.z, blk * sizeof(double), cudaMemcpyDeviceToDevice, L->st), "zold");
            solve_step(L, 0.0, opt->newton_tol, opt->itermax, false);
            after(1);
        }
    };
    // ---- forward, keeping the checkpoints ----
    ck(cudaMemcpyAsync(ckp, L->W.z, blk * sizeof(double), cudaMemcpyDeviceToDevice, L->st), "checkpoint");
    for (int k = 1; k <= ns; k++) {
        step(k, [](int) {});
        if (k % K == 0 && k / K < nck)
            ck(cudaMemcpyAsync(ckp + blk * (k / K), L->W.z, blk * sizeof(double), cudaMemcpyDeviceToDevice, L->st),
               "checkpoint");
    }
    ck(cudaMemcpyAsync(zfin, L->W.z, blk * sizeof(double), cudaMemcpyDeviceToDevice, L->st), "final state");
    if (status) {
        ck(cudaStreamSynchronize(L->st), "forward");
        to_host(L, status, L->W.status, M * sizeof(int), "status copy");
    }
    // ---- backward sweep ----
    DevAdj A{};
    A.g = CA.alloc<double>(blk);
    A.lam = CA.alloc<double>(blk);
    A.cadj = CA.alloc<double>((size_t)M * std::max(1, L->P.n_cl) * 2);
    A.grad = CA.alloc<double>((size_t)M * std::max(1, L->n_par));
    A.J = CA.alloc<double>(M);
    A.gen_w = L->d_gen_w;
    A.n_gen = L->n_gen;
    A.w_speed = obj->w_speed;
    A.w_volt = obj->w_volt;
    A.v_min = obj->v_min;
    ck(cudaMemsetAsync(A.g, 0, blk * sizeof(double), L->st), "memset");
    ck(cudaMemsetAsync(A.lam, 0, blk * sizeof(double), L->st), "memset");
    ck(cudaMemsetAsync(A.grad, 0, (size_t)M * std::max(1, L->n_par) * sizeof(double), L->st), "memset");
    ck(cudaMemsetAsync(A.J, 0, M * sizeof(double), L->st), "memset");
    DevClu Cs = L->C;
    Cs.n_save = 1;
    for (int v : L->cplan.rhs_base) Cs.n_save = std::max(Cs.n_save, v);
    Cs.save_lu = CA.alloc<double>((size_t)M * std::max(1, Cs.n_tasks) * Cs.n_save * 32);
    Cs.save_cc = CA.alloc<double>((size_t)M * std::max(1, L->P.n_cl) * 6);
    for (int c = nck - 1; c >= 0; c--) {
        const int ka = c * K, kb = std::min(ns, ka + K);
        // recompute the segment from its checkpoint, keeping every solve's state
        ck(cudaMemcpyAsync(L->W.z, ckp + blk * c, blk * sizeof(double), cudaMemcpyDeviceToDevice, L->st), "restore");
        launch_fault_status(L->P, L->d_fl_on_step, L->d_fl_off_step, L->d_fl_on, L->n_fl, ka, L->st);
        for (int k = ka + 1; k <= kb; k++)
            step(k, [&](int kind) {
                ck(cudaMemcpyAsync(seg + blk * (2 * (k - ka - 1) + kind), L->W.z, blk * sizeof(double),
                                   cudaMemcpyDeviceToDevice, L->st),
                   "segment state");
            });
        for (int k = kb; k > ka; k--) {
            if (ev.count(k)) {
                // the dt = 0 re-solve after step k, for the scenarios that took it
                ck(cudaMemcpyAsync(L->W.z, seg + blk * (2 * (k - ka - 1) + 1), blk * sizeof(double),
                                   cudaMemcpyDeviceToDevice, L->st),
                   "state");
                ck(cudaMemcpyAsync(L->W.active, d_mask[k], M, cudaMemcpyDeviceToDevice, L->st), "mask");
                launch_fault_status(L->P, L->d_fl_on_step, L->d_fl_off_step, L->d_fl_on, L->n_fl, k, L->st);
                adj_solve(L, A, Cs, 0.0);
            }
            // the regular solve of step k: its state is trajectory point k
            ck(cudaMemcpyAsync(L->W.z, seg + blk * (2 * (k - ka - 1)), blk * sizeof(double),
                               cudaMemcpyDeviceToDevice, L->st),
               "state");
            ck(cudaMemsetAsync(L->W.active, 1, M, L->st), "memset");
            launch_fault_status(L->P, L->d_fl_on_step, L->d_fl_off_step, L->d_fl_on, L->n_fl, k - 1, L->st);
            launch_adj_objective(L->P, L->W, A, opt->dt, L->st);
            adj_solve(L, A, Cs, opt->dt);
        }
    }
    ck(cudaMemcpyAsync(L->W.z, zfin, blk * sizeof(double), cudaMemcpyDeviceToDevice, L->st), "final state");
    launch_fault_status(L->P, L->d_fl_on_step, L->d_fl_off_step, L->d_fl_on, L->n_fl, ns, L->st);
    ck(cudaEventRecord(e1, L->st), "event");
    ck(cudaStreamSynchronize(L->st), "adjoint");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    L->t_total_ms = ms;
    if (!L->profiling) harvest_counts(L);
    {
        int err = 0;
        to_host(L, &err, L->D.err, sizeof(int), "error flag");
        if (err) {
            // the status words still say which scenarios' waits gave up (bit 8)
            if (status) to_host(L, status, L->W.status, M * sizeof(int), "status copy");
            fail(GP_E_TIMEOUT, "a dataflow wait of the reduced-system solve ran out its iteration limit");
        }
    }
    if (J) to_host(L, J, A.J, M * sizeof(double), "J copy");
    if (grad_p && L->n_par > 0)
        to_host(L, grad_p, A.grad, (size_t)M * L->n_par * sizeof(double), "grad copy");
    if (grad_z0) to_host(L, grad_z0, A.g, blk * sizeof(double), "grad z0 copy");
    API_END
}

int32_t gp_set_mixed_policy(gp_layout *L, int32_t max_age, double rho_max, int32_t exact_after, int32_t predict) {
    API_BEGIN
    if (!L) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    if (max_age < 1 || !(rho_max > 0.0) || exact_after < 1 || predict < 0 || predict > 3)
        fail(GP_E_INVALID, "bad mixed-solver policy");
    L->mx_predict = predict;
    L->mx_max_age = max_age;
    L->mx_rho_max = rho_max;
    L->mx_exact_after = exact_after;
    L->Mx.max_age = max_age;
    L->Mx.rho_max = rho_max;
    L->Mx.exact_after = exact_after;
    drop_graphs(L);   // the graphs hold the policy by value
    API_END
}

// Front position (supernode s, column-major offset) of the reduced entry
// (r, c), both in the original reduced numbering.
std::pair<int, int> front_entry(const gp::Symbolic &sym, int r, int c) {
    const int pi = sym.iperm[r], pj = sym.iperm[c];
    const int s = sym.sup_of[std::min(pi, pj)];
    auto pos = [&](int k) -> int {
        const int st0 = sym.sup_start[s], en = sym.sup_start[s + 1];
        if (k >= st0 && k < en) return k - st0;
        auto b = sym.rows.begin() + sym.row_ptr[s], e = sym.rows.begin() + sym.row_ptr[s + 1];
        auto it = std::lower_bound(b, e, k);
        if (it == e || *it != k) fail(GP_E_INVALID, "entry outside the symbolic structure");
        return (en - st0) + (int)(it - b);
    };
    return {s, pos(pi) + pos(pj) * sym.front_m(s)};
}

int32_t gp_set_line_trips(gp_layout *L, int32_t n, const gp_line_trip *trips) {
    API_BEGIN
    if (!L || (n > 0 && !trips) || n < 0) fail(GP_E_INVALID, "bad arguments");
    DeviceScope dev(L);
    if (n == 0 && L->n_tr == 0 && L->P.tr_ptr) return GP_OK;
    const int M = L->M;
    std::vector<std::vector<int>> per(M);
    for (int e = 0; e < n; e++) {
        const gp_line_trip &t = trips[e];
        if (t.from_bus < 0 || t.from_bus >= L->n_bus || t.to_bus < 0 || t.to_bus >= L->n_bus ||
            t.from_bus == t.to_bus)
            fail(GP_E_INVALID, "line trip %d: buses %d-%d", e, t.from_bus, t.to_bus);
        if (t.scenario >= M) fail(GP_E_INVALID, "line trip %d: scenario %d out of range", e, t.scenario);
        bool adjacent = false;
        for (int q = L->h_adj_ptr[t.from_bus]; q < L->h_adj_ptr[t.from_bus + 1]; q++)
            adjacent = adjacent || L->h_adj[q] == t.to_bus;
        if (!adjacent) fail(GP_E_INVALID, "line trip %d: no branch between buses %d and %d", e, t.from_bus, t.to_bus);
        if (t.scenario < 0)
            for (int m = 0; m < M; m++) per[m].push_back(e);
        else
            per[t.scenario].push_back(e);
    }
    std::vector<int> ptr(M + 1, 0), fb, tb, on, off, scen;
    std::vector<double> y;
    for (int m = 0; m < M; m++) {
        for (int e : per[m]) {
            const gp_line_trip &t = trips[e];
            fb.push_back(t.from_bus);
            tb.push_back(t.to_bus);
            for (const double *v : {t.yff, t.yft, t.ytf, t.ytt}) {
                y.push_back(v[0]);
                y.push_back(v[1]);
            }
            on.push_back(t.on_step);
            off.push_back(t.off_step);
            scen.push_back(m);
        }
        ptr[m + 1] = (int)fb.size();
    }
    // assembly entries of the off-diagonal blocks: + realified y_ft at
    // (from, to), + realified y_tf at (to, from)
    const gp::Symbolic &sym = L->sym;
    std::vector<std::vector<std::array<double, 3>>> per_s(sym.nsup);   // (position, entry, value)
    for (int e = 0; e < (int)fb.size(); e++)
        for (int side = 0; side < 2; side++) {
            const int rb = side == 0 ? fb[e] : tb[e], cb = side == 0 ? tb[e] : fb[e];
            const double g = y[8 * e + (side == 0 ? 2 : 4)], b = y[8 * e + (side == 0 ? 3 : 5)];
            const double blk[4] = {g, -b, b, g};   // (vr,vr) (vr,vi) (vi,vr) (vi,vi)
            for (int q = 0; q < 4; q++) {
                const auto fe = front_entry(sym, 2 * rb + q / 2, 2 * cb + q % 2);
                per_s[fe.first].push_back({(double)fe.second, (double)e, blk[q]});
            }
        }
    std::vector<int> ap(sym.nsup + 1, 0), apos, atr;
    std::vector<double> aval;
    for (int s = 0; s < sym.nsup; s++) {
        for (const auto &t : per_s[s]) {
            apos.push_back((int)t[0]);
            atr.push_back((int)t[1]);
            aval.push_back(t[2]);
        }
        ap[s + 1] = (int)apos.size();
    }
    L->trip_arena.release();
    DeviceArena &A = L->trip_arena;
    auto up_i = [&](const std::vector<int> &v) { return A.upload(v.empty() ? std::vector<int>{0} : v); };
    L->n_tr = (int)fb.size();
    L->P.n_tr = L->n_tr;
    L->P.tr_ptr = up_i(ptr);
    L->P.tr_from = up_i(fb);
    L->P.tr_to = up_i(tb);
    L->P.tr_y = A.upload(y.empty() ? std::vector<double>{0.0} : y);
    L->d_tr_on = A.alloc<uint8_t>(std::max(1, L->n_tr));
    fill(L, L->d_tr_on, 0, std::max(1, L->n_tr));
    L->P.tr_on = L->d_tr_on;
    L->d_tr_on_step = up_i(on);
    L->d_tr_off_step = up_i(off);
    L->d_tr_scen = up_i(scen);
    L->h_tr_on_step = on;
    L->h_tr_off_step = off;
    if (L->n_tr > 0) {
        L->S.asmt_ptr = up_i(ap);
        L->S.asmt_pos = up_i(apos);
        L->S.asmt_tr = up_i(atr);
        L->S.asmt_val = A.upload(aval.empty() ? std::vector<double>{0.0} : aval);
    } else {
        L->S.asmt_ptr = L->S.asmt_pos = L->S.asmt_tr = nullptr;
        L->S.asmt_val = nullptr;
    }
    drop_graphs(L);   // the graphs hold the problem and structure by value
    API_END
}

int32_t gp_initialize(gp_layout *L, const double *v_polar, const double *gen_pq, const double *sg_pq, double *z0,
                      double *u0, double *p) {
    API_BEGIN
    if (!L || !v_polar || (!gen_pq && L->h_ntab[GP_GENROU] > 0) || (!sg_pq && L->h_ntab[GP_STATIC_GEN] > 0))
        fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    const size_t M = L->M;
    DeviceArena A;
    A.st = L->st;
    struct Release {
        DeviceArena &a;
        ~Release() { a.release(); }
    } rel{A};
    const double *d_v = A.upload(v_polar, M * L->n_bus * 2);
    const double *d_g = A.upload(gen_pq ? gen_pq : v_polar, gen_pq ? M * L->h_ntab[GP_GENROU] * 2 : 1);
    const double *d_s = A.upload(sg_pq ? sg_pq : v_polar, sg_pq ? M * L->h_ntab[GP_STATIC_GEN] * 2 : 1);
    int *d_bad = A.alloc<int>(1);
    ck(cudaMemsetAsync(d_bad, 0, sizeof(int), L->st), "memset");
    gp::launch_initialize(L->P, L->W, d_v, d_g, d_s, d_bad, L->st);
    gp::launch_zip_const(L->P, L->W, L->d_zl_k, L->st);   // the loads' admittances changed
    ck(cudaGetLastError(), "initialise");
    ck(cudaMemcpyAsync(L->z_init, L->W.z, M * L->n_sys * sizeof(double), cudaMemcpyDeviceToDevice, L->st),
       "initial state");
    int bad = 0;
    ck(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, L->st), "status copy");
    ck(cudaStreamSynchronize(L->st), "initialise");
    if (z0) to_host(L, z0, L->W.z, M * L->n_sys * sizeof(double), "state copy");
    if (u0) to_host(L, u0, L->W.u0, M * L->n_ctrl * sizeof(double), "control copy");
    if (p) to_host(L, p, L->W.p, M * L->n_par * sizeof(double), "parameter copy");
    if (bad) fail(GP_E_NUMERIC, "%d machine initialisation(s) left a residual of 1e-9 or more", bad);
    API_END
}

int32_t gp_set_device_disconnects(gp_layout *L, int32_t n, const gp_device_disconnect *events) {
    API_BEGIN
    if (!L || (n > 0 && !events) || n < 0) fail(GP_E_INVALID, "bad arguments");
    DeviceScope dev(L);
    if (n == 0 && L->n_dc == 0) return GP_OK;
    const int M = L->M, nzl = L->h_ntab[GP_ZIPLOAD], nsg = L->h_ntab[GP_STATIC_GEN], ncl = L->P.n_cl;
    // flag areas: ZIP loads, static generators, cluster exciters
    const size_t o_zl = 0, o_sg = o_zl + (size_t)M * nzl, o_cl = o_sg + (size_t)M * nsg;
    const size_t bytes = o_cl + (size_t)M * ncl;
    std::vector<int> on, scen, idx;
    for (int e = 0; e < n; e++) {
        const gp_device_disconnect &d = events[e];
        if (d.scenario >= M) fail(GP_E_INVALID, "disconnection %d: scenario %d out of range", e, d.scenario);
        if (d.type < 0 || d.type >= GP_NTYPES || d.index < 0 || d.index >= L->h_ntab[d.type])
            fail(GP_E_INVALID, "disconnection %d: no device %d of type %d", e, d.index, d.type);
        size_t base = 0;
        int row = d.index, stride = 0;
        if (d.type == GP_ZIPLOAD) {
            base = o_zl;
            stride = nzl;
        } else if (d.type == GP_STATIC_GEN) {
            if (L->h_sg_type[d.index] == 2 || L->h_sg_type[d.index] == 3)
                fail(GP_E_INVALID, "disconnection %d: a PV or slack static generator owns algebraic rows "
                                   "(offline, its Jacobian is singular)", e);
            base = o_sg;
            stride = nsg;
        } else if (d.type == GP_SEXS || d.type == GP_ESDC1A) {
            row = -1;
            for (int c = 0; c < ncl && row < 0; c++)
                if (L->h_cl_ext[c] == d.type && L->h_cl_ex[c] == d.index) row = c;
            if (row < 0) fail(GP_E_INVALID, "disconnection %d: exciter %d belongs to no machine cluster", e, d.index);
            base = o_cl;
            stride = ncl;
        } else {
            fail(GP_E_INVALID, "disconnection %d: device type %d owns algebraic rows (offline, its Jacobian is "
                               "singular)", e, d.type);
        }
        for (int m = 0; m < M; m++) {
            if (d.scenario >= 0 && d.scenario != m) continue;
            on.push_back(d.on_step);
            scen.push_back(m);
            idx.push_back((int)(base + (size_t)m * stride + row));
        }
    }
    L->dc_arena.release();
    DeviceArena &A = L->dc_arena;
    L->n_dc = (int)on.size();
    L->h_dc_on_step = on;
    if (L->n_dc > 0) {
        auto up_i = [&](const std::vector<int> &v) { return A.upload(v); };
        L->dc_bytes = bytes;
        L->d_dc_flags = A.alloc<uint8_t>(std::max<size_t>(1, bytes));
        fill(L, L->d_dc_flags, 0, std::max<size_t>(1, bytes));
        L->d_dc_on_step = up_i(on);
        L->d_dc_scen = up_i(scen);
        L->d_dc_idx = up_i(idx);
        L->P.zl_off = L->d_dc_flags + o_zl;
        L->P.sg_off = L->d_dc_flags + o_sg;
        L->P.exc_off = L->d_dc_flags + o_cl;
    } else {
        L->dc_bytes = 0;
        L->d_dc_flags = nullptr;
        L->d_dc_on_step = L->d_dc_scen = L->d_dc_idx = nullptr;
        L->P.zl_off = L->P.sg_off = L->P.exc_off = nullptr;
    }
    drop_graphs(L);   // the graphs hold the problem by value
    API_END
}

int32_t gp_set_wait_limit(gp_layout *L, int32_t polls) {
    API_BEGIN
    if (!L || polls < 1) fail(GP_E_INVALID, "gp_set_wait_limit: null layout or polls < 1");
    DeviceScope dev(L);
    if (L->D.wait_limit != polls) {
        L->D.wait_limit = polls;
        drop_graphs(L);   // the graphs hold the schedule by value
    }
    API_END
}

int32_t gp_set_profiling(gp_layout *L, int32_t on) {
    API_BEGIN
    if (!L) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    if ((on != 0) != L->profiling) {
        L->profiling = on != 0;
        drop_graphs(L);
    }
    API_END
}

int32_t gp_last_timing(const gp_layout *L, double out[16]) {
    API_BEGIN
    if (!L || !out) fail(GP_E_INVALID, "null argument");
    for (int i = 0; i < 16; i++) out[i] = 0.0;
    out[0] = L->t_total_ms;
    out[1] = L->ph_ms[0];
    out[2] = L->ph_ms[1];
    out[3] = L->ph_ms[2];
    out[4] = L->ph_ms[3] + L->ph_ms[4];
    out[5] = L->iters_total;
    out[6] = L->launches;
    out[7] = L->ph_ms[5];
    out[8] = L->factor_launches;
    out[9] = L->solves;
    out[10] = L->refreshes;
    out[11] = L->exact_iters;
    out[12] = L->retries;
    API_END
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Residual with file-scope scratch (gp_residual_static)
// ---------------------------------------------------------------------------

namespace {

// 16 MiB of device scratch; nothing in it is assumed to survive between calls.
constexpr size_t kStaticScratchBytes = size_t(1) << 24;
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
void *g_static_ptr[kMaxDevices] = {};

// Address of g_static_scratch on the current device, looked up once per
// device (the first call on a device does it; make that call before any
// stream capture).
unsigned char *static_scratch() {
    int dev = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) fail(GP_E_INVALID, "device ordinal %d out of range", dev);
    if (!g_static_ptr[dev]) {
        void *ptr = nullptr;
        ck(cudaGetSymbolAddress(&ptr, g_static_scratch), "cudaGetSymbolAddress");
        g_static_ptr[dev] = ptr;
    }
    return (unsigned char *)g_static_ptr[dev];
}

// Carves 256-byte aligned pieces off the scratch array.
struct Carver {
    unsigned char *base;
    size_t used = 0;
    template <class T>
    T *take(size_t n) {
        T *p = (T *)(base + used);
        used += (n * sizeof(T) + 255) & ~size_t(255);
        return p;
    }
};

}  // namespace

extern "C" int32_t gp_residual_static(gp_layout *L, const double *zold, double dt, double *f) {
    API_BEGIN
    if (!L || !zold || !f) fail(GP_E_INVALID, "null argument");
    DeviceScope dev(L);
    const size_t M = L->M;
    const gp::DevProblem &P0 = L->P;
    // bytes the residual needs, with the same 256-byte rounding as Carver
    auto rnd = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t need = rnd(M * P0.n_sys * 8) * 2 + rnd(M * 3 * std::max(1, P0.net) * 8) +
                        rnd(M * 8 * std::max(1, P0.n_cl) * 8) + rnd(M * std::max(1, P0.n_var) * 8) +
                        rnd(M * std::max(1, P0.n_red) * 8) + rnd(M * 8) + rnd(M) + rnd(4) + rnd(8) +
                        rnd((M + 1) * 4);
    if (need > kStaticScratchBytes)
        fail(GP_E_INVALID, "gp_residual_static needs %zu bytes of scratch; at most %zu are available", need,
             kStaticScratchBytes);
    Carver cv{static_scratch()};
    gp::DevWork W = L->W;
    gp::DevProblem P = L->P;
    W.zold = cv.take<double>(M * P.n_sys);
    W.f = cv.take<double>(M * P.n_sys);
    W.yx = cv.take<double>(M * 3 * std::max(1, P.net));
    W.clout = cv.take<double>(M * 8 * std::max(1, P.n_cl));
    W.svar = cv.take<double>(M * std::max(1, P.n_var));
    W.xperm = cv.take<double>(M * std::max(1, P.n_red));
    W.norm = cv.take<unsigned long long>(M);
    W.active = cv.take<uint8_t>(M);
    W.flag = cv.take<int>(4);
    W.dt = cv.take<double>(1);
    int *fl_ptr = cv.take<int>(M + 1);
    // no fault applied: every scenario's fault range is empty
    P.fl_ptr = fl_ptr;
    P.fl_bus = fl_ptr;
    P.fl_on = W.active;
    P.fl_yf = W.dt;
    cudaStream_t st = L->st;
    ck(cudaMemsetAsync(fl_ptr, 0, (M + 1) * sizeof(int), st), "memset");
    ck(cudaMemsetAsync(W.active, 1, M, st), "memset");
    ck(cudaMemcpyAsync(W.zold, zold, M * P.n_sys * sizeof(double), cudaMemcpyHostToDevice, st), "zold");
    ck(cudaMemcpyAsync(W.dt, &dt, sizeof(double), cudaMemcpyHostToDevice, st), "dt");
    const gp::DevMixed exact{};
    gp::launch_reset_norm(P, W, exact, st);
    gp::launch_cluster(P, W, L->C, exact, 1, st);
    gp::launch_network(P, W, exact, 1, st);
    ck(cudaGetLastError(), "residual launch");
    ck(cudaMemcpyAsync(f, W.f, M * P.n_sys * sizeof(double), cudaMemcpyDeviceToHost, st), "residual copy");
    ck(cudaStreamSynchronize(st), "residual");
    API_END
}
