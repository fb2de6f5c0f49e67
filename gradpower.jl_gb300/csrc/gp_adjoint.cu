// Discrete adjoint of the batched backward-Euler integration.
//
// Every Newton solve s of the forward run (regular steps and the dt = 0
// re-solves after an event) is a constraint F_s(y_s, y_{s-1}, p) = 0 with
//   F_i = y_i - y_{s-1,i} - dt_s f_i(y_s, p)   on differential rows,
//   F_i = g_i(y_s, p)                          on algebraic rows,
// and the objective is J = sum over the stored trajectory points of
// dt * r(y).  The adjoint runs the solves backwards:
//   J_s^T lambda_s = dJ/dy_s + E lambda_{s+1}       (E: differential rows)
//   dJ/dp = sum_s dt_s lambda_s^T df/dp  (differential rows)
//   dJ/dz0 = E lambda_1.
// J_s is the Newton Jacobian at the converged y_s.  It is applied through
// the same Schur structure as the forward step:
//   S^T lambda_v = g_v - (A^-1 B)^T g_w,   lambda_w = A^-T (g_w - C^T lambda_v),
// with A^-1 B from the cluster kernel, A^-T by the cluster program's solve
// operations run backwards with their operands exchanged, and S^T factored
// by the multifrontal kernels from transposed assembly lists.
//
// The reference's adjoint entry point (GradPower.adjoint, used by
// examples/adjoint.jl and test/test_adjoint_event_offset.jl) is no longer in
// its sources (src/nlp.jl:50-53); this follows the formulation those files
// exercise: the objective sum_t dt * functional(traj[:, t+1])
// (src/dynamics.jl:330-337), the gradient with respect to p at a fixed
// initial state, and the Jacobian of each step taken with the fault status
// of that step.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "gp_devices.cuh"
#include "gp_internal.h"

namespace gp {

namespace {

__device__ __forceinline__ DevRef devref_of(const DTab &T, int k) {
    DevRef d;
    d.dp = T.diff_ptr[k];
    d.ap = T.alg_ptr[k];
    d.cp = T.ctrl_ptr[k];
    d.pp = T.par_ptr[k];
    d.bus = T.bus[k];
    d.link0 = T.link0[k];
    d.link1 = T.link1[k];
    return d;
}

// Captures the raw right-hand side of one row.
struct RowSink {
    int row;
    double f;
    __device__ void put(int, int, double) {}
    __device__ void putv(int, int, double) {}
    __device__ void putf(int r, double x) {
        if (r == row) f = x;
    }
};

__device__ __forceinline__ double bus_vm(const DevProblem &P, const double *z, int bus) {
    const double vr = z[P.net + 2 * bus], vi = z[P.net + 2 * bus + 1];
    const double vm = sqrt(vr * vr + vi * vi);
    return vm == 0.0 ? 1e-12 : vm;
}

// dJ/dp += dt * lambda_row * d f_row / d p for the differentiated parameters
// of one cluster: machine inertia H and damping D, exciter gain (SEXS K,
// ESDC1A KA), governor droop (TGOV1 R, IEESGO gain K1).  Every one of them
// enters one differential row only.
__device__ void param_partials(const DevProblem &P, int c, const double *z, const double *u0, const double *p,
                               const double *lam, double dt, double *grad) {
    {
        const DevRef d = devref_of(P.dev[0], P.cl_gen[c]);
        RowSink rs{d.dp + 4, 0.0};
        double Cc[6], Ic[2];
        genrou_eval(d, P.net, z, u0, p, rs, Cc, Ic);
        const double H = p[d.pp + 6], w = z[d.dp + 4], lw = lam[d.dp + 4];
        grad[d.pp + 6] += dt * lw * (-rs.f / H);
        grad[d.pp + 7] += dt * lw * (-w / (2.0 * H));
    }
    const int gt = P.cl_gov_type[c];
    if (gt == 1) {
        const DevRef d = devref_of(P.dev[1], P.cl_gov[c]);
        const double T1 = p[d.pp], w = d.link0 < 0 ? 0.0 : z[d.link0];
        grad[d.pp + 6] += dt * lam[d.dp] * (w / T1);
    } else if (gt == 2) {
        const DevRef d = devref_of(P.dev[2], P.cl_gov[c]);
        const double R = p[d.pp], T1 = p[d.pp + 1], pref = p[d.pp + 7];
        const double w = d.link0 < 0 ? 0.0 : z[d.link0];
        grad[d.pp] += dt * lam[d.dp + 1] * (-(pref - w) / (R * R * T1));
    }
    const int et = P.cl_exc_type[c];
    if (et == 3) {
        const DevRef d = devref_of(P.dev[3], P.cl_exc[c]);
        const double TA_TB = p[d.pp], TE = p[d.pp + 3], vref = p[d.pp + 6];
        const double vs = d.link0 >= 0 ? z[d.link0] : 0.0;
        const double err = vref - bus_vm(P, z, d.bus) + vs;
        grad[d.pp + 2] += dt * lam[d.dp + 1] * ((z[d.dp] + TA_TB * err) / TE);
    } else if (et == 4) {
        const DevRef d = devref_of(P.dev[4], P.cl_exc[c]);
        const double Ta = p[d.pp + 1], Kf = p[d.pp + 2], Tf = p[d.pp + 3], vref = p[d.pp + 9];
        const double vs = d.link0 >= 0 ? z[d.link0] : 0.0;
        const double u = vref - bus_vm(P, z, d.bus) + vs - z[d.dp + 1] - (Kf / Tf) * z[d.dp + 2];
        grad[d.pp] += dt * lam[d.dp] * (u / Ta);
    }
}

// Objective at a stored trajectory point, one CTA per scenario:
//   J += dt * (w_speed * sum_gen w^2 + w_volt * sum_bus max(0, v_min - |V|)^2)
// and its gradient added to g.  The sum runs in a fixed order (per-thread
// partial sums, then a tree), so the value does not depend on scheduling.
__global__ void __launch_bounds__(256) adj_objective_kernel(DevProblem P, DevWork W, DevAdj A, double dt) {
    __shared__ double part[256];
    const int m = blockIdx.x;
    if (!W.active[m]) return;
    const double *z = W.z + (size_t)m * P.n_sys;
    double *g = A.g + (size_t)m * P.n_sys;
    double acc = 0.0;
    if (A.w_speed != 0.0)
        for (int k = threadIdx.x; k < A.n_gen; k += blockDim.x) {
            const int i = A.gen_w[k];
            const double w = z[i];
            acc += A.w_speed * w * w;
            g[i] += dt * A.w_speed * 2.0 * w;
        }
    if (A.w_volt != 0.0)
        for (int b = threadIdx.x; b < P.n_bus; b += blockDim.x) {
            const double vr = z[P.net + 2 * b], vi = z[P.net + 2 * b + 1];
            const double vm = sqrt(vr * vr + vi * vi);
            const double s = A.v_min - vm;
            if (s > 0.0 && vm > 0.0) {
                acc += A.w_volt * s * s;
                const double k = -dt * A.w_volt * 2.0 * s / vm;
                g[P.net + 2 * b] += k * vr;
                g[P.net + 2 * b + 1] += k * vi;
            }
        }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) A.J[m] += dt * part[0];
}

// (A^-1 B)^T g_w per cluster: two sums over the cluster's states with the
// A^-1 B columns the cluster kernel left in yx.
__global__ void adj_cluster_rhs_kernel(DevProblem P, DevWork W, DevAdj A) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.M * P.n_cl) return;
    const int m = (int)(t / P.n_cl), c = (int)(t % P.n_cl);
    if (!W.active[m]) return;
    const int n_da = P.n_diff + P.n_alg;
    const int ws = P.cl_w_start[c], wn = P.cl_w_size[c];
    const double *y1 = W.yx + (size_t)m * 3 * n_da + n_da + ws;
    const double *y2 = y1 + n_da;
    const double *g = A.g + (size_t)m * P.n_sys + ws;
    double s0 = 0.0, s1 = 0.0;
    for (int j = 0; j < wn; j++) {
        s0 += y1[j] * g[j];
        s1 += y2[j] * g[j];
    }
    A.cadj[((size_t)m * P.n_cl + c) * 2] = s0;
    A.cadj[((size_t)m * P.n_cl + c) * 2 + 1] = s1;
}

// Right-hand side of S^T lambda_v: the network rows minus the cluster terms,
// and the static-generator rows, in the permuted order of the factors.
__global__ void adj_network_rhs_kernel(DevProblem P, DevWork W, DevAdj A) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.M * P.n_bus) return;
    const int m = (int)(t / P.n_bus), b = (int)(t % P.n_bus);
    if (!W.active[m]) return;
    const double *g = A.g + (size_t)m * P.n_sys;
    double *xp = W.xperm + (size_t)m * P.n_red;
    double r0 = g[P.net + 2 * b], r1 = g[P.net + 2 * b + 1];
    for (int q = P.bus_cl_ptr[b]; q < P.bus_cl_ptr[b + 1]; q++) {
        const double *ca = A.cadj + ((size_t)m * P.n_cl + P.bus_cl[q]) * 2;
        r0 -= ca[0];
        r1 -= ca[1];
    }
    xp[P.iperm[2 * b]] = r0;
    xp[P.iperm[2 * b + 1]] = r1;
    const DTab &SG = P.dev[7];
    for (int q = P.bus_sg_ptr[b]; q < P.bus_sg_ptr[b + 1]; q++) {
        const int k = P.bus_sg[q];
        const int r = P.sg_red[k], ap = SG.alg_ptr[k], na = SG.link0[k] == 2 ? 1 : (SG.link0[k] == 3 ? 2 : 0);
        for (int j = 0; j < na; j++) xp[P.iperm[r + j]] = g[ap + j];
    }
}

// Cluster states of the adjoint solve, lane per cluster as in the forward
// cluster kernel: lambda_w = A^-T (g_w - C^T lambda_v) with the saved FP64
// LU values, the parameter partials, and g_w <- E lambda_w.
__global__ void __launch_bounds__(32) adj_cluster_back_kernel(DevProblem P, DevWork W, DevClu Cl, DevAdj A) {
    extern __shared__ double vals[];
    const int task = blockIdx.x, m = blockIdx.y, lane = threadIdx.x;
    if (!W.active[m]) return;
    const int cls = Cl.task_class[task];
    const int cnt = Cl.task_count[task];
    if (lane >= cnt) return;
    const int c = Cl.order[Cl.task_first[task] + lane];
    const int ws = P.cl_w_start[c], Wn = P.cl_w_size[c];
    const int rb = Cl.rhs_base[cls];
    const double *sv = Cl.save_lu + (((size_t)m * Cl.n_tasks + task) * Cl.n_save) * 32 + lane;
    for (int s = 0; s < rb; s++) vals[s * 32 + lane] = sv[s * 32];
    double *R = vals + (size_t)rb * 32;
    double *g = A.g + (size_t)m * P.n_sys;
    const int *pc = Cl.perm_col + cls * 32;
    for (int j = 0; j < Wn; j++) R[j * 32 + lane] = g[ws + pc[j]];
    // C^T lambda_v: the network rows of the cluster's bus couple to delta,
    // i_q and i_d
    const int bus = P.dev[0].bus[P.cl_gen[c]];
    const double *xp = W.xperm + (size_t)m * P.n_red;
    const double lvr = xp[P.iperm[2 * bus]], lvi = xp[P.iperm[2 * bus + 1]];
    const double *cc = Cl.save_cc + ((size_t)m * P.n_cl + c) * 6;
    const int *p3 = Cl.pos3 + cls * 3;
    for (int t = 0; t < 3; t++) R[p3[t] * 32 + lane] -= cc[t] * lvr + cc[3 + t] * lvi;
    // A^-T: the solve operations backwards, operands exchanged
    const CluOp *ops = Cl.ops;
    const int qm = Cl.prog_mid[cls], q1 = Cl.prog_ptr[cls + 1];
    for (int q = q1 - 1; q >= qm; q--) {
        const CluOp o = ops[q];
        if (o.code == OP_FMS3) R[o.b * 32 + lane] -= vals[o.a * 32 + lane] * R[o.d * 32 + lane];
        else if (o.code == OP_MUL3) R[o.d * 32 + lane] *= vals[o.a * 32 + lane];
    }
    const int *rp = Cl.row_pos + cls * 32;
    double *lam = A.lam + (size_t)m * P.n_sys;
    for (int r = 0; r < Wn; r++) lam[ws + r] = R[rp[r] * 32 + lane];
    const double dt = *W.dt;
    if (dt != 0.0)
        param_partials(P, c, W.z + (size_t)m * P.n_sys, W.u0 + (size_t)m * P.n_ctrl, W.p + (size_t)m * P.n_par, lam,
                       dt, A.grad + (size_t)m * P.n_par);
    for (int r = 0; r < Wn; r++) g[ws + r] = P.is_diff[ws + r] ? lam[ws + r] : 0.0;
}

// Network and static-generator states: lambda from the S^T solve; they are
// algebraic, so E lambda is zero there.
__global__ void adj_net_back_kernel(DevProblem P, DevWork W, DevAdj A, const int *state_bus, const int *red_of) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.M * P.n_sys) return;
    const int m = (int)(t / P.n_sys), i = (int)(t % P.n_sys);
    if (!W.active[m]) return;
    int red = -1;
    if (i >= P.net) red = i - P.net;
    else if (state_bus[i] < 0) red = red_of[i];
    if (red < 0) return;
    A.lam[(size_t)m * P.n_sys + i] = W.xperm[(size_t)m * P.n_red + P.iperm[red]];
    A.g[(size_t)m * P.n_sys + i] = 0.0;
}

// Fault status after the event schedule's toggles at steps 1..upto (an
// entry switched on and off at the same step ends off, as in events_kernel).
__global__ void fault_status_kernel(const int *on_step, const int *off_step, uint8_t *fl_on, int n_fl, int upto) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_fl) return;
    const int a = on_step[e], b = off_step[e];
    fl_on[e] = (a <= upto) && !(b <= upto && b >= a);
}

__global__ void set_double_kernel(double *dst, double v) { *dst = v; }

}  // namespace

// Sets a device scalar in stream order (the value travels as a kernel
// argument, so no host buffer has to outlive the call).
void launch_set_double(double *dst, double v, cudaStream_t st) { set_double_kernel<<<1, 1, 0, st>>>(dst, v); }

void launch_adj_objective(const DevProblem &P, const DevWork &W, const DevAdj &A, double dt, cudaStream_t st) {
    adj_objective_kernel<<<P.M, 256, 0, st>>>(P, W, A, dt);
}

void launch_adj_rhs(const DevProblem &P, const DevWork &W, const DevClu &C, const DevAdj &A, cudaStream_t st) {
    (void)C;
    const long long tc = (long long)P.M * P.n_cl;
    if (tc > 0) adj_cluster_rhs_kernel<<<(int)((tc + 127) / 128), 128, 0, st>>>(P, W, A);
    const long long tb = (long long)P.M * P.n_bus;
    adj_network_rhs_kernel<<<(int)((tb + 255) / 256), 256, 0, st>>>(P, W, A);
}

void launch_adj_back(const DevProblem &P, const DevWork &W, const DevClu &C, const DevAdj &A, const int *state_maps,
                     cudaStream_t st) {
    if (C.n_tasks > 0) {
        dim3 grid(C.n_tasks, P.M);
        adj_cluster_back_kernel<<<grid, 32, (size_t)C.max_slots * 32 * sizeof(double), st>>>(P, W, C, A);
    }
    const int n_da = P.n_diff + P.n_alg;
    const long long t = (long long)P.M * P.n_sys;
    adj_net_back_kernel<<<(int)((t + 255) / 256), 256, 0, st>>>(P, W, A, state_maps, state_maps + n_da);
}

void launch_fault_status(const DevProblem &P, const int *fl_on_step, const int *fl_off_step, uint8_t *fl_on,
                         int n_fl, int upto, cudaStream_t st) {
    (void)P;
    if (n_fl > 0) fault_status_kernel<<<(n_fl + 255) / 256, 256, 0, st>>>(fl_on_step, fl_off_step, fl_on, n_fl, upto);
}

int adj_smem_optin(int bytes) {
    if (cudaFuncSetAttribute(adj_cluster_back_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
        cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return bytes;
}

}  // namespace gp
