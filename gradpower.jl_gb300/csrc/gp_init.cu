// Device initialisation of a batch of scenarios whose power flows are
// solved: the restatement of initialize_dynamics! (src/dynamics.jl:123-250)
// on the GPU.  One thread per (scenario, machine cluster) initialises the
// machine (GENROU, src/generators.jl:159-285: a Newton solve of its steady
// state at the power-flow injection) and then its governor, exciter and
// stabiliser (closed forms of their steady states); one thread per
// (scenario, bus / ZIP load / static generator) sets the bus voltages, the
// loads' admittances at the solved |V| and the static generators' totals.
#include "gp_internal.h"

namespace gp {

namespace {

constexpr int kGi = 12;   // e_qp, e_dp, phi_1d, phi_2q, w, delta, v_q, v_d, i_q, i_d, e_fd, p_m

// GENROU steady-state equations at terminal voltage vm∠va and output
// pg + j qg (initialize_dynamics!(::Genrou), src/generators.jl:208-285).
__device__ void genrou_init_f(const double *x, const double *P, double pg, double qg, double vm, double va,
                              double *f) {
    const double x_d = P[0], x_q = P[1], x_dp = P[2], x_qp = P[3], x_ddp = P[4], xl = P[5], H = P[6];
    const double T_d0p = P[8], T_q0p = P[9], T_d0dp = P[10], T_q0dp = P[11];
    const double x_qdp = x_ddp;
    const double e_qp = x[0], e_dp = x[1], phi_1d = x[2], phi_2q = x[3], w = x[4], delta = x[5];
    const double v_q = x[6], v_d = x[7], i_q = x[8], i_d = x[9], e_fd = x[10], p_m = x[11];
    const double dpl = x_dp - xl, qpl = x_qp - xl;
    const double psi_de = (x_ddp - xl) / dpl * e_qp + (x_dp - x_ddp) / dpl * phi_1d;
    const double psi_qe = -(x_ddp - xl) / qpl * e_dp + (x_qp - x_ddp) / qpl * phi_2q;
    double sa, sb;
    sat_coef(P[12], P[13], sa, sb);
    const double psi2 = sqrt(psi_de * psi_de + psi_qe * psi_qe);
    const double Se = (sb == 0.0 || psi2 <= sa || psi2 == 0.0) ? 0.0 : sb * (psi2 - sa) * (psi2 - sa) / psi2;
    f[0] = (-e_qp + e_fd - (i_d - (-x_ddp + x_dp) * (-e_qp + i_d * dpl + phi_1d) / (dpl * dpl)) * (x_d - x_dp) -
            Se * psi_de) / T_d0p;
    f[1] = (-e_dp + (i_q - (-x_qdp + x_qp) * (e_dp + i_q * qpl + phi_2q) / (qpl * qpl)) * (x_q - x_qp)) / T_q0p;
    f[2] = (e_qp - i_d * dpl - phi_1d) / T_d0dp;
    f[3] = (-e_dp - i_q * qpl - phi_2q) / T_q0dp;
    f[4] = (p_m - psi_de * i_q + psi_qe * i_d) / (2.0 * H);
    f[5] = 2.0 * 3.14159265358979323846 * 60.0 * w;
    f[6] = i_d - ((x_ddp - xl) / dpl * e_qp + (x_dp - x_ddp) / dpl * phi_1d - v_q) / x_ddp;
    f[7] = i_q - (-(x_qdp - xl) / qpl * e_dp + (x_qp - x_qdp) / qpl * phi_2q + v_d) / x_qdp;
    double sd, cd;
    sincos(delta - va, &sd, &cd);
    f[8] = v_d - vm * sd;
    f[9] = v_q - vm * cd;
    f[10] = v_d * i_d + v_q * i_q - pg;
    f[11] = v_q * i_d - v_d * i_q - qg;
}

// The starting point (initial_guess!(::Genrou), src/generators.jl:159-206):
// the rotor angle from the q-axis voltage behind x_q, currents from the
// terminal power, fluxes and voltages from the steady-state relations.
__device__ void genrou_init_guess(const double *P, double pg, double qg, double vm, double va, double *x) {
    const double x_d = P[0], x_q = P[1], x_dp = P[2], x_qp = P[3], xl = P[5];
    double sva, cva;
    sincos(va, &sva, &cva);
    const double vr = vm * cva, vi = vm * sva;
    // ig = (pg - j qg) / conj(vt) = (pg - j qg) vt / |vt|^2
    const double den = vr * vr + vi * vi;
    const double igr = (pg * vr + qg * vi) / den, igi = (pg * vi - qg * vr) / den;
    // delta = angle(vt + j x_q ig)
    const double delta = atan2(vi + x_q * igr, vr - x_q * igi);
    double sd, cd;
    sincos(delta - va, &sd, &cd);
    const double v_d = vm * sd, v_q = vm * cd;
    const double vv = v_d * v_d + v_q * v_q;
    const double i_d = (pg * v_d + qg * v_q) / vv, i_q = (pg * v_q - qg * v_d) / vv;
    const double phi_d = v_q, phi_q = -v_d;
    const double e_dp = -x_qp * i_q - phi_q, e_qp = x_dp * i_d + phi_d;
    x[0] = e_qp;
    x[1] = e_dp;
    x[2] = e_qp - (x_dp - xl) * i_d;
    x[3] = -e_dp - (x_qp - xl) * i_q;
    x[4] = 0.0;
    x[5] = delta;
    x[6] = v_q;
    x[7] = v_d;
    x[8] = i_q;
    x[9] = i_d;
    x[10] = e_qp + (x_d - x_dp) * i_d;
    x[11] = pg;
}

// max |f_i|, NaN if any f_i is NaN (fmax would drop it and report a
// diverged machine as converged)
__device__ double max_abs(const double *f, int n) {
    double e = 0.0;
    for (int i = 0; i < n; i++) {
        const double a = fabs(f[i]);
        if (!(a <= e)) e = a;
    }
    return e;
}

// Newton on the machine's 12 equations with a central-difference Jacobian
// and partially pivoted elimination (the host restatement's batched_newton,
// which stands in for the reference's nlsolve call, src/dynamics.jl:49: a
// converging method lands on the same root to rounding).  Returns the final
// max |f|.
__device__ double genrou_init_solve(const double *P, double pg, double qg, double vm, double va, double *x) {
    double f[kGi], fp[kGi], fm[kGi], J[kGi][kGi];
    for (int it = 0; it < 50; it++) {
        genrou_init_f(x, P, pg, qg, vm, va, f);
        if (max_abs(f, kGi) < 1e-13) break;
        for (int j = 0; j < kGi; j++) {
            const double h = 1e-7 * fmax(1.0, fabs(x[j])), xj = x[j];
            x[j] = xj + h;
            genrou_init_f(x, P, pg, qg, vm, va, fp);
            x[j] = xj - h;
            genrou_init_f(x, P, pg, qg, vm, va, fm);
            x[j] = xj;
            for (int i = 0; i < kGi; i++) J[i][j] = (fp[i] - fm[i]) / (2.0 * h);
        }
        // J dx = f by Gaussian elimination with partial pivoting
        for (int k = 0; k < kGi; k++) {
            int piv = k;
            for (int i = k + 1; i < kGi; i++)
                if (fabs(J[i][k]) > fabs(J[piv][k])) piv = i;
            if (J[piv][k] == 0.0) return INFINITY;
            if (piv != k) {
                for (int j = 0; j < kGi; j++) {
                    const double t = J[k][j];
                    J[k][j] = J[piv][j];
                    J[piv][j] = t;
                }
                const double t = f[k];
                f[k] = f[piv];
                f[piv] = t;
            }
            for (int i = k + 1; i < kGi; i++) {
                const double l = J[i][k] / J[k][k];
                for (int j = k + 1; j < kGi; j++) J[i][j] -= l * J[k][j];
                f[i] -= l * f[k];
            }
        }
        for (int k = kGi - 1; k >= 0; k--) {
            double s = f[k];
            for (int j = k + 1; j < kGi; j++) s -= J[k][j] * f[j];
            f[k] = s / J[k][k];
        }
        for (int i = 0; i < kGi; i++) x[i] -= f[i];
    }
    genrou_init_f(x, P, pg, qg, vm, va, f);
    return max_abs(f, kGi);
}

// Stores v at a[i] when 0 <= i < n (indices come from the caller's tables).
__device__ __forceinline__ void put(double *a, int n, int i, double v) {
    if (i >= 0 && i < n) a[i] = v;
}

// One thread per (scenario, machine cluster): the machine, then the
// controllers of its cluster with the machine's e_fd0 and p_m (their
// steady states in closed form: the points the reference's controller
// solves start from satisfy their equations to rounding).
__global__ void init_cluster_kernel(DevProblem P, const double *vpol, const double *gen_pq, double *Z, double *U,
                                    double *Pv, int *bad) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.M * P.n_cl) return;
    const int m = (int)(t / P.n_cl), c = (int)(t % P.n_cl);
    double *z = Z + (size_t)m * P.n_sys, *u = U + (size_t)m * P.n_ctrl, *p = Pv + (size_t)m * P.n_par;
    const DTab &G = P.dev[0];
    const int g = P.cl_gen[c];
    const int bus = G.bus[g];
    const double vm = vpol[((size_t)m * P.n_bus + bus) * 2], va = vpol[((size_t)m * P.n_bus + bus) * 2 + 1];
    const double pg = gen_pq[((size_t)m * G.n + g) * 2], qg = gen_pq[((size_t)m * G.n + g) * 2 + 1];
    double par[14];
    for (int i = 0; i < 14; i++) par[i] = G.par_ptr[g] + i < P.n_par ? p[G.par_ptr[g] + i] : 0.0;
    double x[kGi];
    genrou_init_guess(par, pg, qg, vm, va, x);
    const double err = genrou_init_solve(par, pg, qg, vm, va, x);
    if (!(err < 1e-9)) atomicAdd(bad, 1);
    for (int i = 0; i < 6; i++) put(z, P.n_sys, G.diff_ptr[g] + i, x[i]);
    for (int i = 0; i < 4; i++) put(z, P.n_sys, G.alg_ptr[g] + i, x[6 + i]);
    put(u, P.n_ctrl, G.ctrl_ptr[g], x[10]);
    put(u, P.n_ctrl, G.ctrl_ptr[g] + 1, x[11]);
    const double e_fd0 = x[10];
    const int gt = P.cl_gov_type[c];
    if (gt == 1) {   // IEESGO: pref = pg, the lead-lag chain at rest
        const DTab &T = P.dev[1];
        const int k = P.cl_gov[c], pp = T.par_ptr[k];
        const double K2 = p[pp + 7], K3 = p[pp + 8], pref = pg;
        const double xs[5] = {0.0, 0.0, pref, K2 * pref, K2 * K3 * pref};
        for (int i = 0; i < 5; i++) put(z, P.n_sys, T.diff_ptr[k] + i, xs[i]);
        put(z, P.n_sys, T.alg_ptr[k], pg);
        put(u, P.n_ctrl, T.ctrl_ptr[k], pref);
        put(p, P.n_par, pp + 11, pref);
    } else if (gt == 2) {   // TGOV1: x2 = p_m = pg, pref = R pg
        const DTab &T = P.dev[2];
        const int k = P.cl_gov[c], pp = T.par_ptr[k];
        const double R = p[pp], T2 = p[pp + 4], T3 = p[pp + 5];
        const double pref = R * pg;
        put(z, P.n_sys, T.diff_ptr[k], (1.0 - T2 / T3) * pg);
        put(z, P.n_sys, T.diff_ptr[k] + 1, pg);
        put(z, P.n_sys, T.alg_ptr[k], pg);
        put(u, P.n_ctrl, T.ctrl_ptr[k], pref);
        put(p, P.n_par, pp + 7, pref);
    }
    const int et = P.cl_exc_type[c];
    if (et == 3) {   // SEXS: vref = e_fd0 / K + |V|
        const DTab &T = P.dev[3];
        const int k = P.cl_exc[c], pp = T.par_ptr[k];
        const double TA_TB = p[pp], K = p[pp + 2];
        const double vg = e_fd0 / K + vm;
        put(z, P.n_sys, T.diff_ptr[k], (1.0 - TA_TB) * (vg - vm));
        put(z, P.n_sys, T.diff_ptr[k] + 1, e_fd0);
        put(u, P.n_ctrl, T.ctrl_ptr[k], vg);
        put(p, P.n_par, pp + 6, vg);
    } else if (et == 4) {   // ESDC1A: the regulator output holds e_fd0 against Ke and saturation
        const DTab &T = P.dev[4];
        const int k = P.cl_exc[c], pp = T.par_ptr[k];
        const double Ka = p[pp], Kf = p[pp + 2], Tf = p[pp + 3], Ke = p[pp + 4], sat_a = p[pp + 7],
                     sat_b = p[pp + 8];
        const double sat = (sat_b == 0.0 || e_fd0 <= sat_a) ? 0.0 : sat_b * (e_fd0 - sat_a) * (e_fd0 - sat_a);
        const double vr1 = Ke * e_fd0 + sat;
        put(z, P.n_sys, T.diff_ptr[k], vr1);
        put(z, P.n_sys, T.diff_ptr[k] + 1, -(Kf / Tf) * e_fd0);
        put(z, P.n_sys, T.diff_ptr[k] + 2, e_fd0);
        put(p, P.n_par, pp + 9, vm + vr1 / Ka);
    }
    if (P.cl_pss[c] >= 0) {   // IEEEST: at rest (speed deviation 0)
        const DTab &T = P.dev[5];
        const int k = P.cl_pss[c];
        for (int i = 0; i < 7; i++) put(z, P.n_sys, T.diff_ptr[k] + i, 0.0);
        put(z, P.n_sys, T.alg_ptr[k], 0.0);
        put(u, P.n_ctrl, T.ctrl_ptr[k], 0.0);
    }
}

// One thread per (scenario, bus | ZIP load | static generator).
__global__ void init_network_kernel(DevProblem P, const double *vpol, const double *sg_pq, double *Z, double *Pv) {
    const DTab &ZL = P.dev[6], &SG = P.dev[7];
    const int per = P.n_bus + ZL.n + SG.n;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.M * per) return;
    const int m = (int)(t / per), i = (int)(t % per);
    double *z = Z + (size_t)m * P.n_sys, *p = Pv + (size_t)m * P.n_par;
    const double *v = vpol + (size_t)m * P.n_bus * 2;
    if (i < P.n_bus) {
        double s, c;
        sincos(v[2 * i + 1], &s, &c);
        put(z, P.n_sys, P.net + 2 * i, v[2 * i] * c);
        put(z, P.n_sys, P.net + 2 * i + 1, v[2 * i] * s);
    } else if (i < P.n_bus + ZL.n) {
        // the admittance that draws the load's power at the solved |V|
        const int k = i - P.n_bus, pp = ZL.par_ptr[k];
        const double v0 = v[2 * ZL.bus[k]], v2 = v0 * v0;
        put(p, P.n_par, pp + 6, v0);
        put(p, P.n_par, pp + 7, p[pp] / v2);
        put(p, P.n_par, pp + 8, p[pp + 1] / v2);
    } else {
        const int k = i - P.n_bus - ZL.n, pp = SG.par_ptr[k], bt = SG.link0[k];
        const double p0 = sg_pq[((size_t)m * SG.n + k) * 2], q0 = sg_pq[((size_t)m * SG.n + k) * 2 + 1];
        if (bt == 2) put(z, P.n_sys, SG.alg_ptr[k], q0);
        else if (bt == 3) {
            put(z, P.n_sys, SG.alg_ptr[k], p0);
            put(z, P.n_sys, SG.alg_ptr[k] + 1, q0);
        }
        put(p, P.n_par, pp, p0);
        put(p, P.n_par, pp + 1, q0);
    }
}

}  // namespace

void launch_initialize(const DevProblem &P, const DevWork &W, const double *vpol, const double *gen_pq,
                       const double *sg_pq, int *bad, cudaStream_t st) {
    const long long nn = (long long)P.M * (P.n_bus + P.dev[6].n + P.dev[7].n);
    if (nn > 0) init_network_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(P, vpol, sg_pq, W.z, W.p);
    const long long nc = (long long)P.M * P.n_cl;
    if (nc > 0) init_cluster_kernel<<<(unsigned)((nc + 63) / 64), 64, 0, st>>>(P, vpol, gen_pq, W.z, W.u0, W.p, bad);
}

}  // namespace gp
