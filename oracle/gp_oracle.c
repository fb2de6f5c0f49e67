/*
 * gp_oracle.c — CPU oracle for the batched backward-Euler Newton step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the reference
 * GradPower.jl CPU path for one scenario so that the GPU library can be
 * checked against it; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline call it.  The library never links it.
 *
 * What it restates (GradPower.jl file:line):
 *   residual           _rhs_fun_batched!        src/dynamics.jl:265-327
 *     GENROU            _genrou_residual_one!    src/kernels/genrou.jl:48-141
 *     IEESGO            _ieesgo_residual_one!    src/kernels/ieesgo.jl:133-164
 *     TGOV1             _tgov1_residual_one!     src/kernels/tgov1.jl:73-100
 *     SEXS              _sexs_residual_one!      src/kernels/sexs.jl:74-103
 *     ESDC1A            _esdc1a_residual_one!    src/kernels/esdc1a.jl:97-131
 *     IEEEST            _ieeest_residual_one!    src/kernels/ieeest.jl:207-241
 *     ZIPLoad           _zipload_residual_one!   src/kernels/zipload.jl:33-85
 *     StaticGenerator   _static_gen_residual_one! src/kernels/static_gen.jl:107-148
 *   backward Euler     beuler_batched!          src/dynamics.jl:366-391
 *   Jacobian           _rhs_jac_batched!        src/dynamics.jl:823-857 and the
 *                      *_jacobian_one! leaves of the same kernel files
 *   BE scaling         _jacobian_beuler_indices! src/dynamics.jl:481-500
 *   pattern            preallocate_jacobian     src/dynamics.jl:687-794
 *   Newton             newton_step!             src/numerics.jl:55-176
 *   Schur Newton       newton_step_schur!       src/schur.jl:253-426,
 *                      dense LU _lu_factor!/_lu_solve! src/schur.jl:436-493
 *   time loop          integrate!               src/dynamics.jl:502-655
 *
 * The sparse LU is a left-looking Gilbert–Peierls factorisation with
 * threshold partial pivoting (tol 1e-3, diagonal preferred) after a
 * minimum-degree column ordering — the published method that KLU, the
 * reference's solver, is built on.  As in the reference, the first
 * factorisation pivots and later ones reuse the pivot sequence
 * (klu!), falling back to a fresh pivoting factorisation on a zero pivot.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/gradpower_gb300.h"

#define TWOPI60 (2.0 * 3.14159265358979323846 * 60.0)

/* ------------------------------------------------------------------ */
/* small helpers                                                        */
/* ------------------------------------------------------------------ */

typedef struct {
    int n, cap;
    int *r, *c;
    double *v;
} trip_t;

static void trip_push(trip_t *t, int r, int c, double v) {
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 1024;
        t->r = (int *)realloc(t->r, sizeof(int) * t->cap);
        t->c = (int *)realloc(t->c, sizeof(int) * t->cap);
        t->v = (double *)realloc(t->v, sizeof(double) * t->cap);
    }
    t->r[t->n] = r;
    t->c[t->n] = c;
    t->v[t->n] = v;
    t->n++;
}

static void trip_free(trip_t *t) {
    free(t->r);
    free(t->c);
    free(t->v);
    memset(t, 0, sizeof(*t));
}

static int online(const gp_device_table *T, int k) { return T->online == NULL || T->online[k]; }

static int n_sys_of(const gp_problem *P) { return P->n_diff + P->n_alg + 2 * P->n_bus; }
static int net_ptr_of(const gp_problem *P) { return P->n_diff + P->n_alg; }

/* Genrou quadratic saturation (src/generators.jl:71-85). */
static void genrou_sat_coef(double s1, double s2, double *a_out, double *b_out) {
    *a_out = 0.0;
    *b_out = 0.0;
    if (s1 <= 0.0 || s2 <= 0.0) return;
    const double e1 = 1.0, e2 = 1.2;
    double a = sqrt(s1 * e1 / (s2 * e2));
    if (a == 1.0) return;
    *a_out = e2 - (e1 - e2) / (a - 1.0);
    *b_out = s2 * e2 * (a - 1.0) * (a - 1.0) / ((e1 - e2) * (e1 - e2));
}

static double genrou_sat_se(double psi, double sa, double sb) {
    if (sb == 0.0 || psi <= sa || psi == 0.0) return 0.0;
    return sb * (psi - sa) * (psi - sa) / psi;
}

/* fault flags: which faults of this scenario are active; line trips and
 * which of them are tripped */
typedef struct {
    int n;
    const gp_fault *f;
    const uint8_t *on;
    int ntr;
    const gp_line_trip *tr;
    const uint8_t *tr_on;
} faults_t;

/* The tripped line's admittance terms of bus b: diagonal yb, to the other
 * end yo; 0 when the trip does not touch b. */
static int trip_terms(const gp_line_trip *t, int b, const double **yb, const double **yo, int *other) {
    if (t->from_bus == b) { *yb = t->yff; *yo = t->yft; *other = t->to_bus; return 1; }
    if (t->to_bus == b) { *yb = t->ytt; *yo = t->ytf; *other = t->from_bus; return 1; }
    return 0;
}

/* ------------------------------------------------------------------ */
/* residual (src/dynamics.jl:265-327 and the kernel leaves)            */
/* ------------------------------------------------------------------ */

static void residual_rhs(const gp_problem *P, const double *z, const double *u0, const double *p,
                         const faults_t *F, double *f) {
    const int net = net_ptr_of(P);
    const int nsys = n_sys_of(P);
    memset(f, 0, sizeof(double) * nsys);
    /* f_net = -Ybus * v (realified) */
    for (int i = 0; i < P->n_bus; i++) {
        double ar = 0.0, ai = 0.0;
        for (int k = P->y_rowptr[i]; k < P->y_rowptr[i + 1]; k++) {
            int j = P->y_colidx[k];
            double g = P->y_re[k], b = P->y_im[k];
            double vr = z[net + 2 * j], vi = z[net + 2 * j + 1];
            ar += g * vr - b * vi;
            ai += b * vr + g * vi;
        }
        f[net + 2 * i] = -ar;
        f[net + 2 * i + 1] = -ai;
    }
    /* GENROU */
    const gp_device_table *G = &P->dev[GP_GENROU];
    for (int k = 0; k < G->n; k++) {
        if (!online(G, k)) continue;
        int dp = G->diff_ptr[k], ap = G->alg_ptr[k], cp = G->ctrl_ptr[k], pp = G->par_ptr[k];
        int bus = G->bus[k];
        double x_d = p[pp], x_q = p[pp + 1], x_dp = p[pp + 2], x_qp = p[pp + 3], x_ddp = p[pp + 4],
               xl = p[pp + 5], H = p[pp + 6], D = p[pp + 7], T_d0p = p[pp + 8], T_q0p = p[pp + 9],
               T_d0dp = p[pp + 10], T_q0dp = p[pp + 11], S1 = p[pp + 12], S2 = p[pp + 13];
        double x_qdp = x_ddp;
        double e_qp = z[dp], e_dp = z[dp + 1], phi_1d = z[dp + 2], phi_2q = z[dp + 3], w = z[dp + 4],
               delta = z[dp + 5];
        double v_q = z[ap], v_d = z[ap + 1], i_q = z[ap + 2], i_d = z[ap + 3];
        int vr_idx = net + 2 * bus, vi_idx = vr_idx + 1;
        double vr = z[vr_idx], vi = z[vi_idx];
        int pm_idx = G->link0[k], efd_idx = G->link1 ? G->link1[k] : -1;
        double e_fd = efd_idx >= 0 ? z[efd_idx] : u0[cp];
        double p_m = pm_idx >= 0 ? z[pm_idx] : u0[cp + 1];
        double psi_de = (x_ddp - xl) / (x_dp - xl) * e_qp + (x_dp - x_ddp) / (x_dp - xl) * phi_1d;
        double psi_qe = -(x_ddp - xl) / (x_qp - xl) * e_dp + (x_qp - x_ddp) / (x_qp - xl) * phi_2q;
        double sa, sb;
        genrou_sat_coef(S1, S2, &sa, &sb);
        double psi2 = sqrt(psi_de * psi_de + psi_qe * psi_qe);
        double Se = genrou_sat_se(psi2, sa, sb);
        f[dp] = (-e_qp + e_fd -
                 (i_d - (-x_ddp + x_dp) * (-e_qp + i_d * (x_dp - xl) + phi_1d) / ((x_dp - xl) * (x_dp - xl))) *
                     (x_d - x_dp) -
                 Se * psi_de) /
                T_d0p;
        f[dp + 1] = (-e_dp +
                     (i_q - (-x_qdp + x_qp) * (e_dp + i_q * (x_qp - xl) + phi_2q) / ((x_qp - xl) * (x_qp - xl))) *
                         (x_q - x_qp)) /
                    T_q0p;
        f[dp + 2] = (e_qp - i_d * (x_dp - xl) - phi_1d) / T_d0dp;
        f[dp + 3] = (-e_dp - i_q * (x_qp - xl) - phi_2q) / T_q0dp;
        f[dp + 4] = (p_m - D * w - psi_de * i_q + psi_qe * i_d) / (2.0 * H);
        f[dp + 5] = TWOPI60 * w;
        f[ap] = i_d - ((x_ddp - xl) / (x_dp - xl) * e_qp + (x_dp - x_ddp) / (x_dp - xl) * phi_1d - v_q) / x_ddp;
        f[ap + 1] = i_q - (-(x_qdp - xl) / (x_qp - xl) * e_dp + (x_qp - x_qdp) / (x_qp - xl) * phi_2q + v_d) / x_qdp;
        double sd = sin(delta), cd = cos(delta);
        f[ap + 2] = v_d - (vr * sd - vi * cd);
        f[ap + 3] = v_q - (vr * cd + vi * sd);
        f[vr_idx] += sd * i_d + cd * i_q;
        f[vi_idx] += -cd * i_d + sd * i_q;
    }
    /* IEESGO */
    const gp_device_table *IG = &P->dev[GP_IEESGO];
    for (int k = 0; k < IG->n; k++) {
        if (!online(IG, k)) continue;
        int dp = IG->diff_ptr[k], ap = IG->alg_ptr[k], pp = IG->par_ptr[k], wi = IG->link0[k];
        double T1 = p[pp], T2 = p[pp + 1], T3 = p[pp + 2], T4 = p[pp + 3], T5 = p[pp + 4], T6 = p[pp + 5];
        double K1 = p[pp + 6], K2 = p[pp + 7], K3 = p[pp + 8], pref = p[pp + 11];
        double PF0 = z[dp], PLL = z[dp + 1], TP1 = z[dp + 2], TP2 = z[dp + 3], TP3 = z[dp + 4], p_m = z[ap];
        double w = wi < 0 ? 0.0 : z[wi];
        f[dp] = (1.0 / T1) * (K1 * w - PF0);
        f[dp + 1] = (1.0 / T3) * ((1.0 - (T2 / T3)) * PF0 - PLL);
        double SatP = pref - (T2 / T3) * PF0 - PLL;
        f[dp + 2] = (1.0 / T4) * (SatP - TP1);
        f[dp + 3] = (1.0 / T5) * (K2 * TP1 - TP2);
        f[dp + 4] = (1.0 / T6) * (K3 * TP2 - TP3);
        f[ap] = TP1 * (1.0 - K2) + TP2 * (1.0 - K3) + TP3 - p_m;
    }
    /* TGOV1 */
    const gp_device_table *TG = &P->dev[GP_TGOV1];
    for (int k = 0; k < TG->n; k++) {
        if (!online(TG, k)) continue;
        int dp = TG->diff_ptr[k], ap = TG->alg_ptr[k], pp = TG->par_ptr[k], wi = TG->link0[k];
        double R = p[pp], T1 = p[pp + 1], T2 = p[pp + 4], T3 = p[pp + 5], DT = p[pp + 6], pref = p[pp + 7];
        double x1 = z[dp], x2 = z[dp + 1], p_m = z[ap];
        double w = wi < 0 ? 0.0 : z[wi];
        double r23 = T2 / T3;
        f[dp] = (-x1 + (1.0 - r23) * x2) / T3;
        f[dp + 1] = ((pref - w) / R - x2) / T1;
        f[ap] = x1 + r23 * x2 - DT * w - p_m;
    }
    /* IEEEST */
    const gp_device_table *PS = &P->dev[GP_IEEEST];
    for (int k = 0; k < PS->n; k++) {
        if (!online(PS, k)) continue;
        int dp = PS->diff_ptr[k], ap = PS->alg_ptr[k], pp = PS->par_ptr[k], wi = PS->link0[k];
        double A1 = p[pp], A2 = p[pp + 1], A3 = p[pp + 2], A4 = p[pp + 3], A5 = p[pp + 4], A6 = p[pp + 5];
        double T1 = p[pp + 6], T2 = p[pp + 7], T3 = p[pp + 8], T4 = p[pp + 9], T5 = p[pp + 10], T6 = p[pp + 11],
               KS = p[pp + 12];
        double s0 = z[dp], s1 = z[dp + 1], s2 = z[dp + 2], s3 = z[dp + 3], s4 = z[dp + 4], s5 = z[dp + 5],
               s6 = z[dp + 6], vs = z[ap];
        double sig = wi >= 0 ? z[wi] : 0.0;
        double q = s1 - s3 - A3 * s2;
        double y2 = s3 + A5 * s2 + (A6 / A4) * q;
        double y3 = s4 + (T1 / T2) * (y2 - s4);
        double y4 = s5 + (T3 / T4) * (y3 - s5);
        f[dp] = (sig - s1 - A1 * s0) / A2;
        f[dp + 1] = s0;
        f[dp + 2] = (s1 - s3 - A3 * s2) / A4;
        f[dp + 3] = s2;
        f[dp + 4] = (y2 - s4) / T2;
        f[dp + 5] = (y3 - s5) / T4;
        f[dp + 6] = (KS * y4 - s6) / T6;
        f[ap] = vs - (T5 / T6) * (KS * y4 - s6);
    }
    /* SEXS */
    const gp_device_table *SX = &P->dev[GP_SEXS];
    for (int k = 0; k < SX->n; k++) {
        if (!online(SX, k)) continue;
        int dp = SX->diff_ptr[k], pp = SX->par_ptr[k], vsi = SX->link0[k];
        int vr_idx = net + 2 * SX->bus[k];
        double TA_TB = p[pp], TB = p[pp + 1], K = p[pp + 2], TE = p[pp + 3], vref = p[pp + 6];
        double x1 = z[dp], e_fd = z[dp + 1], vr = z[vr_idx], vi = z[vr_idx + 1];
        double vm = sqrt(vr * vr + vi * vi);
        vm = vm == 0.0 ? 1e-12 : vm;
        double vs = vsi >= 0 ? z[vsi] : 0.0;
        double err = vref - vm + vs;
        f[dp] = (-x1 + (1.0 - TA_TB) * err) / TB;
        f[dp + 1] = (-e_fd + K * (x1 + TA_TB * err)) / TE;
    }
    /* ESDC1A */
    const gp_device_table *EX = &P->dev[GP_ESDC1A];
    for (int k = 0; k < EX->n; k++) {
        if (!online(EX, k)) continue;
        int dp = EX->diff_ptr[k], pp = EX->par_ptr[k], vsi = EX->link0[k];
        int vr_idx = net + 2 * EX->bus[k];
        double Ka = p[pp], Ta = p[pp + 1], Kf = p[pp + 2], Tf = p[pp + 3], Ke = p[pp + 4], Te = p[pp + 5];
        double sat_a = p[pp + 7], sat_b = p[pp + 8], vref = p[pp + 9];
        double vr1 = z[dp], vr2 = z[dp + 1], e_fd = z[dp + 2], vr = z[vr_idx], vi = z[vr_idx + 1];
        double vm = sqrt(vr * vr + vi * vi);
        vm = vm == 0.0 ? 1e-12 : vm;
        double vs = vsi >= 0 ? z[vsi] : 0.0;
        double sat = (sat_b == 0.0 || e_fd <= sat_a) ? 0.0 : sat_b * (e_fd - sat_a) * (e_fd - sat_a);
        f[dp] = (Ka * (vref - vm + vs - vr2 - (Kf / Tf) * e_fd) - vr1) / Ta;
        f[dp + 1] = -((Kf / Tf) * e_fd + vr2) / Tf;
        f[dp + 2] = (vr1 - Ke * e_fd - sat) / Te;
    }
    /* ZIPLoad */
    const gp_device_table *ZL = &P->dev[GP_ZIPLOAD];
    for (int k = 0; k < ZL->n; k++) {
        if (!online(ZL, k)) continue;
        int pp = ZL->par_ptr[k];
        int vr_idx = net + 2 * ZL->bus[k], vi_idx = vr_idx + 1;
        double vr = z[vr_idx], vi = z[vi_idx];
        double pl = p[pp], ql = p[pp + 1], al = p[pp + 2];
        double yre = al * p[pp + 7], yim = al * p[pp + 8];
        double vm2 = vr * vr + vi * vi, vm2_tld = 0.2;
        f[vr_idx] -= vr * yre - vi * yim;
        f[vi_idx] -= vr * yim + vi * yre;
        double den = vm2 > vm2_tld ? vm2 : vm2_tld;
        f[vr_idx] -= (1.0 - al) * (pl * vr - ql * vi) / den;
        f[vi_idx] -= (1.0 - al) * (ql * vr + pl * vi) / den;
    }
    /* StaticGenerator */
    const gp_device_table *SG = &P->dev[GP_STATIC_GEN];
    for (int k = 0; k < SG->n; k++) {
        if (!online(SG, k)) continue;
        int pp = SG->par_ptr[k], ap = SG->alg_ptr[k], bt = SG->link0[k];
        int vr_idx = net + 2 * SG->bus[k], vi_idx = vr_idx + 1;
        double vr = z[vr_idx], vi = z[vi_idx];
        double vm2r = vr * vr + vi * vi, vm2 = vm2r > 0.2 ? vm2r : 0.2;
        double P_, Q_;
        if (bt == 2) { P_ = p[pp]; Q_ = z[ap]; }
        else if (bt == 3) { P_ = z[ap]; Q_ = z[ap + 1]; }
        else { P_ = p[pp]; Q_ = p[pp + 1]; }
        f[vr_idx] += (P_ * vr + Q_ * vi) / vm2;
        f[vi_idx] += (P_ * vi - Q_ * vr) / vm2;
        if (bt == 2) {
            double vset = p[pp + 2];
            f[ap] = vr * vr + vi * vi - vset * vset;
        } else if (bt == 3) {
            double vset = p[pp + 2], aset = p[pp + 3];
            f[ap] = vr - vset * cos(aset);
            f[ap + 1] = vi - vset * sin(aset);
        }
    }
    /* fault shunts (src/dynamics.jl:314-327) */
    for (int e = 0; e < F->n; e++) {
        if (!F->on[e]) continue;
        int vr_idx = net + 2 * F->f[e].bus;
        double yf = 1.0 / F->f[e].rfault;
        f[vr_idx] -= yf * z[vr_idx];
        f[vr_idx + 1] -= yf * z[vr_idx + 1];
    }
    /* tripped lines: their Ybus terms removed, f = -Y V gains +y_line V
     * (_apply_trip_line!, src/GradPower.jl:551-564) */
    for (int e = 0; e < F->ntr; e++) {
        if (!F->tr_on[e]) continue;
        const gp_line_trip *t = &F->tr[e];
        const int ends[2] = {t->from_bus, t->to_bus};
        for (int q = 0; q < 2; q++) {
            const double *yb, *yo;
            int o;
            if (q == 1 && t->to_bus == t->from_bus) break;
            trip_terms(t, ends[q], &yb, &yo, &o);
            int r = net + 2 * ends[q], c = net + 2 * o;
            double vr = z[r], vi = z[r + 1], vro = z[c], vio = z[c + 1];
            f[r] += yb[0] * vr - yb[1] * vi + yo[0] * vro - yo[1] * vio;
            f[r + 1] += yb[1] * vr + yb[0] * vi + yo[1] * vro + yo[0] * vio;
        }
    }
}

static void residual_be(const gp_problem *P, const double *z, const double *zold, const double *u0,
                        const double *p, const faults_t *F, double dt, double *f) {
    residual_rhs(P, z, u0, p, F, f);
    int nda = P->n_diff + P->n_alg;
    for (int i = 0; i < nda; i++)
        if (P->is_diff[i]) f[i] = z[i] - zold[i] - dt * f[i];
}

/* ------------------------------------------------------------------ */
/* Jacobian as triplets (values of every entry the reference writes)   */
/* ------------------------------------------------------------------ */

static void jacobian_rhs(const gp_problem *P, const double *z, const double *u0, const double *p,
                         const faults_t *F, trip_t *t) {
    (void)u0;
    const int net = net_ptr_of(P);
    /* network: -Ybus (current_injection_jacobian!, src/dynamics.jl:865-893) */
    for (int i = 0; i < P->n_bus; i++)
        for (int k = P->y_rowptr[i]; k < P->y_rowptr[i + 1]; k++) {
            int j = P->y_colidx[k];
            double g = P->y_re[k], b = P->y_im[k];
            int r = net + 2 * i, c = net + 2 * j;
            trip_push(t, r, c, -g);
            trip_push(t, r + 1, c + 1, -g);
            trip_push(t, r, c + 1, b);
            trip_push(t, r + 1, c, -b);
        }
    /* GENROU (src/kernels/genrou.jl:407-559) */
    const gp_device_table *G = &P->dev[GP_GENROU];
    for (int k = 0; k < G->n; k++) {
        if (!online(G, k)) continue;
        int dp = G->diff_ptr[k], ap = G->alg_ptr[k], pp = G->par_ptr[k], bus = G->bus[k];
        double x_d = p[pp], x_q = p[pp + 1], x_dp = p[pp + 2], x_qp = p[pp + 3], x_ddp = p[pp + 4],
               xl = p[pp + 5], H = p[pp + 6], D = p[pp + 7], T_d0p = p[pp + 8], T_q0p = p[pp + 9],
               T_d0dp = p[pp + 10], T_q0dp = p[pp + 11], S1 = p[pp + 12], S2 = p[pp + 13];
        double x_qdp = x_ddp;
        double e_qp = z[dp], e_dp = z[dp + 1], phi_1d = z[dp + 2], phi_2q = z[dp + 3], delta = z[dp + 5];
        double i_q = z[ap + 2], i_d = z[ap + 3];
        double sd = sin(delta), cd = cos(delta);
        double psi_de = (x_ddp - xl) / (x_dp - xl) * e_qp + (x_dp - x_ddp) / (x_dp - xl) * phi_1d;
        double psi_qe = -(x_ddp - xl) / (x_qp - xl) * e_dp + (x_qp - x_ddp) / (x_qp - xl) * phi_2q;
        double sa, sb;
        genrou_sat_coef(S1, S2, &sa, &sb);
        double psi2 = sqrt(psi_de * psi_de + psi_qe * psi_qe);
        double Se = genrou_sat_se(psi2, sa, sb);
        double dSe;
        if (sb == 0.0 || psi2 <= sa || psi2 == 0.0) dSe = 0.0;
        else {
            double g = psi2 - sa;
            dSe = sb * (2.0 * g * psi2 - g * g) / (psi2 * psi2);
        }
        double dpsi_de = psi2 == 0.0 ? 0.0 : psi_de / psi2;
        double dpsi_qe = psi2 == 0.0 ? 0.0 : psi_qe / psi2;
        double a_eqp = (x_ddp - xl) / (x_dp - xl), a_phi1d = (x_dp - x_ddp) / (x_dp - xl);
        double b_edp = -(x_ddp - xl) / (x_qp - xl), b_phi2q = (x_qp - x_ddp) / (x_qp - xl);
        double dT_dde = -(dSe * dpsi_de * psi_de + Se);
        double dT_dqe = -(dSe * dpsi_qe * psi_de);
        int e_qp_i = dp, e_dp_i = dp + 1, phi_1d_i = dp + 2, phi_2q_i = dp + 3, w_i = dp + 4, delta_i = dp + 5;
        int v_q_i = ap, v_d_i = ap + 1, i_q_i = ap + 2, i_d_i = ap + 3;
        int vr_i = net + 2 * bus, vi_i = vr_i + 1;
        double dpl = x_dp - xl, qpl = x_qp - xl;
        trip_push(t, dp, e_qp_i, (-(x_d - x_dp) * (-x_ddp + x_dp) / (dpl * dpl) - 1) / T_d0p + dT_dde * a_eqp / T_d0p);
        trip_push(t, dp, phi_1d_i, (x_d - x_dp) * (-x_ddp + x_dp) / (dpl * dpl) / T_d0p + dT_dde * a_phi1d / T_d0p);
        trip_push(t, dp, i_d_i, -(x_d - x_dp) * (-(-x_ddp + x_dp) / dpl + 1) / T_d0p);
        trip_push(t, dp, e_dp_i, dT_dqe * b_edp / T_d0p);
        trip_push(t, dp, phi_2q_i, dT_dqe * b_phi2q / T_d0p);
        int efd_idx = G->link1 ? G->link1[k] : -1, pm_idx = G->link0[k];
        if (efd_idx >= 0) trip_push(t, dp, efd_idx, 1.0 / T_d0p);
        trip_push(t, dp + 1, e_dp_i, (-(x_q - x_qp) * (-x_qdp + x_qp) / (qpl * qpl) - 1) / T_q0p);
        trip_push(t, dp + 1, phi_2q_i, -(x_q - x_qp) * (-x_qdp + x_qp) / (qpl * qpl) / T_q0p);
        trip_push(t, dp + 1, i_q_i, (x_q - x_qp) * (-(-x_qdp + x_qp) / qpl + 1) / T_q0p);
        trip_push(t, dp + 2, e_qp_i, 1.0 / T_d0dp);
        trip_push(t, dp + 2, phi_1d_i, -1.0 / T_d0dp);
        trip_push(t, dp + 2, i_d_i, (-x_dp + xl) / T_d0dp);
        trip_push(t, dp + 3, e_dp_i, -1.0 / T_q0dp);
        trip_push(t, dp + 3, phi_2q_i, -1.0 / T_q0dp);
        trip_push(t, dp + 3, i_q_i, (-x_qp + xl) / T_q0dp);
        trip_push(t, dp + 4, e_qp_i, -0.5 * i_q * (x_ddp - xl) / (H * dpl));
        trip_push(t, dp + 4, e_dp_i, 0.5 * i_d * (-x_ddp + xl) / (H * qpl));
        trip_push(t, dp + 4, phi_1d_i, -0.5 * i_q * (-x_ddp + x_dp) / (H * dpl));
        trip_push(t, dp + 4, phi_2q_i, 0.5 * i_d * (-x_ddp + x_qp) / (H * qpl));
        trip_push(t, dp + 4, w_i, -0.5 * D / H);
        if (pm_idx >= 0) trip_push(t, dp + 4, pm_idx, 0.5 / H);
        trip_push(t, dp + 4, i_q_i, 0.5 * (-e_qp * (x_ddp - xl) / dpl - phi_1d * (-x_ddp + x_dp) / dpl) / H);
        trip_push(t, dp + 4, i_d_i, 0.5 * (e_dp * (-x_ddp + xl) / qpl + phi_2q * (-x_ddp + x_qp) / qpl) / H);
        trip_push(t, dp + 5, w_i, TWOPI60);
        trip_push(t, ap, e_qp_i, -(x_ddp - xl) / (x_ddp * dpl));
        trip_push(t, ap, phi_1d_i, -(-x_ddp + x_dp) / (x_ddp * dpl));
        trip_push(t, ap, v_q_i, 1.0 / x_ddp);
        trip_push(t, ap, i_d_i, 1.0);
        trip_push(t, ap + 1, e_dp_i, -(-x_qdp + xl) / (x_qdp * qpl));
        trip_push(t, ap + 1, phi_2q_i, -(-x_qdp + x_qp) / (x_qdp * qpl));
        trip_push(t, ap + 1, v_d_i, -1.0 / x_qdp);
        trip_push(t, ap + 1, i_q_i, 1.0);
        double vr = z[vr_i], vi = z[vi_i];
        trip_push(t, ap + 2, delta_i, -vr * cd - vi * sd);
        trip_push(t, ap + 2, v_d_i, 1.0);
        trip_push(t, ap + 2, vr_i, -sd);
        trip_push(t, ap + 2, vi_i, cd);
        trip_push(t, ap + 3, delta_i, vr * sd - vi * cd);
        trip_push(t, ap + 3, v_q_i, 1.0);
        trip_push(t, ap + 3, vr_i, -cd);
        trip_push(t, ap + 3, vi_i, -sd);
        trip_push(t, vr_i, delta_i, i_d * cd - i_q * sd);
        trip_push(t, vr_i, i_q_i, cd);
        trip_push(t, vr_i, i_d_i, sd);
        trip_push(t, vi_i, delta_i, i_d * sd + i_q * cd);
        trip_push(t, vi_i, i_q_i, sd);
        trip_push(t, vi_i, i_d_i, -cd);
    }
    /* IEESGO (src/kernels/ieesgo.jl:184-224) */
    const gp_device_table *IG = &P->dev[GP_IEESGO];
    for (int k = 0; k < IG->n; k++) {
        if (!online(IG, k)) continue;
        int dp = IG->diff_ptr[k], ap = IG->alg_ptr[k], pp = IG->par_ptr[k], wi = IG->link0[k];
        double T1 = p[pp], T2 = p[pp + 1], T3 = p[pp + 2], T4 = p[pp + 3], T5 = p[pp + 4], T6 = p[pp + 5];
        double K1 = p[pp + 6], K2 = p[pp + 7], K3 = p[pp + 8];
        trip_push(t, dp, dp, -1.0 / T1);
        if (wi >= 0) trip_push(t, dp, wi, K1 / T1);
        trip_push(t, dp + 1, dp, (1.0 - T2 / T3) / T3);
        trip_push(t, dp + 1, dp + 1, -1.0 / T3);
        trip_push(t, dp + 2, dp, -T2 / (T3 * T4));
        trip_push(t, dp + 2, dp + 1, -1.0 / T4);
        trip_push(t, dp + 2, dp + 2, -1.0 / T4);
        trip_push(t, dp + 3, dp + 2, K2 / T5);
        trip_push(t, dp + 3, dp + 3, -1.0 / T5);
        trip_push(t, dp + 4, dp + 3, K3 / T6);
        trip_push(t, dp + 4, dp + 4, -1.0 / T6);
        trip_push(t, ap, dp + 2, 1.0 - K2);
        trip_push(t, ap, dp + 3, 1.0 - K3);
        trip_push(t, ap, dp + 4, 1.0);
        trip_push(t, ap, ap, -1.0);
    }
    /* TGOV1 (src/kernels/tgov1.jl:116-146) */
    const gp_device_table *TG = &P->dev[GP_TGOV1];
    for (int k = 0; k < TG->n; k++) {
        if (!online(TG, k)) continue;
        int dp = TG->diff_ptr[k], ap = TG->alg_ptr[k], pp = TG->par_ptr[k], wi = TG->link0[k];
        double R = p[pp], T1 = p[pp + 1], T2 = p[pp + 4], T3 = p[pp + 5], DT = p[pp + 6];
        double r23 = T2 / T3;
        trip_push(t, dp, dp, -1.0 / T3);
        trip_push(t, dp, dp + 1, (1.0 - r23) / T3);
        trip_push(t, dp + 1, dp + 1, -1.0 / T1);
        if (wi >= 0) trip_push(t, dp + 1, wi, -1.0 / (R * T1));
        trip_push(t, ap, dp, 1.0);
        trip_push(t, ap, dp + 1, r23);
        if (wi >= 0) trip_push(t, ap, wi, -DT);
        trip_push(t, ap, ap, -1.0);
    }
    /* IEEEST (src/kernels/ieeest.jl:276-359) */
    const gp_device_table *PS = &P->dev[GP_IEEEST];
    for (int k = 0; k < PS->n; k++) {
        if (!online(PS, k)) continue;
        int dp = PS->diff_ptr[k], ap = PS->alg_ptr[k], pp = PS->par_ptr[k], wi = PS->link0[k];
        double A1 = p[pp], A2 = p[pp + 1], A3 = p[pp + 2], A4 = p[pp + 3], A5 = p[pp + 4], A6 = p[pp + 5];
        double T1 = p[pp + 6], T2 = p[pp + 7], T3 = p[pp + 8], T4 = p[pp + 9], T5 = p[pp + 10], T6 = p[pp + 11],
               KS = p[pp + 12];
        double rA = A6 / A4;
        double d2[3] = {rA, A5 - A3 * rA, 1.0 - rA};
        double r12 = T1 / T2;
        double d3[4] = {r12 * d2[0], r12 * d2[1], r12 * d2[2], 1.0 - r12};
        double r34 = T3 / T4;
        double d4[5] = {r34 * d3[0], r34 * d3[1], r34 * d3[2], r34 * d3[3], 1.0 - r34};
        trip_push(t, dp, dp, -A1 / A2);
        trip_push(t, dp, dp + 1, -1.0 / A2);
        if (wi >= 0) trip_push(t, dp, wi, 1.0 / A2);
        trip_push(t, dp + 1, dp, 1.0);
        trip_push(t, dp + 2, dp + 1, 1.0 / A4);
        trip_push(t, dp + 2, dp + 2, -A3 / A4);
        trip_push(t, dp + 2, dp + 3, -1.0 / A4);
        trip_push(t, dp + 3, dp + 2, 1.0);
        for (int j = 0; j < 3; j++) trip_push(t, dp + 4, dp + 1 + j, d2[j] / T2);
        trip_push(t, dp + 4, dp + 4, -1.0 / T2);
        for (int j = 0; j < 4; j++) trip_push(t, dp + 5, dp + 1 + j, d3[j] / T4);
        trip_push(t, dp + 5, dp + 5, -1.0 / T4);
        for (int j = 0; j < 5; j++) trip_push(t, dp + 6, dp + 1 + j, KS * d4[j] / T6);
        trip_push(t, dp + 6, dp + 6, -1.0 / T6);
        double r56 = T5 / T6;
        for (int j = 0; j < 5; j++) trip_push(t, ap, dp + 1 + j, -r56 * KS * d4[j]);
        trip_push(t, ap, dp + 6, r56);
        trip_push(t, ap, ap, 1.0);
    }
    /* SEXS (src/kernels/sexs.jl:118-156) */
    const gp_device_table *SX = &P->dev[GP_SEXS];
    for (int k = 0; k < SX->n; k++) {
        if (!online(SX, k)) continue;
        int dp = SX->diff_ptr[k], pp = SX->par_ptr[k], vsi = SX->link0[k];
        int vr_i = net + 2 * SX->bus[k];
        double TA_TB = p[pp], TB = p[pp + 1], K = p[pp + 2], TE = p[pp + 3];
        double vr = z[vr_i], vi = z[vr_i + 1];
        double vm = sqrt(vr * vr + vi * vi);
        vm = vm == 0.0 ? 1e-12 : vm;
        double dvr = vr / vm, dvi = vi / vm;
        trip_push(t, dp, dp, -1.0 / TB);
        trip_push(t, dp, vr_i, -(1.0 - TA_TB) * dvr / TB);
        trip_push(t, dp, vr_i + 1, -(1.0 - TA_TB) * dvi / TB);
        if (vsi >= 0) trip_push(t, dp, vsi, (1.0 - TA_TB) / TB);
        trip_push(t, dp + 1, dp, K / TE);
        trip_push(t, dp + 1, dp + 1, -1.0 / TE);
        trip_push(t, dp + 1, vr_i, -K * TA_TB * dvr / TE);
        trip_push(t, dp + 1, vr_i + 1, -K * TA_TB * dvi / TE);
        if (vsi >= 0) trip_push(t, dp + 1, vsi, K * TA_TB / TE);
    }
    /* ESDC1A (src/kernels/esdc1a.jl:150-196) */
    const gp_device_table *EX = &P->dev[GP_ESDC1A];
    for (int k = 0; k < EX->n; k++) {
        if (!online(EX, k)) continue;
        int dp = EX->diff_ptr[k], pp = EX->par_ptr[k], vsi = EX->link0[k];
        int vr_i = net + 2 * EX->bus[k];
        double Ka = p[pp], Ta = p[pp + 1], Kf = p[pp + 2], Tf = p[pp + 3], Ke = p[pp + 4], Te = p[pp + 5];
        double sat_a = p[pp + 7], sat_b = p[pp + 8];
        double e_fd = z[dp + 2], vr = z[vr_i], vi = z[vr_i + 1];
        double vm = sqrt(vr * vr + vi * vi);
        vm = vm == 0.0 ? 1e-12 : vm;
        double dvr = vr / vm, dvi = vi / vm;
        double dsat = (sat_b == 0.0 || e_fd <= sat_a) ? 0.0 : 2.0 * sat_b * (e_fd - sat_a);
        trip_push(t, dp, dp, -1.0 / Ta);
        trip_push(t, dp, dp + 1, -Ka / Ta);
        trip_push(t, dp, dp + 2, -Ka * Kf / (Ta * Tf));
        trip_push(t, dp, vr_i, -Ka * dvr / Ta);
        trip_push(t, dp, vr_i + 1, -Ka * dvi / Ta);
        if (vsi >= 0) trip_push(t, dp, vsi, Ka / Ta);
        trip_push(t, dp + 1, dp + 1, -1.0 / Tf);
        trip_push(t, dp + 1, dp + 2, -Kf / (Tf * Tf));
        trip_push(t, dp + 2, dp, 1.0 / Te);
        trip_push(t, dp + 2, dp + 2, -(Ke + dsat) / Te);
    }
    /* ZIPLoad (src/kernels/zipload.jl:133-179) */
    const gp_device_table *ZL = &P->dev[GP_ZIPLOAD];
    for (int k = 0; k < ZL->n; k++) {
        if (!online(ZL, k)) continue;
        int pp = ZL->par_ptr[k];
        int vr_i = net + 2 * ZL->bus[k], vi_i = vr_i + 1;
        double vr = z[vr_i], vi = z[vi_i];
        double pl = p[pp], ql = p[pp + 1], al = p[pp + 2], yre = p[pp + 7], yim = p[pp + 8];
        double vm2 = vr * vr + vi * vi, vm2_tld = 0.2;
        double a11 = -al * yre, a12 = al * yim, a21 = -al * yim, a22 = -al * yre;
        double p11, p12, p21, p22;
        if (vm2 > vm2_tld) {
            double iv4 = 1.0 / (vm2 * vm2);
            p11 = (1.0 - al) * ((pl * vr - ql * vi) * 2.0 * vr - pl * vm2) * iv4;
            p12 = (1.0 - al) * ((pl * vr - ql * vi) * 2.0 * vi + ql * vm2) * iv4;
            p21 = (1.0 - al) * ((ql * vr + pl * vi) * 2.0 * vr - ql * vm2) * iv4;
            p22 = (1.0 - al) * ((ql * vr + pl * vi) * 2.0 * vi - pl * vm2) * iv4;
        } else {
            double ith = 1.0 / vm2_tld;
            p11 = (1.0 - al) * (-pl) * ith;
            p12 = (1.0 - al) * (ql)*ith;
            p21 = (1.0 - al) * (-ql) * ith;
            p22 = (1.0 - al) * (-pl) * ith;
        }
        trip_push(t, vr_i, vr_i, a11 + p11);
        trip_push(t, vr_i, vi_i, a12 + p12);
        trip_push(t, vi_i, vr_i, a21 + p21);
        trip_push(t, vi_i, vi_i, a22 + p22);
    }
    /* StaticGenerator (src/kernels/static_gen.jl:168-220) */
    const gp_device_table *SG = &P->dev[GP_STATIC_GEN];
    for (int k = 0; k < SG->n; k++) {
        if (!online(SG, k)) continue;
        int pp = SG->par_ptr[k], ap = SG->alg_ptr[k], bt = SG->link0[k];
        int vr_i = net + 2 * SG->bus[k], vi_i = vr_i + 1;
        double vr = z[vr_i], vi = z[vi_i];
        double vm2r = vr * vr + vi * vi, vm2 = vm2r > 0.2 ? vm2r : 0.2;
        double P_, Q_;
        if (bt == 2) { P_ = p[pp]; Q_ = z[ap]; }
        else if (bt == 3) { P_ = z[ap]; Q_ = z[ap + 1]; }
        else { P_ = p[pp]; Q_ = p[pp + 1]; }
        double irn = P_ * vr + Q_ * vi, iin = P_ * vi - Q_ * vr;
        double d11, d12, d21, d22;
        if (vm2r > 0.2) {
            double vm4 = vm2 * vm2;
            d11 = P_ / vm2 - 2.0 * vr * irn / vm4;
            d12 = Q_ / vm2 - 2.0 * vi * irn / vm4;
            d21 = -Q_ / vm2 - 2.0 * vr * iin / vm4;
            d22 = P_ / vm2 - 2.0 * vi * iin / vm4;
        } else {
            d11 = P_ / vm2;
            d12 = Q_ / vm2;
            d21 = -Q_ / vm2;
            d22 = P_ / vm2;
        }
        trip_push(t, vr_i, vr_i, d11);
        trip_push(t, vr_i, vi_i, d12);
        trip_push(t, vi_i, vr_i, d21);
        trip_push(t, vi_i, vi_i, d22);
        if (bt == 2) {
            trip_push(t, ap, vr_i, 2.0 * vr);
            trip_push(t, ap, vi_i, 2.0 * vi);
            trip_push(t, vr_i, ap, vi / vm2);
            trip_push(t, vi_i, ap, -vr / vm2);
        } else if (bt == 3) {
            trip_push(t, ap, vr_i, 1.0);
            trip_push(t, ap + 1, vi_i, 1.0);
            trip_push(t, vr_i, ap, vr / vm2);
            trip_push(t, vi_i, ap, vi / vm2);
            trip_push(t, vr_i, ap + 1, vi / vm2);
            trip_push(t, vi_i, ap + 1, -vr / vm2);
        }
    }
    /* faults (src/dynamics.jl:844-857) */
    for (int e = 0; e < F->n; e++) {
        if (!F->on[e]) continue;
        int r = net + 2 * F->f[e].bus;
        double yf = 1.0 / F->f[e].rfault;
        trip_push(t, r, r, -yf);
        trip_push(t, r + 1, r + 1, -yf);
    }
    /* tripped lines: + the realified line terms (the inverse of the
     * network's -Ybus blocks) */
    for (int e = 0; e < F->ntr; e++) {
        if (!F->tr_on[e]) continue;
        const gp_line_trip *tr = &F->tr[e];
        const int ends[2] = {tr->from_bus, tr->to_bus};
        for (int q = 0; q < 2; q++) {
            const double *yb, *yo;
            int o;
            if (q == 1 && tr->to_bus == tr->from_bus) break;
            trip_terms(tr, ends[q], &yb, &yo, &o);
            int r = net + 2 * ends[q], c = net + 2 * o;
            trip_push(t, r, r, yb[0]);
            trip_push(t, r + 1, r + 1, yb[0]);
            trip_push(t, r, r + 1, -yb[1]);
            trip_push(t, r + 1, r, yb[1]);
            trip_push(t, r, c, yo[0]);
            trip_push(t, r + 1, c + 1, yo[0]);
            trip_push(t, r, c + 1, -yo[1]);
            trip_push(t, r + 1, c, yo[1]);
        }
    }
}

/* ------------------------------------------------------------------ */
/* CSC pattern of J (preallocate_jacobian) and triplet -> position map */
/* ------------------------------------------------------------------ */

typedef struct {
    int n, nnz;
    int *colptr, *rowind;
    double *val;
} csc_t;

static int cmp_int(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* Build a CSC pattern from (row, col) pairs, duplicates merged. */
static csc_t csc_from_pairs(int n, int m, const int *r, const int *c) {
    csc_t A;
    A.n = n;
    int *cnt = (int *)calloc(n + 1, sizeof(int));
    for (int k = 0; k < m; k++) cnt[c[k] + 1]++;
    for (int j = 0; j < n; j++) cnt[j + 1] += cnt[j];
    int *rows = (int *)malloc(sizeof(int) * (m > 0 ? m : 1));
    int *pos = (int *)malloc(sizeof(int) * (n + 1));
    memcpy(pos, cnt, sizeof(int) * (n + 1));
    for (int k = 0; k < m; k++) rows[pos[c[k]]++] = r[k];
    A.colptr = (int *)malloc(sizeof(int) * (n + 1));
    A.rowind = (int *)malloc(sizeof(int) * (m > 0 ? m : 1));
    int nz = 0;
    A.colptr[0] = 0;
    for (int j = 0; j < n; j++) {
        int a = cnt[j], b = cnt[j + 1];
        qsort(rows + a, b - a, sizeof(int), cmp_int);
        for (int k = a; k < b; k++)
            if (k == a || rows[k] != rows[k - 1]) A.rowind[nz++] = rows[k];
        A.colptr[j + 1] = nz;
    }
    A.nnz = nz;
    A.val = (double *)calloc(nz > 0 ? nz : 1, sizeof(double));
    free(cnt);
    free(rows);
    free(pos);
    return A;
}

static void csc_free(csc_t *A) {
    free(A->colptr);
    free(A->rowind);
    free(A->val);
    memset(A, 0, sizeof(*A));
}

static int csc_find(const csc_t *A, int r, int c) {
    int lo = A->colptr[c], hi = A->colptr[c + 1] - 1;
    while (lo <= hi) {
        int mid = (lo + hi) / 2;
        if (A->rowind[mid] == r) return mid;
        if (A->rowind[mid] < r) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

/* ------------------------------------------------------------------ */
/* minimum-degree ordering on the pattern of A + A^T                    */
/* ------------------------------------------------------------------ */

typedef struct {
    int n, cap;
    int *v;
} ivec_t;

static void iv_set_sorted_union(ivec_t *a, const int *b, int nb, int skip1, int skip2) {
    /* a := a ∪ b  (both sorted), excluding skip1/skip2 */
    int *out = (int *)malloc(sizeof(int) * (a->n + nb + 1));
    int i = 0, j = 0, k = 0;
    while (i < a->n || j < nb) {
        int x;
        if (j >= nb || (i < a->n && a->v[i] < b[j])) x = a->v[i++];
        else if (i >= a->n || b[j] < a->v[i]) x = b[j++];
        else { x = a->v[i++]; j++; }
        if (x == skip1 || x == skip2) continue;
        out[k++] = x;
    }
    free(a->v);
    a->v = out;
    a->n = k;
    a->cap = k;
}

/* Returns perm[k] = node eliminated k-th. */
static int *min_degree_order(int n, const int *colptr, const int *rowind) {
    ivec_t *adj = (ivec_t *)calloc(n, sizeof(ivec_t));
    /* symmetric pattern without diagonal */
    int *deg0 = (int *)calloc(n, sizeof(int));
    for (int j = 0; j < n; j++)
        for (int k = colptr[j]; k < colptr[j + 1]; k++) {
            int i = rowind[k];
            if (i != j) { deg0[i]++; deg0[j]++; }
        }
    for (int i = 0; i < n; i++) { adj[i].v = (int *)malloc(sizeof(int) * (deg0[i] + 1)); adj[i].cap = deg0[i] + 1; }
    for (int j = 0; j < n; j++)
        for (int k = colptr[j]; k < colptr[j + 1]; k++) {
            int i = rowind[k];
            if (i != j) { adj[i].v[adj[i].n++] = j; adj[j].v[adj[j].n++] = i; }
        }
    for (int i = 0; i < n; i++) {
        qsort(adj[i].v, adj[i].n, sizeof(int), cmp_int);
        int k = 0;
        for (int q = 0; q < adj[i].n; q++)
            if (q == 0 || adj[i].v[q] != adj[i].v[q - 1]) adj[i].v[k++] = adj[i].v[q];
        adj[i].n = k;
    }
    free(deg0);
    /* degree buckets with lazy deletion: a binary heap of (deg, node) */
    int hcap = 4 * n + 16, hn = 0;
    long long *heap = (long long *)malloc(sizeof(long long) * hcap);
#define HKEY(d, v) (((long long)(d) << 32) | (unsigned)(v))
#define HPUSH(key)                                                              \
    do {                                                                        \
        if (hn == hcap) { hcap *= 2; heap = (long long *)realloc(heap, sizeof(long long) * hcap); } \
        int _i = hn++;                                                          \
        heap[_i] = (key);                                                       \
        while (_i > 0 && heap[(_i - 1) / 2] > heap[_i]) {                       \
            long long _t = heap[_i]; heap[_i] = heap[(_i - 1) / 2]; heap[(_i - 1) / 2] = _t; _i = (_i - 1) / 2; \
        }                                                                       \
    } while (0)
    for (int i = 0; i < n; i++) HPUSH(HKEY(adj[i].n, i));
    char *done = (char *)calloc(n, 1);
    int *perm = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
    int np = 0;
    while (np < n) {
        /* pop */
        long long top = heap[0];
        heap[0] = heap[--hn];
        int i = 0;
        for (;;) {
            int l = 2 * i + 1, r = l + 1, s = i;
            if (l < hn && heap[l] < heap[s]) s = l;
            if (r < hn && heap[r] < heap[s]) s = r;
            if (s == i) break;
            long long t = heap[i]; heap[i] = heap[s]; heap[s] = t; i = s;
        }
        int v = (int)(top & 0xffffffff), d = (int)(top >> 32);
        if (done[v] || d != adj[v].n) continue;
        done[v] = 1;
        perm[np++] = v;
        /* eliminate v: its neighbours form a clique */
        int nv = adj[v].n;
        int *nb = adj[v].v;
        for (int q = 0; q < nv; q++) {
            int a = nb[q];
            iv_set_sorted_union(&adj[a], nb, nv, a, v);
            HPUSH(HKEY(adj[a].n, a));
        }
        free(adj[v].v);
        adj[v].v = NULL;
        adj[v].n = 0;
    }
#undef HPUSH
#undef HKEY
    for (int i = 0; i < n; i++) free(adj[i].v);
    free(adj);
    free(heap);
    free(done);
    return perm;
}

/* ------------------------------------------------------------------ */
/* left-looking sparse LU with partial pivoting (Gilbert–Peierls)       */
/* ------------------------------------------------------------------ */

typedef struct {
    int n;
    int *q;           /* column order: step k factors original column q[k] */
    int *prow;        /* prow[k] = original row chosen as pivot k */
    int *pinv;        /* pinv[row] = k */
    /* L(:,k): original rows (not yet pivotal at step k), values divided by pivot */
    int *Lp, *Li;
    double *Lx;
    int lcap;
    /* U(:,k): pivot indices j < k in topological order, values */
    int *Up, *Uj;
    double *Ux;
    int ucap;
    double *Ud;       /* pivots */
    int valid;
    /* workspace */
    double *x;
    int *stack, *mark, *xi;
} splu_t;

static void splu_init(splu_t *F, int n, int *q) {
    memset(F, 0, sizeof(*F));
    F->n = n;
    F->q = q;
    F->prow = (int *)malloc(sizeof(int) * n);
    F->pinv = (int *)malloc(sizeof(int) * n);
    F->Lp = (int *)malloc(sizeof(int) * (n + 1));
    F->Up = (int *)malloc(sizeof(int) * (n + 1));
    F->Ud = (double *)malloc(sizeof(double) * n);
    F->lcap = F->ucap = 4 * n + 16;
    F->Li = (int *)malloc(sizeof(int) * F->lcap);
    F->Lx = (double *)malloc(sizeof(double) * F->lcap);
    F->Uj = (int *)malloc(sizeof(int) * F->ucap);
    F->Ux = (double *)malloc(sizeof(double) * F->ucap);
    F->x = (double *)calloc(n, sizeof(double));
    F->stack = (int *)malloc(sizeof(int) * 2 * n);
    F->mark = (int *)calloc(n, sizeof(int));
    F->xi = (int *)malloc(sizeof(int) * n);
}

static void splu_free(splu_t *F) {
    free(F->q); free(F->prow); free(F->pinv); free(F->Lp); free(F->Li); free(F->Lx);
    free(F->Up); free(F->Uj); free(F->Ux); free(F->Ud); free(F->x); free(F->stack);
    free(F->mark); free(F->xi);
    memset(F, 0, sizeof(*F));
}

/* Pivoting factorisation.  Returns 0, or -1 on a structurally/numerically
 * zero column. */
static int splu_factor(splu_t *F, const csc_t *A, double tol) {
    int n = F->n;
    for (int i = 0; i < n; i++) { F->pinv[i] = -1; F->mark[i] = 0; }
    int lnz = 0, unz = 0, stamp = 0;
    F->Lp[0] = 0;
    F->Up[0] = 0;
    for (int k = 0; k < n; k++) {
        int col = F->q[k];
        stamp++;
        /* reach of A(:,col) in the graph of L (pivotal rows point to L columns) */
        int top = n;
        for (int p = A->colptr[col]; p < A->colptr[col + 1]; p++) {
            int i0 = A->rowind[p];
            if (F->mark[i0] == stamp) continue;
            /* iterative DFS */
            int sp = 0;
            F->stack[sp++] = i0;
            F->stack[sp++] = -1; /* child cursor */
            F->mark[i0] = stamp;
            while (sp > 0) {
                int i = F->stack[sp - 2];
                int j = F->pinv[i];
                int cur = F->stack[sp - 1];
                int start = j >= 0 ? F->Lp[j] : 0, end = j >= 0 ? F->Lp[j + 1] : 0;
                if (cur < 0) cur = start;
                int pushed = 0;
                for (; cur < end; cur++) {
                    int r = F->Li[cur];
                    if (F->mark[r] != stamp) {
                        F->mark[r] = stamp;
                        F->stack[sp - 1] = cur + 1;
                        F->stack[sp++] = r;
                        F->stack[sp++] = -1;
                        pushed = 1;
                        break;
                    }
                }
                if (!pushed) {
                    sp -= 2;
                    F->xi[--top] = i;
                }
            }
        }
        /* numeric: x = L \ A(:,col) */
        for (int p = top; p < n; p++) F->x[F->xi[p]] = 0.0;
        for (int p = A->colptr[col]; p < A->colptr[col + 1]; p++) F->x[A->rowind[p]] = A->val[p];
        for (int p = top; p < n; p++) {
            int i = F->xi[p];
            int j = F->pinv[i];
            if (j < 0) continue;
            double xj = F->x[i];
            for (int q2 = F->Lp[j]; q2 < F->Lp[j + 1]; q2++) F->x[F->Li[q2]] -= F->Lx[q2] * xj;
        }
        /* pivot */
        int ipiv = -1;
        double amax = -1.0;
        for (int p = top; p < n; p++) {
            int i = F->xi[p];
            if (F->pinv[i] < 0) {
                double a = fabs(F->x[i]);
                if (a > amax) { amax = a; ipiv = i; }
            }
        }
        if (ipiv < 0 || amax <= 0.0) return -1;
        if (F->pinv[col] < 0 && F->mark[col] == stamp && fabs(F->x[col]) >= tol * amax) ipiv = col;
        double piv = F->x[ipiv];
        /* store U(:,k) (pivotal rows in topological order) */
        int need_u = n - top, need_l = n - top;
        if (unz + need_u > F->ucap) {
            while (unz + need_u > F->ucap) F->ucap *= 2;
            F->Uj = (int *)realloc(F->Uj, sizeof(int) * F->ucap);
            F->Ux = (double *)realloc(F->Ux, sizeof(double) * F->ucap);
        }
        if (lnz + need_l > F->lcap) {
            while (lnz + need_l > F->lcap) F->lcap *= 2;
            F->Li = (int *)realloc(F->Li, sizeof(int) * F->lcap);
            F->Lx = (double *)realloc(F->Lx, sizeof(double) * F->lcap);
        }
        for (int p = top; p < n; p++) {
            int i = F->xi[p];
            int j = F->pinv[i];
            if (j >= 0) { F->Uj[unz] = j; F->Ux[unz] = F->x[i]; unz++; }
        }
        F->Up[k + 1] = unz;
        F->Ud[k] = piv;
        F->prow[k] = ipiv;
        F->pinv[ipiv] = k;
        for (int p = top; p < n; p++) {
            int i = F->xi[p];
            if (F->pinv[i] < 0) { F->Li[lnz] = i; F->Lx[lnz] = F->x[i] / piv; lnz++; }
        }
        F->Lp[k + 1] = lnz;
    }
    F->valid = 1;
    return 0;
}

/* Refactorisation with the stored pivot sequence and patterns (klu!).
 * Returns -1 on an exactly zero pivot. */
static int splu_refactor(splu_t *F, const csc_t *A) {
    int n = F->n;
    for (int k = 0; k < n; k++) {
        int col = F->q[k];
        /* clear x over the union of U and L patterns and the pivot row */
        for (int p = F->Up[k]; p < F->Up[k + 1]; p++) F->x[F->prow[F->Uj[p]]] = 0.0;
        for (int p = F->Lp[k]; p < F->Lp[k + 1]; p++) F->x[F->Li[p]] = 0.0;
        F->x[F->prow[k]] = 0.0;
        for (int p = A->colptr[col]; p < A->colptr[col + 1]; p++) F->x[A->rowind[p]] = A->val[p];
        for (int p = F->Up[k]; p < F->Up[k + 1]; p++) {
            int j = F->Uj[p];
            double xj = F->x[F->prow[j]];
            F->Ux[p] = xj;
            for (int q2 = F->Lp[j]; q2 < F->Lp[j + 1]; q2++) F->x[F->Li[q2]] -= F->Lx[q2] * xj;
        }
        double piv = F->x[F->prow[k]];
        if (piv == 0.0 || !isfinite(piv)) return -1;
        F->Ud[k] = piv;
        for (int p = F->Lp[k]; p < F->Lp[k + 1]; p++) F->Lx[p] = F->x[F->Li[p]] / piv;
    }
    return 0;
}

/* Solve A x = b in place (b indexed by original rows, x by original columns). */
static void splu_solve(splu_t *F, double *b, double *work) {
    int n = F->n;
    /* forward: y(k) = b(prow[k]) - sum L */
    for (int i = 0; i < n; i++) work[i] = b[i];
    for (int k = 0; k < n; k++) {
        double yk = work[F->prow[k]];
        for (int p = F->Lp[k]; p < F->Lp[k + 1]; p++) work[F->Li[p]] -= F->Lx[p] * yk;
    }
    /* y in pivot order */
    double *y = b;
    for (int k = 0; k < n; k++) y[k] = work[F->prow[k]];
    /* backward: U x = y with U stored by columns */
    for (int k = n - 1; k >= 0; k--) {
        y[k] /= F->Ud[k];
        double xk = y[k];
        for (int p = F->Up[k]; p < F->Up[k + 1]; p++) y[F->Uj[p]] -= F->Ux[p] * xk;
    }
    /* x(q[k]) = y(k) */
    for (int k = 0; k < n; k++) work[F->q[k]] = y[k];
    for (int i = 0; i < n; i++) b[i] = work[i];
}

static long long splu_nnz(const splu_t *F) { return (long long)F->Lp[F->n] + F->Up[F->n] + F->n; }

/* ------------------------------------------------------------------ */
/* per-problem symbolic state                                           */
/* ------------------------------------------------------------------ */

typedef struct {
    const gp_problem *P;
    int nsys, nda, net;
    csc_t J;             /* pattern of J */
    int *is_diff_row;    /* [nsys] */
    /* Schur */
    int n_red;
    int *red_idx;        /* reduced -> global */
    int *g2r;            /* global -> reduced or -1 */
    csc_t S;
    int nt;              /* non-trivial clusters */
    int *nt_cl;          /* cluster ids */
} sym_t;

/* Collect the pattern by evaluating the Jacobian once on a state with all
 * faults on (every entry the kernels can write), plus the diagonals of the
 * differential rows and the network adjacency blocks. */
static void sym_build(sym_t *S, const gp_problem *P, const double *z, const double *u0, const double *p,
                      int nf, const gp_fault *faults) {
    memset(S, 0, sizeof(*S));
    S->P = P;
    S->nsys = n_sys_of(P);
    S->nda = P->n_diff + P->n_alg;
    S->net = net_ptr_of(P);
    trip_t t = {0};
    uint8_t *on = (uint8_t *)malloc(nf > 0 ? nf : 1);
    for (int e = 0; e < nf; e++) on[e] = 1;
    faults_t F = {nf, faults, on};
    jacobian_rhs(P, z, u0, p, &F, &t);
    free(on);
    for (int i = 0; i < S->nda; i++)
        if (P->is_diff[i]) trip_push(&t, i, i, 0.0);
    for (int b = 0; b < P->n_bus; b++) {
        int r = S->net + 2 * b;
        trip_push(&t, r, r, 0); trip_push(&t, r, r + 1, 0); trip_push(&t, r + 1, r, 0); trip_push(&t, r + 1, r + 1, 0);
        for (int k = P->adj_rowptr[b]; k < P->adj_rowptr[b + 1]; k++) {
            int c = S->net + 2 * P->adj_colidx[k];
            trip_push(&t, r, c, 0); trip_push(&t, r, c + 1, 0); trip_push(&t, r + 1, c, 0); trip_push(&t, r + 1, c + 1, 0);
        }
    }
    S->J = csc_from_pairs(S->nsys, t.n, t.r, t.c);
    trip_free(&t);
    S->is_diff_row = (int *)calloc(S->nsys, sizeof(int));
    for (int i = 0; i < S->nda; i++) S->is_diff_row[i] = P->is_diff[i];
    /* Schur sets (src/schur.jl:53-168) */
    S->g2r = (int *)malloc(sizeof(int) * S->nsys);
    for (int i = 0; i < S->nsys; i++) S->g2r[i] = -1;
    S->red_idx = (int *)malloc(sizeof(int) * S->nsys);
    S->nt_cl = (int *)malloc(sizeof(int) * (P->n_clusters + 1));
    int nr = 0;
    for (int c = 0; c < P->n_clusters; c++) {
        int trivial = P->cl_gen[c] < 0;
        if (trivial || P->cl_w_size[c] == 0) {
            for (int j = 0; j < P->cl_w_size[c]; j++) S->red_idx[nr++] = P->cl_w_start[c] + j;
        } else {
            S->nt_cl[S->nt++] = c;
        }
    }
    for (int i = S->net; i < S->nsys; i++) S->red_idx[nr++] = i;
    /* sort (reduced_global is sorted in the reference) */
    qsort(S->red_idx, nr, sizeof(int), cmp_int);
    S->n_red = nr;
    for (int k = 0; k < nr; k++) S->g2r[S->red_idx[k]] = k;
    /* S pattern: J restricted to reduced rows/cols + bus diagonal blocks + full diagonal */
    trip_t s = {0};
    for (int lj = 0; lj < nr; lj++) {
        int gj = S->red_idx[lj];
        for (int q = S->J.colptr[gj]; q < S->J.colptr[gj + 1]; q++) {
            int li = S->g2r[S->J.rowind[q]];
            if (li >= 0) trip_push(&s, li, lj, 0);
        }
        trip_push(&s, lj, lj, 0);
    }
    S->S = csc_from_pairs(nr, s.n, s.r, s.c);
    trip_free(&s);
}

static void sym_free(sym_t *S) {
    csc_free(&S->J);
    csc_free(&S->S);
    free(S->is_diff_row);
    free(S->red_idx);
    free(S->g2r);
    free(S->nt_cl);
}

/* Assemble J values (BE-scaled) into S->J.val. */
static void assemble_J(sym_t *S, const double *z, const double *u0, const double *p, const faults_t *F,
                       double dt, trip_t *t) {
    t->n = 0;
    jacobian_rhs(S->P, z, u0, p, F, t);
    memset(S->J.val, 0, sizeof(double) * S->J.nnz);
    for (int k = 0; k < t->n; k++) {
        int pos = csc_find(&S->J, t->r[k], t->c[k]);
        S->J.val[pos] += t->v[k];
    }
    /* _jacobian_beuler_indices! */
    for (int c = 0; c < S->nsys; c++)
        for (int q = S->J.colptr[c]; q < S->J.colptr[c + 1]; q++) {
            int r = S->J.rowind[q];
            if (r < S->nda && S->is_diff_row[r]) {
                S->J.val[q] *= -dt;
                if (r == c) S->J.val[q] += 1.0;
            }
        }
}

/* ------------------------------------------------------------------ */
/* dense LU with partial pivoting (src/schur.jl:436-493)               */
/* ------------------------------------------------------------------ */

static void dense_lu(double *A, int *ipiv, int n) { /* column-major A[i + j*n] */
    for (int k = 0; k < n; k++) {
        double mx = fabs(A[k + k * n]);
        int mr = k;
        for (int i = k + 1; i < n; i++) {
            double v = fabs(A[i + k * n]);
            if (v > mx) { mx = v; mr = i; }
        }
        ipiv[k] = mr;
        if (mr != k)
            for (int j = 0; j < n; j++) { double t = A[k + j * n]; A[k + j * n] = A[mr + j * n]; A[mr + j * n] = t; }
        double akk = A[k + k * n];
        if (akk != 0.0) {
            double inv = 1.0 / akk;
            for (int i = k + 1; i < n; i++) {
                A[i + k * n] *= inv;
                for (int j = k + 1; j < n; j++) A[i + j * n] -= A[i + k * n] * A[k + j * n];
            }
        }
    }
}

static void dense_solve(const double *A, const int *ipiv, double *b, int n) {
    for (int k = 0; k < n; k++) {
        int p = ipiv[k];
        if (p != k) { double t = b[k]; b[k] = b[p]; b[p] = t; }
    }
    for (int k = 0; k < n; k++)
        for (int i = k + 1; i < n; i++) b[i] -= A[i + k * n] * b[k];
    for (int k = n - 1; k >= 0; k--) {
        b[k] /= A[k + k * n];
        for (int i = 0; i < k; i++) b[i] -= A[i + k * n] * b[k];
    }
}

/* ------------------------------------------------------------------ */
/* Newton steps                                                         */
/* ------------------------------------------------------------------ */

typedef struct {
    sym_t *S;
    splu_t LU;          /* monolithic factor of J or of S */
    int have_lu;
    trip_t t;
    double *f, *dx, *work, *zb;
    /* Schur workspace */
    double *Ak, *Bk, *Ck, *tmp, *rhs, *dz;
    int *ipiv;
    int wmax;
    long long factor_count, refactor_count;
} newton_ws;

static int factor_or_refactor(newton_ws *W, const csc_t *A, int fresh) {
    if (!W->have_lu) {
        int *q = min_degree_order(A->n, A->colptr, A->rowind);
        splu_init(&W->LU, A->n, q);
        W->have_lu = 1;
        fresh = 1;
    }
    if (!fresh && W->LU.valid) {
        if (splu_refactor(&W->LU, A) == 0) { W->refactor_count++; return 0; }
    }
    W->factor_count++;
    return splu_factor(&W->LU, A, 1e-3);
}

static double inf_norm(const double *f, int n) {
    double m = 0.0;
    for (int i = 0; i < n; i++) {
        double a = fabs(f[i]);
        if (!(a <= m)) m = a; /* propagates NaN */
    }
    return m;
}

/* Newton solve on the full Jacobian.  Returns iterations (linear solves);
 * *ok = 1 when converged.  fresh_first = 1 follows the batched CPU path
 * _newton_step_batched! (src/batched.jl:389-402): a new pivoting
 * factorisation (klu) at the first iteration of every Newton call and
 * klu! refactorisations after it.  fresh_first = 0 follows integrate! /
 * newton_step! (src/numerics.jl:138-167): the pivot sequence of the
 * factorisation made at z0 is reused for the whole run, with a fresh
 * factorisation only when a pivot is exactly zero. */
static int newton_mono(newton_ws *W, double *z, const double *zold, const double *u0, const double *p,
                       const faults_t *F, double dt, double tol, int itermax, int *ok, int fresh_first) {
    sym_t *S = W->S;
    int n = S->nsys;
    memcpy(W->zb, z, sizeof(double) * n);
    *ok = 0;
    int it;
    for (it = 0; it < itermax; it++) {
        residual_be(S->P, W->zb, zold, u0, p, F, dt, W->f);
        double nf = inf_norm(W->f, n);
        if (nf < tol) { *ok = 1; break; }
        if (!isfinite(nf)) break;
        assemble_J(S, W->zb, u0, p, F, dt, &W->t);
        if (factor_or_refactor(W, &S->J, fresh_first && it == 0) != 0) break;
        memcpy(W->dx, W->f, sizeof(double) * n);
        splu_solve(&W->LU, W->dx, W->work);
        for (int i = 0; i < n; i++) W->zb[i] -= W->dx[i];
    }
    memcpy(z, W->zb, sizeof(double) * n);
    return it;
}

/* One Schur reduction at the iterate zb (src/schur.jl:285-360): the BE
 * residual into W->f, J, the reduced matrix S = J_red - sum_k C_k A_k^-1 B_k
 * into S->S.val and the reduced right-hand side -(f_red - sum_k C_k A_k^-1
 * f_wk) into W->rhs.  Returns the residual's infinity norm. */
static double schur_reduce(newton_ws *W, const double *zold, const double *u0, const double *p, const faults_t *F,
                           double dt) {
    sym_t *S = W->S;
    const gp_problem *P = S->P;
    int n = S->nsys, nr = S->n_red;
    residual_be(P, W->zb, zold, u0, p, F, dt, W->f);
    double nf = inf_norm(W->f, n);
    assemble_J(S, W->zb, u0, p, F, dt, &W->t);
    /* S := J restricted to the reduced set */
    memset(S->S.val, 0, sizeof(double) * S->S.nnz);
    for (int lj = 0; lj < nr; lj++) {
        int gj = S->red_idx[lj];
        for (int q = S->J.colptr[gj]; q < S->J.colptr[gj + 1]; q++) {
            int li = S->g2r[S->J.rowind[q]];
            if (li >= 0) S->S.val[csc_find(&S->S, li, lj)] = S->J.val[q];
        }
    }
    for (int i = 0; i < nr; i++) W->rhs[i] = W->f[S->red_idx[i]];
    /* per non-trivial cluster */
    for (int ci = 0; ci < S->nt; ci++) {
        int c = S->nt_cl[ci];
        int ws = P->cl_w_start[c], wk = P->cl_w_size[c], bus = P->cl_bus[c];
        int vr_g = S->net + 2 * bus, vr_l = S->g2r[vr_g], vi_l = S->g2r[vr_g + 1];
        double *A = W->Ak, *B = W->Bk, *C = W->Ck;
        memset(A, 0, sizeof(double) * wk * wk);
        memset(B, 0, sizeof(double) * wk * 2);
        memset(C, 0, sizeof(double) * wk * 2);
        for (int j = 0; j < wk; j++)
            for (int q = S->J.colptr[ws + j]; q < S->J.colptr[ws + j + 1]; q++) {
                int r = S->J.rowind[q];
                if (r >= ws && r < ws + wk) A[(r - ws) + j * wk] = S->J.val[q];
                else if (r == vr_g) C[0 + 2 * j] = S->J.val[q];
                else if (r == vr_g + 1) C[1 + 2 * j] = S->J.val[q];
            }
        for (int b2 = 0; b2 < 2; b2++)
            for (int q = S->J.colptr[vr_g + b2]; q < S->J.colptr[vr_g + b2 + 1]; q++) {
                int r = S->J.rowind[q];
                if (r >= ws && r < ws + wk) B[(r - ws) + b2 * wk] = S->J.val[q];
            }
        dense_lu(A, W->ipiv, wk);
        double D[4];
        for (int b2 = 0; b2 < 2; b2++) {
            for (int i = 0; i < wk; i++) W->tmp[i] = B[i + b2 * wk];
            dense_solve(A, W->ipiv, W->tmp, wk);
            double d1 = 0, d2 = 0;
            for (int i = 0; i < wk; i++) { d1 += C[0 + 2 * i] * W->tmp[i]; d2 += C[1 + 2 * i] * W->tmp[i]; }
            D[0 + 2 * b2] = d1;
            D[1 + 2 * b2] = d2;
        }
        S->S.val[csc_find(&S->S, vr_l, vr_l)] -= D[0];
        S->S.val[csc_find(&S->S, vi_l, vr_l)] -= D[1];
        S->S.val[csc_find(&S->S, vr_l, vi_l)] -= D[2];
        S->S.val[csc_find(&S->S, vi_l, vi_l)] -= D[3];
        for (int i = 0; i < wk; i++) W->tmp[i] = W->f[ws + i];
        dense_solve(A, W->ipiv, W->tmp, wk);
        for (int i = 0; i < wk; i++) {
            W->rhs[vr_l] -= C[0 + 2 * i] * W->tmp[i];
            W->rhs[vi_l] -= C[1 + 2 * i] * W->tmp[i];
        }
    }
    for (int i = 0; i < nr; i++) W->rhs[i] = -W->rhs[i];
    return nf;
}

/* Back-substitution of the cluster rows from the reduced solution in
 * W->rhs, then zb += dz (src/schur.jl:380-420). */
static void schur_backsub(newton_ws *W) {
    sym_t *S = W->S;
    const gp_problem *P = S->P;
    int n = S->nsys, nr = S->n_red;
    for (int i = 0; i < nr; i++) W->dz[S->red_idx[i]] = W->rhs[i];
    /* recompute each cluster's factor (values are kept only for the
     * current cluster in this restatement) */
    for (int ci = 0; ci < S->nt; ci++) {
        int c = S->nt_cl[ci];
        int ws = P->cl_w_start[c], wk = P->cl_w_size[c], bus = P->cl_bus[c];
        int vr_g = S->net + 2 * bus;
        double *A = W->Ak, *B = W->Bk;
        memset(A, 0, sizeof(double) * wk * wk);
        memset(B, 0, sizeof(double) * wk * 2);
        for (int j = 0; j < wk; j++)
            for (int q = S->J.colptr[ws + j]; q < S->J.colptr[ws + j + 1]; q++) {
                int r = S->J.rowind[q];
                if (r >= ws && r < ws + wk) A[(r - ws) + j * wk] = S->J.val[q];
            }
        for (int b2 = 0; b2 < 2; b2++)
            for (int q = S->J.colptr[vr_g + b2]; q < S->J.colptr[vr_g + b2 + 1]; q++) {
                int r = S->J.rowind[q];
                if (r >= ws && r < ws + wk) B[(r - ws) + b2 * wk] = S->J.val[q];
            }
        dense_lu(A, W->ipiv, wk);
        double dv1 = W->dz[vr_g], dv2 = W->dz[vr_g + 1];
        for (int i = 0; i < wk; i++) W->tmp[i] = W->f[ws + i] + B[i] * dv1 + B[i + wk] * dv2;
        dense_solve(A, W->ipiv, W->tmp, wk);
        for (int i = 0; i < wk; i++) W->dz[ws + i] = -W->tmp[i];
    }
    for (int i = 0; i < n; i++) W->zb[i] += W->dz[i];
}

/* newton_step_schur! (src/schur.jl:253-426). */
static int newton_schur(newton_ws *W, double *z, const double *zold, const double *u0, const double *p,
                        const faults_t *F, double dt, double tol, int itermax, int *ok) {
    sym_t *S = W->S;
    int n = S->nsys;
    memcpy(W->zb, z, sizeof(double) * n);
    *ok = 0;
    int it;
    for (it = 0; it < itermax; it++) {
        double nf = schur_reduce(W, zold, u0, p, F, dt);
        if (nf < tol) { *ok = 1; break; }
        if (!isfinite(nf)) break;
        if (factor_or_refactor(W, &S->S, it == 0) != 0) break;
        splu_solve(&W->LU, W->rhs, W->work);
        schur_backsub(W);
    }
    memcpy(z, W->zb, sizeof(double) * n);
    return it;
}

/* Shared-factor Newton step (_newton_step_shared_multi_gpu!,
 * ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2523-2627): the cluster blocks,
 * the residual and the reduced right-hand side at the current iterate, the
 * reduced solve with the frozen matrix P of scenario 0 at the initial
 * state, or with P plus the scenario's fault shunt while the fault is on
 * (the matrix the reference's Woodbury correction inverts, factored here
 * directly: Pf). */
static int newton_frozen(newton_ws *W, double *z, const double *zold, const double *u0, const double *p,
                         const faults_t *F, double dt, double tol, int itermax, int *ok, splu_t *LP, splu_t *LPf) {
    sym_t *S = W->S;
    int n = S->nsys;
    int fault_on = 0;
    for (int e = 0; e < F->n; e++) fault_on |= F->on[e];
    memcpy(W->zb, z, sizeof(double) * n);
    *ok = 0;
    int it;
    for (it = 0; it < itermax; it++) {
        double nf = schur_reduce(W, zold, u0, p, F, dt);
        if (nf < tol) { *ok = 1; break; }
        if (!isfinite(nf)) break;
        splu_solve(fault_on ? LPf : LP, W->rhs, W->work);
        schur_backsub(W);
    }
    memcpy(z, W->zb, sizeof(double) * n);
    return it;
}

static void ws_init(newton_ws *W, sym_t *S) {
    memset(W, 0, sizeof(*W));
    W->S = S;
    int n = S->nsys;
    W->f = (double *)malloc(sizeof(double) * n);
    W->dx = (double *)malloc(sizeof(double) * n);
    W->work = (double *)malloc(sizeof(double) * n);
    W->zb = (double *)malloc(sizeof(double) * n);
    W->dz = (double *)calloc(n, sizeof(double));
    W->rhs = (double *)malloc(sizeof(double) * (S->n_red + 1));
    int wm = 1;
    for (int c = 0; c < S->P->n_clusters; c++)
        if (S->P->cl_w_size[c] > wm) wm = S->P->cl_w_size[c];
    W->wmax = wm;
    W->Ak = (double *)malloc(sizeof(double) * wm * wm);
    W->Bk = (double *)malloc(sizeof(double) * wm * 2);
    W->Ck = (double *)malloc(sizeof(double) * wm * 2);
    W->tmp = (double *)malloc(sizeof(double) * wm);
    W->ipiv = (int *)malloc(sizeof(int) * wm);
}

static void ws_free(newton_ws *W) {
    if (W->have_lu) splu_free(&W->LU);
    trip_free(&W->t);
    free(W->f); free(W->dx); free(W->work); free(W->zb); free(W->dz); free(W->rhs);
    free(W->Ak); free(W->Bk); free(W->Ck); free(W->tmp); free(W->ipiv);
}

/* ------------------------------------------------------------------ */
/* integrate! for one scenario (src/dynamics.jl:502-655)               */
/* ------------------------------------------------------------------ */

static int integrate_one(const gp_problem *P0, const double *z0, const double *u0, const double *p, int nf,
                         const gp_fault *faults, int ntr, const gp_line_trip *trips, int ndc,
                         const gp_device_disconnect *dcs, double dt, int nsteps, double tol, int itermax, int solver,
                         const double *z0_s0, const double *u0_s0, const double *p_s0, double *traj, double *zfinal,
                         int *iters, long long *stats) {
    /* device disconnections: a private copy of the problem whose online
     * flags this scenario's events clear, for the rest of the run
     * (_set_device_offline!, src/GradPower.jl:672-698; every kernel skips an
     * offline device, the device kernels of src/kernels/) */
    gp_problem Pm = *P0;
    uint8_t *onl[GP_NTYPES] = {0};
    for (int e = 0; e < ndc; e++) {
        const int t = dcs[e].type, nt = P0->dev[t].n;
        if (onl[t]) continue;
        onl[t] = (uint8_t *)malloc(nt > 0 ? nt : 1);
        for (int k = 0; k < nt; k++) onl[t][k] = P0->dev[t].online ? P0->dev[t].online[k] : 1;
        Pm.dev[t].online = onl[t];
    }
    const gp_problem *P = &Pm;
    int n = n_sys_of(P);
    sym_t S;
    sym_build(&S, P, z0, u0, p, nf, faults);
    newton_ws W;
    ws_init(&W, &S);
    double *z = (double *)malloc(sizeof(double) * n);
    double *zold = (double *)malloc(sizeof(double) * n);
    memcpy(z, z0, sizeof(double) * n);
    if (traj) memcpy(traj, z, sizeof(double) * n);
    uint8_t *on = (uint8_t *)calloc(nf > 0 ? nf : 1, 1);
    uint8_t *tr_on = (uint8_t *)calloc(ntr > 0 ? ntr : 1, 1);
    faults_t F = {nf, faults, on, ntr, trips, tr_on};
    int status = 0;
    if (solver == 2) {
        /* integrate! factors J at z0 once before the loop (src/dynamics.jl:572-580) */
        assemble_J(&S, z, u0, p, &F, dt, &W.t);
        if (factor_or_refactor(&W, &S.J, 1) != 0) status = 2;
    }
    /* shared-factor path: P = S of scenario 0 at its initial state, no
     * fault, this call's dt (_factor_shared_P_gpu!, ext/...:2149-2172); Pf =
     * P with the scenario's fault shunt on its bus diagonal */
    splu_t LP, LPf;
    int have_p = 0;
    if (solver == 3) {
        uint8_t none = 0;
        faults_t F0 = {0, faults, &none};
        memcpy(W.zb, z0_s0, sizeof(double) * n);
        schur_reduce(&W, z0_s0, u0_s0, p_s0, &F0, dt);
        int *q = min_degree_order(S.S.n, S.S.colptr, S.S.rowind);
        int *q2 = (int *)malloc(sizeof(int) * (S.S.n > 0 ? S.S.n : 1));
        memcpy(q2, q, sizeof(int) * S.S.n);
        splu_init(&LP, S.S.n, q);
        splu_init(&LPf, S.S.n, q2);
        have_p = 1;
        if (splu_factor(&LP, &S.S, 1e-3) != 0) status = 2;
        if (nf > 0) {
            const int vr_l = S.g2r[S.net + 2 * faults[0].bus], vi_l = S.g2r[S.net + 2 * faults[0].bus + 1];
            S.S.val[csc_find(&S.S, vr_l, vr_l)] -= 1.0 / faults[0].rfault;
            S.S.val[csc_find(&S.S, vi_l, vi_l)] -= 1.0 / faults[0].rfault;
        }
        if (splu_factor(&LPf, &S.S, 1e-3) != 0) status = 2;
    }
    for (int k = 1; k <= nsteps && status != 2; k++) {
        int ok;
        memcpy(zold, z, sizeof(double) * n);
        int it = solver == 3   ? newton_frozen(&W, z, zold, u0, p, &F, dt, tol, itermax, &ok, &LP, &LPf)
                 : solver != 1 ? newton_mono(&W, z, zold, u0, p, &F, dt, tol, itermax, &ok, solver == 0)
                               : newton_schur(&W, z, zold, u0, p, &F, dt, tol, itermax, &ok);
        if (!ok) status = isfinite(inf_norm(z, n)) ? 1 : 2;
        if (iters) { iters[2 * (k - 1)] = it; iters[2 * (k - 1) + 1] = 0; }
        if (traj) memcpy(traj + (size_t)k * n, z, sizeof(double) * n);
        int any = 0;
        for (int e = 0; e < nf; e++) {
            if (faults[e].on_step == k) { on[e] = 1; any = 1; }
            if (faults[e].off_step == k) { on[e] = 0; any = 1; }
        }
        for (int e = 0; e < ntr; e++) {
            if (trips[e].on_step == k) { tr_on[e] = 1; any = 1; }
            if (trips[e].off_step == k) { tr_on[e] = 0; any = 1; }
        }
        for (int e = 0; e < ndc; e++)
            if (dcs[e].on_step == k) { onl[dcs[e].type][dcs[e].index] = 0; any = 1; }
        if (any) {
            memcpy(zold, z, sizeof(double) * n);
            it = solver == 3   ? newton_frozen(&W, z, zold, u0, p, &F, 0.0, tol, itermax, &ok, &LP, &LPf)
                 : solver != 1 ? newton_mono(&W, z, zold, u0, p, &F, 0.0, tol, itermax, &ok, solver == 0)
                               : newton_schur(&W, z, zold, u0, p, &F, 0.0, tol, itermax, &ok);
            if (!ok) status = isfinite(inf_norm(z, n)) ? 1 : 2;
            if (iters) iters[2 * (k - 1) + 1] = it;
        }
    }
    if (zfinal) memcpy(zfinal, z, sizeof(double) * n);
    if (stats) {
        stats[0] = W.factor_count;
        stats[1] = W.refactor_count;
        stats[2] = W.have_lu ? splu_nnz(&W.LU) : 0;
        stats[3] = S.J.nnz;
        stats[4] = S.S.nnz;
        stats[5] = S.n_red;
    }
    if (have_p) {
        splu_free(&LP);
        splu_free(&LPf);
    }
    free(on);
    free(tr_on);
    for (int t = 0; t < GP_NTYPES; t++) free(onl[t]);
    free(z);
    free(zold);
    ws_free(&W);
    sym_free(&S);
    return status;
}

/* ------------------------------------------------------------------ */
/* exported entry points (called through ctypes by the test harness)   */
/* ------------------------------------------------------------------ */

/* Integrate M scenarios, each as an independent run.  Faults with
 * scenario == -1 apply to every scenario.  solver: 0 monolithic sparse LU
 * with the batched path's factorisation schedule (integrate_batched!),
 * 1 Schur path (newton_step_schur!), 2 monolithic with integrate!'s
 * schedule (one pivoting factorisation at z0, refactorisations after),
 * 3 shared-factor path (integrate_gpu_shared_multi!: the reduced matrix of
 * scenario 0 at its initial state, factored once, with each scenario's
 * fault shunt; every scenario has at most one fault bus and rfault).  traj [M][nsteps+1][n_sys] or NULL; zfinal [M][n_sys]
 * or NULL; iters [M][2*nsteps] or NULL; status [M]; stats [M][6] or NULL. */
int gpo_integrate_events(const gp_problem *P, int M, const double *z0, const double *u0, const double *p, int nf,
                         const gp_fault *faults, int ntr_all, const gp_line_trip *trips_all, int ndc_all,
                         const gp_device_disconnect *dcs_all, double dt, int nsteps, double tol, int itermax,
                         int solver, int nthreads, double *traj, double *zfinal, int *iters, int *status,
                         long long *stats) {
    int n = n_sys_of(P);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int m = 0; m < M; m++) {
        int cnt = 0;
        for (int e = 0; e < nf; e++)
            if (faults[e].scenario < 0 || faults[e].scenario == m) cnt++;
        gp_fault *fm = (gp_fault *)malloc(sizeof(gp_fault) * (cnt > 0 ? cnt : 1));
        cnt = 0;
        for (int e = 0; e < nf; e++)
            if (faults[e].scenario < 0 || faults[e].scenario == m) fm[cnt++] = faults[e];
        int ct = 0;
        for (int e = 0; e < ntr_all; e++)
            if (trips_all[e].scenario < 0 || trips_all[e].scenario == m) ct++;
        gp_line_trip *tm = (gp_line_trip *)malloc(sizeof(gp_line_trip) * (ct > 0 ? ct : 1));
        ct = 0;
        for (int e = 0; e < ntr_all; e++)
            if (trips_all[e].scenario < 0 || trips_all[e].scenario == m) tm[ct++] = trips_all[e];
        int cd = 0;
        for (int e = 0; e < ndc_all; e++)
            if (dcs_all[e].scenario < 0 || dcs_all[e].scenario == m) cd++;
        gp_device_disconnect *dm = (gp_device_disconnect *)malloc(sizeof(gp_device_disconnect) * (cd > 0 ? cd : 1));
        cd = 0;
        for (int e = 0; e < ndc_all; e++)
            if (dcs_all[e].scenario < 0 || dcs_all[e].scenario == m) dm[cd++] = dcs_all[e];
        status[m] = integrate_one(P, z0 + (size_t)m * n, u0 + (size_t)m * P->n_ctrl, p + (size_t)m * P->n_par, cnt,
                                  fm, ct, tm, cd, dm, dt, nsteps, tol, itermax, solver, z0, u0, p,
                                  traj ? traj + (size_t)m * (nsteps + 1) * n : NULL,
                                  zfinal ? zfinal + (size_t)m * n : NULL,
                                  iters ? iters + (size_t)m * 2 * nsteps : NULL,
                                  stats ? stats + (size_t)m * 6 : NULL);
        free(fm);
        free(tm);
        free(dm);
    }
    (void)nthreads;
    return 0;
}

int gpo_integrate_trips(const gp_problem *P, int M, const double *z0, const double *u0, const double *p, int nf,
                        const gp_fault *faults, int ntr_all, const gp_line_trip *trips_all, double dt, int nsteps,
                        double tol, int itermax, int solver, int nthreads, double *traj, double *zfinal,
                        int *iters, int *status, long long *stats) {
    return gpo_integrate_events(P, M, z0, u0, p, nf, faults, ntr_all, trips_all, 0, NULL, dt, nsteps, tol, itermax,
                                solver, nthreads, traj, zfinal, iters, status, stats);
}

int gpo_integrate(const gp_problem *P, int M, const double *z0, const double *u0, const double *p, int nf,
                  const gp_fault *faults, double dt, int nsteps, double tol, int itermax, int solver,
                  int nthreads, double *traj, double *zfinal, int *iters, int *status, long long *stats) {
    return gpo_integrate_trips(P, M, z0, u0, p, nf, faults, 0, NULL, dt, nsteps, tol, itermax, solver, nthreads,
                               traj, zfinal, iters, status, stats);
}

/* Backward-Euler residual of one scenario with the flagged faults on. */
int gpo_residual(const gp_problem *P, const double *z, const double *zold, const double *u0, const double *p,
                 int nf, const gp_fault *faults, const uint8_t *fault_on, double dt, double *f) {
    faults_t F = {nf, faults, fault_on};
    residual_be(P, z, zold, u0, p, &F, dt, f);
    return 0;
}

/* Backward-Euler Jacobian of one scenario as a dense row-major matrix
 * (small systems only; used by the finite-difference tests). */
int gpo_jacobian_dense(const gp_problem *P, const double *z, const double *u0, const double *p, int nf,
                       const gp_fault *faults, const uint8_t *fault_on, double dt, double *Jd) {
    int n = n_sys_of(P), nda = P->n_diff + P->n_alg;
    faults_t F = {nf, faults, fault_on};
    trip_t t = {0};
    jacobian_rhs(P, z, u0, p, &F, &t);
    memset(Jd, 0, sizeof(double) * (size_t)n * n);
    for (int k = 0; k < t.n; k++) Jd[(size_t)t.r[k] * n + t.c[k]] += t.v[k];
    for (int i = 0; i < nda; i++)
        if (P->is_diff[i]) {
            for (int j = 0; j < n; j++) Jd[(size_t)i * n + j] *= -dt;
            Jd[(size_t)i * n + i] += 1.0;
        }
    trip_free(&t);
    return 0;
}

/* The residual and the dense Jacobian with line trips: trips [ntr] of this
 * scenario, trip_on [ntr] which of them are tripped. */
int gpo_residual_trips(const gp_problem *P, const double *z, const double *zold, const double *u0, const double *p,
                       int ntr, const gp_line_trip *trips, const uint8_t *trip_on, double dt, double *f) {
    faults_t F = {0, NULL, NULL, ntr, trips, trip_on};
    residual_be(P, z, zold, u0, p, &F, dt, f);
    return 0;
}

int gpo_jacobian_dense_trips(const gp_problem *P, const double *z, const double *u0, const double *p, int ntr,
                             const gp_line_trip *trips, const uint8_t *trip_on, double dt, double *Jd) {
    int n = n_sys_of(P), nda = P->n_diff + P->n_alg;
    faults_t F = {0, NULL, NULL, ntr, trips, trip_on};
    trip_t t = {0};
    jacobian_rhs(P, z, u0, p, &F, &t);
    memset(Jd, 0, sizeof(double) * (size_t)n * n);
    for (int k = 0; k < t.n; k++) Jd[(size_t)t.r[k] * n + t.c[k]] += t.v[k];
    for (int i = 0; i < nda; i++)
        if (P->is_diff[i]) {
            for (int j = 0; j < n; j++) Jd[(size_t)i * n + j] *= -dt;
            Jd[(size_t)i * n + i] += 1.0;
        }
    trip_free(&t);
    return 0;
}

int gpo_version(void) { return GP_ABI_VERSION; }
