// Device-model equations of one generator cluster, shared by the GPU
// cluster kernel and by the host (pattern extraction, self-test).
//
// Each *_eval writes the raw right-hand side f (before the backward-Euler
// scaling) and the Jacobian entries of its rows through a Sink:
//   sink.put(r, c, v)    d f_r / d z_c          (r, c absolute z indices)
//   sink.putv(r, k, v)   d f_r / d v_bus[k]     (k = 0 vr, 1 vi)
//   sink.putf(r, v)      f_r
// Equations: src/kernels/genrou.jl:48-141 and 407-559, ieesgo.jl:133-224,
// tgov1.jl:73-146, sexs.jl:74-156, esdc1a.jl:97-196, ieeest.jl:207-359
// (GradPower.jl).
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define GP_HD __host__ __device__ __forceinline__
#else
#define GP_HD inline
#endif

namespace gp {

constexpr double kTwoPi60 = 2.0 * 3.14159265358979323846 * 60.0;

// Pointers of one device row of a struct-of-arrays table.
struct DevRef {
    int dp, ap, cp, pp, bus, link0, link1;
};

GP_HD void sat_coef(double s1, double s2, double &sa, double &sb) {
    sa = 0.0;
    sb = 0.0;
    if (s1 <= 0.0 || s2 <= 0.0) return;
    const double e1 = 1.0, e2 = 1.2;
    double a = sqrt(s1 * e1 / (s2 * e2));
    if (a == 1.0) return;
    sa = e2 - (e1 - e2) / (a - 1.0);
    sb = s2 * e2 * (a - 1.0) * (a - 1.0) / ((e1 - e2) * (e1 - e2));
}

// GENROU.  C receives the network-row couplings d f_vr/d{delta,i_q,i_d},
// d f_vi/d{delta,i_q,i_d}; I the injected current (vr, vi rows).
template <class Sink>
GP_HD void genrou_eval(const DevRef &d, int net, const double *z, const double *u0, const double *p, Sink &M,
                       double *C, double *I) {
    const int dp = d.dp, ap = d.ap, cp = d.cp, pp = d.pp;
    const double x_d = p[pp], x_q = p[pp + 1], x_dp = p[pp + 2], x_qp = p[pp + 3], x_ddp = p[pp + 4],
                 xl = p[pp + 5], H = p[pp + 6], D = p[pp + 7], T_d0p = p[pp + 8], T_q0p = p[pp + 9],
                 T_d0dp = p[pp + 10], T_q0dp = p[pp + 11], S1 = p[pp + 12], S2 = p[pp + 13];
    const double x_qdp = x_ddp;
    const double e_qp = z[dp], e_dp = z[dp + 1], phi_1d = z[dp + 2], phi_2q = z[dp + 3], w = z[dp + 4],
                 delta = z[dp + 5];
    const double v_q = z[ap], v_d = z[ap + 1], i_q = z[ap + 2], i_d = z[ap + 3];
    const int vr_idx = net + 2 * d.bus;
    const double vr = z[vr_idx], vi = z[vr_idx + 1];
    const int pm_idx = d.link0, efd_idx = d.link1;
    const double e_fd = efd_idx >= 0 ? z[efd_idx] : u0[cp];
    const double p_m = pm_idx >= 0 ? z[pm_idx] : u0[cp + 1];
    const double dpl = x_dp - xl, qpl = x_qp - xl;
    const double psi_de = (x_ddp - xl) / dpl * e_qp + (x_dp - x_ddp) / dpl * phi_1d;
    const double psi_qe = -(x_ddp - xl) / qpl * e_dp + (x_qp - x_ddp) / qpl * phi_2q;
    double sa, sb;
    sat_coef(S1, S2, sa, sb);
    const double psi2 = sqrt(psi_de * psi_de + psi_qe * psi_qe);
    const bool sat_on = !(sb == 0.0 || psi2 <= sa || psi2 == 0.0);
    const double Se = sat_on ? sb * (psi2 - sa) * (psi2 - sa) / psi2 : 0.0;
    const double sd = sin(delta), cd = cos(delta);
    M.putf(dp, (-e_qp + e_fd - (i_d - (-x_ddp + x_dp) * (-e_qp + i_d * dpl + phi_1d) / (dpl * dpl)) * (x_d - x_dp) -
                Se * psi_de) / T_d0p);
    M.putf(dp + 1, (-e_dp + (i_q - (-x_qdp + x_qp) * (e_dp + i_q * qpl + phi_2q) / (qpl * qpl)) * (x_q - x_qp)) / T_q0p);
    M.putf(dp + 2, (e_qp - i_d * dpl - phi_1d) / T_d0dp);
    M.putf(dp + 3, (-e_dp - i_q * qpl - phi_2q) / T_q0dp);
    M.putf(dp + 4, (p_m - D * w - psi_de * i_q + psi_qe * i_d) / (2.0 * H));
    M.putf(dp + 5, kTwoPi60 * w);
    M.putf(ap, i_d - ((x_ddp - xl) / dpl * e_qp + (x_dp - x_ddp) / dpl * phi_1d - v_q) / x_ddp);
    M.putf(ap + 1, i_q - (-(x_qdp - xl) / qpl * e_dp + (x_qp - x_qdp) / qpl * phi_2q + v_d) / x_qdp);
    M.putf(ap + 2, v_d - (vr * sd - vi * cd));
    M.putf(ap + 3, v_q - (vr * cd + vi * sd));
    double dSe = 0.0;
    if (sat_on) {
        double g = psi2 - sa;
        dSe = sb * (2.0 * g * psi2 - g * g) / (psi2 * psi2);
    }
    const double dpd = psi2 == 0.0 ? 0.0 : psi_de / psi2;
    const double dpq = psi2 == 0.0 ? 0.0 : psi_qe / psi2;
    const double a_eqp = (x_ddp - xl) / dpl, a_phi1d = (x_dp - x_ddp) / dpl;
    const double b_edp = -(x_ddp - xl) / qpl, b_phi2q = (x_qp - x_ddp) / qpl;
    const double dT_dde = -(dSe * dpd * psi_de + Se);
    const double dT_dqe = -(dSe * dpq * psi_de);
    const int c_eqp = dp, c_edp = dp + 1, c_phi1d = dp + 2, c_phi2q = dp + 3, c_w = dp + 4, c_delta = dp + 5;
    const int c_vq = ap, c_vd = ap + 1, c_iq = ap + 2, c_id = ap + 3;
    M.put(dp, c_eqp, (-(x_d - x_dp) * (-x_ddp + x_dp) / (dpl * dpl) - 1) / T_d0p + dT_dde * a_eqp / T_d0p);
    M.put(dp, c_phi1d, (x_d - x_dp) * (-x_ddp + x_dp) / (dpl * dpl) / T_d0p + dT_dde * a_phi1d / T_d0p);
    M.put(dp, c_id, -(x_d - x_dp) * (-(-x_ddp + x_dp) / dpl + 1) / T_d0p);
    M.put(dp, c_edp, dT_dqe * b_edp / T_d0p);
    M.put(dp, c_phi2q, dT_dqe * b_phi2q / T_d0p);
    if (efd_idx >= 0) M.put(dp, efd_idx, 1.0 / T_d0p);
    M.put(dp + 1, c_edp, (-(x_q - x_qp) * (-x_qdp + x_qp) / (qpl * qpl) - 1) / T_q0p);
    M.put(dp + 1, c_phi2q, -(x_q - x_qp) * (-x_qdp + x_qp) / (qpl * qpl) / T_q0p);
    M.put(dp + 1, c_iq, (x_q - x_qp) * (-(-x_qdp + x_qp) / qpl + 1) / T_q0p);
    M.put(dp + 2, c_eqp, 1.0 / T_d0dp);
    M.put(dp + 2, c_phi1d, -1.0 / T_d0dp);
    M.put(dp + 2, c_id, (-x_dp + xl) / T_d0dp);
    M.put(dp + 3, c_edp, -1.0 / T_q0dp);
    M.put(dp + 3, c_phi2q, -1.0 / T_q0dp);
    M.put(dp + 3, c_iq, (-x_qp + xl) / T_q0dp);
    M.put(dp + 4, c_eqp, -0.5 * i_q * (x_ddp - xl) / (H * dpl));
    M.put(dp + 4, c_edp, 0.5 * i_d * (-x_ddp + xl) / (H * qpl));
    M.put(dp + 4, c_phi1d, -0.5 * i_q * (-x_ddp + x_dp) / (H * dpl));
    M.put(dp + 4, c_phi2q, 0.5 * i_d * (-x_ddp + x_qp) / (H * qpl));
    M.put(dp + 4, c_w, -0.5 * D / H);
    if (pm_idx >= 0) M.put(dp + 4, pm_idx, 0.5 / H);
    M.put(dp + 4, c_iq, 0.5 * (-e_qp * (x_ddp - xl) / dpl - phi_1d * (-x_ddp + x_dp) / dpl) / H);
    M.put(dp + 4, c_id, 0.5 * (e_dp * (-x_ddp + xl) / qpl + phi_2q * (-x_ddp + x_qp) / qpl) / H);
    M.put(dp + 5, c_w, kTwoPi60);
    M.put(ap, c_eqp, -(x_ddp - xl) / (x_ddp * dpl));
    M.put(ap, c_phi1d, -(-x_ddp + x_dp) / (x_ddp * dpl));
    M.put(ap, c_vq, 1.0 / x_ddp);
    M.put(ap, c_id, 1.0);
    M.put(ap + 1, c_edp, -(-x_qdp + xl) / (x_qdp * qpl));
    M.put(ap + 1, c_phi2q, -(-x_qdp + x_qp) / (x_qdp * qpl));
    M.put(ap + 1, c_vd, -1.0 / x_qdp);
    M.put(ap + 1, c_iq, 1.0);
    M.put(ap + 2, c_delta, -vr * cd - vi * sd);
    M.put(ap + 2, c_vd, 1.0);
    M.putv(ap + 2, 0, -sd);
    M.putv(ap + 2, 1, cd);
    M.put(ap + 3, c_delta, vr * sd - vi * cd);
    M.put(ap + 3, c_vq, 1.0);
    M.putv(ap + 3, 0, -cd);
    M.putv(ap + 3, 1, -sd);
    C[0] = i_d * cd - i_q * sd;
    C[1] = cd;
    C[2] = sd;
    C[3] = i_d * sd + i_q * cd;
    C[4] = sd;
    C[5] = -cd;
    I[0] = sd * i_d + cd * i_q;
    I[1] = -cd * i_d + sd * i_q;
}

template <class Sink>
GP_HD void ieesgo_eval(const DevRef &d, const double *z, const double *p, Sink &M) {
    const int dp = d.dp, ap = d.ap, pp = d.pp, wi = d.link0;
    const double T1 = p[pp], T2 = p[pp + 1], T3 = p[pp + 2], T4 = p[pp + 3], T5 = p[pp + 4], T6 = p[pp + 5];
    const double K1 = p[pp + 6], K2 = p[pp + 7], K3 = p[pp + 8], pref = p[pp + 11];
    const double PF0 = z[dp], PLL = z[dp + 1], TP1 = z[dp + 2], TP2 = z[dp + 3], TP3 = z[dp + 4], p_m = z[ap];
    const double w = wi < 0 ? 0.0 : z[wi];
    M.putf(dp, (1.0 / T1) * (K1 * w - PF0));
    M.putf(dp + 1, (1.0 / T3) * ((1.0 - (T2 / T3)) * PF0 - PLL));
    const double SatP = pref - (T2 / T3) * PF0 - PLL;
    M.putf(dp + 2, (1.0 / T4) * (SatP - TP1));
    M.putf(dp + 3, (1.0 / T5) * (K2 * TP1 - TP2));
    M.putf(dp + 4, (1.0 / T6) * (K3 * TP2 - TP3));
    M.putf(ap, TP1 * (1.0 - K2) + TP2 * (1.0 - K3) + TP3 - p_m);
    M.put(dp, dp, -1.0 / T1);
    if (wi >= 0) M.put(dp, wi, K1 / T1);
    M.put(dp + 1, dp, (1.0 - T2 / T3) / T3);
    M.put(dp + 1, dp + 1, -1.0 / T3);
    M.put(dp + 2, dp, -T2 / (T3 * T4));
    M.put(dp + 2, dp + 1, -1.0 / T4);
    M.put(dp + 2, dp + 2, -1.0 / T4);
    M.put(dp + 3, dp + 2, K2 / T5);
    M.put(dp + 3, dp + 3, -1.0 / T5);
    M.put(dp + 4, dp + 3, K3 / T6);
    M.put(dp + 4, dp + 4, -1.0 / T6);
    M.put(ap, dp + 2, 1.0 - K2);
    M.put(ap, dp + 3, 1.0 - K3);
    M.put(ap, dp + 4, 1.0);
    M.put(ap, ap, -1.0);
}

template <class Sink>
GP_HD void tgov1_eval(const DevRef &d, const double *z, const double *p, Sink &M) {
    const int dp = d.dp, ap = d.ap, pp = d.pp, wi = d.link0;
    const double R = p[pp], T1 = p[pp + 1], T2 = p[pp + 4], T3 = p[pp + 5], DT = p[pp + 6], pref = p[pp + 7];
    const double x1 = z[dp], x2 = z[dp + 1], p_m = z[ap];
    const double w = wi < 0 ? 0.0 : z[wi];
    const double r23 = T2 / T3;
    M.putf(dp, (-x1 + (1.0 - r23) * x2) / T3);
    M.putf(dp + 1, ((pref - w) / R - x2) / T1);
    M.putf(ap, x1 + r23 * x2 - DT * w - p_m);
    M.put(dp, dp, -1.0 / T3);
    M.put(dp, dp + 1, (1.0 - r23) / T3);
    M.put(dp + 1, dp + 1, -1.0 / T1);
    if (wi >= 0) M.put(dp + 1, wi, -1.0 / (R * T1));
    M.put(ap, dp, 1.0);
    M.put(ap, dp + 1, r23);
    if (wi >= 0) M.put(ap, wi, -DT);
    M.put(ap, ap, -1.0);
}

template <class Sink>
GP_HD void sexs_eval(const DevRef &d, int net, const double *z, const double *p, Sink &M) {
    const int dp = d.dp, pp = d.pp, vsi = d.link0;
    const int vr_idx = net + 2 * d.bus;
    const double TA_TB = p[pp], TB = p[pp + 1], K = p[pp + 2], TE = p[pp + 3], vref = p[pp + 6];
    const double x1 = z[dp], e_fd = z[dp + 1], vr = z[vr_idx], vi = z[vr_idx + 1];
    double vm = sqrt(vr * vr + vi * vi);
    vm = vm == 0.0 ? 1e-12 : vm;
    const double vs = vsi >= 0 ? z[vsi] : 0.0;
    const double err = vref - vm + vs;
    M.putf(dp, (-x1 + (1.0 - TA_TB) * err) / TB);
    M.putf(dp + 1, (-e_fd + K * (x1 + TA_TB * err)) / TE);
    const double dvr = vr / vm, dvi = vi / vm;
    M.put(dp, dp, -1.0 / TB);
    M.putv(dp, 0, -(1.0 - TA_TB) * dvr / TB);
    M.putv(dp, 1, -(1.0 - TA_TB) * dvi / TB);
    if (vsi >= 0) M.put(dp, vsi, (1.0 - TA_TB) / TB);
    M.put(dp + 1, dp, K / TE);
    M.put(dp + 1, dp + 1, -1.0 / TE);
    M.putv(dp + 1, 0, -K * TA_TB * dvr / TE);
    M.putv(dp + 1, 1, -K * TA_TB * dvi / TE);
    if (vsi >= 0) M.put(dp + 1, vsi, K * TA_TB / TE);
}

template <class Sink>
GP_HD void esdc1a_eval(const DevRef &d, int net, const double *z, const double *p, Sink &M) {
    const int dp = d.dp, pp = d.pp, vsi = d.link0;
    const int vr_idx = net + 2 * d.bus;
    const double Ka = p[pp], Ta = p[pp + 1], Kf = p[pp + 2], Tf = p[pp + 3], Ke = p[pp + 4], Te = p[pp + 5];
    const double sat_a = p[pp + 7], sat_b = p[pp + 8], vref = p[pp + 9];
    const double vr1 = z[dp], vr2 = z[dp + 1], e_fd = z[dp + 2], vr = z[vr_idx], vi = z[vr_idx + 1];
    double vm = sqrt(vr * vr + vi * vi);
    vm = vm == 0.0 ? 1e-12 : vm;
    const double vs = vsi >= 0 ? z[vsi] : 0.0;
    const bool son = !(sat_b == 0.0 || e_fd <= sat_a);
    const double sat = son ? sat_b * (e_fd - sat_a) * (e_fd - sat_a) : 0.0;
    M.putf(dp, (Ka * (vref - vm + vs - vr2 - (Kf / Tf) * e_fd) - vr1) / Ta);
    M.putf(dp + 1, -((Kf / Tf) * e_fd + vr2) / Tf);
    M.putf(dp + 2, (vr1 - Ke * e_fd - sat) / Te);
    const double dvr = vr / vm, dvi = vi / vm;
    const double dsat = son ? 2.0 * sat_b * (e_fd - sat_a) : 0.0;
    M.put(dp, dp, -1.0 / Ta);
    M.put(dp, dp + 1, -Ka / Ta);
    M.put(dp, dp + 2, -Ka * Kf / (Ta * Tf));
    M.putv(dp, 0, -Ka * dvr / Ta);
    M.putv(dp, 1, -Ka * dvi / Ta);
    if (vsi >= 0) M.put(dp, vsi, Ka / Ta);
    M.put(dp + 1, dp + 1, -1.0 / Tf);
    M.put(dp + 1, dp + 2, -Kf / (Tf * Tf));
    M.put(dp + 2, dp, 1.0 / Te);
    M.put(dp + 2, dp + 2, -(Ke + dsat) / Te);
}

template <class Sink>
GP_HD void ieeest_eval(const DevRef &d, const double *z, const double *p, Sink &M) {
    const int dp = d.dp, ap = d.ap, pp = d.pp, wi = d.link0;
    const double A1 = p[pp], A2 = p[pp + 1], A3 = p[pp + 2], A4 = p[pp + 3], A5 = p[pp + 4], A6 = p[pp + 5];
    const double T1 = p[pp + 6], T2 = p[pp + 7], T3 = p[pp + 8], T4 = p[pp + 9], T5 = p[pp + 10], T6 = p[pp + 11],
                 KS = p[pp + 12];
    const double s0 = z[dp], s1 = z[dp + 1], s2 = z[dp + 2], s3 = z[dp + 3], s4 = z[dp + 4], s5 = z[dp + 5],
                 s6 = z[dp + 6], vs = z[ap];
    const double sig = wi >= 0 ? z[wi] : 0.0;
    const double q = s1 - s3 - A3 * s2;
    const double y2 = s3 + A5 * s2 + (A6 / A4) * q;
    const double y3 = s4 + (T1 / T2) * (y2 - s4);
    const double y4 = s5 + (T3 / T4) * (y3 - s5);
    M.putf(dp, (sig - s1 - A1 * s0) / A2);
    M.putf(dp + 1, s0);
    M.putf(dp + 2, (s1 - s3 - A3 * s2) / A4);
    M.putf(dp + 3, s2);
    M.putf(dp + 4, (y2 - s4) / T2);
    M.putf(dp + 5, (y3 - s5) / T4);
    M.putf(dp + 6, (KS * y4 - s6) / T6);
    M.putf(ap, vs - (T5 / T6) * (KS * y4 - s6));
    const double rA = A6 / A4;
    const double d20 = rA, d21 = A5 - A3 * rA, d22 = 1.0 - rA;
    const double r12 = T1 / T2;
    const double d30 = r12 * d20, d31 = r12 * d21, d32 = r12 * d22, d33 = 1.0 - r12;
    const double r34 = T3 / T4;
    const double d40 = r34 * d30, d41 = r34 * d31, d42 = r34 * d32, d43 = r34 * d33, d44 = 1.0 - r34;
    M.put(dp, dp, -A1 / A2);
    M.put(dp, dp + 1, -1.0 / A2);
    if (wi >= 0) M.put(dp, wi, 1.0 / A2);
    M.put(dp + 1, dp, 1.0);
    M.put(dp + 2, dp + 1, 1.0 / A4);
    M.put(dp + 2, dp + 2, -A3 / A4);
    M.put(dp + 2, dp + 3, -1.0 / A4);
    M.put(dp + 3, dp + 2, 1.0);
    M.put(dp + 4, dp + 1, d20 / T2);
    M.put(dp + 4, dp + 2, d21 / T2);
    M.put(dp + 4, dp + 3, d22 / T2);
    M.put(dp + 4, dp + 4, -1.0 / T2);
    M.put(dp + 5, dp + 1, d30 / T4);
    M.put(dp + 5, dp + 2, d31 / T4);
    M.put(dp + 5, dp + 3, d32 / T4);
    M.put(dp + 5, dp + 4, d33 / T4);
    M.put(dp + 5, dp + 5, -1.0 / T4);
    M.put(dp + 6, dp + 1, KS * d40 / T6);
    M.put(dp + 6, dp + 2, KS * d41 / T6);
    M.put(dp + 6, dp + 3, KS * d42 / T6);
    M.put(dp + 6, dp + 4, KS * d43 / T6);
    M.put(dp + 6, dp + 5, KS * d44 / T6);
    M.put(dp + 6, dp + 6, -1.0 / T6);
    const double r56 = T5 / T6;
    M.put(ap, dp + 1, -r56 * KS * d40);
    M.put(ap, dp + 2, -r56 * KS * d41);
    M.put(ap, dp + 3, -r56 * KS * d42);
    M.put(ap, dp + 4, -r56 * KS * d43);
    M.put(ap, dp + 5, -r56 * KS * d44);
    M.put(ap, dp + 6, r56);
    M.put(ap, ap, 1.0);
}

// Cluster program operations (see the sparse cluster LU in gp_kernels.cu).
enum : unsigned char {
    OP_SCL = 1,   // v[d] *= -dt                       (backward-Euler row scaling)
    OP_DIAG = 2,  // v[d] += 1                         (backward-Euler diagonal)
    OP_BEF = 3,   // R2[d] = z[d] - zold[d] - dt R2[d] (backward-Euler residual, d = local row)
    OP_RCP = 4,   // v[d] = 1 / v[a]
    OP_MUL = 5,   // v[d] *= v[a]
    OP_FMS = 6,   // v[d] -= v[a] v[b]
    OP_FMS3 = 7,  // R[c][d] -= v[a] R[c][b], c = 0..2 (d, b local rows)
    OP_MUL3 = 8,  // R[c][d] *= v[a],         c = 0..2
    OP_ROW = 9,   // marker: slot d holds the residual of local row a (no arithmetic)
};

struct CluOp {
    unsigned char code, pad;
    short d, a, b;
};

}  // namespace gp
