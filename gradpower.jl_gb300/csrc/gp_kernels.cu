// Device kernels of the batched backward-Euler Newton step.
//
//  cluster_kernel  one warp per (generator cluster, scenario): evaluates
//                  the cluster's residual rows and Jacobian block
//                  [A_k | B_k] (src/kernels/{genrou,ieesgo,tgov1,sexs,
//                  esdc1a,ieeest}.jl), applies the backward-Euler scaling
//                  (src/dynamics.jl:366-391, 481-500), factors A_k with
//                  partial pivoting held in registers (one row per lane) and
//                  returns A_k^-1 f_k, A_k^-1 B_k and the Schur terms
//                  C_k A_k^-1 B_k, C_k A_k^-1 f_k (src/schur.jl:195-247,
//                  324-346) — the reference's gather + cuBLAS getrf/getrs
//                  sequence (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:1825-1887,
//                  2750-2779) fused into one pass.
//  network_kernel  one thread per (bus, scenario): complex Ybus row times
//                  V fused with machine injections, ZIP loads
//                  (src/kernels/zipload.jl), static generators
//                  (src/kernels/static_gen.jl) and fault shunts
//                  (src/dynamics.jl:314-327); writes the bus's 2x2 diagonal
//                  block of the reduced matrix S and its right-hand side.
//  factor/fwd/bwd  level-scheduled multifrontal LU of S (one CTA per
//                  (supernode, scenario)) and the two triangular solves; the
//                  replacement of cuDSS factorization/solve
//                  (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2782-2799).
//  update_kernel   z += dz: network and static-generator unknowns from the
//                  solve, cluster states by back-substitution
//                  dw_k = -(A_k^-1 f_k + A_k^-1 B_k dv) (src/schur.jl:383-409).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "gp_internal.h"

namespace gp {

#define FULL_MASK 0xffffffffu
constexpr double TWOPI60 = 2.0 * 3.14159265358979323846 * 60.0;

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long norm_bits(double v) {
    // non-negative doubles order like their bit patterns; NaN counts as +inf
    if (!(v == v)) return 0x7ff0000000000000ull;
    return (unsigned long long)__double_as_longlong(fabs(v));
}

// Cluster matrix in shared memory: row = state - ws, columns 0..28 the
// cluster states, 29/30 the bus voltage (vr, vi), 31 the residual.
constexpr int LDM = 32;
constexpr int WMAX = 29;
constexpr int COL_VR = 29, COL_VI = 30, COL_F = 31;
constexpr int CK_WARPS = 4;

struct CMat {
    double *A;
    int ws;
    __device__ __forceinline__ void put(int r, int c, double v) const { A[(r - ws) * LDM + (c - ws)] = v; }
    __device__ __forceinline__ void putv(int r, int which, double v) const { A[(r - ws) * LDM + COL_VR + which] = v; }
    __device__ __forceinline__ void putf(int r, double v) const { A[(r - ws) * LDM + COL_F] = v; }
};

__device__ __forceinline__ void genrou_sat_coef(double s1, double s2, double &sa, double &sb) {
    sa = 0.0;
    sb = 0.0;
    if (s1 <= 0.0 || s2 <= 0.0) return;
    const double e1 = 1.0, e2 = 1.2;
    double a = sqrt(s1 * e1 / (s2 * e2));
    if (a == 1.0) return;
    sa = e2 - (e1 - e2) / (a - 1.0);
    sb = s2 * e2 * (a - 1.0) * (a - 1.0) / ((e1 - e2) * (e1 - e2));
}

// GENROU residual rows + Jacobian (src/kernels/genrou.jl:48-141, 407-559).
// Returns the network-row couplings C (d f_vr/d{delta,i_q,i_d},
// d f_vi/d{delta,i_q,i_d}) and the injected current.
__device__ void genrou_eval(const DevProblem &P, int k, const double *z, const double *u0, const double *p,
                            const CMat &M, double *C, double *I, int *loc) {
    const DTab &G = P.dev[0];
    const int dp = G.diff_ptr[k], ap = G.alg_ptr[k], cp = G.ctrl_ptr[k], pp = G.par_ptr[k], bus = G.bus[k];
    const double x_d = p[pp], x_q = p[pp + 1], x_dp = p[pp + 2], x_qp = p[pp + 3], x_ddp = p[pp + 4],
                 xl = p[pp + 5], H = p[pp + 6], D = p[pp + 7], T_d0p = p[pp + 8], T_q0p = p[pp + 9],
                 T_d0dp = p[pp + 10], T_q0dp = p[pp + 11], S1 = p[pp + 12], S2 = p[pp + 13];
    const double x_qdp = x_ddp;
    const double e_qp = z[dp], e_dp = z[dp + 1], phi_1d = z[dp + 2], phi_2q = z[dp + 3], w = z[dp + 4],
                 delta = z[dp + 5];
    const double v_q = z[ap], v_d = z[ap + 1], i_q = z[ap + 2], i_d = z[ap + 3];
    const int vr_idx = P.net + 2 * bus;
    const double vr = z[vr_idx], vi = z[vr_idx + 1];
    const int pm_idx = G.link0[k], efd_idx = G.link1[k];
    const double e_fd = efd_idx >= 0 ? z[efd_idx] : u0[cp];
    const double p_m = pm_idx >= 0 ? z[pm_idx] : u0[cp + 1];
    const double dpl = x_dp - xl, qpl = x_qp - xl;
    const double psi_de = (x_ddp - xl) / dpl * e_qp + (x_dp - x_ddp) / dpl * phi_1d;
    const double psi_qe = -(x_ddp - xl) / qpl * e_dp + (x_qp - x_ddp) / qpl * phi_2q;
    double sa, sb;
    genrou_sat_coef(S1, S2, sa, sb);
    const double psi2 = sqrt(psi_de * psi_de + psi_qe * psi_qe);
    const bool sat_on = !(sb == 0.0 || psi2 <= sa || psi2 == 0.0);
    const double Se = sat_on ? sb * (psi2 - sa) * (psi2 - sa) / psi2 : 0.0;
    double sd, cd;
    sincos(delta, &sd, &cd);
    // residual
    M.putf(dp, (-e_qp + e_fd - (i_d - (-x_ddp + x_dp) * (-e_qp + i_d * dpl + phi_1d) / (dpl * dpl)) * (x_d - x_dp) -
                Se * psi_de) / T_d0p);
    M.putf(dp + 1, (-e_dp + (i_q - (-x_qdp + x_qp) * (e_dp + i_q * qpl + phi_2q) / (qpl * qpl)) * (x_q - x_qp)) / T_q0p);
    M.putf(dp + 2, (e_qp - i_d * dpl - phi_1d) / T_d0dp);
    M.putf(dp + 3, (-e_dp - i_q * qpl - phi_2q) / T_q0dp);
    M.putf(dp + 4, (p_m - D * w - psi_de * i_q + psi_qe * i_d) / (2.0 * H));
    M.putf(dp + 5, TWOPI60 * w);
    M.putf(ap, i_d - ((x_ddp - xl) / dpl * e_qp + (x_dp - x_ddp) / dpl * phi_1d - v_q) / x_ddp);
    M.putf(ap + 1, i_q - (-(x_qdp - xl) / qpl * e_dp + (x_qp - x_qdp) / qpl * phi_2q + v_d) / x_qdp);
    M.putf(ap + 2, v_d - (vr * sd - vi * cd));
    M.putf(ap + 3, v_q - (vr * cd + vi * sd));
    // Jacobian
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
    M.put(dp + 5, c_w, TWOPI60);
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
    // network coupling (not part of the cluster block)
    C[0] = i_d * cd - i_q * sd;
    C[1] = cd;
    C[2] = sd;
    C[3] = i_d * sd + i_q * cd;
    C[4] = sd;
    C[5] = -cd;
    I[0] = sd * i_d + cd * i_q;
    I[1] = -cd * i_d + sd * i_q;
    loc[0] = c_delta - M.ws;
    loc[1] = c_iq - M.ws;
    loc[2] = c_id - M.ws;
}

// IEESGO (src/kernels/ieesgo.jl:133-224)
__device__ void ieesgo_eval(const DevProblem &P, int k, const double *z, const double *p, const CMat &M) {
    const DTab &T = P.dev[1];
    const int dp = T.diff_ptr[k], ap = T.alg_ptr[k], pp = T.par_ptr[k], wi = T.link0[k];
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

// TGOV1 (src/kernels/tgov1.jl:73-146)
__device__ void tgov1_eval(const DevProblem &P, int k, const double *z, const double *p, const CMat &M) {
    const DTab &T = P.dev[2];
    const int dp = T.diff_ptr[k], ap = T.alg_ptr[k], pp = T.par_ptr[k], wi = T.link0[k];
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

// SEXS (src/kernels/sexs.jl:74-156)
__device__ void sexs_eval(const DevProblem &P, int k, const double *z, const double *p, const CMat &M) {
    const DTab &T = P.dev[3];
    const int dp = T.diff_ptr[k], pp = T.par_ptr[k], vsi = T.link0[k];
    const int vr_idx = P.net + 2 * T.bus[k];
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

// ESDC1A (src/kernels/esdc1a.jl:97-196)
__device__ void esdc1a_eval(const DevProblem &P, int k, const double *z, const double *p, const CMat &M) {
    const DTab &T = P.dev[4];
    const int dp = T.diff_ptr[k], pp = T.par_ptr[k], vsi = T.link0[k];
    const int vr_idx = P.net + 2 * T.bus[k];
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

// IEEEST (src/kernels/ieeest.jl:207-359)
__device__ void ieeest_eval(const DevProblem &P, int k, const double *z, const double *p, const CMat &M) {
    const DTab &T = P.dev[5];
    const int dp = T.diff_ptr[k], ap = T.alg_ptr[k], pp = T.par_ptr[k], wi = T.link0[k];
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
    const double d2[3] = {rA, A5 - A3 * rA, 1.0 - rA};
    const double r12 = T1 / T2;
    const double d3[4] = {r12 * d2[0], r12 * d2[1], r12 * d2[2], 1.0 - r12};
    const double r34 = T3 / T4;
    const double d4[5] = {r34 * d3[0], r34 * d3[1], r34 * d3[2], r34 * d3[3], 1.0 - r34};
    M.put(dp, dp, -A1 / A2);
    M.put(dp, dp + 1, -1.0 / A2);
    if (wi >= 0) M.put(dp, wi, 1.0 / A2);
    M.put(dp + 1, dp, 1.0);
    M.put(dp + 2, dp + 1, 1.0 / A4);
    M.put(dp + 2, dp + 2, -A3 / A4);
    M.put(dp + 2, dp + 3, -1.0 / A4);
    M.put(dp + 3, dp + 2, 1.0);
#pragma unroll
    for (int j = 0; j < 3; j++) M.put(dp + 4, dp + 1 + j, d2[j] / T2);
    M.put(dp + 4, dp + 4, -1.0 / T2);
#pragma unroll
    for (int j = 0; j < 4; j++) M.put(dp + 5, dp + 1 + j, d3[j] / T4);
    M.put(dp + 5, dp + 5, -1.0 / T4);
#pragma unroll
    for (int j = 0; j < 5; j++) M.put(dp + 6, dp + 1 + j, KS * d4[j] / T6);
    M.put(dp + 6, dp + 6, -1.0 / T6);
    const double r56 = T5 / T6;
#pragma unroll
    for (int j = 0; j < 5; j++) M.put(ap, dp + 1 + j, -r56 * KS * d4[j]);
    M.put(ap, dp + 6, r56);
    M.put(ap, ap, 1.0);
}

// ---------------------------------------------------------------------------
// cluster kernel
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(CK_WARPS * 32) cluster_kernel(DevProblem P, DevWork W, int want_f) {
    __shared__ double sA[CK_WARPS][WMAX * LDM];
    __shared__ double sC[CK_WARPS][8];
    __shared__ int sLoc[CK_WARPS][3];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long task = (long long)blockIdx.x * CK_WARPS + warp;
    if (task >= (long long)P.M * P.n_cl) return;
    const int m = (int)(task / P.n_cl), c = (int)(task % P.n_cl);
    if (!W.active[m]) return;
    const int ws = P.cl_w_start[c], Wn = P.cl_w_size[c];
    const double *z = W.z + (size_t)m * P.n_sys;
    const double *zold = W.zold + (size_t)m * P.n_sys;
    const double *u0 = W.u0 + (size_t)m * P.n_ctrl;
    const double *p = W.p + (size_t)m * P.n_par;
    double *A = sA[warp];
    for (int i = lane; i < Wn * LDM; i += 32) A[i] = 0.0;
    __syncwarp();
    CMat Mx{A, ws};
    if (lane == 0) {
        genrou_eval(P, P.cl_gen[c], z, u0, p, Mx, sC[warp], sC[warp] + 6, sLoc[warp]);
    } else if (lane == 1) {
        const int gt = P.cl_gov_type[c];
        if (gt == 1) ieesgo_eval(P, P.cl_gov[c], z, p, Mx);
        else if (gt == 2) tgov1_eval(P, P.cl_gov[c], z, p, Mx);
    } else if (lane == 2) {
        const int et = P.cl_exc_type[c];
        if (et == 3) sexs_eval(P, P.cl_exc[c], z, p, Mx);
        else if (et == 4) esdc1a_eval(P, P.cl_exc[c], z, p, Mx);
    } else if (lane == 3) {
        if (P.cl_pss[c] >= 0) ieeest_eval(P, P.cl_pss[c], z, p, Mx);
    }
    __syncwarp();
    const bool has_row = lane < Wn;
    double a[LDM];
#pragma unroll
    for (int j = 0; j < LDM; j++) a[j] = has_row ? A[lane * LDM + j] : 0.0;
    // backward Euler on differential rows
    const double dt = *W.dt;
    if (has_row && P.is_diff[ws + lane]) {
#pragma unroll
        for (int j = 0; j < COL_F; j++) a[j] *= -dt;
#pragma unroll
        for (int j = 0; j < WMAX; j++)
            if (j == lane) a[j] += 1.0;
        a[COL_F] = z[ws + lane] - zold[ws + lane] - dt * a[COL_F];
    }
    if (want_f && has_row) W.f[(size_t)m * P.n_sys + ws + lane] = a[COL_F];
    // residual norm
    unsigned long long nb = has_row ? norm_bits(a[COL_F]) : 0ull;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_xor_sync(FULL_MASK, nb, off);
        nb = o > nb ? o : nb;
    }
    if (lane == 0) atomicMax(W.norm + m, nb);
    // LU with partial pivoting: lane i owns row i; the three right-hand
    // sides (B(:,vr), B(:,vi), f) ride along as columns 29..31.
    bool pivoted = !has_row;
    int mystep = -1;
#pragma unroll
    for (int k = 0; k < WMAX; k++) {
        if (k < Wn) {
            double cand = pivoted ? -1.0 : fabs(a[k]);
            int cl = lane;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                double ov = __shfl_xor_sync(FULL_MASK, cand, off);
                int ol = __shfl_xor_sync(FULL_MASK, cl, off);
                if (ov > cand || (ov == cand && ol < cl)) { cand = ov; cl = ol; }
            }
            const int pl = cl;
            const double pk = __shfl_sync(FULL_MASK, a[k], pl);
            const bool elim = !pivoted && lane != pl;
            const double l = elim ? a[k] / pk : 0.0;
            if (lane == pl) { pivoted = true; mystep = k; }
#pragma unroll
            for (int j = k + 1; j < LDM; j++) {
                if (j < Wn || j >= WMAX) {
                    const double pr = __shfl_sync(FULL_MASK, a[j], pl);
                    if (elim) a[j] -= l * pr;
                }
            }
        }
    }
    // back substitution for the three right-hand sides
#pragma unroll
    for (int k = WMAX - 1; k >= 0; k--) {
        if (k < Wn) {
            const unsigned own = __ballot_sync(FULL_MASK, mystep == k);
            const int q = __ffs(own) - 1;
            const double d = __shfl_sync(FULL_MASK, a[k], q);
            const double x1 = __shfl_sync(FULL_MASK, a[COL_VR], q) / d;
            const double x2 = __shfl_sync(FULL_MASK, a[COL_VI], q) / d;
            const double y = __shfl_sync(FULL_MASK, a[COL_F], q) / d;
            if (lane == q) {
                a[COL_VR] = x1;
                a[COL_VI] = x2;
                a[COL_F] = y;
            } else if (mystep >= 0 && mystep < k) {
                const double u = a[k];
                a[COL_VR] -= u * x1;
                a[COL_VI] -= u * x2;
                a[COL_F] -= u * y;
            }
        }
    }
    const int n_da = P.n_diff + P.n_alg;
    if (mystep >= 0) {
        double *yx = W.yx + (size_t)m * 3 * n_da + ws + mystep;
        yx[0] = a[COL_F];
        yx[n_da] = a[COL_VR];
        yx[2 * n_da] = a[COL_VI];
    }
    // Schur terms: D = C X, r = C y over the three coupled states
    double X1[3], X2[3], Y[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {
        const int kk = sLoc[warp][t];
        const unsigned own = __ballot_sync(FULL_MASK, mystep == kk);
        const int q = __ffs(own) - 1;
        X1[t] = __shfl_sync(FULL_MASK, a[COL_VR], q);
        X2[t] = __shfl_sync(FULL_MASK, a[COL_VI], q);
        Y[t] = __shfl_sync(FULL_MASK, a[COL_F], q);
    }
    if (lane == 0) {
        const double *Cc = sC[warp];
        double *o = W.clout + ((size_t)m * P.n_cl + c) * 8;
        o[0] = Cc[0] * X1[0] + Cc[1] * X1[1] + Cc[2] * X1[2];
        o[1] = Cc[0] * X2[0] + Cc[1] * X2[1] + Cc[2] * X2[2];
        o[2] = Cc[3] * X1[0] + Cc[4] * X1[1] + Cc[5] * X1[2];
        o[3] = Cc[3] * X2[0] + Cc[4] * X2[1] + Cc[5] * X2[2];
        o[4] = Cc[0] * Y[0] + Cc[1] * Y[1] + Cc[2] * Y[2];
        o[5] = Cc[3] * Y[0] + Cc[4] * Y[1] + Cc[5] * Y[2];
        o[6] = Cc[6];
        o[7] = Cc[7];
    }
}

void launch_cluster(const DevProblem &P, const DevWork &W, int want_f, cudaStream_t st) {
    long long tasks = (long long)P.M * P.n_cl;
    if (tasks == 0) return;
    int blocks = (int)((tasks + CK_WARPS - 1) / CK_WARPS);
    cluster_kernel<<<blocks, CK_WARPS * 32, 0, st>>>(P, W, want_f);
}

// ---------------------------------------------------------------------------
// network kernel
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) network_kernel(DevProblem P, DevWork W, int want_f) {
    const long long task = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = task < (long long)P.M * P.n_bus;
    const int m = valid ? (int)(task / P.n_bus) : P.M;
    const int b = valid ? (int)(task % P.n_bus) : 0;
    const bool act = valid && W.active[m];
    unsigned long long nb = 0ull;
    if (act) {
        const double *z = W.z + (size_t)m * P.n_sys;
        const double *p = W.p + (size_t)m * P.n_par;
        const int net = P.net;
        const double vr = z[net + 2 * b], vi = z[net + 2 * b + 1];
        double fr = 0.0, fi = 0.0, d00 = 0.0, d01 = 0.0, d10 = 0.0, d11 = 0.0, rr = 0.0, ri = 0.0;
        for (int q = P.y_rowptr[b]; q < P.y_rowptr[b + 1]; q++) {
            const int j = P.y_colidx[q];
            const double g = P.y_re[q], bb = P.y_im[q];
            const double vrj = z[net + 2 * j], vij = z[net + 2 * j + 1];
            fr -= g * vrj - bb * vij;
            fi -= bb * vrj + g * vij;
            if (j == b) { d00 -= g; d01 += bb; d10 -= bb; d11 -= g; }
        }
        for (int q = P.bus_cl_ptr[b]; q < P.bus_cl_ptr[b + 1]; q++) {
            const double *o = W.clout + ((size_t)m * P.n_cl + P.bus_cl[q]) * 8;
            d00 -= o[0]; d01 -= o[1]; d10 -= o[2]; d11 -= o[3];
            rr += o[4]; ri += o[5];
            fr += o[6]; fi += o[7];
        }
        const DTab &ZL = P.dev[6];
        for (int q = P.bus_zl_ptr[b]; q < P.bus_zl_ptr[b + 1]; q++) {
            const int k = P.bus_zl[q];
            const int pp = ZL.par_ptr[k];
            const double pl = p[pp], ql = p[pp + 1], al = p[pp + 2], yre0 = p[pp + 7], yim0 = p[pp + 8];
            const double yre = al * yre0, yim = al * yim0;
            const double vm2 = vr * vr + vi * vi, vm2_tld = 0.2;
            fr -= vr * yre - vi * yim;
            fi -= vr * yim + vi * yre;
            const double den = vm2 > vm2_tld ? vm2 : vm2_tld;
            fr -= (1.0 - al) * (pl * vr - ql * vi) / den;
            fi -= (1.0 - al) * (ql * vr + pl * vi) / den;
            double p11, p12, p21, p22;
            if (vm2 > vm2_tld) {
                const double iv4 = 1.0 / (vm2 * vm2);
                p11 = (1.0 - al) * ((pl * vr - ql * vi) * 2.0 * vr - pl * vm2) * iv4;
                p12 = (1.0 - al) * ((pl * vr - ql * vi) * 2.0 * vi + ql * vm2) * iv4;
                p21 = (1.0 - al) * ((ql * vr + pl * vi) * 2.0 * vr - ql * vm2) * iv4;
                p22 = (1.0 - al) * ((ql * vr + pl * vi) * 2.0 * vi - pl * vm2) * iv4;
            } else {
                const double ith = 1.0 / vm2_tld;
                p11 = (1.0 - al) * (-pl) * ith;
                p12 = (1.0 - al) * (ql)*ith;
                p21 = (1.0 - al) * (-ql) * ith;
                p22 = (1.0 - al) * (-pl) * ith;
            }
            d00 += -al * yre0 + p11;
            d01 += al * yim0 + p12;
            d10 += -al * yim0 + p21;
            d11 += -al * yre0 + p22;
        }
        const DTab &SG = P.dev[7];
        for (int q = P.bus_sg_ptr[b]; q < P.bus_sg_ptr[b + 1]; q++) {
            const int k = P.bus_sg[q];
            const int pp = SG.par_ptr[k], ap = SG.alg_ptr[k], bt = SG.link0[k];
            const double vm2r = vr * vr + vi * vi, vm2 = vm2r > 0.2 ? vm2r : 0.2;
            double Pg, Qg;
            if (bt == 2) { Pg = p[pp]; Qg = z[ap]; }
            else if (bt == 3) { Pg = z[ap]; Qg = z[ap + 1]; }
            else { Pg = p[pp]; Qg = p[pp + 1]; }
            const double irn = Pg * vr + Qg * vi, iin = Pg * vi - Qg * vr;
            fr += irn / vm2;
            fi += iin / vm2;
            if (vm2r > 0.2) {
                const double vm4 = vm2 * vm2;
                d00 += Pg / vm2 - 2.0 * vr * irn / vm4;
                d01 += Qg / vm2 - 2.0 * vi * irn / vm4;
                d10 += -Qg / vm2 - 2.0 * vr * iin / vm4;
                d11 += Pg / vm2 - 2.0 * vi * iin / vm4;
            } else {
                d00 += Pg / vm2;
                d01 += Qg / vm2;
                d10 += -Qg / vm2;
                d11 += Pg / vm2;
            }
            double *sv = W.svar + (size_t)m * P.n_var + P.sg_var[k];
            double *xp = W.xperm + (size_t)m * P.n_red;
            const int r0 = P.sg_red[k];
            if (bt == 2) {
                const double vset = p[pp + 2];
                const double fa = vr * vr + vi * vi - vset * vset;
                // (ap,vr) (ap,vi) (vr,ap) (vi,ap)
                sv[0] = 2.0 * vr; sv[1] = 2.0 * vi; sv[2] = vi / vm2; sv[3] = -vr / vm2;
                xp[P.iperm[r0]] = -fa;
                if (want_f) W.f[(size_t)m * P.n_sys + ap] = fa;
                const unsigned long long t = norm_bits(fa);
                nb = t > nb ? t : nb;
            } else if (bt == 3) {
                const double vset = p[pp + 2], aset = p[pp + 3];
                const double fa0 = vr - vset * cos(aset), fa1 = vi - vset * sin(aset);
                // (ap,vr) (ap+1,vi) (vr,ap) (vi,ap) (vr,ap+1) (vi,ap+1)
                sv[0] = 1.0; sv[1] = 1.0; sv[2] = vr / vm2; sv[3] = vi / vm2; sv[4] = vi / vm2; sv[5] = -vr / vm2;
                xp[P.iperm[r0]] = -fa0;
                xp[P.iperm[r0 + 1]] = -fa1;
                if (want_f) {
                    W.f[(size_t)m * P.n_sys + ap] = fa0;
                    W.f[(size_t)m * P.n_sys + ap + 1] = fa1;
                }
                unsigned long long t = norm_bits(fa0);
                nb = t > nb ? t : nb;
                t = norm_bits(fa1);
                nb = t > nb ? t : nb;
            }
        }
        for (int e = P.fl_ptr[m]; e < P.fl_ptr[m + 1]; e++) {
            if (P.fl_on[e] && P.fl_bus[e] == b) {
                const double yf = P.fl_yf[e];
                fr -= yf * vr;
                fi -= yf * vi;
                d00 -= yf;
                d11 -= yf;
            }
        }
        if (want_f) {
            W.f[(size_t)m * P.n_sys + net + 2 * b] = fr;
            W.f[(size_t)m * P.n_sys + net + 2 * b + 1] = fi;
        }
        double *sv = W.svar + (size_t)m * P.n_var + 4 * b;
        sv[0] = d00; sv[1] = d01; sv[2] = d10; sv[3] = d11;
        double *xp = W.xperm + (size_t)m * P.n_red;
        xp[P.iperm[2 * b]] = -(fr - rr);
        xp[P.iperm[2 * b + 1]] = -(fi - ri);
        unsigned long long t = norm_bits(fr);
        nb = t > nb ? t : nb;
        t = norm_bits(fi);
        nb = t > nb ? t : nb;
    }
    // segmented max over lanes of the same scenario, one atomic per segment
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        unsigned long long o = __shfl_down_sync(FULL_MASK, nb, off);
        int om = __shfl_down_sync(FULL_MASK, m, off);
        if (lane + off < 32 && om == m) nb = o > nb ? o : nb;
    }
    const int mprev = __shfl_up_sync(FULL_MASK, m, 1);
    if (act && (lane == 0 || mprev != m)) atomicMax(W.norm + m, nb);
}

void launch_network(const DevProblem &P, const DevWork &W, int want_f, cudaStream_t st) {
    long long tasks = (long long)P.M * P.n_bus;
    int blocks = (int)((tasks + 255) / 256);
    network_kernel<<<blocks, 256, 0, st>>>(P, W, want_f);
}

// ---------------------------------------------------------------------------
// convergence bookkeeping
// ---------------------------------------------------------------------------

__global__ void reset_norm_kernel(DevWork W, int M) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < M) W.norm[m] = 0ull;
    if (m == 0) *W.flag = 0;
}

void launch_reset_norm(const DevProblem &P, const DevWork &W, cudaStream_t st) {
    reset_norm_kernel<<<(P.M + 255) / 256, 256, 0, st>>>(W, P.M);
}

__global__ void check_kernel(DevWork W, int M, double tol, int itermax) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M || !W.active[m]) return;
    const unsigned long long bits = W.norm[m];
    const double nrm = __longlong_as_double((long long)bits);
    if (nrm < tol) {
        W.active[m] = 0;
    } else if (bits >= 0x7ff0000000000000ull) {
        W.active[m] = 0;
        W.status[m] |= 2;
    } else if (W.iters[m] >= itermax) {
        W.active[m] = 0;
        W.status[m] |= 1;
    } else {
        W.iters[m] += 1;
        atomicAdd(W.flag, 1);
    }
}

void launch_check(const DevProblem &P, const DevWork &W, double tol, int itermax, cudaStream_t st) {
    check_kernel<<<(P.M + 255) / 256, 256, 0, st>>>(W, P.M, tol, itermax);
}

// ---------------------------------------------------------------------------
// multifrontal factorisation and solves
// ---------------------------------------------------------------------------

__global__ void factor_kernel(DevProblem P, DevWork W, DevSym S, int lvl_begin) {
    extern __shared__ double smem[];
    const int s = S.level_sups[lvl_begin + blockIdx.x];
    const int m = blockIdx.y;
    if (!W.active[m]) return;
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int r = S.row_ptr[s + 1] - S.row_ptr[s];
    const int mm = ns + r;
    double *F = smem;
    __shared__ int s_piv;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < mm * mm; i += nt) F[i] = 0.0;
    __syncthreads();
    for (int e = S.asmc_ptr[s] + tid; e < S.asmc_ptr[s + 1]; e += nt) F[S.asmc_pos[e]] += S.asmc_val[e];
    const double *sv = W.svar + (size_t)m * P.n_var;
    for (int e = S.asmv_ptr[s] + tid; e < S.asmv_ptr[s + 1]; e += nt) F[S.asmv_pos[e]] += sv[S.asmv_idx[e]];
    __syncthreads();
    const double *fronts = S.fronts + (size_t)m * S.front_total;
    for (int q = S.child_ptr[s]; q < S.child_ptr[s + 1]; q++) {
        const int c = S.children[q];
        const int nc = S.sup_start[c + 1] - S.sup_start[c];
        const int rc = S.row_ptr[c + 1] - S.row_ptr[c];
        const int mc = nc + rc;
        const int *rel = S.relmap + S.relmap_ptr[c];
        const double *Fc = fronts + S.front_off[c];
        for (int t = tid; t < rc * rc; t += nt) {
            const int a = t % rc, b = t / rc;
            F[rel[a] + rel[b] * mm] += Fc[(nc + a) + (size_t)(nc + b) * mc];
        }
        __syncthreads();
    }
    int *ipiv = S.ipiv + (size_t)m * S.n + start;
    for (int k = 0; k < ns; k++) {
        if (tid < 32) {
            double best = -1.0;
            int bi = k;
            for (int i = k + tid; i < ns; i += 32) {
                const double v = fabs(F[i + k * mm]);
                if (v > best) { best = v; bi = i; }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const double ov = __shfl_xor_sync(FULL_MASK, best, off);
                const int oi = __shfl_xor_sync(FULL_MASK, bi, off);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (tid == 0) {
                s_piv = bi;
                ipiv[k] = bi;
                if (best == 0.0) atomicOr(W.status + m, 4);
            }
        }
        __syncthreads();
        const int pv = s_piv;
        if (pv != k) {
            for (int j = tid; j < mm; j += nt) {
                const double t = F[k + j * mm];
                F[k + j * mm] = F[pv + j * mm];
                F[pv + j * mm] = t;
            }
            __syncthreads();
        }
        const double pk = F[k + k * mm];
        const double inv = 1.0 / pk;
        for (int i = k + 1 + tid; i < mm; i += nt) F[i + k * mm] *= inv;
        __syncthreads();
        const int len = mm - k - 1;
        for (int t = tid; t < len * len; t += nt) {
            const int i = k + 1 + t % len, j = k + 1 + t / len;
            F[i + j * mm] -= F[i + k * mm] * F[k + j * mm];
        }
        __syncthreads();
    }
    double *out = S.fronts + (size_t)m * S.front_total + S.front_off[s];
    for (int i = tid; i < mm * mm; i += nt) out[i] = F[i];
}

static int block_for(int max_front) {
    if (max_front <= 16) return 64;
    if (max_front <= 48) return 128;
    return 256;
}

void launch_factor_level(const DevProblem &P, const DevWork &W, const DevSym &S, int lvl_begin, int lvl_count,
                         int max_front, cudaStream_t st) {
    dim3 grid(lvl_count, P.M);
    size_t smem = (size_t)max_front * max_front * sizeof(double);
    factor_kernel<<<grid, block_for(max_front), smem, st>>>(P, W, S, lvl_begin);
}

// Opt the factorisation kernel into the largest dynamic shared memory the
// device allows next to its static shared memory; returns that size, or -1
// if the runtime refused.
int factor_smem_limit() {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return -1;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, factor_kernel) != cudaSuccess) return -1;
    const int dyn = v - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return dyn;
}

// forward solve: bottom-up, extend-add of the children's update vectors
__global__ void fwd_kernel(DevProblem P, DevWork W, DevSym S, int lvl_begin) {
    extern __shared__ double smem[];
    const int s = S.level_sups[lvl_begin + blockIdx.x];
    const int m = blockIdx.y;
    if (!W.active[m]) return;
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int r = S.row_ptr[s + 1] - S.row_ptr[s];
    const int mm = ns + r;
    double *t = smem, *u = smem + ns;
    const int tid = threadIdx.x, nt = blockDim.x;
    double *x = W.xperm + (size_t)m * P.n_red;
    double *uv = S.uvec + (size_t)m * S.uvec_total;
    for (int i = tid; i < ns; i += nt) t[i] = x[start + i];
    for (int i = tid; i < r; i += nt) u[i] = 0.0;
    __syncthreads();
    for (int q = S.child_ptr[s]; q < S.child_ptr[s + 1]; q++) {
        const int c = S.children[q];
        const int rc = S.row_ptr[c + 1] - S.row_ptr[c];
        const int *rel = S.relmap + S.relmap_ptr[c];
        const double *uc = uv + S.uvec_off[c];
        for (int a = tid; a < rc; a += nt) {
            const int pos = rel[a];
            if (pos < ns) t[pos] += uc[a];
            else u[pos - ns] += uc[a];
        }
        __syncthreads();
    }
    const double *F = S.fronts + (size_t)m * S.front_total + S.front_off[s];
    const int *ipiv = S.ipiv + (size_t)m * S.n + start;
    if (tid == 0)
        for (int k = 0; k < ns; k++) {
            const int pv = ipiv[k];
            if (pv != k) { const double tt = t[k]; t[k] = t[pv]; t[pv] = tt; }
        }
    __syncthreads();
    for (int k = 0; k < ns; k++) {
        const double tk = t[k];
        for (int i = k + 1 + tid; i < ns; i += nt) t[i] -= F[i + k * mm] * tk;
        __syncthreads();
    }
    for (int i = tid; i < r; i += nt) {
        double acc = 0.0;
        for (int k = 0; k < ns; k++) acc += F[(ns + i) + (size_t)k * mm] * t[k];
        u[i] -= acc;
    }
    __syncthreads();
    for (int i = tid; i < ns; i += nt) x[start + i] = t[i];
    double *us = uv + S.uvec_off[s];
    for (int i = tid; i < r; i += nt) us[i] = u[i];
}

void launch_fwd_level(const DevProblem &P, const DevWork &W, const DevSym &S, int lvl_begin, int lvl_count,
                      int max_front, cudaStream_t st) {
    dim3 grid(lvl_count, P.M);
    fwd_kernel<<<grid, max_front <= 32 ? 32 : 128, (size_t)max_front * sizeof(double), st>>>(P, W, S, lvl_begin);
}

// backward solve: top-down, gathers of the ancestors' solution
__global__ void bwd_kernel(DevProblem P, DevWork W, DevSym S, int lvl_begin) {
    extern __shared__ double smem[];
    const int s = S.level_sups[lvl_begin + blockIdx.x];
    const int m = blockIdx.y;
    if (!W.active[m]) return;
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int r = S.row_ptr[s + 1] - S.row_ptr[s];
    const int mm = ns + r;
    double *t = smem;
    const int tid = threadIdx.x, nt = blockDim.x;
    double *x = W.xperm + (size_t)m * P.n_red;
    const double *F = S.fronts + (size_t)m * S.front_total + S.front_off[s];
    const int *rows = S.rows + S.row_ptr[s];
    for (int i = tid; i < ns; i += nt) {
        double acc = 0.0;
        for (int a = 0; a < r; a++) acc += F[i + (size_t)(ns + a) * mm] * x[rows[a]];
        t[i] = x[start + i] - acc;
    }
    __syncthreads();
    for (int k = ns - 1; k >= 0; k--) {
        if (tid == 0) t[k] /= F[k + k * mm];
        __syncthreads();
        const double tk = t[k];
        for (int i = tid; i < k; i += nt) t[i] -= F[i + k * mm] * tk;
        __syncthreads();
    }
    for (int i = tid; i < ns; i += nt) x[start + i] = t[i];
}

void launch_bwd_level(const DevProblem &P, const DevWork &W, const DevSym &S, int lvl_begin, int lvl_count,
                      int max_front, cudaStream_t st) {
    dim3 grid(lvl_count, P.M);
    bwd_kernel<<<grid, max_front <= 32 ? 32 : 128, (size_t)max_front * sizeof(double), st>>>(P, W, S, lvl_begin);
}

// ---------------------------------------------------------------------------
// Newton update
// ---------------------------------------------------------------------------

// state_bus[i]: bus of the non-trivial cluster owning cluster state i, or
// -1 when the state is a reduced unknown (static generator); red_of[i] its
// reduced index in that case.
__global__ void update_kernel(DevProblem P, DevWork W, const int *state_bus, const int *red_of) {
    const long long task = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= (long long)P.M * P.n_sys) return;
    const int m = (int)(task / P.n_sys), i = (int)(task % P.n_sys);
    if (!W.active[m]) return;
    double *z = W.z + (size_t)m * P.n_sys;
    const double *x = W.xperm + (size_t)m * P.n_red;
    const int n_da = P.n_diff + P.n_alg;
    if (i >= P.net) {
        z[i] += x[P.iperm[i - P.net]];
    } else {
        const int b = state_bus[i];
        if (b >= 0) {
            const double *yx = W.yx + (size_t)m * 3 * n_da;
            const double dvr = x[P.iperm[2 * b]], dvi = x[P.iperm[2 * b + 1]];
            z[i] -= yx[i] + yx[n_da + i] * dvr + yx[2 * n_da + i] * dvi;
        } else {
            z[i] += x[P.iperm[red_of[i]]];
        }
    }
}

void launch_update(const DevProblem &P, const DevWork &W, const DevSym &S, const int *perm, cudaStream_t st) {
    (void)S;
    // `perm` carries the two state maps back to back: state_bus then red_of
    const int n_da = P.n_diff + P.n_alg;
    long long tasks = (long long)P.M * P.n_sys;
    update_kernel<<<(int)((tasks + 255) / 256), 256, 0, st>>>(P, W, perm, perm + n_da);
}

// ---------------------------------------------------------------------------
// events
// ---------------------------------------------------------------------------

__global__ void events_kernel(const int *on_step, const int *off_step, const int *scen, uint8_t *fl_on,
                              uint8_t *active, int n_fl, int step) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_fl) return;
    // a fault switched on and off at the same step ends off, as the
    // reference applies the schedule entries in order (src/dynamics.jl:604-629)
    bool hit = false;
    if (on_step[e] == step) { fl_on[e] = 1; hit = true; }
    if (off_step[e] == step) { fl_on[e] = 0; hit = true; }
    if (hit) active[scen[e]] = 1;
}

void launch_events(const DevProblem &P, const DevWork &W, const int *fl_on_step, const int *fl_off_step,
                   const int *fl_scen, uint8_t *fl_on, int n_fl, int step, cudaStream_t st) {
    (void)P;
    if (n_fl == 0) return;
    events_kernel<<<(n_fl + 255) / 256, 256, 0, st>>>(fl_on_step, fl_off_step, fl_scen, fl_on, W.active, n_fl, step);
}

}  // namespace gp
