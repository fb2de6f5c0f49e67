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

// Constants of a device that depend on its parameters only (reciprocals of
// time constants, reactance ratios, saturation coefficients).  K(slot, f)
// returns the constant in that slot: ComputeK evaluates f; RecordK
// evaluates it and stores it (slot-major, stride apart); LoadK reads the
// stored value and never evaluates f.  Slots: machine 0-15, governor
// 16-21, exciter 22-25, stabiliser 26-34.
constexpr int kConstSlots = 36;
struct ComputeK {
    static constexpr bool kLoad = false;
    template <class F>
    GP_HD double operator()(int, F f) const { return f(); }
    GP_HD void rec(int, double) const {}
    GP_HD double at(int) const { return 0.0; }
};
struct RecordK {
    double *k;
    int stride;
    static constexpr bool kLoad = false;
    template <class F>
    GP_HD double operator()(int i, F f) const {
        const double v = f();
        k[i * stride] = v;
        return v;
    }
    GP_HD void rec(int i, double v) const { k[i * stride] = v; }
    GP_HD double at(int) const { return 0.0; }
};
struct LoadK {
    const double *k;
    int stride;
    static constexpr bool kLoad = true;
    template <class F>
    GP_HD double operator()(int i, F) const { return k[i * stride]; }
    GP_HD void rec(int, double) const {}
    GP_HD double at(int i) const { return k[i * stride]; }
};

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
template <class Sink, class KP = ComputeK>
GP_HD void genrou_eval(const DevRef &d, int net, const double *z, const double *u0, const double *p, Sink &M,
                       double *C, double *I, const KP &kc = KP()) {
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
    // every division by a parameter is taken once, as a reciprocal
    // (FP64 division is dear on this GPU; the equations are unchanged)
    const double dpl = x_dp - xl, qpl = x_qp - xl;
    const double idpl = kc(0, [&] { return 1.0 / dpl; }), iqpl = kc(1, [&] { return 1.0 / qpl; });
    const double iTd = kc(2, [&] { return 1.0 / T_d0p; }), iTq = kc(3, [&] { return 1.0 / T_q0p; });
    const double iTdd = kc(4, [&] { return 1.0 / T_d0dp; }), iTqd = kc(5, [&] { return 1.0 / T_q0dp; });
    const double i2H = kc(6, [&] { return 0.5 / H; }), ixd = kc(7, [&] { return 1.0 / x_ddp; });   // x_qdp = x_ddp
    const double a_eqp = kc(8, [&] { return (x_ddp - xl) * idpl; });
    const double a_phi1d = kc(9, [&] { return (x_dp - x_ddp) * idpl; });
    const double b_edp = kc(10, [&] { return -(x_ddp - xl) * iqpl; });
    const double b_phi2q = kc(11, [&] { return (x_qp - x_ddp) * iqpl; });
    const double kd = kc(12, [&] { return (x_dp - x_ddp) * idpl * idpl; });
    const double kq = kc(13, [&] { return (x_qp - x_qdp) * iqpl * iqpl; });
    const double psi_de = a_eqp * e_qp + a_phi1d * phi_1d;
    const double psi_qe = b_edp * e_dp + b_phi2q * phi_2q;
    double sa, sb;
    if constexpr (KP::kLoad) {
        sa = kc.at(14);
        sb = kc.at(15);
    } else {
        sat_coef(S1, S2, sa, sb);
        kc.rec(14, sa);
        kc.rec(15, sb);
    }
    const double psi2 = sqrt(psi_de * psi_de + psi_qe * psi_qe);
    const bool sat_on = !(sb == 0.0 || psi2 <= sa || psi2 == 0.0);
    const double ipsi2 = psi2 == 0.0 ? 0.0 : 1.0 / psi2;
    const double Se = sat_on ? sb * (psi2 - sa) * (psi2 - sa) * ipsi2 : 0.0;
    double sd, cd;
#ifdef __CUDA_ARCH__
    sincos(delta, &sd, &cd);
#else
    sd = sin(delta);
    cd = cos(delta);
#endif
    M.putf(dp, (-e_qp + e_fd - (i_d - kd * (-e_qp + i_d * dpl + phi_1d)) * (x_d - x_dp) - Se * psi_de) * iTd);
    M.putf(dp + 1, (-e_dp + (i_q - kq * (e_dp + i_q * qpl + phi_2q)) * (x_q - x_qp)) * iTq);
    M.putf(dp + 2, (e_qp - i_d * dpl - phi_1d) * iTdd);
    M.putf(dp + 3, (-e_dp - i_q * qpl - phi_2q) * iTqd);
    M.putf(dp + 4, (p_m - D * w - psi_de * i_q + psi_qe * i_d) * i2H);
    M.putf(dp + 5, kTwoPi60 * w);
    M.putf(ap, i_d - (psi_de - v_q) * ixd);
    M.putf(ap + 1, i_q - (psi_qe + v_d) * ixd);
    M.putf(ap + 2, v_d - (vr * sd - vi * cd));
    M.putf(ap + 3, v_q - (vr * cd + vi * sd));
    double dSe = 0.0;
    if (sat_on) {
        double g = psi2 - sa;
        dSe = sb * (2.0 * g * psi2 - g * g) * ipsi2 * ipsi2;
    }
    const double dpd = psi_de * ipsi2;
    const double dpq = psi_qe * ipsi2;
    const double dT_dde = -(dSe * dpd * psi_de + Se);
    const double dT_dqe = -(dSe * dpq * psi_de);
    const int c_eqp = dp, c_edp = dp + 1, c_phi1d = dp + 2, c_phi2q = dp + 3, c_w = dp + 4, c_delta = dp + 5;
    const int c_vq = ap, c_vd = ap + 1, c_iq = ap + 2, c_id = ap + 3;
    M.put(dp, c_eqp, (-(x_d - x_dp) * kd - 1) * iTd + dT_dde * a_eqp * iTd);
    M.put(dp, c_phi1d, (x_d - x_dp) * kd * iTd + dT_dde * a_phi1d * iTd);
    M.put(dp, c_id, -(x_d - x_dp) * (-(x_dp - x_ddp) * idpl + 1) * iTd);
    M.put(dp, c_edp, dT_dqe * b_edp * iTd);
    M.put(dp, c_phi2q, dT_dqe * b_phi2q * iTd);
    if (efd_idx >= 0) M.put(dp, efd_idx, iTd);
    M.put(dp + 1, c_edp, (-(x_q - x_qp) * kq - 1) * iTq);
    M.put(dp + 1, c_phi2q, -(x_q - x_qp) * kq * iTq);
    M.put(dp + 1, c_iq, (x_q - x_qp) * (-(x_qp - x_qdp) * iqpl + 1) * iTq);
    M.put(dp + 2, c_eqp, iTdd);
    M.put(dp + 2, c_phi1d, -iTdd);
    M.put(dp + 2, c_id, (-x_dp + xl) * iTdd);
    M.put(dp + 3, c_edp, -iTqd);
    M.put(dp + 3, c_phi2q, -iTqd);
    M.put(dp + 3, c_iq, (-x_qp + xl) * iTqd);
    M.put(dp + 4, c_eqp, -i_q * a_eqp * i2H);
    M.put(dp + 4, c_edp, i_d * b_edp * i2H);
    M.put(dp + 4, c_phi1d, -i_q * a_phi1d * i2H);
    M.put(dp + 4, c_phi2q, i_d * b_phi2q * i2H);
    M.put(dp + 4, c_w, -D * i2H);
    if (pm_idx >= 0) M.put(dp + 4, pm_idx, i2H);
    M.put(dp + 4, c_iq, -psi_de * i2H);
    M.put(dp + 4, c_id, psi_qe * i2H);
    M.put(dp + 5, c_w, kTwoPi60);
    M.put(ap, c_eqp, -a_eqp * ixd);
    M.put(ap, c_phi1d, -a_phi1d * ixd);
    M.put(ap, c_vq, ixd);
    M.put(ap, c_id, 1.0);
    M.put(ap + 1, c_edp, -b_edp * ixd);
    M.put(ap + 1, c_phi2q, -b_phi2q * ixd);
    M.put(ap + 1, c_vd, -ixd);
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

template <class Sink, class KP = ComputeK>
GP_HD void ieesgo_eval(const DevRef &d, const double *z, const double *p, Sink &M, const KP &kc = KP()) {
    const int dp = d.dp, ap = d.ap, pp = d.pp, wi = d.link0;
    const double T1 = p[pp], T2 = p[pp + 1], T3 = p[pp + 2], T4 = p[pp + 3], T5 = p[pp + 4], T6 = p[pp + 5];
    const double K1 = p[pp + 6], K2 = p[pp + 7], K3 = p[pp + 8], pref = p[pp + 11];
    const double PF0 = z[dp], PLL = z[dp + 1], TP1 = z[dp + 2], TP2 = z[dp + 3], TP3 = z[dp + 4], p_m = z[ap];
    const double w = wi < 0 ? 0.0 : z[wi];
    const double i1 = kc(16, [&] { return 1.0 / T1; }), i3 = kc(17, [&] { return 1.0 / T3; });
    const double i4 = kc(18, [&] { return 1.0 / T4; }), i5 = kc(19, [&] { return 1.0 / T5; });
    const double i6 = kc(20, [&] { return 1.0 / T6; }), r23 = kc(21, [&] { return T2 * i3; });
    M.putf(dp, i1 * (K1 * w - PF0));
    M.putf(dp + 1, i3 * ((1.0 - r23) * PF0 - PLL));
    const double SatP = pref - r23 * PF0 - PLL;
    M.putf(dp + 2, i4 * (SatP - TP1));
    M.putf(dp + 3, i5 * (K2 * TP1 - TP2));
    M.putf(dp + 4, i6 * (K3 * TP2 - TP3));
    M.putf(ap, TP1 * (1.0 - K2) + TP2 * (1.0 - K3) + TP3 - p_m);
    M.put(dp, dp, -i1);
    if (wi >= 0) M.put(dp, wi, K1 * i1);
    M.put(dp + 1, dp, (1.0 - r23) * i3);
    M.put(dp + 1, dp + 1, -i3);
    M.put(dp + 2, dp, -r23 * i4);
    M.put(dp + 2, dp + 1, -i4);
    M.put(dp + 2, dp + 2, -i4);
    M.put(dp + 3, dp + 2, K2 * i5);
    M.put(dp + 3, dp + 3, -i5);
    M.put(dp + 4, dp + 3, K3 * i6);
    M.put(dp + 4, dp + 4, -i6);
    M.put(ap, dp + 2, 1.0 - K2);
    M.put(ap, dp + 3, 1.0 - K3);
    M.put(ap, dp + 4, 1.0);
    M.put(ap, ap, -1.0);
}

template <class Sink, class KP = ComputeK>
GP_HD void tgov1_eval(const DevRef &d, const double *z, const double *p, Sink &M, const KP &kc = KP()) {
    const int dp = d.dp, ap = d.ap, pp = d.pp, wi = d.link0;
    const double R = p[pp], T1 = p[pp + 1], T2 = p[pp + 4], T3 = p[pp + 5], DT = p[pp + 6], pref = p[pp + 7];
    const double x1 = z[dp], x2 = z[dp + 1], p_m = z[ap];
    const double w = wi < 0 ? 0.0 : z[wi];
    const double i1 = kc(16, [&] { return 1.0 / T1; }), i3 = kc(17, [&] { return 1.0 / T3; });
    const double iR = kc(18, [&] { return 1.0 / R; }), r23 = kc(19, [&] { return T2 * i3; });
    M.putf(dp, (-x1 + (1.0 - r23) * x2) * i3);
    M.putf(dp + 1, ((pref - w) * iR - x2) * i1);
    M.putf(ap, x1 + r23 * x2 - DT * w - p_m);
    M.put(dp, dp, -i3);
    M.put(dp, dp + 1, (1.0 - r23) * i3);
    M.put(dp + 1, dp + 1, -i1);
    if (wi >= 0) M.put(dp + 1, wi, -iR * i1);
    M.put(ap, dp, 1.0);
    M.put(ap, dp + 1, r23);
    if (wi >= 0) M.put(ap, wi, -DT);
    M.put(ap, ap, -1.0);
}

template <class Sink, class KP = ComputeK>
GP_HD void sexs_eval(const DevRef &d, int net, const double *z, const double *p, Sink &M, const KP &kc = KP()) {
    const int dp = d.dp, pp = d.pp, vsi = d.link0;
    const int vr_idx = net + 2 * d.bus;
    const double TA_TB = p[pp], TB = p[pp + 1], K = p[pp + 2], TE = p[pp + 3], vref = p[pp + 6];
    const double x1 = z[dp], e_fd = z[dp + 1], vr = z[vr_idx], vi = z[vr_idx + 1];
    double vm = sqrt(vr * vr + vi * vi);
    vm = vm == 0.0 ? 1e-12 : vm;
    const double vs = vsi >= 0 ? z[vsi] : 0.0;
    const double err = vref - vm + vs;
    const double iTB = kc(22, [&] { return 1.0 / TB; }), iTE = kc(23, [&] { return 1.0 / TE; });
    M.putf(dp, (-x1 + (1.0 - TA_TB) * err) * iTB);
    M.putf(dp + 1, (-e_fd + K * (x1 + TA_TB * err)) * iTE);
    const double ivm = 1.0 / vm, dvr = vr * ivm, dvi = vi * ivm;
    M.put(dp, dp, -iTB);
    M.putv(dp, 0, -(1.0 - TA_TB) * dvr * iTB);
    M.putv(dp, 1, -(1.0 - TA_TB) * dvi * iTB);
    if (vsi >= 0) M.put(dp, vsi, (1.0 - TA_TB) * iTB);
    M.put(dp + 1, dp, K * iTE);
    M.put(dp + 1, dp + 1, -iTE);
    M.putv(dp + 1, 0, -K * TA_TB * dvr * iTE);
    M.putv(dp + 1, 1, -K * TA_TB * dvi * iTE);
    if (vsi >= 0) M.put(dp + 1, vsi, K * TA_TB * iTE);
}

template <class Sink, class KP = ComputeK>
GP_HD void esdc1a_eval(const DevRef &d, int net, const double *z, const double *p, Sink &M, const KP &kc = KP()) {
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
    const double iTa = kc(22, [&] { return 1.0 / Ta; }), iTf = kc(23, [&] { return 1.0 / Tf; });
    const double iTe = kc(24, [&] { return 1.0 / Te; }), kft = kc(25, [&] { return Kf * iTf; });
    M.putf(dp, (Ka * (vref - vm + vs - vr2 - kft * e_fd) - vr1) * iTa);
    M.putf(dp + 1, -(kft * e_fd + vr2) * iTf);
    M.putf(dp + 2, (vr1 - Ke * e_fd - sat) * iTe);
    const double ivm = 1.0 / vm, dvr = vr * ivm, dvi = vi * ivm;
    const double dsat = son ? 2.0 * sat_b * (e_fd - sat_a) : 0.0;
    M.put(dp, dp, -iTa);
    M.put(dp, dp + 1, -Ka * iTa);
    M.put(dp, dp + 2, -Ka * kft * iTa);
    M.putv(dp, 0, -Ka * dvr * iTa);
    M.putv(dp, 1, -Ka * dvi * iTa);
    if (vsi >= 0) M.put(dp, vsi, Ka * iTa);
    M.put(dp + 1, dp + 1, -iTf);
    M.put(dp + 1, dp + 2, -kft * iTf);
    M.put(dp + 2, dp, iTe);
    M.put(dp + 2, dp + 2, -(Ke + dsat) * iTe);
}

template <class Sink, class KP = ComputeK>
GP_HD void ieeest_eval(const DevRef &d, const double *z, const double *p, Sink &M, const KP &kc = KP()) {
    const int dp = d.dp, ap = d.ap, pp = d.pp, wi = d.link0;
    const double A1 = p[pp], A2 = p[pp + 1], A3 = p[pp + 2], A4 = p[pp + 3], A5 = p[pp + 4], A6 = p[pp + 5];
    const double T1 = p[pp + 6], T2 = p[pp + 7], T3 = p[pp + 8], T4 = p[pp + 9], T5 = p[pp + 10], T6 = p[pp + 11],
                 KS = p[pp + 12];
    const double s0 = z[dp], s1 = z[dp + 1], s2 = z[dp + 2], s3 = z[dp + 3], s4 = z[dp + 4], s5 = z[dp + 5],
                 s6 = z[dp + 6], vs = z[ap];
    const double sig = wi >= 0 ? z[wi] : 0.0;
    const double iA2 = kc(26, [&] { return 1.0 / A2; }), iA4 = kc(27, [&] { return 1.0 / A4; });
    const double iT2 = kc(28, [&] { return 1.0 / T2; }), iT4 = kc(29, [&] { return 1.0 / T4; });
    const double iT6 = kc(30, [&] { return 1.0 / T6; }), rA = kc(31, [&] { return A6 * iA4; });
    const double r12 = kc(32, [&] { return T1 * iT2; }), r34 = kc(33, [&] { return T3 * iT4; });
    const double r56 = kc(34, [&] { return T5 * iT6; });
    const double q = s1 - s3 - A3 * s2;
    const double y2 = s3 + A5 * s2 + rA * q;
    const double y3 = s4 + r12 * (y2 - s4);
    const double y4 = s5 + r34 * (y3 - s5);
    M.putf(dp, (sig - s1 - A1 * s0) * iA2);
    M.putf(dp + 1, s0);
    M.putf(dp + 2, (s1 - s3 - A3 * s2) * iA4);
    M.putf(dp + 3, s2);
    M.putf(dp + 4, (y2 - s4) * iT2);
    M.putf(dp + 5, (y3 - s5) * iT4);
    M.putf(dp + 6, (KS * y4 - s6) * iT6);
    M.putf(ap, vs - r56 * (KS * y4 - s6));
    const double d20 = rA, d21 = A5 - A3 * rA, d22 = 1.0 - rA;
    const double d30 = r12 * d20, d31 = r12 * d21, d32 = r12 * d22, d33 = 1.0 - r12;
    const double d40 = r34 * d30, d41 = r34 * d31, d42 = r34 * d32, d43 = r34 * d33, d44 = 1.0 - r34;
    M.put(dp, dp, -A1 * iA2);
    M.put(dp, dp + 1, -iA2);
    if (wi >= 0) M.put(dp, wi, iA2);
    M.put(dp + 1, dp, 1.0);
    M.put(dp + 2, dp + 1, iA4);
    M.put(dp + 2, dp + 2, -A3 * iA4);
    M.put(dp + 2, dp + 3, -iA4);
    M.put(dp + 3, dp + 2, 1.0);
    M.put(dp + 4, dp + 1, d20 * iT2);
    M.put(dp + 4, dp + 2, d21 * iT2);
    M.put(dp + 4, dp + 3, d22 * iT2);
    M.put(dp + 4, dp + 4, -iT2);
    M.put(dp + 5, dp + 1, d30 * iT4);
    M.put(dp + 5, dp + 2, d31 * iT4);
    M.put(dp + 5, dp + 3, d32 * iT4);
    M.put(dp + 5, dp + 4, d33 * iT4);
    M.put(dp + 5, dp + 5, -iT4);
    M.put(dp + 6, dp + 1, KS * d40 * iT6);
    M.put(dp + 6, dp + 2, KS * d41 * iT6);
    M.put(dp + 6, dp + 3, KS * d42 * iT6);
    M.put(dp + 6, dp + 4, KS * d43 * iT6);
    M.put(dp + 6, dp + 5, KS * d44 * iT6);
    M.put(dp + 6, dp + 6, -iT6);
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
