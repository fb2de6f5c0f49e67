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
//  update_kernel   z += dz: network and static-generator unknowns from the
//                  solve, cluster states by back-substitution
//                  dw_k = -(A_k^-1 f_k + A_k^-1 B_k dv) (src/schur.jl:383-409).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "gp_devices.cuh"
#include "gp_internal.h"
#include "gp_warp.cuh"

namespace gp {

#define FULL_MASK 0xffffffffu

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long norm_bits(double v) {
    // the bit pattern of |v| (non-negative doubles order like their bit
    // patterns); NaN counts as +inf.  Integer operations only: the FP64
    // pipe is the scarce one on this GPU.
    const unsigned long long a = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return a > 0x7ff0000000000000ull ? 0x7ff0000000000000ull : a;
}

// ---------------------------------------------------------------------------
// cluster kernel: one lane per (cluster, scenario), 32 clusters of one
// pattern class per warp; the class program does the backward-Euler scaling,
// the static-pivot sparse LU and the solves for [B(:,vr) B(:,vi) f].
// ---------------------------------------------------------------------------

struct LaneSink {
    double *v;             // vals[slot * 32 + lane]
    const short *slot_of;  // class map, local (r, c) -> slot
    int ws, lane;
    __device__ __forceinline__ void put(int r, int c, double x) {
        v[(int)slot_of[(r - ws) * 32 + (c - ws)] * 32 + lane] = x;
    }
    __device__ __forceinline__ void putv(int r, int k, double x) {
        v[(int)slot_of[(r - ws) * 32 + 29 + k] * 32 + lane] = x;
    }
    __device__ __forceinline__ void putf(int r, double x) { v[(int)slot_of[(r - ws) * 32 + 31] * 32 + lane] = x; }
};

__device__ __forceinline__ DevRef devref(const DTab &T, int k) {
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

// The cluster's device table entries are read first, all together, so that
// their round trips overlap instead of each device's starting after the
// previous device's equations.
template <class Sink, class KP = ComputeK>
__device__ __forceinline__ void eval_cluster(const DevProblem &P, int c, const double *z, const double *u0,
                                             const double *p, Sink &sink, double Cc[6], double Ic[2],
                                             const KP &kc = KP(), bool exc_on = true) {
    const int gt = P.cl_gov_type[c], et0 = P.cl_exc_type[c], ip = P.cl_pss[c];
    const int ig = P.cl_gen[c], igv = P.cl_gov[c], iex = P.cl_exc[c];
    const int et = exc_on ? et0 : -1;   // an offline exciter's states hold
    const DevRef dg = devref(P.dev[0], ig);
    DevRef dgv{}, dex{}, dps{};
    if (gt == 1 || gt == 2) dgv = devref(P.dev[gt], igv);
    if (et == 3 || et == 4) dex = devref(P.dev[et], iex);
    if (ip >= 0) dps = devref(P.dev[5], ip);
    genrou_eval(dg, P.net, z, u0, p, sink, Cc, Ic, kc);
    if (gt == 1) ieesgo_eval(dgv, z, p, sink, kc);
    else if (gt == 2) tgov1_eval(dgv, z, p, sink, kc);
    if (et == 3) sexs_eval(dex, P.net, z, p, sink, kc);
    else if (et == 4) esdc1a_eval(dex, P.net, z, p, sink, kc);
    if (ip >= 0) ieeest_eval(dps, z, p, sink, kc);
}

// Sink that drops every entry (the evaluation of the parameter constants).
struct NullSink {
    __device__ __forceinline__ void put(int, int, double) {}
    __device__ __forceinline__ void putv(int, int, double) {}
    __device__ __forceinline__ void putf(int, double) {}
};

// Parameter constants of every cluster's devices for every scenario, stored
// for cluster_keep_kernel (they depend on the parameters alone; run once per
// integration, after the parameters are set).
__global__ void __launch_bounds__(32) cluster_const_kernel(DevProblem P, DevWork W, DevClu Cl, DevMixed Mx) {
    const int task = blockIdx.x, m = blockIdx.y, lane = threadIdx.x;
    if (lane >= Cl.task_count[task]) return;
    const int c = Cl.order[Cl.task_first[task] + lane];
    const double *z = W.z + (size_t)m * P.n_sys;
    double Cc[6], Ic[2];
    NullSink sink;
    RecordK rk{Mx.kc + (((size_t)m * Cl.n_tasks + task) * kConstSlots) * 32 + lane, 32};
    eval_cluster(P, c, z, W.u0 + (size_t)m * P.n_ctrl, W.p + (size_t)m * P.n_par, sink, Cc, Ic, rk);
}

// The factorisation part of a class program and the solves of the three
// right-hand-side columns R0, R1 (B) and R2 (f), on one lane's slots.
template <class T>
__device__ __forceinline__ void clu_program(T *vals, T *R0, T *R1, T *R2, const CluOp *ops, int qm, int q1,
                                            int lane) {
    for (int q = qm; q < q1; q++) {
        const CluOp o = ops[q];
        switch (o.code) {
        case OP_RCP:
            vals[o.d * 32 + lane] = recip(vals[o.a * 32 + lane]);
            break;
        case OP_MUL:
            vals[o.d * 32 + lane] *= vals[o.a * 32 + lane];
            break;
        case OP_FMS:
            vals[o.d * 32 + lane] -= vals[o.a * 32 + lane] * vals[o.b * 32 + lane];
            break;
        case OP_FMS3: {
            const T l = vals[o.a * 32 + lane];
            R0[o.d * 32 + lane] -= l * R0[o.b * 32 + lane];
            R1[o.d * 32 + lane] -= l * R1[o.b * 32 + lane];
            R2[o.d * 32 + lane] -= l * R2[o.b * 32 + lane];
            break;
        }
        case OP_MUL3: {
            const T l = vals[o.a * 32 + lane];
            R0[o.d * 32 + lane] *= l;
            R1[o.d * 32 + lane] *= l;
            R2[o.d * 32 + lane] *= l;
            break;
        }
        default:
            break;
        }
    }
}

// Modes per scenario: 0 exact Newton (Jacobian block, FP64 LU, three solves;
// also the mixed solver's MX_EXACT); 1 the same, and the LU values and
// coupling rows are kept in FP32 for the following iterations (MX_FP32).
// The mixed solver's MX_KEEP scenarios (residual only, solved with the kept
// FP32 LU) run cluster_keep_kernel instead.
__global__ void __launch_bounds__(32) cluster_kernel(DevProblem P, DevWork W, DevClu Cl, DevMixed Mx, int want_f) {
    extern __shared__ double vals[];
    const int task = blockIdx.x, m = blockIdx.y, lane = threadIdx.x;
    if (!W.active[m]) return;
    const int r = Mx.on ? Mx.refac[m] : MX_EXACT;
    if (r == MX_KEEP) return;
    const int mode = r == MX_FP32 ? 1 : 0;
    const int cls = Cl.task_class[task];
    const int cnt = Cl.task_count[task];
    const bool act = lane < cnt;
    const int c = act ? Cl.order[Cl.task_first[task] + lane] : Cl.order[Cl.task_first[task]];
    const int ws = P.cl_w_start[c], Wn = P.cl_w_size[c];
    const int nslot = Cl.nslot[cls];
    for (int s = 0; s < nslot; s++) vals[s * 32 + lane] = 0.0;
    const double *z = W.z + (size_t)m * P.n_sys;
    const double *zold = W.zold + (size_t)m * P.n_sys;
    const double *u0 = W.u0 + (size_t)m * P.n_ctrl;
    const double *p = W.p + (size_t)m * P.n_par;
    double Cc[6] = {0, 0, 0, 0, 0, 0}, Ic[2] = {0, 0};
    const CluOp *ops = Cl.ops;
    const int q0 = Cl.prog_ptr[cls], qm = Cl.prog_mid[cls], q1 = Cl.prog_ptr[cls + 1];
    if (act) {
        LaneSink sink{vals, Cl.slot_of + (size_t)cls * 1024, ws, lane};
        eval_cluster(P, c, z, u0, p, sink, Cc, Ic, ComputeK(), !P.exc_off || !P.exc_off[(size_t)m * P.n_cl + c]);
    } else {
        // idle lanes factor an identity so that no lane divides by zero
        for (int q = qm; q < q1; q++)
            if (ops[q].code == OP_RCP) vals[ops[q].a * 32 + lane] = 1.0;
    }
    const double dt = *W.dt;
    const int rb = Cl.rhs_base[cls];
    double *R0 = vals + (size_t)rb * 32, *R1 = R0 + (size_t)Wn * 32, *R2 = R1 + (size_t)Wn * 32;
    // backward-Euler scaling, eight ops and their state loads in flight
    for (int q = q0; q < qm; q += 8) {
        CluOp o[8];
        double zn[8], zo[8];
#pragma unroll
        for (int u = 0; u < 8; u++) o[u] = ops[min(q + u, qm - 1)];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const bool ld = act && q + u < qm && o[u].code == OP_BEF;
            zn[u] = ld ? z[ws + o[u].a] : 0.0;
            zo[u] = ld ? zold[ws + o[u].a] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (q + u >= qm) break;
            double *vd = vals + o[u].d * 32 + lane;
            if (o[u].code == OP_SCL) *vd *= -dt;
            else if (o[u].code == OP_DIAG) *vd += 1.0;
            else if (o[u].code == OP_BEF) *vd = act ? zn[u] - zo[u] - dt * *vd : 0.0;
        }
    }
    // residual norm (and the residual itself for the parity probe)
    const int *pc = Cl.perm_col + cls * 32;
    unsigned long long nb = 0ull;
    for (int j = 0; j < Wn; j++) {
        const unsigned long long t = norm_bits(R2[j * 32 + lane]);
        nb = t > nb ? t : nb;
    }
    if (!act) nb = 0ull;
    if (want_f && act) {
        // R2 is indexed by pivot position; OP_BEF / OP_ROW name the local row
        // whose residual each position holds
        for (int q = q0; q < qm; q++)
            if (ops[q].code == OP_BEF || ops[q].code == OP_ROW)
                W.f[(size_t)m * P.n_sys + ws + ops[q].a] = vals[ops[q].d * 32 + lane];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(FULL_MASK, nb, off);
        nb = o > nb ? o : nb;
    }
    if (lane == 0) atomicMax(W.norm + m, nb);
    float *keep = Mx.on ? Mx.lu + (((size_t)m * Cl.n_tasks + task) * Mx.n_lu) * 32 + lane : nullptr;
    const int n_da = P.n_diff + P.n_alg;
    double *yx = W.yx + (size_t)m * 3 * n_da + ws;
    const int *p3 = Cl.pos3 + cls * 3;
    double X0[3], X1[3], X2[3];
    if (mode == 1) {
        // MX_FP32: the factors are kept in FP32, so the factorisation and
        // the three solves run in FP32 too.  The slots are converted in place:
        // float slot s lies in the first half of double slot s / 2, which was
        // read before (each slot is read into registers before the warp
        // writes over it).
        float *fv = reinterpret_cast<float *>(vals);
        for (int s = 0; s < nslot; s++) {
            const float x = (float)vals[s * 32 + lane];
            __syncwarp();
            fv[s * 32 + lane] = x;
            __syncwarp();
        }
        float *F0 = fv + (size_t)rb * 32, *F1 = F0 + (size_t)Wn * 32, *F2 = F1 + (size_t)Wn * 32;
        clu_program<float>(fv, F0, F1, F2, ops, qm, q1, lane);
        for (int s = 0; s < rb; s++) keep[s * 32] = fv[s * 32 + lane];
        if (!act) return;
        for (int j = 0; j < Wn; j++) {
            const int st = pc[j];
            yx[st] = (double)F2[j * 32 + lane];
            yx[n_da + st] = (double)F0[j * 32 + lane];
            yx[2 * n_da + st] = (double)F1[j * 32 + lane];
        }
#pragma unroll
        for (int t = 0; t < 3; t++) {
            X0[t] = (double)F2[p3[t] * 32 + lane];
            X1[t] = (double)F0[p3[t] * 32 + lane];
            X2[t] = (double)F1[p3[t] * 32 + lane];
        }
    } else {
        // factorisation and solves in FP64
        clu_program<double>(vals, R0, R1, R2, ops, qm, q1, lane);
        if (Cl.save_lu) {
            double *sv = Cl.save_lu + (((size_t)m * Cl.n_tasks + task) * Cl.n_save) * 32 + lane;
            for (int s = 0; s < rb; s++) sv[s * 32] = vals[s * 32 + lane];
        }
        if (!act) return;
        for (int j = 0; j < Wn; j++) {
            const int st = pc[j];
            yx[st] = R2[j * 32 + lane];
            yx[n_da + st] = R0[j * 32 + lane];
            yx[2 * n_da + st] = R1[j * 32 + lane];
        }
#pragma unroll
        for (int t = 0; t < 3; t++) {
            X0[t] = R2[p3[t] * 32 + lane];
            X1[t] = R0[p3[t] * 32 + lane];
            X2[t] = R1[p3[t] * 32 + lane];
        }
    }
    double *o = W.clout + ((size_t)m * P.n_cl + c) * 8;
    o[0] = Cc[0] * X1[0] + Cc[1] * X1[1] + Cc[2] * X1[2];
    o[1] = Cc[0] * X2[0] + Cc[1] * X2[1] + Cc[2] * X2[2];
    o[2] = Cc[3] * X1[0] + Cc[4] * X1[1] + Cc[5] * X1[2];
    o[3] = Cc[3] * X2[0] + Cc[4] * X2[1] + Cc[5] * X2[2];
    o[4] = Cc[0] * X0[0] + Cc[1] * X0[1] + Cc[2] * X0[2];
    o[5] = Cc[3] * X0[0] + Cc[4] * X0[1] + Cc[5] * X0[2];
    o[6] = Ic[0];
    o[7] = Ic[1];
    if (mode == 1) {
        float *cc = Mx.cc + ((size_t)m * P.n_cl + c) * 6;
        for (int t = 0; t < 6; t++) cc[t] = (float)Cc[t];
    }
    if (Cl.save_cc) {
        double *cc = Cl.save_cc + ((size_t)m * P.n_cl + c) * 6;
        for (int t = 0; t < 6; t++) cc[t] = Cc[t];
    }
}

// Sink of a residual-only evaluation: Jacobian entries are dropped (the
// compiler removes their arithmetic), residuals go to their positions in the
// staged residual column.
struct KeepSink {
    double *v;
    const short *slot_of;
    int ws, lane, base;
    __device__ __forceinline__ void put(int, int, double) {}
    __device__ __forceinline__ void putv(int, int, double) {}
    __device__ __forceinline__ void putf(int r, double x) {
        v[((int)slot_of[(r - ws) * 32 + 31] - base) * 32 + lane] = x;
    }
};

// MX_KEEP scenarios of the mixed solver: the FP64 residual and its solve
// with the kept FP32 LU, nothing else.  Only the residual column is staged in
// shared memory (W values per lane instead of the whole program's slots), the
// LU values are read straight from the kept copy, and the op list is the
// solve part of the program alone, so many more warps fit on an SM.  The
// solve runs in FP32, like the kept LU it applies: FP64 arithmetic and
// FP32<->FP64 conversions are scarce on this GPU, and the correction of an
// iteration on kept factors is inexact at the FP32 level anyway (the residual
// that drives it stays FP64).
__global__ void __launch_bounds__(32, 16) cluster_keep_kernel(DevProblem P, DevWork W, DevClu Cl, DevMixed Mx,
                                                             int want_f) {
    extern __shared__ double R2[];   // [max_w][32] FP64 residual by pivot position, then [max_w][32] FP32
    float *Rf = reinterpret_cast<float *>(R2 + (size_t)Cl.max_w * 32);
    const int task = blockIdx.x, m = blockIdx.y, lane = threadIdx.x;
    if (!W.active[m] || Mx.refac[m] != MX_KEEP) return;
    const int cls = Cl.task_class[task];
    const int cnt = Cl.task_count[task];
    const bool act = lane < cnt;
    const int c = act ? Cl.order[Cl.task_first[task] + lane] : Cl.order[Cl.task_first[task]];
    const int ws = P.cl_w_start[c], Wn = P.cl_w_size[c];
    const int rb = Cl.rhs_base[cls], base = rb + 2 * Wn;
    for (int j = 0; j < Wn; j++) R2[j * 32 + lane] = 0.0;
    const double *z = W.z + (size_t)m * P.n_sys;
    const double *zold = W.zold + (size_t)m * P.n_sys;
    double Cc[6] = {0, 0, 0, 0, 0, 0}, Ic[2] = {0, 0};
    if (act) {
        KeepSink sink{R2, Cl.slot_of + (size_t)cls * 1024, ws, lane, base};
        LoadK lk{Mx.kc + (((size_t)m * Cl.n_tasks + task) * kConstSlots) * 32 + lane, 32};
        eval_cluster(P, c, z, W.u0 + (size_t)m * P.n_ctrl, W.p + (size_t)m * P.n_par, sink, Cc, Ic, lk,
                     !P.exc_off || !P.exc_off[(size_t)m * P.n_cl + c]);
    }
    const double dt = *W.dt;
    const CluOp *ops = Cl.ops;
    const int q0 = Cl.prog_ptr[cls], qm = Cl.prog_mid[cls], qs = Cl.prog_sol[cls], q1 = Cl.prog_ptr[cls + 1];
    // backward-Euler rows, eight ops and their state loads in flight
    for (int q = q0; q < qm; q += 8) {
        CluOp o[8];
        double zn[8], zo[8];
#pragma unroll
        for (int u = 0; u < 8; u++) o[u] = ops[min(q + u, qm - 1)];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const bool ld = act && q + u < qm && o[u].code == OP_BEF;
            zn[u] = ld ? z[ws + o[u].a] : 0.0;
            zo[u] = ld ? zold[ws + o[u].a] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (q + u < qm && o[u].code == OP_BEF) {
                double *vd = R2 + (o[u].d - base) * 32 + lane;
                *vd = act ? zn[u] - zo[u] - dt * *vd : 0.0;
            }
    }
    unsigned long long nb = 0ull;
    for (int j = 0; j < Wn; j++) {
        const unsigned long long t = norm_bits(R2[j * 32 + lane]);
        nb = t > nb ? t : nb;
    }
    if (!act) nb = 0ull;
    if (want_f && act) {
        for (int q = q0; q < qm; q++)
            if (ops[q].code == OP_BEF || ops[q].code == OP_ROW)
                W.f[(size_t)m * P.n_sys + ws + ops[q].a] = R2[(ops[q].d - base) * 32 + lane];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(FULL_MASK, nb, off);
        nb = o > nb ? o : nb;
    }
    if (lane == 0) atomicMax(W.norm + m, nb);
    for (int j = 0; j < Wn; j++) Rf[j * 32 + lane] = (float)R2[j * 32 + lane];
    // the solves (OP_FMS3 / OP_MUL3 on the residual column), eight ops and
    // their LU values loaded ahead of the arithmetic
    const float *kl = Mx.lu + (((size_t)m * Cl.n_tasks + task) * Mx.n_lu) * 32 + lane;
    constexpr int kAhead = 8;
    for (int q = qs; q < q1; q += kAhead) {
        CluOp o[kAhead];
        float l[kAhead];
#pragma unroll
        for (int u = 0; u < kAhead; u++) {
            o[u] = ops[min(q + u, q1 - 1)];
            l[u] = kl[o[u].a * 32];
        }
#pragma unroll
        for (int u = 0; u < kAhead; u++) {
            if (q + u >= q1) break;
            if (o[u].code == OP_FMS3) Rf[o[u].d * 32 + lane] = fmaf(-l[u], Rf[o[u].b * 32 + lane], Rf[o[u].d * 32 + lane]);
            else Rf[o[u].d * 32 + lane] *= l[u];
        }
    }
    if (!act) return;
    const int n_da = P.n_diff + P.n_alg;
    double *yx = W.yx + (size_t)m * 3 * n_da + ws;
    const int *pc = Cl.perm_col + cls * 32;
    const int *p3 = Cl.pos3 + cls * 3;
    for (int j = 0; j < Wn; j++) yx[pc[j]] = (double)Rf[j * 32 + lane];
    const float Y0 = Rf[p3[0] * 32 + lane], Y1 = Rf[p3[1] * 32 + lane], Y2 = Rf[p3[2] * 32 + lane];
    const float *cc = Mx.cc + ((size_t)m * P.n_cl + c) * 6;
    double *o = W.clout + ((size_t)m * P.n_cl + c) * 8;
    o[4] = (double)fmaf(cc[2], Y2, fmaf(cc[1], Y1, cc[0] * Y0));
    o[5] = (double)fmaf(cc[5], Y2, fmaf(cc[4], Y1, cc[3] * Y0));
    o[6] = Ic[0];
    o[7] = Ic[1];
}

int launch_cluster(const DevProblem &P, const DevWork &W, const DevClu &C, const DevMixed &Mx, int want_f,
                   cudaStream_t st) {
    if (C.n_tasks == 0) return 0;
    dim3 grid(C.n_tasks, P.M);
    cluster_kernel<<<grid, 32, (size_t)C.max_slots * 32 * sizeof(double), st>>>(P, W, C, Mx, want_f);
    if (!Mx.on) return 1;
    cluster_keep_kernel<<<grid, 32, (size_t)C.max_w * 32 * (sizeof(double) + sizeof(float)), st>>>(P, W, C, Mx,
                                                                                                  want_f);
    return 2;
}

// Parameter products of every ZIP load per scenario for network_kernel:
// (1 - al) P, (1 - al) Q, al g0, al b0.
__global__ void zip_const_kernel(DevProblem P, DevWork W, double *out) {
    const DTab &ZL = P.dev[6];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.M * ZL.n) return;
    const int m = (int)(t / ZL.n), k = (int)(t % ZL.n);
    const double *p = W.p + (size_t)m * P.n_par + ZL.par_ptr[k];
    const double al = p[2];
    double *o = out + (size_t)t * 4;
    o[0] = (1.0 - al) * p[0];
    o[1] = (1.0 - al) * p[1];
    o[2] = al * p[7];
    o[3] = al * p[8];
}

void launch_zip_const(const DevProblem &P, const DevWork &W, double *out, cudaStream_t st) {
    const long long n = (long long)P.M * P.dev[6].n;
    if (n > 0) zip_const_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(P, W, out);
}

void launch_cluster_const(const DevProblem &P, const DevWork &W, const DevClu &C, const DevMixed &Mx,
                          cudaStream_t st) {
    if (C.n_tasks == 0) return;
    cluster_const_kernel<<<dim3(C.n_tasks, P.M), 32, 0, st>>>(P, W, C, Mx);
}

int cluster_smem_optin(int bytes) {
    if (cudaFuncSetAttribute(cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return bytes;
}

// ---------------------------------------------------------------------------
// network kernel
// ---------------------------------------------------------------------------

// With the mixed solver, a scenario iterating on kept factors needs only the
// residual and the right-hand side: the entries of S (diagonal blocks,
// static-generator couplings) are skipped for it.
__global__ void __launch_bounds__(64) network_kernel(DevProblem P, DevWork W, DevMixed Mx, int want_f,
                                                      int skip_s) {
    const long long task = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = task < (long long)P.M * P.n_bus;
    const int m = valid ? (int)(task / P.n_bus) : P.M;
    // buses in the order of their work (devices, then Ybus row length), so
    // that the lanes of a warp run the same loop trip counts
    const int b = valid ? P.bus_order[(int)(task % P.n_bus)] : 0;
    const bool act = valid && W.active[m];
    unsigned long long nb = 0ull;
    if (act) {
        const bool need_s = !skip_s && !(Mx.on && Mx.refac[m] == MX_KEEP);
        const double *z = W.z + (size_t)m * P.n_sys;
        const double *p = W.p + (size_t)m * P.n_par;
        const int net = P.net;
        const double vr = z[net + 2 * b], vi = z[net + 2 * b + 1];
        double fr = 0.0, fi = 0.0, d00 = 0.0, d01 = 0.0, d10 = 0.0, d11 = 0.0, rr = 0.0, ri = 0.0;
        for (int q = P.y_rowptr[b]; q < P.y_rowptr[b + 1]; q++) {
            const int j = P.y_colidx[q];
            const double2 y = P.y_val[q];   // one 16-byte load
            const double g = y.x, bb = y.y;
            const double vrj = z[net + 2 * j], vij = z[net + 2 * j + 1];
            // -(g + j bb)(vrj + j vij), two FMAs per part
            fr = fma(-g, vrj, fma(bb, vij, fr));
            fi = fma(-bb, vrj, fma(-g, vij, fi));
            if (need_s && j == b) { d00 -= g; d01 += bb; d10 -= bb; d11 -= g; }
        }
        for (int q = P.bus_cl_ptr[b]; q < P.bus_cl_ptr[b + 1]; q++) {
            const double *o = W.clout + ((size_t)m * P.n_cl + P.bus_cl[q]) * 8;
            if (need_s) { d00 -= o[0]; d01 -= o[1]; d10 -= o[2]; d11 -= o[3]; }
            rr += o[4]; ri += o[5];
            fr += o[6]; fi += o[7];
        }
        const DTab &ZL = P.dev[6];
        for (int q = P.bus_zl_ptr[b]; q < P.bus_zl_ptr[b + 1]; q++) {
            const int k = P.bus_zl[q];
            if (P.zl_off && P.zl_off[(size_t)m * ZL.n + k]) continue;
            // the load's parameter products ((1 - al) P, (1 - al) Q, al y0),
            // from the table zip_const_kernel fills once per call
            const double *kz = P.zl_k + ((size_t)m * ZL.n + k) * 4;
            const double A1 = kz[0], A2 = kz[1], B1 = kz[2], B2 = kz[3];
            const double vm2 = vr * vr + vi * vi, vm2_tld = 0.2;
            const bool above = vm2 > vm2_tld;
            // one division per load (FP64 division is dear here)
            const double inv = 1.0 / (above ? vm2 : vm2_tld);
            // the constant-impedance part al*y0 and the constant-power part
            // (1 - al)(P - jQ)/max(|V|^2, 0.2) multiply the same V: one
            // complex admittance a + jc; f -= (a + jc) V in FMA form
            const double a = fma(inv, A1, B1), c = fma(inv, A2, B2);
            fr = fma(vi, c, fma(-vr, a, fr));
            fi = fma(-vi, a, fma(-vr, c, fi));
            if (!need_s) continue;
            double p11, p12, p21, p22;
            if (above) {
                const double iv4 = inv * inv;
                p11 = ((A1 * vr - A2 * vi) * 2.0 * vr - A1 * vm2) * iv4;
                p12 = ((A1 * vr - A2 * vi) * 2.0 * vi + A2 * vm2) * iv4;
                p21 = ((A2 * vr + A1 * vi) * 2.0 * vr - A2 * vm2) * iv4;
                p22 = ((A2 * vr + A1 * vi) * 2.0 * vi - A1 * vm2) * iv4;
            } else {
                p11 = -A1 * inv;
                p12 = A2 * inv;
                p21 = -A2 * inv;
                p22 = -A1 * inv;
            }
            d00 += -B1 + p11;
            d01 += B2 + p12;
            d10 += -B2 + p21;
            d11 += -B1 + p22;
        }
        const DTab &SG = P.dev[7];
        for (int q = P.bus_sg_ptr[b]; q < P.bus_sg_ptr[b + 1]; q++) {
            const int k = P.bus_sg[q];
            if (P.sg_off && P.sg_off[(size_t)m * SG.n + k]) continue;   // constant-power ones only
            const int pp = SG.par_ptr[k], ap = SG.alg_ptr[k], bt = SG.link0[k];
            const double vm2r = vr * vr + vi * vi, vm2 = vm2r > 0.2 ? vm2r : 0.2;
            double Pg, Qg;
            if (bt == 2) { Pg = p[pp]; Qg = z[ap]; }
            else if (bt == 3) { Pg = z[ap]; Qg = z[ap + 1]; }
            else { Pg = p[pp]; Qg = p[pp + 1]; }
            const double irn = Pg * vr + Qg * vi, iin = Pg * vi - Qg * vr;
            const double inv = 1.0 / vm2;
            fr += irn * inv;
            fi += iin * inv;
            if (!need_s) {
                double *xp = W.xperm + (size_t)m * P.n_red;
                const int r0 = P.sg_red[k];
                if (bt == 2) {
                    const double vset = p[pp + 2];
                    const double fa = vr * vr + vi * vi - vset * vset;
                    xp[P.iperm[r0]] = -fa;
                    if (want_f) W.f[(size_t)m * P.n_sys + ap] = fa;
                    const unsigned long long t = norm_bits(fa);
                    nb = t > nb ? t : nb;
                } else if (bt == 3) {
                    const double vset = p[pp + 2], aset = p[pp + 3];
                    const double fa0 = vr - vset * cos(aset), fa1 = vi - vset * sin(aset);
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
                continue;
            }
            if (vm2r > 0.2) {
                const double iv4 = inv * inv;
                d00 += Pg * inv - 2.0 * vr * irn * iv4;
                d01 += Qg * inv - 2.0 * vi * irn * iv4;
                d10 += -Qg * inv - 2.0 * vr * iin * iv4;
                d11 += Pg * inv - 2.0 * vi * iin * iv4;
            } else {
                d00 += Pg * inv;
                d01 += Qg * inv;
                d10 += -Qg * inv;
                d11 += Pg * inv;
            }
            double *sv = W.svar + (size_t)m * P.n_var + P.sg_var[k];
            double *xp = W.xperm + (size_t)m * P.n_red;
            const int r0 = P.sg_red[k];
            if (bt == 2) {
                const double vset = p[pp + 2];
                const double fa = vr * vr + vi * vi - vset * vset;
                // (ap,vr) (ap,vi) (vr,ap) (vi,ap)
                sv[0] = 2.0 * vr; sv[1] = 2.0 * vi; sv[2] = vi * inv; sv[3] = -vr * inv;
                xp[P.iperm[r0]] = -fa;
                if (want_f) W.f[(size_t)m * P.n_sys + ap] = fa;
                const unsigned long long t = norm_bits(fa);
                nb = t > nb ? t : nb;
            } else if (bt == 3) {
                const double vset = p[pp + 2], aset = p[pp + 3];
                const double fa0 = vr - vset * cos(aset), fa1 = vi - vset * sin(aset);
                // (ap,vr) (ap+1,vi) (vr,ap) (vi,ap) (vr,ap+1) (vi,ap+1)
                sv[0] = 1.0; sv[1] = 1.0; sv[2] = vr * inv; sv[3] = vi * inv; sv[4] = vi * inv; sv[5] = -vr * inv;
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
        // tripped lines: their Ybus terms removed (f = -Y V gains
        // +y_line V; the S diagonal block gains the realified y_line)
        for (int e = P.tr_ptr[m]; e < P.tr_ptr[m + 1]; e++) {
            if (!P.tr_on[e]) continue;
            const int fb = P.tr_from[e], tb = P.tr_to[e];
            if (fb != b && tb != b) continue;
            const double *y = P.tr_y + 8 * (size_t)e + (fb == b ? 0 : 4);   // (yff, yft) or (ytf, ytt)
            const double ybr = fb == b ? y[0] : y[2], ybi = fb == b ? y[1] : y[3];
            const double yor = fb == b ? y[2] : y[0], yoi = fb == b ? y[3] : y[1];
            const int o = fb == b ? tb : fb;
            const double vro = z[net + 2 * o], vio = z[net + 2 * o + 1];
            fr += ybr * vr - ybi * vi + yor * vro - yoi * vio;
            fi += ybi * vr + ybr * vi + yoi * vro + yor * vio;
            if (need_s) { d00 += ybr; d01 -= ybi; d10 += ybi; d11 += ybr; }
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
        if (need_s) {
            double *sv = W.svar + (size_t)m * P.n_var + 4 * b;
            sv[0] = d00; sv[1] = d01; sv[2] = d10; sv[3] = d11;
        }
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

void launch_network(const DevProblem &P, const DevWork &W, const DevMixed &Mx, int want_f, cudaStream_t st,
                    int skip_s) {
    // 64-thread blocks: the buses' work differs (devices, row lengths), and
    // small blocks retire and refill the SMs evenly (network phase 9.45 ->
    // 9.0 ms over 0.3 s of the 70k-bus workload against 256-thread blocks;
    // 128: 9.17, 32: 8.97)
    long long tasks = (long long)P.M * P.n_bus;
    int blocks = (int)((tasks + 63) / 64);
    network_kernel<<<blocks, 64, 0, st>>>(P, W, Mx, want_f, skip_s);
}

// ---------------------------------------------------------------------------
// shared-factor Woodbury path
// ---------------------------------------------------------------------------
// The reduced matrix P (scenario 0 at the call's initial state, no fault) is
// factored once per call and shared by every scenario and iteration.  A
// scenario's fault (bus b, admittance yf) subtracts yf from the two
// diagonal entries of its bus: S_m = P - yf U U^T with U = [e_vr e_vi], and
// by the Woodbury identity S_m^-1 r = x - W H^-1 U^T x, x = P^-1 r,
// W = P^-1 U, H = U^T W - I / yf (integrate_gpu_shared_multi!,
// ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2441-2489, 2560-2574; every
// scenario of the table has one fault bus and admittance, checked by the
// host).

// The scenario's fault: its first table entry (-1: none); *on when one of
// its windows is on.
__device__ __forceinline__ int wb_fault(const DevProblem &P, int m, bool *on) {
    const int e0 = P.fl_ptr[m], e1 = P.fl_ptr[m + 1];
    bool any = false;
    for (int e = e0; e < e1; e++) any = any || P.fl_on[e];
    *on = any;
    return e0 < e1 ? e0 : -1;
}

__global__ void wb_unit_kernel(DevProblem P, DevWork W, int col) {
    const long long task = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= (long long)P.M * P.n_red) return;
    const int m = (int)(task / P.n_red), i = (int)(task % P.n_red);
    bool on;
    const int e = wb_fault(P, m, &on);
    W.xperm[task] = e >= 0 && i == P.iperm[2 * P.fl_bus[e] + col] ? 1.0 : 0.0;
}

__global__ void wb_setup_kernel(DevProblem P, const double *W1, const double *W2, double *Hinv) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= P.M) return;
    bool on;
    const int e = wb_fault(P, m, &on);
    double *h = Hinv + 4 * (size_t)m;
    if (e < 0) {
        h[0] = h[1] = h[2] = h[3] = 0.0;
        return;
    }
    const size_t o = (size_t)m * P.n_red;
    const int r0 = P.iperm[2 * P.fl_bus[e]], r1 = P.iperm[2 * P.fl_bus[e] + 1];
    const double rf = 1.0 / P.fl_yf[e];
    const double a = W1[o + r0] - rf, b = W2[o + r0], c = W1[o + r1], d = W2[o + r1] - rf;
    const double det = a * d - b * c;
    h[0] = d / det;
    h[1] = -b / det;
    h[2] = -c / det;
    h[3] = a / det;
}

__global__ void wb_dots_kernel(DevProblem P, DevWork W, const double *Hinv, double *sv) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= P.M) return;
    bool on;
    const int e = wb_fault(P, m, &on);
    double s0 = 0.0, s1 = 0.0;
    if (e >= 0 && on && W.active[m]) {
        const double *x = W.xperm + (size_t)m * P.n_red;
        const double t0 = x[P.iperm[2 * P.fl_bus[e]]], t1 = x[P.iperm[2 * P.fl_bus[e] + 1]];
        const double *h = Hinv + 4 * (size_t)m;
        s0 = h[0] * t0 + h[1] * t1;
        s1 = h[2] * t0 + h[3] * t1;
    }
    sv[2 * m] = s0;
    sv[2 * m + 1] = s1;
}

__global__ void wb_apply_kernel(DevProblem P, DevWork W, const double *W1, const double *W2, const double *sv) {
    const long long task = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= (long long)P.M * P.n_red) return;
    const int m = (int)(task / P.n_red);
    const double s0 = sv[2 * m], s1 = sv[2 * m + 1];
    if (s0 != 0.0 || s1 != 0.0) W.xperm[task] -= W1[task] * s0 + W2[task] * s1;
}

void launch_wb_unit(const DevProblem &P, const DevWork &W, int col, cudaStream_t st) {
    const long long tasks = (long long)P.M * P.n_red;
    wb_unit_kernel<<<(unsigned)((tasks + 255) / 256), 256, 0, st>>>(P, W, col);
}

void launch_wb_setup(const DevProblem &P, const double *W1, const double *W2, double *Hinv, cudaStream_t st) {
    wb_setup_kernel<<<(P.M + 127) / 128, 128, 0, st>>>(P, W1, W2, Hinv);
}

void launch_wb_correct(const DevProblem &P, const DevWork &W, const double *W1, const double *W2,
                       const double *Hinv, double *s, cudaStream_t st) {
    wb_dots_kernel<<<(P.M + 127) / 128, 128, 0, st>>>(P, W, Hinv, s);
    const long long tasks = (long long)P.M * P.n_red;
    wb_apply_kernel<<<(unsigned)((tasks + 255) / 256), 256, 0, st>>>(P, W, W1, W2, s);
}

// ---------------------------------------------------------------------------
// convergence bookkeeping
// ---------------------------------------------------------------------------

// Start of a Newton iteration: clears the residual norms and the counters;
// the mixed solver takes the modes decided at the previous check.
__global__ void reset_norm_kernel(DevWork W, DevMixed Mx, int M) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < M) {
        W.norm[m] = 0ull;
        if (Mx.on) {
            const uint8_t r = Mx.refac_next[m];
            Mx.refac[m] = r;
            Mx.refac_next[m] = MX_KEEP;
            if (r == MX_FP32) Mx.age[m] = 0;
        }
    }
    if (m == 0) {
        W.flag[0] = 0;
        W.flag[1] = 0;
        W.flag[2] = 0;
    }
}

void launch_reset_norm(const DevProblem &P, const DevWork &W, const DevMixed &Mx, cudaStream_t st) {
    reset_norm_kernel<<<(P.M + 255) / 256, 256, 0, st>>>(W, Mx, P.M);
}

// Start of a Newton solve of the mixed solver: scenarios whose factors have
// served max_age solves, or every scenario when `force` (first solve, event
// re-solves and the solve after them), refresh them at the first iteration;
// a retried solve is exact from its first iteration.  Refreshes are taken
// together: a refresh costs one factorisation launch whatever the number of
// scenarios in it, so when one scenario refreshes, every scenario does.
// One CTA, so that the decision can be shared.
__global__ void __launch_bounds__(1024) mixed_start_kernel(DevWork W, DevMixed Mx, int M, int force) {
    bool any = false;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        if (!W.active[m]) continue;
        if (Mx.all_exact[m]) Mx.refac_next[m] = MX_EXACT;
        else if (force || Mx.age[m] >= Mx.max_age) {
            Mx.refac_next[m] = MX_FP32;
            any = true;
        }
        Mx.age[m] += 1;
    }
    if (__syncthreads_or(any))
        for (int m = threadIdx.x; m < M; m += blockDim.x)
            if (W.active[m] && Mx.refac_next[m] == MX_KEEP) Mx.refac_next[m] = MX_FP32;
}

void launch_mixed_start(const DevProblem &P, const DevWork &W, const DevMixed &Mx, int force, cudaStream_t st) {
    mixed_start_kernel<<<1, std::min(1024, (P.M + 31) / 32 * 32), 0, st>>>(W, Mx, P.M, force);
}

// Restart of the solves marked for a retry: the state goes back to the
// step's starting point (zold), the scenario iterates again from zero
// updates, exactly.  The retry marks are cleared by the host afterwards.
__global__ void retry_start_kernel(DevProblem P, DevWork W, DevMixed Mx) {
    const long long task = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= (long long)P.M * P.n_sys) return;
    const int m = (int)(task / P.n_sys), i = (int)(task % P.n_sys);
    if (!Mx.retry[m]) return;
    W.z[(size_t)m * P.n_sys + i] = W.zold[(size_t)m * P.n_sys + i];
    if (i == 0) {
        W.active[m] = 1;
        W.iters[m] = 0;
        Mx.all_exact[m] = 1;
    }
}

__global__ void predict_kernel(double *z, const double *zold, double *zprev, double *zprev2, double *zprev3, size_t n,
                               int order) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = zold[i], b = zprev[i], c = zprev2[i];
    if (order == 1) z[i] = 2.0 * a - b;
    else if (order == 2) z[i] = 3.0 * (a - b) + c;
    else if (order == 3) z[i] = 4.0 * (a + c) - 6.0 * b - zprev3[i];
    zprev3[i] = c;
    zprev2[i] = b;
    zprev[i] = a;
}

void launch_predict(double *z, const double *zold, double *zprev, double *zprev2, double *zprev3, size_t n,
                    int order, cudaStream_t st) {
    predict_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(z, zold, zprev, zprev2, zprev3, n, order);
}

void launch_retry_start(const DevProblem &P, const DevWork &W, const DevMixed &Mx, cudaStream_t st) {
    const long long tasks = (long long)P.M * P.n_sys;
    retry_start_kernel<<<(int)((tasks + 255) / 256), 256, 0, st>>>(P, W, Mx);
}


// Convergence test (infinity norm of the FP64 residual), the itermax and
// non-finite checks, and for the mixed solver the mode of the next
// iteration, from the contraction of the step just taken (prev_mode: the
// factors it used):
//  - a step with kept factors that reduced the residual by less than the
//    factor rho_max refreshes them;
//  - a step with freshly refreshed FP32 factors that did not halve the
//    residual means FP32 factors are too coarse for this scenario now: it
//    takes exact Newton steps (fresh FP64 factors) until the solve ends;
//  - so does every scenario still iterating after exact_after iterations.
// A scenario that went exact refreshes its kept factors at the next solve.
// When one scenario refreshes, every scenario on kept factors does.
// A mixed solve that ends at itermax or on a non-finite residual with
// inexact steps is not reported: it is marked for a retry from the step's
// starting point with exact Newton steps, whose outcome is reported.
__global__ void __launch_bounds__(1024) check_kernel(DevWork W, DevMixed Mx, int M, double tol, int itermax,
                                                    LoopCtl ctl) {
    bool any = false;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        if (!W.active[m]) continue;
        const unsigned long long bits = W.norm[m];
        const double nrm = __longlong_as_double((long long)bits);
        const bool can_retry = Mx.on && !Mx.all_exact[m];
        if (nrm < tol) {
            W.active[m] = 0;
        } else if (bits >= 0x7ff0000000000000ull || W.iters[m] >= itermax) {
            W.active[m] = 0;
            if (can_retry) {
                Mx.retry[m] = 1;
                atomicAdd(W.flag + 3, 1);
            } else {
                W.status[m] |= bits >= 0x7ff0000000000000ull ? 2 : 1;
            }
        } else {
            if (Mx.on) {
                const int cur = Mx.refac[m], used = Mx.prev_mode[m];
                const bool stepped = W.iters[m] > 0;
                int next = MX_KEEP;
                if (cur == MX_EXACT || W.iters[m] + 1 >= Mx.exact_after ||
                    (stepped && used == MX_FP32 && nrm > 0.5 * Mx.prev_norm[m]))
                    next = MX_EXACT;
                else if (stepped && used == MX_KEEP && nrm > Mx.rho_max * Mx.prev_norm[m])
                    next = MX_FP32;
                if (next == MX_EXACT) Mx.age[m] = Mx.max_age;
                if (next == MX_FP32) any = true;
                Mx.refac_next[m] = (uint8_t)next;
                Mx.prev_mode[m] = (uint8_t)cur;
                Mx.prev_norm[m] = nrm;
                if (cur == MX_FP32) atomicAdd(W.flag + 1, 1);
                else if (cur == MX_EXACT) atomicAdd(W.flag + 2, 1);
            }
            W.iters[m] += 1;
            atomicAdd(W.flag, 1);
        }
    }
    // refreshes are taken together (see mixed_start_kernel)
    if (Mx.on && __syncthreads_or(any))
        for (int m = threadIdx.x; m < M; m += blockDim.x)
            if (W.active[m] && Mx.refac_next[m] == MX_KEEP) Mx.refac_next[m] = MX_FP32;
    if (!ctl.on) return;
    // device-driven loop: the next solve, if any, and its factorisations
    __syncthreads();
    if (threadIdx.x == 0) {
        const int act = atomicAdd(W.flag, 0), n32 = atomicAdd(W.flag + 1, 0), n64 = atomicAdd(W.flag + 2, 0);
        const int v = ctl.mixed ? (n32 > 0 ? 1 : 0) | (n64 > 0 ? 2 : 0) : 0;
        cudaGraphSetConditional(ctl.loop, act > 0 ? 1u : 0u);
        if (ctl.mixed) cudaGraphSetConditional(ctl.var, (unsigned)v);
        ctl.cnt[0] += 1;
        if (act > 0) {
            ctl.cnt[1] += 1;
            ctl.cnt[2] += n32;
            ctl.cnt[3] += n64;
            ctl.cnt[4 + v] += 1;
        }
    }
}

void launch_check(const DevProblem &P, const DevWork &W, const DevMixed &Mx, double tol, int itermax,
                  const LoopCtl &ctl, cudaStream_t st) {
    check_kernel<<<1, std::min(1024, (P.M + 31) / 32 * 32), 0, st>>>(W, Mx, P.M, tol, itermax, ctl);
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

__global__ void disconnect_kernel(const int *on_step, const int *scen, const int *idx, uint8_t *flags,
                                  uint8_t *active, int n, int step) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n || on_step[e] != step) return;
    flags[idx[e]] = 1;
    active[scen[e]] = 1;
}

void launch_disconnects(const int *on_step, const int *scen, const int *idx, uint8_t *flags, uint8_t *active,
                        int n, int step, cudaStream_t st) {
    if (n == 0) return;
    disconnect_kernel<<<(n + 255) / 256, 256, 0, st>>>(on_step, scen, idx, flags, active, n, step);
}

}  // namespace gp
