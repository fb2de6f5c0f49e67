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

#include "gp_devices.cuh"
#include "gp_internal.h"

namespace gp {

#define FULL_MASK 0xffffffffu

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long norm_bits(double v) {
    // non-negative doubles order like their bit patterns; NaN counts as +inf
    if (!(v == v)) return 0x7ff0000000000000ull;
    return (unsigned long long)__double_as_longlong(fabs(v));
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

__global__ void __launch_bounds__(32) cluster_kernel(DevProblem P, DevWork W, DevClu Cl, int want_f) {
    extern __shared__ double vals[];
    const int task = blockIdx.x, m = blockIdx.y, lane = threadIdx.x;
    if (!W.active[m]) return;
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
    LaneSink sink{vals, Cl.slot_of + (size_t)cls * 1024, ws, lane};
    double Cc[6] = {0, 0, 0, 0, 0, 0}, Ic[2] = {0, 0};
    if (act) {
        genrou_eval(devref(P.dev[0], P.cl_gen[c]), P.net, z, u0, p, sink, Cc, Ic);
        const int gt = P.cl_gov_type[c];
        if (gt == 1) ieesgo_eval(devref(P.dev[1], P.cl_gov[c]), z, p, sink);
        else if (gt == 2) tgov1_eval(devref(P.dev[2], P.cl_gov[c]), z, p, sink);
        const int et = P.cl_exc_type[c];
        if (et == 3) sexs_eval(devref(P.dev[3], P.cl_exc[c]), P.net, z, p, sink);
        else if (et == 4) esdc1a_eval(devref(P.dev[4], P.cl_exc[c]), P.net, z, p, sink);
        if (P.cl_pss[c] >= 0) ieeest_eval(devref(P.dev[5], P.cl_pss[c]), z, p, sink);
    } else {
        // idle lanes factor an identity so that no lane divides by zero
        const CluOp *o = Cl.ops + Cl.prog_ptr[cls];
        for (int q = Cl.prog_mid[cls] - Cl.prog_ptr[cls]; q < Cl.prog_ptr[cls + 1] - Cl.prog_ptr[cls]; q++)
            if (o[q].code == OP_RCP) vals[o[q].a * 32 + lane] = 1.0;
    }
    const double dt = *W.dt;
    const int rb = Cl.rhs_base[cls];
    double *R0 = vals + (size_t)rb * 32, *R1 = R0 + (size_t)Wn * 32, *R2 = R1 + (size_t)Wn * 32;
    const CluOp *ops = Cl.ops;
    const int q0 = Cl.prog_ptr[cls], qm = Cl.prog_mid[cls], q1 = Cl.prog_ptr[cls + 1];
    // backward-Euler scaling
    for (int q = q0; q < qm; q++) {
        const CluOp o = ops[q];
        double *vd = vals + o.d * 32 + lane;
        if (o.code == OP_SCL) *vd *= -dt;
        else if (o.code == OP_DIAG) *vd += 1.0;
        else if (o.code == OP_BEF) *vd = act ? z[ws + o.a] - zold[ws + o.a] - dt * *vd : 0.0;
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
    // factorisation and solves
    for (int q = qm; q < q1; q++) {
        const CluOp o = ops[q];
        switch (o.code) {
        case OP_RCP:
            vals[o.d * 32 + lane] = 1.0 / vals[o.a * 32 + lane];
            break;
        case OP_MUL:
            vals[o.d * 32 + lane] *= vals[o.a * 32 + lane];
            break;
        case OP_FMS:
            vals[o.d * 32 + lane] -= vals[o.a * 32 + lane] * vals[o.b * 32 + lane];
            break;
        case OP_FMS3: {
            const double l = vals[o.a * 32 + lane];
            R0[o.d * 32 + lane] -= l * R0[o.b * 32 + lane];
            R1[o.d * 32 + lane] -= l * R1[o.b * 32 + lane];
            R2[o.d * 32 + lane] -= l * R2[o.b * 32 + lane];
            break;
        }
        case OP_MUL3: {
            const double l = vals[o.a * 32 + lane];
            R0[o.d * 32 + lane] *= l;
            R1[o.d * 32 + lane] *= l;
            R2[o.d * 32 + lane] *= l;
            break;
        }
        default:
            break;
        }
    }
    if (!act) return;
    const int n_da = P.n_diff + P.n_alg;
    double *yx = W.yx + (size_t)m * 3 * n_da + ws;
    for (int j = 0; j < Wn; j++) {
        const int st = pc[j];
        yx[st] = R2[j * 32 + lane];
        yx[n_da + st] = R0[j * 32 + lane];
        yx[2 * n_da + st] = R1[j * 32 + lane];
    }
    const int *p3 = Cl.pos3 + cls * 3;
    double X1[3], X2[3], Y[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {
        X1[t] = R0[p3[t] * 32 + lane];
        X2[t] = R1[p3[t] * 32 + lane];
        Y[t] = R2[p3[t] * 32 + lane];
    }
    double *o = W.clout + ((size_t)m * P.n_cl + c) * 8;
    o[0] = Cc[0] * X1[0] + Cc[1] * X1[1] + Cc[2] * X1[2];
    o[1] = Cc[0] * X2[0] + Cc[1] * X2[1] + Cc[2] * X2[2];
    o[2] = Cc[3] * X1[0] + Cc[4] * X1[1] + Cc[5] * X1[2];
    o[3] = Cc[3] * X2[0] + Cc[4] * X2[1] + Cc[5] * X2[2];
    o[4] = Cc[0] * Y[0] + Cc[1] * Y[1] + Cc[2] * Y[2];
    o[5] = Cc[3] * Y[0] + Cc[4] * Y[1] + Cc[5] * Y[2];
    o[6] = Ic[0];
    o[7] = Ic[1];
}

void launch_cluster(const DevProblem &P, const DevWork &W, const DevClu &C, int want_f, cudaStream_t st) {
    if (C.n_tasks == 0) return;
    dim3 grid(C.n_tasks, P.M);
    cluster_kernel<<<grid, 32, (size_t)C.max_slots * 32 * sizeof(double), st>>>(P, W, C, want_f);
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
