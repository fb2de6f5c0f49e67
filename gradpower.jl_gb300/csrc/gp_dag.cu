// Dataflow multifrontal factorisation of the reduced
// network matrix S, batched over scenarios.
//
// This replaces cuDSS's factorization/solve of S
// (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2782-2799).  A task is one
// (supernode, scenario) pair.  Tasks are numbered in a topological order of
// the assembly tree (children before parents) and claimed in that order
// from an atomic counter by persistent warps or CTAs.  A task waits only on
// tasks with smaller numbers (its children; for the backward solve, its
// parent in the reversed order), which were claimed earlier by warps or
// CTAs that are running, so the smallest unfinished claimed task can always
// proceed and the kernel cannot deadlock.  Every wait is bounded: after
// D.wait_limit polls it raises the error flag, every other wait then returns
// at once, and the kernel finishes with the scenario marked in `status`.
//
// Factorisation, in two launches (three for FP64):
//  - factor_group_kernel (FP64 only): supernodes whose whole subtree has
//    fronts of at most kTinyFront rows, 32 / kTinyLanes scenarios a warp
//    (kTinyLanes lanes per front);
//  - factor_small_kernel: supernodes whose whole subtree has fronts of at
//    most 32 rows, one warp per task, the front in shared memory;
//  - factor_big_kernel: the rest, one CTA per task.
// Partial pivoting is restricted to a supernode's pivot rows.  The FP32
// elimination is blocked (the pivot panel column by column, then one
// triangular solve and one update of the rest of the front); the FP64 one
// is right-looking.  The front is column-major (leading dimension = front
// rows) in shared memory; of it, the factorisation stores the update matrix
// that the parent's extend-add reads (in `fronts`, at the front's offset)
// and, for the triangular solves, the L panel and the U rows in the
// solve-ordered arrays lfac and ufac (DevSym::lu_off).
//
// The factor type T is double (exact Newton) or float (factors kept and
// reused across Newton iterations).  The FP64 factorisation also does the
// forward solve (the right-hand side rides along as an extra column); the
// triangular solves are in gp_solve.cu.  Row interchanges are stored as one
// composed permutation per supernode (ipiv[start + i] = assembled row that
// became pivot row i), which the solves apply as a single gather.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "gp_internal.h"
#include "gp_warp.cuh"

namespace gp {

namespace {

constexpr unsigned FULL = kFullMask;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kSmallFront = 32;
// FP64 factorisations run the subtrees whose fronts have at most
// kTinyFront rows first, in a launch of their own with a smaller front
// buffer: more fronts in flight, where the 32-row buffers hold an SM to 24
// (factorisation 693 -> 670 ms per FP64 run), and several fronts a warp
// (factor_group_kernel).  FP32 ones keep one launch: their 32-row buffers
// already allow 48 warps, and the launch boundary would cost the overlap of
// the two regions (74 -> 81 ms per mixed run).
constexpr int kTinyFront = 20;
// lanes a tiny front gets in factor_group_kernel (32 / kTinyLanes fronts a
// warp).  16: two fronts a warp.  8 (four fronts a warp, a quarter fewer
// FP64 instructions by count) measured slower: the same shared memory then
// holds half the warps, and the kernel also waits on its loads (FP64
// factorisation 141.2 -> 144.7 ms over 0.3 s of the 70k-bus workload).
constexpr int kTinyLanes = 16;
// update-matrix entries a thread loads ahead in the extend-add: none in the
// warp kernel, which runs at 40 registers a thread and many warps a SM
template <class G>
__host__ __device__ constexpr int asm_batch() {
    return G::size > 32 ? 8 : 1;
}

template <class T>
__device__ __forceinline__ T ldcg(const T *p) {
    return __ldcg(p);
}

// One warp waits for the children of supernode s (scenario m) whose
// schedule rank is at least `from_rank`; with `split`, on each part of a
// split child.
__device__ bool warp_wait_children(const DevSym &S, const DevDag &D, const int *done, int s, int m, int M,
                                   int epoch, int from_rank, bool split = false) {
    const int lane = threadIdx.x & 31;
    const int c0 = S.child_ptr[s], nc = S.child_ptr[s + 1] - c0;
    bool ok = true;
    for (int q = lane; q < nc; q += 32) {
        const int c = S.children[c0 + q];
        const int rc = D.rank[c];
        if (rc < from_rank) continue;
        const int np = split ? D.nparts[c] : 1;
        if (np == 1) {
            ok = wait_epoch(done + (size_t)c * M + m, epoch, D.err, D.wait_limit) && ok;
        } else {
            const int *pd = D.pdone + ((size_t)(rc - D.tail0) * M + m) * kMaxParts;
            for (int p = 0; p < np; p++) ok = wait_epoch(pd + p, epoch, D.err, D.wait_limit) && ok;
        }
    }
    ok = __all_sync(FULL, ok);
    __syncwarp();
    return ok;
}

// The same for several scenarios a warp: each W-lane group (W = 8 or 16)
// waits for the children of supernode s in its own scenario m (the whole
// warp calls it); true when every wait of the caller's group succeeded.
template <int W>
__device__ bool group_wait_children(const DevSym &S, const DevDag &D, const int *done, int s, int m, int M,
                                    int epoch) {
    static_assert(W == 8 || W == 16, "lane groups of 8 or 16");
    const int c0 = S.child_ptr[s], nc = S.child_ptr[s + 1] - c0;
    bool ok = true;
    for (int q = threadIdx.x & (W - 1); q < nc; q += W) {
        const int c = S.children[c0 + q];
        ok = wait_epoch(done + (size_t)c * M + m, epoch, D.err, D.wait_limit) && ok;
    }
    const unsigned bad = __ballot_sync(FULL, !ok);
    __syncwarp();
    return (bad & (((1u << W) - 1u) << (threadIdx.x & 31 & ~(W - 1)))) == 0;
}

// Magnitude of a factor entry as an unsigned key that orders like |v|
// (sign bit cleared; NaN above +inf), so that pivot search and reductions
// run on the integer pipes instead of the (scarce) FP64 pipe.
__device__ __forceinline__ unsigned long long mag_key(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned long long mag_key(float v) {
    return (unsigned long long)(__float_as_uint(v) & 0x7fffffffu);
}

// Pivot of column k among rows [k, ns) of a front: index of the largest
// magnitude, the smallest index on ties.  Called by a whole warp; every lane
// returns the same result.  zero is set when the column is zero there.
template <class T>
struct KeyOf {
    using type = unsigned long long;
};
template <>
struct KeyOf<float> {
    using type = unsigned;
};

// LW < 32: the warp is LW-lane segments, each searching its own front (the
// whole warp calls it).
template <class T, int LW = 32>
__device__ __forceinline__ int warp_pivot(const T *F, int mm, int k, int ns, bool &zero) {
    using K = typename KeyOf<T>::type;
    const int lane = threadIdx.x & (LW - 1);
    K bk = 0;
    int bi = k;
    for (int i = k + lane; i < ns; i += LW) {
        const K v = (K)mag_key(F[i + k * mm]);
        if (v > bk) { bk = v; bi = i; }
    }
#pragma unroll
    for (int off = LW / 2; off > 0; off >>= 1) {
        const K ok = __shfl_xor_sync(FULL, bk, off, LW);
        const int oi = __shfl_xor_sync(FULL, bi, off, LW);
        if (ok > bk || (ok == bk && oi < bi)) { bk = ok; bi = oi; }
    }
    zero = bk == 0;
    return bi;
}

// Thread groups that factor one front: a warp, the whole CTA, or a W-lane
// part of a warp (32 / W fronts a warp, each group on its own front of the
// same supernode).  size: threads of the group; lanes: threads of the lead
// segment that searches pivots and scales the multipliers; active(): false
// for a group that only follows another's front (it computes that front
// and stores nothing).
struct WarpGroup {
    static constexpr int size = 32, lanes = 32;
    __device__ int idx() const { return threadIdx.x & 31; }
    __device__ int lane() const { return threadIdx.x & 31; }
    __device__ bool lead_warp() const { return true; }
    __device__ bool active() const { return true; }
    __device__ void sync() const { __syncwarp(); }
};
struct BlockGroup {
    static constexpr int size = kThreads, lanes = 32;
    __device__ int idx() const { return threadIdx.x; }
    __device__ int lane() const { return threadIdx.x & 31; }
    __device__ bool lead_warp() const { return threadIdx.x < 32; }
    __device__ bool active() const { return true; }
    __device__ void sync() const { __syncthreads(); }
};
template <int W>
struct LaneGroup {
    static constexpr int size = W, lanes = W;
    bool act;
    __device__ int idx() const { return threadIdx.x & (W - 1); }
    __device__ int lane() const { return threadIdx.x & (W - 1); }
    __device__ bool lead_warp() const { return true; }
    __device__ bool active() const { return act; }
    // every group runs the same supernode, so they meet every barrier
    __device__ void sync() const { __syncwarp(); }
};

// Columns per panel of the blocked elimination of CTA-sized fronts.
template <class T>
struct PanelOf {
    static constexpr int cols = 8;
};

// Elimination of a front by the whole CTA (fronts above the warp size),
// blocked right-looking in panels of PanelOf<T>::cols pivot columns:
//  (a) the panel, column by column: warp 0 finds the pivot among the pivot
//      rows, swaps the two rows within the panel, stores the multipliers
//      and the pivot's reciprocal, and updates the panel's later columns;
//      in registers (lane l holds rows kb + l + 32 j) when the panel has at
//      most 32 * kPanelRows rows, else in shared memory with the CTA
//      updating the panel's later columns;
//  (b) the panel's row interchanges applied to every other column;
//  (c) U of the panel rows right of it, by a forward substitution per
//      column with the panel's unit lower block (values in registers);
//  (d) the trailing update A -= L U (rank = panel width): a warp takes four
//      columns and its lanes the rows, each lane the same four columns of
//      up to five rows, sums in registers; the U entries are broadcasts and
//      the L and A entries consecutive across lanes (no bank conflicts).
// Every entry receives the same operations in the same order as in the
// column-by-column right-looking elimination (each update one FMA, the
// updates of an entry in pivot order), so the factors are the same.  The
// columns beyond the front (nc > mm: the right-hand side of the FP64
// factorisation) are carried through (b)-(d) like any other column.  The
// front is left with the multipliers below the diagonal, U above it, the
// pivots' reciprocals on it, piv[k] the row swapped with row k at step k.
// Rows a lane holds in the register panel.
constexpr int kPanelRows = 5;

// Value of register slot j (a runtime index) of a per-lane array.
template <class T, int J>
__device__ __forceinline__ T slot(const T (&r)[J], int j) {
    T v = r[0];
#pragma unroll
    for (int q = 1; q < J; q++)
        if (j == q) v = r[q];
    return v;
}

// The warp's largest key and, among the lanes holding it, the smallest
// index; every lane returns both.
__device__ __forceinline__ void warp_argmax(unsigned &key, int &bi) {
    const unsigned kmax = __reduce_max_sync(FULL, key);
    bi = (int)__reduce_min_sync(FULL, key == kmax ? (unsigned)bi : 0xffffffffu);
    key = kmax;
}
__device__ __forceinline__ void warp_argmax(unsigned long long &key, int &bi) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(FULL, key, off);
        const int oi = __shfl_xor_sync(FULL, bi, off);
        if (ok > key || (ok == key && oi < bi)) {
            key = ok;
            bi = oi;
        }
    }
}

// Panel [kb, ke) factored by one warp in registers: lane l holds rows kb +
// l + 32 j (j < J) of the panel's columns.  Per column: the pivot among the
// pivot rows (largest magnitude, smallest row on ties), the pivot row and
// row k exchanged through shuffles, the multipliers, the rank-1 update of
// the panel's later columns; no barrier.
template <class T, int J>
__device__ void panel_warp(T *F, int mm, int ns, int kb, int ke, int *piv, int *status) {
    constexpr int NP = PanelOf<T>::cols;
    using K = typename KeyOf<T>::type;
    const int lane = threadIdx.x & 31, nb = ke - kb;
    T P[J][NP];
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = kb + lane + 32 * j;
#pragma unroll
        for (int c = 0; c < NP; c++) P[j][c] = (i < mm && c < nb) ? F[i + (kb + c) * mm] : T(0);
    }
#pragma unroll
    for (int c = 0; c < NP; c++) {
        if (c >= nb) break;
        const int k = kb + c;
        // pivot among rows k..ns-1
        K key = 0;
        int bi = k;
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = kb + lane + 32 * j;
            const K v = (K)mag_key(P[j][c]);
            if (i >= k && i < ns && v > key) { key = v; bi = i; }
        }
        warp_argmax(key, bi);
        const int pv = bi;
        if (lane == 0) {
            piv[k] = pv;
            if (key == 0) atomicOr(status, 4);
        }
        // the pivot row (u) and row k (w), broadcast
        const int lp = (pv - kb) & 31, jp = (pv - kb) >> 5, lk = (k - kb) & 31, jk = (k - kb) >> 5;
        T u[NP], w[NP];
#pragma unroll
        for (int q = 0; q < NP; q++) {
            T col[J];
#pragma unroll
            for (int j = 0; j < J; j++) col[j] = P[j][q];
            u[q] = __shfl_sync(FULL, slot(col, jp), lp);
            w[q] = __shfl_sync(FULL, slot(col, jk), lk);
        }
        const T inv = recip(u[c]);
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = kb + lane + 32 * j;
            if (i == pv && pv != k) {
#pragma unroll
                for (int q = 0; q < NP; q++) P[j][q] = w[q];
            }
            if (i == k) {
#pragma unroll
                for (int q = 0; q < NP; q++) P[j][q] = u[q];
                P[j][c] = inv;
            }
        }
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = kb + lane + 32 * j;
            if (i > k && i < mm) {
                const T l = P[j][c] * inv;
                P[j][c] = l;
#pragma unroll
                for (int q = 0; q < NP; q++)
                    if (q > c) P[j][q] -= l * u[q];
            }
        }
    }
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = kb + lane + 32 * j;
#pragma unroll
        for (int c = 0; c < NP; c++)
            if (i < mm && c < nb) F[i + (kb + c) * mm] = P[j][c];
    }
    __syncwarp();
}

// The register panel for rows kb..mm-1 (at most 32 * kPanelRows of them).
template <class T>
__device__ __forceinline__ void panel_regs(T *F, int mm, int ns, int kb, int ke, int *piv, int *status) {
    switch ((mm - kb + 31) >> 5) {
    case 1: panel_warp<T, 1>(F, mm, ns, kb, ke, piv, status); break;
    case 2: panel_warp<T, 2>(F, mm, ns, kb, ke, piv, status); break;
    case 3: panel_warp<T, 3>(F, mm, ns, kb, ke, piv, status); break;
    case 4: panel_warp<T, 4>(F, mm, ns, kb, ke, piv, status); break;
    default: panel_warp<T, 5>(F, mm, ns, kb, ke, piv, status); break;
    }
}

template <class T>
__device__ void eliminate_cta(T *F, int mm, int ns, int nc, int *piv, int *status) {
    constexpr int NP = PanelOf<T>::cols;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    for (int kb = 0; kb < ns; kb += NP) {
        const int ke = min(ns, kb + NP), nb = ke - kb;
        // ---- (a) the panel ----
        if (mm - kb <= 32 * kPanelRows) {
            if (warp == 0) panel_regs<T>(F, mm, ns, kb, ke, piv, status);
            __syncthreads();
        } else
        for (int k = kb; k < ke; k++) {
            if (warp == 0) {
                bool zero;
                const int pv = warp_pivot(F, mm, k, ns, zero);
                if (lane == 0) {
                    piv[k] = pv;
                    if (zero) atomicOr(status, 4);
                }
                if (pv != k && lane < nb) {
                    const T a = F[k + (kb + lane) * mm];
                    F[k + (kb + lane) * mm] = F[pv + (kb + lane) * mm];
                    F[pv + (kb + lane) * mm] = a;
                }
                __syncwarp();
                const T inv = recip(F[k + k * mm]);
                for (int i = k + 1 + lane; i < mm; i += 32) F[i + k * mm] *= inv;
                __syncwarp();
                if (lane == 0) F[k + k * mm] = inv;
            }
            __syncthreads();
            // rank-1 update of the panel's later columns, rows k+1..mm-1:
            // threads over rows, the columns split between the CTA's halves
            const int half = blockDim.x >> 1, h = tid >= half, rt = tid - h * half;
            for (int j = k + 1 + h; j < ke; j += 2) {
                const T u = F[k + j * mm];
                for (int i = k + 1 + rt; i < mm; i += half) F[i + j * mm] -= F[i + k * mm] * u;
            }
            __syncthreads();
        }
        // ---- (b) the panel's interchanges on the other columns ----
        for (int j = tid; j < nc; j += blockDim.x) {
            if (j >= kb && j < ke) continue;
            for (int k = kb; k < ke; k++) {
                const int pv = piv[k];
                if (pv != k) {
                    const T a = F[k + j * mm];
                    F[k + j * mm] = F[pv + j * mm];
                    F[pv + j * mm] = a;
                }
            }
        }
        __syncthreads();
        if (ke >= nc) break;
        // ---- (c) U of the panel rows, columns ke..nc-1 ----
        for (int j = ke + tid; j < nc; j += blockDim.x) {
            T u[NP];
#pragma unroll
            for (int q = 0; q < NP; q++) u[q] = q < nb ? F[kb + q + j * mm] : T(0);
#pragma unroll
            for (int q = 0; q < NP; q++)
#pragma unroll
                for (int p = q + 1; p < NP; p++)
                    if (p < nb) u[p] -= F[kb + p + (kb + q) * mm] * u[q];
#pragma unroll
            for (int q = 0; q < NP; q++)
                if (q < nb) F[kb + q + j * mm] = u[q];
        }
        __syncthreads();
        // ---- (d) trailing update, rows ke..mm-1, columns ke..nc-1 ----
        // (tiles of four columns and up to 160 rows, five per lane; a
        // look-ahead, warp 0 factoring the next panel while the other warps
        // update, measured no faster: the update keeps the SM busy)
        auto tile = [&](int c0, int r0) {
            T acc[5][4];
#pragma unroll
            for (int q = 0; q < 5; q++) {
                const int i = r0 + lane + 32 * q;
#pragma unroll
                for (int c = 0; c < 4; c++) acc[q][c] = (i < mm && c0 + c < nc) ? F[i + (c0 + c) * mm] : T(0);
            }
#pragma unroll
            for (int kk = 0; kk < NP; kk++) {
                const int k = kb + kk;
                if (k >= ke) break;
                T u[4], l[5];
#pragma unroll
                for (int c = 0; c < 4; c++) u[c] = c0 + c < nc ? F[k + (c0 + c) * mm] : T(0);
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    const int i = r0 + lane + 32 * q;
                    l[q] = i < mm ? F[i + k * mm] : T(0);
                }
#pragma unroll
                for (int q = 0; q < 5; q++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[q][c] = fma(-l[q], u[c], acc[q][c]);
            }
#pragma unroll
            for (int q = 0; q < 5; q++) {
                const int i = r0 + lane + 32 * q;
#pragma unroll
                for (int c = 0; c < 4; c++)
                    if (i < mm && c0 + c < nc) F[i + (c0 + c) * mm] = acc[q][c];
            }
        };
        const int nq = (nc - ke + 3) >> 2, nr = (mm - ke + 159) / 160;
        for (int t = warp; t < nq * nr; t += nwarp) tile(ke + 4 * (t % nq), ke + 160 * (t / nq));
        __syncthreads();
    }
}

// Factors the front of supernode s for scenario m in shared memory F
// (leading dimension mm = front rows) and stores it to global memory.
//  - Assembly: constant entries of S, the scenario's entries from svar, and
//    the children's update matrices.
//  - Partial pivoting within the pivot rows; the multipliers are stored
//    below the diagonal, and the reciprocal of each pivot on the diagonal.
//  - RHS: column mm carries the right-hand side (the supernode's entries of
//    xperm plus the children's update vectors), so that the elimination is
//    also the forward solve.  It leaves the forward-solved entries in xperm
//    and this supernode's update vector in uvec.
template <class T, bool RHS, class G, class Wait, class Done>
__device__ void factor_front(const DevProblem &P, const DevWork &W, const DevSym &S, T *fronts, T *lfac, T *ufac,
                             int s, int m, T *F, int *piv, G g, Wait wait, Done done) {
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int mm = ns + S.row_ptr[s + 1] - S.row_ptr[s];
    const int nc = mm + (RHS ? 1 : 0);
    const int idx = g.idx(), step = G::size;
    T *fr = fronts + (size_t)m * S.front_total;
    double *x = W.xperm + (size_t)m * P.n_red;
    double *uv = S.uvec + (size_t)m * S.uvec_total;
    // ---- assembly ----
    for (int i = idx; i < mm * nc; i += step) F[i] = T(0);
    g.sync();
    for (int e = S.asmc_ptr[s] + idx; e < S.asmc_ptr[s + 1]; e += step) F[S.asmc_pos[e]] += (T)S.asmc_val[e];
    if (RHS)
        for (int i = idx; i < ns; i += step) F[mm * mm + i] = (T)x[start + i];
    g.sync();
    const double *sv = W.svar + (size_t)m * P.n_var;
    for (int e = S.asmv_ptr[s] + idx; e < S.asmv_ptr[s + 1]; e += step) F[S.asmv_pos[e]] += (T)sv[S.asmv_idx[e]];
    if (S.asmt_ptr)
        for (int e = S.asmt_ptr[s] + idx; e < S.asmt_ptr[s + 1]; e += step) {
            const int t = S.asmt_tr[e];
            if (P.tr_on[t] && t >= P.tr_ptr[m] && t < P.tr_ptr[m + 1]) F[S.asmt_pos[e]] += (T)S.asmt_val[e];
        }
    g.sync();
    // the entries above need nothing from the children: only now wait for
    // them (bounded; wait() ends with a barrier of the group)
    wait();
    if (G::size > 32 && S.pa_base && S.pa_base[s] >= 0) {
        // CTA fronts: every entry sums its children's contributions (host
        // lists, child order) without a barrier between children; kPa
        // entries a thread per round, their loads issued together (the
        // round trips to L2 of a round overlap)
        const int *pp = S.pa_ptr + S.pa_base[s];
        const int n2 = mm * mm;
        constexpr int kPa = 8;
        for (int p0 = idx; p0 < n2; p0 += kPa * step) {
            T acc[kPa];
            int e0[kPa], e1[kPa], kmax = 0;
#pragma unroll
            for (int u = 0; u < kPa; u++) {
                const int p = p0 + u * step;
                e0[u] = p < n2 ? pp[p] : 0;
                e1[u] = p < n2 ? pp[p + 1] : 0;
                acc[u] = p < n2 ? F[p] : T(0);
                kmax = max(kmax, e1[u] - e0[u]);
            }
            for (int k = 0; k < kmax; k++)
#pragma unroll
                for (int u = 0; u < kPa; u++)
                    if (e0[u] + k < e1[u]) acc[u] += ldcg(fr + S.pa_src[e0[u] + k]);
#pragma unroll
            for (int u = 0; u < kPa; u++)
                if (p0 + u * step < n2) F[p0 + u * step] = acc[u];
        }
        if (RHS) {
            const int *rp = S.pr_ptr + S.pr_base[s];
            for (int i = idx; i < mm; i += step) {
                T acc = F[mm * mm + i];
                for (int e = rp[i]; e < rp[i + 1]; e++) acc += (T)ldcg(uv + S.pr_src[e]);
                F[mm * mm + i] = acc;
            }
        }
        g.sync();
    } else
    for (int q = S.child_ptr[s]; q < S.child_ptr[s + 1]; q++) {
        const int c = S.children[q];
        const int ncc = S.sup_start[c + 1] - S.sup_start[c];
        const int rc = S.row_ptr[c + 1] - S.row_ptr[c];
        const int mc = ncc + rc;
        const int *rel = S.relmap + S.relmap_ptr[c];
        const T *Fc = fr + S.front_off[c];
        // (a, b) = (t % rc, t / rc), advanced by the stride without a
        // division per entry.  A thread loads asm_batch entries (and their
        // positions) before it adds any of them, so that their round trips
        // to L2 overlap instead of following one another
        const int rcs = rc > 0 ? rc : 1;   // (a child always has update rows)
        int a = idx % rcs, b = idx / rcs;
        const int da = step % rcs, db = step / rcs;
        const int n = rc * rc;
        constexpr int kAsmBatch = asm_batch<G>();
        for (int t0 = idx; t0 < n; t0 += kAsmBatch * step) {
            T val[kAsmBatch];
            int pos[kAsmBatch];
#pragma unroll
            for (int u = 0; u < kAsmBatch; u++) {
                if (t0 + u * step < n) {
                    pos[u] = rel[a] + rel[b] * mm;
                    val[u] = ldcg(Fc + (ncc + a) + (size_t)(ncc + b) * mc);
                }
                a += da;
                b += db;
                if (a >= rc) { a -= rc; b++; }
            }
#pragma unroll
            for (int u = 0; u < kAsmBatch; u++)
                if (t0 + u * step < n) F[pos[u]] += val[u];
        }
        if (RHS) {
            const double *uc = uv + S.uvec_off[c];
            for (int a = idx; a < rc; a += step) F[mm * mm + rel[a]] += (T)ldcg(uc + a);
        }
        g.sync();
    }
    // ---- elimination ----
    // FP64: right-looking, column by column over the whole front, each
    // column's updates spread evenly over every thread of the group (FP64
    // runs at two FMAs a clock per SM on GB300: the elimination is bound by
    // the FP64 pipe, and this keeps all four of its SM sub-partitions busy,
    // where a panel factored by one warp would idle three of them).  FP32:
    // blocked; CTA fronts in panels (eliminate_cta), warp fronts with the
    // pivot panel (columns 0..ns-1) column by column, then the right part
    // (columns ns..nc-1) once: U12 = L11^-1 A12 by forward substitution, one
    // column per thread, and A22 -= L21 U12, four entries per thread with the
    // sums in registers.  All of them give every entry the same operations
    // in the same order.
    constexpr bool kBlocked = sizeof(T) == 4;
    if constexpr (kBlocked && G::size > 32) {
        static_assert(!RHS, "the FP32 factorisation carries no right-hand side");
        eliminate_cta<T>(F, mm, ns, nc, piv, W.status + m);
    } else {
    for (int k = 0; k < ns; k++) {
        if (g.lead_warp()) {
            constexpr int LW = G::lanes;
            const int lane = g.lane();
            bool zero;
            const int pv = warp_pivot<T, LW>(F, mm, k, ns, zero);
            if (lane == 0) {
                piv[k] = pv;
                if (zero && g.active()) atomicOr(W.status + m, 4);
            }
            if (pv != k)
                for (int j = lane; j < nc; j += LW) {
                    const T a = F[k + j * mm];
                    F[k + j * mm] = F[pv + j * mm];
                    F[pv + j * mm] = a;
                }
            __syncwarp();
            const T inv = recip(F[k + k * mm]);
            for (int i = k + 1 + lane; i < mm; i += LW) F[i + k * mm] *= inv;
            __syncwarp();
            if (lane == 0) F[k + k * mm] = inv;
        }
        g.sync();
        // rank-1 update: rows k+1.., columns k+1.. of the whole front
        // (right-looking) or of the panel only (blocked)
        const int lr = mm - k - 1, lc = (kBlocked ? ns : nc) - k - 1;
        if (lr > 0 && lc > 0) {
            int i = idx % lr, j = idx / lr;
            const int di = step % lr, dj = step / lr;
            const T *lk = F + k * mm;
            for (int t = idx; t < lr * lc; t += step) {
                const int ii = k + 1 + i, jj = k + 1 + j;
                F[ii + jj * mm] -= lk[ii] * F[k + jj * mm];
                i += di;
                j += dj;
                if (i >= lr) { i -= lr; j++; }
            }
        }
        g.sync();
    }
    if (kBlocked) {
        for (int j = ns + idx; j < nc; j += step) {
            T *cj = F + j * mm;
            for (int k = 0; k < ns; k++) {
                const T u = cj[k];
                const T *lk = F + k * mm;
                for (int i = k + 1; i < ns; i++) cj[i] -= lk[i] * u;
            }
        }
        g.sync();
        const int r = mm - ns, n = r * (nc - ns);
        // entry t0 + q * step is (ns + t % r, ns + t / r); the four row and
        // column indices advance by 4 * step without a division per entry
        const int rr = r > 0 ? r : 1;   // (no entries when r == 0)
        int rq[4], cq[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            rq[q] = (idx + q * step) % rr;
            cq[q] = (idx + q * step) / rr;
        }
        const int dr = (4 * step) % rr, dc = (4 * step) / rr;
        for (int t0 = idx; t0 < n; t0 += 4 * step) {
            int ri[4], cj[4];
            T acc[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const bool in = t0 + q * step < n;
                ri[q] = ns + (in ? rq[q] : r - 1);
                cj[q] = (ns + (in ? cq[q] : nc - ns - 1)) * mm;
                acc[q] = F[ri[q] + cj[q]];
                rq[q] += dr;
                cq[q] += dc;
                if (rq[q] >= r) { rq[q] -= r; cq[q]++; }
            }
            for (int k = 0; k < ns; k++) {
                const T *lk = F + k * mm;
#pragma unroll
                for (int q = 0; q < 4; q++) acc[q] -= lk[ri[q]] * F[k + cj[q]];
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (t0 + q * step < n) F[ri[q] + cj[q]] = acc[q];
        }
        g.sync();
    }
    }
    // ---- store ----
    // the row interchanges, composed: pivot row i of the factored front is
    // row perm[i] of the assembled one
    if (idx == 0) {
        int *perm = piv + ns;
        for (int i = 0; i < ns; i++) perm[i] = i;
        for (int k = 0; k < ns; k++) {
            const int p = piv[k], t = perm[k];
            perm[k] = perm[p];
            perm[p] = t;
        }
    }
    // first what the parent's assembly reads: the columns ns..mm-1 (their
    // rows ns..mm-1 are the update matrix) as one contiguous range and, with
    // RHS, the update vector (and the forward-solved entries); then done(),
    // and only after it the solve-ordered copies of the factors, which
    // nothing reads before the solves: the L panel (columns 0..ns-1,
    // contiguous as in F; skipped when lfac is null), the U rows (rows
    // 0..ns-1, leading dimension ns; the 2D index advances by the stride, one
    // division per thread) and the composed pivots
    const bool act = g.active();
    if (act) {
        T *out = fr + S.front_off[s];
        for (int i = ns * mm + idx; i < mm * mm; i += step) out[i] = F[i];
    }
    if (RHS && act) {
        for (int i = idx; i < ns; i += step) x[start + i] = (double)F[mm * mm + i];
        double *us = uv + S.uvec_off[s];
        for (int a = idx; a < mm - ns; a += step) us[a] = (double)F[mm * mm + ns + a];
    }
    g.sync();
    done();
    if (act) {
        if (lfac) {
            T *lo = lfac + (size_t)m * S.lu_total + S.lu_off[s];
            for (int i = idx; i < mm * ns; i += step) lo[i] = F[i];
        }
        T *uo = ufac + (size_t)m * S.lu_total + S.lu_off[s];
        int i = idx % ns, c = idx / ns;
        const int di = step % ns, dc = step / ns;
        for (int e = idx; e < ns * mm; e += step) {
            uo[e] = F[i + c * mm];
            i += di;
            c += dc;
            if (i >= ns) { i -= ns; c++; }
        }
    }
    if (act) {
        int *ipiv = S.ipiv + (size_t)m * S.n + start;
        for (int i = idx; i < ns; i += step) ipiv[i] = piv[ns + i];
    }
    g.sync();
}

// ---- split fronts ----------------------------------------------------------
// One part of a front factored by np CTAs together (np parts, each a task of
// the CTA kernel).  The front's columns are dealt in blocks of kSplitPanel:
// column j belongs to part (j / kSplitPanel) % np, which keeps its columns
// in shared memory (local index jl, leading dimension mm).  Each part
// assembles its own columns.  Panel p (pivot columns p*kSplitPanel ..) is
// factored by its part, column by column (pivot among the pivot rows,
// largest magnitude, smallest row on ties; multipliers; rank-1 update of the
// panel's later columns), and published: its columns and pivot rows to
// global memory, then a flag set to the epoch.  Every part (the owner
// included) then applies the panel's row interchanges to its other columns,
// computes the U rows of its columns right of the panel and updates them
// below it (rank kSplitPanel).  Every entry receives the same operations in
// the same order as in the one-CTA elimination, so the factors are the same.
// A part waits (bounded) only on the panels of the other parts of its own
// front, which are the tasks next to it in the claim order, so with at
// least kMaxParts resident CTAs the kernel cannot deadlock.
// Shared memory: the local columns (mm x ncl_cap), the panel read from
// global memory (mm x kSplitPanel), the pivot rows and their composition.
template <class T, bool RHS, class Wait, class Done>
__device__ void factor_part(const DevProblem &P, const DevWork &W, const DevSym &S, const DevDag &D, T *fronts,
                            T *lfac, T *ufac, int s, int m, int k, int part, int np, int epoch,
                            unsigned char *smem, Wait wait, Done done) {
    constexpr int B = kSplitPanel;
    using K = typename KeyOf<T>::type;
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int mm = ns + S.row_ptr[s + 1] - S.row_ptr[s];
    const int nc = mm + (RHS ? 1 : 0);
    auto owned_below = [&](int j) { return split_owned_below(j, part, np); };
    auto jof = [&](int jl) { return split_col(jl, part, np); };
    const int ncl = owned_below(nc);
    T *Fl = reinterpret_cast<T *>(smem);
    T *Pn = Fl + (size_t)mm * split_cols_cap(nc, np);
    int *piv = reinterpret_cast<int *>(Pn + (size_t)mm * B);
    int *perm = piv + mm;
    T *fr = fronts + (size_t)m * S.front_total;
    double *x = W.xperm + (size_t)m * P.n_red;
    double *uv = S.uvec + (size_t)m * S.uvec_total;
    // front position p = i + j * mm -> local entry, -1 when another part's
    auto local = [&](int p) {
        const int j = p / mm;
        return split_owner(j, np) != part ? -1 : (p - j * mm) + owned_below(j) * mm;
    };
    const int jr = split_owner(mm, np) == part ? owned_below(mm) : -1;   // local right-hand side
    // ---- assembly of the part's columns ----
    for (int e = tid; e < mm * ncl; e += nthr) Fl[e] = T(0);
    __syncthreads();
    for (int q = S.asmc_ptr[s] + tid; q < S.asmc_ptr[s + 1]; q += nthr) {
        const int e = local(S.asmc_pos[q]);
        if (e >= 0) Fl[e] += (T)S.asmc_val[q];
    }
    if (RHS && jr >= 0)
        for (int i = tid; i < ns; i += nthr) Fl[i + jr * mm] = (T)x[start + i];
    __syncthreads();
    const double *sv = W.svar + (size_t)m * P.n_var;
    for (int q = S.asmv_ptr[s] + tid; q < S.asmv_ptr[s + 1]; q += nthr) {
        const int e = local(S.asmv_pos[q]);
        if (e >= 0) Fl[e] += (T)sv[S.asmv_idx[q]];
    }
    if (S.asmt_ptr)
        for (int q = S.asmt_ptr[s] + tid; q < S.asmt_ptr[s + 1]; q += nthr) {
            const int t = S.asmt_tr[q];
            if (P.tr_on[t] && t >= P.tr_ptr[m] && t < P.tr_ptr[m + 1]) {
                const int e = local(S.asmt_pos[q]);
                if (e >= 0) Fl[e] += (T)S.asmt_val[q];
            }
        }
    __syncthreads();
    wait();
    {
        // the children's update matrices, entry by entry from the host lists
        // (child order), four entries a thread with their loads together
        const int *pp = S.pa_ptr + S.pa_base[s];
        for (int e0 = tid; e0 < mm * ncl; e0 += 4 * nthr) {
            T acc[4];
            int a0[4], a1[4], kmax = 0;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int e = e0 + u * nthr;
                a0[u] = a1[u] = 0;
                acc[u] = T(0);
                if (e < mm * ncl) {
                    const int jl = e / mm, i = e - jl * mm;
                    acc[u] = Fl[e];
                    if (jl != jr) {
                        const int p = i + jof(jl) * mm;
                        a0[u] = pp[p];
                        a1[u] = pp[p + 1];
                    }
                }
                kmax = max(kmax, a1[u] - a0[u]);
            }
            for (int kk = 0; kk < kmax; kk++)
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (a0[u] + kk < a1[u]) acc[u] += ldcg(fr + S.pa_src[a0[u] + kk]);
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (e0 + u * nthr < mm * ncl) Fl[e0 + u * nthr] = acc[u];
        }
        // (the loop above also wrote the right-hand-side column back as it
        // found it: its children's update vectors are added after a barrier)
        __syncthreads();
        if (RHS && jr >= 0) {
            const int *rp = S.pr_ptr + S.pr_base[s];
            for (int i = tid; i < mm; i += nthr) {
                T acc = Fl[i + jr * mm];
                for (int e = rp[i]; e < rp[i + 1]; e++) acc += (T)ldcg(uv + S.pr_src[e]);
                Fl[i + jr * mm] = acc;
            }
        }
    }
    __syncthreads();
    // ---- elimination, panel by panel ----
    const int npan = (ns + B - 1) / B;
    int *ppv = D.ppiv + ((size_t)k * P.M + m) * D.max_split_ns;
    T *pb = reinterpret_cast<T *>(D.pbuf) + (size_t)m * D.pb_total + D.pb_off[k];
    int *pfl = D.pflag + ((size_t)k * P.M + m) * D.max_panels;
    for (int pn = 0; pn < npan; pn++) {
        const int kb = pn * B, ke = min(ns, kb + B), nb = ke - kb;
        const bool own = pn % np == part;
        const int jlp = own ? owned_below(kb) : -1;   // local index of column kb
        const T *L;                                    // panel column c at L + c * mm
        if (own) {
            T *Fp = Fl + (size_t)jlp * mm;
            for (int kk = kb; kk < ke; kk++) {
                T *col = Fp + (size_t)(kk - kb) * mm;
                if (warp == 0) {
                    K key = 0;
                    int bi = kk;
                    for (int i = kk + lane; i < ns; i += 32) {
                        const K v = (K)mag_key(col[i]);
                        if (v > key) { key = v; bi = i; }
                    }
                    warp_argmax(key, bi);
                    if (lane == 0) {
                        piv[kk] = bi;
                        if (key == 0) atomicOr(W.status + m, 4);
                    }
                    if (bi != kk && lane < nb) {
                        const T a = Fp[kk + lane * mm];
                        Fp[kk + lane * mm] = Fp[bi + lane * mm];
                        Fp[bi + lane * mm] = a;
                    }
                    __syncwarp();
                    const T inv = recip(col[kk]);
                    for (int i = kk + 1 + lane; i < mm; i += 32) col[i] *= inv;
                    __syncwarp();
                    if (lane == 0) col[kk] = inv;
                }
                __syncthreads();
                const int lr = mm - kk - 1, lc = ke - kk - 1;
                for (int t = tid; t < lr * lc; t += nthr) {
                    const int c = t / lr, i = t - c * lr;
                    Fp[(kk + 1 + i) + (kk - kb + 1 + c) * mm] -= col[kk + 1 + i] * Fp[kk + (kk - kb + 1 + c) * mm];
                }
                __syncthreads();
            }
            T *dst = pb + (size_t)pn * mm * B;
            for (int e = tid; e < mm * nb; e += nthr) dst[e] = Fp[e];
            for (int i = tid; i < nb; i += nthr) ppv[kb + i] = piv[kb + i];
            __syncthreads();
            if (tid == 0) signal_done(pfl + pn, epoch);
            L = Fp;
        } else {
            if (warp == 0) {
                if (lane == 0 && !wait_epoch(pfl + pn, epoch, D.err, D.wait_limit)) atomicOr(W.status + m, 8);
            }
            __syncthreads();
            const T *src = pb + (size_t)pn * mm * B;
            for (int e = tid; e < mm * nb; e += nthr) Pn[e] = ldcg(src + e);
            for (int i = tid; i < nb; i += nthr) piv[kb + i] = __ldcg(ppv + kb + i);
            __syncthreads();
            L = Pn;
        }
        // ---- the panel's row interchanges on the part's other columns ----
        for (int jl = tid; jl < ncl; jl += nthr) {
            if (own && jl >= jlp && jl < jlp + nb) continue;
            for (int kk = kb; kk < ke; kk++) {
                const int pv = piv[kk];
                if (pv != kk) {
                    const T a = Fl[kk + jl * mm];
                    Fl[kk + jl * mm] = Fl[pv + jl * mm];
                    Fl[pv + jl * mm] = a;
                }
            }
        }
        __syncthreads();
        // ---- U rows of the part's columns right of the panel ----
        const int jl0 = owned_below(ke);
        for (int jl = jl0 + tid; jl < ncl; jl += nthr) {
            T u[B];
#pragma unroll
            for (int q = 0; q < B; q++) u[q] = q < nb ? Fl[kb + q + jl * mm] : T(0);
#pragma unroll
            for (int q = 0; q < B; q++)
#pragma unroll
                for (int p = q + 1; p < B; p++)
                    if (p < nb) u[p] -= L[kb + p + q * mm] * u[q];
#pragma unroll
            for (int q = 0; q < B; q++)
                if (q < nb) Fl[kb + q + jl * mm] = u[q];
        }
        __syncthreads();
        // ---- their update below the panel, rank nb: a warp takes four
        // columns and up to 160 rows, the sums in registers ----
        const int nq = (ncl - jl0 + 3) >> 2, nr = (mm - ke + 159) / 160;
        for (int t = warp; t < nq * nr; t += nwarp) {
            const int c0 = jl0 + 4 * (t % nq), r0 = ke + 160 * (t / nq);
            T acc[5][4];
#pragma unroll
            for (int q = 0; q < 5; q++) {
                const int i = r0 + lane + 32 * q;
#pragma unroll
                for (int c = 0; c < 4; c++) acc[q][c] = (i < mm && c0 + c < ncl) ? Fl[i + (c0 + c) * mm] : T(0);
            }
            for (int q = 0; q < nb; q++) {
                T u[4], l[5];
#pragma unroll
                for (int c = 0; c < 4; c++) u[c] = c0 + c < ncl ? Fl[kb + q + (c0 + c) * mm] : T(0);
#pragma unroll
                for (int r = 0; r < 5; r++) {
                    const int i = r0 + lane + 32 * r;
                    l[r] = i < mm ? L[i + q * mm] : T(0);
                }
#pragma unroll
                for (int r = 0; r < 5; r++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[r][c] = fma(-l[r], u[c], acc[r][c]);
            }
#pragma unroll
            for (int q = 0; q < 5; q++) {
                const int i = r0 + lane + 32 * q;
#pragma unroll
                for (int c = 0; c < 4; c++)
                    if (i < mm && c0 + c < ncl) Fl[i + (c0 + c) * mm] = acc[q][c];
            }
        }
        __syncthreads();
    }
    // ---- store: first what the parent reads (columns ns..mm-1 whole, the
    // update matrix, and the part's share of the right-hand side), then
    // done(), then the L panel columns and the U rows of the part's columns
    // and the composed pivots, which nothing reads before the solves ----
    {
        T *out = fr + S.front_off[s];
        for (int e = tid; e < mm * ncl; e += nthr) {
            const int jl = e / mm, i = e - jl * mm, j = jof(jl);
            if (j >= ns && j < mm) out[i + (size_t)j * mm] = Fl[e];
        }
        if (RHS && jr >= 0) {
            for (int i = tid; i < ns; i += nthr) x[start + i] = (double)Fl[i + jr * mm];
            double *us = uv + S.uvec_off[s];
            for (int a = tid; a < mm - ns; a += nthr) us[a] = (double)Fl[ns + a + jr * mm];
        }
        __syncthreads();
        done();
        T *lo = lfac ? lfac + (size_t)m * S.lu_total + S.lu_off[s] : nullptr;
        T *uo = ufac + (size_t)m * S.lu_total + S.lu_off[s];
        for (int e = tid; e < mm * ncl; e += nthr) {
            const int jl = e / mm, i = e - jl * mm, j = jof(jl);
            if (j >= mm) continue;
            const T v = Fl[e];
            if (j < ns && lo) lo[i + (size_t)j * mm] = v;
            if (i < ns) uo[i + (size_t)j * ns] = v;
        }
        if (part == 0) {
            if (tid == 0) {
                for (int i = 0; i < ns; i++) perm[i] = i;
                for (int kk = 0; kk < ns; kk++) {
                    const int pv = piv[kk], t = perm[kk];
                    perm[kk] = perm[pv];
                    perm[pv] = t;
                }
            }
            __syncthreads();
            int *ipiv = S.ipiv + (size_t)m * S.n + start;
            for (int i = tid; i < ns; i += nthr) ipiv[i] = perm[i];
        }
    }
    __syncthreads();
}

// Shared memory of the factorisation kernels: the front (with the
// right-hand-side column) and 2 * front rows ints for the pivot indices and
// their composed permutation, each part 16-byte aligned; per warp of the
// warp kernel, for fronts of at most cap rows.
template <class T>
__host__ __device__ constexpr int warp_front_bytes(int cap) {
    return (cap * (cap + 1) * (int)sizeof(T) + 15) & ~15;
}
template <class T>
__host__ __device__ constexpr int warp_area_bytes(int cap) {
    return warp_front_bytes<T>(cap) + 2 * cap * 4;
}
template <class T>
__host__ __device__ inline int big_front_bytes(int max_front) {
    return (max_front * (max_front + 1) * (int)sizeof(T) + 15) & ~15;
}

// Ranks [r0, r1) of the order, one warp per task, fronts of at most cap
// rows; tasks claimed from counter ctr.
template <class T, bool RHS>
__global__ void __launch_bounds__(kThreads, 6) factor_small_kernel(DevProblem P, DevWork W, DevSym S, DevDag D,
                                                                T *fronts, T *lfac, T *ufac, const uint8_t *mask,
                                                                int want, int r0, int r1, int cap, int ctr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char *wbase = smem_raw + (size_t)warp * warp_area_bytes<T>(cap);
    T *F = reinterpret_cast<T *>(wbase);
    int *piv = reinterpret_cast<int *>(wbase + warp_front_bytes<T>(cap));
    const int M = P.M;
    const int epoch = *D.epoch;
    const int n_tasks = (r1 - r0) * M;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(D.ctr + ctr, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= n_tasks) break;
        const int s = D.order[r0 + t / M], m = t % M;
        if (mask[m] != want) continue;
        factor_front<T, RHS>(
            P, W, S, fronts, lfac, ufac, s, m, F, piv, WarpGroup{},
            [&] {
                if (!warp_wait_children(S, D, D.fdone, s, m, M, epoch, 0) && lane == 0) atomicOr(W.status + m, 8);
            },
            [&] {
                if (lane == 0) signal_done(D.fdone + (size_t)s * M + m, epoch);
            });
    }
}

// Ranks [r0, r1) of the order, G = 32 / W scenarios a warp: a task is a
// (supernode, group of G scenarios), and each W-lane group of the warp
// factors the front of one of them (fronts of at most cap rows, a buffer per
// group).  The fronts belong to the same supernode, so the groups run the
// same loops, and each instruction of a pivot column's steps (pivot search,
// reciprocal, multipliers) serves G fronts.  The FP64 elimination of small
// fronts is bound by the FP64 pipe, which charges a warp instruction the
// same whatever its active lanes, and these steps, one per column whatever
// the front's size, would otherwise occupy it once per front.  A group
// whose scenario this launch does not factor (M not a multiple of G, or
// masked out) follows the task's first factored scenario and stores
// nothing.
template <class T, bool RHS, int W>
__global__ void __launch_bounds__(kThreads, W == 16 ? 4 : 2) factor_group_kernel(DevProblem P, DevWork W_, DevSym S, DevDag D,
                                                                T *fronts, T *lfac, T *ufac, const uint8_t *mask,
                                                                int want, int r0, int r1, int cap, int ctr) {
    constexpr int G = 32 / W;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, gi = lane / W;
    unsigned char *gbase = smem_raw + (size_t)(G * warp + gi) * warp_area_bytes<T>(cap);
    T *F = reinterpret_cast<T *>(gbase);
    int *piv = reinterpret_cast<int *>(gbase + warp_front_bytes<T>(cap));
    const int M = P.M, Mg = (M + G - 1) / G;
    const int epoch = *D.epoch;
    const int n_tasks = (r1 - r0) * Mg;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(D.ctr + ctr, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= n_tasks) break;
        const int s = D.order[r0 + t / Mg], m0 = G * (t % Mg);
        int first = -1;
        bool act = false;
#pragma unroll
        for (int g = 0; g < G; g++) {
            const bool v = m0 + g < M && mask[m0 + g] == want;
            if (v && first < 0) first = m0 + g;
            if (g == gi) act = v;
        }
        if (first < 0) continue;
        const int m = act ? m0 + gi : first;
        factor_front<T, RHS>(
            P, W_, S, fronts, lfac, ufac, s, m, F, piv, LaneGroup<W>{act},
            [&] {
                if (!group_wait_children<W>(S, D, D.fdone, s, m, M, epoch) && (lane & (W - 1)) == 0 && act)
                    atomicOr(W_.status + m, 8);
            },
            [&] {
                if ((lane & (W - 1)) == 0 && act) signal_done(D.fdone + (size_t)s * M + m, epoch);
            });
    }
}

template <class T, bool RHS>
__global__ void __launch_bounds__(kThreads, 3) factor_big_kernel(DevProblem P, DevWork W, DevSym S, DevDag D,
                                                              T *fronts, T *lfac, T *ufac, const uint8_t *mask,
                                                              int want) {
    // FP64 factorisations split the large fronts of the tail (factor_part);
    // FP32 ones factor every front with one CTA (eliminate_cta)
    constexpr bool kSplit = sizeof(T) == 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *F = reinterpret_cast<T *>(smem_raw);
    int *piv = reinterpret_cast<int *>(smem_raw + big_front_bytes<T>(kSplit ? D.max_big_whole : D.max_big_front));
    __shared__ int s_task, s_ok;
    const int tid = threadIdx.x, lane = tid & 31;
    const int M = P.M;
    const int epoch = *D.epoch;
    const int n_tasks = kSplit ? D.big_units * M : (D.nsup - D.n_small) * M;
    const int t_tail = kSplit ? (D.tail0 - D.n_small) * M : n_tasks;   // first task of the tail
    // the tail's cumulative part counts, for the task decoding
    __shared__ int s_units[kSplitTailMax + 1];
    if (kSplit)
        for (int i = tid; i <= D.n_tail; i += blockDim.x) s_units[i] = D.tail_units[i];
    for (;;) {
        __syncthreads();
        if (tid == 0) s_task = atomicAdd(D.ctr + 1, 1);
        __syncthreads();
        const int t = s_task;
        if (t >= n_tasks) break;
        // task -> (rank, scenario, part): below the tail one task per
        // (rank, scenario); in the tail the parts of one (rank, scenario)
        // are consecutive tasks
        int rank, m, part = 0, np = 1;
        if (!kSplit || t < t_tail) {
            rank = D.n_small + t / M;
            m = t % M;
        } else {
            const int u = t - t_tail;
            int lo = 0, hi = D.n_tail - 1;   // the tail rank k with s_units[k] * M <= u
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_units[mid] * M <= u) lo = mid;
                else hi = mid - 1;
            }
            np = s_units[lo + 1] - s_units[lo];
            const int w = u - s_units[lo] * M;
            m = w / np;
            part = w - m * np;
            rank = D.tail0 + lo;
        }
        const int s = D.order[rank];
        if (mask[m] != want) continue;
        // the children (bounded wait), called by the assembly once the
        // entries that need nothing from them are in place
        auto wait = [&] {
            if (tid < 32) {
                const bool ok = warp_wait_children(S, D, D.fdone, s, m, M, epoch, D.n_small, kSplit);
                if (lane == 0) s_ok = ok;
            }
            __syncthreads();
            if (!s_ok && tid == 0) atomicOr(W.status + m, 8);
        };
        if (np == 1) {
            factor_front<T, RHS>(P, W, S, fronts, lfac, ufac, s, m, F, piv, BlockGroup{}, wait, [&] {
                if (tid == 0) signal_done(D.fdone + (size_t)s * M + m, epoch);
            });
        } else if constexpr (kSplit) {
            const int k = rank - D.tail0;
            factor_part<T, RHS>(P, W, S, D, fronts, lfac, ufac, s, m, k, part, np, epoch, smem_raw, wait, [&] {
                if (tid == 0) signal_done(D.pdone + ((size_t)k * M + m) * kMaxParts + part, epoch);
            });
        }
    }
}

// Re-arms the claim counters and moves to a new epoch: done flags of the
// previous solve no longer match.  The error flag stays raised until the
// host clears it.
__global__ void dag_begin_kernel(DevDag D) {
    if (threadIdx.x < 8) D.ctr[threadIdx.x] = 0;
    if (threadIdx.x == 0) *D.epoch += 1;
}

// The FP64 factorisation carries the right-hand side (fused forward solve);
// the FP32 one is reused across iterations and solved in gp_solve.cu.
template <class T>
struct FusedRhs {
    static constexpr bool value = false;
};
template <>
struct FusedRhs<double> {
    static constexpr bool value = true;
};

template <class T>
int configure_one(DagGrid &g, int nsm, int tiny_bytes, int small_bytes, int big_bytes) {
    constexpr bool R = FusedRhs<T>::value;
    int occ = 0;
    if (cudaFuncSetAttribute(factor_small_kernel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, small_bytes) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, factor_small_kernel<T, R>, kThreads, small_bytes) !=
            cudaSuccess || occ < 1)
        return -1;
    g.small = nsm * occ;
    if constexpr (sizeof(T) == 8) {
        // the tiny fronts of FP64 factorisations: two scenarios a warp
        if (cudaFuncSetAttribute(factor_group_kernel<T, R, kTinyLanes>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tiny_bytes) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, factor_group_kernel<T, R, kTinyLanes>, kThreads,
                                                          tiny_bytes) !=
                cudaSuccess || occ < 1)
            return -1;
        g.tiny = nsm * occ;
    } else {
        g.tiny = 0;
    }
    if (cudaFuncSetAttribute(factor_big_kernel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, big_bytes) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, factor_big_kernel<T, R>, kThreads, big_bytes) !=
            cudaSuccess || occ < 1)
        return -1;
    g.big = nsm * occ;
    return 0;
}

int blocks_for(int grid_max, long long warp_tasks, int per_block) {
    const long long need = (warp_tasks + per_block - 1) / per_block;
    return (int)(need < grid_max ? (need > 0 ? need : 1) : grid_max);
}

}  // namespace

int dag_configure(const DevDag &D, int fp32, DagGrid &g) {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    // FP32: every front of the CTA kernel whole; FP64: the fronts that are
    // not split whole, and the parts of the split ones
    const int mb = std::max(1, fp32 ? D.max_big_front : D.max_big_whole);
    const int small_bytes = kWarps * (fp32 ? warp_area_bytes<float>(kSmallFront) : warp_area_bytes<double>(kSmallFront));
    const int tiny_bytes = fp32 ? 0 : (32 / kTinyLanes) * kWarps * warp_area_bytes<double>(kTinyFront);
    const int whole = (fp32 ? big_front_bytes<float>(mb) : big_front_bytes<double>(mb)) + 2 * mb * 4;
    const int part = fp32 ? 0 : ((D.max_part_entries * 8 + 15) & ~15) + D.max_part_ints * 4;
    const int big_bytes = std::max(whole, part);
    const int rc = fp32 ? configure_one<float>(g, nsm, tiny_bytes, small_bytes, big_bytes)
                        : configure_one<double>(g, nsm, tiny_bytes, small_bytes, big_bytes);
    if (rc != 0) {
        cudaGetLastError();
        return -1;
    }
    g.tiny_bytes = tiny_bytes;
    g.small_bytes = small_bytes;
    g.big_bytes = big_bytes;
    return 0;
}

int dag_small_front() { return kSmallFront; }
int dag_tiny_front() { return kTinyFront; }

void launch_dag_begin(const DevDag &D, cudaStream_t st) { dag_begin_kernel<<<1, 32, 0, st>>>(D); }

namespace {
__global__ void recip_check_kernel(const double *x, double *r, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = recip(x[i]);
}
}  // namespace

void launch_recip_check(const double *x, double *r, int n, cudaStream_t st) {
    if (n > 0) recip_check_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, r, n);
}

template <class T>
void launch_dag_factor(const DevProblem &P, const DevWork &W, const DevSym &S, const DevDag &D, const DagGrid &g,
                       T *fronts, T *lfac, T *ufac, const uint8_t *mask, int want, cudaStream_t st) {
    constexpr bool R = FusedRhs<T>::value;
    const int n_tiny = sizeof(T) == 8 ? D.n_tiny : 0;
    constexpr int G = 32 / kTinyLanes;
    const long long tt = (long long)n_tiny * ((P.M + G - 1) / G), ts = (long long)(D.n_small - n_tiny) * P.M,
                    tb = (long long)(sizeof(T) == 8 ? D.big_units : D.nsup - D.n_small) * P.M;
    if constexpr (sizeof(T) == 8) {
        if (tt > 0)
            factor_group_kernel<T, R, kTinyLanes><<<blocks_for(g.tiny, tt, kWarps), kThreads, g.tiny_bytes, st>>>(
                P, W, S, D, fronts, lfac, ufac, mask, want, 0, n_tiny, kTinyFront, 7);
    }
    if (ts > 0)
        factor_small_kernel<T, R><<<blocks_for(g.small, ts, kWarps), kThreads, g.small_bytes, st>>>(
            P, W, S, D, fronts, lfac, ufac, mask, want, n_tiny, D.n_small, kSmallFront, 0);
    if (tb > 0)
        factor_big_kernel<T, R><<<blocks_for(g.big, tb, 1), kThreads, g.big_bytes, st>>>(P, W, S, D, fronts, lfac,
                                                                                          ufac, mask, want);
}

template void launch_dag_factor<double>(const DevProblem &, const DevWork &, const DevSym &, const DevDag &,
                                        const DagGrid &, double *, double *, double *, const uint8_t *, int,
                                        cudaStream_t);
template void launch_dag_factor<float>(const DevProblem &, const DevWork &, const DevSym &, const DevDag &,
                                       const DagGrid &, float *, float *, float *, const uint8_t *, int,
                                       cudaStream_t);

}  // namespace gp
