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
// Factorisation, in two launches:
//  - factor_small_kernel: supernodes whose whole subtree has fronts of at
//    most 32 rows, one warp per task, the front in shared memory;
//  - factor_big_kernel: the rest, one CTA per task.
// Partial pivoting is restricted to a supernode's pivot rows.  The FP32
// elimination is blocked (the pivot panel column by column, then one
// triangular solve and one update of the rest of the front); the FP64 one
// is right-looking.  The front
// (column-major, leading dimension = front rows) keeps L, U and the update
// matrix that the parent's extend-add reads.
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
// schedule rank is at least `from_rank`.
__device__ bool warp_wait_children(const DevSym &S, const DevDag &D, const int *done, int s, int m, int M,
                                   int epoch, int from_rank) {
    const int lane = threadIdx.x & 31;
    const int c0 = S.child_ptr[s], nc = S.child_ptr[s + 1] - c0;
    bool ok = true;
    for (int q = lane; q < nc; q += 32) {
        const int c = S.children[c0 + q];
        if (D.rank[c] >= from_rank) ok = wait_epoch(done + (size_t)c * M + m, epoch, D.err, D.wait_limit) && ok;
    }
    ok = __all_sync(FULL, ok);
    __syncwarp();
    return ok;
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

template <class T>
__device__ __forceinline__ int warp_pivot(const T *F, int mm, int k, int ns, bool &zero) {
    using K = typename KeyOf<T>::type;
    const int lane = threadIdx.x & 31;
    K bk = 0;
    int bi = k;
    for (int i = k + lane; i < ns; i += 32) {
        const K v = (K)mag_key(F[i + k * mm]);
        if (v > bk) { bk = v; bi = i; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const K ok = __shfl_xor_sync(FULL, bk, off);
        const int oi = __shfl_xor_sync(FULL, bi, off);
        if (ok > bk || (ok == bk && oi < bi)) { bk = ok; bi = oi; }
    }
    zero = bk == 0;
    return bi;
}

// Thread groups that factor one front: a warp, or the whole CTA.
struct WarpGroup {
    static constexpr int size = 32;
    __device__ int idx() const { return threadIdx.x & 31; }
    __device__ bool lead_warp() const { return true; }
    __device__ void sync() const { __syncwarp(); }
};
struct BlockGroup {
    static constexpr int size = kThreads;
    __device__ int idx() const { return threadIdx.x; }
    __device__ bool lead_warp() const { return threadIdx.x < 32; }
    __device__ void sync() const { __syncthreads(); }
};

// Columns per panel of the blocked FP32 elimination of CTA-sized fronts.
constexpr int kPanel = 8;

// Elimination of an FP32 front by the whole CTA (fronts above the warp
// size), blocked right-looking in panels of kPanel pivot columns:
//  (a) the panel, column by column: warp 0 finds the pivot among the pivot
//      rows (one max and one min reduction), swaps the two rows within the
//      panel, stores the multipliers and the pivot's reciprocal; the CTA then
//      updates the panel's later columns (a rank-1 update kPanel columns
//      wide, not the whole front);
//  (b) the panel's row interchanges applied to every other column;
//  (c) U of the panel rows right of it, by a forward substitution per
//      column with the panel's unit lower block (values in registers);
//  (d) the trailing update A -= L U (rank kPanel): a warp takes four
//      columns and its lanes the rows, each lane the same four columns of
//      up to five rows, sums in registers; the U entries are broadcasts and
//      the L and A entries consecutive across lanes (no bank conflicts).
// The front is left in the layout of the other paths: multipliers below the
// diagonal, U above it, the pivots' reciprocals on it, piv[k] the row
// swapped with row k at step k.
// Rows a lane holds in the register panel (rows of the panel beyond
// 32 * kPanelRows take the shared-memory path).
constexpr int kPanelRows = 5;

// Value of register slot j (a runtime index) of a per-lane array.
template <int J>
__device__ __forceinline__ float slot(const float (&r)[J], int j) {
    float v = r[0];
#pragma unroll
    for (int q = 1; q < J; q++)
        if (j == q) v = r[q];
    return v;
}

// Panel [kb, ke) of an FP32 front factored by one warp in registers: lane l
// holds rows kb + l + 32 j (j < J) of the panel's columns.  Per column: the
// pivot among the pivot rows by a max and a min reduction, the pivot row and
// row k exchanged through shuffles, the multipliers, the rank-1 update of
// the panel's later columns; no barrier.  Same operations, in the same
// order, as the shared-memory path.
template <int J>
__device__ void panel_warp32(float *F, int mm, int ns, int kb, int ke, int *piv, int *status) {
    const int lane = threadIdx.x & 31, nb = ke - kb;
    float P[J][kPanel];
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = kb + lane + 32 * j;
#pragma unroll
        for (int c = 0; c < kPanel; c++) P[j][c] = (i < mm && c < nb) ? F[i + (kb + c) * mm] : 0.0f;
    }
#pragma unroll
    for (int c = 0; c < kPanel; c++) {
        if (c >= nb) break;
        const int k = kb + c;
        // pivot among rows k..ns-1
        unsigned key = 0u;
        int bi = k;
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = kb + lane + 32 * j;
            const unsigned v = __float_as_uint(P[j][c]) & 0x7fffffffu;
            if (i >= k && i < ns && v > key) { key = v; bi = i; }
        }
        const unsigned kmax = __reduce_max_sync(FULL, key);
        const int pv = (int)__reduce_min_sync(FULL, key == kmax ? (unsigned)bi : 0xffffffffu);
        if (lane == 0) {
            piv[k] = pv;
            if (kmax == 0u) atomicOr(status, 4);
        }
        // the pivot row (u) and row k (w), broadcast
        const int lp = (pv - kb) & 31, jp = (pv - kb) >> 5, lk = (k - kb) & 31, jk = (k - kb) >> 5;
        float u[kPanel], w[kPanel];
#pragma unroll
        for (int q = 0; q < kPanel; q++) {
            float col[J];
#pragma unroll
            for (int j = 0; j < J; j++) col[j] = P[j][q];
            u[q] = __shfl_sync(FULL, slot(col, jp), lp);
            w[q] = __shfl_sync(FULL, slot(col, jk), lk);
        }
        const float inv = 1.0f / u[c];
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = kb + lane + 32 * j;
            if (i == pv && pv != k) {
#pragma unroll
                for (int q = 0; q < kPanel; q++) P[j][q] = w[q];
            }
            if (i == k) {
#pragma unroll
                for (int q = 0; q < kPanel; q++) P[j][q] = u[q];
                P[j][c] = inv;
            }
        }
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = kb + lane + 32 * j;
            if (i > k && i < mm) {
                const float l = P[j][c] * inv;
                P[j][c] = l;
#pragma unroll
                for (int q = 0; q < kPanel; q++)
                    if (q > c) P[j][q] -= l * u[q];
            }
        }
    }
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = kb + lane + 32 * j;
#pragma unroll
        for (int c = 0; c < kPanel; c++)
            if (i < mm && c < nb) F[i + (kb + c) * mm] = P[j][c];
    }
    __syncwarp();
}

__device__ void eliminate_cta32(float *F, int mm, int ns, int nc, int *piv, int *status) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    for (int kb = 0; kb < ns; kb += kPanel) {
        const int ke = min(ns, kb + kPanel), nb = ke - kb;
        // ---- (a) the panel ----
        if (mm - kb <= 32 * kPanelRows) {
            if (warp == 0) {
                switch ((mm - kb + 31) >> 5) {
                case 1: panel_warp32<1>(F, mm, ns, kb, ke, piv, status); break;
                case 2: panel_warp32<2>(F, mm, ns, kb, ke, piv, status); break;
                case 3: panel_warp32<3>(F, mm, ns, kb, ke, piv, status); break;
                case 4: panel_warp32<4>(F, mm, ns, kb, ke, piv, status); break;
                default: panel_warp32<5>(F, mm, ns, kb, ke, piv, status); break;
                }
            }
            __syncthreads();
        } else
        for (int k = kb; k < ke; k++) {
            if (warp == 0) {
                unsigned key = 0u;
                int bi = k;
                for (int i = k + lane; i < ns; i += 32) {
                    const unsigned v = __float_as_uint(F[i + k * mm]) & 0x7fffffffu;
                    if (v > key) { key = v; bi = i; }
                }
                const unsigned kmax = __reduce_max_sync(FULL, key);
                const int pv = (int)__reduce_min_sync(FULL, key == kmax ? (unsigned)bi : 0xffffffffu);
                if (lane == 0) {
                    piv[k] = pv;
                    if (kmax == 0u) atomicOr(status, 4);
                }
                if (pv != k && lane < nb) {
                    const float a = F[k + (kb + lane) * mm];
                    F[k + (kb + lane) * mm] = F[pv + (kb + lane) * mm];
                    F[pv + (kb + lane) * mm] = a;
                }
                __syncwarp();
                const float inv = 1.0f / F[k + k * mm];
                for (int i = k + 1 + lane; i < mm; i += 32) F[i + k * mm] *= inv;
                __syncwarp();
                if (lane == 0) F[k + k * mm] = inv;
            }
            __syncthreads();
            // rank-1 update of the panel's later columns, rows k+1..mm-1:
            // threads over rows, the columns split between the CTA's halves
            const int half = blockDim.x >> 1, h = tid >= half, rt = tid - h * half;
            for (int j = k + 1 + h; j < ke; j += 2) {
                const float u = F[k + j * mm];
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
                    const float a = F[k + j * mm];
                    F[k + j * mm] = F[pv + j * mm];
                    F[pv + j * mm] = a;
                }
            }
        }
        __syncthreads();
        if (ke >= nc) break;
        // ---- (c) U of the panel rows, columns ke..nc-1 ----
        for (int j = ke + tid; j < nc; j += blockDim.x) {
            float u[kPanel];
#pragma unroll
            for (int q = 0; q < kPanel; q++) u[q] = q < nb ? F[kb + q + j * mm] : 0.0f;
#pragma unroll
            for (int q = 0; q < kPanel; q++)
#pragma unroll
                for (int p = q + 1; p < kPanel; p++)
                    if (p < nb) u[p] -= F[kb + p + (kb + q) * mm] * u[q];
#pragma unroll
            for (int q = 0; q < kPanel; q++)
                if (q < nb) F[kb + q + j * mm] = u[q];
        }
        __syncthreads();
        // ---- (d) trailing update, rows ke..mm-1, columns ke..nc-1 ----
        // (rows in chunks of 160: five per lane)
        const int nq = (nc - ke + 3) >> 2, nr = (mm - ke + 159) / 160;
        for (int t = warp; t < nq * nr; t += nwarp) {
            const int c0 = ke + 4 * (t % nq), r0 = ke + 160 * (t / nq);
            float acc[5][4];
#pragma unroll
            for (int q = 0; q < 5; q++) {
                const int i = r0 + lane + 32 * q;
#pragma unroll
                for (int c = 0; c < 4; c++) acc[q][c] = (i < mm && c0 + c < nc) ? F[i + (c0 + c) * mm] : 0.0f;
            }
            for (int k = kb; k < ke; k++) {
                float u[4], l[5];
#pragma unroll
                for (int c = 0; c < 4; c++) u[c] = c0 + c < nc ? F[k + (c0 + c) * mm] : 0.0f;
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    const int i = r0 + lane + 32 * q;
                    l[q] = i < mm ? F[i + k * mm] : 0.0f;
                }
#pragma unroll
                for (int q = 0; q < 5; q++)
#pragma unroll
                    for (int c = 0; c < 4; c++) acc[q][c] = fmaf(-l[q], u[c], acc[q][c]);
            }
#pragma unroll
            for (int q = 0; q < 5; q++) {
                const int i = r0 + lane + 32 * q;
#pragma unroll
                for (int c = 0; c < 4; c++)
                    if (i < mm && c0 + c < nc) F[i + (c0 + c) * mm] = acc[q][c];
            }
        }
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
template <class T, bool RHS, class G>
__device__ void factor_front(const DevProblem &P, const DevWork &W, const DevSym &S, T *fronts, int s, int m, T *F,
                             int *piv, G g) {
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
    if (G::size > 32 && S.pa_base && S.pa_base[s] >= 0) {
        // CTA fronts: every entry sums its children's contributions (host
        // lists, child order) without a barrier between children; four
        // entries a thread per round, their loads issued together
        const int *pp = S.pa_ptr + S.pa_base[s];
        const int n2 = mm * mm;
        for (int p0 = idx; p0 < n2; p0 += 4 * step) {
            T acc[4];
            int e0[4], e1[4], kmax = 0;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int p = p0 + u * step;
                e0[u] = p < n2 ? pp[p] : 0;
                e1[u] = p < n2 ? pp[p + 1] : 0;
                acc[u] = p < n2 ? F[p] : T(0);
                kmax = max(kmax, e1[u] - e0[u]);
            }
            for (int k = 0; k < kmax; k++)
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (e0[u] + k < e1[u]) acc[u] += ldcg(fr + S.pa_src[e0[u] + k]);
#pragma unroll
            for (int u = 0; u < 4; u++)
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
    // FP64: right-looking, column by column over the whole front (every
    // update of a column is an independent FMA, which keeps GB300's long
    // FP64 pipeline busy).  FP32: blocked; the pivot panel (columns
    // 0..ns-1) column by column, then the right part (columns ns..nc-1) once:
    // U12 = L11^-1 A12 by forward substitution, one column per thread, and
    // A22 -= L21 U12, four entries per thread with the sums in registers.
    // Both give every entry the same operations in the same order.
    constexpr bool kBlocked = sizeof(T) == 4;
    if constexpr (kBlocked && G::size > 32) {
        static_assert(!RHS, "the FP32 factorisation carries no right-hand side");
        eliminate_cta32(F, mm, ns, nc, piv, W.status + m);
    } else {
    for (int k = 0; k < ns; k++) {
        if (g.lead_warp()) {
            const int lane = threadIdx.x & 31;
            bool zero;
            const int pv = warp_pivot(F, mm, k, ns, zero);
            if (lane == 0) {
                piv[k] = pv;
                if (zero) atomicOr(W.status + m, 4);
            }
            if (pv != k)
                for (int j = lane; j < nc; j += 32) {
                    const T a = F[k + j * mm];
                    F[k + j * mm] = F[pv + j * mm];
                    F[pv + j * mm] = a;
                }
            __syncwarp();
            const T inv = T(1) / F[k + k * mm];
            for (int i = k + 1 + lane; i < mm; i += 32) F[i + k * mm] *= inv;
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
    T *out = fr + S.front_off[s];
    for (int i = idx; i < mm * mm; i += step) out[i] = F[i];
    g.sync();
    int *ipiv = S.ipiv + (size_t)m * S.n + start;
    for (int i = idx; i < ns; i += step) ipiv[i] = piv[ns + i];
    if (RHS) {
        for (int i = idx; i < ns; i += step) x[start + i] = (double)F[mm * mm + i];
        double *us = uv + S.uvec_off[s];
        for (int a = idx; a < mm - ns; a += step) us[a] = (double)F[mm * mm + ns + a];
    }
    g.sync();
}

// Shared memory of the factorisation kernels: the front (with the
// right-hand-side column) and 2 * front rows ints for the pivot indices and
// their composed permutation, each part 16-byte aligned.
template <class T>
__host__ __device__ constexpr int small_front_bytes() {
    return (kSmallFront * (kSmallFront + 1) * (int)sizeof(T) + 15) & ~15;
}
template <class T>
__host__ __device__ constexpr int small_warp_bytes() {
    return small_front_bytes<T>() + 2 * kSmallFront * 4;
}
template <class T>
__host__ __device__ inline int big_front_bytes(int max_front) {
    return (max_front * (max_front + 1) * (int)sizeof(T) + 15) & ~15;
}

template <class T, bool RHS>
__global__ void __launch_bounds__(kThreads, 6) factor_small_kernel(DevProblem P, DevWork W, DevSym S, DevDag D,
                                                                T *fronts, const uint8_t *mask, int want) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char *wbase = smem_raw + (size_t)warp * small_warp_bytes<T>();
    T *F = reinterpret_cast<T *>(wbase);
    int *piv = reinterpret_cast<int *>(wbase + small_front_bytes<T>());
    const int M = P.M;
    const int epoch = *D.epoch;
    const int n_tasks = D.n_small * M;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(D.ctr + 0, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= n_tasks) break;
        const int s = D.order[t / M], m = t % M;
        if (mask[m] != want) continue;
        if (!warp_wait_children(S, D, D.fdone, s, m, M, epoch, 0) && lane == 0) atomicOr(W.status + m, 8);
        factor_front<T, RHS>(P, W, S, fronts, s, m, F, piv, WarpGroup{});
        if (lane == 0) signal_done(D.fdone + (size_t)s * M + m, epoch);
    }
}

template <class T, bool RHS>
__global__ void __launch_bounds__(kThreads, 3) factor_big_kernel(DevProblem P, DevWork W, DevSym S, DevDag D,
                                                              T *fronts, const uint8_t *mask, int want) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *F = reinterpret_cast<T *>(smem_raw);
    int *piv = reinterpret_cast<int *>(smem_raw + big_front_bytes<T>(D.max_big_front));
    __shared__ int s_task, s_ok;
    const int tid = threadIdx.x, lane = tid & 31;
    const int M = P.M;
    const int epoch = *D.epoch;
    const int n_tasks = (D.nsup - D.n_small) * M;
    for (;;) {
        __syncthreads();
        if (tid == 0) s_task = atomicAdd(D.ctr + 1, 1);
        __syncthreads();
        const int t = s_task;
        if (t >= n_tasks) break;
        const int s = D.order[D.n_small + t / M], m = t % M;
        if (mask[m] != want) continue;
        if (tid < 32) {
            const bool ok = warp_wait_children(S, D, D.fdone, s, m, M, epoch, D.n_small);
            if (lane == 0) s_ok = ok;
        }
        __syncthreads();
        if (!s_ok && tid == 0) atomicOr(W.status + m, 8);
        factor_front<T, RHS>(P, W, S, fronts, s, m, F, piv, BlockGroup{});
        if (tid == 0) signal_done(D.fdone + (size_t)s * M + m, epoch);
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
int configure_one(DagGrid &g, int nsm, int small_bytes, int big_bytes) {
    constexpr bool R = FusedRhs<T>::value;
    int occ = 0;
    if (cudaFuncSetAttribute(factor_small_kernel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, small_bytes) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, factor_small_kernel<T, R>, kThreads, small_bytes) !=
            cudaSuccess || occ < 1)
        return -1;
    g.small = nsm * occ;
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
    const int mb = std::max(1, D.max_big_front);
    const int small_bytes = kWarps * (fp32 ? small_warp_bytes<float>() : small_warp_bytes<double>());
    const int big_bytes = (fp32 ? big_front_bytes<float>(mb) : big_front_bytes<double>(mb)) + 2 * mb * 4;
    const int rc = fp32 ? configure_one<float>(g, nsm, small_bytes, big_bytes)
                        : configure_one<double>(g, nsm, small_bytes, big_bytes);
    if (rc != 0) {
        cudaGetLastError();
        return -1;
    }
    g.small_bytes = small_bytes;
    g.big_bytes = big_bytes;
    return 0;
}

int dag_small_front() { return kSmallFront; }

void launch_dag_begin(const DevDag &D, cudaStream_t st) { dag_begin_kernel<<<1, 32, 0, st>>>(D); }

template <class T>
void launch_dag_factor(const DevProblem &P, const DevWork &W, const DevSym &S, const DevDag &D, const DagGrid &g,
                       T *fronts, const uint8_t *mask, int want, cudaStream_t st) {
    constexpr bool R = FusedRhs<T>::value;
    const long long ts = (long long)D.n_small * P.M, tb = (long long)(D.nsup - D.n_small) * P.M;
    if (ts > 0)
        factor_small_kernel<T, R><<<blocks_for(g.small, ts, kWarps), kThreads, g.small_bytes, st>>>(P, W, S, D,
                                                                                                   fronts, mask, want);
    if (tb > 0)
        factor_big_kernel<T, R><<<blocks_for(g.big, tb, 1), kThreads, g.big_bytes, st>>>(P, W, S, D, fronts, mask, want);
}

template void launch_dag_factor<double>(const DevProblem &, const DevWork &, const DevSym &, const DevDag &,
                                        const DagGrid &, double *, const uint8_t *, int, cudaStream_t);
template void launch_dag_factor<float>(const DevProblem &, const DevWork &, const DevSym &, const DevDag &,
                                       const DagGrid &, float *, const uint8_t *, int, cudaStream_t);

}  // namespace gp
