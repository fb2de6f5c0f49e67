// Triangular solves with the multifrontal factors of the reduced network
// matrix S, batched over scenarios: the replacement of cuDSS's solve phase
// (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2796-2799).
//
// The assembly tree is split once on the host (gp_api.cu, make_blocks):
//  - blocks: subtrees whose fronts are small.  One warp per (block,
//    scenario) keeps the block's right-hand-side vector, index maps and
//    pivot permutations in shared memory and runs the whole block: children
//    before parents forward, parents before children backward.  Blocks are
//    independent: no flags, no waits.  One launch per direction.
//  - top: the supernodes above the blocks.  A persistent dataflow kernel
//    whose warps claim (supernode, scenario) tasks in a topological order
//    (children first forward, parents first backward) and wait, bounded, on
//    the done flags of the tasks they depend on.  One launch per direction.
// Forward: blocks, then top.  Backward: top, then blocks.
//
// Within a front, one warp holds up to kMaxJ rows per lane in registers
// (row i in lane i % 32, register i / 32).  The unit-lower and upper
// triangular parts are swept column by column, the pivot value broadcast by
// a shuffle; the factor columns are loaded chunk by chunk ahead of the
// arithmetic, so that the sweep waits on memory once per chunk rather than
// once per column.  The U12 product of the backward solve is a row-dot
// product spread over all lanes.
//
// Front layout (column-major, leading dimension mm = ns + r): columns
// 0..ns-1 hold L (unit lower, below the diagonal), U11 above it and the
// reciprocal of each pivot on the diagonal; rows 0..ns-1 of columns
// ns..mm-1 hold U12.  ipiv holds per supernode the composed row permutation
// (pivot row i = assembled row ipiv[start + i]).  Arithmetic is in the
// factor type, chosen per scenario (FrontSel): double for exact Newton,
// float for the kept factors of the mixed solver; xperm and uvec are double.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "gp_internal.h"
#include "gp_warp.cuh"

namespace gp {

namespace {

constexpr unsigned FULL = kFullMask;
constexpr int kBlkWarps = 4;   // block tasks per CTA
constexpr int kTopWarps = 4;   // dataflow warps per CTA
constexpr int kMaxJ = 8;       // register rows per lane: fronts up to 256 rows

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

__device__ __forceinline__ bool use64(const FrontSel &fs, int m) {
    return fs.f32 == nullptr || (fs.mode != nullptr && fs.mode[m] == MX_EXACT);
}

template <class T>
__device__ __forceinline__ const T *front_base(const FrontSel &fs);
template <>
__device__ __forceinline__ const float *front_base<float>(const FrontSel &fs) {
    return fs.f32;
}
template <>
__device__ __forceinline__ const double *front_base<double>(const FrontSel &fs) {
    return fs.f64;
}

template <class T, int J>
__device__ __forceinline__ T pick(const T (&r)[J], int j) {
    T v = r[0];
#pragma unroll
    for (int q = 1; q < J; q++)
        if (j == q) v = r[q];
    return v;
}

template <class T, int J>
__device__ __forceinline__ void place(T (&r)[J], int j, T v) {
#pragma unroll
    for (int q = 0; q < J; q++)
        if (j == q) r[q] = v;
}

// Columns loaded per chunk: the chunk's loads stay in registers.
template <int J>
struct Chunk {
    static constexpr int value = J <= 1 ? 16 : (J <= 2 ? 8 : (J <= 4 ? 4 : 2));
};

// ---- forward elimination of one front ------------------------------------
// v[0..mm) (shared memory): the assembled right-hand side of the front.
// On return v[0..ns) holds the forward-solved pivot entries and v[ns..mm)
// the update vector for the parent.
template <class T, int J, class Perm>
__device__ void fwd_front_j(const T *__restrict__ F, Perm perm, int ns, int mm, T *v) {
    const int lane = threadIdx.x & 31;
    T r[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + 32 * j;
        r[j] = i < ns ? v[perm(i)] : (i < mm ? v[i] : T(0));
    }
    constexpr int CH = Chunk<J>::value;
    for (int k0 = 0; k0 < ns; k0 += CH) {
        T c[CH][J];
#pragma unroll
        for (int kk = 0; kk < CH; kk++) {
            const int k = k0 + kk;
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int i = lane + 32 * j;
                c[kk][j] = (k < ns && i > k && i < mm) ? F[i + k * mm] : T(0);
            }
        }
#pragma unroll
        for (int kk = 0; kk < CH; kk++) {
            const int k = k0 + kk;
            if (k < ns) {
                const T vk = __shfl_sync(FULL, pick(r, k >> 5), k & 31);
#pragma unroll
                for (int j = 0; j < J; j++) r[j] -= c[kk][j] * vk;
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + 32 * j;
        if (i < mm) v[i] = r[j];
    }
    __syncwarp();
}

// Fronts beyond the register path: the same steps on shared memory (sc: a
// scratch vector of ns entries).
template <class T, class Perm>
__device__ void fwd_front_smem(const T *__restrict__ F, Perm perm, int ns, int mm, T *v, T *sc) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < ns; i += 32) sc[i] = v[perm(i)];
    __syncwarp();
    for (int i = lane; i < ns; i += 32) v[i] = sc[i];
    __syncwarp();
    for (int k = 0; k < ns; k++) {
        const T vk = v[k];
        for (int i = k + 1 + lane; i < mm; i += 32) v[i] -= F[i + k * mm] * vk;
        __syncwarp();
    }
}

template <class T, class Perm>
__device__ void fwd_front(const T *F, Perm perm, int ns, int mm, T *v, T *sc) {
    switch ((mm + 31) >> 5) {
    case 1: fwd_front_j<T, 1>(F, perm, ns, mm, v); break;
    case 2: fwd_front_j<T, 2>(F, perm, ns, mm, v); break;
    case 3: fwd_front_j<T, 3>(F, perm, ns, mm, v); break;
    case 4: fwd_front_j<T, 4>(F, perm, ns, mm, v); break;
    case 5: fwd_front_j<T, 5>(F, perm, ns, mm, v); break;
    case 6: fwd_front_j<T, 6>(F, perm, ns, mm, v); break;
    case 7: fwd_front_j<T, 7>(F, perm, ns, mm, v); break;
    case 8: fwd_front_j<T, 8>(F, perm, ns, mm, v); break;
    default: fwd_front_smem<T>(F, perm, ns, mm, v, sc); break;
    }
}

// ---- backward substitution of one front ----------------------------------
// v[0..ns): forward-solved pivot entries; v[ns..mm): the solution entries of
// the update rows.  On return v[0..ns) holds the solution of the pivot rows.
template <class T>
__device__ __forceinline__ void bwd_u12(const T *__restrict__ F, int ns, int mm, T *v) {
    warp_row_dots<T>(F + ns * mm, 1, mm, ns, mm - ns, [&](int a) { return v[ns + a]; },
                     [&](int i, T acc) { v[i] -= acc; });
    __syncwarp();
}

template <class T, int J>
__device__ void bwd_front_j(const T *__restrict__ F, int ns, int mm, T *v) {
    const int lane = threadIdx.x & 31;
    bwd_u12<T>(F, ns, mm, v);
    T r[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + 32 * j;
        r[j] = i < ns ? v[i] : T(0);
    }
    constexpr int CH = Chunk<J>::value;
    for (int k1 = ns - 1; k1 >= 0; k1 -= CH) {
        T c[CH][J], d[CH];
#pragma unroll
        for (int kk = 0; kk < CH; kk++) {
            const int k = k1 - kk;
            d[kk] = k >= 0 ? F[k + k * mm] : T(0);
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int i = lane + 32 * j;
                c[kk][j] = (k >= 0 && i < k) ? F[i + k * mm] : T(0);
            }
        }
#pragma unroll
        for (int kk = 0; kk < CH; kk++) {
            const int k = k1 - kk;
            if (k >= 0) {
                const T tk = __shfl_sync(FULL, pick(r, k >> 5), k & 31) * d[kk];   // reciprocal pivot
                if (lane == (k & 31)) place(r, k >> 5, tk);
#pragma unroll
                for (int j = 0; j < J; j++) r[j] -= c[kk][j] * tk;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + 32 * j;
        if (i < ns) v[i] = r[j];
    }
    __syncwarp();
}

template <class T>
__device__ void bwd_front_smem(const T *__restrict__ F, int ns, int mm, T *v) {
    const int lane = threadIdx.x & 31;
    bwd_u12<T>(F, ns, mm, v);
    for (int k = ns - 1; k >= 0; k--) {
        const T tk = v[k] * F[k + k * mm];
        __syncwarp();
        if (lane == 0) v[k] = tk;
        for (int i = lane; i < k; i += 32) v[i] -= F[i + k * mm] * tk;
        __syncwarp();
    }
}

template <class T>
__device__ void bwd_front(const T *F, int ns, int mm, T *v) {
    switch ((mm + 31) >> 5) {
    case 1: bwd_front_j<T, 1>(F, ns, mm, v); break;
    case 2: bwd_front_j<T, 2>(F, ns, mm, v); break;
    case 3: bwd_front_j<T, 3>(F, ns, mm, v); break;
    case 4: bwd_front_j<T, 4>(F, ns, mm, v); break;
    case 5: bwd_front_j<T, 5>(F, ns, mm, v); break;
    case 6: bwd_front_j<T, 6>(F, ns, mm, v); break;
    case 7: bwd_front_j<T, 7>(F, ns, mm, v); break;
    case 8: bwd_front_j<T, 8>(F, ns, mm, v); break;
    default: bwd_front_smem<T>(F, ns, mm, v); break;
    }
}

// ---- blocks ----------------------------------------------------------------

// Shared-memory staging area of one warp's block task.  Every section, and
// the whole area, is a multiple of 16 bytes, so that the int4 entry tables
// of every warp's area (base = warp * total) stay 16-byte aligned.  The
// vector is sized for double whatever the factor type.
struct BlkLayout {
    int e0, e1, foff, map, piv, v, total;
};

__host__ __device__ inline BlkLayout blk_layout(const DevBlk &B) {
    BlkLayout o;
    o.e0 = 0;
    o.e1 = o.e0 + B.max_n * 16;
    o.foff = o.e1 + B.max_n * 16;
    o.map = o.foff + align16(B.max_n * 8);
    o.piv = o.map + align16(B.max_map * 4);
    o.v = o.piv + align16(B.max_p * 4);
    o.total = o.v + align16(B.max_v * 8);
    return o;
}

struct BlkTask {
    int e0, n;
    const int4 *E0, *E1;
    const long long *FO;
    const int *mp, *pv;
};

// Stages the block's entries, front offsets, index maps and (forward) the
// pivot permutations; the caller syncs.
__device__ BlkTask stage_block(const DevSym &S, const DevBlk &B, int blk, int m, unsigned char *base,
                               const BlkLayout &lay, const int *map, bool with_piv) {
    const int lane = threadIdx.x & 31;
    int4 *E0 = reinterpret_cast<int4 *>(base + lay.e0);
    int4 *E1 = reinterpret_cast<int4 *>(base + lay.e1);
    long long *FO = reinterpret_cast<long long *>(base + lay.foff);
    int *mp = reinterpret_cast<int *>(base + lay.map);
    int *pv = reinterpret_cast<int *>(base + lay.piv);
    const int e0 = B.blk_ptr[blk], n = B.blk_ptr[blk + 1] - e0;
    for (int q = lane; q < n; q += 32) {
        const int4 a = B.ent0[e0 + q];
        E0[q] = a;
        E1[q] = B.ent1[e0 + q];
        FO[q] = (long long)S.front_off[a.x];
    }
    const int mb = B.map_ptr[blk], nmap = B.map_ptr[blk + 1] - mb;
    for (int i = lane; i < nmap; i += 32) mp[i] = map[mb + i];
    __syncwarp();
    if (with_piv) {
        const int *ip = S.ipiv + (size_t)m * S.n;
        for (int q = 0; q < n; q++) {
            const int4 a = E0[q], b = E1[q];
            for (int i = lane; i < a.z; i += 32) pv[b.w + i] = ip[a.y + i];
        }
    }
    return BlkTask{e0, n, E0, E1, FO, mp, pv};
}

template <class T>
__device__ void fwd_block(const DevProblem &P, const DevWork &W, const DevSym &S, const FrontSel &fs,
                          const BlkTask &t, int m, T *vs) {
    const int lane = threadIdx.x & 31;
    const double *x = W.xperm + (size_t)m * P.n_red;
    for (int q = 0; q < t.n; q++) {
        const int4 a = t.E0[q], b = t.E1[q];
        for (int i = lane; i < a.z + a.w; i += 32) vs[b.y + i] = i < a.z ? (T)x[a.y + i] : T(0);
    }
    __syncwarp();
    const T *fr = front_base<T>(fs) + (size_t)m * S.front_total;
    double *xo = W.xperm + (size_t)m * P.n_red;
    double *uv = S.uvec + (size_t)m * S.uvec_total;
    for (int q = 0; q < t.n; q++) {
        const int4 a = t.E0[q], b = t.E1[q];
        const int ns = a.z, r = a.w;
        T *v = vs + b.y;
        const int *pv = t.pv + b.w;
        fwd_front<T>(fr + t.FO[q], [&](int i) { return pv[i]; }, ns, ns + r, v, v);
        for (int i = lane; i < ns; i += 32) xo[a.y + i] = (double)v[i];
        if (q < t.n - 1) {
            const int *pm = t.mp + b.z;
            for (int i = lane; i < r; i += 32) vs[pm[i]] += v[ns + i];
        } else {
            double *us = uv + S.uvec_off[a.x];
            for (int i = lane; i < r; i += 32) us[i] = (double)v[ns + i];
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(32 * kBlkWarps) fwd_blocks_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                                     FrontSel fs) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5;
    const long long task = (long long)blockIdx.x * kBlkWarps + warp;
    if (task >= (long long)B.nblk * P.M) return;
    const int blk = (int)(task / P.M), m = (int)(task % P.M);
    if (!W.active[m]) return;
    const bool d = use64(fs, m);
    if (d && fs.fused64) return;
    const BlkLayout lay = blk_layout(B);
    unsigned char *base = smem + (size_t)warp * lay.total;
    const BlkTask t = stage_block(S, B, blk, m, base, lay, B.map_fwd, true);
    __syncwarp();
    if (d) fwd_block<double>(P, W, S, fs, t, m, reinterpret_cast<double *>(base + lay.v));
    else fwd_block<float>(P, W, S, fs, t, m, reinterpret_cast<float *>(base + lay.v));
}

template <class T>
__device__ void bwd_block(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B,
                          const FrontSel &fs, const BlkTask &t, int blk, int m, T *vs) {
    const int lane = threadIdx.x & 31;
    double *x = W.xperm + (size_t)m * P.n_red;
    for (int q = 0; q < t.n; q++) {
        const int4 a = t.E0[q], b = t.E1[q];
        for (int i = lane; i < a.z; i += 32) vs[b.y + i] = (T)x[a.y + i];
    }
    const int xb = B.ext_ptr[blk], next = B.ext_ptr[blk + 1] - xb;
    for (int k = lane; k < next; k += 32) vs[B.ext_pos[xb + k]] = (T)x[B.ext_row[xb + k]];
    __syncwarp();
    const T *fr = front_base<T>(fs) + (size_t)m * S.front_total;
    for (int q = t.n - 1; q >= 0; q--) {
        const int4 a = t.E0[q], b = t.E1[q];
        const int ns = a.z, r = a.w;
        T *v = vs + b.y;
        const int *gm = t.mp + b.z;
        for (int c = lane; c < r; c += 32) v[ns + c] = vs[gm[c]];
        __syncwarp();
        bwd_front<T>(fr + t.FO[q], ns, ns + r, v);
        for (int i = lane; i < ns; i += 32) x[a.y + i] = (double)v[i];
    }
}

__global__ void __launch_bounds__(32 * kBlkWarps) bwd_blocks_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                                     FrontSel fs) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5;
    const long long task = (long long)blockIdx.x * kBlkWarps + warp;
    if (task >= (long long)B.nblk * P.M) return;
    const int blk = (int)(task / P.M), m = (int)(task % P.M);
    if (!W.active[m]) return;
    const BlkLayout lay = blk_layout(B);
    unsigned char *base = smem + (size_t)warp * lay.total;
    const BlkTask t = stage_block(S, B, blk, m, base, lay, B.map_bwd, false);
    __syncwarp();
    if (use64(fs, m)) bwd_block<double>(P, W, S, B, fs, t, blk, m, reinterpret_cast<double *>(base + lay.v));
    else bwd_block<float>(P, W, S, B, fs, t, blk, m, reinterpret_cast<float *>(base + lay.v));
}

// ---- top region: dataflow ---------------------------------------------------

template <class T>
__device__ void fwd_top_one(const DevProblem &P, const DevWork &W, const DevSym &S, const FrontSel &fs, int s,
                            int m, T *v, T *sc) {
    const int lane = threadIdx.x & 31;
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int r = S.row_ptr[s + 1] - S.row_ptr[s];
    const int mm = ns + r;
    double *x = W.xperm + (size_t)m * P.n_red;
    double *uv = S.uvec + (size_t)m * S.uvec_total;
    for (int i = lane; i < mm; i += 32) v[i] = i < ns ? (T)x[start + i] : T(0);
    __syncwarp();
    for (int q = S.child_ptr[s]; q < S.child_ptr[s + 1]; q++) {
        const int c = S.children[q];
        const int rc = S.row_ptr[c + 1] - S.row_ptr[c];
        const int *rel = S.relmap + S.relmap_ptr[c];
        const double *uc = uv + S.uvec_off[c];
        for (int a = lane; a < rc; a += 32) v[rel[a]] += (T)__ldcg(uc + a);
        __syncwarp();
    }
    const T *F = front_base<T>(fs) + (size_t)m * S.front_total + S.front_off[s];
    const int *ip = S.ipiv + (size_t)m * S.n + start;
    fwd_front<T>(F, [&](int i) { return ip[i]; }, ns, mm, v, sc);
    for (int i = lane; i < ns; i += 32) x[start + i] = (double)v[i];
    double *us = uv + S.uvec_off[s];
    for (int i = lane; i < r; i += 32) us[i] = (double)v[ns + i];
    __syncwarp();
}

template <class T>
__device__ void bwd_top_one(const DevProblem &P, const DevWork &W, const DevSym &S, const FrontSel &fs, int s,
                            int m, T *v) {
    const int lane = threadIdx.x & 31;
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int r = S.row_ptr[s + 1] - S.row_ptr[s];
    const int mm = ns + r;
    double *x = W.xperm + (size_t)m * P.n_red;
    const int *rows = S.rows + S.row_ptr[s];
    for (int i = lane; i < mm; i += 32) v[i] = (T)__ldcg(x + (i < ns ? start + i : rows[i - ns]));
    __syncwarp();
    const T *F = front_base<T>(fs) + (size_t)m * S.front_total + S.front_off[s];
    bwd_front<T>(F, ns, mm, v);
    for (int i = lane; i < ns; i += 32) x[start + i] = (double)v[i];
    __syncwarp();
}

// One warp waits for the top-region children of supernode s (scenario m).
__device__ bool wait_top_children(const DevSym &S, const DevBlk &B, const DevDag &D, int s, int m, int M,
                                  int epoch) {
    const int lane = threadIdx.x & 31;
    const int c0 = S.child_ptr[s], nc = S.child_ptr[s + 1] - c0;
    bool ok = true;
    for (int q = lane; q < nc; q += 32) {
        const int c = S.children[c0 + q];
        if (B.top_rank[c] >= 0) ok = wait_epoch(D.xdone + (size_t)c * M + m, epoch, D.err) && ok;
    }
    ok = __all_sync(FULL, ok);
    __syncwarp();
    return ok;
}

__global__ void __launch_bounds__(32 * kTopWarps) fwd_top_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                                 DevDag D, FrontSel fs) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double *vb = reinterpret_cast<double *>(smem) + (size_t)warp * 2 * B.top_max_front;
    const int M = P.M;
    const int epoch = *D.epoch;
    const int n_tasks = B.n_top * M;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(D.ctr + 2, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= n_tasks) break;
        const int s = B.top_order[t / M], m = t % M;
        if (!W.active[m]) continue;
        const bool d = use64(fs, m);
        if (d && fs.fused64) continue;
        if (!wait_top_children(S, B, D, s, m, M, epoch) && lane == 0) atomicOr(W.status + m, 8);
        if (d) fwd_top_one<double>(P, W, S, fs, s, m, vb, vb + B.top_max_front);
        else {
            float *vf = reinterpret_cast<float *>(vb);
            fwd_top_one<float>(P, W, S, fs, s, m, vf, vf + B.top_max_front);
        }
        if (lane == 0) signal_done(D.xdone + (size_t)s * M + m, epoch);
    }
}

__global__ void __launch_bounds__(32 * kTopWarps) bwd_top_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                                 DevDag D, FrontSel fs) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double *vb = reinterpret_cast<double *>(smem) + (size_t)warp * 2 * B.top_max_front;
    const int M = P.M;
    const int epoch = *D.epoch;
    const int n_tasks = B.n_top * M;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(D.ctr + 3, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= n_tasks) break;
        const int s = B.top_order[B.n_top - 1 - t / M], m = t % M;
        if (!W.active[m]) continue;
        const int par = D.parent[s];
        if (par >= 0) {
            bool ok = true;
            if (lane == 0) ok = wait_epoch(D.bdone + (size_t)par * M + m, epoch, D.err);
            ok = __shfl_sync(FULL, ok, 0);
            __syncwarp();
            if (!ok && lane == 0) atomicOr(W.status + m, 8);
        }
        if (use64(fs, m)) bwd_top_one<double>(P, W, S, fs, s, m, vb);
        else bwd_top_one<float>(P, W, S, fs, s, m, reinterpret_cast<float *>(vb));
        if (lane == 0) signal_done(D.bdone + (size_t)s * M + m, epoch);
    }
}

int grid_for(int resident, long long warp_tasks, int per_block) {
    const long long need = (warp_tasks + per_block - 1) / per_block;
    return (int)std::max<long long>(1, std::min<long long>(need, resident));
}

}  // namespace

int solve_block_front_limit() { return 32 * kMaxJ; }

int solve_configure(const DevBlk &B, SolveGrid &g) {
    int dev = 0, nsm = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return -1;
    g.blk_bytes = kBlkWarps * blk_layout(B).total;
    g.top_bytes = kTopWarps * 2 * std::max(1, B.top_max_front) * (int)sizeof(double);
    if (cudaFuncSetAttribute(fwd_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g.blk_bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(bwd_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g.blk_bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(fwd_top_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g.top_bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(bwd_top_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g.top_bytes) !=
            cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fwd_top_kernel, 32 * kTopWarps, g.top_bytes) !=
            cudaSuccess || occ < 1)
        return -1;
    g.top_fwd = nsm * occ;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bwd_top_kernel, 32 * kTopWarps, g.top_bytes) !=
            cudaSuccess || occ < 1)
        return -1;
    g.top_bwd = nsm * occ;
    return 0;
}

void launch_solve_fwd(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const DevDag &D,
                      const SolveGrid &g, FrontSel fs, cudaStream_t st) {
    const long long tasks = (long long)B.nblk * P.M;
    if (tasks > 0)
        fwd_blocks_kernel<<<(int)((tasks + kBlkWarps - 1) / kBlkWarps), 32 * kBlkWarps, g.blk_bytes, st>>>(P, W, S,
                                                                                                          B, fs);
    const long long top = (long long)B.n_top * P.M;
    if (top > 0)
        fwd_top_kernel<<<grid_for(g.top_fwd, top, kTopWarps), 32 * kTopWarps, g.top_bytes, st>>>(P, W, S, B, D, fs);
}

void launch_solve_bwd(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const DevDag &D,
                      const SolveGrid &g, FrontSel fs, cudaStream_t st) {
    const long long top = (long long)B.n_top * P.M;
    if (top > 0)
        bwd_top_kernel<<<grid_for(g.top_bwd, top, kTopWarps), 32 * kTopWarps, g.top_bytes, st>>>(P, W, S, B, D, fs);
    const long long tasks = (long long)B.nblk * P.M;
    if (tasks > 0)
        bwd_blocks_kernel<<<(int)((tasks + kBlkWarps - 1) / kBlkWarps), 32 * kBlkWarps, g.blk_bytes, st>>>(P, W, S,
                                                                                                          B, fs);
}

}  // namespace gp
