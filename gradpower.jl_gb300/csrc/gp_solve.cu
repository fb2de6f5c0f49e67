// Triangular solves with the multifrontal factors of the reduced network
// matrix S, batched over scenarios: the replacement of cuDSS's solve phase
// (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2788-2799).
//
// The assembly tree is split once on the host (gp_api.cu, build_blocks):
//  - blocks: subtrees of at most a few dozen supernodes whose factor slices
//    fit a warp's shared-memory budget.  One warp per (block, scenario)
//    stages everything its block needs with cp.async (factor slices, pivot
//    rows, right-hand side, index maps, and for the backward solve the
//    solution entries of the rows above the block), then runs the whole
//    block from shared memory: children before parents forward, parents
//    before children backward.  Blocks are independent: no flags, no waits.
//  - top: the remaining supernodes near the root, one CTA per scenario,
//    level by level with a barrier between levels (a level's supernodes go
//    to the CTA's warps).
// Forward: blocks, then top.  Backward: top, then blocks.
//
// Factor slices in a front (column-major, leading dimension mm = ns + r):
// columns 0..ns-1 hold L (unit lower, below the diagonal), U11 above it and
// the reciprocal of each pivot on the diagonal; rows 0..ns-1 of columns
// ns..mm-1 hold U12.  Arithmetic is in the factor type T (double for the
// exact Newton solve, float for the kept factors of the mixed solver); the
// global vectors (xperm, uvec) stay double.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "gp_internal.h"
#include "gp_warp.cuh"

namespace gp {

namespace {

constexpr int kBlkWarps = 2;       // independent block tasks per CTA
constexpr int kTopThreads = 1024;

__device__ __forceinline__ void cp_async(void *dst, const void *src, int bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

// Shared-memory layout of one warp's block staging area.  Every section,
// and the whole area, is a multiple of 16 bytes long, so that the int4
// entry tables of every warp's area (base = warp * total) stay 16-byte
// aligned.
struct BlkLayout {
    int l, v, xs, piv, e0, e1, foff, map, xe, total;
};

template <class T>
__host__ __device__ BlkLayout blk_layout(const DevBlk &B) {
    BlkLayout o;
    o.l = 0;
    o.v = o.l + align16(B.max_l * (int)sizeof(T));
    o.xs = o.v + align16(B.max_v * (int)sizeof(T));
    o.piv = o.xs + align16(B.max_p * 8);
    o.e0 = o.piv + align16(B.max_p * 4);
    o.e1 = o.e0 + B.max_n * 16;
    o.foff = o.e1 + B.max_n * 16;
    o.map = o.foff + align16(B.max_n * 8);
    o.xe = o.map + align16(B.max_map * 4);
    o.total = o.xe + align16(B.max_ext * 8);
    return o;
}
static_assert(align16(8) == 16 && align16(16) == 16, "align16");

template <class T>
__global__ void __launch_bounds__(32 * kBlkWarps) fwd_blocks_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                                     const T *fronts) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long task = (long long)blockIdx.x * kBlkWarps + warp;
    if (task >= (long long)B.nblk * P.M) return;
    const int blk = (int)(task / P.M), m = (int)(task % P.M);
    if (!W.active[m]) return;
    const BlkLayout lay = blk_layout<T>(B);
    unsigned char *base = smem + (size_t)warp * lay.total;
    T *Ls = reinterpret_cast<T *>(base + lay.l);
    T *vs = reinterpret_cast<T *>(base + lay.v);
    double *xs = reinterpret_cast<double *>(base + lay.xs);
    int *pv = reinterpret_cast<int *>(base + lay.piv);
    int4 *E0 = reinterpret_cast<int4 *>(base + lay.e0);
    int4 *E1 = reinterpret_cast<int4 *>(base + lay.e1);
    long long *FO = reinterpret_cast<long long *>(base + lay.foff);
    int *mp = reinterpret_cast<int *>(base + lay.map);
    const int e0 = B.blk_ptr[blk], n = B.blk_ptr[blk + 1] - e0;
    for (int q = lane; q < n; q += 32) {
        const int4 a = B.ent0[e0 + q];
        E0[q] = a;
        E1[q] = B.ent1[e0 + q];
        FO[q] = (long long)S.front_off[a.x];
    }
    __syncwarp();
    const T *fr = fronts + (size_t)m * S.front_total;
    const double *x = W.xperm + (size_t)m * P.n_red;
    const int *ip = S.ipiv + (size_t)m * S.n;
    const int mb = B.map_ptr[blk], nmap = B.map_ptr[blk + 1] - mb;
    for (int i = lane; i < nmap; i += 32) cp_async(mp + i, B.map_fwd + mb + i, 4);
    for (int q = 0; q < n; q++) {
        const int4 a = E0[q], b = E1[q];
        const int ns = a.z, mm = a.z + a.w;
        const T *src = fr + FO[q];
        for (int i = lane; i < mm * ns; i += 32) cp_async(Ls + b.x + i, src + i, (int)sizeof(T));
        for (int i = lane; i < ns; i += 32) {
            cp_async(xs + b.w + i, x + a.y + i, 8);
            cp_async(pv + b.w + i, ip + a.y + i, 4);
        }
    }
    cp_async_wait_all();
    __syncwarp();
    for (int q = 0; q < n; q++) {
        const int4 a = E0[q], b = E1[q];
        const int ns = a.z, r = a.w;
        for (int i = lane; i < ns; i += 32) vs[b.y + i] = (T)xs[b.w + i];
        for (int i = lane; i < r; i += 32) vs[b.y + ns + i] = T(0);
    }
    __syncwarp();
    double *uv = S.uvec + (size_t)m * S.uvec_total;
    double *xo = W.xperm + (size_t)m * P.n_red;
    for (int q = 0; q < n; q++) {
        const int4 a = E0[q], b = E1[q];
        const int s = a.x, start = a.y, ns = a.z, r = a.w, mm = ns + r;
        const T *Lq = Ls + b.x;
        T *t = vs + b.y, *u = t + ns;
        if (lane == 0)
            for (int k = 0; k < ns; k++) {
                const int p = pv[b.w + k];
                if (p != k) { const T tmp = t[k]; t[k] = t[p]; t[p] = tmp; }
            }
        __syncwarp();
        for (int k = 0; k < ns; k++) {
            const T tk = t[k];
            for (int i = k + 1 + lane; i < ns; i += 32) t[i] -= Lq[i + k * mm] * tk;
            __syncwarp();
        }
        warp_row_dots<T>(Lq + ns, 1, mm, r, ns, [&](int k) { return t[k]; }, [&](int i, T acc) { u[i] -= acc; });
        __syncwarp();
        if (q < n - 1) {
            const int *pm = mp + b.z;
            for (int i = lane; i < r; i += 32) vs[pm[i]] += u[i];
        } else {
            double *us = uv + S.uvec_off[s];
            for (int i = lane; i < r; i += 32) us[i] = (double)u[i];
        }
        for (int i = lane; i < ns; i += 32) xo[start + i] = (double)t[i];
        __syncwarp();
    }
}

template <class T>
__global__ void __launch_bounds__(32 * kBlkWarps) bwd_blocks_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                                     const T *fronts) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long task = (long long)blockIdx.x * kBlkWarps + warp;
    if (task >= (long long)B.nblk * P.M) return;
    const int blk = (int)(task / P.M), m = (int)(task % P.M);
    if (!W.active[m]) return;
    const BlkLayout lay = blk_layout<T>(B);
    unsigned char *base = smem + (size_t)warp * lay.total;
    T *Ls = reinterpret_cast<T *>(base + lay.l);
    T *vs = reinterpret_cast<T *>(base + lay.v);
    double *xs = reinterpret_cast<double *>(base + lay.xs);
    int4 *E0 = reinterpret_cast<int4 *>(base + lay.e0);
    int4 *E1 = reinterpret_cast<int4 *>(base + lay.e1);
    long long *FO = reinterpret_cast<long long *>(base + lay.foff);
    int *mp = reinterpret_cast<int *>(base + lay.map);
    double *xe = reinterpret_cast<double *>(base + lay.xe);
    const int e0 = B.blk_ptr[blk], n = B.blk_ptr[blk + 1] - e0;
    for (int q = lane; q < n; q += 32) {
        const int4 a = B.ent0[e0 + q];
        E0[q] = a;
        E1[q] = B.ent1[e0 + q];
        FO[q] = (long long)S.front_off[a.x];
    }
    __syncwarp();
    const T *fr = fronts + (size_t)m * S.front_total;
    double *x = W.xperm + (size_t)m * P.n_red;
    const int mb = B.map_ptr[blk], nmap = B.map_ptr[blk + 1] - mb;
    for (int i = lane; i < nmap; i += 32) cp_async(mp + i, B.map_bwd + mb + i, 4);
    const int xb = B.ext_ptr[blk], next = B.ext_ptr[blk + 1] - xb;
    for (int k = lane; k < next; k += 32) cp_async(xe + k, x + B.ext_row[xb + k], 8);
    for (int q = 0; q < n; q++) {
        const int4 a = E0[q], b = E1[q];
        const int ns = a.z, r = a.w, mm = ns + r;
        const T *src = fr + FO[q];
        // columns 0..ns-1, then U12 packed ns x r (leading dimension ns)
        for (int i = lane; i < mm * ns; i += 32) cp_async(Ls + b.x + i, src + i, (int)sizeof(T));
        T *u12 = Ls + b.x + mm * ns;
        for (int e = lane; e < ns * r; e += 32) {
            const int i = e % ns, c = e / ns;
            cp_async(u12 + e, src + i + (size_t)(ns + c) * mm, (int)sizeof(T));
        }
        for (int i = lane; i < ns; i += 32) cp_async(xs + b.w + i, x + a.y + i, 8);
    }
    cp_async_wait_all();
    __syncwarp();
    for (int q = 0; q < n; q++) {
        const int4 a = E0[q], b = E1[q];
        for (int i = lane; i < a.z; i += 32) vs[b.y + i] = (T)xs[b.w + i];
    }
    for (int k = lane; k < next; k += 32) vs[B.ext_pos[xb + k]] = (T)xe[k];
    __syncwarp();
    for (int q = n - 1; q >= 0; q--) {
        const int4 a = E0[q], b = E1[q];
        const int start = a.y, ns = a.z, r = a.w, mm = ns + r;
        const T *Lq = Ls + b.x;
        const T *u12 = Lq + mm * ns;
        T *t = vs + b.y;
        const int *gm = mp + b.z;
        warp_row_dots<T>(u12, 1, ns, ns, r, [&](int c) { return vs[gm[c]]; }, [&](int i, T acc) { t[i] -= acc; });
        __syncwarp();
        for (int k = ns - 1; k >= 0; k--) {
            const T tk = t[k] * Lq[k + k * mm];   // reciprocal of the pivot
            __syncwarp();
            if (lane == 0) t[k] = tk;
            for (int i = lane; i < k; i += 32) t[i] -= Lq[i + k * mm] * tk;
            __syncwarp();
        }
        for (int i = lane; i < ns; i += 32) x[start + i] = (double)t[i];
        __syncwarp();
    }
}

// Forward solve of one top-region supernode by one warp (children's update
// vectors read from global memory).
template <class T>
__device__ void fwd_top_one(const DevProblem &P, const DevWork &W, const DevSym &S, const T *fronts, int s, int m,
                            T *tv) {
    const int lane = threadIdx.x & 31;
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int r = S.row_ptr[s + 1] - S.row_ptr[s];
    const int mm = ns + r;
    double *x = W.xperm + (size_t)m * P.n_red;
    double *uv = S.uvec + (size_t)m * S.uvec_total;
    for (int i = lane; i < ns; i += 32) tv[i] = (T)x[start + i];
    for (int i = lane; i < r; i += 32) tv[ns + i] = T(0);
    __syncwarp();
    for (int q = S.child_ptr[s]; q < S.child_ptr[s + 1]; q++) {
        const int c = S.children[q];
        const int rc = S.row_ptr[c + 1] - S.row_ptr[c];
        const int *rel = S.relmap + S.relmap_ptr[c];
        const double *uc = uv + S.uvec_off[c];
        for (int a = lane; a < rc; a += 32) tv[rel[a]] += (T)uc[a];
        __syncwarp();
    }
    const T *F = fronts + (size_t)m * S.front_total + S.front_off[s];
    const int *ipiv = S.ipiv + (size_t)m * S.n + start;
    if (lane == 0)
        for (int k = 0; k < ns; k++) {
            const int pv = ipiv[k];
            if (pv != k) { const T t = tv[k]; tv[k] = tv[pv]; tv[pv] = t; }
        }
    __syncwarp();
    for (int k = 0; k < ns; k++) {
        const T tk = tv[k];
        for (int i = k + 1 + lane; i < ns; i += 32) tv[i] -= F[i + k * mm] * tk;
        __syncwarp();
    }
    double *us = uv + S.uvec_off[s];
    warp_row_dots<T>(F + ns, 1, mm, r, ns, [&](int k) { return tv[k]; },
                     [&](int a, T acc) { us[a] = (double)(tv[ns + a] - acc); });
    for (int i = lane; i < ns; i += 32) x[start + i] = (double)tv[i];
    __syncwarp();
}

template <class T>
__device__ void bwd_top_one(const DevProblem &P, const DevWork &W, const DevSym &S, const T *fronts, int s, int m,
                            T *tv) {
    const int lane = threadIdx.x & 31;
    const int start = S.sup_start[s];
    const int ns = S.sup_start[s + 1] - start;
    const int r = S.row_ptr[s + 1] - S.row_ptr[s];
    const int mm = ns + r;
    double *x = W.xperm + (size_t)m * P.n_red;
    const T *F = fronts + (size_t)m * S.front_total + S.front_off[s];
    const int *rows = S.rows + S.row_ptr[s];
    warp_row_dots<T>(F + (size_t)ns * mm, 1, mm, ns, r, [&](int a) { return (T)x[rows[a]]; },
                     [&](int i, T acc) { tv[i] = (T)x[start + i] - acc; });
    __syncwarp();
    for (int k = ns - 1; k >= 0; k--) {
        const T tk = tv[k] * F[k + k * mm];   // reciprocal of the pivot
        if (lane == 0) x[start + k] = (double)tk;
        for (int i = lane; i < k; i += 32) tv[i] -= F[i + k * mm] * tk;
        __syncwarp();
    }
}

template <class T>
__global__ void __launch_bounds__(kTopThreads) fwd_top_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                              const T *fronts) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int m = blockIdx.x, warp = threadIdx.x >> 5;
    if (!W.active[m]) return;
    T *tv = reinterpret_cast<T *>(smem) + (size_t)warp * B.top_max_front;
    for (int l = 0; l < B.n_top_levels; l++) {
        for (int q = B.top_ptr[l] + warp; q < B.top_ptr[l + 1]; q += kTopThreads / 32)
            fwd_top_one<T>(P, W, S, fronts, B.top_sups[q], m, tv);
        __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(kTopThreads) bwd_top_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                              const T *fronts) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int m = blockIdx.x, warp = threadIdx.x >> 5;
    if (!W.active[m]) return;
    T *tv = reinterpret_cast<T *>(smem) + (size_t)warp * B.top_max_front;
    for (int l = B.n_top_levels - 1; l >= 0; l--) {
        for (int q = B.top_ptr[l] + warp; q < B.top_ptr[l + 1]; q += kTopThreads / 32)
            bwd_top_one<T>(P, W, S, fronts, B.top_sups[q], m, tv);
        __syncthreads();
    }
}

template <class T>
int configure_solve_t(const DevBlk &B) {
    const int blk_bytes = kBlkWarps * blk_layout<T>(B).total;
    const int top_bytes = (kTopThreads / 32) * std::max(1, B.top_max_front) * (int)sizeof(T);
    if (cudaFuncSetAttribute(fwd_blocks_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, blk_bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(bwd_blocks_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, blk_bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(fwd_top_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, top_bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(bwd_top_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, top_bytes) !=
            cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return 0;
}

}  // namespace

int solve_configure(const DevBlk &B) {
    if (configure_solve_t<float>(B) != 0 || configure_solve_t<double>(B) != 0) return -1;
    return 0;
}

int solve_block_bytes(const DevBlk &B, int fp32) {
    return kBlkWarps * (fp32 ? blk_layout<float>(B).total : blk_layout<double>(B).total);
}

template <class T>
void launch_solve_fwd(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const T *fronts,
                      cudaStream_t st) {
    const long long tasks = (long long)B.nblk * P.M;
    if (tasks > 0)
        fwd_blocks_kernel<T><<<(int)((tasks + kBlkWarps - 1) / kBlkWarps), 32 * kBlkWarps,
                               kBlkWarps * blk_layout<T>(B).total, st>>>(P, W, S, B, fronts);
    if (B.n_top_levels > 0)
        fwd_top_kernel<T><<<P.M, kTopThreads, (kTopThreads / 32) * B.top_max_front * sizeof(T), st>>>(P, W, S, B,
                                                                                                      fronts);
}

template <class T>
void launch_solve_bwd(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const T *fronts,
                      cudaStream_t st) {
    if (B.n_top_levels > 0)
        bwd_top_kernel<T><<<P.M, kTopThreads, (kTopThreads / 32) * B.top_max_front * sizeof(T), st>>>(P, W, S, B,
                                                                                                      fronts);
    const long long tasks = (long long)B.nblk * P.M;
    if (tasks > 0)
        bwd_blocks_kernel<T><<<(int)((tasks + kBlkWarps - 1) / kBlkWarps), 32 * kBlkWarps,
                               kBlkWarps * blk_layout<T>(B).total, st>>>(P, W, S, B, fronts);
}

template void launch_solve_fwd<float>(const DevProblem &, const DevWork &, const DevSym &, const DevBlk &,
                                      const float *, cudaStream_t);
template void launch_solve_fwd<double>(const DevProblem &, const DevWork &, const DevSym &, const DevBlk &,
                                       const double *, cudaStream_t);
template void launch_solve_bwd<float>(const DevProblem &, const DevWork &, const DevSym &, const DevBlk &,
                                      const float *, cudaStream_t);
template void launch_solve_bwd<double>(const DevProblem &, const DevWork &, const DevSym &, const DevBlk &,
                                       const double *, cudaStream_t);

}  // namespace gp
