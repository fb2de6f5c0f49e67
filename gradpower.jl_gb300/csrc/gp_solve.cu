// Triangular solves with the multifrontal factors of the reduced network
// matrix S, batched over scenarios: the replacement of cuDSS's solve phase
// (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2796-2799).
//
// The assembly tree is split once on the host (gp_api.cu, make_blocks):
//  - blocks: subtrees whose fronts are small.  One warp per (block,
//    scenario) keeps the block's right-hand-side vector, index maps and
//    pivot permutations in shared memory and runs the whole block: children
//    before parents forward, parents before children backward.  Inside a
//    block nothing waits; a block hands its root's update vector to the top
//    region (forward) and takes the entries of its external rows from it
//    (backward).
//  - top: the supernodes above the blocks, tasks (supernode, scenario)
//    claimed in a topological order (children first forward, parents first
//    backward).  A task copies the part of the front it needs into shared
//    memory (cp.async, all threads) and loads its own right-hand-side
//    entries before it waits, bounded, on the tasks it depends on; one warp
//    then sweeps the front from shared memory.
//  - in the forward pass the top region's first levels (fronts of at most
//    kBlkFront rows) are tasks of one warp each, a supernode per task
//    waiting on its children.
// One persistent kernel per direction runs them all: forward, the warps
// claim the block tasks, then the lower top tasks, and the CTAs then the
// rest of the top region; backward, the CTAs claim the top tasks, then the
// warps the block tasks.
//
// Hand-offs between tasks.  On FP64 factors a task signals a done flag
// (release store after a barrier) and its dependants poll the flag, then
// read the values.  On FP32 factors the values themselves carry the epoch
// (tagged 64-bit words, gp_warp.cuh): a block root or top task stores its
// update vector (forward) or its solved pivot entries (backward) as tagged
// words, and the tasks that consume them poll those words directly, so that
// a hand-off costs one store and the polls that see it, with no fence.
//
// Within a front, one warp holds up to kMaxJ rows per lane in registers
// (row i in lane i % 32, register i / 32).  The unit-lower and upper
// triangular parts are swept column by column, the pivot value broadcast by
// a shuffle; the factor columns are read chunk by chunk ahead of the
// arithmetic.  The U12 product of the backward solve is a row-dot product
// spread over all lanes.
//
// Factor layout: the factorisation writes each supernode's factors twice,
// in solve order (DevSym::lu_off; a block's supernodes are consecutive, so a
// block's factors are one contiguous range).  The forward pass reads the L
// panel (mm x ns, column-major, leading dimension mm = ns + r: unit-lower L
// below the diagonal), the backward pass the U rows (ns x mm, leading
// dimension ns: U11 with the reciprocal of each pivot on its diagonal, then
// U12), so that each pass streams only the entries it uses, contiguously.
// ipiv holds per supernode the composed row permutation (pivot row i =
// assembled row ipiv[start + i]).  Arithmetic is in the factor type, chosen
// per scenario (FrontSel): double for exact Newton, float for the kept
// factors of the mixed solver; xperm and uvec are double.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>

#include "gp_internal.h"
#include "gp_warp.cuh"

namespace gp {

namespace {

constexpr unsigned FULL = kFullMask;
constexpr int kBlkWarps = 4;   // block tasks per CTA
constexpr int kTopThreads = 128;             // threads of a top-region task
constexpr int kTopStage = 20 * 1024;         // shared memory for a task's factor columns
constexpr int kMaxJ = 8;       // register rows per lane: fronts up to 256 rows
constexpr int kBlkFront = 64;  // largest front inside a block (two rows per lane)

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

// Shared memory of one top-region CTA: two vectors sized for double and one
// int vector (top_max_front entries each), then the factor staging area.
__host__ __device__ constexpr int top_vec_bytes(int tmf) { return align16(tmf * (8 + 8 + 4)); }
// the forward tasks' extend-add lists (row pointers, then entries)
__host__ __device__ constexpr int top_idx_bytes(int tmf, int mx) { return align16((tmf + 1) * 4) + align16(mx * 4); }

__device__ __forceinline__ void cp_async(void *dst, const void *src, int bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Solves on FP32 factors pass values between tasks as tagged words
// (gp_warp.cuh); solves on FP64 factors keep the done flags.
template <class T>
struct Tagged {
    static constexpr bool value = std::is_same<T, float>::value;
};

// Thread tid of nthr polls the tagged words src[idx(e)], e = tid, tid +
// nthr, ... < n, until each carries epoch, and hands each value to put(e,
// v); four loads in flight per thread before the first poll.  False when a
// wait gave up.
template <class Idx, class Put>
__device__ bool poll_tagged(const unsigned long long *src, int n, int tid, int nthr, int epoch, const DevDag &D,
                            Idx idx, Put put) {
    bool ok = true;
    for (int e0 = tid; e0 < n; e0 += 4 * nthr) {
        unsigned long long w[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = e0 + q * nthr;
            w[q] = e < n ? ld_relaxed_u64(src + idx(e)) : 0ull;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = e0 + q * nthr;
            if (e < n) {
                if (!tag_ok(w[q], epoch)) w[q] = wait_tag(src + idx(e), epoch, D.err, D.wait_limit, ok);
                put(e, tag_val(w[q]));
            }
        }
    }
    return ok;
}

__device__ __forceinline__ bool use64(const FrontSel &fs, int m) {
    return fs.l32 == nullptr || (fs.mode != nullptr && fs.mode[m] == MX_EXACT);
}

// The solve-ordered factors of scenario m in the factor type: the L panels
// (forward) and the U rows (backward), both indexed by DevSym::lu_off.
template <class T>
struct Fac;
template <>
struct Fac<float> {
    static __device__ __forceinline__ const float *l(const FrontSel &fs) { return fs.l32; }
    static __device__ __forceinline__ const float *u(const FrontSel &fs) { return fs.u32; }
};
template <>
struct Fac<double> {
    static __device__ __forceinline__ const double *l(const FrontSel &fs) { return fs.l64; }
    static __device__ __forceinline__ const double *u(const FrontSel &fs) { return fs.u64; }
};
template <class T>
__device__ __forceinline__ const T *lfac(const FrontSel &fs, const DevSym &S, int m) {
    return Fac<T>::l(fs) + (size_t)(fs.shared ? 0 : m) * S.lu_total;
}
template <class T>
__device__ __forceinline__ const T *ufac(const FrontSel &fs, const DevSym &S, int m) {
    return Fac<T>::u(fs) + (size_t)(fs.shared ? 0 : m) * S.lu_total;
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

// Columns read per chunk of a sweep.
template <int J>
struct Chunk {
    static constexpr int value = J <= 2 ? 8 : (J <= 4 ? 4 : 2);
};

// ---- forward elimination -------------------------------------------------
// Sweeps columns k in [k0, k1) of the unit-lower factor over rows (k, mm):
// v[i] -= L(i, k) v[k], with L(i, k) = F[i + (k - kbase) * ld].  v[0..mm)
// is in shared memory; rows below ns are first gathered through the pivot
// permutation perm (identity after the first chunk).
// LW < 32: the warp works as 32 / LW segments of LW lanes, each segment on
// its own vector v and front F (same shape), rows i = lane + LW * j.
template <class T, int J, class Perm, int CH = Chunk<J>::value, int LW = 32>
__device__ void fwd_cols_j(const T *__restrict__ F, int ld, int kbase, int k0, int k1, int ns, int mm, T *v,
                           Perm perm) {
    const int lane = threadIdx.x & (LW - 1);
    T r[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + LW * j;
        r[j] = i < ns ? v[perm(i)] : (i < mm ? v[i] : T(0));
    }
    for (int kc = k0; kc < k1; kc += CH) {
        T c[CH][J];
#pragma unroll
        for (int kk = 0; kk < CH; kk++) {
            const int k = kc + kk;
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int i = lane + LW * j;
                c[kk][j] = (k < k1 && i > k && i < mm) ? F[i + (k - kbase) * ld] : T(0);
            }
        }
#pragma unroll
        for (int kk = 0; kk < CH; kk++) {
            const int k = kc + kk;
            if (k < k1) {
                const T vk = __shfl_sync(FULL, pick(r, k / LW), k % LW, LW);
#pragma unroll
                for (int j = 0; j < J; j++) r[j] -= c[kk][j] * vk;
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + LW * j;
        if (i < mm) v[i] = r[j];
    }
    __syncwarp();
}

// Fronts beyond the register path: the same sweep on shared memory, the
// permutation gathered through sc.
template <class T, class Perm>
__device__ void fwd_cols_smem(const T *__restrict__ F, int ld, int kbase, int k0, int k1, int ns, int mm, T *v,
                              T *sc, Perm perm, bool gather) {
    const int lane = threadIdx.x & 31;
    if (gather) {
        for (int i = lane; i < ns; i += 32) sc[i] = v[perm(i)];
        __syncwarp();
        for (int i = lane; i < ns; i += 32) v[i] = sc[i];
        __syncwarp();
    }
    for (int k = k0; k < k1; k++) {
        const T vk = v[k];
        for (int i = k + 1 + lane; i < mm; i += 32) v[i] -= F[i + (k - kbase) * ld] * vk;
        __syncwarp();
    }
}

struct Ident {
    __device__ int operator()(int i) const { return i; }
};

template <class T, class Perm>
__device__ void fwd_cols(const T *F, int ld, int kbase, int k0, int k1, int ns, int mm, T *v, T *sc, Perm perm,
                         bool gather) {
    if (!gather) {
        switch ((mm + 31) >> 5) {
        case 1: fwd_cols_j<T, 1>(F, ld, kbase, k0, k1, ns, mm, v, Ident{}); return;
        case 2: fwd_cols_j<T, 2>(F, ld, kbase, k0, k1, ns, mm, v, Ident{}); return;
        case 3: fwd_cols_j<T, 3>(F, ld, kbase, k0, k1, ns, mm, v, Ident{}); return;
        case 4: fwd_cols_j<T, 4>(F, ld, kbase, k0, k1, ns, mm, v, Ident{}); return;
        case 5: fwd_cols_j<T, 5>(F, ld, kbase, k0, k1, ns, mm, v, Ident{}); return;
        case 6: fwd_cols_j<T, 6>(F, ld, kbase, k0, k1, ns, mm, v, Ident{}); return;
        case 7: fwd_cols_j<T, 7>(F, ld, kbase, k0, k1, ns, mm, v, Ident{}); return;
        case 8: fwd_cols_j<T, 8>(F, ld, kbase, k0, k1, ns, mm, v, Ident{}); return;
        default: fwd_cols_smem<T>(F, ld, kbase, k0, k1, ns, mm, v, sc, Ident{}, false); return;
        }
    }
    switch ((mm + 31) >> 5) {
    case 1: fwd_cols_j<T, 1>(F, ld, kbase, k0, k1, ns, mm, v, perm); return;
    case 2: fwd_cols_j<T, 2>(F, ld, kbase, k0, k1, ns, mm, v, perm); return;
    case 3: fwd_cols_j<T, 3>(F, ld, kbase, k0, k1, ns, mm, v, perm); return;
    case 4: fwd_cols_j<T, 4>(F, ld, kbase, k0, k1, ns, mm, v, perm); return;
    case 5: fwd_cols_j<T, 5>(F, ld, kbase, k0, k1, ns, mm, v, perm); return;
    case 6: fwd_cols_j<T, 6>(F, ld, kbase, k0, k1, ns, mm, v, perm); return;
    case 7: fwd_cols_j<T, 7>(F, ld, kbase, k0, k1, ns, mm, v, perm); return;
    case 8: fwd_cols_j<T, 8>(F, ld, kbase, k0, k1, ns, mm, v, perm); return;
    default: fwd_cols_smem<T>(F, ld, kbase, k0, k1, ns, mm, v, sc, perm, true); return;
    }
}

// ---- backward substitution -----------------------------------------------
// U12 columns c in [c0, c1) (front columns, ns <= c < mm):
// v[i] -= U(i, c) v[c] for i < ns, U(i, c) = F[i + (c - cbase) * ld].
template <class T, int LW = 32>
__device__ __forceinline__ void bwd_u12(const T *__restrict__ F, int ld, int cbase, int c0, int c1, int ns, T *v) {
    warp_row_dots<T, LW>(F + (c0 - cbase) * ld, 1, ld, ns, c1 - c0, [&](int a) { return v[c0 + a]; },
                         [&](int i, T acc) { v[i] -= acc; });
    __syncwarp();
}

// U11 columns k from k1 - 1 down to k0: v[k] *= U(k, k) (the stored
// reciprocal pivot), then v[i] -= U(i, k) v[k] for i < k.
template <class T, int J, int CH = Chunk<J>::value, int LW = 32>
__device__ void bwd_cols_j(const T *__restrict__ F, int ld, int kbase, int k0, int k1, int ns, T *v) {
    const int lane = threadIdx.x & (LW - 1);
    T r[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + LW * j;
        r[j] = i < ns ? v[i] : T(0);
    }
    for (int kc = k1 - 1; kc >= k0; kc -= CH) {
        T c[CH][J], d[CH];
#pragma unroll
        for (int kk = 0; kk < CH; kk++) {
            const int k = kc - kk;
            d[kk] = k >= k0 ? F[k + (k - kbase) * ld] : T(0);
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int i = lane + LW * j;
                c[kk][j] = (k >= k0 && i < k) ? F[i + (k - kbase) * ld] : T(0);
            }
        }
#pragma unroll
        for (int kk = 0; kk < CH; kk++) {
            const int k = kc - kk;
            if (k >= k0) {
                const T tk = __shfl_sync(FULL, pick(r, k / LW), k % LW, LW) * d[kk];
                if (lane == k % LW) place(r, k / LW, tk);
#pragma unroll
                for (int j = 0; j < J; j++) r[j] -= c[kk][j] * tk;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + LW * j;
        if (i < ns) v[i] = r[j];
    }
    __syncwarp();
}

template <class T>
__device__ void bwd_cols_smem(const T *__restrict__ F, int ld, int kbase, int k0, int k1, T *v) {
    const int lane = threadIdx.x & 31;
    for (int k = k1 - 1; k >= k0; k--) {
        const T tk = v[k] * F[k + (k - kbase) * ld];
        __syncwarp();
        if (lane == 0) v[k] = tk;
        for (int i = lane; i < k; i += 32) v[i] -= F[i + (k - kbase) * ld] * tk;
        __syncwarp();
    }
}

template <class T>
__device__ void bwd_cols(const T *F, int ld, int kbase, int k0, int k1, int ns, T *v) {
    switch ((ns + 31) >> 5) {
    case 1: bwd_cols_j<T, 1>(F, ld, kbase, k0, k1, ns, v); return;
    case 2: bwd_cols_j<T, 2>(F, ld, kbase, k0, k1, ns, v); return;
    case 3: bwd_cols_j<T, 3>(F, ld, kbase, k0, k1, ns, v); return;
    case 4: bwd_cols_j<T, 4>(F, ld, kbase, k0, k1, ns, v); return;
    case 5: bwd_cols_j<T, 5>(F, ld, kbase, k0, k1, ns, v); return;
    case 6: bwd_cols_j<T, 6>(F, ld, kbase, k0, k1, ns, v); return;
    case 7: bwd_cols_j<T, 7>(F, ld, kbase, k0, k1, ns, v); return;
    case 8: bwd_cols_j<T, 8>(F, ld, kbase, k0, k1, ns, v); return;
    default: bwd_cols_smem<T>(F, ld, kbase, k0, k1, v); return;
    }
}

// Block fronts (at most kBlkFront rows): the whole front from global memory.
// (block fronts are small: four columns per chunk)
template <class T, class Perm, int LW = 32>
__device__ void fwd_front_blk(const T *F, Perm perm, int ns, int mm, T *v) {
    static_assert(kBlkFront <= 4 * LW, "rows per lane");
    if (mm <= LW) fwd_cols_j<T, 1, Perm, 4, LW>(F, mm, 0, 0, ns, ns, mm, v, perm);
    else if (mm <= 2 * LW) fwd_cols_j<T, 2, Perm, 4, LW>(F, mm, 0, 0, ns, ns, mm, v, perm);
    else if constexpr (LW < 32) {
        if (mm <= 3 * LW) fwd_cols_j<T, 3, Perm, 2, LW>(F, mm, 0, 0, ns, ns, mm, v, perm);
        else fwd_cols_j<T, 4, Perm, 2, LW>(F, mm, 0, 0, ns, ns, mm, v, perm);
    }
}

// U: the front's U rows (ns x mm, leading dimension ns).
template <class T, int LW = 32>
__device__ void bwd_front_blk(const T *U, int ns, int mm, T *v) {
    bwd_u12<T, LW>(U, ns, 0, ns, mm, ns, v);
    if (ns <= LW) bwd_cols_j<T, 1, 4, LW>(U, ns, 0, 0, ns, ns, v);
    else if (ns <= 2 * LW) bwd_cols_j<T, 2, 4, LW>(U, ns, 0, 0, ns, ns, v);
    else if constexpr (LW < 32) {
        if (ns <= 3 * LW) bwd_cols_j<T, 3, 2, LW>(U, ns, 0, 0, ns, ns, v);
        else bwd_cols_j<T, 4, 2, LW>(U, ns, 0, 0, ns, ns, v);
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
// pivot permutations of the factors of scenario mf; the caller syncs.
__device__ BlkTask stage_block(const DevSym &S, const DevBlk &B, int blk, int mf, unsigned char *base,
                               const BlkLayout &lay, const int *map, bool with_piv) {
    const int lane = threadIdx.x & 31;
    int4 *E0 = reinterpret_cast<int4 *>(base + lay.e0);
    int4 *E1 = reinterpret_cast<int4 *>(base + lay.e1);
    long long *FO = reinterpret_cast<long long *>(base + lay.foff);
    int *mp = reinterpret_cast<int *>(base + lay.map);
    int *pv = reinterpret_cast<int *>(base + lay.piv);
    const int e0 = B.blk_ptr[blk], n = B.blk_ptr[blk + 1] - e0;
    for (int q0 = lane; q0 < n; q0 += 64) {
        int4 a[2], b[2];
        long long f[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int q = q0 + 32 * u;
            a[u] = q < n ? B.ent0[e0 + q] : make_int4(0, 0, 0, 0);
            b[u] = q < n ? B.ent1[e0 + q] : make_int4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < 2; u++) f[u] = q0 + 32 * u < n ? (long long)S.lu_off[a[u].x] : 0;
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int q = q0 + 32 * u;
            if (q < n) {
                E0[q] = a[u];
                E1[q] = b[u];
                FO[q] = f[u];
            }
        }
    }
    // (the loops below keep four loads a lane in flight: a store waiting on
    // its load would otherwise hold back the next iteration's load)
    const int mb = B.map_ptr[blk], nmap = B.map_ptr[blk + 1] - mb;
    for (int i0 = lane; i0 < nmap; i0 += 4 * 32) {
        int v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) v[u] = i0 + 32 * u < nmap ? map[mb + i0 + 32 * u] : 0;
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (i0 + 32 * u < nmap) mp[i0 + 32 * u] = v[u];
    }
    if (with_piv) {
        const int *ip = S.ipiv + (size_t)mf * S.n;
        const int p0 = B.pcol_ptr[blk], np = B.pcol_ptr[blk + 1] - p0;
        for (int e0 = lane; e0 < np; e0 += 4 * 32) {
            int c[4], v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) c[u] = e0 + 32 * u < np ? B.pcol[p0 + e0 + 32 * u] : 0;
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = e0 + 32 * u < np ? ip[c[u]] : 0;
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (e0 + 32 * u < np) pv[e0 + 32 * u] = v[u];
        }
    }
    return BlkTask{e0, n, E0, E1, FO, mp, pv};
}

// The pivot rows' entries of x into a block's vector vs (entry e of the
// block's pivot list at vs[pvs[e]]), four loads a lane in flight; LW-lane
// segments each on their own vector.
template <class T, int LW>
__device__ void gather_pivot_rows(const DevBlk &B, int blk, const double *x, T *vs) {
    const int lane = threadIdx.x & (LW - 1);
    const int p0 = B.pcol_ptr[blk], np = B.pcol_ptr[blk + 1] - p0;
    for (int e0 = lane; e0 < np; e0 += 4 * LW) {
        int c[4], q[4];
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const bool in = e0 + LW * u < np;
            c[u] = in ? B.pcol[p0 + e0 + LW * u] : 0;
            q[u] = in ? B.pvs[p0 + e0 + LW * u] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) v[u] = e0 + LW * u < np ? (T)x[c[u]] : T(0);
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (e0 + LW * u < np) vs[q[u]] = v[u];
    }
}

__device__ __forceinline__ void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// Pulls the factor entries a block task's sweep will read into L1 before
// the sweep (and, backward, before the waits on the top region), so that
// the sweep's column chunks do not each wait on L2.  The block's L panels
// (forward) or U rows (backward) are one contiguous range of the
// solve-ordered factors; every address lies inside it.
template <class T, int LW = 32>
__device__ void prefetch_block(const T *fac, const BlkTask &t) {
    const int lane = threadIdx.x & (LW - 1);
    const int4 a = t.E0[t.n - 1];
    const T *f0 = fac + t.FO[0], *f1 = fac + t.FO[t.n - 1] + (size_t)(a.z + a.w) * a.z - 1;
    const uintptr_t l0 = (uintptr_t)f0 & ~(uintptr_t)127, l1 = (uintptr_t)f1;
    for (uintptr_t ad = l0 + (uintptr_t)lane * 128; ad <= l1; ad += LW * 128)
        prefetch_l1(reinterpret_cast<const void *>(ad));
}

// Pivot rows of one segment in the interleaved byte table.
struct PermBytes {
    const unsigned char *p;
    __device__ int operator()(int i) const { return p[2 * i]; }
};

// Two scenarios per warp (LW = 16, segment seg = 0, 1 of the warp): the
// pivots of both, one byte each (pivot rows are within the supernode's
// pivot block, fewer than kBlkFront), interleaved in the pivot area.
__device__ void stage_piv_pair(const DevSym &S, const DevBlk &B, int blk, int m0, int m1, unsigned char *pvb) {
    const int lane = threadIdx.x & 15, seg = (threadIdx.x >> 4) & 1;
    const int *ip = S.ipiv + (size_t)(seg ? m1 : m0) * S.n;
    const int p0 = B.pcol_ptr[blk], np = B.pcol_ptr[blk + 1] - p0;
    for (int e0 = lane; e0 < np; e0 += 4 * 16) {
        int c[4], v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) c[u] = e0 + 16 * u < np ? B.pcol[p0 + e0 + 16 * u] : 0;
#pragma unroll
        for (int u = 0; u < 4; u++) v[u] = e0 + 16 * u < np ? ip[c[u]] : 0;
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (e0 + 16 * u < np) pvb[2 * (e0 + 16 * u) + seg] = (unsigned char)v[u];
    }
}

// The forward sweep of one block for scenario m.  LW = 32: the warp on one
// scenario, pivots in t.pv; LW = 16: each half-warp on its own scenario
// (same block, so the same control flow), pivots in pvb.
template <class T, int LW = 32>
__device__ void fwd_block(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, int blk,
                          const DevDag &D, int epoch, const FrontSel &fs, const BlkTask &t, int m, T *vs,
                          const unsigned char *pvb = nullptr) {
    const int lane = threadIdx.x & (LW - 1), seg = (threadIdx.x >> 4) & 1;
    const double *x = W.xperm + (size_t)m * P.n_red;
    // the block's vector: zero, then the pivot rows' right-hand side
    {
        const int4 al = t.E0[t.n - 1], bl = t.E1[t.n - 1];
        const int nv = bl.y + al.z + al.w;
        for (int i = lane; i < nv; i += LW) vs[i] = T(0);
        __syncwarp();
        gather_pivot_rows<T, LW>(B, blk, x, vs);
    }
    __syncwarp();
    const T *fr = lfac<T>(fs, S, m);
    double *xo = W.xperm + (size_t)m * P.n_red;
    double *uv = S.uvec + (size_t)m * S.uvec_total;
    for (int q = 0; q < t.n; q++) {
        const int4 a = t.E0[q], b = t.E1[q];
        const int ns = a.z, r = a.w;
        T *v = vs + b.y;
        if constexpr (LW == 32) {
            const int *pv = t.pv + b.w;
            fwd_front_blk<T>(fr + t.FO[q], [&](int i) { return pv[i]; }, ns, ns + r, v);
        } else {
            const unsigned char *pb = pvb + 2 * b.w + seg;
            fwd_front_blk<T, PermBytes, LW>(fr + t.FO[q], PermBytes{pb}, ns, ns + r, v);
        }
        for (int i = lane; i < ns; i += LW) xo[a.y + i] = (double)v[i];
        if (q < t.n - 1) {
            const int *pm = t.mp + b.z;
            for (int i = lane; i < r; i += LW) vs[pm[i]] += v[ns + i];
        } else if constexpr (Tagged<T>::value) {
            unsigned long long *ut = D.utag + (size_t)m * S.uvec_total + S.uvec_off[a.x];
            for (int i = lane; i < r; i += LW) st_relaxed_u64(ut + i, tag_f32(v[ns + i], epoch));
        } else {
            double *us = uv + S.uvec_off[a.x];
            for (int i = lane; i < r; i += LW) us[i] = (double)v[ns + i];
        }
        __syncwarp();
    }
}

// FP32 factors: the entries of rows outside the block (pivots of top
// supernodes) are polled as tagged words; FP64: the caller has waited on the
// parent's done flag.
template <class T, int LW = 32>
__device__ void bwd_block(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const DevDag &D,
                          int epoch, const FrontSel &fs, const BlkTask &t, int blk, int m, T *vs) {
    const int lane = threadIdx.x & (LW - 1);
    double *x = W.xperm + (size_t)m * P.n_red;
    gather_pivot_rows<T, LW>(B, blk, x, vs);
    const int xb = B.ext_ptr[blk], next = B.ext_ptr[blk + 1] - xb;
    if constexpr (Tagged<T>::value) {
        const unsigned long long *xt = D.xtag + (size_t)m * P.n_red;
        const bool ok = poll_tagged(
            xt, next, lane, LW, epoch, D, [&](int k) { return B.ext_row[xb + k]; },
            [&](int k, float v) { vs[B.ext_pos[xb + k]] = v; });
        if (!ok) atomicOr(W.status + m, 8);
    } else {
        for (int k = lane; k < next; k += LW) vs[B.ext_pos[xb + k]] = (T)x[B.ext_row[xb + k]];
    }
    __syncwarp();
    const T *fr = ufac<T>(fs, S, m);
    for (int q = t.n - 1; q >= 0; q--) {
        const int4 a = t.E0[q], b = t.E1[q];
        const int ns = a.z, r = a.w;
        T *v = vs + b.y;
        const int *gm = t.mp + b.z;
        for (int c = lane; c < r; c += LW) v[ns + c] = vs[gm[c]];
        __syncwarp();
        bwd_front_blk<T, LW>(fr + t.FO[q], ns, ns + r, v);
        for (int i = lane; i < ns; i += LW) x[a.y + i] = (double)v[i];
    }
}

// ---- lower top region, forward: one warp per task ---------------------------
// In the forward pass the top supernodes of the first levels (fronts of at
// most kBlkFront rows) are tasks of one warp each, like a block of one
// supernode that waits on its children: through tagged words on FP32
// factors, through done flags on FP64 factors.  The warp keeps the front's
// vector in its shared-memory area and reads the factors through L1 (pulled
// in before the waits).  (The backward pass keeps CTA tasks there: warp
// tasks measured slower, 97.8 against 101.2 ms of solves per mixed run.)

template <class T>
__device__ void fwd_top_warp(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B,
                             const DevDag &D, const FrontSel &fs, int s, int rank, int m, int epoch, T *v) {
    const int lane = threadIdx.x & 31;
    const int start = S.sup_start[s], ns = S.sup_start[s + 1] - start;
    const int r = S.row_ptr[s + 1] - S.row_ptr[s], mm = ns + r;
    const T *L = lfac<T>(fs, S, m) + S.lu_off[s];
    {
        const uintptr_t l0 = (uintptr_t)L & ~(uintptr_t)127, l1 = (uintptr_t)(L + (size_t)mm * ns - 1);
        for (uintptr_t ad = l0 + (uintptr_t)lane * 128; ad <= l1; ad += 32 * 128)
            prefetch_l1(reinterpret_cast<const void *>(ad));
    }
    double *x = W.xperm + (size_t)m * P.n_red;
    const int *xr = B.top_xrow + B.top_xptr[rank];
    bool ok = true;
    if constexpr (!Tagged<T>::value) {
        // FP64 factors: the children's done flags, then their update vectors
        const int c0 = S.child_ptr[s], nch = S.child_ptr[s + 1] - c0;
        for (int q = lane; q < nch; q += 32)
            ok = wait_epoch(D.xdone + (size_t)S.children[c0 + q] * P.M + m, epoch, D.err, D.wait_limit) && ok;
        ok = __all_sync(FULL, ok);
    }
    const double *uv = S.uvec + (size_t)m * S.uvec_total;
    const unsigned long long *ut = D.utag + (size_t)m * S.uvec_total;
    // rows over lanes; each row sums its children's entries in child order
    // (the CTA tasks' order), four loads in flight
    for (int i = lane; i < mm; i += 32) {
        T acc = i < ns ? (T)x[start + i] : T(0);
        const int e1 = xr[i + 1];
        for (int e = xr[i]; e < e1; e += 4) {
            int off[4];
#pragma unroll
            for (int u = 0; u < 4; u++) off[u] = e + u < e1 ? B.top_xent[e + u] : 0;
            if constexpr (Tagged<T>::value) {
                unsigned long long w[4];
#pragma unroll
                for (int u = 0; u < 4; u++) w[u] = e + u < e1 ? ld_relaxed_u64(ut + off[u]) : 0ull;
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (e + u < e1) {
                        if (!tag_ok(w[u], epoch)) w[u] = wait_tag(ut + off[u], epoch, D.err, D.wait_limit, ok);
                        acc += tag_val(w[u]);
                    }
            } else {
                double w[4];
#pragma unroll
                for (int u = 0; u < 4; u++) w[u] = e + u < e1 ? __ldcg(uv + off[u]) : 0.0;
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (e + u < e1) acc += (T)w[u];
            }
        }
        v[i] = acc;
    }
    if (!__all_sync(FULL, ok) && lane == 0) atomicOr(W.status + m, 8);
    __syncwarp();
    const int *ip = S.ipiv + (size_t)(fs.shared ? 0 : m) * S.n + start;
    fwd_front_blk<T>(L, [&](int i) { return ip[i]; }, ns, mm, v);
    for (int i = lane; i < ns; i += 32) x[start + i] = (double)v[i];
    if constexpr (Tagged<T>::value) {
        unsigned long long *uo = D.utag + (size_t)m * S.uvec_total + S.uvec_off[s];
        for (int i = lane; i < r; i += 32) st_relaxed_u64(uo + i, tag_f32(v[ns + i], epoch));
    } else {
        double *us = S.uvec + (size_t)m * S.uvec_total + S.uvec_off[s];
        for (int i = lane; i < r; i += 32) us[i] = (double)v[ns + i];
        __syncwarp();
        if (lane == 0) signal_done(D.xdone + (size_t)s * P.M + m, epoch);
    }
    __syncwarp();
}

// ---- top region: dataflow of CTA tasks ------------------------------------

// All threads of the CTA copy n consecutive factor entries into Fs.
template <class T>
__device__ void stage_range(T *Fs, const T *F, int n) {
    for (int e = threadIdx.x; e < n; e += blockDim.x) cp_async(Fs + e, F + e, (int)sizeof(T));
}

struct TopCtx {
    int s, m, rank, start, ns, r, mm;
};

__device__ __forceinline__ TopCtx top_ctx(const DevSym &S, int s, int m, int rank) {
    TopCtx c;
    c.s = s;
    c.m = m;
    c.rank = rank;
    c.start = S.sup_start[s];
    c.ns = S.sup_start[s + 1] - c.start;
    c.r = S.row_ptr[s + 1] - S.row_ptr[s];
    c.mm = c.ns + c.r;
    return c;
}

// Waits (warp 0) on the done flags of the children (block roots and top
// supernodes); false when a wait gave up.  Ends with a CTA barrier.
__device__ bool wait_top_children(const DevSym &S, const DevBlk &B, const DevDag &D, int s, int m, int M, int epoch,
                                  int *s_ok) {
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int c0 = S.child_ptr[s], nc = S.child_ptr[s + 1] - c0;
        bool ok = true;
        for (int q = lane; q < nc; q += 32) {
            const int c = S.children[c0 + q];
            ok = wait_epoch(D.xdone + (size_t)c * M + m, epoch, D.err, D.wait_limit) && ok;
        }
        ok = __all_sync(FULL, ok);
        if (lane == 0) *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

__device__ bool wait_top_parent(const DevDag &D, int s, int m, int M, int epoch, int *s_ok) {
    const int par = D.parent[s];
    if (threadIdx.x == 0) *s_ok = par < 0 ? 1 : (int)wait_epoch(D.bdone + (size_t)par * M + m, epoch, D.err, D.wait_limit);
    __syncthreads();
    return *s_ok != 0;
}

template <class T>
__device__ void fwd_top_task(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B,
                             const DevDag &D, const FrontSel &fs, const TopCtx &t, int epoch, unsigned char *smem,
                             int *s_ok) {
    const int tmf = B.top_max_front;
    T *v = reinterpret_cast<T *>(smem);
    T *sc = reinterpret_cast<T *>(smem + tmf * 8);
    int *pi = reinterpret_cast<int *>(smem + tmf * 16);
    int *sxr = reinterpret_cast<int *>(smem + top_vec_bytes(tmf));
    int *sxe = sxr + align16((tmf + 1) * 4) / 4;
    T *Fs = reinterpret_cast<T *>(smem + top_vec_bytes(tmf) + top_idx_bytes(tmf, B.top_max_xent));
    const T *F = lfac<T>(fs, S, t.m) + S.lu_off[t.s];   // L panel, leading dimension mm
    const int cap = kTopStage / ((int)sizeof(T) * t.mm);   // columns per staged chunk
    double *x = W.xperm + (size_t)t.m * P.n_red;
    double *uv = S.uvec + (size_t)t.m * S.uvec_total;
    const int *ip = S.ipiv + (size_t)(fs.shared ? 0 : t.m) * S.n + t.start;
    // independent of other tasks: own entries, pivot permutation, factor
    // columns and the extend-add lists, all fetched before the wait so that
    // only the children's update entries remain on the path after it
    const int *xr = B.top_xrow + B.top_xptr[t.rank];
    for (int i = threadIdx.x; i <= t.mm; i += blockDim.x) sxr[i] = xr[i];
    for (int i = threadIdx.x; i < t.mm; i += blockDim.x) v[i] = i < t.ns ? (T)x[t.start + i] : T(0);
    for (int i = threadIdx.x; i < t.ns; i += blockDim.x) pi[i] = ip[i];
    int k1 = min(t.ns, cap);
    stage_range<T>(Fs, F, k1 * t.mm);
    __syncthreads();
    const int ne = sxr[t.mm] - sxr[0];
    for (int e = threadIdx.x; e < ne; e += blockDim.x) sxe[e] = B.top_xent[sxr[0] + e];
    if constexpr (Tagged<T>::value) {
        // the children's entries, polled as tagged words by the thread that
        // staged their offsets, replace the offsets in sxe
        const unsigned long long *ut = D.utag + (size_t)t.m * S.uvec_total;
        const bool ok = poll_tagged(
            ut, ne, threadIdx.x, blockDim.x, epoch, D, [&](int e) { return sxe[e]; },
            [&](int e, float val) { sxe[e] = __float_as_int(val); });
        if (!ok) atomicOr(W.status + t.m, 8);
        __syncthreads();
    } else {
        if (!wait_top_children(S, B, D, t.s, t.m, P.M, epoch, s_ok) && threadIdx.x == 0)
            atomicOr(W.status + t.m, 8);
    }
    // extend-add: one thread per front row sums the children's entries in
    // child order (the update vectors of the children were written by other
    // CTAs: read through L2)
    {
        const int e0 = sxr[0];
        for (int i = threadIdx.x; i < t.mm; i += blockDim.x) {
            T acc = v[i];
            for (int e = sxr[i] - e0; e < sxr[i + 1] - e0; e++) {
                if constexpr (Tagged<T>::value) acc += __int_as_float(sxe[e]);
                else acc += (T)__ldcg(uv + sxe[e]);
            }
            v[i] = acc;
        }
    }
    int k0 = 0;
    bool gather = true;
    for (;;) {
        cp_async_wait_all();
        __syncthreads();
        if (threadIdx.x < 32)
            fwd_cols<T>(Fs, t.mm, k0, k0, k1, t.ns, t.mm, v, sc, [&](int i) { return pi[i]; }, gather);
        __syncthreads();
        gather = false;
        if (k1 >= t.ns) break;
        k0 = k1;
        k1 = min(t.ns, k0 + cap);
        stage_range<T>(Fs, F + (size_t)k0 * t.mm, (k1 - k0) * t.mm);
    }
    for (int i = threadIdx.x; i < t.ns; i += blockDim.x) x[t.start + i] = (double)v[i];
    if constexpr (Tagged<T>::value) {
        unsigned long long *ut = D.utag + (size_t)t.m * S.uvec_total + S.uvec_off[t.s];
        for (int i = threadIdx.x; i < t.r; i += blockDim.x) st_relaxed_u64(ut + i, tag_f32(v[t.ns + i], epoch));
    } else {
        double *us = uv + S.uvec_off[t.s];
        for (int i = threadIdx.x; i < t.r; i += blockDim.x) us[i] = (double)v[t.ns + i];
    }
}

template <class T>
__device__ void bwd_top_task(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B,
                             const DevDag &D, const FrontSel &fs, const TopCtx &t, int epoch, unsigned char *smem,
                             int *s_ok) {
    const int tmf = B.top_max_front;
    T *v = reinterpret_cast<T *>(smem);
    int *pi = reinterpret_cast<int *>(smem + tmf * 16);
    T *Fs = reinterpret_cast<T *>(smem + top_vec_bytes(tmf));
    const T *F = ufac<T>(fs, S, t.m) + S.lu_off[t.s];   // U rows, leading dimension ns
    const int cap = kTopStage / ((int)sizeof(T) * max(1, t.ns));   // columns per staged chunk
    double *x = W.xperm + (size_t)t.m * P.n_red;
    const int *rows = S.rows + S.row_ptr[t.s];
    for (int i = threadIdx.x; i < t.ns; i += blockDim.x) v[i] = (T)x[t.start + i];
    for (int a = threadIdx.x; a < t.r; a += blockDim.x) pi[a] = rows[a];
    // chunks run over the front's columns from mm - 1 down to 0: U12 first,
    // then U11 from the last pivot column
    int c1 = t.mm, c0 = max(0, t.mm - cap);
    stage_range<T>(Fs, F + (size_t)c0 * t.ns, (c1 - c0) * t.ns);
    if constexpr (Tagged<T>::value) {
        // the entries of the front's rows (pivots of ancestors), polled as
        // tagged words by the thread that staged their row indices
        const unsigned long long *xt = D.xtag + (size_t)t.m * P.n_red;
        const bool ok = poll_tagged(
            xt, t.r, threadIdx.x, blockDim.x, epoch, D, [&](int a) { return pi[a]; },
            [&](int a, float val) { v[t.ns + a] = val; });
        if (!ok) atomicOr(W.status + t.m, 8);
    } else {
        if (!wait_top_parent(D, t.s, t.m, P.M, epoch, s_ok) && threadIdx.x == 0) atomicOr(W.status + t.m, 8);
        for (int a = threadIdx.x; a < t.r; a += blockDim.x) v[t.ns + a] = (T)__ldcg(x + pi[a]);
    }
    for (;;) {
        cp_async_wait_all();
        __syncthreads();
        if (threadIdx.x < 32) {
            const int u0 = max(c0, t.ns);
            if (u0 < c1) bwd_u12<T>(Fs, t.ns, c0, u0, c1, t.ns, v);
            if (c0 < t.ns) bwd_cols<T>(Fs, t.ns, c0, c0, min(c1, t.ns), t.ns, v);
        }
        __syncthreads();
        if (c0 == 0) break;
        c1 = c0;
        c0 = max(0, c1 - cap);
        stage_range<T>(Fs, F + (size_t)c0 * t.ns, (c1 - c0) * t.ns);
    }
    for (int i = threadIdx.x; i < t.ns; i += blockDim.x) x[t.start + i] = (double)v[i];
    if constexpr (Tagged<T>::value) {
        unsigned long long *xt = D.xtag + (size_t)t.m * P.n_red + t.start;
        for (int i = threadIdx.x; i < t.ns; i += blockDim.x) st_relaxed_u64(xt + i, tag_f32(v[i], epoch));
    }
}

// ---- the solves: one persistent kernel per direction ------------------------
// Forward: the warps first claim block tasks (no waits); each block hands
// its root's update vector on.  Once every block task is claimed, the warps
// claim the lower top tasks (children first), and once those are claimed the
// CTAs claim the rest of the top region; every task waits only on its own
// children, so the top region starts as soon as the blocks below it are
// done.  Backward: the CTAs first claim the top tasks (parents first), then
// the warps the block tasks, each waiting only on the entries above it.  A task only ever waits on
// tasks claimed before it by running warps or CTAs, so the kernels cannot
// deadlock; every wait is bounded.

// Mixed solves pair the scenarios in the block phase (two per warp); a pair
// runs in the two half-warps when both scenarios are active and on FP32
// factors (the FP32 vector of each fits half of the area sized for FP64).
__device__ __forceinline__ bool pair_mode(const FrontSel &fs) { return fs.l32 != nullptr && !fs.shared; }
__device__ __forceinline__ bool pair_ok(const DevWork &W, const FrontSel &fs, int m) {
    return W.active[m] && !use64(fs, m);
}

__device__ __forceinline__ unsigned char *warp_area(unsigned char *smem, const BlkLayout &lay) {
    return smem + (size_t)(threadIdx.x >> 5) * lay.total;
}

__global__ void __launch_bounds__(kTopThreads, 8) fwd_solve_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                                   DevDag D, FrontSel fs) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_task, s_ok;
    const int lane = threadIdx.x & 31;
    const int M = P.M;
    const int epoch = *D.epoch;
    {
        // mixed solves: a warp task is a block for a pair of scenarios, both
        // on FP32 factors in the two half-warps when it can (else each
        // scenario of the pair in turn with the whole warp)
        const int MP = pair_mode(fs) ? (M + 1) / 2 : M;
        const long long n_blk = (long long)B.nblk * MP;
        const BlkLayout lay = blk_layout(B);
        unsigned char *base = warp_area(smem, lay);
        for (;;) {
            long long t = 0;
            if (lane == 0) t = atomicAdd(D.ctr + 4, 1);
            t = __shfl_sync(FULL, t, 0);
            if (t >= n_blk) break;
            const int blk = (int)(t / MP), u = (int)(t % MP);
            if (MP != M) {
                const int m0 = 2 * u, m1 = 2 * u + 1;
                if (m1 < M && pair_ok(W, fs, m0) && pair_ok(W, fs, m1)) {
                    const int seg = (threadIdx.x >> 4) & 1, m = seg ? m1 : m0;
                    const BlkTask bt = stage_block(S, B, blk, 0, base, lay, B.map_fwd, false);
                    __syncwarp();
                    unsigned char *pvb = base + lay.piv;
                    stage_piv_pair(S, B, blk, m0, m1, pvb);
                    prefetch_block<float, 16>(lfac<float>(fs, S, m), bt);
                    __syncwarp();
                    fwd_block<float, 16>(P, W, S, B, blk, D, epoch, fs, bt, m,
                                         reinterpret_cast<float *>(base + lay.v) + seg * B.max_v, pvb);
                    __syncwarp();
                    continue;
                }
            }
            for (int h = 0; h < (MP != M ? 2 : 1); h++) {
                const int m = MP != M ? 2 * u + h : u;
                if (m >= M || !W.active[m]) continue;
                const bool d = use64(fs, m);
                if (d && fs.fused64) continue;
                const BlkTask bt = stage_block(S, B, blk, fs.shared ? 0 : m, base, lay, B.map_fwd, true);
                __syncwarp();
                if (d) prefetch_block<double>(lfac<double>(fs, S, m), bt);
                else prefetch_block<float>(lfac<float>(fs, S, m), bt);
                if (d) fwd_block<double>(P, W, S, B, blk, D, epoch, fs, bt, m, reinterpret_cast<double *>(base + lay.v));
                else fwd_block<float>(P, W, S, B, blk, D, epoch, fs, bt, m, reinterpret_cast<float *>(base + lay.v));
                __syncwarp();
                if (d && lane == 0) signal_done(D.xdone + (size_t)bt.E0[bt.n - 1].x * M + m, epoch);
                __syncwarp();
            }
        }
        // the lower top region, one warp per task, children first
        const long long n_lt = (long long)B.n_lower_top * M;
        for (;;) {
            long long t = 0;
            if (lane == 0) t = atomicAdd(D.ctr + 6, 1);
            t = __shfl_sync(FULL, t, 0);
            if (t >= n_lt) break;
            const int rank = (int)(t / M), m = (int)(t % M);
            if (!W.active[m]) continue;
            const bool d = use64(fs, m);
            if (d && fs.fused64) continue;
            const int s = B.top_order[rank];
            if (d) fwd_top_warp<double>(P, W, S, B, D, fs, s, rank, m, epoch, reinterpret_cast<double *>(base + lay.v));
            else fwd_top_warp<float>(P, W, S, B, D, fs, s, rank, m, epoch, reinterpret_cast<float *>(base + lay.v));
        }
    }
    // the rest of the top region, one CTA per task
    const int n_tasks = (B.n_top - B.n_lower_top) * M;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_task = atomicAdd(D.ctr + 2, 1);
        __syncthreads();
        const int t = s_task;
        if (t >= n_tasks) break;
        const int rank = B.n_lower_top + t / M, m = t % M;
        const int s = B.top_order[rank];
        if (!W.active[m]) continue;
        const bool d = use64(fs, m);
        if (d && fs.fused64) continue;
        const TopCtx c = top_ctx(S, s, m, rank);
        if (d) {
            fwd_top_task<double>(P, W, S, B, D, fs, c, epoch, smem, &s_ok);
            __syncthreads();
            if (threadIdx.x == 0) signal_done(D.xdone + (size_t)s * M + m, epoch);
        } else {
            fwd_top_task<float>(P, W, S, B, D, fs, c, epoch, smem, &s_ok);
        }
    }
}

__global__ void __launch_bounds__(kTopThreads, 8) bwd_solve_kernel(DevProblem P, DevWork W, DevSym S, DevBlk B,
                                                                   DevDag D, FrontSel fs) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_task, s_ok;
    const int lane = threadIdx.x & 31;
    const int M = P.M;
    const int epoch = *D.epoch;
    // the top region, one CTA per task, parents first
    const int n_tasks = B.n_top * M;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_task = atomicAdd(D.ctr + 3, 1);
        __syncthreads();
        const int t = s_task;
        if (t >= n_tasks) break;
        const int rank = B.n_top - 1 - t / M, m = t % M;
        const int s = B.top_order[rank];
        if (!W.active[m]) continue;
        const TopCtx c = top_ctx(S, s, m, rank);
        if (use64(fs, m)) {
            bwd_top_task<double>(P, W, S, B, D, fs, c, epoch, smem, &s_ok);
            __syncthreads();
            if (threadIdx.x == 0) signal_done(D.bdone + (size_t)s * M + m, epoch);
        } else {
            bwd_top_task<float>(P, W, S, B, D, fs, c, epoch, smem, &s_ok);
        }
    }
    const BlkLayout lay = blk_layout(B);
    unsigned char *base = warp_area(smem, lay);
    const int MP = pair_mode(fs) ? (M + 1) / 2 : M;
    const long long n_blk = (long long)B.nblk * MP;
    for (;;) {
        long long t = 0;
        if (lane == 0) t = atomicAdd(D.ctr + 5, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= n_blk) break;
        const int blk = (int)(t / MP), u = (int)(t % MP);
        if (MP != M) {
            const int m0 = 2 * u, m1 = 2 * u + 1;
            if (m1 < M && pair_ok(W, fs, m0) && pair_ok(W, fs, m1)) {
                const int seg = (threadIdx.x >> 4) & 1, m = seg ? m1 : m0;
                const BlkTask bt = stage_block(S, B, blk, 0, base, lay, B.map_bwd, false);
                __syncwarp();
                prefetch_block<float, 16>(ufac<float>(fs, S, m), bt);
                __syncwarp();
                bwd_block<float, 16>(P, W, S, B, D, epoch, fs, bt, blk, m,
                                     reinterpret_cast<float *>(base + lay.v) + seg * B.max_v);
                __syncwarp();
                continue;
            }
        }
        for (int h = 0; h < (MP != M ? 2 : 1); h++) {
            const int m = MP != M ? 2 * u + h : u;
            if (m >= M || !W.active[m]) continue;
            const BlkTask bt = stage_block(S, B, blk, fs.shared ? 0 : m, base, lay, B.map_bwd, false);
            __syncwarp();
            const bool d = use64(fs, m);
            if (d) prefetch_block<double>(ufac<double>(fs, S, m), bt);
            else prefetch_block<float>(ufac<float>(fs, S, m), bt);
            const int par = d ? D.parent[bt.E0[bt.n - 1].x] : -1;   // (FP64 factors wait on it)
            if (par >= 0) {
                bool ok = true;
                if (lane == 0) ok = wait_epoch(D.bdone + (size_t)par * M + m, epoch, D.err, D.wait_limit);
                ok = __shfl_sync(FULL, ok, 0);
                if (!ok && lane == 0) atomicOr(W.status + m, 8);
            }
            __syncwarp();
            if (d) bwd_block<double>(P, W, S, B, D, epoch, fs, bt, blk, m, reinterpret_cast<double *>(base + lay.v));
            else bwd_block<float>(P, W, S, B, D, epoch, fs, bt, blk, m, reinterpret_cast<float *>(base + lay.v));
            __syncwarp();
        }
    }
}

int grid_for(int resident, long long tasks, int per_block) {
    const long long need = (tasks + per_block - 1) / per_block;
    return (int)std::max<long long>(1, std::min<long long>(need, resident));
}

}  // namespace

int solve_block_front_limit() { return kBlkFront; }

int solve_configure(const DevBlk &B, SolveGrid &g) {
    int dev = 0, nsm = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return -1;
    // a staged chunk holds at least one whole front column in FP64
    if ((long)B.top_max_front * 8 > kTopStage) return -2;
    static_assert(kBlkWarps * 32 == kTopThreads, "one CTA runs block tasks per warp and top tasks together");
    g.blk_bytes = kBlkWarps * blk_layout(B).total;
    g.top_bytes = std::max(g.blk_bytes, top_vec_bytes(std::max(1, B.top_max_front)) +
                                            top_idx_bytes(std::max(1, B.top_max_front), B.top_max_xent) + kTopStage);
    if (cudaFuncSetAttribute(fwd_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g.top_bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(bwd_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, g.top_bytes) !=
            cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fwd_solve_kernel, kTopThreads, g.top_bytes) !=
            cudaSuccess || occ < 1)
        return -1;
    g.top_fwd = nsm * occ;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bwd_solve_kernel, kTopThreads, g.top_bytes) !=
            cudaSuccess || occ < 1)
        return -1;
    g.top_bwd = nsm * occ;
    return 0;
}

void launch_solve_fwd(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const DevDag &D,
                      const SolveGrid &g, FrontSel fs, cudaStream_t st) {
    const long long work = std::max((long long)B.nblk * P.M / kBlkWarps + 1, (long long)B.n_top * P.M);
    if (B.nblk + B.n_top > 0)
        fwd_solve_kernel<<<grid_for(g.top_fwd, work, 1), kTopThreads, g.top_bytes, st>>>(P, W, S, B, D, fs);
}

void launch_solve_bwd(const DevProblem &P, const DevWork &W, const DevSym &S, const DevBlk &B, const DevDag &D,
                      const SolveGrid &g, FrontSel fs, cudaStream_t st) {
    const long long work = std::max((long long)B.nblk * P.M / kBlkWarps + 1, (long long)B.n_top * P.M);
    if (B.nblk + B.n_top > 0)
        bwd_solve_kernel<<<grid_for(g.top_bwd, work, 1), kTopThreads, g.top_bytes, st>>>(P, W, S, B, D, fs);
}

}  // namespace gp
