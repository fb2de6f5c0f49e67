// Warp-level helpers shared by the reduced-system factorisation and solves.
#pragma once
#include <cuda_runtime.h>

namespace gp {

constexpr unsigned kFullMask = 0xffffffffu;

// ---- flags between tasks of one persistent kernel ----------------------
// A task signals completion by storing the current epoch (release); a
// waiting task polls with relaxed loads and acquires on success.  Every wait
// is bounded: after `limit` polls (DevDag::wait_limit, 2^20 unless the host
// sets another) it raises the error flag and gives up, and every other wait
// then returns at once, so the kernel always ends.

__device__ __forceinline__ int ld_relaxed(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits until *flag == epoch; false when it gave up (error flag raised here
// or by another task).  The error flag is read every 32nd poll only, so that
// a poll is one load on the path between a signal and its waiter.
__device__ inline bool wait_epoch(const int *flag, int epoch, int *err, int limit) {
    for (int it = 0; it < limit; ++it) {
        if (ld_relaxed(flag) == epoch) {
            fence_acquire();
            return true;
        }
        if ((it & 31) == 31 && ld_relaxed(err)) return false;
        __nanosleep(32);
    }
    atomicExch(err, 1);
    return false;
}

// Called by one thread after a CTA or warp barrier that orders the task's
// writes before it; the release store makes them visible with the flag.
__device__ __forceinline__ void signal_done(int *flag, int epoch) { st_release(flag, epoch); }

// ---- tagged words: a value that carries its own epoch ------------------
// An FP32 value and the epoch of the solve that wrote it in one 64-bit word
// (value in the low half, epoch in the high half), stored and loaded as one
// single-copy-atomic access.  A reader polls the word itself: no flag, no
// release fence on the writer's side, no second load after the flag.

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long tag_f32(float v, int epoch) {
    return ((unsigned long long)(unsigned)epoch << 32) | __float_as_uint(v);
}

__device__ __forceinline__ bool tag_ok(unsigned long long w, int epoch) { return (int)(w >> 32) == epoch; }

__device__ __forceinline__ float tag_val(unsigned long long w) { return __uint_as_float((unsigned)w); }

// Polls *p until it carries epoch, bounded like wait_epoch; clears ok when
// the wait gave up.
__device__ inline unsigned long long wait_tag(const unsigned long long *p, int epoch, int *err, int limit, bool &ok) {
    for (int it = 0; it < limit; ++it) {
        const unsigned long long w = ld_relaxed_u64(p);
        if (tag_ok(w, epoch)) return w;
        if ((it & 31) == 31 && ld_relaxed(err)) {
            ok = false;
            return w;
        }
        __nanosleep(32);
    }
    atomicExch(err, 1);
    ok = false;
    return 0ull;
}

// ---- reciprocal of a pivot ----------------------------------------------
// float: the IEEE division.  double: the PTX approximate reciprocal
// (rcp.approx.ftz.f64) refined by two Newton-Raphson steps r <- r + r (1 -
// x r), each step two fused multiply-adds (the FMA form of the iteration in
// P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34 (1990) 111-119).  A step
// squares the relative error, so from the seed's error two steps leave the
// result within about one ulp of 1/x (the library's tests bound it against
// the division).  Four FMAs on the FP64 pipe, which runs at two FMAs a clock
// per SM on GB300 and is what the elimination of small fronts spends most
// of its time on: a warp computes one reciprocal per pivot column.  Zero,
// subnormal, very large, infinite and NaN pivots take the division, so
// that they give the division's result exactly.
__device__ __forceinline__ float recip(float x) { return 1.0f / x; }
__device__ __forceinline__ double recip(double x) {
    const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
    if (e == 0u || e > 0x7fcu) return 1.0 / x;
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double t = fma(-x, r, 1.0);
    r = fma(r, t, r);
    t = fma(-x, r, 1.0);
    return fma(r, t, r);
}

// Next power of two >= n, for 1 <= n <= 32.
__device__ __forceinline__ int np2(int n) { return n <= 1 ? 1 : 1 << (32 - __clz(n - 1)); }

// Row dot products out_i = sum_j A[i*si + j*sj] * v(j), i < nrow, j < ncol,
// by one warp, accumulated in Acc.  Rows are spread over groups of G lanes
// (G = 32 / np2(nrow), 1 when nrow >= 32) that split the j range and combine
// by shuffles in a fixed order, so that short rows still fill the warp.
// emit(i, acc) runs on the first lane of each group.
// LW < 32: the warp is LW-lane segments, each on its own data (same nrow
// and ncol in every segment).
template <class Acc, int LW = 32, class T, class V, class E>
__device__ __forceinline__ void warp_row_dots(const T *A, int si, int sj, int nrow, int ncol, V v, E emit) {
    const int lane = threadIdx.x & (LW - 1);
    const int G = nrow >= LW ? 1 : LW / np2(nrow);
    const int rows_per_pass = LW / G;
    const int g = lane & (G - 1);
    for (int i0 = 0; i0 < nrow; i0 += rows_per_pass) {
        const int i = i0 + lane / G;
        Acc acc = Acc(0);
        if (i < nrow)
            for (int j = g; j < ncol; j += G) acc += (Acc)A[i * si + j * sj] * (Acc)v(j);
        for (int off = G >> 1; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off, LW);
        if (g == 0 && i < nrow) emit(i, acc);
    }
}

}  // namespace gp
