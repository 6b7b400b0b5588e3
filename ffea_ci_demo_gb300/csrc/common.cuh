// common.cuh -- device-side building blocks of the blob-step engine.
//
//  * DevStatus: the per-blob status word that kernels set instead of trapping
//    (inversion count, CG non-convergence, non-finite output, barrier timeout).
//  * barrier_ep / grid_sync_ep (the cooperative CG kernels) and group_sync
//    (the batch kernel's groups): barriers of co-resident blocks whose wait is
//    bounded by %globaltimer; on timeout they record FFEA_GPU_ETIMEOUT and
//    every block leaves its loop.
//  * deterministic block / grid reductions of doubles (fixed shuffle tree,
//    then every block sums the per-block partials in the same order).
//  * MRG32k3a in exact 32-bit modular integer arithmetic (the generator of
//    L'Ecuyer 1999 used by the reference's RngStream, src/RngStream.cpp), with
//    jump-ahead by precomputed transition-matrix powers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <cuda/atomic>

namespace ffea {

struct DevStatus {
    int inversions;   // elements with det sign change this step
    int cg_fail;      // CG hit max_iterations_cg
    int nonfinite;    // non-finite solver output
    int timeout;      // a bounded wait gave up
    int abort;        // any of the above: later kernels of the step return at once
    int last_iters;   // CG iterations of the last completed solve
    long long total_iters;
    int steps_done;   // completed steps since the counter was reset
    int pad;
};

struct GridBarrier {
    unsigned int count;     // arrivals since the last reset
    unsigned int pad0[31];  // on its own 128-byte line
    unsigned int passed;    // group_sync: barriers completed since the last reset (written by the last arriver)
    unsigned int pad1[31];
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded barrier of nblk co-resident blocks (the grid of a cooperative launch, or one group of it) sharing
// *gb, whose count must be zero when the kernel starts (the launch before it on the stream resets it).
// Arrival is a release reduction on gb->count (no value returned), and every block polls gb->count with
// acquire loads until it reaches (epoch + 1) * nblk, so the last arrival is the only write on the critical
// path. For the cooperative CG kernels (one block per SM, one counter for the grid); the batch kernel's many
// small groups keep group_sync. `epoch` counts the barriers this launch has passed on *gb (the same in every block and thread of the
// barrier; the caller keeps it, starting at 0). Returns false if this block gave up waiting or another block
// recorded a timeout; the caller then leaves its loop.
__device__ __forceinline__ bool barrier_ep(GridBarrier *gb, unsigned int nblk, DevStatus *st,
                                           unsigned long long limit_ns, unsigned int &epoch) {
    ++epoch;
    if (nblk == 1u) {  // one block: its global writes are visible to itself after __syncthreads
        __syncthreads();
        return true;
    }
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned int target = epoch * nblk;
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&gb->count) : "memory");
        const unsigned long long t0 = globaltimer_ns();
        unsigned int polls = 0;
        for (;;) {
            unsigned int c;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(&gb->count) : "memory");
            if ((int)(c - target) >= 0) break;
            if ((++polls & 255u) == 0u) {
                if (globaltimer_ns() - t0 > limit_ns) {
                    atomicExch(&st->timeout, 1);
                    atomicExch(&st->abort, 1);
                    ok = 0;
                    break;
                }
                if (*((volatile int *)&st->timeout)) { ok = 0; break; }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Barrier of the nblk blocks of one group of the batch kernel, whose *gb (zero at launch) no other group uses.
// Arrival is one relaxed atomic on gb->count after a release fence; the block that completes barrier k
// (arrival number (k + 1) nblk - 1) publishes k + 1 in gb->passed, which lives on its own cache line and is the
// only word the others poll (volatile loads), followed by one acquire fence. With many small groups (up to
// sixteen blocks of different groups on one SM) this measured faster than barrier_ep, whose polls share the
// line of the arrivals (solve 117.8 against 120.8 ms on the 256-blob ensemble). A one-block group needs only
// __syncthreads.
__device__ __forceinline__ bool group_sync(GridBarrier *gb, unsigned int nblk, DevStatus *st,
                                           unsigned long long limit_ns) {
    if (nblk == 1u) {
        __syncthreads();
        return true;
    }
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        const unsigned int old = atomicAdd(&gb->count, 1u);
        const unsigned int k1 = old / nblk + 1u;
        if (old == k1 * nblk - 1u) {
            atomicExch(&gb->passed, k1);
        } else {
            volatile unsigned int *passed = &gb->passed;
            const unsigned long long t0 = globaltimer_ns();
            unsigned int polls = 0;
            while ((int)(*passed - k1) < 0) {
                if ((++polls & 255u) == 0u) {
                    if (globaltimer_ns() - t0 > limit_ns) {
                        atomicExch(&st->timeout, 1);
                        atomicExch(&st->abort, 1);
                        ok = 0;
                        break;
                    }
                    if (*((volatile int *)&st->timeout)) { ok = 0; break; }
                }
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// The barrier of the whole grid.
__device__ __forceinline__ bool grid_sync_ep(GridBarrier *gb, DevStatus *st, unsigned long long limit_ns,
                                             unsigned int &epoch) {
    return barrier_ep(gb, gridDim.x, st, limit_ns, epoch);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum of `v` over the block in a fixed order; the result is valid in every thread.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem /* NV*32 */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) smem[i * 32 + wid] = v[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double t = (lane < nw) ? smem[i * 32 + lane] : 0.0;
        v[i] = warp_sum(t);
    }
    __syncthreads();
}

// Every block sums partials[i*stride + b] over b < nb in the same fixed order;
// warp w of the block handles values w, w + nwarps, ... in parallel.
template <int NV>
__device__ __forceinline__ void grid_partials_sum(const double *partials, int stride, int nb, double (&out)[NV],
                                                  double *smem) {
    __shared__ double s_out[NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = wid; i < NV; i += nw) {
        double t = 0.0;
        for (int b = lane; b < nb; b += 32) t += __ldcg(partials + i * stride + b);
        t = warp_sum(t);
        if (lane == 0) s_out[i] = t;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) out[i] = s_out[i];
    __syncthreads();
    (void)smem;
}

// ---------------------------------------------------------------------------
// double-float (pairs of FP32, ~48-bit significand) accumulation. GB300 runs
// FP64 at 1/64 of the FP32 rate, so reductions over nodes keep their extra
// precision in FP32 pairs: two_sum is Knuth's error-free sum, df_add the
// usual accurate pair addition.
// ---------------------------------------------------------------------------
struct df32 {
    float hi, lo;
};

__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
    const float s = a.hi + b.hi;
    const float v = s - a.hi;
    float e = (a.hi - (s - v)) + (b.hi - v);
    e += a.lo + b.lo;
    const float hi = s + e;
    return {hi, e - (hi - s)};
}

__device__ __forceinline__ df32 df_add_f(df32 a, float b) { return df_add(a, df32{b, 0.f}); }

__device__ __forceinline__ df32 warp_sum_df(df32 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        df32 w;
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        v = df_add(v, w);
    }
    return v;
}

// Block reduction of NV double-float values; thread 0 gets the sums in out[] (other threads: undefined).
// smem needs NV * 32 float2.
template <int NV>
__device__ __forceinline__ void block_sum_df(const df32 (&v)[NV], float2 *smem, df32 (&out)[NV]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const df32 w = warp_sum_df(v[i]);
        if (lane == 0) smem[i * 32 + wid] = make_float2(w.hi, w.lo);
    }
    __syncthreads();
    for (int i = wid; i < NV; i += nw) {
        df32 t = {0.f, 0.f};
        if (lane < nw) t = df32{smem[i * 32 + lane].x, smem[i * 32 + lane].y};
        t = warp_sum_df(t);
        if (lane == 0) smem[i * 32] = make_float2(t.hi, t.lo);
    }
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) out[i] = df32{smem[i * 32].x, smem[i * 32].y};
    __syncthreads();
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block reduction of NV per-thread FP32 values: FP32 within each warp (32 values), double-float
// across the warps (warp 0). Thread 0 gets the block totals. smem needs NV * 32 floats; the caller
// must pass a __syncthreads() before smem is written again.
template <int NV>
__device__ __forceinline__ void block_reduce_f(const float (&v)[NV], float *smem, df32 (&out)[NV]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const float w = warp_sum_f(v[i]);
        if (lane == 0) smem[i * 32 + wid] = w;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            df32 t = {lane < nw ? smem[i * 32 + lane] : 0.f, 0.f};
            t = warp_sum_df(t);
            if (lane == 0) out[i] = t;
        }
    }
}

// Every block sums the per-block pairs partials[i*stride + b], b < nb, in the same order; results
// (as doubles, hi + lo) land in s_out[0..NV) in shared memory for the whole block.
template <int NV>
__device__ __forceinline__ void grid_sum_df(const float2 *partials, int stride, int nb, double *s_out) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = wid; i < NV; i += nw) {
        df32 t = {0.f, 0.f};
        for (int b = lane; b < nb; b += 32) {
            const float2 q = __ldcg(partials + i * stride + b);
            t = df_add(t, df32{q.x, q.y});
        }
        t = warp_sum_df(t);
        if (lane == 0) s_out[i] = (double)t.hi + (double)t.lo;
    }
    __syncthreads();
}

// FP64 block reduction through shared memory: one warp per value sums the block's threads, so the
// FP64 pipe sees ~blockDim adds per value instead of a shuffle tree in every warp.
// smem needs NV * blockDim doubles; thread 0 gets out[].
template <int NV>
__device__ __forceinline__ void block_sum_smem(const double (&v)[NV], double *smem, double (&out)[NV]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5, nt = blockDim.x;
#pragma unroll
    for (int i = 0; i < NV; ++i) smem[i * nt + threadIdx.x] = v[i];
    __syncthreads();
    for (int i = wid; i < NV; i += nw) {
        double t = 0.0;
        for (int k = lane; k < nt; k += 32) t += smem[i * nt + k];
        t = warp_sum(t);
        if (lane == 0) smem[i * nt] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) out[i] = smem[i * nt];
    __syncthreads();
}

// FP64 cross-block sums (one warp per value), results in s_out[] for the whole block.
template <int NV>
__device__ __forceinline__ void grid_sum_d(const double *partials, int stride, int nb, double *s_out) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = wid; i < NV; i += nw) {
        double t = 0.0;
        for (int b = lane; b < nb; b += 32) t += __ldcg(partials + i * stride + b);
        t = warp_sum(t);
        if (lane == 0) s_out[i] = t;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// MRG32k3a
// ---------------------------------------------------------------------------
constexpr uint32_t MRG_M1 = 4294967087u;  // 2^32 - 209
constexpr uint32_t MRG_M2 = 4294944443u;  // 2^32 - 22853

__host__ __device__ __forceinline__ uint32_t mod_m1(uint64_t x) {
    x = (x >> 32) * 209ull + (x & 0xffffffffull);
    x = (x >> 32) * 209ull + (x & 0xffffffffull);
    return (uint32_t)(x >= MRG_M1 ? x - MRG_M1 : x);
}
__host__ __device__ __forceinline__ uint32_t mod_m2(uint64_t x) {
    x = (x >> 32) * 22853ull + (x & 0xffffffffull);
    x = (x >> 32) * 22853ull + (x & 0xffffffffull);
    return (uint32_t)(x >= MRG_M2 ? x - MRG_M2 : x);
}

// x mod m1 for x < 2^54: 2^32 = 209 (mod m1), so one fold leaves x < 2^22 209 + 2^32 < 2 m1
__host__ __device__ __forceinline__ uint32_t mod_m1_54(uint64_t x) {
    x = (x >> 32) * 209ull + (x & 0xffffffffull);
    return (uint32_t)(x >= MRG_M1 ? x - MRG_M1 : x);
}
// x mod m2 for x < 2^54: 2^32 = 22853 (mod m2); the first fold leaves x < 2^37, the second < 2 m2
__host__ __device__ __forceinline__ uint32_t mod_m2_54(uint64_t x) {
    x = (x >> 32) * 22853ull + (x & 0xffffffffull);
    x = (x >> 32) * 22853ull + (x & 0xffffffffull);
    return (uint32_t)(x >= MRG_M2 ? x - MRG_M2 : x);
}

// one jump: a pair of 3x3 transition-matrix powers (component 1 mod m1, component 2 mod m2)
struct MrgJump {
    uint32_t a[9];
    uint32_t b[9];
};

// o = J s. Each product a s < 2^64 is folded once before the row sum, hi 2^32 + lo = hi 209 + lo (mod m1) and
// hi 22853 + lo (mod m2): a row of three folded products stays below 3 (2^47 + 2^32) < 2^54, reduced once.
__host__ __device__ __forceinline__ void mrg_apply(const MrgJump &J, const uint32_t s[6], uint32_t o[6]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        uint64_t acc = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint64_t p = (uint64_t)J.a[3 * i + k] * s[k];
            acc += (p >> 32) * 209ull + (p & 0xffffffffull);
        }
        o[i] = mod_m1_54(acc);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        uint64_t acc = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint64_t p = (uint64_t)J.b[3 * i + k] * s[3 + k];
            acc += (p >> 32) * 22853ull + (p & 0xffffffffull);
        }
        o[3 + i] = mod_m2_54(acc);
    }
}

// One MRG32k3a step (RngStream::U01's recurrences, src/RngStream.cpp:266-289, on integers): advances s and
// returns p1 - p2 (+ m1 when p1 <= p2), the integer in [1, m1] whose value / (m1 + 1) is the draw.
// component 1: x_n = 1403580 x_{n-2} - 810728 x_{n-3} (mod m1), formed as 1403580 x_{n-2} + 810728 (m1 - x_{n-3});
// component 2: x_n = 527612 x_{n-1} - 1370589 x_{n-3} (mod m2), likewise; both sums stay below 2^54.
__host__ __device__ __forceinline__ uint32_t mrg_step(uint32_t s[6]) {
    const uint32_t p1 = mod_m1_54(1403580ull * s[1] + 810728ull * (uint64_t)(MRG_M1 - s[0]));
    s[0] = s[1];
    s[1] = s[2];
    s[2] = p1;
    const uint32_t p2 = mod_m2_54(527612ull * s[5] + 1370589ull * (uint64_t)(MRG_M2 - s[3]));
    s[3] = s[4];
    s[4] = s[5];
    s[5] = p2;
    return p1 > p2 ? p1 - p2 : p1 - p2 + MRG_M1;
}

// One MRG32k3a draw in (0,1), formed as RngStream::U01 forms it (src/RngStream.cpp:266-289).
__host__ __device__ __forceinline__ double mrg_u01(uint32_t s[6]) {
    const double norm = 1.0 / (4294967087.0 + 1.0);
    return (double)mrg_step(s) * norm;
}

// RAND(-.5,.5) of include/tetra_element_linear.h:119
__host__ __device__ __forceinline__ double mrg_rand_half(uint32_t s[6]) {
    return (-.5) + ((.5) - (-.5)) * mrg_u01(s);
}

}  // namespace ffea
