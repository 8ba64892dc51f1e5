// btm_team.cuh - execution teams shared by the FP64 and mixed-precision
// engines: one CTA (BlockTeam) or a whole cooperative grid (GridTeam);
// deterministic fixed-order team reductions and a bounded software grid
// barrier.  Header-only device code.
#pragma once
#include "btm_common.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace btm {

// std::max / std::min selection semantics (first argument on ties and NaN)
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smaxf(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float sminf(float a, float b) { return (b < a) ? b : a; }

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr uint64_t kBarrierTimeoutNs = 2000000000ull;  // 2 s: a stuck barrier aborts the solve

// ---------------------------------------------------------------------------
// teams
// ---------------------------------------------------------------------------
struct BlockTeam {
    double *red;   // shared [2][32][kRedSlots]
    int buf;
    __device__ __forceinline__ int rank() const { return threadIdx.x; }
    __device__ __forceinline__ int size() const { return blockDim.x; }
    __device__ __forceinline__ bool leader() const { return threadIdx.x == 0; }
    __device__ __forceinline__ bool sync() { __syncthreads(); return true; }
    __device__ __forceinline__ bool ok() const { return true; }

    // Sum N values over the team; every thread receives the identical totals.
    template <int N>
    __device__ __forceinline__ void sum(double *v) {
#pragma unroll
        for (int j = 0; j < N; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        double *rb = red + buf * 32 * kRedSlots;
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < N; ++j) rb[warp * kRedSlots + j] = v[j];
        __syncthreads();
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = 0.0;
            for (int q = 0; q < nw; ++q) s += rb[q * kRedSlots + j];
            v[j] = s;
        }
        buf ^= 1;
    }
    template <int N>
    __device__ __forceinline__ void maxr(double *v) {
#pragma unroll
        for (int j = 0; j < N; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[j] = smax(v[j], __shfl_xor_sync(0xffffffffu, v[j], o));
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        double *rb = red + buf * 32 * kRedSlots;
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < N; ++j) rb[warp * kRedSlots + j] = v[j];
        __syncthreads();
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = rb[j];
            for (int q = 1; q < nw; ++q) s = smax(s, rb[q * kRedSlots + j]);
            v[j] = s;
        }
        buf ^= 1;
    }

    // FP32 sums (Krylov dot products of the mixed-precision engine): a warp
    // butterfly, then every warp re-reduces the per-warp partials with the
    // same butterfly, so all threads hold identical totals after one barrier.
    // The fold stays in FP32: on GB300 a chain of dependent FP64 additions per
    // reduction doubled the BiCGSTAB time, and pairwise FP32 summation of at
    // most 16k products is accurate to ~1e-6, far inside what the Krylov
    // scalars need (the equation defects themselves are FP64).
    template <int N>
    __device__ __forceinline__ void sumf(float *v) {
#pragma unroll
        for (int j = 0; j < N; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        float *rb = reinterpret_cast<float *>(red + buf * 32 * kRedSlots);   // [slot][warp]
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < N; ++j) rb[j * 32 + warp] = v[j];
        __syncthreads();
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            float s = lane < nw ? rb[j * 32 + lane] : 0.0f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            v[j] = s;
        }
        buf ^= 1;
    }
    // FP64 sums folded across warps by lane 0 only (same totals as sum<N>
    // would give in every thread, with FP64 work per warp instead of per thread)
    template <int N>
    __device__ __forceinline__ void sumd(double *v) {
#pragma unroll
        for (int j = 0; j < N; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        double *rb = red + buf * 32 * kRedSlots;
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < N; ++j) rb[warp * kRedSlots + j] = v[j];
        __syncthreads();
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = 0.0;
            if (lane == 0)
                for (int q = 0; q < nw; ++q) s += rb[q * kRedSlots + j];
            v[j] = __shfl_sync(0xffffffffu, s, 0);
        }
        buf ^= 1;
    }
    // FP32 maxima with smax semantics (a NaN in the first operand survives)
    template <int N>
    __device__ __forceinline__ void maxf(float *v) {
#pragma unroll
        for (int j = 0; j < N; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[j] = smaxf(v[j], __shfl_xor_sync(0xffffffffu, v[j], o));
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        float *rb = reinterpret_cast<float *>(red + buf * 32 * kRedSlots);
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < N; ++j) rb[warp * kRedSlots + j] = v[j];
        __syncthreads();
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            float s = rb[j];
            for (int q = 1; q < nw; ++q) s = smaxf(s, rb[q * kRedSlots + j]);
            v[j] = s;
        }
        buf ^= 1;
    }
};

// One CTA per instance whose AMG solves use the reference-order AMG
// (btm_ramg.cuh).  A distinct type so that only the kernel instantiated for
// it carries that solver in its call graph (the plain kernel keeps its
// register allocation).
struct BlockTeamRef : BlockTeam {};

struct GridTeam {
    double *red;            // shared [2][32][kRedSlots]
    int buf;
    double *gpart;          // global [2][gridDim][kRedSlots]
    unsigned int *bar;      // [0] arrivals, [1] generation
    int32_t *err;
    int *shAbort;           // shared flag
    __device__ __forceinline__ int rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ __forceinline__ int size() const { return gridDim.x * blockDim.x; }
    __device__ __forceinline__ bool leader() const { return blockIdx.x == 0 && threadIdx.x == 0; }
    __device__ __forceinline__ bool ok() const { return *shAbort == 0; }

    // Software grid barrier for a cooperative launch (all CTAs co-resident).
    // Every wait is bounded: after kBarrierTimeoutNs the CTA flags the error
    // and the whole team abandons the solve.
    __device__ bool sync() {
        __syncthreads();
        if (threadIdx.x == 0) {
            volatile unsigned int *vgen = bar + 1;
            unsigned int gen = *vgen;
            __threadfence();
            unsigned int arrived = atomicAdd(bar, 1u);
            if (arrived == gridDim.x - 1) {
                atomicExch(bar, 0u);
                __threadfence();
                atomicAdd(bar + 1, 1u);
            } else {
                uint64_t t0 = globaltimer_ns();
                while (*vgen == gen) {
                    if (*(volatile int32_t *)err) { *shAbort = 1; break; }
                    if (globaltimer_ns() - t0 > kBarrierTimeoutNs) {
                        atomicExch(err, 2);
                        *shAbort = 1;
                        break;
                    }
                    __nanosleep(20);
                }
            }
            __threadfence();
            if (*(volatile int32_t *)err) *shAbort = 1;
        }
        __syncthreads();
        return *shAbort == 0;
    }

    template <int N>
    __device__ void sum(double *v) {
#pragma unroll
        for (int j = 0; j < N; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        double *rb = red + buf * 32 * kRedSlots;
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < N; ++j) rb[warp * kRedSlots + j] = v[j];
        __syncthreads();
        if (threadIdx.x == 0) {
            const int nw = blockDim.x >> 5;
            double *gp = gpart + ((size_t)buf * gridDim.x + blockIdx.x) * kRedSlots;
            for (int j = 0; j < N; ++j) {
                double s = 0.0;
                for (int q = 0; q < nw; ++q) s += rb[q * kRedSlots + j];
                gp[j] = s;
            }
        }
        sync();
        // each lane folds a fixed strided subset of the CTA partials, then a
        // butterfly: identical totals in every thread of every CTA
        const double *gp = gpart + (size_t)buf * gridDim.x * kRedSlots;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = 0.0;
            for (int q = lane; q < (int)gridDim.x; q += 32) s += __ldcg(gp + q * kRedSlots + j);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            v[j] = s;
        }
        buf ^= 1;
    }
    template <int N>
    __device__ void maxr(double *v) {
#pragma unroll
        for (int j = 0; j < N; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[j] = smax(v[j], __shfl_xor_sync(0xffffffffu, v[j], o));
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        double *rb = red + buf * 32 * kRedSlots;
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < N; ++j) rb[warp * kRedSlots + j] = v[j];
        __syncthreads();
        if (threadIdx.x == 0) {
            const int nw = blockDim.x >> 5;
            double *gp = gpart + ((size_t)buf * gridDim.x + blockIdx.x) * kRedSlots;
            for (int j = 0; j < N; ++j) {
                double s = rb[j];
                for (int q = 1; q < nw; ++q) s = smax(s, rb[q * kRedSlots + j]);
                gp[j] = s;
            }
        }
        sync();
        const double *gp = gpart + (size_t)buf * gridDim.x * kRedSlots;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double s = __ldcg(gp + j);
            for (int q = lane; q < (int)gridDim.x; q += 32) s = smax(s, __ldcg(gp + q * kRedSlots + j));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s = smax(s, __shfl_xor_sync(0xffffffffu, s, o));
            v[j] = s;
        }
        buf ^= 1;
    }
    // FP32 values, FP64 accumulation from the warp level up (see BlockTeam::sumf)
    template <int N>
    __device__ void sumf(float *v) {
        double d[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
            d[j] = (double)v[j];
        }
        // the warp-level totals enter the FP64 grid reduction as lane-0 values
        const int lane = threadIdx.x & 31;
        if (lane != 0)
#pragma unroll
            for (int j = 0; j < N; ++j) d[j] = 0.0;
        sum<N>(d);
#pragma unroll
        for (int j = 0; j < N; ++j) v[j] = (float)d[j];
    }
    template <int N>
    __device__ void sumd(double *v) { sum<N>(v); }
    template <int N>
    __device__ void maxf(float *v) {
        double d[N];
#pragma unroll
        for (int j = 0; j < N; ++j) d[j] = (double)v[j];
        maxr<N>(d);
#pragma unroll
        for (int j = 0; j < N; ++j) v[j] = (float)d[j];
    }
};

// Loads that must see writes made by other CTAs in the same launch (after a
// grid barrier) bypass L1: in grid mode every field read goes through __ldcg.
// In block mode one CTA owns the data and plain loads are coherent.
template <class T> struct Ld;
template <> struct Ld<BlockTeam> {
    __device__ __forceinline__ static double f(const double *p) { return *p; }
    __device__ __forceinline__ static float f(const float *p) { return *p; }
};
template <> struct Ld<BlockTeamRef> : Ld<BlockTeam> {};
template <> struct Ld<GridTeam> {
    __device__ __forceinline__ static double f(const double *p) { return __ldcg(p); }
    __device__ __forceinline__ static float f(const float *p) { return __ldcg(p); }
};
#define LD(ptr) (Ld<T>::f(ptr))

}  // namespace btm
