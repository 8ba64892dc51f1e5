// btm_engine.cu - the GB300 SIMPLE / SST k-omega engine (sm_103a).
//
// One persistent launch runs a whole forward solve G(x, theta): every phase of
// the reference outer iteration (incompressible/src/SIMPLESolver.cpp:731-1036)
// is a device function templated on a "team":
//   * BlockTeam - one CTA owns one instance (small meshes; a batch of N
//     instances is a grid of N CTAs, each retiring when its solve ends);
//   * GridTeam  - every CTA of a cooperative launch owns one large instance,
//     phases separated by a bounded software grid barrier.
// Control flow is team-uniform: all decisions use values every thread of the
// team computed identically (deterministic fixed-order reductions).
//
// Floating point: the file is compiled with -fmad=false and every face sum is
// evaluated per cell in ascending face order, the order in which the
// reference's face loops scatter into that cell.  Assembly, gradients and the
// LDU mat-vec therefore round exactly like the reference; only dot products
// (parallel trees) and transcendental library calls differ in the last bits.
// There are no floating-point atomics anywhere.
#include "btm_common.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace btm {

// std::max / std::min selection semantics (first argument on ties and NaN)
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int kThreads = 512;
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
};

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
};

// CTA 0 working alone inside a grid launch (coarse AMG levels): same as a
// BlockTeam but its loads bypass L1 like the grid team's.
struct BlockTeamCG : BlockTeam {};

// Loads that must see writes made by other CTAs in the same launch (after a
// grid barrier) bypass L1: in grid mode every field read goes through __ldcg.
// In block mode one CTA owns the data and plain loads are coherent.
template <class T> struct Ld;
template <> struct Ld<BlockTeam> {
    __device__ __forceinline__ static double f(const double *p) { return *p; }
};
template <> struct Ld<GridTeam> {
    __device__ __forceinline__ static double f(const double *p) { return __ldcg(p); }
};
template <> struct Ld<BlockTeamCG> {
    __device__ __forceinline__ static double f(const double *p) { return __ldcg(p); }
};
#define LD(ptr) (Ld<T>::f(ptr))

// ---------------------------------------------------------------------------
// SST point functions (core/src/SSTModel.cpp:9-96, core/include/SSTModel.hpp:30-39)
// ---------------------------------------------------------------------------
struct Coef {
    double sk1, sw1, b1, al1, sk2, sw2, b2, al2, bstar, a1, kappa;
    int variant;
};
__device__ __forceinline__ Coef load_coef(const DevInst &I) {
    Coef c;
    c.sk1 = I.coeff[0]; c.sw1 = I.coeff[1]; c.b1 = I.coeff[2]; c.al1 = I.coeff[3];
    c.sk2 = I.coeff[4]; c.sw2 = I.coeff[5]; c.b2 = I.coeff[6]; c.al2 = I.coeff[7];
    c.bstar = I.coeff[8]; c.a1 = I.coeff[9]; c.kappa = I.coeff[10];
    c.variant = I.variant;
    return c;
}
__device__ __forceinline__ double blend(double p1, double p2, double F1) { return F1 * p1 + (1.0 - F1) * p2; }

__device__ __forceinline__ double sst_F1(const Coef &c, double k, double omega, double y, double nu, double CDkw_pos) {
    double sqrtK = sqrt(smax(k, 0.0));
    double omSafe = smax(omega, 1e-20);
    double ySafe = smax(y, 1e-20);
    double y2s = ySafe * ySafe;
    double term1 = sqrtK / (c.bstar * omSafe * ySafe);
    double term2 = 500.0 * nu / (y2s * omSafe);
    double CDpos = smax(CDkw_pos, 1e-20);
    double term3 = 4.0 * c.sw2 * smax(k, 0.0) / (CDpos * y2s);
    double arg1 = smin(smax(term1, term2), term3);
    double a4 = arg1 * arg1 * arg1 * arg1;
    return tanh(a4);
}
__device__ __forceinline__ double sst_F2(const Coef &c, double k, double omega, double y, double nu) {
    double sqrtK = sqrt(smax(k, 0.0));
    double omSafe = smax(omega, 1e-20);
    double ySafe = smax(y, 1e-20);
    double y2 = ySafe * ySafe;
    double term1 = 2.0 * sqrtK / (c.bstar * omSafe * ySafe);
    double term2 = 500.0 * nu / (y2 * omSafe);
    double arg2 = smax(term1, term2);
    return tanh(arg2 * arg2);
}
__device__ __forceinline__ double sst_nut(const Coef &c, double k, double omega, double S, double F2) {
    double kSafe = smax(k, 0.0);
    if (c.variant == 1) return kSafe / smax(omega, 1e-20);
    double denom = smax(c.a1 * omega, S * F2);
    denom = smax(denom, 1e-20);
    return c.a1 * kSafe / denom;
}
__device__ __forceinline__ double sst_Pk(const Coef &c, double nuT, double S, double k, double omega) {
    double Pk_raw = nuT * S * S;
    double Pk_lim = 10.0 * c.bstar * smax(k, 0.0) * smax(omega, 1e-20);
    return smin(Pk_raw, Pk_lim);
}
__device__ __forceinline__ double sst_Pw(const Coef &c, double nuT, double S, double k, double omega) {
    double S2 = S * S;
    double lim = 10.0 * c.bstar * smax(k, 0.0) * smax(omega, 1e-20) / smax(nuT, 1e-30);
    return smin(S2, lim);
}

// ---------------------------------------------------------------------------
// Green-Gauss gradients (core/include/Field.hpp:122-152): per cell, internal
// faces in ascending face order, then boundary faces, then / V.
// ---------------------------------------------------------------------------
template <class T, int NF>
__device__ __forceinline__ void gg_cell(const DevMesh &M, int c, const double *const *phi,
                                        const double *const *phib, double *gx, double *gy, double *gz) {
    double ax[NF], ay[NF], az[NF], pc[NF];
#pragma unroll
    for (int q = 0; q < NF; ++q) { ax[q] = 0.0; ay[q] = 0.0; az[q] = 0.0; pc[q] = LD(phi[q] + c); }
    const int e0 = M.cfOff[c], e1 = M.cfOff[c + 1];
    for (int e = e0; e < e1; ++e) {
        const int f = M.cfFace[e];
        const int oth = M.cfOther[e];
        const double w = M.w[f], sx = M.sfx[f], sy = M.sfy[f], sz = M.sfz[f];
        if (oth >= 0) {
#pragma unroll
            for (int q = 0; q < NF; ++q) {
                double phiF = pc[q] * w + LD(phi[q] + oth) * (1.0 - w);
                ax[q] = ax[q] + sx * phiF;
                ay[q] = ay[q] + sy * phiF;
                az[q] = az[q] + sz * phiF;
            }
        } else {
            const int o = -(oth + 1);
#pragma unroll
            for (int q = 0; q < NF; ++q) {
                double phiF = LD(phi[q] + o) * w + pc[q] * (1.0 - w);
                ax[q] = ax[q] - sx * phiF;
                ay[q] = ay[q] - sy * phiF;
                az[q] = az[q] - sz * phiF;
            }
        }
    }
    const int b0 = M.cbOff[c], b1 = M.cbOff[c + 1];
    for (int e = b0; e < b1; ++e) {
        const int b = M.cbFace[e];
        const double sx = M.bsfx[b], sy = M.bsfy[b], sz = M.bsfz[b];
#pragma unroll
        for (int q = 0; q < NF; ++q) {
            double pb = LD(phib[q] + b);
            ax[q] = ax[q] + sx * pb;
            ay[q] = ay[q] + sy * pb;
            az[q] = az[q] + sz * pb;
        }
    }
    const double V = M.vol[c];
    if (V > 1e-30) {
#pragma unroll
        for (int q = 0; q < NF; ++q) { ax[q] = ax[q] / V; ay[q] = ay[q] / V; az[q] = az[q] / V; }
    }
#pragma unroll
    for (int q = 0; q < NF; ++q) { gx[q] = ax[q]; gy[q] = ay[q]; gz[q] = az[q]; }
}

// gradient of one scalar into (gx, gy, gz)
template <class T>
__device__ __noinline__ void phase_grad1(T &tm, const DevMesh &M, const double *phi, const double *phib,
                            double *ox, double *oy, double *oz) {
    const double *P[1] = {phi};
    const double *PB[1] = {phib};
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        double gx[1], gy[1], gz[1];
        gg_cell<T, 1>(M, c, P, PB, gx, gy, gz);
        ox[c] = gx[0]; oy[c] = gy[0]; oz[c] = gz[0];
    }
}

// velocity gradients (Field.hpp:232-246): g[3*i+j] = dU_i/dx_j; `which` selects
// components (bit i) so a partially updated U only recomputes what changed
template <class T>
__device__ __noinline__ void phase_velgrad(T &tm, const DevMesh &M, DevInst &I, int which) {
    const double *U[3] = {I.ux, I.uy, I.uz};
    const double *UB[3] = {I.ubx, I.uby, I.ubz};
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        if (which == 7) {
            double gx[3], gy[3], gz[3];
            gg_cell<T, 3>(M, c, U, UB, gx, gy, gz);
#pragma unroll
            for (int i = 0; i < 3; ++i) { I.g[3 * i][c] = gx[i]; I.g[3 * i + 1][c] = gy[i]; I.g[3 * i + 2][c] = gz[i]; }
        } else {
            for (int i = 0; i < 3; ++i) {
                if (!(which & (1 << i))) continue;
                const double *P[1] = {U[i]};
                const double *PB[1] = {UB[i]};
                double gx[1], gy[1], gz[1];
                gg_cell<T, 1>(M, c, P, PB, gx, gy, gz);
                I.g[3 * i][c] = gx[0]; I.g[3 * i + 1][c] = gy[0]; I.g[3 * i + 2][c] = gz[0];
            }
        }
    }
}

// SSTModel::computeFields + frozen |S| + startup floor (SIMPLESolver.cpp:736-768).
// Requires velocity gradients in I.g.  nutMin < 0 skips the floor.
template <class T>
__device__ __noinline__ void phase_sst(T &tm, const DevMesh &M, DevInst &I, double nutMin) {
    const Coef cf = load_coef(I);
    const double nu = I.nu;
    const double *P[2] = {I.k, I.om};
    const double *PB[2] = {I.kb, I.omb};
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        double S11 = LD(I.g[0] + c), S22 = LD(I.g[4] + c), S33 = LD(I.g[8] + c);
        double S12 = 0.5 * (LD(I.g[1] + c) + LD(I.g[3] + c));
        double S13 = 0.5 * (LD(I.g[2] + c) + LD(I.g[6] + c));
        double S23 = 0.5 * (LD(I.g[5] + c) + LD(I.g[7] + c));
        double Sc = sqrt(2.0 * (S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23)));
        double gx[2], gy[2], gz[2];
        gg_cell<T, 2>(M, c, P, PB, gx, gy, gz);
        double kc = smax(LD(I.k + c), 0.0);
        double wc = smax(LD(I.om + c), 1e-20);
        double y = smax(M.wd[c], 1e-20);
        double omSafe = smax(wc, 1e-20);
        double CDkw = 2.0 * cf.sw2 / omSafe * (gx[0] * gx[1] + gy[0] * gy[1] + gz[0] * gz[1]);
        double CDpos = smax(CDkw, 1e-20);
        double F1 = (cf.variant == 2) ? 1.0 : sst_F1(cf, kc, wc, y, nu, CDpos);
        double F2 = sst_F2(cf, kc, wc, y, nu);
        double nuT = sst_nut(cf, kc, wc, Sc, F2);
        double Pk = sst_Pk(cf, nuT, Sc, kc, wc);
        I.smag[c] = Sc;
        I.cdkw[c] = CDkw;
        I.f1[c] = F1;
        I.f2[c] = F2;
        I.pk[c] = Pk;
        I.nut[c] = (nutMin < 0.0) ? nuT : smax(nuT, nutMin);
    }
}

// ---------------------------------------------------------------------------
// assembly (SIMPLESolver.cpp:56-203, 322-450, 483-669)
// ---------------------------------------------------------------------------
// Face pass of the momentum system: upper/lower coefficients and the
// transpose-stress flux of component `comp` (StressOperators.hpp:331-340).
template <class T>
__device__ __noinline__ void phase_mom_faces(T &tm, const DevMesh &M, DevInst &I, int comp) {
    const double nu = I.nu;
    const double *gc0 = I.g[comp], *gc1 = I.g[3 + comp], *gc2 = I.g[6 + comp];
    for (int f = tm.rank(); f < M.nIF; f += tm.size()) {
        const int o = M.own[f], n = M.nbr[f];
        const double Sf = M.area[f], delta = M.deltaC[f], w = M.w[f];
        const double nuo = LD(I.nut + o), nun = LD(I.nut + n);
        double nuEff_o = nu + nuo;
        double nuEff_n = nu + nun;
        double nuEff_f = w * nuEff_o + (1.0 - w) * nuEff_n;
        double Df = nuEff_f * Sf / delta;
        double Ufx = LD(I.ux + o) * w + LD(I.ux + n) * (1.0 - w);
        double Ufy = LD(I.uy + o) * w + LD(I.uy + n) * (1.0 - w);
        double Ufz = LD(I.uz + o) * w + LD(I.uz + n) * (1.0 - w);
        const double nx = M.nx[f], ny = M.ny[f], nz = M.nz[f];
        double mFlux = (Ufx * nx + Ufy * ny + Ufz * nz) * Sf;
        double cPos = smax(mFlux, 0.0);
        double cNeg = smax(-mFlux, 0.0);
        I.upper[f] = -(Df + cNeg);
        I.lower[f] = -(Df + cPos);
        double cfac = w * nuo + (1.0 - w) * nun;
        double gx = LD(gc0 + o) * w + LD(gc0 + n) * (1.0 - w);
        double gy = LD(gc1 + o) * w + LD(gc1 + n) * (1.0 - w);
        double gz = LD(gc2 + o) * w + LD(gc2 + n) * (1.0 - w);
        I.fflux[f] = cfac * (gx * nx + gy * ny + gz * nz) * Sf;
    }
}

// Cell pass of the momentum system (diag, source, relaxation).
template <class T>
__device__ __noinline__ void phase_mom_cells(T &tm, const DevMesh &M, DevInst &I, int comp) {
    const double nu = I.nu;
    const double alphaU = I.S.alphaU;
    const double fb = I.S.bodyForce[comp];
    const double *Uc = comp == 0 ? I.ux : (comp == 1 ? I.uy : I.uz);
    const double *Ubc = comp == 0 ? I.ubx : (comp == 1 ? I.uby : I.ubz);
    const double *gp = comp == 0 ? I.gpx : (comp == 1 ? I.gpy : I.gpz);
    const double *gc0 = I.g[comp], *gc1 = I.g[3 + comp], *gc2 = I.g[6 + comp];
    const bool wallFn = I.S.useWallFn != 0;
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        double diag = 0.0, ts = 0.0, src = 0.0;
        const int e0 = M.cfOff[c], e1 = M.cfOff[c + 1];
        for (int e = e0; e < e1; ++e) {
            const int f = M.cfFace[e];
            if (M.cfOther[e] >= 0) {
                diag = diag + (-LD(I.lower + f));
                ts = ts + LD(I.fflux + f);
            } else {
                diag = diag + (-LD(I.upper + f));
                ts = ts - LD(I.fflux + f);
            }
        }
        const double nutc = LD(I.nut + c);
        for (int e = M.cbOff[c]; e < M.cbOff[c + 1]; ++e) {
            const int b = M.cbFace[e];
            const double Sf = M.barea[b], delta = M.bdeltaC[b];
            double nuEff = (M.bwall[b] && !wallFn) ? nu : nu + nutc;
            double Db = nuEff * Sf / delta;
            double Ub = LD(Ubc + b);
            double mFlux = (LD(I.ubx + b) * M.bnx[b] + LD(I.uby + b) * M.bny[b] + LD(I.ubz + b) * M.bnz[b]) * Sf;
            if (mFlux >= 0) {
                diag = diag + (mFlux + Db);
                src = src + Db * Ub;
            } else {
                diag = diag + Db;
                src = src + (Db - mFlux) * Ub;
            }
        }
        // transpose stress, wall-aware boundary treatment in patch order
        const double gcx = LD(gc0 + c), gcy = LD(gc1 + c), gcz = LD(gc2 + c);
        for (int e = M.cbpOff[c]; e < M.cbpOff[c + 1]; ++e) {
            const int b = M.cbpFace[e];
            double cfac = M.bwall[b] ? 0.0 : nutc;
            double flux = cfac * (gcx * M.bnx[b] + gcy * M.bny[b] + gcz * M.bnz[b]) * M.barea[b];
            ts = ts + flux;
        }
        const double vol = M.vol[c];
        src = src - LD(gp + c) * vol;
        if (fb != 0.0) src = src + fb * vol;
        src = src + ts;
        const double phi_old = LD(Uc + c);
        src = src + (1.0 - alphaU) / alphaU * diag * phi_old;
        diag = diag / alphaU;
        I.diag[c] = diag;
        I.src[c] = src;
        if (comp == 0) I.aPx[c] = diag;
    }
}

// Pressure-correction face pass: Laplacian coefficient and (Rhie-Chow) mass flux.
template <class T>
__device__ __noinline__ void phase_p_faces(T &tm, const DevMesh &M, DevInst &I) {
    const bool rc = M.rhieChow != 0;
    for (int f = tm.rank(); f < M.nIF; f += tm.size()) {
        const int o = M.own[f], n = M.nbr[f];
        const double Sf = M.area[f], delta = M.deltaC[f], w = M.w[f];
        const double Vo = M.vol[o], Vn = M.vol[n];
        const double aPo = LD(I.aPx + o), aPn = LD(I.aPx + n);
        double dP_o = (fabs(aPo) > 1e-30) ? Vo / aPo : 0.0;
        double dP_n = (fabs(aPn) > 1e-30) ? Vn / aPn : 0.0;
        double dP_f = w * dP_o + (1.0 - w) * dP_n;
        double coeff = dP_f * Sf / delta;
        I.upper[f] = -coeff;
        I.lower[f] = -coeff;
        double Ufx = LD(I.ux + o) * w + LD(I.ux + n) * (1.0 - w);
        double Ufy = LD(I.uy + o) * w + LD(I.uy + n) * (1.0 - w);
        double Ufz = LD(I.uz + o) * w + LD(I.uz + n) * (1.0 - w);
        double massFlux = (Ufx * M.nx[f] + Ufy * M.ny[f] + Ufz * M.nz[f]) * Sf;
        if (rc) {
            double gbx = LD(I.gpx + o) * w + LD(I.gpx + n) * (1.0 - w);
            double gby = LD(I.gpy + o) * w + LD(I.gpy + n) * (1.0 - w);
            double gbz = LD(I.gpz + o) * w + LD(I.gpz + n) * (1.0 - w);
            massFlux += -dP_f * Sf * ((LD(I.p + n) - LD(I.p + o)) / delta - (gbx * M.ex[f] + gby * M.ey[f] + gbz * M.ez[f]));
        }
        I.fflux[f] = massFlux;
    }
}

template <class T>
__device__ __noinline__ void phase_p_cells(T &tm, const DevMesh &M, DevInst &I) {
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        double diag = 0.0, src = 0.0;
        for (int e = M.cfOff[c]; e < M.cfOff[c + 1]; ++e) {
            const int f = M.cfFace[e];
            diag = diag + (-LD(I.upper + f));
            if (M.cfOther[e] >= 0) src = src - LD(I.fflux + f);
            else src = src + LD(I.fflux + f);
        }
        const double aPc = LD(I.aPx + c);
        for (int e = M.cbpOff[c]; e < M.cbpOff[c + 1]; ++e) {
            const int b = M.cbpFace[e];
            const double Sf = M.barea[b];
            double massFlux = (LD(I.ubx + b) * M.bnx[b] + LD(I.uby + b) * M.bny[b] + LD(I.ubz + b) * M.bnz[b]) * Sf;
            src = src - massFlux;
            if (M.bout[b]) {
                double dP_o = (fabs(aPc) > 1e-30) ? M.vol[c] / aPc : 0.0;
                double coeff = dP_o * Sf / M.bdeltaC[b];
                diag = diag + coeff;
            }
        }
        if (!M.hasOutlet && c == 0) diag += fabs(diag) > 1e-30 ? diag : 1.0;
        I.diag[c] = diag;
        I.src[c] = src;
        I.pp[c] = 0.0;
    }
}

// k (which = 0) or omega (which = 1) face pass
template <class T>
__device__ __noinline__ void phase_turb_faces(T &tm, const DevMesh &M, DevInst &I, int which) {
    const Coef cf = load_coef(I);
    const double nu = I.nu;
    const double s1 = which == 0 ? cf.sk1 : cf.sw1, s2 = which == 0 ? cf.sk2 : cf.sw2;
    for (int f = tm.rank(); f < M.nIF; f += tm.size()) {
        const int o = M.own[f], n = M.nbr[f];
        const double Sf = M.area[f], delta = M.deltaC[f], w = M.w[f];
        double F1_f = w * LD(I.f1 + o) + (1.0 - w) * LD(I.f1 + n);
        double sg = blend(s1, s2, F1_f);
        double nuEff_o = nu + sg * LD(I.nut + o);
        double nuEff_n = nu + sg * LD(I.nut + n);
        double nuEff_f = w * nuEff_o + (1.0 - w) * nuEff_n;
        double Df = nuEff_f * Sf / delta;
        double Ufx = LD(I.ux + o) * w + LD(I.ux + n) * (1.0 - w);
        double Ufy = LD(I.uy + o) * w + LD(I.uy + n) * (1.0 - w);
        double Ufz = LD(I.uz + o) * w + LD(I.uz + n) * (1.0 - w);
        double mFlux = (Ufx * M.nx[f] + Ufy * M.ny[f] + Ufz * M.nz[f]) * Sf;
        double cPos = smax(mFlux, 0.0);
        double cNeg = smax(-mFlux, 0.0);
        I.upper[f] = -(Df + cNeg);
        I.lower[f] = -(Df + cPos);
    }
}

template <class T>
__device__ __noinline__ void phase_turb_cells(T &tm, const DevMesh &M, DevInst &I, int which) {
    const Coef cf = load_coef(I);
    const double nu = I.nu;
    const double s1 = which == 0 ? cf.sk1 : cf.sw1, s2 = which == 0 ? cf.sk2 : cf.sw2;
    const double *phib = which == 0 ? I.kb : I.omb;
    const double *phi = which == 0 ? I.k : I.om;
    const double alpha = which == 0 ? I.S.alphaK : I.S.alphaW;
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        double diag = 0.0, src = 0.0;
        for (int e = M.cfOff[c]; e < M.cfOff[c + 1]; ++e) {
            const int f = M.cfFace[e];
            if (M.cfOther[e] >= 0) diag = diag + (-LD(I.lower + f));
            else diag = diag + (-LD(I.upper + f));
        }
        const double F1c = LD(I.f1 + c), nutc = LD(I.nut + c);
        for (int e = M.cbOff[c]; e < M.cbOff[c + 1]; ++e) {
            const int b = M.cbFace[e];
            const double Sf = M.barea[b], delta = M.bdeltaC[b];
            double sg = blend(s1, s2, F1c);
            double nuEff = nu + sg * nutc;
            double Db = nuEff * Sf / delta;
            double vb = LD(phib + b);
            double mFlux = (LD(I.ubx + b) * M.bnx[b] + LD(I.uby + b) * M.bny[b] + LD(I.ubz + b) * M.bnz[b]) * Sf;
            if (mFlux >= 0) {
                diag = diag + (mFlux + Db);
                src = src + Db * vb;
            } else {
                diag = diag + Db;
                src = src + (Db - mFlux) * vb;
            }
        }
        const double vol = M.vol[c];
        const double omc = LD(I.om + c);
        if (which == 0) {
            src = src + LD(I.pk + c) * vol;
            double destruction = cf.bstar * smax(omc, 1e-20);
            diag = diag + destruction * vol;
        } else {
            double omC = smax(omc, 1e-20);
            double alphaB = blend(cf.al1, cf.al2, F1c);
            double S = LD(I.smag + c);
            src = src + alphaB * sst_Pw(cf, nutc, S, LD(I.k + c), omc) * vol;
            double betaB = blend(cf.b1, cf.b2, F1c);
            diag = diag + betaB * omC * vol;
            src = src + (1.0 - F1c) * LD(I.cdkw + c) * vol;
        }
        src = src + (1.0 - alpha) / alpha * diag * LD(phi + c);
        diag = diag / alpha;
        I.diag[c] = diag;
        I.src[c] = src;
    }
}

// ---------------------------------------------------------------------------
// boundary conditions (core/include/BoundaryCondition.hpp:196-342)
// ---------------------------------------------------------------------------
template <class T>
__device__ void phase_bc_u(T &tm, const DevMesh &M, DevInst &I) {
    for (int b = tm.rank(); b < M.nB; b += tm.size()) {
        const int code = M.bcU[b];
        if (code == BC_NONE) continue;
        const int o = M.bown[b];
        if (code == BC_FIXED) {
            I.ubx[b] = M.bvUx[b]; I.uby[b] = M.bvUy[b]; I.ubz[b] = M.bvUz[b];
        } else if (code == BC_SYMMETRY) {
            double ux = LD(I.ux + o), uy = LD(I.uy + o), uz = LD(I.uz + o);
            double nx = M.bnx[b], ny = M.bny[b], nz = M.bnz[b];
            double d = ux * nx + uy * ny + uz * nz;
            I.ubx[b] = ux - nx * d; I.uby[b] = uy - ny * d; I.ubz[b] = uz - nz * d;
        } else {
            I.ubx[b] = LD(I.ux + o); I.uby[b] = LD(I.uy + o); I.ubz[b] = LD(I.uz + o);
        }
    }
}
template <class T>
__device__ void phase_bc_p(T &tm, const DevMesh &M, DevInst &I) {
    for (int b = tm.rank(); b < M.nB; b += tm.size()) {
        const int code = M.bcP[b];
        if (code == BC_NONE) continue;
        I.pb[b] = (code == BC_FIXED) ? M.bvP[b] : LD(I.p + M.bown[b]);
    }
}
// clamp the boundary values (Field::clamp, Field.hpp:89-92) then the k BC
template <class T>
__device__ void phase_bc_k(T &tm, const DevMesh &M, DevInst &I, bool clamp) {
    const double lo = I.S.kMin, hi = I.S.kMax;
    for (int b = tm.rank(); b < M.nB; b += tm.size()) {
        const int code = M.bcK[b];
        double v = I.kb[b];
        if (clamp) v = smax(lo, smin(hi, v));
        if (code == BC_FIXED) v = M.bvK[b];
        else if (code == BC_ZEROGRAD) v = LD(I.k + M.bown[b]);
        I.kb[b] = v;
    }
}
template <class T>
__device__ void phase_bc_w(T &tm, const DevMesh &M, DevInst &I, double beta1, bool clamp) {
    const double lo = I.S.omegaMin, hi = 1e15, nu = I.nu;
    for (int b = tm.rank(); b < M.nB; b += tm.size()) {
        const int code = M.bcW[b];
        double v = I.omb[b];
        if (clamp) v = smax(lo, smin(hi, v));
        if (code == BC_FIXED) v = M.bvW[b];
        else if (code == BC_ZEROGRAD) v = LD(I.om + M.bown[b]);
        else if (code == BC_WALL_OMEGA) {
            double y1 = M.bdeltaW[b];
            v = 60.0 * nu / (beta1 * y1 * y1);
        }
        I.omb[b] = v;
    }
}

// ---------------------------------------------------------------------------
// linear algebra on the LDU system (core/include/LinearSolver.hpp)
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the Krylov and
// multigrid loops avoid FP64 divisions (reciprocal diagonals computed once per
// solve) and use fused multiply-adds.  These solvers already differ from the
// reference in the last bits through their parallel dot products, so nothing
// is lost: the assembly above keeps the reference's exact rounding.
// ---------------------------------------------------------------------------
// y = A x for one cell: diag*x, then face terms in ascending face order
template <class T>
__device__ __forceinline__ double ldu_row(const DevMesh &M, const DevInst &I, const double *x, int c) {
    double y = LD(I.diag + c) * LD(x + c);
    for (int e = M.cfOff[c]; e < M.cfOff[c + 1]; ++e) {
        const int f = M.cfFace[e];
        const int oth = M.cfOther[e];
        if (oth >= 0) y = fma(LD(I.upper + f), LD(x + oth), y);
        else y = fma(LD(I.lower + f), LD(x + (-(oth + 1))), y);
    }
    return y;
}
// reciprocal for the Jacobi preconditioner (LinearSolver.hpp:137-140): rows
// with |diag| <= 1e-30 pass the residual through unscaled
__device__ __forceinline__ double jac_rd(double d) { return (fabs(d) > 1e-30) ? 1.0 / d : 1.0; }
// reciprocal for Gauss-Seidel rows: 0 marks a row the sweep leaves unchanged
__device__ __forceinline__ double gs_rd(double d) { return (fabs(d) > 1e-30) ? 1.0 / d : 0.0; }

struct SolveResult {
    int iterations;
    double finalRes, initialRes;
    int converged;
};

// BiCGSTABSolver::solve (LinearSolver.hpp:191-247), right Jacobi preconditioned.
// x is updated in place; A = (I.diag, I.upper, I.lower), b = I.src.
template <class T>
__device__ __noinline__ SolveResult team_bicgstab(T &tm, const DevMesh &M, DevInst &I, double *x, int maxIter, double tol) {
    SolveResult res = {0, 0.0, 0.0, 0};
    const int nC = M.nC;
    double acc[2] = {0.0, 0.0};
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        double rc = LD(I.src + c) - ldu_row<T>(M, I, x, c);
        I.r[c] = rc; I.rh[c] = rc; I.pv[c] = 0.0; I.v[c] = 0.0;
        I.rd[c] = jac_rd(LD(I.diag + c));
        acc[0] = fma(rc, rc, acc[0]);
        acc[1] = fma(rc, rc, acc[1]);
    }
    tm.template sum<2>(acc);
    const double r0 = sqrt(acc[0]);
    res.initialRes = r0;
    if (r0 < 1e-30) { res.converged = 1; return res; }
    double rhoN = acc[1];
    double rho = 1, alpha = 1, omega = 1;
    for (int it = 0; it < maxIter; ++it) {
        if (!tm.ok()) break;
        if (fabs(rhoN) < 1e-30) break;
        const double beta = (rhoN / (rho + 1e-30)) * (alpha / (omega + 1e-30));
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            double p = fma(beta, fma(-omega, LD(I.v + c), LD(I.pv + c)), LD(I.r + c));
            I.pv[c] = p;
            I.ph[c] = p * LD(I.rd + c);
        }
        tm.sync();
        double a1[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            double vc = ldu_row<T>(M, I, I.ph, c);
            I.v[c] = vc;
            a1[0] = fma(LD(I.rh + c), vc, a1[0]);
        }
        tm.template sum<1>(a1);
        const double rv = a1[0];
        if (fabs(rv) < 1e-30) break;
        alpha = rhoN / rv;
        double a2[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            double sc = fma(-alpha, LD(I.v + c), LD(I.r + c));
            I.s[c] = sc;
            I.sh[c] = sc * LD(I.rd + c);
            a2[0] = fma(sc, sc, a2[0]);
        }
        tm.template sum<1>(a2);
        const double sn = sqrt(a2[0]);
        if (sn / r0 < tol) {
            for (int c = tm.rank(); c < nC; c += tm.size()) x[c] = fma(alpha, LD(I.ph + c), LD(x + c));
            res.iterations = it + 1; res.finalRes = sn / r0; res.converged = 1;
            tm.sync();
            return res;
        }
        double a3[2] = {0.0, 0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            double tc = ldu_row<T>(M, I, I.sh, c);
            I.t[c] = tc;
            a3[0] = fma(tc, tc, a3[0]);
            a3[1] = fma(tc, LD(I.s + c), a3[1]);
        }
        tm.template sum<2>(a3);
        const double tt = a3[0];
        omega = (tt > 1e-30) ? a3[1] / tt : 0.0;
        double a4[2] = {0.0, 0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            x[c] = LD(x + c) + fma(alpha, LD(I.ph + c), omega * LD(I.sh + c));
            double rc = fma(-omega, LD(I.t + c), LD(I.s + c));
            I.r[c] = rc;
            a4[0] = fma(rc, rc, a4[0]);
            a4[1] = fma(LD(I.rh + c), rc, a4[1]);
        }
        tm.template sum<2>(a4);
        const double rn = sqrt(a4[0]);
        res.iterations = it + 1;
        res.finalRes = rn / r0;
        if (res.finalRes < tol) { res.converged = 1; return res; }
        if (fabs(omega) < 1e-30) break;
        rho = rhoN;
        rhoN = a4[1];
    }
    return res;
}

// ---- pressure AMG ---------------------------------------------------------
__device__ __forceinline__ double *lev_vals(DevInst &I, const DevMesh &M, int l) {
    return l == 0 ? I.diag : I.amgVal + M.lev[l].valOff;
}
__device__ __forceinline__ double *lev_x(DevInst &I, const DevMesh &M, int l) {
    return l == 0 ? I.s : I.amgX + M.lev[l].vecOff;
}
__device__ __forceinline__ double *lev_b(DevInst &I, const DevMesh &M, int l) {
    return l == 0 ? I.r : I.amgB + M.lev[l].vecOff;
}
__device__ __forceinline__ double *lev_r(DevInst &I, const DevMesh &M, int l) {
    return l == 0 ? I.t : I.amgR + M.lev[l].vecOff;
}
// Gauss-Seidel reciprocal diagonals: level 0 at [0, nC), level l at nC + vecOff
__device__ __forceinline__ double *lev_rd(DevInst &I, const DevMesh &M, int l) {
    return l == 0 ? I.amgRd : I.amgRd + M.nC + M.lev[l].vecOff;
}

// numeric Galerkin update of level l from level l-1 (fixed gather order)
template <class T>
__device__ void amg_galerkin(T &tm, const DevMesh &M, DevInst &I, int l) {
    const AmgLevelDev &L = M.lev[l];
    const double *fine = lev_vals(I, M, l - 1);
    double *val = lev_vals(I, M, l);
    for (int k = tm.rank(); k < L.nnz; k += tm.size()) {
        double s = 0.0;
        for (int q = L.gOff[k]; q < L.gOff[k + 1]; ++q) s += LD(fine + L.gIdx[q]);
        val[k] = s;
    }
}

// reciprocal diagonals of level l (after its values are final)
template <class T>
__device__ void amg_level_rd(T &tm, const DevMesh &M, DevInst &I, int l) {
    const AmgLevelDev &L = M.lev[l];
    double *rd = lev_rd(I, M, l);
    const double *val = lev_vals(I, M, l);
    for (int i = tm.rank(); i < L.n; i += tm.size()) {
        double d;
        if (l == 0) d = LD(I.diag + i);
        else d = L.diagPos[i] >= 0 ? LD(val + L.diagPos[i]) : 0.0;
        rd[i] = gs_rd(d);
    }
}

// dense inverse of the coarsest level by Gauss-Jordan with ping-pong buffers;
// one reciprocal per pivot, no pivoting (the level matrix is SPD: Galerkin
// product of the pinned / Dirichlet-bounded pressure Laplacian)
template <class T>
__device__ __noinline__ void amg_coarse_inverse(T &tm, const DevMesh &M, DevInst &I) {
    const int l = M.nLevels - 1;
    const AmgLevelDev &L = M.lev[l];
    const int n = L.n, w2 = 2 * n;
    double *A = I.gj, *B = I.gj + (size_t)n * w2;
    const double *val = lev_vals(I, M, l);
    for (int i = tm.rank(); i < n; i += tm.size()) {
        double *row = A + (size_t)i * w2;
        for (int j = 0; j < w2; ++j) row[j] = 0.0;
        if (l == 0) {
            row[i] = LD(I.diag + i);  // level 0 as coarsest: LDU rows
            for (int e = M.cfOff[i]; e < M.cfOff[i + 1]; ++e) {
                const int f = M.cfFace[e], oth = M.cfOther[e];
                if (oth >= 0) row[oth] = LD(I.upper + f);
                else row[-(oth + 1)] = LD(I.lower + f);
            }
        } else {
            for (int q = L.rowPtr[i]; q < L.rowPtr[i + 1]; ++q) row[L.colIdx[q]] = LD(val + q);
        }
        row[n + i] = 1.0;
    }
    tm.sync();
    for (int k = 0; k < n; ++k) {
        const double piv = LD(A + (size_t)k * w2 + k);
        const bool skip = !(fabs(piv) > 1e-300);
        const double rp = skip ? 0.0 : 1.0 / piv;
        for (int idx = tm.rank(); idx < n * w2; idx += tm.size()) {
            const int i = idx / w2, j = idx - i * w2;
            const double akj = LD(A + (size_t)k * w2 + j) * rp;
            double v = LD(A + idx);
            if (!skip) {
                if (i == k) v = akj;
                else v = fma(-LD(A + (size_t)i * w2 + k), akj, v);
            }
            B[idx] = v;
        }
        tm.sync();
        double *tmp = A; A = B; B = tmp;
    }
    for (int idx = tm.rank(); idx < n * n; idx += tm.size()) {
        const int i = idx / n, j = idx - i * n;
        I.ainv[idx] = LD(A + (size_t)i * w2 + n + j);
    }
    tm.sync();
}

// one colour-ordered Gauss-Seidel sweep (forward or reverse colour order)
template <class T>
__device__ __noinline__ void amg_gs_sweep(T &tm, const DevMesh &M, DevInst &I, int l, bool reverse) {
    const AmgLevelDev &L = M.lev[l];
    double *x = lev_x(I, M, l);
    const double *b = lev_b(I, M, l);
    const double *val = lev_vals(I, M, l);
    const double *rd = lev_rd(I, M, l);
    for (int cc = 0; cc < L.nColors; ++cc) {
        const int col = reverse ? L.nColors - 1 - cc : cc;
        for (int q = L.colorOff[col] + tm.rank(); q < L.colorOff[col + 1]; q += tm.size()) {
            const int i = L.colorRows[q];
            const double ri = LD(rd + i);
            if (ri == 0.0) continue;
            double s = LD(b + i);
            if (l == 0) {
                for (int e = M.cfOff[i]; e < M.cfOff[i + 1]; ++e) {
                    const int f = M.cfFace[e], oth = M.cfOther[e];
                    if (oth >= 0) s = fma(-LD(I.upper + f), LD(x + oth), s);
                    else s = fma(-LD(I.lower + f), LD(x + (-(oth + 1))), s);
                }
            } else {
                for (int q2 = L.rowPtr[i]; q2 < L.rowPtr[i + 1]; ++q2) {
                    const int j = L.colIdx[q2];
                    if (j != i) s = fma(-LD(val + q2), LD(x + j), s);
                }
            }
            x[i] = s * ri;
        }
        tm.sync();
    }
}

// residual of level l and restriction into level l+1 (x_{l+1} = 0)
template <class T>
__device__ __noinline__ void amg_restrict(T &tm, const DevMesh &M, DevInst &I, int l) {
    const AmgLevelDev &L = M.lev[l];
    const double *x = lev_x(I, M, l), *b = lev_b(I, M, l), *val = lev_vals(I, M, l);
    double *r = lev_r(I, M, l);
    for (int i = tm.rank(); i < L.n; i += tm.size()) {
        double s;
        if (l == 0) {
            s = ldu_row<T>(M, I, x, i);
        } else {
            s = 0.0;
            for (int q = L.rowPtr[i]; q < L.rowPtr[i + 1]; ++q) s = fma(LD(val + q), LD(x + L.colIdx[q]), s);
        }
        r[i] = LD(b + i) - s;
    }
    tm.sync();
    const AmgLevelDev &C = M.lev[l + 1];
    double *bc = lev_b(I, M, l + 1), *xc = lev_x(I, M, l + 1);
    for (int J = tm.rank(); J < C.n; J += tm.size()) {
        double s = 0.0;
        for (int q = L.aggOff[J]; q < L.aggOff[J + 1]; ++q) s += LD(r + L.aggMem[q]);
        bc[J] = s;
        xc[J] = 0.0;
    }
    tm.sync();
}

template <class T>
__device__ void amg_prolong(T &tm, const DevMesh &M, DevInst &I, int l) {
    const AmgLevelDev &L = M.lev[l];
    double *x = lev_x(I, M, l);
    const double *xc = lev_x(I, M, l + 1);
    for (int i = tm.rank(); i < L.n; i += tm.size()) x[i] = LD(x + i) + LD(xc + L.map[i]);
    tm.sync();
}

template <class T>
__device__ void amg_coarse_solve(T &tm, const DevMesh &M, DevInst &I) {
    const int l = M.nLevels - 1;
    const int n = M.lev[l].n;
    if (M.coarseDirect) {
        const double *b = lev_b(I, M, l);
        double *x = lev_x(I, M, l);
        for (int i = tm.rank(); i < n; i += tm.size()) {
            double s = 0.0;
            for (int j = 0; j < n; ++j) s = fma(LD(I.ainv + (size_t)i * n + j), LD(b + j), s);
            x[i] = s;
        }
        tm.sync();
    } else {
        for (int s = 0; s < kCoarseSweeps; ++s) amg_gs_sweep(tm, M, I, l, (s & 1) != 0);
    }
}

// V-cycle on levels [l0, nLevels): 2 pre-sweeps (colours ascending), 2 post
// sweeps (colours descending) so the preconditioner is symmetric.
template <class T>
__device__ void amg_vcycle_from(T &tm, const DevMesh &M, DevInst &I, int l0) {
    const int nl = M.nLevels;
    for (int l = l0; l < nl - 1; ++l) {
        amg_gs_sweep(tm, M, I, l, false);
        amg_gs_sweep(tm, M, I, l, false);
        amg_restrict(tm, M, I, l);
    }
    amg_coarse_solve(tm, M, I);
    for (int l = nl - 2; l >= l0; --l) {
        amg_prolong(tm, M, I, l);
        amg_gs_sweep(tm, M, I, l, true);
        amg_gs_sweep(tm, M, I, l, true);
    }
}

// Levels below this size run on CTA 0 alone in grid mode.
constexpr int kSmallLevel = 16384;

template <class T> struct AmgDriver;
template <> struct AmgDriver<BlockTeam> {
    __device__ static void setup(BlockTeam &tm, const DevMesh &M, DevInst &I) {
        amg_level_rd(tm, M, I, 0);
        for (int l = 1; l < M.nLevels; ++l) {
            amg_galerkin(tm, M, I, l);
            tm.sync();
            amg_level_rd(tm, M, I, l);
        }
        tm.sync();
        if (M.coarseDirect) amg_coarse_inverse(tm, M, I);
    }
    __device__ static void vcycle(BlockTeam &tm, const DevMesh &M, DevInst &I) {
        amg_vcycle_from(tm, M, I, 0);
    }
};
template <> struct AmgDriver<GridTeam> {
    __device__ static int split(const DevMesh &M) {
        int l = 0;
        while (l < M.nLevels - 1 && M.lev[l].n >= kSmallLevel) ++l;
        return l;
    }
    __device__ static void setup(GridTeam &tm, const DevMesh &M, DevInst &I) {
        const int ls = split(M);
        amg_level_rd(tm, M, I, 0);
        for (int l = 1; l <= ls && l < M.nLevels; ++l) {
            amg_galerkin(tm, M, I, l);
            tm.sync();
            amg_level_rd(tm, M, I, l);
        }
        tm.sync();
        if (blockIdx.x == 0) {
            BlockTeamCG bt{{tm.red, tm.buf}};
            for (int l = ls + 1; l < M.nLevels; ++l) {
                amg_galerkin(bt, M, I, l);
                bt.sync();
                amg_level_rd(bt, M, I, l);
            }
            bt.sync();
            if (M.coarseDirect) amg_coarse_inverse(bt, M, I);
        }
        tm.sync();
    }
    __device__ static void vcycle(GridTeam &tm, const DevMesh &M, DevInst &I) {
        const int ls = split(M);
        for (int l = 0; l < ls; ++l) {
            amg_gs_sweep(tm, M, I, l, false);
            amg_gs_sweep(tm, M, I, l, false);
            amg_restrict(tm, M, I, l);
        }
        if (blockIdx.x == 0) {
            BlockTeamCG bt{{tm.red, tm.buf}};
            amg_vcycle_from(bt, M, I, ls);
        }
        tm.sync();
        for (int l = ls - 1; l >= 0; --l) {
            amg_prolong(tm, M, I, l);
            amg_gs_sweep(tm, M, I, l, true);
            amg_gs_sweep(tm, M, I, l, true);
        }
    }
};

// AMG-preconditioned CG (AMGSolver::solve, LinearSolver.hpp:602-653) on
// (I.diag, I.upper, I.lower, I.src), x in place (the pressure correction
// starts from zero).  Vectors: r = I.r, z = I.s (V-cycle level-0 x),
// p = I.pv, Ap = I.v, V-cycle scratch I.t.
template <class T>
__device__ __noinline__ SolveResult team_amg_pcg(T &tm, const DevMesh &M, DevInst &I, double *x, int maxIter, double tol) {
    SolveResult res = {0, 0.0, 0.0, 0};
    const int nC = M.nC;
    AmgDriver<T>::setup(tm, M, I);
    double a0[1] = {0.0};
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        double rc = LD(I.src + c) - ldu_row<T>(M, I, x, c);
        I.r[c] = rc;
        I.s[c] = 0.0;
        a0[0] = fma(rc, rc, a0[0]);
    }
    tm.template sum<1>(a0);
    const double r0 = sqrt(a0[0]);
    res.initialRes = r0;
    if (r0 < 1e-30) { res.converged = 1; return res; }
    AmgDriver<T>::vcycle(tm, M, I);
    double a1[1] = {0.0};
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        double z = LD(I.s + c);
        I.pv[c] = z;
        a1[0] = fma(LD(I.r + c), z, a1[0]);
    }
    tm.template sum<1>(a1);
    double rz = a1[0];
    for (int it = 0; it < maxIter; ++it) {
        if (!tm.ok()) break;
        double a2[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            double ap = ldu_row<T>(M, I, I.pv, c);
            I.v[c] = ap;
            a2[0] = fma(LD(I.pv + c), ap, a2[0]);
        }
        tm.template sum<1>(a2);
        const double pAp = a2[0];
        if (fabs(pAp) < 1e-30) break;
        const double alpha = rz / pAp;
        double a3[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            x[c] = fma(alpha, LD(I.pv + c), LD(x + c));
            double rc = fma(-alpha, LD(I.v + c), LD(I.r + c));
            I.r[c] = rc;
            I.s[c] = 0.0;
            a3[0] = fma(rc, rc, a3[0]);
        }
        tm.template sum<1>(a3);
        const double rn = sqrt(a3[0]);
        res.iterations = it + 1;
        res.finalRes = rn / r0;
        if (res.finalRes < tol) { res.converged = 1; return res; }
        AmgDriver<T>::vcycle(tm, M, I);
        double a4[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) a4[0] = fma(LD(I.r + c), LD(I.s + c), a4[0]);
        tm.template sum<1>(a4);
        const double rzNew = a4[0];
        const double beta = rzNew / (rz + 1e-30);
        for (int c = tm.rank(); c < nC; c += tm.size()) I.pv[c] = fma(beta, LD(I.pv + c), LD(I.s + c));
        tm.sync();
        rz = rzNew;
    }
    return res;
}

// Jacobi-preconditioned CG (PCGSolver::solve, LinearSolver.hpp:147-186) on
// (I.diag, I.upper, I.lower, I.src); x in place.  r = I.r, z = I.s, p = I.pv, Ap = I.v.
template <class T>
__device__ __noinline__ SolveResult team_pcg(T &tm, const DevMesh &M, DevInst &I, double *x, int maxIter, double tol) {
    SolveResult res = {0, 0.0, 0.0, 0};
    const int nC = M.nC;
    double a0[2] = {0.0, 0.0};
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        double rc = LD(I.src + c) - ldu_row<T>(M, I, x, c);
        double rdc = jac_rd(LD(I.diag + c));
        double z = rc * rdc;
        I.rd[c] = rdc;
        I.r[c] = rc; I.s[c] = z; I.pv[c] = z;
        a0[0] = fma(rc, rc, a0[0]);
        a0[1] = fma(rc, z, a0[1]);
    }
    tm.template sum<2>(a0);
    const double r0 = sqrt(a0[0]);
    res.initialRes = r0;
    if (r0 < 1e-30) { res.converged = 1; return res; }
    double rz = a0[1];
    for (int it = 0; it < maxIter; ++it) {
        if (!tm.ok()) break;
        double a2[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            double ap = ldu_row<T>(M, I, I.pv, c);
            I.v[c] = ap;
            a2[0] = fma(LD(I.pv + c), ap, a2[0]);
        }
        tm.template sum<1>(a2);
        const double pAp = a2[0];
        if (fabs(pAp) < 1e-30) break;
        const double alpha = rz / pAp;
        double a3[2] = {0.0, 0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            x[c] = fma(alpha, LD(I.pv + c), LD(x + c));
            double rc = fma(-alpha, LD(I.v + c), LD(I.r + c));
            double z = rc * LD(I.rd + c);
            I.r[c] = rc;
            I.s[c] = z;
            a3[0] = fma(rc, rc, a3[0]);
            a3[1] = fma(rc, z, a3[1]);
        }
        tm.template sum<2>(a3);
        const double rn = sqrt(a3[0]);
        res.iterations = it + 1;
        res.finalRes = rn / r0;
        if (res.finalRes < tol) { res.converged = 1; return res; }
        const double beta = a3[1] / (rz + 1e-30);
        for (int c = tm.rank(); c < nC; c += tm.size()) I.pv[c] = fma(beta, LD(I.pv + c), LD(I.s + c));
        tm.sync();
        rz = a3[1];
    }
    return res;
}

// makeSolver semantics for the device: AMG and PCG run the CG family; every
// other name runs BiCGSTAB.  Gauss-Seidel is not offered on the device (the
// host rejects it at case creation).
template <class T>
__device__ SolveResult team_solve(T &tm, const DevMesh &M, DevInst &I, int kind, double *x, int maxIter, double tol) {
    if (kind == 3) return team_amg_pcg(tm, M, I, x, maxIter, tol);
    if (kind == 0) return team_pcg(tm, M, I, x, maxIter, tol);
    return team_bicgstab(tm, M, I, x, maxIter, tol);
}

// ---------------------------------------------------------------------------
// initUniform (SIMPLESolver.cpp:23-51)
// ---------------------------------------------------------------------------
template <class T>
__device__ void phase_init_uniform(T &tm, const DevMesh &M, DevInst &I) {
    const Coef cf = load_coef(I);
    const double nu = I.nu;
    const double U0 = I.init[0], U1 = I.init[1], U2 = I.init[2], p0 = I.init[3], k0 = I.init[4], w0 = I.init[5];
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        I.ux[c] = U0; I.uy[c] = U1; I.uz[c] = U2; I.p[c] = p0; I.k[c] = k0;
        I.f1[c] = 1.0; I.f2[c] = 1.0; I.pk[c] = 0.0; I.cdkw[c] = 0.0;
        double y = smax(M.wd[c], 1e-20);
        double omWall = 60.0 * nu / (cf.b1 * y * y);
        double om = smax(omWall, w0);
        I.om[c] = om;
        I.nut[c] = cf.a1 * k0 / smax(cf.a1 * om, 1e-20);
    }
    for (int b = tm.rank(); b < M.nB; b += tm.size()) {
        I.ubx[b] = U0; I.uby[b] = U1; I.ubz[b] = U2; I.pb[b] = p0; I.kb[b] = k0; I.omb[b] = w0;
    }
    tm.sync();
    phase_bc_u(tm, M, I);
    phase_bc_p(tm, M, I);
    phase_bc_k(tm, M, I, false);
    phase_bc_w(tm, M, I, 0.075, false);  // applyAllBCs uses applyOmegaBC's default beta1
    tm.sync();
}

// ---------------------------------------------------------------------------
// the SIMPLE outer loop (SIMPLESolver::solve, SIMPLESolver.cpp:696-1043)
// ---------------------------------------------------------------------------
// per-phase device timers, kept by the team leader
struct PhaseClock {
    uint64_t acc[8];
    uint64_t t0;
    bool on;
    __device__ void start(bool leader) {
        on = leader;
        for (int q = 0; q < 8; ++q) acc[q] = 0;
        t0 = on ? globaltimer_ns() : 0;
    }
    __device__ __forceinline__ void lap(int phase) {
        if (on) {
            uint64_t t = globaltimer_ns();
            acc[phase] += t - t0;
            t0 = t;
        }
    }
};

template <class T>
__device__ void simple_solve(T &tm, const DevMesh &M, DevInst &I) {
    const DevSettings &S = I.S;
    const Coef cf = load_coef(I);
    const int nC = M.nC, nB = M.nB;
    const double nu = I.nu;
    if (I.initMode == 0) phase_init_uniform(tm, M, I);
    int turbEst = I.initMode == 0 ? 0 : I.turbEstIn;
    double lastKChange = 1.0, lastOmChange = 1.0;
    double normUx0 = 1, normUy0 = 1, normP0 = 1;
    int converged = 0, diverged = 0, finalIter = S.maxIter, ran = 0;
    int64_t inner = 0;
    double last[6] = {0, 0, 0, 0, 0, 0};
    const bool turbScheduled = S.turbStart < S.maxIter;
    PhaseClock clk;
    clk.start(tm.leader());

    for (int iter = 0; iter < S.maxIter; ++iter) {
        if (!tm.ok()) break;
        ran = iter + 1;
        const bool turbActive = iter >= S.turbStart;
        const bool turbUpdate = turbActive && ((iter - S.turbStart) % S.turbInterval == 0);
        // 1. turbulence closure fields at the start-of-iteration U
        phase_velgrad(tm, M, I, 7);
        phase_grad1(tm, M, I.p, I.pb, I.gpx, I.gpy, I.gpz);
        tm.sync();
        if (turbUpdate) {
            if (!turbEst && iter >= S.turbStart + S.nutFloorIters) turbEst = 1;
            const double nutMin = turbEst ? 0.0 : 0.1 * nu;
            phase_sst(tm, M, I, nutMin);
            tm.sync();
        }
        clk.lap(0);
        // 2. momentum, component by component with the latest U
        SolveResult resU[3];
        resU[2].initialRes = 0.0; resU[2].iterations = 0;
        for (int comp = 0; comp < 3; ++comp) {
            if (comp == 2 && !I.solveZ) break;
            if (comp > 0) {
                phase_velgrad(tm, M, I, 1 << (comp - 1));
                tm.sync();
            }
            phase_mom_faces(tm, M, I, comp);
            tm.sync();
            phase_mom_cells(tm, M, I, comp);
            tm.sync();
            clk.lap(1);
            double *x = comp == 0 ? I.ux : (comp == 1 ? I.uy : I.uz);
            resU[comp] = team_solve(tm, M, I, S.momSolver, x, S.innerIter, S.innerTol);
            inner += resU[comp].iterations;
            tm.sync();
            clk.lap(2);
        }
        phase_bc_u(tm, M, I);
        tm.sync();
        // 3. pressure correction
        phase_p_faces(tm, M, I);
        tm.sync();
        phase_p_cells(tm, M, I);
        tm.sync();
        clk.lap(3);
        SolveResult resP = team_solve(tm, M, I, S.pSolver, I.pp, S.innerIter, S.innerTol);
        inner += resP.iterations;
        tm.sync();
        clk.lap(5);
        for (int b = tm.rank(); b < nB; b += tm.size()) I.ppb[b] = M.bcPp[b] == 0 ? LD(I.pp + M.bown[b]) : 0.0;
        tm.sync();
        // 4. corrections (correctVelocity / correctPressure, SIMPLESolver.cpp:456-475)
        {
            const double *P[1] = {I.pp};
            const double *PB[1] = {I.ppb};
            const double alphaP = S.alphaP;
            for (int c = tm.rank(); c < nC; c += tm.size()) {
                double gx[1], gy[1], gz[1];
                gg_cell<T, 1>(M, c, P, PB, gx, gy, gz);
                const double aP = LD(I.aPx + c);
                double rAP = (fabs(aP) > 1e-30) ? 1.0 / aP : 0.0;
                double vol = M.vol[c];
                I.ux[c] = LD(I.ux + c) - rAP * gx[0] * vol;
                I.uy[c] = LD(I.uy + c) - rAP * gy[0] * vol;
                I.uz[c] = LD(I.uz + c) - rAP * gz[0] * vol;
                I.p[c] = LD(I.p + c) + alphaP * LD(I.pp + c);
            }
            tm.sync();
            phase_bc_u(tm, M, I);
            phase_bc_p(tm, M, I);
            tm.sync();
        }
        clk.lap(6);
        // 5. k and omega
        SolveResult resK = {0, 0, 0, 0}, resW = {0, 0, 0, 0};
        if (turbUpdate) {
            for (int c = tm.rank(); c < nC; c += tm.size()) { I.kold[c] = LD(I.k + c); I.omold[c] = LD(I.om + c); }
            phase_turb_faces(tm, M, I, 0);
            tm.sync();
            phase_turb_cells(tm, M, I, 0);
            tm.sync();
            resK = team_solve(tm, M, I, S.turbSolver, I.k, S.innerIter, S.innerTol);
            inner += resK.iterations;
            tm.sync();
            for (int c = tm.rank(); c < nC; c += tm.size()) I.k[c] = smax(S.kMin, smin(S.kMax, LD(I.k + c)));
            tm.sync();
            phase_bc_k(tm, M, I, true);
            tm.sync();
            phase_turb_faces(tm, M, I, 1);
            tm.sync();
            phase_turb_cells(tm, M, I, 1);
            tm.sync();
            resW = team_solve(tm, M, I, S.turbSolver, I.om, S.innerIter, S.innerTol);
            inner += resW.iterations;
            tm.sync();
            for (int c = tm.rank(); c < nC; c += tm.size()) I.om[c] = smax(S.omegaMin, smin(1e15, LD(I.om + c)));
            tm.sync();
            phase_bc_w(tm, M, I, cf.b1, true);
            tm.sync();
            // wall re-pin (SIMPLESolver.cpp:884-908) and change norms (:910-922)
            double mx[4] = {1e-30, 1e-30, 0.0, 0.0};
            const double sbs = sqrt(cf.bstar);
            for (int c = tm.rank(); c < nC; c += tm.size()) {
                const int b = M.pinFace[c];
                double omc = LD(I.om + c);
                if (b >= 0) {
                    double y1 = M.bdeltaW[b];
                    double omRes = 60.0 * nu / (cf.b1 * y1 * y1);
                    if (S.useWallFn) {
                        double k_p = smax(LD(I.k + c), 1e-30);
                        double uTau = sqrt(sbs * k_p);
                        double omLog = uTau / (sbs * S.vonKarman * y1);
                        omc = sqrt(omRes * omRes + omLog * omLog);
                    } else {
                        omc = omRes;
                    }
                    I.om[c] = omc;
                }
                const double kc = LD(I.k + c);
                mx[0] = smax(mx[0], fabs(kc));
                mx[1] = smax(mx[1], fabs(omc));
                mx[2] = smax(mx[2], fabs(kc - LD(I.kold + c)));
                mx[3] = smax(mx[3], fabs(omc - LD(I.omold + c)));
            }
            tm.template maxr<4>(mx);
            lastKChange = mx[2] / mx[0];
            lastOmChange = mx[3] / mx[1];
        }
        clk.lap(7);
        // 6. residual bookkeeping and the convergence / divergence tests
        const double eUx = resU[0].initialRes, eUy = resU[1].initialRes, eUz = resU[2].initialRes;
        const double eP = resP.initialRes;
        const double eK = turbActive ? lastKChange : 0.0, eW = turbActive ? lastOmChange : 0.0;
        last[0] = eUx; last[1] = eUy; last[2] = eUz; last[3] = eP; last[4] = eK; last[5] = eW;
        if (tm.leader() && I.hist && iter < I.histCap)
            for (int q = 0; q < 6; ++q) I.hist[6 * (size_t)iter + q] = last[q];
        if (iter == 0) {
            normUx0 = smax(eUx, 1e-30);
            normUy0 = smax(eUy, 1e-30);
            normP0 = smax(eP, 1e-30);
        } else if (iter < 50) {
            normP0 = smax(normP0, eP);
        }
        const double normMom0 = smax(normUx0, normUy0);
        const double nUx = normMom0 < 1e-20 ? 0.0 : eUx / normMom0;
        const double nUy = normMom0 < 1e-20 ? 0.0 : eUy / normMom0;
        const double nP = normP0 < 1e-20 ? 0.0 : eP / normP0;
        double maxRes = smax(smax(nUx, nUy), nP);
        if (turbActive) maxRes = smax(smax(maxRes, lastKChange), lastOmChange);
        if (!isfinite(eUx) || !isfinite(eUy) || !isfinite(eUz) || !isfinite(eP) || !isfinite(eK) ||
            !isfinite(eW) || !isfinite(lastKChange) || !isfinite(lastOmChange))
            maxRes = INFINITY;
        if (maxRes < S.convTol && iter > 0 && (!turbScheduled || (turbActive && turbEst))) {
            converged = 1;
            finalIter = iter;
            break;
        }
        if (isnan(maxRes) || isinf(maxRes) || maxRes > S.divLimit) {
            diverged = 1;
            finalIter = iter;
            break;
        }
    }
    tm.sync();
    if (tm.leader()) {
        const bool aborted = !tm.ok();
        I.out[0] = aborted ? 4 : (diverged ? 2 : (converged ? 0 : 1));
        I.out[1] = converged;
        I.out[2] = diverged;
        I.out[3] = finalIter;
        I.out[4] = ran;
        I.out[5] = turbEst;
        I.out[6] = aborted ? 1 : 0;
        I.outInner[0] = inner;
        for (int q = 0; q < 6; ++q) I.outLast[q] = last[q];
        for (int q = 0; q < 8; ++q) I.outTime[q] = clk.acc[q];
    }
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// One CTA per instance.  NT threads per CTA; small instances use NT = 256 so
// that two instances share an SM and hide each other's latency.
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_simple_block(DevInst *insts, int n) {
    __shared__ double red[2 * 32 * kRedSlots];
    __shared__ DevMesh sM;
    __shared__ DevInst sI;
    if (blockIdx.x >= n) return;
    if (threadIdx.x == 0) {
        sI = insts[blockIdx.x];
        sM = *sI.M;
    }
    __syncthreads();
    BlockTeam tm{red, 0};
    simple_solve(tm, sM, sI);
}
template __global__ void k_simple_block<256>(DevInst *, int);
template __global__ void k_simple_block<512>(DevInst *, int);

__global__ void __launch_bounds__(kThreads, 1) k_simple_grid(DevInst *inst) {
    __shared__ double red[2 * 32 * kRedSlots];
    __shared__ DevMesh sM;
    __shared__ DevInst sI;
    __shared__ int shAbort;
    if (threadIdx.x == 0) {
        sI = *inst;
        sM = *sI.M;
        shAbort = 0;
    }
    __syncthreads();
    GridTeam tm{red, 0, sI.gpart, sI.barrier, sI.err, &shAbort};
    simple_solve(tm, sM, sI);
}

// Test hook: one phase on one CTA with the state already on the device.
__global__ void __launch_bounds__(kThreads, 1) k_debug(DevInst *inst) {
    __shared__ double red[2 * 32 * kRedSlots];
    __shared__ DevMesh sM;
    __shared__ DevInst sI;
    if (threadIdx.x == 0) {
        sI = *inst;
        sM = *sI.M;
    }
    __syncthreads();
    BlockTeam tm{red, 0};
    const DevMesh &M = sM;
    DevInst &I = sI;
    const int ph = I.dbgPhase, arg = I.dbgArg;
    SolveResult res = {0, 0.0, 0.0, 0};
    switch (ph) {
        case 1:  // greenGaussGrad of p -> gp
            phase_grad1(tm, M, I.p, I.pb, I.gpx, I.gpy, I.gpz);
            break;
        case 2:  // computeFields (no floor) + |S|
            phase_velgrad(tm, M, I, 7);
            tm.sync();
            phase_sst(tm, M, I, -1.0);
            break;
        case 3:  // assembleMomentum(comp = arg)
            phase_velgrad(tm, M, I, 7);
            phase_grad1(tm, M, I.p, I.pb, I.gpx, I.gpy, I.gpz);
            tm.sync();
            phase_mom_faces(tm, M, I, arg);
            tm.sync();
            phase_mom_cells(tm, M, I, arg);
            break;
        case 4:  // assemblePressureCorrection with I.aPx
            phase_grad1(tm, M, I.p, I.pb, I.gpx, I.gpy, I.gpz);
            tm.sync();
            phase_p_faces(tm, M, I);
            tm.sync();
            phase_p_cells(tm, M, I);
            break;
        case 5:
        case 6:  // assembleKEquation / assembleOmegaEquation
            phase_turb_faces(tm, M, I, ph - 5);
            tm.sync();
            phase_turb_cells(tm, M, I, ph - 5);
            break;
        case 7:  // v = A r
            for (int c = tm.rank(); c < M.nC; c += tm.size()) I.v[c] = ldu_row<BlockTeam>(M, I, I.r, c);
            break;
        case 8:  // BiCGSTAB on (diag,upper,lower,src), x = pp
            res = team_bicgstab(tm, M, I, I.pp, I.S.innerIter, I.S.innerTol);
            break;
        case 9:  // AMG-PCG on the same system, x = pp (starts at zero)
            for (int c = tm.rank(); c < M.nC; c += tm.size()) I.pp[c] = 0.0;
            tm.sync();
            res = team_amg_pcg(tm, M, I, I.pp, I.S.innerIter, I.S.innerTol);
            break;
        case 11:  // PCG (Jacobi)
            res = team_pcg(tm, M, I, I.pp, I.S.innerIter, I.S.innerTol);
            break;
    }
    tm.sync();
    if (threadIdx.x == 0) {
        I.outLast[0] = res.iterations;
        I.outLast[1] = res.finalRes;
        I.outLast[2] = res.initialRes;
        I.outLast[3] = res.converged;
    }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
int engine_block_threads() { return kThreads; }

int engine_launch_block(DevInst *dInsts, int n, int threads, void *stream) {
    if (n <= 0) return 0;
    if (threads == 256)
        k_simple_block<256><<<n, 256, 0, (cudaStream_t)stream>>>(dInsts, n);
    else
        k_simple_block<512><<<n, 512, 0, (cudaStream_t)stream>>>(dInsts, n);
    return (int)cudaGetLastError();
}

int engine_grid_blocks(int *blocks_out) {
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int)e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_simple_grid, kThreads, 0);
    if (e != cudaSuccess) return (int)e;
    if (per < 1) per = 1;
    *blocks_out = sms * per;
    return 0;
}

int engine_launch_grid(DevInst *dInst, int blocks, void *stream) {
    void *args[] = {&dInst};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_simple_grid, dim3(blocks), dim3(kThreads), args, 0,
                                                (cudaStream_t)stream);
    return (int)e;
}

int engine_launch_debug(DevInst *dInst, void *stream) {
    k_debug<<<1, kThreads, 0, (cudaStream_t)stream>>>(dInst);
    return (int)cudaGetLastError();
}

}  // namespace btm
