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
#include <type_traits>
#include "btm_team.cuh"
#include "btm_bc.cuh"
#include "btm_phases64.cuh"
#include "btm_observe.cuh"
#include "btm_ramg.cuh"

#include <cuda_runtime.h>
#include <stdint.h>

namespace btm {

constexpr int kThreads = 512;

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

// grid-size dense coarsest inverse (up to kCoarseDirectGrid rows): one warp
// per row, lane-strided partial sums folded by a butterfly
template <class T>
__device__ __noinline__ void amg_coarse_dense_warp(T &tm, const DevMesh &M, DevInst &I) {
    const int l = M.nLevels - 1;
    const int n = M.lev[l].n;
    const double *b = lev_b(I, M, l);
    double *x = lev_x(I, M, l);
    const int lane = tm.rank() & 31;
    for (int i = tm.rank() >> 5; i < n; i += tm.size() >> 5) {
        const double *row = I.ainv + (size_t)i * n;
        double s = 0.0;
        for (int j = lane; j < n; j += 32) s = fma(LD(row + j), LD(b + j), s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) x[i] = s;
    }
    tm.sync();
}

template <class T>
__device__ void amg_coarse_solve(T &tm, const DevMesh &M, DevInst &I) {
    const int l = M.nLevels - 1;
    const int n = M.lev[l].n;
    if (M.coarseDirect && n > kCoarseDirect) {
        amg_coarse_dense_warp(tm, M, I);
    } else if (M.coarseDirect) {
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

// one damped-Jacobi sweep on a coarse level (l >= 1): reads x, writes `out`
constexpr double kJacobiWeight64 = 0.7;
template <class T>
__device__ __noinline__ void amg_jacobi(T &tm, const DevMesh &M, DevInst &I, int l, const double *x, double *out) {
    const AmgLevelDev &L = M.lev[l];
    const double *b = lev_b(I, M, l), *val = lev_vals(I, M, l), *rd = lev_rd(I, M, l);
    for (int i = tm.rank(); i < L.n; i += tm.size()) {
        double s = LD(b + i);
        for (int q = L.rowPtr[i]; q < L.rowPtr[i + 1]; ++q) s = fma(-LD(val + q), LD(x + L.colIdx[q]), s);
        out[i] = fma(kJacobiWeight64 * LD(rd + i), s, LD(x + i));
    }
    tm.sync();
}

// Two smoothing sweeps of level l: multicolour Gauss-Seidel (colours
// ascending before the coarse correction, descending after).  On the
// cooperative grid the coarse levels take a pair of damped-Jacobi sweeps
// (x -> r -> x) instead: one grid barrier per sweep rather than one per
// colour (6-11 colours on Galerkin levels), for ~15-20 % more PCG iterations.
template <class T> struct GridSmoothing { static constexpr bool jacobi = false; };
template <> struct GridSmoothing<GridTeam> { static constexpr bool jacobi = true; };

template <class T>
__device__ void amg_smooth2(T &tm, const DevMesh &M, DevInst &I, int l, bool post) {
    if (l == 0 || !GridSmoothing<T>::jacobi) {
        amg_gs_sweep(tm, M, I, l, post);
        amg_gs_sweep(tm, M, I, l, post);
    } else {
        double *x = lev_x(I, M, l), *tmp = lev_r(I, M, l);
        amg_jacobi(tm, M, I, l, x, tmp);
        amg_jacobi(tm, M, I, l, tmp, x);
    }
}

// V-cycle on levels [l0, nLevels): 2 pre-sweeps, 2 post sweeps, symmetric so
// the preconditioner suits CG.
template <class T>
__device__ void amg_vcycle_from(T &tm, const DevMesh &M, DevInst &I, int l0) {
    const int nl = M.nLevels;
    for (int l = l0; l < nl - 1; ++l) {
        amg_smooth2(tm, M, I, l, false);
        amg_restrict(tm, M, I, l);
    }
    amg_coarse_solve(tm, M, I);
    for (int l = nl - 2; l >= l0; --l) {
        amg_prolong(tm, M, I, l);
        amg_smooth2(tm, M, I, l, true);
    }
}

// Hierarchy refresh and V-cycle, the same on one CTA and on the cooperative
// grid (every level on the whole team; the grid's dense coarsest level has
// up to kCoarseDirectGrid rows and is inverted and applied by all CTAs).
template <class T> struct AmgDriver {
    __device__ static void setup(T &tm, const DevMesh &M, DevInst &I) {
        amg_level_rd(tm, M, I, 0);
        for (int l = 1; l < M.nLevels; ++l) {
            amg_galerkin(tm, M, I, l);
            tm.sync();
            amg_level_rd(tm, M, I, l);
        }
        tm.sync();
        if (M.coarseDirect) amg_coarse_inverse(tm, M, I);
    }
    __device__ static void vcycle(T &tm, const DevMesh &M, DevInst &I) {
        amg_vcycle_from(tm, M, I, 0);
    }
};

// AMGSolver::solve (LinearSolver.hpp:602-653) with the reference's own
// hierarchy rebuilt from this system (btm_ramg.cuh); one CTA.  r = I.r,
// z = I.s (the V-cycle's level-0 x), p = I.pv, Ap = I.v, level-0 residual I.t.
__device__ __noinline__ SolveResult team_ramg_pcg(BlockTeamRef &tm, const DevMesh &M, DevInst &I, double *x,
                                                  int maxIter, double tol) {
    SolveResult res = {0, 0.0, 0.0, 0};
    const int nC = M.nC;
    const uint64_t t0 = tm.leader() ? globaltimer_ns() : 0;
    const int nLev = ramg_setup(tm, M, I);
    if (tm.leader()) I.rg.setupNs += globaltimer_ns() - t0;
    double a0[1] = {0.0};
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        const double rc = I.src[c] - ldu_row<BlockTeamRef>(M, I, x, c);
        I.r[c] = rc;
        I.s[c] = 0.0;
        a0[0] = fma(rc, rc, a0[0]);
    }
    tm.template sum<1>(a0);
    const double r0 = sqrt(a0[0]);
    res.initialRes = r0;
    if (r0 < 1e-30) { res.converged = 1; return res; }
    ramg_precondition(tm, M, I, nLev);
    double a1[1] = {0.0};
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        const double z = I.s[c];
        I.pv[c] = z;
        a1[0] = fma(I.r[c], z, a1[0]);
    }
    tm.template sum<1>(a1);
    double rz = a1[0];
    for (int it = 0; it < maxIter; ++it) {
        double a2[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            const double ap = ldu_row<BlockTeamRef>(M, I, I.pv, c);
            I.v[c] = ap;
            a2[0] = fma(I.pv[c], ap, a2[0]);
        }
        tm.template sum<1>(a2);
        const double pAp = a2[0];
        if (fabs(pAp) < 1e-30) break;
        const double alpha = rz / pAp;
        double a3[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            x[c] = x[c] + alpha * I.pv[c];
            const double rc = I.r[c] - alpha * I.v[c];
            I.r[c] = rc;
            I.s[c] = 0.0;
            a3[0] = fma(rc, rc, a3[0]);
        }
        tm.template sum<1>(a3);
        const double rn = sqrt(a3[0]);
        res.iterations = it + 1;
        res.finalRes = rn / r0;
        if (res.finalRes < tol) { res.converged = 1; return res; }
        ramg_precondition(tm, M, I, nLev);
        double a4[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) a4[0] = fma(I.r[c], I.s[c], a4[0]);
        tm.template sum<1>(a4);
        const double rzNew = a4[0];
        const double beta = rzNew / (rz + 1e-30);
        for (int c = tm.rank(); c < nC; c += tm.size()) I.pv[c] = I.s[c] + beta * I.pv[c];
        tm.sync();
        rz = rzNew;
    }
    return res;
}

// The reference-order AMG runs in the kernel instantiated for BlockTeamRef
// only (one CTA per instance); the other teams keep the per-case hierarchy.
template <class T> struct RefAmg {
    __device__ static bool on(const DevInst &) { return false; }
    __device__ static SolveResult run(T &, const DevMesh &, DevInst &, double *, int, double) {
        return {0, 0.0, 0.0, 0};
    }
};
template <> struct RefAmg<BlockTeamRef> {
    __device__ static bool on(const DevInst &I) { return I.S.refAmg != 0; }
    __device__ static SolveResult run(BlockTeamRef &tm, const DevMesh &M, DevInst &I, double *x, int maxIter,
                                      double tol) {
        return team_ramg_pcg(tm, M, I, x, maxIter, tol);
    }
};

// AMG-preconditioned CG (AMGSolver::solve, LinearSolver.hpp:602-653) on
// (I.diag, I.upper, I.lower, I.src), x in place (the pressure correction
// starts from zero).  Vectors: r = I.r, z = I.s (V-cycle level-0 x),
// p = I.pv, Ap = I.v, V-cycle scratch I.t.
template <class T>
__device__ __noinline__ SolveResult team_amg_pcg(T &tm, const DevMesh &M, DevInst &I, double *x, int maxIter, double tol) {
    if (RefAmg<T>::on(I)) return RefAmg<T>::run(tm, M, I, x, maxIter, tol);
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
    // The reference's breakdown guards (|p.Ap| < 1e-30, rz + 1e-30) are
    // absolute.  On grid meshes (above the one-CTA size) they are applied as
    // if the system had been scaled to a unit-norm right-hand side, as the
    // mixed engine scales it: the p' coefficients of the 2M-cell duct are so
    // small that the absolute guard ended the CG after about 0.6 iterations
    // per outer iteration.  One-CTA meshes (every parity case) keep the
    // reference's absolute guards.
    const double guard = std::is_same<T, GridTeam>::value ? 1e-30 * r0 * r0 : 1e-30;
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
        if (fabs(pAp) < guard) break;
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
        const double beta = rzNew / (rz + guard);
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

// GaussSeidelSolver::solve (LinearSolver.hpp:258-299) on (I.diag, I.upper,
// I.lower, I.src), x in place: in-place sweeps in row order, each row summing
// its neighbours in face order with the latest values, then a residual check
// against |source|.  A sweep runs wavefront by wavefront over the level-0
// row-order dependencies (M.wf0Off / M.wf0Rows): a row reads the new values
// of its lower-index neighbours and the old values of the others, exactly as
// the sequential sweep, with the reference's operation order per row.  Only
// the residual norm (a parallel reduction) differs in the last bits.
template <class T>
__device__ __noinline__ SolveResult team_gauss_seidel(T &tm, const DevMesh &M, DevInst &I, double *x, int maxIter,
                                                      double tol) {
    SolveResult res = {0, 0.0, 0.0, 0};
    const int nC = M.nC;
    double a0[1] = {0.0};
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        const double bc = LD(I.src + c);
        a0[0] = fma(bc, bc, a0[0]);
    }
    tm.template sum<1>(a0);
    double b0 = sqrt(a0[0]);
    res.initialRes = b0;
    if (b0 < 1e-30) b0 = 1.0;
    for (int it = 0; it < maxIter; ++it) {
        if (!tm.ok()) break;
        for (int w = 0; w < M.nWf0; ++w) {
            for (int q = M.wf0Off[w] + tm.rank(); q < M.wf0Off[w + 1]; q += tm.size()) {
                const int i = M.wf0Rows[q];
                const double d = LD(I.diag + i);
                if (fabs(d) <= 1e-30) continue;
                double sacc = LD(I.src + i);
                for (int e = M.cfOff[i]; e < M.cfOff[i + 1]; ++e) {
                    const int f = M.cfFace[e], oth = M.cfOther[e];
                    if (oth >= 0) sacc -= LD(I.upper + f) * LD(x + oth);
                    else sacc -= LD(I.lower + f) * LD(x + (-(oth + 1)));
                }
                x[i] = sacc / d;
            }
            tm.sync();
        }
        double a1[1] = {0.0};
        for (int c = tm.rank(); c < nC; c += tm.size()) {
            const double rc = LD(I.src + c) - ldu_row<T>(M, I, x, c);
            a1[0] = fma(rc, rc, a1[0]);
        }
        tm.template sum<1>(a1);
        res.iterations = it + 1;
        res.finalRes = sqrt(a1[0]) / b0;
        if (res.finalRes < tol) { res.converged = 1; return res; }
    }
    return res;
}

// makeSolver semantics for the device (LinearSolver.hpp:659-665): AMG and
// PCG run the CG family, GaussSeidel the in-place sweep; every other name
// runs BiCGSTAB.
template <class T>
__device__ SolveResult team_solve(T &tm, const DevMesh &M, DevInst &I, int kind, double *x, int maxIter, double tol) {
    if (kind == 3) return team_amg_pcg(tm, M, I, x, maxIter, tol);
    if (kind == 0) return team_pcg(tm, M, I, x, maxIter, tol);
    if (kind == 2) return team_gauss_seidel(tm, M, I, x, maxIter, tol);
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
    int64_t inner = 0, innerMom = 0, innerP = 0, innerTurb = 0;
    double last[6] = {0, 0, 0, 0, 0, 0};
    const bool turbScheduled = S.turbStart < S.maxIter;
    PhaseClock clk;
    clk.start(tm.leader());
    const uint64_t tStart = tm.leader() ? globaltimer_ns() : 0;
    if (tm.leader()) I.rg.setupNs = 0;

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
            if (comp == 0 && I.inj) phase_inj(tm, M, I, I.g, I.nut, iter == 0);
            phase_mom_faces(tm, M, I, comp);
            tm.sync();
            phase_mom_cells(tm, M, I, comp);
            tm.sync();
            clk.lap(1);
            double *x = comp == 0 ? I.ux : (comp == 1 ? I.uy : I.uz);
            resU[comp] = team_solve(tm, M, I, S.momSolver, x, S.innerIter, S.innerTol);
            innerMom += resU[comp].iterations;
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
        innerP += resP.iterations;
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
            innerTurb += resK.iterations;
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
            innerTurb += resW.iterations;
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
        if (I.normFixed) {
            normUx0 = I.normIn[0];
            normUy0 = I.normIn[1];
            normP0 = I.normIn[2];
        } else if (iter == 0) {
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
        I.out[7] = -1;
        inner = innerMom + innerP + innerTurb;
        I.outInner[0] = inner;
        I.outInner[1] = innerMom;
        I.outInner[2] = innerP;
        I.outInner[3] = innerTurb;
        I.outInner[4] = 0;
        for (int q = 0; q < 6; ++q) I.outLast[q] = last[q];
        I.outLast[6] = normUx0;
        I.outLast[7] = normUy0;
        I.outLast[8] = normP0;
        if (I.S.refAmg && I.S.pSolver == 3 && clk.acc[5] >= I.rg.setupNs) {
            // hierarchy setups of the reference-order AMG count as AMG setup
            clk.acc[5] -= I.rg.setupNs;
            clk.acc[4] += I.rg.setupNs;
        }
        for (int q = 0; q < kPhaseSlots; ++q) I.outTime[q] = clk.acc[q];
        I.outTime[kPhaseSlots] = tStart;
        I.outTime[kPhaseSlots + 1] = globaltimer_ns();
        if (I.obsOut) observe_leader<T>(M, I);
        if (I.doneFlag) {
            __threadfence_system();
            *I.doneFlag = 1;
        }
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

// The same for launches that contain instances with the reference-order AMG;
// `xsCap` doubles of dynamic shared memory hold every level's x when they fit.
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_simple_block_ref(DevInst *insts, int n, int xsCap) {
    __shared__ double red[2 * 32 * kRedSlots];
    __shared__ DevMesh sM;
    __shared__ DevInst sI;
    extern __shared__ __align__(16) double xsm[];
    if (blockIdx.x >= n) return;
    if (threadIdx.x == 0) {
        sI = insts[blockIdx.x];
        sM = *sI.M;
        sI.rg.xs = (sI.S.refAmg && (int64_t)sM.nC + sI.rg.rowPool <= xsCap) ? xsm : nullptr;
    }
    __syncthreads();
    BlockTeamRef tm;
    tm.red = red;
    tm.buf = 0;
    simple_solve(tm, sM, sI);
}
template __global__ void k_simple_block_ref<256>(DevInst *, int, int);
template __global__ void k_simple_block_ref<512>(DevInst *, int, int);

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
    BlockTeamRef tm;
    tm.red = red;
    tm.buf = 0;
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
            for (int c = tm.rank(); c < M.nC; c += tm.size()) I.v[c] = ldu_row<BlockTeamRef>(M, I, I.r, c);
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
        case 13:  // Gauss-Seidel
            res = team_gauss_seidel(tm, M, I, I.pp, I.S.innerIter, I.S.innerTol);
            break;
        case 12:  // reference-order AMG hierarchy of (diag, upper, lower)
            if (I.S.refAmg) res.iterations = ramg_setup(tm, M, I);
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
// Mesh::computeWallDistance (core/src/Mesh.cpp:345-373): minimum over the wall
// face centres of |c - w|.  Each thread owns one cell; the wall centres stream
// through shared memory in tiles.  The squared distance is formed exactly as
// (dx*dx + dy*dy) + dz*dz without contraction and the square root is taken
// once of the minimum: sqrt is correctly rounded and monotone, so the result
// is bit-identical to the reference's minimum of square roots.
// ---------------------------------------------------------------------------
constexpr int kWallTile = 1024;
__global__ void __launch_bounds__(256) k_wall_distance(const double *cc, int nC, const double *wp, int nW,
                                                        double *out) {
    __shared__ double sx[kWallTile], sy[kWallTile], sz[kWallTile];
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double x = 0.0, y = 0.0, z = 0.0;
    if (c < nC) { x = cc[3 * (size_t)c]; y = cc[3 * (size_t)c + 1]; z = cc[3 * (size_t)c + 2]; }
    double best = INFINITY;
    for (int t0 = 0; t0 < nW; t0 += kWallTile) {
        const int n = min(kWallTile, nW - t0);
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            sx[j] = wp[3 * (size_t)(t0 + j)];
            sy[j] = wp[3 * (size_t)(t0 + j) + 1];
            sz[j] = wp[3 * (size_t)(t0 + j) + 2];
        }
        __syncthreads();
        for (int j = 0; j < n; ++j) {
            const double dx = __dsub_rn(x, sx[j]), dy = __dsub_rn(y, sy[j]), dz = __dsub_rn(z, sz[j]);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            best = d2 < best ? d2 : best;
        }
        __syncthreads();
    }
    if (c < nC) out[c] = sqrt(best);
}

int engine_wall_distance(const double *dCentres, int nC, const double *dWall, int nW, double *dOut, void *stream) {
    if (nC <= 0) return 0;
    k_wall_distance<<<(nC + 255) / 256, 256, 0, (cudaStream_t)stream>>>(dCentres, nC, dWall, nW, dOut);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
int engine_block_threads() { return kThreads; }

// Dynamic shared memory of the reference-order kernel for the level vectors
// (every level's x: nC + 2 nC + 64 doubles) when they fit within this much.
constexpr int kRamgXsBytes256 = 96 * 1024;    // two CTAs per SM
constexpr int kRamgXsBytes512 = 192 * 1024;   // one CTA per SM

int engine_launch_block(DevInst *dInsts, int n, int threads, void *stream, bool refAmg, int maxCells) {
    if (n <= 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    if (refAmg) {
        const int cap = threads == 256 ? kRamgXsBytes256 : kRamgXsBytes512;
        // only what the level vectors need: the rest of the SM's shared
        // memory / L1 stays L1, which holds level 0's matrix
        const int64_t need = 8 * (3 * (int64_t)maxCells + 64);
        const int bytes = need <= cap ? (int)need : 0;
        cudaError_t e;
        if (threads == 256) {
            e = cudaFuncSetAttribute(k_simple_block_ref<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
            if (e != cudaSuccess) return (int)e;
            k_simple_block_ref<256><<<n, 256, bytes, st>>>(dInsts, n, bytes / 8);
        } else {
            e = cudaFuncSetAttribute(k_simple_block_ref<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
            if (e != cudaSuccess) return (int)e;
            k_simple_block_ref<512><<<n, 512, bytes, st>>>(dInsts, n, bytes / 8);
        }
    } else {
        if (threads == 256) k_simple_block<256><<<n, 256, 0, st>>>(dInsts, n);
        else k_simple_block<512><<<n, 512, 0, st>>>(dInsts, n);
    }
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
