// btm_phases64.cuh - the FP64 closure, gradient and assembly phases and the
// FP64 LDU row product and BiCGSTAB.  The FP64 engine compiles them with
// -fmad=false so the assembly rounds exactly like the reference; the
// mixed-precision engine uses them for its FP64 polishing stage.
#pragma once
#include "btm_common.h"
#include "btm_team.cuh"

namespace btm {

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

// The same closure with FP64 reciprocals formed once per cell (the mixed
// engine's FP64 polishing stage: FP64-accurate, not reference-rounded; GB300
// spends tens of FP64 instructions on every division).
struct SstCell { double F1, F2, nuT, Pk, CDkw; };
__device__ __forceinline__ SstCell sst_cell_fast(const Coef &c, double kc, double wc, double y, double nu, double S,
                                                 double gradDot) {
    SstCell r;
    const double kp = smax(kc, 0.0);
    const double sqrtK = sqrt(kp);
    const double rw = 1.0 / smax(wc, 1e-20);
    const double ySafe = smax(y, 1e-20);
    const double ry = 1.0 / ySafe;
    const double ry2 = ry * ry;
    r.CDkw = 2.0 * c.sw2 * rw * gradDot;
    const double CDpos = smax(r.CDkw, 1e-20);
    const double t1 = sqrtK * rw * ry / c.bstar;
    const double t2 = 500.0 * nu * ry2 * rw;
    if (c.variant == 2) {
        r.F1 = 1.0;
    } else {
        const double t3 = 4.0 * c.sw2 * kp * ry2 / CDpos;
        const double arg1 = smin(smax(t1, t2), t3);
        const double a2 = arg1 * arg1;
        r.F1 = tanh(a2 * a2);
    }
    const double arg2 = smax(2.0 * t1, t2);
    r.F2 = tanh(arg2 * arg2);
    if (c.variant == 1) r.nuT = kp * rw;
    else r.nuT = c.a1 * kp / smax(smax(c.a1 * wc, S * r.F2), 1e-20);
    r.Pk = smin(r.nuT * S * S, 10.0 * c.bstar * kp * smax(wc, 1e-20));
    return r;
}

// ---------------------------------------------------------------------------
// Green-Gauss gradients (core/include/Field.hpp:122-152): per cell, internal
// faces in ascending face order, then boundary faces, then / V.
// ---------------------------------------------------------------------------
template <class T, int NF, bool Fast = false>
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
        if (Fast) {
            const double rv = 1.0 / V;
#pragma unroll
            for (int q = 0; q < NF; ++q) { ax[q] *= rv; ay[q] *= rv; az[q] *= rv; }
        } else {
#pragma unroll
            for (int q = 0; q < NF; ++q) { ax[q] = ax[q] / V; ay[q] = ay[q] / V; az[q] = az[q] / V; }
        }
    }
#pragma unroll
    for (int q = 0; q < NF; ++q) { gx[q] = ax[q]; gy[q] = ay[q]; gz[q] = az[q]; }
}

// gradient of one scalar into (gx, gy, gz)
template <class T, bool Fast = false>
__device__ __noinline__ void phase_grad1(T &tm, const DevMesh &M, const double *phi, const double *phib,
                            double *ox, double *oy, double *oz) {
    const double *P[1] = {phi};
    const double *PB[1] = {phib};
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        double gx[1], gy[1], gz[1];
        gg_cell<T, 1, Fast>(M, c, P, PB, gx, gy, gz);
        ox[c] = gx[0]; oy[c] = gy[0]; oz[c] = gz[0];
    }
}

// velocity gradients (Field.hpp:232-246): g[3*i+j] = dU_i/dx_j; `which` selects
// components (bit i) so a partially updated U only recomputes what changed
template <class T, bool Fast = false>
__device__ __noinline__ void phase_velgrad(T &tm, const DevMesh &M, DevInst &I, int which) {
    const double *U[3] = {I.ux, I.uy, I.uz};
    const double *UB[3] = {I.ubx, I.uby, I.ubz};
    for (int c = tm.rank(); c < M.nC; c += tm.size()) {
        if (which == 7) {
            double gx[3], gy[3], gz[3];
            gg_cell<T, 3, Fast>(M, c, U, UB, gx, gy, gz);
#pragma unroll
            for (int i = 0; i < 3; ++i) { I.g[3 * i][c] = gx[i]; I.g[3 * i + 1][c] = gy[i]; I.g[3 * i + 2][c] = gz[i]; }
        } else {
            for (int i = 0; i < 3; ++i) {
                if (!(which & (1 << i))) continue;
                const double *P[1] = {U[i]};
                const double *PB[1] = {UB[i]};
                double gx[1], gy[1], gz[1];
                gg_cell<T, 1, Fast>(M, c, P, PB, gx, gy, gz);
                I.g[3 * i][c] = gx[0]; I.g[3 * i + 1][c] = gy[0]; I.g[3 * i + 2][c] = gz[0];
            }
        }
    }
}

// SSTModel::computeFields + frozen |S| + startup floor (SIMPLESolver.cpp:736-768).
// Requires velocity gradients in I.g.  nutMin < 0 skips the floor.
template <class T, bool Fast = false>
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
        gg_cell<T, 2, Fast>(M, c, P, PB, gx, gy, gz);
        double kc = smax(LD(I.k + c), 0.0);
        double wc = smax(LD(I.om + c), 1e-20);
        double y = smax(M.wd[c], 1e-20);
        if (Fast) {
            const SstCell r = sst_cell_fast(cf, kc, wc, y, nu, Sc, gx[0] * gx[1] + gy[0] * gy[1] + gz[0] * gz[1]);
            I.smag[c] = Sc;
            I.cdkw[c] = r.CDkw;
            I.f1[c] = r.F1;
            I.f2[c] = r.F2;
            I.pk[c] = r.Pk;
            I.nut[c] = (nutMin < 0.0) ? r.nuT : smax(r.nuT, nutMin);
            continue;
        }
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
template <class T, bool Fast = false>
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
        double Df = Fast ? nuEff_f * M.aOverD[f] : nuEff_f * Sf / delta;
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

// Reynolds-stress injection source (SIMPLESolver::addInjectionSource,
// incompressible/src/SIMPLESolver.cpp:224-315), run before the x-momentum
// assembly of every outer iteration.  Per cell the deferred-correction tensor
// D = 2 k b_target + 2 nu_t dev(S) from the velocity gradients `g`
// (g[3*i+j] = dU_i/dx_j) and eddy viscosity `nut` (FP64, or the mixed
// engine's FP32 stage-1 copies); per cell the
// force q = -sum_f (D_f . n_f) A_f gathered over its internal faces in
// ascending face order (D_f distance-weighted, owner side subtracts) and then
// its boundary faces (owner value), the reference's scatter order; then
// blend = q on the first pass of a solve (or alpha >= 1), else
// blend (1 - alpha) + q alpha.  inj[0..3nC) holds the blend, inj[3nC..9nC) D.
template <class T, class G>
__device__ __noinline__ void phase_inj(T &tm, const DevMesh &M, DevInst &I, const G *const *g, const G *nut,
                                       bool first) {
    const int nC = M.nC;
    double *D = I.inj + 3 * (size_t)nC;
    // the mixed engine's stage 1 skips the w gradients of a 2-D instance
    // (identically zero there)
    const bool wGrad = sizeof(G) == 8 || I.solveZ != 0;
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        const double g6 = wGrad ? (double)LD(g[6] + c) : 0.0, g7 = wGrad ? (double)LD(g[7] + c) : 0.0;
        const double S11 = LD(g[0] + c), S22 = LD(g[4] + c), S33 = wGrad ? (double)LD(g[8] + c) : 0.0;
        const double S12 = 0.5 * ((double)LD(g[1] + c) + (double)LD(g[3] + c));
        const double S13 = 0.5 * ((double)LD(g[2] + c) + g6);
        const double S23 = 0.5 * ((double)LD(g[5] + c) + g7);
        const double trS3 = (S11 + S22 + S33) / 3.0;
        const double twoK = 2.0 * LD(I.k + c), twoNu = 2.0 * (double)LD(nut + c);
        const double *bt = M.bTarget + 6 * (size_t)c;
        D[0 * (size_t)nC + c] = twoK * bt[0] + twoNu * (S11 - trS3);
        D[1 * (size_t)nC + c] = twoK * bt[1] + twoNu * (S22 - trS3);
        D[2 * (size_t)nC + c] = twoK * bt[2] + twoNu * (S33 - trS3);
        D[3 * (size_t)nC + c] = twoK * bt[3] + twoNu * S12;
        D[4 * (size_t)nC + c] = twoK * bt[4] + twoNu * S13;
        D[5 * (size_t)nC + c] = twoK * bt[5] + twoNu * S23;
    }
    tm.sync();
    const double r = I.S.alphaInj;
    const bool fresh = first || r >= 1.0;
    for (int c = tm.rank(); c < nC; c += tm.size()) {
        double qx = 0.0, qy = 0.0, qz = 0.0;
        for (int e = M.cfOff[c]; e < M.cfOff[c + 1]; ++e) {
            const int f = M.cfFace[e], oth = M.cfOther[e];
            const int o = oth >= 0 ? c : -(oth + 1), n = oth >= 0 ? oth : c;
            const double w = M.w[f], wn = 1.0 - w;
            double d[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) d[k] = w * LD(D + k * (size_t)nC + o) + wn * LD(D + k * (size_t)nC + n);
            const double nx = M.nx[f], ny = M.ny[f], nz = M.nz[f], A = M.area[f];
            const double fx = (d[0] * nx + d[3] * ny + d[4] * nz) * A;
            const double fy = (d[3] * nx + d[1] * ny + d[5] * nz) * A;
            const double fz = (d[4] * nx + d[5] * ny + d[2] * nz) * A;
            if (oth >= 0) { qx = qx - fx; qy = qy - fy; qz = qz - fz; }
            else { qx = qx + fx; qy = qy + fy; qz = qz + fz; }
        }
        for (int e = M.cbOff[c]; e < M.cbOff[c + 1]; ++e) {
            const int b = M.cbFace[e];
            double d[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) d[k] = LD(D + k * (size_t)nC + c);
            const double nx = M.bnx[b], ny = M.bny[b], nz = M.bnz[b], A = M.barea[b];
            qx = qx - (d[0] * nx + d[3] * ny + d[4] * nz) * A;
            qy = qy - (d[3] * nx + d[1] * ny + d[5] * nz) * A;
            qz = qz - (d[4] * nx + d[5] * ny + d[2] * nz) * A;
        }
        double *bl = I.inj;
        if (fresh) {
            bl[c] = qx;
            bl[nC + c] = qy;
            bl[2 * (size_t)nC + c] = qz;
        } else {
            bl[c] = LD(bl + c) * (1.0 - r) + qx * r;
            bl[nC + c] = LD(bl + nC + c) * (1.0 - r) + qy * r;
            bl[2 * (size_t)nC + c] = LD(bl + 2 * (size_t)nC + c) * (1.0 - r) + qz * r;
        }
    }
    tm.sync();
}

// Cell pass of the momentum system (diag, source, relaxation).
template <class T, bool Fast = false>
__device__ __noinline__ void phase_mom_cells(T &tm, const DevMesh &M, DevInst &I, int comp) {
    const double nu = I.nu;
    const double alphaU = I.S.alphaU;
    const double relaxDiag = 1.0 / alphaU, relaxSrc = (1.0 - alphaU) / alphaU;
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
            double Db = Fast ? nuEff * M.baOverD[b] : nuEff * Sf / delta;
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
        if (I.inj) src = src + LD(I.inj + (size_t)comp * M.nC + c);
        const double phi_old = LD(Uc + c);
        if (Fast) {
            src = src + relaxSrc * diag * phi_old;
            diag = diag * relaxDiag;
        } else {
            src = src + (1.0 - alphaU) / alphaU * diag * phi_old;
            diag = diag / alphaU;
        }
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
template <class T, bool Fast = false>
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
        double Df = Fast ? nuEff_f * M.aOverD[f] : nuEff_f * Sf / delta;
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

template <class T, bool Fast = false>
__device__ __noinline__ void phase_turb_cells(T &tm, const DevMesh &M, DevInst &I, int which) {
    const Coef cf = load_coef(I);
    const double nu = I.nu;
    const double s1 = which == 0 ? cf.sk1 : cf.sw1, s2 = which == 0 ? cf.sk2 : cf.sw2;
    const double *phib = which == 0 ? I.kb : I.omb;
    const double *phi = which == 0 ? I.k : I.om;
    const double alpha = which == 0 ? I.S.alphaK : I.S.alphaW;
    const double relaxDiag = 1.0 / alpha, relaxSrc = (1.0 - alpha) / alpha;
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
            double Db = Fast ? nuEff * M.baOverD[b] : nuEff * Sf / delta;
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
        if (Fast) {
            src = src + relaxSrc * diag * LD(phi + c);
            diag = diag * relaxDiag;
        } else {
            src = src + (1.0 - alpha) / alpha * diag * LD(phi + c);
            diag = diag / alpha;
        }
        I.diag[c] = diag;
        I.src[c] = src;
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

}  // namespace btm
