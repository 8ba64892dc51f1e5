/*
 * simple_oracle.c - plain-C restatement of the reference incompressible SIMPLE
 * solver with the SST k-omega closure.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the CPU checker the GB300 kernels are
 * compared against (tests/, __graft_entry__.smoke(), bench.py's CPU-baseline
 * leg).  It is never linked into, loaded by or called from the product.
 *
 * Parity: every routine follows the reference's loops and floating-point
 * operation order (face-ordered scatters, sequential dot products, the
 * sequential Gauss-Seidel AMG) and uses the std::min/std::max selection rules,
 * so that, compiled with -ffp-contract=off, it reproduces the reference build
 * bit for bit.  That is checked by tests/test_oracle_pin.py against golden
 * vectors written by the reference itself (tests/golden/make_golden.py).
 * Reference files are cited per function; paths are relative to the reference
 * project root.
 */
#include "simple_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double x, y, z; } v3;

static inline v3 mk(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 vdiv(v3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double vcomp(v3 a, int c) { return c == 0 ? a.x : (c == 1 ? a.y : a.z); }
/* std::max / std::min selection rules (return the first argument on ties/NaN) */
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }

static void *xcalloc(size_t n, size_t sz) {
    void *p = calloc(n ? n : 1, sz);
    if (!p) abort();
    return p;
}

/* ------------------------------------------------------------------------ */
/* mesh access                                                               */
/* ------------------------------------------------------------------------ */
static inline v3 fnormal(const btm_mesh *m, int f) {
    return mk(m->face_normal[3 * f], m->face_normal[3 * f + 1], m->face_normal[3 * f + 2]);
}
static inline v3 fdvec(const btm_mesh *m, int f) {
    return mk(m->face_d[3 * f], m->face_d[3 * f + 1], m->face_d[3 * f + 2]);
}

/* ------------------------------------------------------------------------ */
/* SST coefficients (core/include/SSTModel.hpp:9-40)                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    double sigma_k1, sigma_w1, beta1, alpha1, sigma_k2, sigma_w2, beta2, alpha2, betaStar, a1, kappa;
    int variant;
} Sst;

static Sst sst_from(const double *c, int variant) {
    Sst s;
    s.sigma_k1 = c[0]; s.sigma_w1 = c[1]; s.beta1 = c[2]; s.alpha1 = c[3];
    s.sigma_k2 = c[4]; s.sigma_w2 = c[5]; s.beta2 = c[6]; s.alpha2 = c[7];
    s.betaStar = c[8]; s.a1 = c[9]; s.kappa = c[10];
    s.variant = variant;
    return s;
}
static inline double blend(double p1, double p2, double F1) { return F1 * p1 + (1.0 - F1) * p2; }
static inline double sigma_k(const Sst *s, double F1) { return blend(s->sigma_k1, s->sigma_k2, F1); }
static inline double sigma_w(const Sst *s, double F1) { return blend(s->sigma_w1, s->sigma_w2, F1); }
static inline double beta_b(const Sst *s, double F1) { return blend(s->beta1, s->beta2, F1); }
static inline double alpha_b(const Sst *s, double F1) { return blend(s->alpha1, s->alpha2, F1); }

/* SSTModel point functions (core/src/SSTModel.cpp:9-96) */
static double computeF1(const Sst *s, double k, double omega, double y, double nu, double CDkw_pos) {
    double sqrtK = sqrt(smax(k, 0.0));
    double omSafe = smax(omega, 1e-20);
    double ySafe = smax(y, 1e-20);
    double y2s = ySafe * ySafe;
    double term1 = sqrtK / (s->betaStar * omSafe * ySafe);
    double term2 = 500.0 * nu / (y2s * omSafe);
    double CDpos = smax(CDkw_pos, 1e-20);
    double term3 = 4.0 * s->sigma_w2 * smax(k, 0.0) / (CDpos * y2s);
    double arg1 = smin(smax(term1, term2), term3);
    double a4 = arg1 * arg1 * arg1 * arg1;
    return tanh(a4);
}
static double computeF2(const Sst *s, double k, double omega, double y, double nu) {
    double sqrtK = sqrt(smax(k, 0.0));
    double omSafe = smax(omega, 1e-20);
    double ySafe = smax(y, 1e-20);
    double y2 = ySafe * ySafe;
    double term1 = 2.0 * sqrtK / (s->betaStar * omSafe * ySafe);
    double term2 = 500.0 * nu / (y2 * omSafe);
    double arg2 = smax(term1, term2);
    return tanh(arg2 * arg2);
}
static double crossDiffusion(const Sst *s, v3 gk, v3 gw, double omega) {
    double omSafe = smax(omega, 1e-20);
    return 2.0 * s->sigma_w2 / omSafe * vdot(gk, gw);
}
static double eddyViscosity(const Sst *s, double k, double omega, double S, double F2) {
    double kSafe = smax(k, 0.0);
    if (s->variant == BTM_SST_NOLIMITER) return kSafe / smax(omega, 1e-20);
    double denom = smax(s->a1 * omega, S * F2);
    denom = smax(denom, 1e-20);
    return s->a1 * kSafe / denom;
}
static double production(const Sst *s, double nuT, double S, double k, double omega) {
    double Pk_raw = nuT * S * S;
    double Pk_lim = 10.0 * s->betaStar * smax(k, 0.0) * smax(omega, 1e-20);
    return smin(Pk_raw, Pk_lim);
}
static double productionOmega(const Sst *s, double nuT, double S, double k, double omega) {
    double S2 = S * S;
    double lim = 10.0 * s->betaStar * smax(k, 0.0) * smax(omega, 1e-20) / smax(nuT, 1e-30);
    return smin(S2, lim);
}

/* ------------------------------------------------------------------------ */
/* gradients (core/include/Field.hpp:122-152, 232-267)                        */
/* ------------------------------------------------------------------------ */
static void green_gauss(const btm_mesh *m, const double *phi, const double *phib, v3 *grad) {
    int nIF = m->n_internal_faces, nF = m->n_faces, nC = m->n_cells;
    for (int c = 0; c < nC; ++c) grad[c] = mk(0.0, 0.0, 0.0);
    for (int fi = 0; fi < nIF; ++fi) {
        int o = m->owner[fi], n = m->neighbour[fi];
        double w = m->face_weight[fi];
        double phiF = phi[o] * w + phi[n] * (1.0 - w);
        v3 Sf = vmul(fnormal(m, fi), m->face_area[fi]);
        grad[o] = vadd(grad[o], vmul(Sf, phiF));
        grad[n] = vsub(grad[n], vmul(Sf, phiF));
    }
    for (int fi = nIF; fi < nF; ++fi) {
        int o = m->owner[fi];
        v3 Sf = vmul(fnormal(m, fi), m->face_area[fi]);
        grad[o] = vadd(grad[o], vmul(Sf, phib[fi - nIF]));
    }
    for (int c = 0; c < nC; ++c) {
        double V = m->cell_volume[c];
        if (V > 1e-30) grad[c] = vdiv(grad[c], V);
    }
}

typedef struct { v3 *dudx, *dvdx, *dwdx; } VelGrad;

static void velocity_gradients(const btm_mesh *m, const v3 *U, const v3 *Ub, VelGrad *vg,
                               double *tmp, double *tmpb) {
    int nC = m->n_cells, nB = m->n_faces - m->n_internal_faces;
    v3 *outs[3] = {vg->dudx, vg->dvdx, vg->dwdx};
    for (int c3 = 0; c3 < 3; ++c3) {
        for (int i = 0; i < nC; ++i) tmp[i] = vcomp(U[i], c3);
        for (int b = 0; b < nB; ++b) tmpb[b] = vcomp(Ub[b], c3);
        green_gauss(m, tmp, tmpb, outs[c3]);
    }
}

static void strain_rate(int nC, const VelGrad *vg, double *S) {
    for (int c = 0; c < nC; ++c) {
        double S11 = vg->dudx[c].x, S22 = vg->dvdx[c].y, S33 = vg->dwdx[c].z;
        double S12 = 0.5 * (vg->dudx[c].y + vg->dvdx[c].x);
        double S13 = 0.5 * (vg->dudx[c].z + vg->dwdx[c].x);
        double S23 = 0.5 * (vg->dvdx[c].z + vg->dwdx[c].y);
        S[c] = sqrt(2.0 * (S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23)));
    }
}

/* ------------------------------------------------------------------------ */
/* linear algebra (core/include/LinearSolver.hpp)                            */
/* ------------------------------------------------------------------------ */
typedef struct {
    int nC, nIF;
    double *diag, *upper, *lower, *source;
    const int *own, *nbr;
} Lsys;

static void matvec(const Lsys *A, const double *x, double *y) {
    for (int i = 0; i < A->nC; ++i) y[i] = A->diag[i] * x[i];
    for (int f = 0; f < A->nIF; ++f) {
        y[A->own[f]] += A->upper[f] * x[A->nbr[f]];
        y[A->nbr[f]] += A->lower[f] * x[A->own[f]];
    }
}
static void residual(const Lsys *A, const double *x, double *r) {
    matvec(A, x, r);
    for (int i = 0; i < A->nC; ++i) r[i] = A->source[i] - r[i];
}
static double dot(int n, const double *a, const double *b) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}
static double norm(int n, const double *v) { return sqrt(dot(n, v, v)); }
static void jacobi(const Lsys *A, const double *r, double *z) {
    for (int i = 0; i < A->nC; ++i) z[i] = (fabs(A->diag[i]) > 1e-30) ? r[i] / A->diag[i] : r[i];
}

typedef struct { int iterations; double finalRes, initialRes; int converged; } SolverResult;

/* PCGSolver::solve (LinearSolver.hpp:147-186) */
static SolverResult pcg_solve(const Lsys *A, double *x, int maxIter, double tol) {
    int n = A->nC;
    double *r = xcalloc(n, 8), *z = xcalloc(n, 8), *p = xcalloc(n, 8), *Ap = xcalloc(n, 8);
    SolverResult res = {0, 0.0, 0.0, 0};
    residual(A, x, r);
    double r0 = norm(n, r);
    res.initialRes = r0;
    if (r0 < 1e-30) { res.converged = 1; goto done; }
    jacobi(A, r, z);
    memcpy(p, z, sizeof(double) * n);
    double rz = dot(n, r, z);
    for (int it = 0; it < maxIter; ++it) {
        matvec(A, p, Ap);
        double pAp = dot(n, p, Ap);
        if (fabs(pAp) < 1e-30) break;
        double alpha = rz / pAp;
        for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
        double rn = norm(n, r);
        res.iterations = it + 1;
        res.finalRes = rn / r0;
        if (res.finalRes < tol) { res.converged = 1; goto done; }
        jacobi(A, r, z);
        double rzNew = dot(n, r, z);
        double beta = rzNew / (rz + 1e-30);
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rz = rzNew;
    }
done:
    free(r); free(z); free(p); free(Ap);
    return res;
}

/* BiCGSTABSolver::solve (LinearSolver.hpp:191-247) */
static SolverResult bicgstab_solve(const Lsys *A, double *x, int maxIter, double tol) {
    int n = A->nC;
    double *r = xcalloc(n, 8), *rh = xcalloc(n, 8), *p = xcalloc(n, 8), *v = xcalloc(n, 8);
    double *s = xcalloc(n, 8), *t = xcalloc(n, 8), *ph = xcalloc(n, 8), *sh = xcalloc(n, 8);
    SolverResult res = {0, 0.0, 0.0, 0};
    residual(A, x, r);
    double r0 = norm(n, r);
    res.initialRes = r0;
    if (r0 < 1e-30) { res.converged = 1; goto done; }
    memcpy(rh, r, sizeof(double) * n);
    double rho = 1, alpha = 1, omega = 1;
    for (int it = 0; it < maxIter; ++it) {
        double rhoN = dot(n, rh, r);
        if (fabs(rhoN) < 1e-30) break;
        double beta = (rhoN / (rho + 1e-30)) * (alpha / (omega + 1e-30));
        for (int i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        jacobi(A, p, ph);
        matvec(A, ph, v);
        double rv = dot(n, rh, v);
        if (fabs(rv) < 1e-30) break;
        alpha = rhoN / rv;
        for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
        double sn = norm(n, s);
        if (sn / r0 < tol) {
            for (int i = 0; i < n; ++i) x[i] += alpha * ph[i];
            res.iterations = it + 1; res.finalRes = sn / r0; res.initialRes = r0; res.converged = 1;
            goto done;
        }
        jacobi(A, s, sh);
        matvec(A, sh, t);
        double tt = dot(n, t, t);
        omega = (tt > 1e-30) ? dot(n, t, s) / tt : 0.0;
        for (int i = 0; i < n; ++i) x[i] += alpha * ph[i] + omega * sh[i];
        for (int i = 0; i < n; ++i) r[i] = s[i] - omega * t[i];
        double rn = norm(n, r);
        res.iterations = it + 1;
        res.finalRes = rn / r0;
        if (res.finalRes < tol) { res.converged = 1; goto done; }
        if (fabs(omega) < 1e-30) break;
        rho = rhoN;
    }
done:
    free(r); free(rh); free(p); free(v); free(s); free(t); free(ph); free(sh);
    return res;
}

/* GaussSeidelSolver::solve (LinearSolver.hpp:258-299) */
static SolverResult gs_solve(const Lsys *A, double *x, int maxIter, double tol) {
    int n = A->nC;
    SolverResult res = {0, 0.0, 0.0, 0};
    double *r = xcalloc(n, 8);
    double b0 = norm(n, A->source);
    res.initialRes = b0;
    if (b0 < 1e-30) b0 = 1.0;
    int *deg = xcalloc(n, sizeof(int)), *off = xcalloc(n + 1, sizeof(int));
    for (int f = 0; f < A->nIF; ++f) { ++deg[A->own[f]]; ++deg[A->nbr[f]]; }
    for (int i = 0; i < n; ++i) off[i + 1] = off[i] + deg[i];
    int *adjIdx = xcalloc(off[n], sizeof(int));
    double *adjCoef = xcalloc(off[n], 8);
    int *cursor = xcalloc(n, sizeof(int));
    for (int i = 0; i < n; ++i) cursor[i] = off[i];
    for (int f = 0; f < A->nIF; ++f) {
        int o = A->own[f], nb = A->nbr[f];
        adjIdx[cursor[o]] = nb; adjCoef[cursor[o]++] = A->upper[f];
        adjIdx[cursor[nb]] = o; adjCoef[cursor[nb]++] = A->lower[f];
    }
    for (int it = 0; it < maxIter; ++it) {
        for (int i = 0; i < n; ++i) {
            if (fabs(A->diag[i]) <= 1e-30) continue;
            double s = A->source[i];
            for (int a = off[i]; a < off[i + 1]; ++a) s -= adjCoef[a] * x[adjIdx[a]];
            x[i] = s / A->diag[i];
        }
        residual(A, x, r);
        res.iterations = it + 1;
        res.finalRes = norm(n, r) / b0;
        if (res.finalRes < tol) { res.converged = 1; break; }
    }
    free(r); free(deg); free(off); free(adjIdx); free(adjCoef); free(cursor);
    return res;
}

/* ---- AMG (LinearSolver.hpp:304-656) ----------------------------------- */
typedef struct {
    int nRows;
    int *rowPtr, *colIdx;
    double *values, *diag;
} Csr;

static void csr_free(Csr *A) { free(A->rowPtr); free(A->colIdx); free(A->values); free(A->diag); }

/* lduToCSR (LinearSolver.hpp:344-404) */
static Csr ldu_to_csr(const Lsys *A) {
    int n = A->nC;
    Csr c;
    int *count = xcalloc(n, sizeof(int));
    for (int i = 0; i < n; ++i) count[i] = 1;
    for (int f = 0; f < A->nIF; ++f) { count[A->own[f]]++; count[A->nbr[f]]++; }
    c.nRows = n;
    c.rowPtr = xcalloc(n + 1, sizeof(int));
    for (int i = 0; i < n; ++i) c.rowPtr[i + 1] = c.rowPtr[i] + count[i];
    int nnz = c.rowPtr[n];
    c.colIdx = xcalloc(nnz, sizeof(int));
    c.values = xcalloc(nnz, 8);
    c.diag = xcalloc(n, 8);
    int *pos = xcalloc(n, sizeof(int));
    for (int i = 0; i < n; ++i) pos[i] = c.rowPtr[i];
    for (int i = 0; i < n; ++i) {
        c.colIdx[pos[i]] = i; c.values[pos[i]] = A->diag[i]; c.diag[i] = A->diag[i]; pos[i]++;
    }
    for (int f = 0; f < A->nIF; ++f) {
        int o = A->own[f], nb = A->nbr[f];
        c.colIdx[pos[o]] = nb; c.values[pos[o]] = A->upper[f]; pos[o]++;
        c.colIdx[pos[nb]] = o; c.values[pos[nb]] = A->lower[f]; pos[nb]++;
    }
    for (int i = 0; i < n; ++i) {
        int start = c.rowPtr[i], end = c.rowPtr[i + 1];
        for (int a = start + 1; a < end; ++a) {
            int key_c = c.colIdx[a];
            double key_v = c.values[a];
            int b = a - 1;
            while (b >= start && c.colIdx[b] > key_c) {
                c.colIdx[b + 1] = c.colIdx[b];
                c.values[b + 1] = c.values[b];
                b--;
            }
            c.colIdx[b + 1] = key_c;
            c.values[b + 1] = key_v;
        }
    }
    free(count); free(pos);
    return c;
}

static void csr_residual(const Csr *A, const double *x, const double *b, double *r) {
    for (int i = 0; i < A->nRows; ++i) {
        double s = 0.0;
        for (int j = A->rowPtr[i]; j < A->rowPtr[i + 1]; ++j) s += A->values[j] * x[A->colIdx[j]];
        r[i] = b[i] - s;
    }
}
static void csr_gs_sweep(const Csr *A, double *x, const double *b) {
    for (int i = 0; i < A->nRows; ++i) {
        double s = b[i];
        for (int j = A->rowPtr[i]; j < A->rowPtr[i + 1]; ++j)
            if (A->colIdx[j] != i) s -= A->values[j] * x[A->colIdx[j]];
        if (fabs(A->diag[i]) > 1e-30) x[i] = s / A->diag[i];
    }
}

/* buildAggregates (LinearSolver.hpp:407-443) */
static int build_aggregates(const Csr *A, int *map) {
    int n = A->nRows, nCoarse = 0;
    for (int i = 0; i < n; ++i) map[i] = -1;
    for (int i = 0; i < n; ++i) {
        if (map[i] >= 0) continue;
        int agg = nCoarse++;
        map[i] = agg;
        double aii = fabs(A->diag[i]);
        for (int j = A->rowPtr[i]; j < A->rowPtr[i + 1]; ++j) {
            int c = A->colIdx[j];
            if (c == i || map[c] >= 0) continue;
            double ajj = fabs(A->diag[c]);
            double strength = fabs(A->values[j]) / sqrt(aii * ajj + 1e-30);
            if (strength > 0.25) map[c] = agg;
        }
    }
    for (int i = 0; i < n; ++i) {
        if (map[i] >= 0) continue;
        double bestStr = -1.0;
        int bestAgg = 0;
        for (int j = A->rowPtr[i]; j < A->rowPtr[i + 1]; ++j) {
            int c = A->colIdx[j];
            if (c == i && map[c] < 0) continue;
            if (map[c] >= 0 && fabs(A->values[j]) > bestStr) {
                bestStr = fabs(A->values[j]);
                bestAgg = map[c];
            }
        }
        map[i] = bestAgg;
    }
    return nCoarse;
}

/* galerkinProduct (LinearSolver.hpp:446-485).  Each coarse entry (I,J) sums
 * its fine contributions in (fine row ascending, fine column ascending) order,
 * the order of the reference's single pass over the fine rows. */
static int cmp_int_pair(const void *a, const void *b) {
    const int *x = a, *y = b;
    return (x[0] > y[0]) - (x[0] < y[0]);
}
static Csr galerkin(const Csr *A, const int *map, int nCoarse) {
    int n = A->nRows;
    int *moff = xcalloc(nCoarse + 1, sizeof(int)), *mem = xcalloc(n, sizeof(int));
    for (int i = 0; i < n; ++i) moff[map[i] + 1]++;
    for (int I = 0; I < nCoarse; ++I) moff[I + 1] += moff[I];
    int *cur = xcalloc(nCoarse, sizeof(int));
    for (int I = 0; I < nCoarse; ++I) cur[I] = moff[I];
    for (int i = 0; i < n; ++i) mem[cur[map[i]]++] = i;
    int *marker = xcalloc(nCoarse, sizeof(int)), *pos = xcalloc(nCoarse, sizeof(int));
    for (int I = 0; I < nCoarse; ++I) marker[I] = -1;
    int cap = A->rowPtr[n] + 16;
    int *cols = xcalloc(cap, sizeof(int));
    double *vals = xcalloc(cap, 8);
    int *rowPtr = xcalloc(nCoarse + 1, sizeof(int));
    int nnz = 0;
    int *pairs = xcalloc(2 * (size_t)cap, sizeof(int));
    for (int I = 0; I < nCoarse; ++I) {
        int start = nnz;
        for (int q = moff[I]; q < moff[I + 1]; ++q) {
            int i = mem[q];
            for (int j = A->rowPtr[i]; j < A->rowPtr[i + 1]; ++j) {
                int J = map[A->colIdx[j]];
                if (marker[J] != I) {
                    marker[J] = I;
                    pos[J] = nnz;
                    cols[nnz] = J;
                    vals[nnz] = 0.0;
                    nnz++;
                }
                vals[pos[J]] += A->values[j];
            }
        }
        /* sort the row's entries by column (std::sort of (col, val) pairs) */
        int len = nnz - start;
        for (int e = 0; e < len; ++e) { pairs[2 * e] = cols[start + e]; pairs[2 * e + 1] = start + e; }
        qsort(pairs, len, 2 * sizeof(int), cmp_int_pair);
        int *tc = xcalloc(len, sizeof(int));
        double *tv = xcalloc(len, 8);
        for (int e = 0; e < len; ++e) { tc[e] = pairs[2 * e]; tv[e] = vals[pairs[2 * e + 1]]; }
        for (int e = 0; e < len; ++e) { cols[start + e] = tc[e]; vals[start + e] = tv[e]; }
        free(tc); free(tv);
        rowPtr[I + 1] = nnz;
    }
    Csr c;
    c.nRows = nCoarse;
    c.rowPtr = rowPtr;
    c.colIdx = xcalloc(nnz, sizeof(int));
    c.values = xcalloc(nnz, 8);
    memcpy(c.colIdx, cols, sizeof(int) * nnz);
    memcpy(c.values, vals, 8 * (size_t)nnz);
    c.diag = xcalloc(nCoarse, 8);
    for (int I = 0; I < nCoarse; ++I)
        for (int j = rowPtr[I]; j < rowPtr[I + 1]; ++j)
            if (c.colIdx[j] == I) c.diag[I] = c.values[j];
    free(moff); free(mem); free(cur); free(marker); free(pos); free(cols); free(vals); free(pairs);
    return c;
}

#define AMG_MAX_LEVELS 21
typedef struct {
    Csr A;
    int *map;
    int nCoarse;
    double *x, *b, *r;
} AmgLevel;
typedef struct { int nLevels; AmgLevel lev[AMG_MAX_LEVELS]; } Amg;

static void amg_free(Amg *g) {
    for (int l = 0; l < g->nLevels; ++l) {
        csr_free(&g->lev[l].A);
        free(g->lev[l].map); free(g->lev[l].x); free(g->lev[l].b); free(g->lev[l].r);
    }
    g->nLevels = 0;
}

/* AMGSolver::setup (LinearSolver.hpp:516-551) */
static void amg_setup(Amg *g, const Lsys *A) {
    memset(g, 0, sizeof *g);
    g->lev[0].A = ldu_to_csr(A);
    g->nLevels = 1;
    for (int l = 0; l < 20; ++l) {
        AmgLevel *fine = &g->lev[l];
        if (fine->A.nRows <= 50) break;
        int *map = xcalloc(fine->A.nRows, sizeof(int));
        int nc = build_aggregates(&fine->A, map);
        if (nc == 0 || nc >= fine->A.nRows) { free(map); break; }
        fine->map = map;
        fine->nCoarse = nc;
        g->lev[l + 1].A = galerkin(&fine->A, map, nc);
        g->nLevels = l + 2;
    }
    for (int l = 0; l < g->nLevels; ++l) {
        int n = g->lev[l].A.nRows;
        g->lev[l].x = xcalloc(n, 8);
        g->lev[l].b = xcalloc(n, 8);
        g->lev[l].r = xcalloc(n, 8);
    }
}

/* SSTModel point functions for known-answer checks: which = 0 production
 * (nuT, S, k, omega), 1 productionOmega (nuT, S, k, omega), 2 F1 (k, omega,
 * y, nu, CDkw+), 3 F2 (k, omega, y, nu), 4 eddy viscosity (k, omega, S, F2). */
double oracle_sst_point(const double *coeffs, int variant, int which, const double *a) {
    Sst s = sst_from(coeffs, variant);
    switch (which) {
        case 0: return production(&s, a[0], a[1], a[2], a[3]);
        case 1: return productionOmega(&s, a[0], a[1], a[2], a[3]);
        case 2: return computeF1(&s, a[0], a[1], a[2], a[3], a[4]);
        case 3: return computeF2(&s, a[0], a[1], a[2], a[3]);
        default: return eddyViscosity(&s, a[0], a[1], a[2], a[3]);
    }
}

/* AMGSolver::setup's coarsening loop (LinearSolver.hpp:516-551) on a given
 * CSR matrix (rows sorted by column): buildAggregates + galerkinProduct until
 * a level has at most 50 rows, stops coarsening, or max_levels levels exist.
 * sizes[max_levels]; maps receives the aggregation map of every level that
 * has one, concatenated.  Returns the level count. */
int oracle_amg_levels(int n, const int *rowPtr, const int *colIdx, const double *values, int max_levels,
                      int *sizes, int *maps) {
    Csr A;
    A.nRows = n;
    A.rowPtr = xcalloc(n + 1, sizeof(int));
    memcpy(A.rowPtr, rowPtr, sizeof(int) * (n + 1));
    A.colIdx = xcalloc(rowPtr[n] > 0 ? rowPtr[n] : 1, sizeof(int));
    memcpy(A.colIdx, colIdx, sizeof(int) * rowPtr[n]);
    A.values = xcalloc(rowPtr[n] > 0 ? rowPtr[n] : 1, 8);
    memcpy(A.values, values, 8 * (size_t)rowPtr[n]);
    A.diag = xcalloc(n, 8);
    for (int i = 0; i < n; ++i)
        for (int j = rowPtr[i]; j < rowPtr[i + 1]; ++j)
            if (colIdx[j] == i) A.diag[i] = values[j];
    int levels = 1, at = 0;
    sizes[0] = n;
    while (levels < max_levels && A.nRows > 50) {
        int *map = xcalloc(A.nRows, sizeof(int));
        int nc = build_aggregates(&A, map);
        if (nc == 0 || nc >= A.nRows) { free(map); break; }
        memcpy(maps + at, map, sizeof(int) * A.nRows);
        at += A.nRows;
        Csr Cm = galerkin(&A, map, nc);
        free(map);
        csr_free(&A);
        A = Cm;
        sizes[levels++] = nc;
    }
    csr_free(&A);
    return levels;
}

/* AMGSolver::vcycle (LinearSolver.hpp:553-589) */
static void amg_vcycle(Amg *g, int level) {
    AmgLevel *lev = &g->lev[level];
    int n = lev->A.nRows;
    if (level == g->nLevels - 1) {
        for (int s = 0; s < 50; ++s) csr_gs_sweep(&lev->A, lev->x, lev->b);
        return;
    }
    for (int s = 0; s < 2; ++s) csr_gs_sweep(&lev->A, lev->x, lev->b);
    csr_residual(&lev->A, lev->x, lev->b, lev->r);
    AmgLevel *coarse = &g->lev[level + 1];
    int nc = coarse->A.nRows;
    for (int I = 0; I < nc; ++I) { coarse->b[I] = 0.0; coarse->x[I] = 0.0; }
    for (int i = 0; i < n; ++i) coarse->b[lev->map[i]] += lev->r[i];
    amg_vcycle(g, level + 1);
    for (int i = 0; i < n; ++i) lev->x[i] += coarse->x[lev->map[i]];
    for (int s = 0; s < 2; ++s) csr_gs_sweep(&lev->A, lev->x, lev->b);
}

static void amg_precondition(Amg *g, const double *r, double *z) {
    AmgLevel *l0 = &g->lev[0];
    int n = l0->A.nRows;
    memcpy(l0->b, r, sizeof(double) * n);
    for (int i = 0; i < n; ++i) l0->x[i] = 0.0;
    amg_vcycle(g, 0);
    memcpy(z, l0->x, sizeof(double) * n);
}

/* AMGSolver::solve (LinearSolver.hpp:602-653) */
static SolverResult amg_solve(const Lsys *A, double *x, int maxIter, double tol) {
    Amg g;
    amg_setup(&g, A);
    int n = A->nC;
    double *r = xcalloc(n, 8), *z = xcalloc(n, 8), *p = xcalloc(n, 8), *Ap = xcalloc(n, 8);
    SolverResult res = {0, 0.0, 0.0, 0};
    residual(A, x, r);
    double r0 = norm(n, r);
    res.initialRes = r0;
    if (r0 < 1e-30) { res.converged = 1; goto done; }
    amg_precondition(&g, r, z);
    memcpy(p, z, sizeof(double) * n);
    double rz = dot(n, r, z);
    for (int it = 0; it < maxIter; ++it) {
        matvec(A, p, Ap);
        double pAp = dot(n, p, Ap);
        if (fabs(pAp) < 1e-30) break;
        double alpha = rz / pAp;
        for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
        double rn = norm(n, r);
        res.iterations = it + 1;
        res.finalRes = rn / r0;
        if (res.finalRes < tol) { res.converged = 1; goto done; }
        amg_precondition(&g, r, z);
        double rzNew = dot(n, r, z);
        double beta = rzNew / (rz + 1e-30);
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rz = rzNew;
    }
done:
    free(r); free(z); free(p); free(Ap);
    amg_free(&g);
    return res;
}

/* makeSolver (LinearSolver.hpp:659-665): unknown names are BiCGSTAB */
static SolverResult linear_solve(int kind, const Lsys *A, double *x, int maxIter, double tol) {
    switch (kind) {
        case BTM_LS_PCG: return pcg_solve(A, x, maxIter, tol);
        case BTM_LS_GAUSSSEIDEL: return gs_solve(A, x, maxIter, tol);
        case BTM_LS_AMG: return amg_solve(A, x, maxIter, tol);
        default: return bicgstab_solve(A, x, maxIter, tol);
    }
}

/* ------------------------------------------------------------------------ */
/* SIMPLE solver (incompressible/src/SIMPLESolver.cpp)                        */
/* ------------------------------------------------------------------------ */
typedef struct {
    v3 *U, *Ub;
    double *p, *pb, *k, *kb, *om, *omb, *nuT, *F1, *F2, *Pk, *CDkw;
    int turbEstablished;
} Fields;

typedef struct {
    const btm_mesh *m;
    const btm_patch_bc *bcs;
    double nu;
    const btm_settings *s;
    Sst sst;
    int nC, nF, nIF, nB, nP;
    char *isWall;          /* per face: belongs to a 'wall' patch */
    double *aP, *aPunrelaxed;
    /* scratch */
    VelGrad vg;
    v3 *gradTmp;
    double *tmp, *tmpb;
    int64_t innerIters;
    /* Reynolds-stress injection (SIMPLESolver.hpp:93-105) */
    const double *bTarget6;
    v3 *injBlend;
    int injHave;
    double injRelax;
} Solver;

/* target anisotropy of the next oracle_solve (NULL: no injection) */
static const double *g_bTarget6 = NULL;
void oracle_set_target_anisotropy(const double *b6) { g_bTarget6 = b6; }

static void solver_init(Solver *S, const btm_mesh *m, const btm_patch_bc *bcs, double nu,
                        const btm_settings *s, const double *coeffs, int variant) {
    memset(S, 0, sizeof *S);
    S->m = m; S->bcs = bcs; S->nu = nu; S->s = s;
    S->sst = sst_from(coeffs, variant);
    S->nC = m->n_cells; S->nF = m->n_faces; S->nIF = m->n_internal_faces;
    S->nB = S->nF - S->nIF; S->nP = m->n_patches;
    S->isWall = xcalloc(S->nF, 1);
    for (int p = 0; p < S->nP; ++p)
        if (m->patch_type[p] == BTM_PATCH_WALL)
            for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) S->isWall[m->patch_faces[q]] = 1;
    S->aP = xcalloc(S->nC, 8);
    S->aPunrelaxed = xcalloc(S->nC, 8);
    S->vg.dudx = xcalloc(S->nC, sizeof(v3));
    S->vg.dvdx = xcalloc(S->nC, sizeof(v3));
    S->vg.dwdx = xcalloc(S->nC, sizeof(v3));
    S->gradTmp = xcalloc(S->nC, sizeof(v3));
    S->tmp = xcalloc(S->nC, 8);
    S->tmpb = xcalloc(S->nB > 0 ? S->nB : 1, 8);
}
static void solver_free(Solver *S) {
    free(S->injBlend);
    free(S->isWall); free(S->aP); free(S->aPunrelaxed);
    free(S->vg.dudx); free(S->vg.dvdx); free(S->vg.dwdx); free(S->gradTmp);
    free(S->tmp); free(S->tmpb);
}

static void fields_alloc(Fields *f, int nC, int nB) {
    f->U = xcalloc(nC, sizeof(v3)); f->Ub = xcalloc(nB, sizeof(v3));
    f->p = xcalloc(nC, 8); f->pb = xcalloc(nB, 8);
    f->k = xcalloc(nC, 8); f->kb = xcalloc(nB, 8);
    f->om = xcalloc(nC, 8); f->omb = xcalloc(nB, 8);
    f->nuT = xcalloc(nC, 8); f->F1 = xcalloc(nC, 8); f->F2 = xcalloc(nC, 8);
    f->Pk = xcalloc(nC, 8); f->CDkw = xcalloc(nC, 8);
    f->turbEstablished = 0;
}
static void fields_free(Fields *f) {
    free(f->U); free(f->Ub); free(f->p); free(f->pb); free(f->k); free(f->kb); free(f->om);
    free(f->omb); free(f->nuT); free(f->F1); free(f->F2); free(f->Pk); free(f->CDkw);
}

/* ---- boundary conditions (core/include/BoundaryCondition.hpp:196-342) --- */
static void apply_velocity_bc(const Solver *S, Fields *f) {
    const btm_mesh *m = S->m;
    for (int p = 0; p < S->nP; ++p) {
        const btm_patch_bc *bc = &S->bcs[p];
        for (int q = m->patch_offset[p], kk = 0; q < m->patch_offset[p + 1]; ++q, ++kk) {
            int fi = m->patch_faces[q], b = fi - S->nIF;
            switch (bc->u_type) {
                case BTM_BC_WALL_NO_SLIP: f->Ub[b] = mk(0, 0, 0); break;
                case BTM_BC_WALL_MOVING: f->Ub[b] = mk(bc->u_value[0], bc->u_value[1], bc->u_value[2]); break;
                case BTM_BC_INLET_VELOCITY:
                case BTM_BC_DIRICHLET:
                    f->Ub[b] = bc->u_profile ? mk(bc->u_profile[3 * kk], bc->u_profile[3 * kk + 1], bc->u_profile[3 * kk + 2])
                                             : mk(bc->u_value[0], bc->u_value[1], bc->u_value[2]);
                    break;
                case BTM_BC_SYMMETRY: {
                    v3 Uo = f->U[m->owner[fi]];
                    v3 n = fnormal(m, fi);
                    f->Ub[b] = vsub(Uo, vmul(n, vdot(Uo, n)));
                    break;
                }
                default: f->Ub[b] = f->U[m->owner[fi]]; break;
            }
        }
    }
}
static void apply_pressure_bc(const Solver *S, const double *pc, double *pbnd) {
    const btm_mesh *m = S->m;
    for (int p = 0; p < S->nP; ++p) {
        const btm_patch_bc *bc = &S->bcs[p];
        for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) {
            int fi = m->patch_faces[q];
            if (bc->p_type == BTM_BC_OUTLET_PRESSURE || bc->p_type == BTM_BC_DIRICHLET)
                pbnd[fi - S->nIF] = bc->p_value;
            else
                pbnd[fi - S->nIF] = pc[m->owner[fi]];
        }
    }
}
static void apply_k_bc(const Solver *S, Fields *f) {
    const btm_mesh *m = S->m;
    for (int p = 0; p < S->nP; ++p) {
        const btm_patch_bc *bc = &S->bcs[p];
        for (int q = m->patch_offset[p], j = 0; q < m->patch_offset[p + 1]; ++q, ++j) {
            int fi = m->patch_faces[q], b = fi - S->nIF;
            switch (bc->k_type) {
                case BTM_BC_WALL_KOMEGA: f->kb[b] = 0.0; break;
                case BTM_BC_DIRICHLET: f->kb[b] = bc->k_profile ? bc->k_profile[j] : bc->k_value; break;
                default: f->kb[b] = f->k[m->owner[fi]]; break;
            }
        }
    }
}
static void apply_omega_bc(const Solver *S, Fields *f, double beta1) {
    const btm_mesh *m = S->m;
    for (int p = 0; p < S->nP; ++p) {
        const btm_patch_bc *bc = &S->bcs[p];
        for (int q = m->patch_offset[p], j = 0; q < m->patch_offset[p + 1]; ++q, ++j) {
            int fi = m->patch_faces[q], b = fi - S->nIF;
            switch (bc->omega_type) {
                case BTM_BC_WALL_KOMEGA: {
                    double y1 = smax(m->face_delta[fi], 1e-20);
                    f->omb[b] = 60.0 * S->nu / (beta1 * y1 * y1);
                    break;
                }
                case BTM_BC_DIRICHLET: f->omb[b] = bc->omega_profile ? bc->omega_profile[j] : bc->omega_value; break;
                default: f->omb[b] = f->om[m->owner[fi]]; break;
            }
        }
    }
}

/* SIMPLESolver::initUniform (SIMPLESolver.cpp:23-51) */
static void init_uniform(Solver *S, Fields *f, v3 Uinit, double pInit, double kInit, double omInit) {
    int nC = S->nC, nB = S->nB;
    for (int i = 0; i < nC; ++i) {
        f->U[i] = Uinit; f->p[i] = pInit; f->k[i] = kInit; f->om[i] = omInit;
        f->F1[i] = 1.0; f->F2[i] = 1.0; f->Pk[i] = 0.0; f->CDkw[i] = 0.0; f->nuT[i] = 0.0;
    }
    for (int b = 0; b < nB; ++b) { f->Ub[b] = Uinit; f->pb[b] = pInit; f->kb[b] = kInit; f->omb[b] = omInit; }
    f->turbEstablished = 0;
    const double *wd = S->m->wall_distance;
    for (int ci = 0; ci < nC; ++ci) {
        double y = smax(wd[ci], 1e-20);
        double omWall = 60.0 * S->nu / (S->sst.beta1 * y * y);
        f->om[ci] = smax(omWall, omInit);
    }
    for (int ci = 0; ci < nC; ++ci)
        f->nuT[ci] = S->sst.a1 * kInit / smax(S->sst.a1 * f->om[ci], 1e-20);
    /* applyAllBCs: applyOmegaBC with its default beta1 = 0.075 */
    apply_velocity_bc(S, f);
    apply_pressure_bc(S, f->p, f->pb);
    apply_k_bc(S, f);
    apply_omega_bc(S, f, 0.075);
}

/* SSTModel::computeFields (core/src/SSTModel.cpp:122-172); also returns |S| */
static void compute_sst(Solver *S, Fields *f, double *Smag) {
    const btm_mesh *m = S->m;
    int nC = S->nC;
    velocity_gradients(m, f->U, f->Ub, &S->vg, S->tmp, S->tmpb);
    strain_rate(nC, &S->vg, Smag);
    v3 *gk = xcalloc(nC, sizeof(v3)), *gw = xcalloc(nC, sizeof(v3));
    green_gauss(m, f->k, f->kb, gk);
    green_gauss(m, f->om, f->omb, gw);
    for (int ci = 0; ci < nC; ++ci) {
        double kc = smax(f->k[ci], 0.0);
        double wc = smax(f->om[ci], 1e-20);
        double y = smax(m->wall_distance[ci], 1e-20);
        double Sc = Smag[ci];
        double CDkw = crossDiffusion(&S->sst, gk[ci], gw[ci], wc);
        f->CDkw[ci] = CDkw;
        double CDpos = smax(CDkw, 1e-20);
        f->F1[ci] = (S->sst.variant == BTM_SST_KOMEGA) ? 1.0 : computeF1(&S->sst, kc, wc, y, S->nu, CDpos);
        f->F2[ci] = computeF2(&S->sst, kc, wc, y, S->nu);
        f->nuT[ci] = eddyViscosity(&S->sst, kc, wc, Sc, f->F2[ci]);
        f->Pk[ci] = production(&S->sst, f->nuT[ci], Sc, kc, wc);
    }
    free(gk); free(gw);
}

static void sys_zero(Lsys *A) {
    memset(A->diag, 0, sizeof(double) * A->nC);
    memset(A->source, 0, sizeof(double) * A->nC);
    memset(A->upper, 0, sizeof(double) * A->nIF);
    memset(A->lower, 0, sizeof(double) * A->nIF);
}

/* transposeStressSource with zero wall coefficient (core/include/StressOperators.hpp:312-365) */
static void transpose_stress(Solver *S, const Fields *f, int comp, double *src) {
    const btm_mesh *m = S->m;
    velocity_gradients(m, f->U, f->Ub, &S->vg, S->tmp, S->tmpb);
    const VelGrad *vg = &S->vg;
#define GCOL(ci) (comp == 0 ? mk(vg->dudx[ci].x, vg->dvdx[ci].x, vg->dwdx[ci].x) \
                : comp == 1 ? mk(vg->dudx[ci].y, vg->dvdx[ci].y, vg->dwdx[ci].y)   \
                            : mk(vg->dudx[ci].z, vg->dvdx[ci].z, vg->dwdx[ci].z))
    for (int c = 0; c < S->nC; ++c) src[c] = 0.0;
    for (int fi = 0; fi < S->nIF; ++fi) {
        int o = m->owner[fi], n = m->neighbour[fi];
        double w = m->face_weight[fi];
        double cf = w * f->nuT[o] + (1.0 - w) * f->nuT[n];
        v3 g = vadd(vmul(GCOL(o), w), vmul(GCOL(n), 1.0 - w));
        double flux = cf * vdot(g, fnormal(m, fi)) * m->face_area[fi];
        src[o] += flux;
        src[n] -= flux;
    }
    for (int p = 0; p < S->nP; ++p) {
        int isWall = m->patch_type[p] == BTM_PATCH_WALL;
        for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) {
            int fi = m->patch_faces[q], o = m->owner[fi];
            double cf = isWall ? 0.0 : f->nuT[o];
            double flux = cf * vdot(GCOL(o), fnormal(m, fi)) * m->face_area[fi];
            src[o] += flux;
        }
    }
#undef GCOL
}

/* SIMPLESolver::addInjectionSource (SIMPLESolver.cpp:224-315): on the x pass
 * the deferred-correction tensor D = 2 k b + 2 nuT dev(S) per cell, the force
 * q = -sum_f (D_f . n_f) A_f (internal faces in face order, then boundary
 * faces with the owner value) and its blend at injRelax; every pass adds the
 * blend's component to the source. */
static v3 ddotn(const double *d, v3 n) {
    return mk(d[0] * n.x + d[3] * n.y + d[4] * n.z, d[3] * n.x + d[1] * n.y + d[5] * n.z,
              d[4] * n.x + d[5] * n.y + d[2] * n.z);
}
static void add_injection(Solver *S, Lsys *sys, const Fields *f, int comp) {
    const btm_mesh *m = S->m;
    int nC = S->nC;
    if (comp == 0) {
        velocity_gradients(m, f->U, f->Ub, &S->vg, S->tmp, S->tmpb);
        double *D = xcalloc(6 * (size_t)nC, 8);
        for (int ci = 0; ci < nC; ++ci) {
            const double S11 = S->vg.dudx[ci].x, S22 = S->vg.dvdx[ci].y, S33 = S->vg.dwdx[ci].z;
            const double S12 = 0.5 * (S->vg.dudx[ci].y + S->vg.dvdx[ci].x);
            const double S13 = 0.5 * (S->vg.dudx[ci].z + S->vg.dwdx[ci].x);
            const double S23 = 0.5 * (S->vg.dvdx[ci].z + S->vg.dwdx[ci].y);
            const double trS3 = (S11 + S22 + S33) / 3.0;
            const double twoK = 2.0 * f->k[ci], twoNu = 2.0 * f->nuT[ci];
            const double *bt = S->bTarget6 + 6 * (size_t)ci;
            D[6 * ci + 0] = twoK * bt[0] + twoNu * (S11 - trS3);
            D[6 * ci + 1] = twoK * bt[1] + twoNu * (S22 - trS3);
            D[6 * ci + 2] = twoK * bt[2] + twoNu * (S33 - trS3);
            D[6 * ci + 3] = twoK * bt[3] + twoNu * S12;
            D[6 * ci + 4] = twoK * bt[4] + twoNu * S13;
            D[6 * ci + 5] = twoK * bt[5] + twoNu * S23;
        }
        v3 *q = xcalloc(nC, sizeof(v3));
        for (int fi = 0; fi < S->nIF; ++fi) {
            int o = m->owner[fi], n = m->neighbour[fi];
            double w = m->face_weight[fi], Df[6];
            for (int c = 0; c < 6; ++c) Df[c] = w * D[6 * o + c] + (1.0 - w) * D[6 * n + c];
            v3 flux = vmul(ddotn(Df, fnormal(m, fi)), m->face_area[fi]);
            q[o] = vsub(q[o], flux);
            q[n] = vadd(q[n], flux);
        }
        for (int fi = S->nIF; fi < S->nF; ++fi) {
            int o = m->owner[fi];
            q[o] = vsub(q[o], vmul(ddotn(D + 6 * o, fnormal(m, fi)), m->face_area[fi]));
        }
        if (!S->injHave || S->injRelax >= 1.0) {
            memcpy(S->injBlend, q, sizeof(v3) * nC);
        } else {
            for (int ci = 0; ci < nC; ++ci)
                S->injBlend[ci] = vadd(vmul(S->injBlend[ci], 1.0 - S->injRelax), vmul(q[ci], S->injRelax));
        }
        S->injHave = 1;
        free(q);
        free(D);
    }
    for (int ci = 0; ci < nC; ++ci) sys->source[ci] += vcomp(S->injBlend[ci], comp);
}

/* SIMPLESolver::assembleMomentum (SIMPLESolver.cpp:56-203) */
static void assemble_momentum(Solver *S, Lsys *sys, const Fields *f, int comp, double *aP) {
    const btm_mesh *m = S->m;
    const btm_settings *st = S->s;
    double nu = S->nu;
    sys_zero(sys);
    for (int fi = 0; fi < S->nIF; ++fi) {
        int o = m->owner[fi], n = m->neighbour[fi];
        double Sf = m->face_area[fi];
        double delta = smax(m->face_delta[fi], 1e-20);
        double w = m->face_weight[fi];
        double nuEff_o = nu + f->nuT[o];
        double nuEff_n = nu + f->nuT[n];
        double nuEff_f = w * nuEff_o + (1.0 - w) * nuEff_n;
        double Df = nuEff_f * Sf / delta;
        v3 Uf = vadd(vmul(f->U[o], w), vmul(f->U[n], 1.0 - w));
        v3 nn = fnormal(m, fi);
        double mFlux = (Uf.x * nn.x + Uf.y * nn.y + Uf.z * nn.z) * Sf;
        double cPos = smax(mFlux, 0.0);
        double cNeg = smax(-mFlux, 0.0);
        sys->diag[o] += Df + cPos;
        sys->diag[n] += Df + cNeg;
        sys->upper[fi] = -(Df + cNeg);
        sys->lower[fi] = -(Df + cPos);
    }
    for (int fi = S->nIF; fi < S->nF; ++fi) {
        int o = m->owner[fi], b = fi - S->nIF;
        double Sf = m->face_area[fi];
        double delta = smax(m->face_delta[fi], 1e-20);
        double nuEff = (S->isWall[fi] && !st->use_wall_functions) ? nu : nu + f->nuT[o];
        double Db = nuEff * Sf / delta;
        double Ub = vcomp(f->Ub[b], comp);
        v3 Ubv = f->Ub[b];
        v3 nn = fnormal(m, fi);
        double mFlux = (Ubv.x * nn.x + Ubv.y * nn.y + Ubv.z * nn.z) * Sf;
        if (mFlux >= 0) {
            sys->diag[o] += mFlux + Db;
            sys->source[o] += Db * Ub;
        } else {
            sys->diag[o] += Db;
            sys->source[o] += (Db - mFlux) * Ub;
        }
    }
    v3 *gradP = S->gradTmp;
    green_gauss(m, f->p, f->pb, gradP);
    for (int ci = 0; ci < S->nC; ++ci) {
        double vol = m->cell_volume[ci];
        double dpdx = vcomp(gradP[ci], comp);
        sys->source[ci] -= dpdx * vol;
    }
    double fb = st->body_force[comp];
    if (fb != 0.0)
        for (int ci = 0; ci < S->nC; ++ci) sys->source[ci] += fb * m->cell_volume[ci];
    double *tsrc = xcalloc(S->nC, 8);
    transpose_stress(S, f, comp, tsrc);
    for (int ci = 0; ci < S->nC; ++ci) sys->source[ci] += tsrc[ci];
    free(tsrc);
    if (S->bTarget6) add_injection(S, sys, f, comp);
    double alphaU = st->alpha_u;
    for (int ci = 0; ci < S->nC; ++ci) {
        double phi_old = vcomp(f->U[ci], comp);
        S->aPunrelaxed[ci] = sys->diag[ci];
        sys->source[ci] += (1.0 - alphaU) / alphaU * sys->diag[ci] * phi_old;
        sys->diag[ci] /= alphaU;
        aP[ci] = sys->diag[ci];
    }
}

static int has_outlet(const Solver *S) {
    const btm_mesh *m = S->m;
    for (int p = 0; p < S->nP; ++p)
        if (m->patch_type[p] == BTM_PATCH_OUTLET && m->patch_offset[p + 1] > m->patch_offset[p]) return 1;
    return 0;
}

/* SIMPLESolver::assemblePressureCorrection (SIMPLESolver.cpp:322-450) */
static void assemble_pressure(Solver *S, Lsys *sys, const Fields *f, const double *aP, double *pPrime,
                              double *pPrimeB) {
    const btm_mesh *m = S->m;
    sys_zero(sys);
    for (int i = 0; i < S->nC; ++i) pPrime[i] = 0.0;
    for (int b = 0; b < S->nB; ++b) pPrimeB[b] = 0.0;
    int hasOut = has_outlet(S);
    int rcActive = !hasOut || S->s->rhie_chow_all_meshes;
    v3 *gradP = S->gradTmp;
    if (rcActive) green_gauss(m, f->p, f->pb, gradP);
    for (int fi = 0; fi < S->nIF; ++fi) {
        int o = m->owner[fi], n = m->neighbour[fi];
        double Sf = m->face_area[fi];
        double delta = smax(m->face_delta[fi], 1e-20);
        double w = m->face_weight[fi];
        double Vo = m->cell_volume[o], Vn = m->cell_volume[n];
        double dP_o = (fabs(aP[o]) > 1e-30) ? Vo / aP[o] : 0.0;
        double dP_n = (fabs(aP[n]) > 1e-30) ? Vn / aP[n] : 0.0;
        double dP_f = w * dP_o + (1.0 - w) * dP_n;
        double coeff = dP_f * Sf / delta;
        sys->diag[o] += coeff;
        sys->diag[n] += coeff;
        sys->upper[fi] = -coeff;
        sys->lower[fi] = -coeff;
        v3 Uf = vadd(vmul(f->U[o], w), vmul(f->U[n], 1.0 - w));
        v3 nn = fnormal(m, fi);
        double massFlux = (Uf.x * nn.x + Uf.y * nn.y + Uf.z * nn.z) * Sf;
        if (rcActive) {
            v3 ehat = vdiv(fdvec(m, fi), smax(m->face_delta[fi], 1e-30));
            v3 gbar = vadd(vmul(gradP[o], w), vmul(gradP[n], 1.0 - w));
            massFlux += -dP_f * Sf * ((f->p[n] - f->p[o]) / delta - vdot(gbar, ehat));
        }
        sys->source[o] -= massFlux;
        sys->source[n] += massFlux;
    }
    for (int p = 0; p < S->nP; ++p) {
        int isOutlet = m->patch_type[p] == BTM_PATCH_OUTLET;
        for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) {
            int fi = m->patch_faces[q], o = m->owner[fi];
            double Sf = m->face_area[fi];
            double delta = smax(m->face_delta[fi], 1e-20);
            v3 Ub = f->Ub[fi - S->nIF];
            v3 nn = fnormal(m, fi);
            double massFlux = (Ub.x * nn.x + Ub.y * nn.y + Ub.z * nn.z) * Sf;
            sys->source[o] -= massFlux;
            if (isOutlet) {
                double Vo = m->cell_volume[o];
                double dP_o = (fabs(aP[o]) > 1e-30) ? Vo / aP[o] : 0.0;
                double coeff = dP_o * Sf / delta;
                sys->diag[o] += coeff;
            }
        }
    }
    if (!hasOut && S->nC > 0) sys->diag[0] += fabs(sys->diag[0]) > 1e-30 ? sys->diag[0] : 1.0;
}

/* SIMPLESolver::assembleKEquation (SIMPLESolver.cpp:483-560) */
static void assemble_k(Solver *S, Lsys *sys, const Fields *f) {
    const btm_mesh *m = S->m;
    double nu = S->nu;
    sys_zero(sys);
    for (int fi = 0; fi < S->nIF; ++fi) {
        int o = m->owner[fi], n = m->neighbour[fi];
        double Sf = m->face_area[fi];
        double delta = smax(m->face_delta[fi], 1e-20);
        double w = m->face_weight[fi];
        double F1_f = w * f->F1[o] + (1.0 - w) * f->F1[n];
        double sk = sigma_k(&S->sst, F1_f);
        double nuEff_o = nu + sk * f->nuT[o];
        double nuEff_n = nu + sk * f->nuT[n];
        double nuEff_f = w * nuEff_o + (1.0 - w) * nuEff_n;
        double Df = nuEff_f * Sf / delta;
        v3 Uf = vadd(vmul(f->U[o], w), vmul(f->U[n], 1.0 - w));
        v3 nn = fnormal(m, fi);
        double mFlux = (Uf.x * nn.x + Uf.y * nn.y + Uf.z * nn.z) * Sf;
        double cPos = smax(mFlux, 0.0), cNeg = smax(-mFlux, 0.0);
        sys->diag[o] += Df + cPos;
        sys->diag[n] += Df + cNeg;
        sys->upper[fi] = -(Df + cNeg);
        sys->lower[fi] = -(Df + cPos);
    }
    for (int fi = S->nIF; fi < S->nF; ++fi) {
        int o = m->owner[fi], b = fi - S->nIF;
        double Sf = m->face_area[fi];
        double delta = smax(m->face_delta[fi], 1e-20);
        double sk = sigma_k(&S->sst, f->F1[o]);
        double nuEff = nu + sk * f->nuT[o];
        double Db = nuEff * Sf / delta;
        double kb = f->kb[b];
        v3 Ub = f->Ub[b];
        v3 nn = fnormal(m, fi);
        double mFlux = (Ub.x * nn.x + Ub.y * nn.y + Ub.z * nn.z) * Sf;
        if (mFlux >= 0) {
            sys->diag[o] += mFlux + Db;
            sys->source[o] += Db * kb;
        } else {
            sys->diag[o] += Db;
            sys->source[o] += (Db - mFlux) * kb;
        }
    }
    for (int ci = 0; ci < S->nC; ++ci) {
        double vol = m->cell_volume[ci];
        sys->source[ci] += f->Pk[ci] * vol;
        double destruction = S->sst.betaStar * smax(f->om[ci], 1e-20);
        sys->diag[ci] += destruction * vol;
    }
    double alphaK = S->s->alpha_k;
    for (int ci = 0; ci < S->nC; ++ci) {
        sys->source[ci] += (1.0 - alphaK) / alphaK * sys->diag[ci] * f->k[ci];
        sys->diag[ci] /= alphaK;
    }
}

/* SIMPLESolver::assembleOmegaEquation (SIMPLESolver.cpp:567-669) */
static void assemble_omega(Solver *S, Lsys *sys, const Fields *f, const double *Smag) {
    const btm_mesh *m = S->m;
    double nu = S->nu;
    sys_zero(sys);
    for (int fi = 0; fi < S->nIF; ++fi) {
        int o = m->owner[fi], n = m->neighbour[fi];
        double Sf = m->face_area[fi];
        double delta = smax(m->face_delta[fi], 1e-20);
        double w = m->face_weight[fi];
        double F1_f = w * f->F1[o] + (1.0 - w) * f->F1[n];
        double sw = sigma_w(&S->sst, F1_f);
        double nuEff_o = nu + sw * f->nuT[o];
        double nuEff_n = nu + sw * f->nuT[n];
        double nuEff_f = w * nuEff_o + (1.0 - w) * nuEff_n;
        double Df = nuEff_f * Sf / delta;
        v3 Uf = vadd(vmul(f->U[o], w), vmul(f->U[n], 1.0 - w));
        v3 nn = fnormal(m, fi);
        double mFlux = (Uf.x * nn.x + Uf.y * nn.y + Uf.z * nn.z) * Sf;
        double cPos = smax(mFlux, 0.0), cNeg = smax(-mFlux, 0.0);
        sys->diag[o] += Df + cPos;
        sys->diag[n] += Df + cNeg;
        sys->upper[fi] = -(Df + cNeg);
        sys->lower[fi] = -(Df + cPos);
    }
    for (int fi = S->nIF; fi < S->nF; ++fi) {
        int o = m->owner[fi], b = fi - S->nIF;
        double Sf = m->face_area[fi];
        double delta = smax(m->face_delta[fi], 1e-20);
        double sw = sigma_w(&S->sst, f->F1[o]);
        double nuEff = nu + sw * f->nuT[o];
        double Db = nuEff * Sf / delta;
        double wb = f->omb[b];
        v3 Ub = f->Ub[b];
        v3 nn = fnormal(m, fi);
        double mFlux = (Ub.x * nn.x + Ub.y * nn.y + Ub.z * nn.z) * Sf;
        if (mFlux >= 0) {
            sys->diag[o] += mFlux + Db;
            sys->source[o] += Db * wb;
        } else {
            sys->diag[o] += Db;
            sys->source[o] += (Db - mFlux) * wb;
        }
    }
    for (int ci = 0; ci < S->nC; ++ci) {
        double vol = m->cell_volume[ci];
        double F1 = f->F1[ci];
        double omC = smax(f->om[ci], 1e-20);
        double alphaB = alpha_b(&S->sst, F1);
        double Sc = Smag[ci];
        sys->source[ci] += alphaB * productionOmega(&S->sst, f->nuT[ci], Sc, f->k[ci], f->om[ci]) * vol;
        double betaB = beta_b(&S->sst, F1);
        sys->diag[ci] += betaB * omC * vol;
        sys->source[ci] += (1.0 - F1) * f->CDkw[ci] * vol;
    }
    double alphaW = S->s->alpha_omega;
    for (int ci = 0; ci < S->nC; ++ci) {
        sys->source[ci] += (1.0 - alphaW) / alphaW * sys->diag[ci] * f->om[ci];
        sys->diag[ci] /= alphaW;
    }
}

static Lsys make_sys(const Solver *S) {
    Lsys A;
    A.nC = S->nC; A.nIF = S->nIF;
    A.diag = xcalloc(S->nC, 8); A.source = xcalloc(S->nC, 8);
    A.upper = xcalloc(S->nIF, 8); A.lower = xcalloc(S->nIF, 8);
    A.own = S->m->owner; A.nbr = S->m->neighbour;
    return A;
}
static void free_sys(Lsys *A) { free(A->diag); free(A->source); free(A->upper); free(A->lower); }

static inline double clampd(double v, double lo, double hi) { return smax(lo, smin(hi, v)); }

/* SIMPLESolver::solve (SIMPLESolver.cpp:696-1043) */
static void simple_solve(Solver *S, Fields *f, btm_history *hist) {
    const btm_mesh *m = S->m;
    const btm_settings *st = S->s;
    int nC = S->nC, nB = S->nB;
    Lsys momSys = make_sys(S), pSys = make_sys(S), kSys = make_sys(S), omSys = make_sys(S);
    double *pPrime = xcalloc(nC, 8), *pPrimeB = xcalloc(nB > 0 ? nB : 1, 8);
    double *SmagFrozen = xcalloc(nC, 8);
    double *aPstore = xcalloc(nC, 8), *vec = xcalloc(nC, 8);
    double *kOld = xcalloc(nC, 8), *omOld = xcalloc(nC, 8);
    v3 *gradPp = xcalloc(nC, sizeof(v3));
    double lastKChange = 1.0, lastOmChange = 1.0;
    double normUx0 = 1, normUy0 = 1, normP0 = 1;
    int converged = 0, diverged = 0, finalIter = st->max_iterations, ran = 0;
    double lastEntry[6] = {0, 0, 0, 0, 0, 0};
    S->innerIters = 0;

    for (int iter = 0; iter < st->max_iterations; ++iter) {
        ran = iter + 1;
        int turbActive = iter >= st->turb_start_iter;
        int turbUpdate = turbActive && ((iter - st->turb_start_iter) % st->turb_update_interval == 0);
        if (turbUpdate) {
            compute_sst(S, f, SmagFrozen);
            if (!f->turbEstablished && iter >= st->turb_start_iter + st->nut_floor_iters)
                f->turbEstablished = 1;
            double nuTMin = f->turbEstablished ? 0.0 : 0.1 * S->nu;
            for (int ci = 0; ci < nC; ++ci) f->nuT[ci] = smax(f->nuT[ci], nuTMin);
        }
        SolverResult resU[3];
        for (int comp = 0; comp < 3; ++comp) {
            assemble_momentum(S, &momSys, f, comp, S->aP);
            for (int ci = 0; ci < nC; ++ci) vec[ci] = vcomp(f->U[ci], comp);
            resU[comp] = linear_solve(st->momentum_solver, &momSys, vec, st->inner_iterations, st->inner_tolerance);
            S->innerIters += resU[comp].iterations;
            for (int ci = 0; ci < nC; ++ci) {
                if (comp == 0) f->U[ci].x = vec[ci];
                else if (comp == 1) f->U[ci].y = vec[ci];
                else f->U[ci].z = vec[ci];
            }
            if (comp == 0) memcpy(aPstore, S->aP, sizeof(double) * nC);
        }
        apply_velocity_bc(S, f);

        assemble_pressure(S, &pSys, f, aPstore, pPrime, pPrimeB);
        for (int ci = 0; ci < nC; ++ci) vec[ci] = 0.0;
        SolverResult resP = linear_solve(st->pressure_solver, &pSys, vec, st->inner_iterations, st->inner_tolerance);
        S->innerIters += resP.iterations;
        for (int ci = 0; ci < nC; ++ci) pPrime[ci] = vec[ci];
        for (int p = 0; p < S->nP; ++p) {
            if (m->patch_type[p] == BTM_PATCH_OUTLET) continue;
            for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) {
                int fi = m->patch_faces[q];
                pPrimeB[fi - S->nIF] = pPrime[m->owner[fi]];
            }
        }
        /* correctVelocity / correctPressure (SIMPLESolver.cpp:456-475) */
        green_gauss(m, pPrime, pPrimeB, gradPp);
        for (int ci = 0; ci < nC; ++ci) {
            double rAP = (fabs(aPstore[ci]) > 1e-30) ? 1.0 / aPstore[ci] : 0.0;
            double vol = m->cell_volume[ci];
            f->U[ci].x -= rAP * gradPp[ci].x * vol;
            f->U[ci].y -= rAP * gradPp[ci].y * vol;
            f->U[ci].z -= rAP * gradPp[ci].z * vol;
        }
        apply_velocity_bc(S, f);
        for (int ci = 0; ci < nC; ++ci) f->p[ci] += st->alpha_p * pPrime[ci];
        apply_pressure_bc(S, f->p, f->pb);

        SolverResult resK = {0, 0, 0, 0}, resOm = {0, 0, 0, 0};
        if (turbUpdate) {
            memcpy(kOld, f->k, sizeof(double) * nC);
            memcpy(omOld, f->om, sizeof(double) * nC);
            assemble_k(S, &kSys, f);
            memcpy(vec, f->k, sizeof(double) * nC);
            resK = linear_solve(st->turbulence_solver, &kSys, vec, st->inner_iterations, st->inner_tolerance);
            S->innerIters += resK.iterations;
            memcpy(f->k, vec, sizeof(double) * nC);
            for (int ci = 0; ci < nC; ++ci) f->k[ci] = clampd(f->k[ci], st->k_min, st->k_max);
            for (int b = 0; b < nB; ++b) f->kb[b] = clampd(f->kb[b], st->k_min, st->k_max);
            apply_k_bc(S, f);

            assemble_omega(S, &omSys, f, SmagFrozen);
            memcpy(vec, f->om, sizeof(double) * nC);
            resOm = linear_solve(st->turbulence_solver, &omSys, vec, st->inner_iterations, st->inner_tolerance);
            S->innerIters += resOm.iterations;
            memcpy(f->om, vec, sizeof(double) * nC);
            for (int ci = 0; ci < nC; ++ci) f->om[ci] = clampd(f->om[ci], st->omega_min, 1e15);
            for (int b = 0; b < nB; ++b) f->omb[b] = clampd(f->omb[b], st->omega_min, 1e15);
            apply_omega_bc(S, f, S->sst.beta1);

            double betaStar = S->sst.betaStar, kappa = st->von_karman;
            for (int p = 0; p < S->nP; ++p) {
                if (m->patch_type[p] != BTM_PATCH_WALL) continue;
                for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) {
                    int fi = m->patch_faces[q], o = m->owner[fi];
                    double y1 = smax(m->face_delta[fi], 1e-20);
                    double omRes = 60.0 * S->nu / (S->sst.beta1 * y1 * y1);
                    if (st->use_wall_functions) {
                        double k_p = smax(f->k[o], 1e-30);
                        double uTau = sqrt(sqrt(betaStar) * k_p);
                        double omLog = uTau / (sqrt(betaStar) * kappa * y1);
                        f->om[o] = sqrt(omRes * omRes + omLog * omLog);
                    } else {
                        f->om[o] = omRes;
                    }
                }
            }
            double kMaxVal = 1e-30, omMaxVal = 1e-30, kMaxDiff = 0.0, omMaxDiff = 0.0;
            for (int ci = 0; ci < nC; ++ci) {
                kMaxVal = smax(kMaxVal, fabs(f->k[ci]));
                omMaxVal = smax(omMaxVal, fabs(f->om[ci]));
                kMaxDiff = smax(kMaxDiff, fabs(f->k[ci] - kOld[ci]));
                omMaxDiff = smax(omMaxDiff, fabs(f->om[ci] - omOld[ci]));
            }
            lastKChange = kMaxDiff / kMaxVal;
            lastOmChange = omMaxDiff / omMaxVal;
        }

        double eUx = resU[0].initialRes, eUy = resU[1].initialRes, eUz = resU[2].initialRes;
        double eP = resP.initialRes;
        double eK = turbActive ? lastKChange : 0.0, eOm = turbActive ? lastOmChange : 0.0;
        lastEntry[0] = eUx; lastEntry[1] = eUy; lastEntry[2] = eUz;
        lastEntry[3] = eP; lastEntry[4] = eK; lastEntry[5] = eOm;
        if (hist && hist->residuals && iter < hist->residual_capacity)
            memcpy(hist->residuals + 6 * iter, lastEntry, sizeof lastEntry);
        if (iter == 0) {
            normUx0 = smax(eUx, 1e-30);
            normUy0 = smax(eUy, 1e-30);
            normP0 = smax(eP, 1e-30);
        } else if (iter < 50) {
            normP0 = smax(normP0, eP);
        }
        double normMom0 = smax(normUx0, normUy0);
        double nUx = normMom0 < 1e-20 ? 0.0 : eUx / normMom0;
        double nUy = normMom0 < 1e-20 ? 0.0 : eUy / normMom0;
        double nP = normP0 < 1e-20 ? 0.0 : eP / normP0;
        double maxRes = smax(smax(nUx, nUy), nP);  /* std::max({a,b,c}) */
        if (turbActive) maxRes = smax(smax(maxRes, lastKChange), lastOmChange);
        if (!isfinite(eUx) || !isfinite(eUy) || !isfinite(eUz) || !isfinite(eP) || !isfinite(eK) ||
            !isfinite(eOm) || !isfinite(lastKChange) || !isfinite(lastOmChange))
            maxRes = INFINITY;
        int turbScheduled = st->turb_start_iter < st->max_iterations;
        if (maxRes < st->convergence_tol && iter > 0 && (!turbScheduled || (turbActive && f->turbEstablished))) {
            converged = 1;
            finalIter = iter;
            break;
        }
        if (isnan(maxRes) || isinf(maxRes) || maxRes > st->divergence_limit) {
            diverged = 1;
            finalIter = iter;
            break;
        }
    }
    if (hist) {
        hist->converged = converged;
        hist->diverged = diverged;
        hist->final_iter = finalIter;
        hist->iterations_run = ran;
        hist->inner_iterations = S->innerIters;
        hist->status = diverged ? BTM_DIVERGED : (converged ? BTM_CONVERGED : BTM_UNCONVERGED);
        memcpy(hist->last_residual, lastEntry, sizeof lastEntry);
    }
    free_sys(&momSys); free_sys(&pSys); free_sys(&kSys); free_sys(&omSys);
    free(pPrime); free(pPrimeB); free(SmagFrozen); free(aPstore); free(vec); free(kOld); free(omOld);
    free(gradPp);
}

/* ------------------------------------------------------------------------ */
/* state marshalling and the exported functions                              */
/* ------------------------------------------------------------------------ */
static void state_in(Fields *f, const btm_state *w, int nC, int nB) {
    for (int i = 0; i < nC; ++i) f->U[i] = mk(w->U[3 * i], w->U[3 * i + 1], w->U[3 * i + 2]);
    for (int b = 0; b < nB; ++b) f->Ub[b] = mk(w->Ub[3 * b], w->Ub[3 * b + 1], w->Ub[3 * b + 2]);
    memcpy(f->p, w->p, 8 * (size_t)nC); memcpy(f->pb, w->pb, 8 * (size_t)nB);
    memcpy(f->k, w->k, 8 * (size_t)nC); memcpy(f->kb, w->kb, 8 * (size_t)nB);
    memcpy(f->om, w->omega, 8 * (size_t)nC); memcpy(f->omb, w->omegab, 8 * (size_t)nB);
    if (w->nuT) memcpy(f->nuT, w->nuT, 8 * (size_t)nC);
    if (w->F1) memcpy(f->F1, w->F1, 8 * (size_t)nC);
    if (w->F2) memcpy(f->F2, w->F2, 8 * (size_t)nC);
    if (w->Pk) memcpy(f->Pk, w->Pk, 8 * (size_t)nC);
    if (w->CDkw) memcpy(f->CDkw, w->CDkw, 8 * (size_t)nC);
    f->turbEstablished = w->turb_established;
}
static void state_out(const Fields *f, btm_state *o, int nC, int nB) {
    if (o->U) for (int i = 0; i < nC; ++i) { o->U[3*i] = f->U[i].x; o->U[3*i+1] = f->U[i].y; o->U[3*i+2] = f->U[i].z; }
    if (o->Ub) for (int b = 0; b < nB; ++b) { o->Ub[3*b] = f->Ub[b].x; o->Ub[3*b+1] = f->Ub[b].y; o->Ub[3*b+2] = f->Ub[b].z; }
#define CP(dst, src, n) if (dst) memcpy(dst, src, 8 * (size_t)(n))
    CP(o->p, f->p, nC); CP(o->pb, f->pb, nB); CP(o->k, f->k, nC); CP(o->kb, f->kb, nB);
    CP(o->omega, f->om, nC); CP(o->omegab, f->omb, nB); CP(o->nuT, f->nuT, nC);
    CP(o->F1, f->F1, nC); CP(o->F2, f->F2, nC); CP(o->Pk, f->Pk, nC); CP(o->CDkw, f->CDkw, nC);
#undef CP
    o->turb_established = f->turbEstablished;
}

int oracle_solve(const btm_mesh *m, const btm_patch_bc *bcs, double nu, const btm_settings *s,
                 const double *coeffs, int variant, const btm_init *init, btm_state *out,
                 btm_history *hist) {
    Solver S;
    solver_init(&S, m, bcs, nu, s, coeffs, variant);
    if (g_bTarget6) {
        /* SIMPLESolver::solve clears the blend and takes alphaInjection (:706-709) */
        S.bTarget6 = g_bTarget6;
        S.injBlend = xcalloc(S.nC, sizeof(v3));
        S.injHave = 0;
        S.injRelax = s->alpha_injection;
    }
    Fields f;
    fields_alloc(&f, S.nC, S.nB > 0 ? S.nB : 1);
    if (init->mode == 0)
        init_uniform(&S, &f, mk(init->u[0], init->u[1], init->u[2]), init->p, init->k, init->omega);
    else
        state_in(&f, init->warm, S.nC, S.nB);
    simple_solve(&S, &f, hist);
    if (out) state_out(&f, out, S.nC, S.nB);
    fields_free(&f);
    solver_free(&S);
    return 0;
}

/* applyVelocityBC / applyPressureBC / applyKBC / applyOmegaBC
 * (core/include/BoundaryCondition.hpp:196-342) on a state: boundary values
 * from the cell values and the patch conditions, default SST coefficients
 * (beta1 of the omega wall value). */
void oracle_apply_bcs(const btm_mesh *m, const btm_patch_bc *bcs, double nu, btm_state *st) {
    btm_settings s;
    memset(&s, 0, sizeof s);
    const double cf[11] = {0.85, 0.5, 0.075, 5.0 / 9.0, 1.0, 0.856, 0.0828, 0.44, 0.09, 0.31, 0.41};
    Solver S;
    solver_init(&S, m, bcs, nu, &s, cf, 0);
    Fields f;
    fields_alloc(&f, S.nC, S.nB > 0 ? S.nB : 1);
    state_in(&f, st, S.nC, S.nB);
    apply_velocity_bc(&S, &f);
    apply_pressure_bc(&S, f.p, f.pb);
    apply_k_bc(&S, &f);
    apply_omega_bc(&S, &f, S.sst.beta1);
    state_out(&f, st, S.nC, S.nB);
    fields_free(&f);
    solver_free(&S);
}

/* transposeStressSource with zero wall coefficient (StressOperators.hpp:312-365)
 * for a coefficient field and a velocity with boundary values: src[n_cells]. */
void oracle_transpose_stress(const btm_mesh *m, const double *coeff, const double *U, const double *Ub, int comp,
                             double *src) {
    btm_settings s;
    memset(&s, 0, sizeof s);
    const double cf[11] = {0.85, 0.5, 0.075, 5.0 / 9.0, 1.0, 0.856, 0.0828, 0.44, 0.09, 0.31, 0.41};
    Solver S;
    solver_init(&S, m, NULL, 1.0, &s, cf, 0);
    Fields f;
    fields_alloc(&f, S.nC, S.nB > 0 ? S.nB : 1);
    for (int c = 0; c < S.nC; ++c) {
        f.U[c] = mk(U[3 * c], U[3 * c + 1], U[3 * c + 2]);
        f.nuT[c] = coeff[c];
    }
    for (int b = 0; b < S.nB; ++b) f.Ub[b] = mk(Ub[3 * b], Ub[3 * b + 1], Ub[3 * b + 2]);
    transpose_stress(&S, &f, comp, src);
    fields_free(&f);
    solver_free(&S);
}

void oracle_green_gauss(const btm_mesh *m, const double *phi, const double *phib, double *grad) {
    v3 *g = xcalloc(m->n_cells, sizeof(v3));
    green_gauss(m, phi, phib, g);
    for (int i = 0; i < m->n_cells; ++i) { grad[3*i] = g[i].x; grad[3*i+1] = g[i].y; grad[3*i+2] = g[i].z; }
    free(g);
}

void oracle_sst_fields(const btm_mesh *m, const double *coeffs, int variant, double nu,
                       const double *U, const double *Ub, const double *k, const double *kb,
                       const double *om, const double *omb, double *nuT, double *F1, double *F2,
                       double *Pk, double *CDkw, double *Smag) {
    btm_settings dummy;
    memset(&dummy, 0, sizeof dummy);
    Solver S;
    solver_init(&S, m, NULL, nu, &dummy, coeffs, variant);
    Fields f;
    int nB = S.nB > 0 ? S.nB : 1;
    fields_alloc(&f, S.nC, nB);
    for (int i = 0; i < S.nC; ++i) f.U[i] = mk(U[3*i], U[3*i+1], U[3*i+2]);
    for (int b = 0; b < S.nB; ++b) f.Ub[b] = mk(Ub[3*b], Ub[3*b+1], Ub[3*b+2]);
    memcpy(f.k, k, 8 * (size_t)S.nC); memcpy(f.kb, kb, 8 * (size_t)S.nB);
    memcpy(f.om, om, 8 * (size_t)S.nC); memcpy(f.omb, omb, 8 * (size_t)S.nB);
    compute_sst(&S, &f, Smag);
    memcpy(nuT, f.nuT, 8 * (size_t)S.nC); memcpy(F1, f.F1, 8 * (size_t)S.nC);
    memcpy(F2, f.F2, 8 * (size_t)S.nC); memcpy(Pk, f.Pk, 8 * (size_t)S.nC);
    memcpy(CDkw, f.CDkw, 8 * (size_t)S.nC);
    fields_free(&f);
    solver_free(&S);
}

void oracle_assemble(const btm_mesh *m, const btm_patch_bc *bcs, double nu,
                     const btm_settings *s, const double *coeffs, int kind,
                     const btm_state *st, const double *aP, const double *Smag,
                     double *diag, double *upper, double *lower, double *source, double *aP_out) {
    Solver S;
    solver_init(&S, m, bcs, nu, s, coeffs, BTM_SST_FULL);
    Fields f;
    fields_alloc(&f, S.nC, S.nB > 0 ? S.nB : 1);
    state_in(&f, st, S.nC, S.nB);
    Lsys A = make_sys(&S);
    if (kind <= 2) {
        assemble_momentum(&S, &A, &f, kind, S.aP);
        if (aP_out) memcpy(aP_out, S.aP, 8 * (size_t)S.nC);
    } else if (kind == 3) {
        double *pp = xcalloc(S.nC, 8), *ppb = xcalloc(S.nB > 0 ? S.nB : 1, 8);
        assemble_pressure(&S, &A, &f, aP, pp, ppb);
        free(pp); free(ppb);
    } else if (kind == 4) {
        assemble_k(&S, &A, &f);
    } else {
        assemble_omega(&S, &A, &f, Smag);
    }
    memcpy(diag, A.diag, 8 * (size_t)S.nC);
    memcpy(source, A.source, 8 * (size_t)S.nC);
    memcpy(upper, A.upper, 8 * (size_t)S.nIF);
    memcpy(lower, A.lower, 8 * (size_t)S.nIF);
    free_sys(&A);
    fields_free(&f);
    solver_free(&S);
}

void oracle_matvec(int nC, int nIF, const int *own, const int *nbr, const double *diag,
                   const double *upper, const double *lower, const double *x, double *y) {
    Lsys A;
    A.nC = nC; A.nIF = nIF; A.own = own; A.nbr = nbr;
    A.diag = (double *)diag; A.upper = (double *)upper; A.lower = (double *)lower; A.source = NULL;
    matvec(&A, x, y);
}

void oracle_linear_solve(int kind, int nC, int nIF, const int *own, const int *nbr,
                         const double *diag, const double *upper, const double *lower,
                         const double *source, double *x, int max_iter, double tol, double *res) {
    Lsys A;
    A.nC = nC; A.nIF = nIF; A.own = own; A.nbr = nbr;
    A.diag = (double *)diag; A.upper = (double *)upper; A.lower = (double *)lower;
    A.source = (double *)source;
    SolverResult r = linear_solve(kind, &A, x, max_iter, tol);
    res[0] = r.iterations; res[1] = r.finalRes; res[2] = r.initialRes; res[3] = r.converged;
}
