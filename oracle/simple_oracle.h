/*
 * simple_oracle.h - plain-C restatement of the reference incompressible
 * SIMPLE / SST k-omega solver (TEST INFRASTRUCTURE ONLY: the checker for the
 * GB300 kernels; never linked into the product).
 *
 * Inputs and outputs use the structs of include/btm_gb300.h.  Every function
 * follows the reference operation order so that, with floating-point
 * contraction disabled, results are bit-identical to the reference build.
 */
#ifndef SIMPLE_ORACLE_H
#define SIMPLE_ORACLE_H

#include "../include/btm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Full solve: SIMPLESolver::initUniform (or warm state) + SIMPLESolver::solve
 * (incompressible/src/SIMPLESolver.cpp:23-51, 696-1043).  Returns 0. */
int oracle_solve(const btm_mesh *m, const btm_patch_bc *bcs, double nu, const btm_settings *s,
                 const double *coeffs, int variant, const btm_init *init, btm_state *out,
                 btm_history *hist);

/* Target anisotropy [6*n_cells] (xx yy zz xy xz yz) for the following
 * oracle_solve calls (SIMPLESolver::setTargetAnisotropy, SIMPLESolver.hpp:89);
 * NULL switches the injection source off.  The array must outlive the calls. */
void oracle_set_target_anisotropy(const double *b6);

/* The four apply*BC functions (core/include/BoundaryCondition.hpp:196-342) on
 * a state's cell values: fills its boundary values (default SST beta1). */
void oracle_apply_bcs(const btm_mesh *m, const btm_patch_bc *bcs, double nu, btm_state *st);

/* transposeStressSource with zero wall coefficient
 * (core/include/StressOperators.hpp:312-365): src is n_cells. */
void oracle_transpose_stress(const btm_mesh *m, const double *coeff, const double *U, const double *Ub, int comp,
                             double *src);

/* greenGaussGrad (core/include/Field.hpp:122-152): grad is n_cells*3. */
void oracle_green_gauss(const btm_mesh *m, const double *phi, const double *phib, double *grad);

/* SSTModel::computeFields + strainRateMagnitude (core/src/SSTModel.cpp:122-172,
 * core/include/Field.hpp:232-267).  U/Ub are xyz-interleaved. */
void oracle_sst_fields(const btm_mesh *m, const double *coeffs, int variant, double nu,
                       const double *U, const double *Ub, const double *k, const double *kb,
                       const double *om, const double *omb, double *nuT, double *F1, double *F2,
                       double *Pk, double *CDkw, double *Smag);

/* Assembly of one linear system from a state.  kind: 0/1/2 = momentum
 * component x/y/z (SIMPLESolver.cpp:56-203), 3 = pressure correction with
 * aP taken from `aP` (:322-450), 4 = k (:483-560), 5 = omega with frozen
 * Smag (:567-669).  Outputs diag/source [n_cells], upper/lower [n_internal];
 * for momentum also aP_out [n_cells] (relaxed diagonal). */
void oracle_assemble(const btm_mesh *m, const btm_patch_bc *bcs, double nu,
                     const btm_settings *s, const double *coeffs, int kind,
                     const btm_state *st, const double *aP, const double *Smag,
                     double *diag, double *upper, double *lower, double *source, double *aP_out);

/* AMGSolver::setup's coarsening (LinearSolver.hpp:516-551) on a CSR matrix:
 * level sizes and the concatenated aggregation maps; returns the level count. */
int oracle_amg_levels(int n, const int *rowPtr, const int *colIdx, const double *values, int max_levels,
                      int *sizes, int *maps);

/* SSTModel point functions (core/src/SSTModel.cpp:9-96): which = 0
 * production, 1 productionOmega, 2 F1, 3 F2, 4 eddy viscosity; arguments as
 * the reference functions take them. */
double oracle_sst_point(const double *coeffs, int variant, int which, const double *args);

/* LinearSystem::matvec (core/include/LinearSolver.hpp:68-77). */
void oracle_matvec(int nC, int nIF, const int *own, const int *nbr, const double *diag,
                   const double *upper, const double *lower, const double *x, double *y);

/* ILinearSolver::solve for solver code BTM_LS_*; res[0..3] = iterations,
 * finalRes, initialRes, converged (LinearSolver.hpp:99-111). */
void oracle_linear_solve(int kind, int nC, int nIF, const int *own, const int *nbr,
                         const double *diag, const double *upper, const double *lower,
                         const double *source, double *x, int max_iter, double tol, double *res);

#ifdef __cplusplus
}
#endif
#endif
