// ref_driver.cpp - a thin extern "C" shim over the reference solver, compiled
// together with the reference's own sources (core/src/Mesh.cpp,
// core/src/SSTModel.cpp, incompressible/src/SIMPLESolver.cpp) by
// oracle/Makefile into oracle/_ref/libref_driver.so.
//
// TEST INFRASTRUCTURE ONLY.  It exists so the golden-vector generator and the
// oracle self-tests can run the unmodified reference algorithm on meshes and
// inputs written by this project (MSH1 files, Mesh.cpp:602-713).  Nothing in
// the product links or loads it.
//
// The shim calls only public reference API: Mesh factories/loaders
// (core/include/Mesh.hpp:107-198), FlowBoundaryConditions
// (core/include/BoundaryCondition.hpp:36-190), SIMPLESolver
// (incompressible/include/SIMPLESolver.hpp:18-27), the header-only linear
// solvers (core/include/LinearSolver.hpp:147-656), greenGaussGrad
// (core/include/Field.hpp:122-152), SSTModel::computeFields
// (core/src/SSTModel.cpp:122-172) and the header-only ObservationOperator
// (core/include/ObservationOperator.hpp:46-378).

#include "Mesh.hpp"
#include "Field.hpp"
#include "FlowFields.hpp"
#include "BoundaryCondition.hpp"
#include "LinearSolver.hpp"
#include "SSTModel.hpp"
#include "SIMPLESolver.hpp"
#include "InferenceParameters.hpp"
#include "ObservationOperator.hpp"

#include "../include/btm_gb300.h"

#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace {

std::string g_err;

const char *patchTypeName(int t) {
    switch (t) {
        case BTM_PATCH_WALL: return "wall";
        case BTM_PATCH_INLET: return "inlet";
        case BTM_PATCH_OUTLET: return "outlet";
        case BTM_PATCH_SYMMETRY: return "symmetry";
        default: return "patch";
    }
}

int patchTypeCode(const std::string &s) {
    if (s == "wall") return BTM_PATCH_WALL;
    if (s == "inlet") return BTM_PATCH_INLET;
    if (s == "outlet") return BTM_PATCH_OUTLET;
    if (s == "symmetry") return BTM_PATCH_SYMMETRY;
    return BTM_PATCH_OTHER;
}

const char *solverName(int code) {
    switch (code) {
        case BTM_LS_PCG: return "PCG";
        case BTM_LS_BICGSTAB: return "BiCGSTAB";
        case BTM_LS_GAUSSSEIDEL: return "GaussSeidel";
        case BTM_LS_AMG: return "AMG";
    }
    return "BiCGSTAB";
}

SolverSettings toSettings(const btm_settings *s, int variant, int verbose) {
    SolverSettings o;
    o.maxIterations = s->max_iterations;
    o.convergenceTol = s->convergence_tol;
    o.divergenceLimit = s->divergence_limit;
    o.alphaU = s->alpha_u;
    o.alphaP = s->alpha_p;
    o.alphaK = s->alpha_k;
    o.alphaOmega = s->alpha_omega;
    o.innerIterations = s->inner_iterations;
    o.innerTolerance = s->inner_tolerance;
    o.turbStartIter = s->turb_start_iter;
    o.turbUpdateInterval = s->turb_update_interval;
    o.nuTFloorIters = s->nut_floor_iters;
    o.rhieChowAllMeshes = s->rhie_chow_all_meshes != 0;
    o.bodyForce = Vec3(s->body_force[0], s->body_force[1], s->body_force[2]);
    o.kMin = s->k_min;
    o.kMax = s->k_max;
    o.omegaMin = s->omega_min;
    o.useWallFunctions = s->use_wall_functions != 0;
    o.vonKarman = s->von_karman;
    o.wallFnE = s->wall_fn_E;
    o.pressureSolver = solverName(s->pressure_solver);
    o.momentumSolver = solverName(s->momentum_solver);
    o.turbulenceSolver = solverName(s->turbulence_solver);
    o.alphaInjection = s->alpha_injection;
    o.sstVariant = variant;
    o.verbose = verbose != 0;
    o.reportInterval = 1000;
    return o;
}

FlowBoundaryConditions toBCs(const Mesh &m, const btm_patch_bc *bcs) {
    FlowBoundaryConditions bc;
    int np = m.nPatches();
    bc.velocityBC.resize(np);
    bc.pressureBC.resize(np);
    bc.kBC.resize(np);
    bc.omegaBC.resize(np);
    for (int p = 0; p < np; ++p) {
        const btm_patch_bc &b = bcs[p];
        const Patch &pat = m.patch(p);
        size_t nf = pat.faces.size();
        PatchBC u, pp, k, w;
        u.type = static_cast<BCType>(b.u_type);
        u.vecValue = Vec3(b.u_value[0], b.u_value[1], b.u_value[2]);
        u.patchName = pat.name;
        if (b.u_profile) {
            u.vecProfile.resize(nf);
            for (size_t i = 0; i < nf; ++i)
                u.vecProfile[i] = Vec3(b.u_profile[3 * i], b.u_profile[3 * i + 1], b.u_profile[3 * i + 2]);
        }
        pp.type = static_cast<BCType>(b.p_type);
        pp.value = b.p_value;
        pp.patchName = pat.name;
        k.type = static_cast<BCType>(b.k_type);
        k.value = b.k_value;
        k.patchName = pat.name;
        if (b.k_profile) k.scalarProfile.assign(b.k_profile, b.k_profile + nf);
        w.type = static_cast<BCType>(b.omega_type);
        w.value = b.omega_value;
        w.patchName = pat.name;
        if (b.omega_profile) w.scalarProfile.assign(b.omega_profile, b.omega_profile + nf);
        bc.velocityBC[p] = u;
        bc.pressureBC[p] = pp;
        bc.kBC[p] = k;
        bc.omegaBC[p] = w;
    }
    return bc;
}

void scalarIn(ScalarField &f, const double *in, const double *bin) {
    for (int i = 0; i < f.size(); ++i) f[i] = in[i];
    if (bin) for (int i = 0; i < f.nBnd(); ++i) f.bnd(i) = bin[i];
}
void scalarOut(const ScalarField &f, double *out, double *bout) {
    if (out) for (int i = 0; i < f.size(); ++i) out[i] = f[i];
    if (bout) for (int i = 0; i < f.nBnd(); ++i) bout[i] = f.bnd(i);
}
void vecIn(VectorField &f, const double *in, const double *bin) {
    for (int i = 0; i < f.size(); ++i) f[i] = Vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
    if (bin) for (int i = 0; i < f.nBnd(); ++i) f.bnd(i) = Vec3(bin[3 * i], bin[3 * i + 1], bin[3 * i + 2]);
}
void vecOut(const VectorField &f, double *out, double *bout) {
    if (out) for (int i = 0; i < f.size(); ++i) { out[3*i] = f[i].x; out[3*i+1] = f[i].y; out[3*i+2] = f[i].z; }
    if (bout) for (int i = 0; i < f.nBnd(); ++i) { bout[3*i] = f.bnd(i).x; bout[3*i+1] = f.bnd(i).y; bout[3*i+2] = f.bnd(i).z; }
}

}  // namespace

// target anisotropy of the following ref_solve calls (empty: none)
std::vector<double> g_bTarget6;

extern "C" {

void ref_set_target_anisotropy(const double *b6, int n_cells) {
    if (b6) g_bTarget6.assign(b6, b6 + 6 * (size_t)n_cells);
    else g_bTarget6.clear();
}

const char *ref_last_error(void) { return g_err.c_str(); }

void *ref_mesh_load(const char *path) {
    try { return new Mesh(Mesh::loadFromFile(path)); }
    catch (const std::exception &e) { g_err = e.what(); return nullptr; }
}
void *ref_mesh_channel(int nx, int ny, double Lx, double Ly) {
    return new Mesh(Mesh::makeChannel2D(nx, ny, Lx, Ly));
}
void *ref_mesh_channel_re(int nx, int ny, double Lx, double Ly, double Re, double yp) {
    return new Mesh(Mesh::makeChannel2D(nx, ny, Lx, Ly, Re, yp));
}
void *ref_mesh_plate(int nx, int ny, double Lx, double Ly, double Re, double yp) {
    return new Mesh(Mesh::makePlate2D(nx, ny, Lx, Ly, Re, yp));
}
void *ref_mesh_bfs(int nxu, int nxd, int nyu, int nyd, double Lu, double Ld, double hs, double H,
                   double Re, double yp) {
    return new Mesh(Mesh::makeBackwardFacingStep2D(nxu, nxd, nyu, nyd, Lu, Ld, hs, H, Re, yp));
}
void *ref_mesh_curved_periodic(const double *xn, const double *yb, int nnodes, double yTop, int ny,
                               double Re, double yp) {
    try {
        std::vector<double> x(xn, xn + nnodes), y(yb, yb + nnodes);
        return new Mesh(Mesh::makeCurvedChannelPeriodic2D(x, y, yTop, ny, Re, yp));
    } catch (const std::exception &e) { g_err = e.what(); return nullptr; }
}
void ref_mesh_free(void *m) { delete static_cast<Mesh *>(m); }
void ref_mesh_wall_distance(void *m) { static_cast<Mesh *>(m)->computeWallDistance(); }
int ref_mesh_set_patch_type(void *m, const char *name, const char *type) {
    try { static_cast<Mesh *>(m)->setPatchType(name, type); return 0; }
    catch (const std::exception &e) { g_err = e.what(); return -1; }
}
int ref_mesh_save(void *m, const char *path) {
    try { static_cast<Mesh *>(m)->saveBinary(path); return 0; }
    catch (const std::exception &e) { g_err = e.what(); return -1; }
}

// sizes[0..5] = nCells, nFaces, nInternal, nPatches, nNodes, sum(cell faces)
void ref_mesh_sizes(void *mp, int *sizes) {
    const Mesh &m = *static_cast<Mesh *>(mp);
    sizes[0] = m.nCells(); sizes[1] = m.nFaces(); sizes[2] = m.nInternalFaces();
    sizes[3] = m.nPatches(); sizes[4] = m.nNodes();
    int s = 0;
    for (int c = 0; c < m.nCells(); ++c) s += static_cast<int>(m.cell(c).faces.size());
    sizes[5] = s;
}

// Copies every mesh array out; wd may be null if wall distance was not computed.
void ref_mesh_dump(void *mp, int *owner, int *nbr, int *patch_id, double *fc, double *fn,
                   double *fa, double *fdel, double *fd, double *fw, double *cc, double *cv,
                   double *wd, int *cell_off, int *cell_faces, int *patch_type, int *patch_off,
                   int *patch_faces, double *nodes) {
    const Mesh &m = *static_cast<Mesh *>(mp);
    for (int i = 0; i < m.nFaces(); ++i) {
        const Face &f = m.face(i);
        owner[i] = f.owner; nbr[i] = f.neighbor; patch_id[i] = f.patchID;
        fc[3*i] = f.center.x; fc[3*i+1] = f.center.y; fc[3*i+2] = f.center.z;
        fn[3*i] = f.normal.x; fn[3*i+1] = f.normal.y; fn[3*i+2] = f.normal.z;
        fa[i] = f.area; fdel[i] = f.delta;
        fd[3*i] = f.d.x; fd[3*i+1] = f.d.y; fd[3*i+2] = f.d.z;
        fw[i] = f.weight;
    }
    int k = 0;
    cell_off[0] = 0;
    for (int c = 0; c < m.nCells(); ++c) {
        const Cell &cl = m.cell(c);
        cc[3*c] = cl.center.x; cc[3*c+1] = cl.center.y; cc[3*c+2] = cl.center.z;
        cv[c] = cl.volume;
        for (int f : cl.faces) cell_faces[k++] = f;
        cell_off[c + 1] = k;
    }
    if (wd && !m.wallDistance().empty())
        for (int c = 0; c < m.nCells(); ++c) wd[c] = m.wallDistance()[c];
    int q = 0;
    patch_off[0] = 0;
    for (int p = 0; p < m.nPatches(); ++p) {
        patch_type[p] = patchTypeCode(m.patch(p).type);
        for (int f : m.patch(p).faces) patch_faces[q++] = f;
        patch_off[p + 1] = q;
    }
    for (int i = 0; i < m.nNodes(); ++i) {
        nodes[3*i] = m.node(i).x; nodes[3*i+1] = m.node(i).y; nodes[3*i+2] = m.node(i).z;
    }
}

// Names of patches, '\n'-separated, written into buf (capacity cap).
int ref_mesh_patch_names(void *mp, char *buf, int cap) {
    const Mesh &m = *static_cast<Mesh *>(mp);
    std::string s;
    for (int p = 0; p < m.nPatches(); ++p) { s += m.patch(p).name; s += '\n'; }
    if (static_cast<int>(s.size()) + 1 > cap) return -1;
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return static_cast<int>(s.size());
}

// FlowBoundaryConditions presets: kind 0 channel, 1 bfs, 2 flat plate, 3 couette.
int ref_bc_preset(void *mp, int kind, double Uin, double kIn, double omIn, int *types_out,
                  double *values_out) {
    const Mesh &m = *static_cast<Mesh *>(mp);
    FlowBoundaryConditions bc;
    switch (kind) {
        case 0: bc = FlowBoundaryConditions::channelDefaults(m, Uin, kIn, omIn); break;
        case 1: bc = FlowBoundaryConditions::bfsDefaults(m, Uin, kIn, omIn); break;
        case 2: bc = FlowBoundaryConditions::flatPlateDefaults(m, Uin, kIn, omIn); break;
        case 3: bc = FlowBoundaryConditions::couetteDefaults(m, Uin, kIn, omIn); break;
        default: return -1;
    }
    for (int p = 0; p < m.nPatches(); ++p) {
        types_out[4*p] = static_cast<int>(bc.velocityBC[p].type);
        types_out[4*p+1] = static_cast<int>(bc.pressureBC[p].type);
        types_out[4*p+2] = static_cast<int>(bc.kBC[p].type);
        types_out[4*p+3] = static_cast<int>(bc.omegaBC[p].type);
        values_out[6*p] = bc.velocityBC[p].vecValue.x;
        values_out[6*p+1] = bc.velocityBC[p].vecValue.y;
        values_out[6*p+2] = bc.velocityBC[p].vecValue.z;
        values_out[6*p+3] = bc.pressureBC[p].value;
        values_out[6*p+4] = bc.kBC[p].value;
        values_out[6*p+5] = bc.omegaBC[p].value;
    }
    return 0;
}

// One SIMPLE solve with the reference solver (initUniform or a warm state,
// then solve).  Mirrors the solve part of ForwardModel::evaluate
// (incompressible/src/ForwardModel.cpp:41-66).  Returns 0 on success.
int ref_solve(void *mp, const btm_patch_bc *bcs, double nu, const btm_settings *st,
              const double *coeffs, int variant, const btm_init *init, btm_state *out,
              btm_history *hist, int verbose) {
    try {
        const Mesh &m = *static_cast<Mesh *>(mp);
        std::vector<double> cv(coeffs, coeffs + 11);
        SSTModel sst(InferenceParameterSet::fromVector(cv));
        sst.variant = static_cast<SSTVariant>(variant);
        FlowBoundaryConditions bc = toBCs(m, bcs);
        SolverSettings s = toSettings(st, variant, verbose);
        SIMPLESolver solver(m, sst, bc, nu, s);
        if (!g_bTarget6.empty()) solver.setTargetAnisotropy(&g_bTarget6);
        FlowFields f(m);
        if (init->mode == 0) {
            solver.initUniform(f, Vec3(init->u[0], init->u[1], init->u[2]), init->p, init->k,
                               init->omega);
        } else {
            const btm_state *w = init->warm;
            vecIn(f.U, w->U, w->Ub);
            scalarIn(f.p, w->p, w->pb);
            scalarIn(f.k, w->k, w->kb);
            scalarIn(f.omega, w->omega, w->omegab);
            scalarIn(f.nuT, w->nuT, nullptr);
            scalarIn(f.F1, w->F1, nullptr);
            scalarIn(f.F2, w->F2, nullptr);
            scalarIn(f.Pk, w->Pk, nullptr);
            scalarIn(f.CDkw, w->CDkw, nullptr);
            f.turbEstablished = w->turb_established != 0;
        }
        ConvergenceHistory h = solver.solve(f);
        if (out) {
            vecOut(f.U, out->U, out->Ub);
            scalarOut(f.p, out->p, out->pb);
            scalarOut(f.k, out->k, out->kb);
            scalarOut(f.omega, out->omega, out->omegab);
            scalarOut(f.nuT, out->nuT, nullptr);
            scalarOut(f.F1, out->F1, nullptr);
            scalarOut(f.F2, out->F2, nullptr);
            scalarOut(f.Pk, out->Pk, nullptr);
            scalarOut(f.CDkw, out->CDkw, nullptr);
            out->turb_established = f.turbEstablished ? 1 : 0;
        }
        if (hist) {
            hist->converged = h.converged;
            hist->diverged = h.diverged;
            hist->final_iter = h.finalIter;
            hist->iterations_run = static_cast<int32_t>(h.entries.size());
            hist->status = h.diverged ? BTM_DIVERGED : (h.converged ? BTM_CONVERGED : BTM_UNCONVERGED);
            hist->inner_iterations = 0;
            if (!h.entries.empty()) {
                const ResidualEntry &e = h.entries.back();
                double v[6] = {e.Ux, e.Uy, e.Uz, e.p, e.k, e.omega};
                std::memcpy(hist->last_residual, v, sizeof v);
            }
            if (hist->residuals) {
                int n = std::min<int>(hist->residual_capacity, static_cast<int>(h.entries.size()));
                for (int i = 0; i < n; ++i) {
                    const ResidualEntry &e = h.entries[i];
                    double *r = hist->residuals + 6 * i;
                    r[0] = e.Ux; r[1] = e.Uy; r[2] = e.Uz; r[3] = e.p; r[4] = e.k; r[5] = e.omega;
                }
            }
        }
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

// ObservationOperator::evaluate and ::logLikelihood
// (core/include/ObservationOperator.hpp:186-378) on a given state: the n
// observables described by `obs` (patches by index into the mesh's patch
// list) are added through the operator's own add* methods, in order.
int ref_observe(void *mp, int n, const btm_observable *obs, double nu, const btm_state *st, double *pred,
                double *loglik) {
    try {
        const Mesh &m = *static_cast<Mesh *>(mp);
        ObservationOperator op;
        for (int i = 0; i < n; ++i) {
            const btm_observable &o = obs[i];
            const std::string patch = (o.patch >= 0 && o.patch < m.nPatches()) ? m.patch(o.patch).name : "";
            const Vec3 loc(o.location[0], o.location[1], o.location[2]);
            switch (o.type) {
                case BTM_OBS_DRAG:
                    op.addDrag(patch, o.observed, o.sigma_obs, o.ref_area, o.ref_velocity, o.sigma_model);
                    break;
                case BTM_OBS_PRESSURE_TAP:
                    op.addPressureTap(loc, o.observed, o.sigma_obs, o.ref_velocity, o.sigma_model, o.ref_pressure,
                                      o.ref_density);
                    break;
                case BTM_OBS_VELOCITY:
                    op.addVelocityProfile(loc, o.component, o.observed, o.sigma_obs, o.sigma_model);
                    break;
                case BTM_OBS_SKIN_FRICTION:
                    op.addSkinFriction(patch, loc, o.observed, o.sigma_obs, o.ref_velocity, o.sigma_model);
                    break;
                case BTM_OBS_SEPARATION:
                    op.addSeparationPoint(patch, o.observed, o.sigma_obs, o.sigma_model);
                    break;
                case BTM_OBS_REATTACHMENT:
                    op.addReattachmentLength(patch, o.observed, o.sigma_obs, o.sigma_model);
                    break;
                default:
                    g_err = "unknown observable type";
                    return -1;
            }
        }
        FlowFields f(m);
        vecIn(f.U, st->U, st->Ub);
        scalarIn(f.p, st->p, st->pb);
        scalarIn(f.k, st->k, st->kb);
        scalarIn(f.omega, st->omega, st->omegab);
        if (st->nuT) scalarIn(f.nuT, st->nuT, nullptr);
        const std::vector<double> h = op.evaluate(m, f, nu);
        for (int i = 0; i < n; ++i) pred[i] = h[i];
        *loglik = op.logLikelihood(m, f, nu);
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

// Green-Gauss gradient of a scalar field (core/include/Field.hpp:122-152).
void ref_green_gauss(void *mp, const double *phi, const double *phib, double *grad) {
    const Mesh &m = *static_cast<Mesh *>(mp);
    ScalarField f(m, "phi");
    scalarIn(f, phi, phib);
    VectorField g = greenGaussGrad(f);
    vecOut(g, grad, nullptr);
}

// SSTModel::computeFields (core/src/SSTModel.cpp:122-172) plus |S|
// (core/include/Field.hpp:254-267).
void ref_sst_fields(void *mp, const double *coeffs, int variant, double nu, const double *U,
                    const double *Ub, const double *k, const double *kb, const double *om,
                    const double *omb, double *nuT, double *F1, double *F2, double *Pk,
                    double *CDkw, double *Smag) {
    const Mesh &m = *static_cast<Mesh *>(mp);
    std::vector<double> cv(coeffs, coeffs + 11);
    SSTModel sst(InferenceParameterSet::fromVector(cv));
    sst.variant = static_cast<SSTVariant>(variant);
    VectorField Uf(m, "U");
    ScalarField kf(m, "k"), wf(m, "w"), a(m), b(m), c(m), d(m), e(m);
    vecIn(Uf, U, Ub);
    scalarIn(kf, k, kb);
    scalarIn(wf, om, omb);
    sst.computeFields(m, kf, wf, Uf, nu, a, b, c, d, e);
    scalarOut(a, nuT, nullptr);
    scalarOut(b, F1, nullptr);
    scalarOut(c, F2, nullptr);
    scalarOut(d, Pk, nullptr);
    scalarOut(e, CDkw, nullptr);
    ScalarField S = strainRateMagnitude(computeVelocityGradients(Uf));
    scalarOut(S, Smag, nullptr);
}

// Linear solve of an LDU system with a named reference solver
// (core/include/LinearSolver.hpp:147-665).  res[0..3] = iterations, finalRes,
// initialRes, converged.
void ref_linear_solve(int kind, int nC, int nIF, const int *own, const int *nbr,
                      const double *diag, const double *upper, const double *lower,
                      const double *source, double *x, int maxIter, double tol, double *res) {
    LinearSystem A(nC, nIF);
    for (int f = 0; f < nIF; ++f) {
        A.own[f] = own[f]; A.nbr[f] = nbr[f]; A.upper[f] = upper[f]; A.lower[f] = lower[f];
    }
    for (int i = 0; i < nC; ++i) { A.diag[i] = diag[i]; A.source[i] = source[i]; }
    auto s = makeSolver(solverName(kind));
    std::vector<double> xv(x, x + nC);
    SolverResult r = s->solve(A, xv, maxIter, tol);
    for (int i = 0; i < nC; ++i) x[i] = xv[i];
    res[0] = r.iterations; res[1] = r.finalRes; res[2] = r.initialRes; res[3] = r.converged ? 1 : 0;
}

// y = A x for an LDU system (LinearSolver.hpp:68-77).
void ref_matvec(int nC, int nIF, const int *own, const int *nbr, const double *diag,
                const double *upper, const double *lower, const double *x, double *y) {
    LinearSystem A(nC, nIF);
    for (int f = 0; f < nIF; ++f) {
        A.own[f] = own[f]; A.nbr[f] = nbr[f]; A.upper[f] = upper[f]; A.lower[f] = lower[f];
    }
    for (int i = 0; i < nC; ++i) A.diag[i] = diag[i];
    std::vector<double> xv(x, x + nC), yv(nC);
    A.matvec(xv, yv);
    for (int i = 0; i < nC; ++i) y[i] = yv[i];
}

}  // extern "C"
