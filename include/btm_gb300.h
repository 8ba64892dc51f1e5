/*
 * btm_gb300.h - C ABI of the GB300-native incompressible SIMPLE / SST k-omega
 * forward model G(x, theta).
 *
 * Plain C: fixed-width integers, plain pointers and sizes, no exceptions and no
 * torch types cross this boundary.  Every entry point returns an int status
 * (BTM_OK = 0, negative = error; btm_last_error() gives the message) except the
 * destroy calls.  All arrays are caller-owned host memory unless a name says
 * "device".  Arithmetic is IEEE FP64 throughout the plain drop-in path.
 *
 * Each entry point names the reference interface it replaces (paths are
 * relative to the reference project root):
 *   - the case (mesh + boundary conditions + viscosity + settings) replaces the
 *     constructor arguments of ForwardModel / SIMPLESolver
 *     (incompressible/include/ForwardModel.hpp:78-90,
 *      incompressible/include/SIMPLESolver.hpp:18-22);
 *   - btm_solve replaces SIMPLESolver::initUniform + SIMPLESolver::solve as
 *     called by ForwardModel::evaluate (incompressible/src/ForwardModel.cpp:41-89,
 *     incompressible/src/SIMPLESolver.cpp:23-51, 696-1043);
 *   - btm_solve_batch has no single reference counterpart: it replaces the
 *     process-pool fan-out of independent evaluate() calls
 *     (python/parallel_mcmc.py:37-57, python/UQ/datasets/channel_calibration.py:189-222).
 */
#ifndef BTM_GB300_H
#define BTM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BTM_ABI_VERSION 6

/* ---- status codes -------------------------------------------------------- */
#define BTM_OK              0
#define BTM_ERR_ARG        -1   /* invalid argument (sizes, null pointers, types) */
#define BTM_ERR_CUDA       -2   /* a CUDA runtime call failed                     */
#define BTM_ERR_NOMEM      -3   /* device or host allocation failed               */
#define BTM_ERR_NODEVICE   -4   /* no CUDA device visible                         */
#define BTM_ERR_TIMEOUT    -5   /* a bounded device-side wait ran out             */
#define BTM_ERR_INTERNAL   -6
#define BTM_EAGAIN          1   /* server: not admitted now / nothing completed within the timeout */

/* ---- solve outcome: the reference EvaluationStatus
 *      (core/include/EvaluationTypes.hpp:6-12, python/Bindings.cpp:276-281) ---- */
#define BTM_CONVERGED           0
#define BTM_UNCONVERGED         1
#define BTM_DIVERGED            2
#define BTM_INVALID_PARAMETERS  3
#define BTM_UNKNOWN             4

/* ---- boundary-condition kinds: the reference BCType
 *      (core/include/BoundaryCondition.hpp:12-18), same order ---------------- */
#define BTM_BC_DIRICHLET        0
#define BTM_BC_NEUMANN          1
#define BTM_BC_INLET_VELOCITY   2
#define BTM_BC_OUTLET_PRESSURE  3
#define BTM_BC_WALL_NO_SLIP     4
#define BTM_BC_WALL_KOMEGA      5
#define BTM_BC_WALL_MOVING      6
#define BTM_BC_SYMMETRY         7
#define BTM_BC_CYCLIC           8

/* ---- patch types: Patch::type strings (core/include/Mesh.hpp:75-80) -------- */
#define BTM_PATCH_OTHER    0
#define BTM_PATCH_WALL     1
#define BTM_PATCH_INLET    2
#define BTM_PATCH_OUTLET   3
#define BTM_PATCH_SYMMETRY 4

/* ---- linear solver names (core/include/LinearSolver.hpp:659-665) ---------- */
#define BTM_LS_PCG          0
#define BTM_LS_BICGSTAB     1
#define BTM_LS_GAUSSSEIDEL  2
#define BTM_LS_AMG          3

/* ---- arithmetic of a solve ------------------------------------------------
 * FP64: the reference's arithmetic throughout (the drop-in).
 * MIXED: FP32 assembly, closure, gradients, Krylov and AMG work; FP64 flow
 * state, equation defects, continuity defect and pressure-correction
 * refinement, and an FP64-assembly final stage, so a converged solve
 * satisfies the FP64 discrete equations.  A mixed solve is converged when
 * the reference's test passes at a tenth of convergence_tol (or, passing at
 * convergence_tol, when 2000 iterations have not lowered the residual by
 * 10 %: its floor): the reference's test at a tolerance t stops a solve
 * a distance proportional to t from the fixed point (about 8e-6 relative L2
 * at t = 1e-8 on the 4x128 channel), so a converged mixed solve lies within
 * a tenth of that.  No reference counterpart. */
#define BTM_PREC_FP64       0
#define BTM_PREC_MIXED      1

/* ---- form of the AMG-preconditioned CG in the FP64 engine -------------------
 * REFERENCE: the reference's AMGSolver (LinearSolver.hpp:497-656): the
 * hierarchy is rebuilt from the actual matrix at every solve by the
 * reference's greedy aggregation (bit-identical maps) and Galerkin product,
 * smoothed by forward Gauss-Seidel in row order (2 + 2 sweeps, 50 on the
 * coarsest level of at most 50 rows), evaluated in parallel by wavefronts of
 * the row-order dependencies.  MULTICOLOUR: the aggregation of the geometric
 * pressure Laplacian once per case, multicolour symmetric Gauss-Seidel and a
 * dense coarsest inverse (fewer dependent steps on meshes numbered in grid
 * order).  AUTO: REFERENCE for FP64 solves on meshes of at most 16384 cells
 * whose level-0 Gauss-Seidel needs at most 32 wavefronts (unstructured or
 * renumbered meshes), MULTICOLOUR otherwise.  Meshes above 16384 cells and the
 * mixed-precision engine always use their own hierarchy.  Not a reference
 * field. */
#define BTM_AMG_AUTO        0
#define BTM_AMG_REFERENCE   1
#define BTM_AMG_MULTICOLOUR 2

/* ---- SST closure variants (core/include/SSTModel.hpp:48) ------------------- */
#define BTM_SST_FULL        0
#define BTM_SST_NOLIMITER   1
#define BTM_SST_KOMEGA      2

/* Unstructured finite-volume mesh with precomputed geometry, the data a
 * reference Mesh holds (core/include/Mesh.hpp:44-198).  Faces [0, n_internal)
 * are internal (owner and neighbour cells), faces [n_internal, n_faces) are
 * boundary faces (neighbour = -1).  Vectors are stored xyz-interleaved. */
typedef struct btm_mesh {
    int32_t n_cells;
    int32_t n_faces;
    int32_t n_internal_faces;
    int32_t n_patches;
    const int32_t *owner;          /* [n_faces]                                 */
    const int32_t *neighbour;      /* [n_faces], -1 on boundary faces           */
    const double  *face_center;    /* [n_faces*3]                               */
    const double  *face_normal;    /* [n_faces*3] unit, outward from the owner  */
    const double  *face_area;      /* [n_faces]                                 */
    const double  *face_delta;     /* [n_faces] owner-to-neighbour distance     */
    const double  *face_d;         /* [n_faces*3] owner-to-neighbour vector     */
    const double  *face_weight;    /* [n_faces] phi_f = w phi_O + (1-w) phi_N   */
    const double  *cell_center;    /* [n_cells*3]                               */
    const double  *cell_volume;    /* [n_cells]                                 */
    const double  *wall_distance;  /* [n_cells]                                 */
    const int32_t *patch_type;     /* [n_patches] BTM_PATCH_*                   */
    const int32_t *patch_offset;   /* [n_patches+1] into patch_faces            */
    const int32_t *patch_faces;    /* [patch_offset[n_patches]] face ids        */
} btm_mesh;

/* Boundary conditions of one patch for the four solved fields: the reference
 * PatchBC of velocityBC/pressureBC/kBC/omegaBC
 * (core/include/BoundaryCondition.hpp:20-41).  Profiles, when non-null, hold
 * one value per patch face in patch-face order (3 per face for velocity). */
typedef struct btm_patch_bc {
    int32_t u_type, p_type, k_type, omega_type;   /* BTM_BC_* */
    double  u_value[3];
    double  p_value;
    double  k_value;
    double  omega_value;
    const double *u_profile;       /* [n_patch_faces*3] or NULL */
    const double *k_profile;       /* [n_patch_faces]   or NULL */
    const double *omega_profile;   /* [n_patch_faces]   or NULL */
} btm_patch_bc;

/* SIMPLE controls: the reference SolverSettings (core/include/FlowFields.hpp:53-132)
 * restricted to the fields the incompressible solve reads. */
typedef struct btm_settings {
    int32_t max_iterations;
    double  convergence_tol;
    double  divergence_limit;
    double  alpha_u, alpha_p, alpha_k, alpha_omega;
    int32_t inner_iterations;
    double  inner_tolerance;
    int32_t turb_start_iter;
    int32_t turb_update_interval;
    int32_t nut_floor_iters;
    int32_t rhie_chow_all_meshes;
    double  body_force[3];
    double  k_min, k_max, omega_min;
    int32_t use_wall_functions;
    double  von_karman;
    double  wall_fn_E;
    int32_t pressure_solver;       /* BTM_LS_* */
    int32_t momentum_solver;
    int32_t turbulence_solver;
    int32_t precision;             /* BTM_PREC_*; not a reference field */
    double  alpha_injection;       /* blend factor of the Reynolds-stress
                                      injection source (alphaInjection) */
    int32_t amg_order;             /* BTM_AMG_*; not a reference field */
    int32_t anderson_depth;        /* mixed engine: depth of the Anderson
                                      acceleration of its outer iteration
                                      (from a scaled residual of 1e-3 on, and
                                      afresh in the FP64-assembly stage),
                                      0 (off) .. BTM_ANDERSON_MAX; ignored by
                                      the FP64 engine; not a reference field */
} btm_settings;
#define BTM_ANDERSON_MAX 8

/* Initial state.  mode 0 = cold uniform start exactly as
 * SIMPLESolver::initUniform (SIMPLESolver.cpp:23-51); mode 1 = warm start from
 * the fields in `warm` (a state previously returned by a solve, as the
 * WarmStartCache does, ForwardModel.cpp:56-63); mode 2 (BTM_INIT_DEVICE) =
 * warm start from the final state of the previous solve still held on the
 * device: the k-th instance of a case in a batch continues from what the
 * k-th instance of that case left (no host copy; BTM_ERR_ARG when that slot
 * has not solved yet).  Not a reference mode. */
#define BTM_INIT_COLD   0
#define BTM_INIT_WARM   1
#define BTM_INIT_DEVICE 2
typedef struct btm_state btm_state;
typedef struct btm_init {
    int32_t mode;
    double  u[3];
    double  p, k, omega;
    const btm_state *warm;
} btm_init;

/* Full flow state: FlowFields (core/include/FlowFields.hpp:9-33).  Cell arrays
 * have n_cells entries (U: n_cells*3), boundary arrays n_faces-n_internal
 * entries (Ub: *3).  Any pointer may be NULL on output to skip that field. */
struct btm_state {
    double *U, *p, *k, *omega, *nuT, *F1, *F2, *Pk, *CDkw;
    double *Ub, *pb, *kb, *omegab;
    int32_t turb_established;
};

/* Convergence record: ConvergenceHistory (FlowFields.hpp:36-49).  The
 * per-iteration residual arrays are optional (capacity 0 = not recorded);
 * each entry is {Ux, Uy, Uz, p, k, omega} as ResidualEntry. */
typedef struct btm_history {
    int32_t status;                /* BTM_CONVERGED / UNCONVERGED / DIVERGED  */
    int32_t converged;
    int32_t diverged;
    int32_t final_iter;            /* hist.finalIter                           */
    int32_t iterations_run;        /* outer iterations executed                */
    int64_t inner_iterations;      /* sum of all linear-solver iterations      */
    double  last_residual[6];      /* last ResidualEntry                       */
    int32_t residual_capacity;     /* rows available in `residuals`            */
    double *residuals;             /* [residual_capacity*6] or NULL            */
    /* device time per phase in ms, the reference's per-solve phase timers
     * (SIMPLESolver.hpp:123-136): [0] SST closure, [1] momentum assembly,
     * [2] momentum solves, [3] p' assembly, [4] p' solver setup (AMG
     * numeric setup, band factorisation), [5] p' solve, [6] corrections +
     * BCs, [7] k/omega assembly+solves, [8] the mixed engine's Anderson
     * update, [9] residual bookkeeping and convergence tests of the mixed
     * engine's FP64-assembly stage */
    double  phase_ms[10];
    /* device time of this instance from the start of its solve to its end,
     * and its end relative to the earliest instance start of the same
     * launch (the latency of a request submitted with the batch) */
    double  solve_ms;
    double  finish_ms;
    /* inner iterations by system: momentum, pressure correction, k and
     * omega, FP64 refinement passes of the pressure correction */
    int64_t inner_split[4];
    /* mixed precision: first outer iteration of the FP64-assembly polishing
     * stage (-1: FP64 engine, or the stage never started) */
    int32_t polish_start;
    /* observables of the case's observation operator (btm_case_set_observations),
     * evaluated on the device at the end of the solve: `predictions` is the
     * caller's [n_obs] buffer or NULL (then nothing is evaluated); log_lik is
     * the Gaussian log-likelihood of those predictions.  Only these n_obs + 1
     * numbers leave the device when `out` is NULL. */
    double *predictions;
    double  log_lik;
} btm_history;

typedef struct btm_case btm_case;

/* Last error message of the calling thread ("" if none). */
const char *btm_last_error(void);
int btm_abi_version(void);

/* Build a device-resident case: mesh connectivity as SoA arrays, cell-to-face
 * gather lists, the pressure AMG hierarchy (aggregation, Galerkin sparsity,
 * colouring) and per-face boundary-condition codes.  `bcs` has n_patches
 * entries.  Replaces ForwardModel/SIMPLESolver construction. */
int btm_case_create(const btm_mesh *mesh, const btm_patch_bc *bcs, double nu,
                    const btm_settings *settings, btm_case **out);
void btm_case_destroy(btm_case *c);
int btm_case_info(const btm_case *c, int32_t *n_cells, int32_t *n_boundary_faces,
                  int32_t *n_amg_levels, int32_t *is_2d);
/* Replace the case's SIMPLE controls (same checks as at creation). */
int btm_case_set_settings(btm_case *c, const btm_settings *settings);

/* ---- a-posteriori Reynolds-stress injection -------------------------------
 * ForwardModel::setTargetAnisotropy / clearTargetAnisotropy
 * (incompressible/src/ForwardModel.cpp:22-26, ForwardModel.hpp:110-118): a
 * per-cell target anisotropy b6[6*n_cells] (xx yy zz xy xz yz) adds, to every
 * later solve of the case, the explicit deferred-correction momentum source
 * -div(2 k b_target + 2 nu_t dev(S)) blended over the outer iterations at
 * settings.alpha_injection (SIMPLESolver.cpp:205-315).  b6 = NULL clears it.
 * The realizability check of the target (barycentric margin of its
 * eigenvalues >= -1e-6, core/include/AnisotropyTools.hpp) runs here once:
 * the target does not change during a solve. */
int btm_case_set_target_anisotropy(btm_case *c, const double *b6);
/* Realizability of the case's target: 1/0 and the worst violation (>= 0);
 * *active = 0 when no target is set. */
int btm_case_injection_realizability(const btm_case *c, int32_t *active, int32_t *all_realizable,
                                     double *max_violation);

/* ---- observation operator on the device -----------------------------------
 * The reference ObservationOperator (core/include/ObservationOperator.hpp:46-378)
 * attached to a case: every solve of the case whose btm_history has a
 * `predictions` buffer evaluates the observables on the device from the final
 * state (same nearest-cell / nearest-wall-face choices, first minimum wins;
 * the same molecular wall-shear formulas and sub-face interpolated zero
 * crossings; the same operation order, so results are bit-identical to a host
 * evaluation of the downloaded fields) and the Gaussian log-likelihood
 * sum_i -0.5 (pred_i - obs_i)^2 / max(sigma_obs^2 + sigma_model^2, 1e-30). */
#define BTM_OBS_DRAG            0   /* C_D = F_x / (q_ref A_ref) over a wall patch  */
#define BTM_OBS_PRESSURE_TAP    1   /* C_p at the nearest cell                       */
#define BTM_OBS_VELOCITY        2   /* U[component] at the nearest cell              */
#define BTM_OBS_SKIN_FRICTION   3   /* C_f at the nearest face of a wall patch       */
#define BTM_OBS_SEPARATION      4   /* first +/- zero crossing of tau_x along a patch */
#define BTM_OBS_REATTACHMENT    5   /* first -/+ zero crossing of tau_x along a patch */
typedef struct btm_observable {
    int32_t type;              /* BTM_OBS_*                                       */
    int32_t patch;             /* patch index (drag, skin friction, crossings)    */
    int32_t component;         /* velocity component 0, 1, 2                      */
    double  location[3];       /* probe / tap / skin-friction location            */
    double  observed, sigma_obs, sigma_model;
    double  ref_area, ref_velocity, ref_pressure, ref_density;
} btm_observable;
/* `mesh` is the mesh the case was created from (the searches run on the host
 * here, once).  n = 0 removes the operator.  Not while solves of the case are
 * in flight. */
int btm_case_set_observations(btm_case *c, const btm_mesh *mesh, int32_t n, const btm_observable *obs);

/* One forward solve on the device.  coeffs[11] are the SST constants in the
 * InferenceParameterSet order (core/include/InferenceParameters.hpp:11-14);
 * variant is BTM_SST_*.  `out` and `hist` may be NULL. */
int btm_solve(btm_case *c, const double *coeffs, int32_t variant,
              const btm_init *init, btm_state *out, btm_history *hist);

/* btm_solve without any device allocation.  No counterpart in the reference.
 * For callers that cannot allocate device memory while they serve requests:
 * programs whose device memory is all owned by their own pool or budget (an
 * extra cudaMalloc from a library would break their accounting), and
 * latency-critical loops that cannot afford cudaMalloc/cudaFree per request
 * (they can synchronise the device).  Such callers create their cases once at
 * start-up and then solve here.  Same kernel, same results as btm_solve
 * with the same launch shape: this call uses the CTA size the case's first
 * btm_solve / btm_solve_batch chose (btm_case_launch_shape), and the size rule
 * (256 threads up to 1024 cells, else 512) before any such call, since the
 * launch-shape probe allocates; give a case one btm_solve at start-up to fix
 * its shape.
 * The per-solve scratch lives in one static device array of 16 MiB per GPU,
 * held from library load until process exit.  Meshes above 16384 cells (the
 * one-CTA limit) and solves whose scratch plus requested residual history
 * would exceed 16 MiB are rejected with BTM_ERR_ARG and a message.  The first call on each device looks up
 * the array's address with that device current and creates the two CUDA
 * events that time the launch (btm_last_launch_ms reports it): make it before
 * any stream capture.  Observables attached to the case are evaluated when
 * hist->predictions is set, as btm_solve does.  Every call reuses the array
 * (each call clears what must start at zero); calls are serialised within a
 * process, and calls from two processes on one GPU at the same time would
 * race. */
int btm_solve_noalloc(btm_case *c, const double *coeffs, int32_t variant,
                      const btm_init *init, btm_state *out, btm_history *hist);

/* n independent solves in one persistent launch (one CTA per instance when the
 * mesh is small enough).  cases[i] may repeat.  coeffs is n*11, variants n,
 * inits n; outs/hists may be NULL or arrays of n. */
int btm_solve_batch(int32_t n, btm_case *const *cases, const double *coeffs,
                    const int32_t *variants, const btm_init *inits,
                    btm_state *outs, btm_history *hists);

/* Launch shape of a case's one-CTA solves in an engine (precision BTM_PREC_*):
 * CTA threads (256: two instances per SM, 512: one; 0 when the mesh runs on
 * the cooperative grid), whether the autotuner chose it, and the tuner's
 * probe (instances) and its times in ms for 256 and 512 threads.  The tuner
 * runs on the first one-CTA solve of a case in each engine (no reference
 * counterpart: it replaces the hand-set pool sizes of the calibration
 * drivers, python/UQ/datasets/channel_calibration.py:189-222). */
int btm_case_launch_shape(const btm_case *c, int32_t precision, int32_t *threads, int32_t *tuned, int32_t *probe,
                          double *probe_ms);

/* Device time of the kernel launches made by the most recent solve call on
 * this thread, measured with CUDA events on the launching stream (ms); a
 * profiling hook with no reference counterpart. */
double btm_last_launch_ms(void);

/* ---- test hooks (no reference counterpart): run one phase of the engine
 * on the device for parity tests against the oracle.  Inputs/outputs are host
 * arrays sized as documented per phase in the engine source. ---------------- */
#define BTM_PHASE_GRAD          1   /* greenGaussGrad                         */
#define BTM_PHASE_SST           2   /* SSTModel::computeFields + |S|           */
#define BTM_PHASE_MOMENTUM      3   /* assembleMomentum (one component)        */
#define BTM_PHASE_PRESSURE      4   /* assemblePressureCorrection              */
#define BTM_PHASE_KEQ           5   /* assembleKEquation                       */
#define BTM_PHASE_OMEGAEQ       6   /* assembleOmegaEquation                   */
#define BTM_PHASE_SPMV          7   /* LinearSystem::matvec                    */
#define BTM_PHASE_BICGSTAB      8   /* BiCGSTABSolver::solve                   */
#define BTM_PHASE_AMGPCG        9   /* AMG-preconditioned CG                   */
#define BTM_PHASE_PCG          11   /* PCGSolver::solve (Jacobi-preconditioned CG) */
#define BTM_PHASE_GS           13   /* GaussSeidelSolver::solve                */
#define BTM_PHASE_AMG_LEVELS   12   /* AMGSolver::setup in the reference order (needs
                                       amg_order = BTM_AMG_REFERENCE): out = level
                                       count, 21 level sizes, the aggregation map of
                                       every level but the coarsest, then per coarse
                                       level its CSR row pointers, columns, values */

/* Run one phase on one CTA with the state packed in `in` (the layout is
 * documented beside the implementation in the host driver) and copy that
 * phase's outputs to `out`.  The linear-solver phases read the system
 * diag|upper|lower|source and the start vector x from `in` and return x
 * followed by {iterations, final relative residual, initial residual,
 * converged}. */
int btm_debug_phase(btm_case *c, int32_t phase, const double *coeffs,
                    int32_t variant, int32_t arg, const double *in, int64_t n_in,
                    double *out, int64_t n_out);

/* Mesh::computeWallDistance (core/src/Mesh.cpp:345-373) on the device:
 * out[c] = min over the wall face centres of |cell_centre[c] - w| (xyz
 * triples), 1e10 when there is no wall face; bit-identical to the reference.
 * Host buffers in and out. */
int btm_wall_distance(int32_t n_cells, const double *cell_centre, int32_t n_wall, const double *wall_centre,
                      double *out);

/* ---- served request loop with continuous batching -------------------------
 *
 * No single reference counterpart: it replaces the calibration layer's
 * pattern of issuing ForwardModel::evaluate calls from many MCMC chains /
 * design loops (python/parallel_mcmc.py:37-57) with one resident server per
 * GPU.  Cases (meshes, AMG structure) stay on the device; each request
 * reserves a solve slot (per-case device slab) when one is free or can be
 * allocated within the HBM budget, otherwise btm_server_submit returns
 * BTM_EAGAIN.  Admitted requests are launched in groups by
 * btm_server_poll / btm_server_flush while earlier groups still run; each
 * instance signals its own completion (a flag in mapped host memory), so a
 * slot is recycled as soon as its solve ends, not when its whole group does.
 * A request runs with its case's launch shape (btm_case_launch_shape: the one
 * a btm_solve / btm_solve_batch of the case chose, else the size rule), so
 * its result is the same bits alone and among other requests.
 * warm_tag >= 0 keeps the request's final state on the device under that tag
 * and starts the next request carrying the same tag (same case) from it.
 * Results (state, history) are written into the caller's buffers, which
 * must stay valid until the request is returned by btm_server_poll. */
typedef struct btm_server btm_server;
typedef struct btm_request {
    int64_t id;                /* caller's request id, returned by poll          */
    btm_case *c;
    const double *coeffs;      /* 11 SST constants                               */
    int32_t variant;
    const btm_init *init;      /* start when the tag has no state yet (NULL: cold defaults) */
    int64_t warm_tag;          /* -1: none                                        */
    btm_state *out;            /* may be NULL                                     */
    btm_history *hist;         /* may be NULL; residual history not recorded      */
    int32_t flags;             /* BTM_REQ_*                                       */
} btm_request;

/* Scale a tag-started solve's residuals by the residual scales of the tag's
 * first (cold) solve instead of its own first defects.  The reference's
 * evaluate() normalises a warm start by that start's (small) iteration-0
 * defects, so a warm start must reduce them by the full tolerance again and
 * its convergence classification depends on what ran before
 * (incompressible/src/ForwardModel.cpp:49-56); with this flag a warm solve is
 * converged when its defects are as small as the chain's cold solve required. */
#define BTM_REQ_TAG_NORMS 1

/* max_slots: solve slots (concurrent instances) over all cases;
 * hbm_budget_bytes: device memory the server may hold for slots and tags. */
int btm_server_create(int32_t max_slots, int64_t hbm_budget_bytes, btm_server **out);
void btm_server_destroy(btm_server *s);
/* BTM_OK: admitted (launched at the next poll/flush); BTM_EAGAIN: no slot or
 * memory free now; negative: error. */
int btm_server_submit(btm_server *s, const btm_request *r);
/* launch every admitted request that is not running yet */
int btm_server_flush(btm_server *s);
/* Launch pending requests, then wait up to timeout_ms for completions; fills
 * ids[0..*n_done) (at most cap).  BTM_EAGAIN when nothing completed in time. */
int btm_server_poll(btm_server *s, int32_t timeout_ms, int64_t *ids, int32_t cap, int32_t *n_done);
/* counters: slots in use, slots allocated, bytes held, requests in flight */
int btm_server_stats(const btm_server *s, int32_t *busy_slots, int32_t *slots, int64_t *bytes, int32_t *inflight);

/* Test hook (no device needed): the host AMG hierarchy btm_case_create builds
 * for `mesh` - the reference's greedy aggregation (LinearSolver.hpp:407-443)
 * on the geometric pressure Laplacian, with the cooperative-grid rules when
 * grid = 1 (0: block rules, -1: by size).  Outputs the level count and sizes
 * [20], the aggregation maps of the levels that have one (concatenated, level
 * 0 first) and level 0's CSR; NULL arrays query *maps_len and *nnz0 only. */
int btm_debug_amg_hierarchy(const btm_mesh *mesh, const btm_patch_bc *bcs, int32_t grid, int32_t *n_levels,
                            int32_t *sizes, int32_t *maps, int32_t *maps_len, int32_t *row_ptr0, int32_t *col0,
                            double *val0, int32_t *nnz0);

#ifdef __cplusplus
}
#endif
#endif /* BTM_GB300_H */
