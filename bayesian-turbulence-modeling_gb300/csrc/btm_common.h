// btm_common.h - data layout shared by the host driver (btm_host.cpp) and the
// device engine (btm_engine.cu).  Plain structs of device pointers; one
// DevMesh per case (read-only after creation), one DevInst per solve instance.
#pragma once
#include <stddef.h>
#include <stdint.h>

namespace btm {

constexpr int kMaxLevels = 20;       // AMG levels (reference cap, LinearSolver.hpp:508)
constexpr int kCoarseDirect = 32;    // coarsest level at or below this size: dense inverse
// Meshes that run on the cooperative grid stop coarsening at this size: the
// Galerkin levels of the strength-0.25 aggregation shrink by only a few per
// cent a level below ~1000 rows (a 120k-cell step mesh reaches the 20-level
// cap at ~530 rows), and each level costs the V-cycle ~27 dependent phases on
// one CTA, while a dense inverse of this size is one grid-wide mat-vec.
constexpr int kCoarseDirectGrid = 1024;
constexpr int kCoarseSweeps = 50;    // GS sweeps when the coarsest level is larger
constexpr int kRedSlots = 4;         // values per fused team reduction
constexpr int kAndersonMax = 8;      // stored differences of the Anderson acceleration (BTM_ANDERSON_MAX)
constexpr int kAaFields = 6;         // Ux, Uy, Uz, p, k, omega
// per-phase device timers: closure, momentum assembly, momentum solve, p' assembly,
// p' solver setup, p' solve, corrections, turbulence, Anderson update, other
constexpr int kPhaseSlots = 10;
// Meshes numbered with at most this bandwidth (max |owner - neighbour|) solve
// the mixed engine's pressure correction by a banded Cholesky factorisation
constexpr int kBandMax = 8;

// Boundary-condition codes per boundary face (resolved on the host from the
// per-patch btm_patch_bc list in patch order, last patch wins).
enum : int32_t {
    BC_NONE = -1,        // face in no patch: boundary value left untouched
    BC_ZEROGRAD = 0,     // value = owner cell value
    BC_FIXED = 1,        // value = stored per-face value
    BC_SYMMETRY = 2,     // velocity only: Uo - n (Uo.n)
    BC_WALL_OMEGA = 3,   // omega only: 60 nu / (beta1 delta^2)
};

struct AmgLevelDev {
    int32_t n;            // rows of this level
    int32_t nnz;          // CSR entries (levels >= 1)
    const int32_t *rowPtr, *colIdx, *diagPos;     // CSR (levels >= 1)
    const int32_t *gOff, *gIdx;                   // Galerkin gather into the finer level's values
    const int32_t *map;                           // this level's rows -> next level's rows
    const int32_t *aggOff, *aggMem;               // next level's rows -> members here (ascending)
    int32_t nColors;
    const int32_t *colorOff, *colorRows;          // rows grouped by colour
    int64_t valOff;       // offset of this level's values in DevInst::amgVal (levels >= 1)
    int64_t vecOff;       // offset of this level's x/b/r in DevInst::amgX/amgB/amgR (levels >= 1)
};

// FP32 copies of the geometry for the mixed-precision engine (reciprocals
// precomputed in FP64, then rounded)
struct DevGeom32 {
    const float *w, *area, *rdelta, *nx, *ny, *nz, *ex, *ey, *ez;   // [nIF]; rdelta = 1 / deltaC
    const float *barea, *brdelta, *bnx, *bny, *bnz;                 // [nB]; brdelta = 1 / bdeltaC
    const float *vol, *rvol, *wd;                                   // [nC]; rvol = 1/V (1 if V <= 1e-30)
};

// Observation operator of a case (ObservationOperator.hpp:46-378), resolved
// on the host: per observable its kind (BTM_OBS_*), the cell or the range of
// listed wall faces it reads, and the constants of its formula; per listed
// face (patch order) what the wall-shear formulas read.
struct ObsDev {
    int32_t n;                 // observables (0: none)
    const int32_t *kind;       // [n] BTM_OBS_*
    const int32_t *at;         // [n] cell (probe, tap), first listed face (patch kinds)
    const int32_t *cnt;        // [n] listed faces (patch kinds)
    const int32_t *comp;       // [n] velocity component
    const double *observed;    // [n]
    const double *var;         // [n] sigma_obs^2 + sigma_model^2, floored at 1e-30
    const double *c0;          // [n] denominator: q_ref A (drag), max(q_ref, 1e-20) (tap, Cf)
    const double *c1;          // [n] p_ref (tap), x of the last patch face (reattachment default)
    // listed faces
    const int32_t *fOwn, *fBnd;            // owner cell, boundary index
    const double *fNx, *fNy, *fNz;         // unit normal
    const double *fArea, *fDelta, *fX;     // area, max(delta, 1e-20), face-centre x
};

// Level table of the reference-order AMG (ints, RamgWork::lev[level *
// kRamgLevInts + field]): rows, offsets of the level's CSR row pointers,
// entries, vectors, its map to the next level (-1: coarsest), the next
// level's member offsets and members, its wavefront offsets, wavefront count
// and entry count.
enum : int { RL_N = 0, RL_PTR, RL_ENT, RL_VEC, RL_MAP, RL_MOFF, RL_MEM, RL_WFO, RL_NWF, RL_NNZ, kRamgLevInts };

// Per-instance pools of the reference-order AMG (btm_ramg.cuh): coarse levels
// rebuilt from the actual matrix at every solve.  rowPool = 2 nC + 64 coarse
// rows, entPool = 3 nnz0 + 256 coarse entries (nnz0: level-0 CSR entries).
struct RamgWork {
    int32_t rowPool, entPool;
    double *val;        // [entPool] coarse values
    double *dg;         // [rowPool] coarse diagonals
    double *rd;         // [nC + rowPool] reciprocal diagonals (level 0, then the coarse levels)
    double *x, *b, *r;  // [rowPool] coarse vectors
    double *cv;         // [nnz0] Galerkin contributions (scratch)
    int32_t *ptr;       // [rowPool + 64] coarse row pointers, level after level
    int32_t *col;       // [entPool]
    int32_t *cj;        // [nnz0] Galerkin contribution columns (scratch)
    int32_t *coff;      // [nC + 1] contribution offsets per coarse row (scratch)
    int32_t *map;       // [nC + rowPool] aggregation map of every level
    int32_t *memOff;    // [rowPool + 64] member offsets of every coarse level
    int32_t *mem;       // [nC + rowPool] members (ascending) of every coarse row
    int32_t *seed;      // [nC] claiming seed per row (-1: the row is a seed)
    int32_t *aux, *aux2;// [nC] aggregate ids, depths, cursors (scratch)
    int32_t *wfOff;     // [rowPool + 64] wavefront offsets of every coarse level
    int32_t *wfRows;    // [rowPool]
    int32_t *lev;       // [(kMaxLevels + 2) * 16] level table
    uint64_t setupNs;   // device time spent in hierarchy setups this solve (leader's clock)
    double *xs;         // shared-memory copy of every level's x (level 0 at 0, level l at
                        // nC + its vector offset), or null when it does not fit
};

struct DevMesh {
    int32_t nC, nIF, nB, nF;
    int32_t is2d;          // all normals z == 0: the z-momentum system is identically zero
    int32_t hasOutlet;     // a non-empty outlet patch exists
    int32_t rhieChow;      // Rhie-Chow dissipation active (no outlet, or forced)
    int32_t maxCellFaces;
    // internal faces [nIF]
    const int32_t *own, *nbr;
    const double *w, *area, *deltaC;              // deltaC = max(delta, 1e-20)
    const double *nx, *ny, *nz, *sfx, *sfy, *sfz; // unit normal, n * area
    const double *ex, *ey, *ez;                   // d / max(delta, 1e-30)
    const double *aOverD;                         // area / deltaC (FP64-accurate fast assembly)
    // boundary faces [nB] (index b = face - nIF)
    const int32_t *bown;
    const double *barea, *bdeltaC, *bdeltaW;      // bdeltaW = max(delta, 1e-20) for omega wall BC
    const double *bnx, *bny, *bnz, *bsfx, *bsfy, *bsfz;
    const double *baOverD;                        // barea / bdeltaC
    const int32_t *bwall;                         // face belongs to a 'wall' patch
    const int32_t *bout;                          // face belongs to an 'outlet' patch
    const int32_t *bcU, *bcP, *bcK, *bcW;         // BC codes (BC_*) per face
    const int32_t *bcPp;                          // p' boundary rule: 0 copy owner, 1 keep zero
    const double *bvUx, *bvUy, *bvUz, *bvP, *bvK, *bvW;
    // cells [nC]
    const double *vol, *wd;
    const int32_t *cfOff;      // [nC+1] internal-face gather list, ascending face index
    const int32_t *cfFace;     // face index
    const int32_t *cfOther;    // other cell, negated-1 when this cell is the neighbour: other = -(x+1)
    const int32_t *cbOff;      // [nC+1] boundary faces, ascending face index (b indices)
    const int32_t *cbFace;
    const int32_t *cbpOff;     // [nC+1] boundary faces in patch iteration order
    const int32_t *cbpFace;
    const int32_t *pinFace;    // [nC] boundary index of the last wall face (patch order), or -1
    // pressure AMG hierarchy
    int32_t nLevels;
    int32_t coarseDirect;      // coarsest level solved by its dense inverse
    AmgLevelDev lev[kMaxLevels];
    int64_t amgValTotal, amgVecTotal;
    // level 0 of the reference-order AMG: entry ids of the lduToCSR layout
    // (lev[0].rowPtr / colIdx) into diag|upper|lower, and the forward
    // Gauss-Seidel wavefronts of that CSR (rows grouped by the depth of their
    // lower-index neighbours)
    const int32_t *r0Ent;
    int32_t nnz0, nWf0;
    int32_t band;          // bandwidth of the cell numbering when <= kBandMax on a one-CTA mesh, else 0
    const int32_t *wf0Off, *wf0Rows;
    DevGeom32 g32;
    ObsDev obs;
    // Reynolds-stress injection target anisotropy [6*nC] (xx yy zz xy xz yz
    // per cell), null when injection is off
    const double *bTarget;
};

// Scalar controls of one solve (SolverSettings fields read by the loop).
struct DevSettings {
    int32_t maxIter, innerIter, turbStart, turbInterval, nutFloorIters, useWallFn;
    int32_t momSolver, turbSolver, pSolver;
    double convTol, divLimit, alphaU, alphaP, alphaK, alphaW, innerTol;
    double bodyForce[3];
    double kMin, kMax, omegaMin, vonKarman;
    double alphaInj;       // blend factor of the Reynolds-stress injection source
    int32_t refAmg;        // AMG solves use the reference-order AMG (btm_ramg.cuh)
    int32_t aaDepth;       // mixed engine: Anderson depth of the outer iteration (0: off)
};

// FP32 bulk of one mixed-precision instance: closure fields, gradients, the
// correction systems, Krylov and AMG work.  The flow state itself (U, p, k,
// omega and their boundary values) stays in the FP64 arrays of DevInst.
struct DevWork32 {
    float *nut, *f1, *f2, *pk, *cdkw, *smag;
    float *g[9];           // velocity gradients dU_i/dx_j at g[3*i+j]
    float *gp[3];          // pressure gradient
    float *diag, *upper, *lower;   // contiguous diag [nC] | upper [nIF] | lower [nIF]
    float *src;            // right-hand side of the correction system
    float *aPx;            // relaxed x-momentum diagonal (pressure-correction coefficient)
    float *pp, *ppb;       // pressure correction and its boundary values
    float *tflux;          // [nIF] transpose-stress face flux
    float *dcoef;          // [nIF] diffusion coefficient D_f of the equation being assembled
    float *r, *rh, *pv, *v, *s, *t, *ph, *sh, *rd, *x;
    float *amgVal, *amgX, *amgB, *amgR, *amgRd;
    double *ainv, *gj;     // FP64 dense inverse of the coarsest level and its Gauss-Jordan buffers
    float *band;           // [nC * (2 kBandMax + 1)] banded Cholesky factor of the pressure correction
    float *bandRd;         // [nC] reciprocal diagonal of that factor
    double *mflux;         // [nIF] FP64 face mass flux (convective defect, continuity defect)
    double *src64;         // [nC] FP64 pressure-correction right-hand side (refinement)
    // Anderson acceleration of the outer iteration: vectors over the
    // interior state, element v*nC + c for field v in (Ux, Uy, Uz, p, k, omega)
    double *aaX;           // [kAaFields nC] the iterate the current outer iteration started from
    double *aaGprev;       // [kAaFields nC] the previous outer iteration's result
    float *aaFprev;        // [kAaFields nC] the previous weighted change (result - iterate)
    float *aaDF, *aaDG;    // [kAndersonMax][kAaFields nC] differences of successive changes / results
};

struct DevInst {
    const DevMesh *M;      // device pointer
    DevSettings S;
    double nu;
    double coeff[11];
    int32_t variant;
    int32_t initMode;      // 0 cold uniform, 1 warm (fields already uploaded)
    double init[6];        // Ux, Uy, Uz, p, k, omega for a cold start
    int32_t solveZ;        // 0 when the z-momentum system is identically zero
    // state [nC] / [nB]
    double *ux, *uy, *uz, *p, *k, *om, *nut, *f1, *f2, *pk, *cdkw;
    double *ubx, *uby, *ubz, *pb, *kb, *omb;
    // work [nC]
    double *smag, *gpx, *gpy, *gpz;
    double *g[9];          // velocity gradients: dU_i/dx_j at g[3*i+j]
    // linear system: diag [nC] | upper [nIF] | lower [nIF] contiguous, so the
    // pressure Galerkin gather indexes one array (diag i, upper nC+f, lower nC+nIF+f)
    double *diag, *upper, *lower;
    double *src, *aPx, *pp, *kold, *omold;
    double *r, *rh, *pv, *v, *s, *t, *ph, *sh;
    double *rd;            // [nC] reciprocal Jacobi diagonal of the system being solved
    double *fflux;         // [nIF] per-face flux scratch
    double *ppb;           // [nB] p' boundary values
    // AMG per-instance values and vectors
    double *amgVal, *amgX, *amgB, *amgR;
    double *amgRd;         // [nC + amgVecTotal] Gauss-Seidel reciprocal diagonals per level
    double *ainv, *gj;     // dense inverse [nc*nc], Gauss-Jordan ping-pong [2*nc*2nc]
    // grid-team reduction partials [2][gridDim][kRedSlots] and barrier words
    double *gpart;
    unsigned int *barrier;  // [2]: arrival count, generation
    int32_t *err;           // error flag (nonzero: abort)
    // outputs
    int32_t *out;           // [8]: status, converged, diverged, finalIter, itersRun, turbEst, _, _
    int64_t *outInner;      // [5] inner iterations: total, momentum, pressure, turbulence, refinement
    uint64_t *outTime;      // [12] ns per phase [0..9] (leader thread's globaltimer), solve start [10] and end [11]
    double *outLast;        // [6] last residual entry, [6..8] the residual scales used
    double *hist;           // [histCap*6] or null
    int32_t histCap;
    int32_t turbEstIn;      // turbEstablished of a warm state
    int32_t normFixed;      // 1: scale residuals by normIn instead of this solve's first defects
    double normIn[3];       // momentum x, momentum y, continuity scales of an earlier cold solve
    // debug phase I/O (test hooks)
    int32_t dbgPhase, dbgArg;
    double *dbgIn, *dbgOut;
    // mixed-precision bulk (null for the FP64 engine)
    DevWork32 f;
    // observation outputs [obs.n + 1]: predictions, then the log-likelihood
    // (null: not evaluated)
    double *obsOut;
    // Reynolds-stress injection: the blended source [3][nC] (x, y, z) and the
    // deferred-correction tensor D [6][nC]; null when the case has no target
    double *inj;
    // served requests: completion flag in mapped host memory (null otherwise),
    // set by the leader after every output is written
    volatile int32_t *doneFlag;
    // reference-order AMG pools (null unless S.refAmg)
    RamgWork rg;
};

// engine entry points (btm_engine.cu)
int engine_block_threads();
// refAmg: some instance of the launch uses the reference-order AMG (the
// kernel instantiated with that solver is launched); maxCells: the largest
// mesh of the launch (sizes that kernel's shared-memory level vectors)
int engine_launch_block(DevInst *dInsts, int n, int threads, void *stream, bool refAmg = false,
                        int maxCells = 0);
int engine_launch_grid(DevInst *dInst, int blocks, void *stream);
int engine_grid_blocks(int *blocks_out);
int engine_launch_debug(DevInst *dInst, void *stream);
int engine_wall_distance(const double *dCentres, int nC, const double *dWall, int nW, double *dOut, void *stream);

// mixed-precision engine entry points (btm_mixed.cu)
size_t mixed_smem_bytes(int nC, int nIF, int64_t vecTotal, int64_t valTotal, int coarseN, int band);
int mixed_launch_block(DevInst *dInsts, int n, int threads, size_t smemBytes, void *stream);
int mixed_grid_blocks(int *blocks_out);
int mixed_launch_grid(DevInst *dInst, int blocks, void *stream);

}  // namespace btm
