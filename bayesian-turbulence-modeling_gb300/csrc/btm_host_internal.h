// btm_host_internal.h - the case object behind the opaque btm_case handle and
// the host helpers shared by btm_host.cpp and btm_noalloc.cu (internal; not
// part of the C ABI).
#pragma once
#include "btm_common.h"

#include "../../include/btm_gb300.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

// One per-instance slab of device scratch and its host-side descriptor.
struct Slab {
    void *dptr = nullptr;
    size_t bytes = 0;
    void *dptr32 = nullptr;   // FP32 bulk of the mixed-precision engine (allocated on first use)
    size_t bytes32 = 0;
    double *dObs = nullptr;   // observation outputs (allocated on first use)
    int obsCap = 0;
    double *dInj = nullptr;   // injection blend and tensor [9*nC] (allocated on first use)
    void *dRamg = nullptr;    // reference-order AMG pools (allocated on first use)
    size_t bytesRamg = 0;
    bool hasState = false;    // a solve has left its final state in the slab
    int lastTurbEst = 0;      // turbEstablished of that state
    btm::DevInst inst{};      // host copy with device pointers
};

struct btm_case {
    int nC = 0, nIF = 0, nB = 0, nF = 0, nP = 0;
    double nu = 0.0;
    btm_settings settings{};
    bool is2d = false, bcZeroZ = true;
    int maxGridBlocks = 0;
    // device
    void *meshArena = nullptr;
    btm::DevMesh dmesh{};            // host copy with device pointers
    btm::DevMesh *dMeshPtr = nullptr;
    int amgCoarseN = 0;
    int64_t amgValTotal = 0, amgVecTotal = 0;
    std::vector<Slab> slabs;
    void *obsArena = nullptr;        // observation plan (dmesh.obs points into it)
    double *injTarget = nullptr;     // injection target anisotropy (dmesh.bTarget)
    bool injAllRealizable = true;
    double injMaxViolation = 0.0;
    std::mutex mtx;
    cudaStream_t stream = nullptr;
    // launch shape per engine (FP64, mixed): CTA threads chosen by the
    // autotuner (0: not tuned), its probe size and the probe times (ms) of
    // 256- and 512-thread CTAs
    int tunedThreads[2] = {0, 0};
    int tuneProbe[2] = {0, 0};
    double tuneMs[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
};

namespace btm_host {
int ensure_device();
void set_error(const std::string &msg);
// the value btm_last_launch_ms reports on this thread
void set_launch_ms(double ms);
// DevInst fields that do not depend on where the scratch lives (settings,
// coefficients, initial-state mode, z-momentum switch)
void fill_inst(btm_case *C, btm::DevInst &I, const double *coeffs, int variant, const btm_init *init);
int block_max_cells();
int block_threads_for(int maxCells);
// CTA threads of a case's one-CTA launches for engine 0 (FP64) / 1 (mixed):
// forced, autotuned, or by the size rule
int case_threads(const btm_case *C, int engine);
// instance slab (FP64 fields and work) and its FP32 bulk for the mixed engine
void make_slab(btm_case *C, Slab &S);
void ensure_mixed(btm_case *C, Slab &S);
// observation outputs of an instance: allocated and wired into S.inst when
// `want` and the case has observables, else S.inst.obsOut = null
void ensure_obs(btm_case *C, Slab &S, bool want);
// copies the n_obs predictions and the log-likelihood of a finished instance
void download_obs(btm_case *C, const btm::DevInst &I, btm_history *h, cudaStream_t st);
void free_slab(Slab &S);
// injection work of an instance: allocated and wired into S.inst when the
// case has a target anisotropy, else S.inst.inj = null
void ensure_inj(btm_case *C, Slab &S);
// reference-order AMG pools of an instance, allocated and wired into S.inst.rg
// when S.inst.S.refAmg (set by fill_inst)
void ensure_ramg(btm_case *C, Slab &S);
// the same pools carved from `base` (nullptr: size only); returns their bytes
size_t ramg_layout(const btm_case *C, char *base, btm::RamgWork &W);
// FP64 state between a caller's btm_state and a slab (synchronises `st`)
void upload_state(btm_case *C, const btm::DevInst &I, const btm_state *ws, cudaStream_t st,
                  std::vector<double> &stage);
void download_state(btm_case *C, const btm::DevInst &I, btm_state *o, cudaStream_t st,
                    std::vector<double> &stage);
}  // namespace btm_host
