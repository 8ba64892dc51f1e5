// btm_bc.cuh - boundary-condition phases on the FP64 boundary state, shared
// by the FP64 and mixed-precision engines (core/include/BoundaryCondition.hpp:196-342),
// and the per-phase device clock.
#pragma once
#include "btm_common.h"
#include "btm_team.cuh"

namespace btm {

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

// per-phase device timers, kept by the team leader
struct PhaseClock {
    uint64_t acc[kPhaseSlots];
    uint64_t t0;
    bool on;
    __device__ void start(bool leader) {
        on = leader;
        for (int q = 0; q < kPhaseSlots; ++q) acc[q] = 0;
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

}  // namespace btm
