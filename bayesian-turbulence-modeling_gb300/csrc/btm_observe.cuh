// btm_observe.cuh - the observation operator and Gaussian log-likelihood on
// the device (ObservationOperator.hpp:159-378), evaluated once from the final
// state of a solve by the team leader, so that only the predictions and the
// log-likelihood leave the device.
//
// Every expression keeps the reference's operation order with explicitly
// rounded operations (no fused multiply-add contraction), so the results are
// bit-identical to a host evaluation of the downloaded fields.  The cells and
// faces each observable reads were chosen on the host (btm_case_set_observations).
#pragma once
#include "btm_team.cuh"

#include "../../include/btm_gb300.h"

namespace btm {

// molecular wall shear of listed face q: tangential velocity of the owner
// cell over the wall distance; `full` gives |u_t|, otherwise its x component
template <class T>
__device__ __forceinline__ double obs_tau(const ObsDev &O, const DevInst &I, double nu, int q, bool full) {
    const int ow = O.fOwn[q];
    const double u0 = LD(I.ux + ow), u1 = LD(I.uy + ow), u2 = LD(I.uz + ow);
    const double n0 = O.fNx[q], n1 = O.fNy[q], n2 = O.fNz[q];
    const double dot = __dadd_rn(__dadd_rn(__dmul_rn(u0, n0), __dmul_rn(u1, n1)), __dmul_rn(u2, n2));
    const double t0 = __dsub_rn(u0, __dmul_rn(n0, dot));
    if (!full) return __ddiv_rn(__dmul_rn(nu, t0), O.fDelta[q]);
    const double t1 = __dsub_rn(u1, __dmul_rn(n1, dot));
    const double t2 = __dsub_rn(u2, __dmul_rn(n2, dot));
    const double m2 = __dadd_rn(__dadd_rn(__dmul_rn(t0, t0), __dmul_rn(t1, t1)), __dmul_rn(t2, t2));
    return __ddiv_rn(__dmul_rn(nu, __dsqrt_rn(m2)), O.fDelta[q]);
}

// x of the first sign change of tau_x along the listed faces (patch order),
// interpolated between the two face centres: + to - (separation) or - to +
// (reattachment); `fallback` when there is none
template <class T>
__device__ double obs_crossing(const ObsDev &O, const DevInst &I, double nu, int a, int cnt, bool sep,
                               double fallback) {
    bool have = false;
    double prevTau = sep ? 1.0 : -1.0, prevX = 0.0;
    for (int q = a; q < a + cnt; ++q) {
        const double tau = obs_tau<T>(O, I, nu, q, false), x = O.fX[q];
        if (have && (sep ? (prevTau > 0.0 && tau <= 0.0) : (prevTau < 0.0 && tau >= 0.0))) {
            const double denom = sep ? __dsub_rn(prevTau, tau) : __dsub_rn(tau, prevTau);
            const double frac = fabs(denom) > 1e-30 ? __ddiv_rn(sep ? prevTau : -prevTau, denom) : 0.0;
            return __dadd_rn(prevX, __dmul_rn(frac, __dsub_rn(x, prevX)));
        }
        prevTau = tau;
        prevX = x;
        have = true;
    }
    return fallback;
}

// predictions into I.obsOut[0, n), the log-likelihood into I.obsOut[n]
template <class T>
__device__ __noinline__ void observe_leader(const DevMesh &M, DevInst &I) {
    const ObsDev &O = M.obs;
    const double nu = I.nu;
    double ll = 0.0;
    for (int k = 0; k < O.n; ++k) {
        const int a = O.at[k], cnt = O.cnt[k];
        double v = 0.0;
        switch (O.kind[k]) {
        case BTM_OBS_DRAG: {
            double force = 0.0;
            for (int q = a; q < a + cnt; ++q) {
                const int ow = O.fOwn[q];
                const double Sf = O.fArea[q];
                force = __dadd_rn(force, __dmul_rn(__dmul_rn(LD(I.p + ow), O.fNx[q]), Sf));
                const double tau = __ddiv_rn(__dmul_rn(nu, __dsub_rn(LD(I.ux + ow), LD(I.ubx + O.fBnd[q]))),
                                             O.fDelta[q]);
                force = __dadd_rn(force, __dmul_rn(tau, Sf));
            }
            v = __ddiv_rn(force, O.c0[k]);
            break;
        }
        case BTM_OBS_PRESSURE_TAP:
            v = __ddiv_rn(__dsub_rn(LD(I.p + a), O.c1[k]), O.c0[k]);
            break;
        case BTM_OBS_VELOCITY:
            v = O.comp[k] == 0 ? LD(I.ux + a) : (O.comp[k] == 1 ? LD(I.uy + a) : LD(I.uz + a));
            break;
        case BTM_OBS_SKIN_FRICTION:
            v = cnt > 0 ? __ddiv_rn(obs_tau<T>(O, I, nu, a, true), O.c0[k]) : 0.0;
            break;
        case BTM_OBS_SEPARATION:
            v = obs_crossing<T>(O, I, nu, a, cnt, true, 0.0);
            break;
        default:
            v = obs_crossing<T>(O, I, nu, a, cnt, false, O.c1[k]);
            break;
        }
        I.obsOut[k] = v;
        const double diff = __dsub_rn(v, O.observed[k]);
        ll = __dadd_rn(ll, __ddiv_rn(__dmul_rn(__dmul_rn(-0.5, diff), diff), O.var[k]));
    }
    I.obsOut[O.n] = ll;
}

}  // namespace btm
