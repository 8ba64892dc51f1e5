// btm_noalloc.cu - btm_solve_noalloc: the single-instance SIMPLE solve (the
// same persistent kernel btm_solve launches) with all of its per-solve device
// scratch taken from one file-scope static __device__ array, so the call never
// allocates device memory.
//
// Who needs it: host programs that hand every byte of device memory to their
// own pool or budget and must not see extra cudaMalloc/cudaFree calls from a
// library, and latency-critical request loops that cannot pay for
// cudaMalloc/cudaFree (which may synchronise the whole device) on every
// request.  Such callers create their cases once at start-up and then solve
// through this entry point.
//
// Limits and sharing rules (also stated in include/btm_gb300.h):
//   * the scratch is kNoAllocScratchBytes (16 MiB) on every GPU that loads the
//     library, held until the process exits; a solve whose scratch would not
//     fit (mesh too large, or too many residual-history rows requested) is
//     rejected with BTM_ERR_ARG and a message giving both sizes;
//   * the first call on a device looks up the array's device address there
//     (cudaGetSymbolAddress with that device current) and creates the two
//     CUDA events that time the launch; make that first call before any
//     stream capture;
//   * observables of the case (btm_case_set_observations) are evaluated into
//     the same array when the caller passes hist->predictions, and only the
//     residual-history rows the solve wrote are copied back;
//   * every call on a device reuses the same array, which keeps the previous
//     call's contents: the control words that must start at zero are cleared
//     by each call; host calls are serialised by a mutex, but two processes
//     (or two libraries' copies) driving the same GPU at once would race.
#include "btm_common.h"
#include "btm_host_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB per device
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mtx;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device (looked up once
// per device, with that device current).
cudaError_t scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

// Carve the DevInst arrays out of `base`; returns the bytes used.  With
// base == nullptr only the size is computed.  Same arrays as the pooled slabs
// of btm_solve; no grid-team reduction buffer (block mode only).  nObs > 0
// adds the observation outputs (n_obs predictions and the log-likelihood).
size_t carve(btm_case *C, char *base, btm::DevInst &I, int histRows, int nObs, bool refAmg, size_t &instOff,
             double **hist, double **obs) {
    const int nC = C->nC, nIF = C->nIF, nB = C->nB;
    const int nc = C->dmesh.coarseDirect ? C->amgCoarseN : 1;
    auto up = [](size_t n) { return (n + 31) & ~size_t(31); };  // doubles, 256-byte granules
    size_t off = 0;
    instOff = off;
    off += (sizeof(btm::DevInst) + 255) & ~size_t(255);
    char *b = base;
    auto take = [&](size_t n) {
        double *p = b ? (double *)(b + off) : nullptr;
        off += up(n) * sizeof(double);
        return p;
    };
    double **cells[] = {&I.ux, &I.uy, &I.uz, &I.p, &I.k, &I.om, &I.nut, &I.f1, &I.f2, &I.pk, &I.cdkw, &I.smag,
                        &I.gpx, &I.gpy, &I.gpz, &I.src, &I.aPx, &I.pp, &I.kold, &I.omold, &I.r, &I.rh,
                        &I.pv, &I.v, &I.s, &I.t, &I.ph, &I.sh, &I.rd};
    for (double **pp : cells) *pp = take(nC);
    for (int q = 0; q < 9; ++q) I.g[q] = take(nC);
    double *sys = take((size_t)nC + 2 * (size_t)nIF);
    I.diag = sys;
    I.upper = sys ? sys + nC : nullptr;
    I.lower = sys ? sys + nC + nIF : nullptr;
    I.fflux = take(std::max(nIF, 1));
    double **bnds[] = {&I.ubx, &I.uby, &I.ubz, &I.pb, &I.kb, &I.omb, &I.ppb};
    for (double **pp : bnds) *pp = take(std::max(nB, 1));
    I.amgVal = take(std::max<int64_t>(C->amgValTotal, 1));
    I.amgX = take(std::max<int64_t>(C->amgVecTotal, 1));
    I.amgB = take(std::max<int64_t>(C->amgVecTotal, 1));
    I.amgR = take(std::max<int64_t>(C->amgVecTotal, 1));
    I.amgRd = take((size_t)nC + C->amgVecTotal);
    I.ainv = take((size_t)nc * nc);
    I.gj = take((size_t)4 * nc * nc);
    I.gpart = take(2 * btm::kRedSlots);
    I.outLast = take(32);
    *hist = histRows > 0 ? take((size_t)6 * histRows) : nullptr;
    *obs = nObs > 0 ? take((size_t)nObs + 1) : nullptr;
    if (refAmg) off += btm_host::ramg_layout(C, b ? b + off : nullptr, I.rg);
    char *ctl = b ? b + off : nullptr;
    I.barrier = (unsigned int *)ctl;
    I.err = (int32_t *)(ctl ? ctl + 64 : nullptr);
    I.out = (int32_t *)(ctl ? ctl + 128 : nullptr);
    I.outInner = (int64_t *)(ctl ? ctl + 192 : nullptr);
    I.outTime = (uint64_t *)(ctl ? ctl + 256 : nullptr);
    off += 512;
    return off;
}

// CUDA events that time the launch, created once per device (an event is not
// device memory the caller accounts for)
cudaEvent_t g_ev[kMaxDevices][2] = {};

cudaError_t launch_events(cudaEvent_t *ev) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    for (int q = 0; q < 2; ++q) {
        if (!g_ev[dev][q]) {
            e = cudaEventCreate(&g_ev[dev][q]);
            if (e != cudaSuccess) return e;
        }
        ev[q] = g_ev[dev][q];
    }
    return cudaSuccess;
}

cudaError_t put_strided(double *dst, const double *src, int n, cudaStream_t st) {
    // AoS x/y/z component (stride 3 doubles) -> contiguous device array
    if (n <= 0) return cudaSuccess;
    return cudaMemcpy2DAsync(dst, sizeof(double), src, 3 * sizeof(double), sizeof(double), n,
                             cudaMemcpyHostToDevice, st);
}
cudaError_t get_strided(double *dst, const double *src, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    return cudaMemcpy2DAsync(dst, 3 * sizeof(double), src, sizeof(double), sizeof(double), n,
                             cudaMemcpyDeviceToHost, st);
}

int fail(int code, const std::string &msg) {
    btm_host::set_error(msg);
    return code;
}

}  // namespace

extern "C" int btm_solve_noalloc(btm_case *C, const double *coeffs, int32_t variant, const btm_init *init,
                                 btm_state *out, btm_history *hist) {
    if (!C || !coeffs) return fail(BTM_ERR_ARG, "null argument");
    if (int e = btm_host::ensure_device()) return e;
    if (C->settings.precision != BTM_PREC_FP64)
        return fail(BTM_ERR_ARG, "btm_solve_noalloc runs the FP64 engine only; set precision to fp64");
    if (init && init->mode != BTM_INIT_COLD && init->mode != BTM_INIT_WARM)
        return fail(BTM_ERR_ARG, "btm_solve_noalloc: the start is cold or warm from a state");
    if (init && init->mode == BTM_INIT_WARM && !init->warm) return fail(BTM_ERR_ARG, "warm init without a state");
    if (C->dmesh.bTarget)
        return fail(BTM_ERR_ARG, "btm_solve_noalloc: Reynolds-stress injection needs per-instance work arrays; "
                                 "use btm_solve");
    if (C->nC > btm_host::block_max_cells())
        return fail(BTM_ERR_ARG, "btm_solve_noalloc: meshes above " + std::to_string(btm_host::block_max_cells()) +
                                     " cells need the cooperative launch; use btm_solve");
    std::lock_guard<std::mutex> lock(g_noalloc_mtx);
    const int histRows = (hist && hist->residuals && hist->residual_capacity > 0) ? hist->residual_capacity : 0;
    const int nObs = (hist && hist->predictions) ? C->dmesh.obs.n : 0;
    btm::DevInst I{};
    size_t instOff = 0;
    double *dHist = nullptr, *dObs = nullptr;
    btm::DevInst probe{};
    btm_host::fill_inst(C, probe, coeffs, variant, init);
    const bool refAmg = probe.S.refAmg != 0;
    const size_t need = carve(C, nullptr, I, histRows, nObs, refAmg, instOff, &dHist, &dObs);
    if (need > kNoAllocScratchBytes)
        return fail(BTM_ERR_ARG, "btm_solve_noalloc: this solve needs " + std::to_string(need) +
                                     " bytes of scratch; the static scratch holds " +
                                     std::to_string(kNoAllocScratchBytes) + " bytes (use btm_solve)");
    void *base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return fail(BTM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    cudaEvent_t ev[2];
    e = launch_events(ev);
    if (e != cudaSuccess) return fail(BTM_ERR_CUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e));
    std::memset(&I, 0, sizeof I);
    carve(C, (char *)base, I, histRows, nObs, refAmg, instOff, &dHist, &dObs);
    btm_host::fill_inst(C, I, coeffs, variant, init);
    I.M = C->dMeshPtr;
    I.hist = dHist;
    I.histCap = histRows;
    I.obsOut = dObs;
    cudaStream_t st = C->stream;
    btm::DevInst *dI = (btm::DevInst *)((char *)base + instOff);
    // Once work is queued on `st`, every exit waits for it: the scratch is
    // shared, and the next caller must not overlap copies still in flight.
    auto drain = [&](int code) {
        cudaStreamSynchronize(st);
        return code;
    };
    auto ck = [&](cudaError_t err, const char *what) -> bool {
        if (err == cudaSuccess) return true;
        btm_host::set_error(std::string(what) + ": " + cudaGetErrorString(err));
        return false;
    };
    // the previous call's control words must not leak into this one
    if (!ck(cudaMemsetAsync(I.barrier, 0, 512, st), "clear control words")) return drain(BTM_ERR_CUDA);
    if (init && init->mode == BTM_INIT_WARM) {
        const btm_state *w = init->warm;
        const int nC = C->nC, nB = C->nB;
        bool ok = ck(put_strided(I.ux, w->U, nC, st), "upload") && ck(put_strided(I.uy, w->U + 1, nC, st), "upload") &&
                  ck(put_strided(I.uz, w->U + 2, nC, st), "upload") &&
                  ck(put_strided(I.ubx, w->Ub, nB, st), "upload") && ck(put_strided(I.uby, w->Ub + 1, nB, st), "upload") &&
                  ck(put_strided(I.ubz, w->Ub + 2, nB, st), "upload");
        const double *cs[] = {w->p, w->k, w->omega, w->nuT, w->F1, w->F2, w->Pk, w->CDkw};
        double *cd[] = {I.p, I.k, I.om, I.nut, I.f1, I.f2, I.pk, I.cdkw};
        for (int q = 0; q < 8 && ok; ++q)
            if (cs[q]) ok = ck(cudaMemcpyAsync(cd[q], cs[q], sizeof(double) * nC, cudaMemcpyHostToDevice, st), "upload");
        const double *bs[] = {w->pb, w->kb, w->omegab};
        double *bd[] = {I.pb, I.kb, I.omb};
        for (int q = 0; q < 3 && ok; ++q)
            if (nB > 0) ok = ck(cudaMemcpyAsync(bd[q], bs[q], sizeof(double) * nB, cudaMemcpyHostToDevice, st), "upload");
        if (!ok) return drain(BTM_ERR_CUDA);
    }
    if (!ck(cudaMemcpyAsync(dI, &I, sizeof I, cudaMemcpyHostToDevice, st), "instance descriptor"))
        return drain(BTM_ERR_CUDA);
    if (!ck(cudaEventRecord(ev[0], st), "event")) return drain(BTM_ERR_CUDA);
    int le = btm::engine_launch_block(dI, 1, btm_host::case_threads(C, 0), st, refAmg, C->nC);
    if (le) {
        btm_host::set_error(std::string("launch: ") + cudaGetErrorString((cudaError_t)le));
        return drain(BTM_ERR_CUDA);
    }
    if (!ck(cudaEventRecord(ev[1], st), "event")) return drain(BTM_ERR_CUDA);
    int32_t outv[8] = {0};
    int64_t innerv[5] = {0, 0, 0, 0, 0};
    int32_t errv = 0;
    double lastv[6] = {0};
    uint64_t tns[btm::kPhaseSlots + 2] = {0};
    bool ok = ck(cudaMemcpyAsync(outv, I.out, sizeof outv, cudaMemcpyDeviceToHost, st), "status") &&
              ck(cudaMemcpyAsync(innerv, I.outInner, sizeof innerv, cudaMemcpyDeviceToHost, st), "status") &&
              ck(cudaMemcpyAsync(lastv, I.outLast, sizeof lastv, cudaMemcpyDeviceToHost, st), "status") &&
              ck(cudaMemcpyAsync(tns, I.outTime, sizeof tns, cudaMemcpyDeviceToHost, st), "status") &&
              ck(cudaMemcpyAsync(&errv, I.err, sizeof errv, cudaMemcpyDeviceToHost, st), "status");
    if (ok && out) {
        const int nC = C->nC, nB = C->nB;
        if (out->U)
            ok = ck(get_strided(out->U, I.ux, nC, st), "download") && ck(get_strided(out->U + 1, I.uy, nC, st), "download") &&
                 ck(get_strided(out->U + 2, I.uz, nC, st), "download");
        if (ok && out->Ub)
            ok = ck(get_strided(out->Ub, I.ubx, nB, st), "download") && ck(get_strided(out->Ub + 1, I.uby, nB, st), "download") &&
                 ck(get_strided(out->Ub + 2, I.ubz, nB, st), "download");
        double *hd[] = {out->p, out->k, out->omega, out->nuT, out->F1, out->F2, out->Pk, out->CDkw};
        const double *dd[] = {I.p, I.k, I.om, I.nut, I.f1, I.f2, I.pk, I.cdkw};
        for (int q = 0; q < 8 && ok; ++q)
            if (hd[q]) ok = ck(cudaMemcpyAsync(hd[q], dd[q], sizeof(double) * nC, cudaMemcpyDeviceToHost, st), "download");
        double *hb[] = {out->pb, out->kb, out->omegab};
        const double *db[] = {I.pb, I.kb, I.omb};
        for (int q = 0; q < 3 && ok; ++q)
            if (hb[q] && nB > 0)
                ok = ck(cudaMemcpyAsync(hb[q], db[q], sizeof(double) * nB, cudaMemcpyDeviceToHost, st), "download");
    }
    std::vector<double> obsv((size_t)nObs + 1, 0.0);
    if (ok && nObs > 0)
        ok = ck(cudaMemcpyAsync(obsv.data(), dObs, sizeof(double) * (nObs + 1), cudaMemcpyDeviceToHost, st),
                "observations");
    cudaError_t se = cudaStreamSynchronize(st);
    if (!ok) return BTM_ERR_CUDA;
    if (se != cudaSuccess) return fail(BTM_ERR_CUDA, std::string("solve: ") + cudaGetErrorString(se));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, ev[0], ev[1]) == cudaSuccess) btm_host::set_launch_ms(ms);
    // Only the rows this solve wrote: the scratch still holds an earlier
    // call's residuals beyond them, and the caller's rows past
    // iterations_run stay untouched, as btm_solve leaves them.
    const int rows = std::min(histRows, outv[4]);
    if (rows > 0) {
        if (!ck(cudaMemcpyAsync(hist->residuals, dHist, sizeof(double) * 6 * rows, cudaMemcpyDeviceToHost, st),
                "history"))
            return drain(BTM_ERR_CUDA);
        se = cudaStreamSynchronize(st);
        if (se != cudaSuccess) return fail(BTM_ERR_CUDA, std::string("history: ") + cudaGetErrorString(se));
    }
    if (out) out->turb_established = outv[5];
    if (hist) {
        hist->status = outv[0];
        hist->converged = outv[1];
        hist->diverged = outv[2];
        hist->final_iter = outv[3];
        hist->iterations_run = outv[4];
        hist->inner_iterations = innerv[0];
        for (int q = 0; q < 4; ++q) hist->inner_split[q] = innerv[q + 1];
        hist->polish_start = outv[7];
        for (int q = 0; q < 6; ++q) hist->last_residual[q] = lastv[q];
        for (int q = 0; q < btm::kPhaseSlots; ++q) hist->phase_ms[q] = 1e-6 * (double)tns[q];
        hist->solve_ms = tns[btm::kPhaseSlots + 1] > tns[btm::kPhaseSlots]
                           ? 1e-6 * (double)(tns[btm::kPhaseSlots + 1] - tns[btm::kPhaseSlots]) : 0.0;
        hist->finish_ms = hist->solve_ms;
        if (nObs > 0) {
            for (int q = 0; q < nObs; ++q) hist->predictions[q] = obsv[q];
            hist->log_lik = obsv[nObs];
        }
    }
    if (errv) return fail(BTM_ERR_TIMEOUT, "a bounded device wait timed out; the solve was abandoned");
    return BTM_OK;
}
