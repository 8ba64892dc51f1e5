// btm_server.cpp - resident request loop with continuous batching (C ABI
// btm_server_*).  One server per GPU holds solve slots: a slot is one
// instance slab of one case (device fields, work and control words).  A
// submitted request reserves a free slot of its case, or allocates a new one
// within the slot count and the HBM budget; otherwise the caller gets
// BTM_EAGAIN and retries after a poll has recycled slots.  Admitted requests
// are launched in groups (one persistent launch per engine and group) while
// earlier groups are still running; every instance raises its own completion
// flag in mapped host memory when its outputs are written, so completions are
// collected per request and slots are recycled immediately.
#include "btm_common.h"
#include "btm_host_internal.h"

#include "../../include/btm_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

struct SrvError : std::runtime_error {
    int code;
    SrvError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void sck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw SrvError(BTM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int sfail(int code, const std::string &msg) {
    btm_host::set_error(msg);
    return code;
}

// The per-instance flow state a warm-start tag keeps on the device (SoA, the
// slab's own layout): U, p, k, omega and the closure fields per cell, and the
// boundary values.
constexpr int kTagCellArrays = 11;   // ux uy uz p k om nut f1 f2 pk cdkw
constexpr int kTagBndArrays = 6;     // ubx uby ubz pb kb omb

struct TagState {
    btm_case *C = nullptr;
    double *d = nullptr;
    size_t bytes = 0;
    int32_t turbEst = 0;
    int32_t solveZ = 1;
    cudaEvent_t ready = nullptr;
    bool valid = false;
    bool hasNorm = false;
    double norm[3] = {0, 0, 0};   // residual scales of the tag's first (cold) solve
};

void tag_arrays(btm_case *C, btm::DevInst &I, double **cell, double **bnd) {
    double *c[kTagCellArrays] = {I.ux, I.uy, I.uz, I.p, I.k, I.om, I.nut, I.f1, I.f2, I.pk, I.cdkw};
    double *b[kTagBndArrays] = {I.ubx, I.uby, I.ubz, I.pb, I.kb, I.omb};
    for (int q = 0; q < kTagCellArrays; ++q) cell[q] = c[q];
    for (int q = 0; q < kTagBndArrays; ++q) bnd[q] = b[q];
    (void)C;
}

// copy the state between a slab and a tag buffer (direction by `toTag`)
void tag_copy(btm_case *C, btm::DevInst &I, TagState &T, bool toTag, cudaStream_t st) {
    double *cell[kTagCellArrays], *bnd[kTagBndArrays];
    tag_arrays(C, I, cell, bnd);
    const size_t nc = (size_t)C->nC, nb = (size_t)std::max(C->nB, 1);
    double *t = T.d;
    for (int q = 0; q < kTagCellArrays; ++q, t += nc)
        sck(cudaMemcpyAsync(toTag ? t : cell[q], toTag ? cell[q] : t, nc * 8, cudaMemcpyDeviceToDevice, st), "tag copy");
    for (int q = 0; q < kTagBndArrays; ++q, t += nb)
        sck(cudaMemcpyAsync(toTag ? t : bnd[q], toTag ? bnd[q] : t, nb * 8, cudaMemcpyDeviceToDevice, st), "tag copy");
}

struct Slot {
    btm_case *C = nullptr;
    bool mixed = false;
    Slab slab;
    int flag = -1;             // index into the mapped completion flags
    enum { FREE, PENDING, RUNNING } state = FREE;
    btm_request req{};
    size_t bytes = 0;
};

}  // namespace

struct btm_server {
    int maxSlots = 0;
    int64_t budget = 0;
    int64_t used = 0;
    std::vector<std::unique_ptr<Slot>> slots;
    std::unordered_map<int64_t, TagState> tags;
    int32_t *hFlags = nullptr;   // mapped host memory [maxSlots]
    int32_t *dFlags = nullptr;   // its device view
    std::vector<cudaStream_t> streams;
    size_t nextStream = 0;
    cudaStream_t copyStream = nullptr;
    std::vector<double> stage;
    std::mutex mtx;
};

namespace {

int64_t slab_bytes(const Slot &s) {
    int64_t b = (int64_t)s.slab.bytes + (int64_t)s.slab.bytes32 + 8 * (int64_t)s.slab.obsCap;
    if (s.slab.dInj && s.C) b += 72 * (int64_t)s.C->nC;   // injection blend and tensor, 9 doubles a cell
    b += (int64_t)s.slab.bytesRamg;                        // reference-order AMG pools
    return b;
}

// Launch every PENDING slot: one persistent launch per engine and CTA size
// (a request gets the CTA size it would get alone, so its result is the same
// bits alone and in the mix), on the next stream of the pool.  The instance
// descriptors go into a stream-ordered device buffer released after the
// launch on the same stream.
void dispatch(btm_server *S) {
    std::vector<Slot *> groups[4];   // [engine * 2 + (CTA size 512)]
    for (auto &p : S->slots)
        if (p->state == Slot::PENDING) {
            const int big = btm_host::case_threads(p->C, p->mixed ? 1 : 0) == 512 ? 1 : 0;
            groups[(p->mixed ? 2 : 0) + big].push_back(p.get());
        }
    for (int g = 0; g < 4; ++g) {
        const int engine = g / 2;
        std::vector<Slot *> &group = groups[g];
        if (group.empty()) continue;
        cudaStream_t st = S->streams[S->nextStream++ % S->streams.size()];
        std::vector<btm::DevInst> arr;
        int maxCells = 0;
        size_t smem = 0;
        bool refAmg = false;
        for (Slot *s : group) {
            arr.push_back(s->slab.inst);
            maxCells = std::max(maxCells, s->C->nC);
            refAmg = refAmg || s->slab.inst.S.refAmg;
            if (s->mixed)
                smem = std::max(smem, btm::mixed_smem_bytes(s->C->nC, s->C->nIF, s->C->amgVecTotal, s->C->amgValTotal,
                                                             s->C->dmesh.coarseDirect ? s->C->amgCoarseN : 1, s->C->dmesh.band));
        }
        // requests that wait on a warm-start tag: their copies were issued on
        // the copy stream, which this launch orders after
        cudaEvent_t copied = nullptr;
        sck(cudaEventCreateWithFlags(&copied, cudaEventDisableTiming), "event");
        sck(cudaEventRecord(copied, S->copyStream), "event");
        sck(cudaStreamWaitEvent(st, copied, 0), "stream wait");
        cudaEventDestroy(copied);
        btm::DevInst *d = nullptr;
        sck(cudaMallocAsync((void **)&d, sizeof(btm::DevInst) * arr.size(), st), "cudaMallocAsync(insts)");
        sck(cudaMemcpyAsync(d, arr.data(), sizeof(btm::DevInst) * arr.size(), cudaMemcpyHostToDevice, st), "insts");
        const int threads = (g & 1) ? 512 : 256;
        int e = engine == 0 ? btm::engine_launch_block(d, (int)arr.size(), threads, st, refAmg, maxCells)
                            : btm::mixed_launch_block(d, (int)arr.size(), threads, smem, st);
        if (e) throw SrvError(BTM_ERR_CUDA, std::string("server launch: ") + cudaGetErrorString((cudaError_t)e));
        sck(cudaFreeAsync(d, st), "cudaFreeAsync(insts)");
        for (Slot *s : group) s->state = Slot::RUNNING;
    }
}

// Collect one finished slot: history, state, tag update; frees the slot.
void complete(btm_server *S, Slot &s) {
    btm::DevInst &I = s.slab.inst;
    int32_t outv[8];
    int64_t innerv[5];
    double lastv[9];
    uint64_t tns[btm::kPhaseSlots + 2];
    int32_t errv = 0;
    cudaStream_t st = S->copyStream;
    sck(cudaMemcpyAsync(outv, I.out, sizeof outv, cudaMemcpyDeviceToHost, st), "status");
    sck(cudaMemcpyAsync(innerv, I.outInner, sizeof innerv, cudaMemcpyDeviceToHost, st), "status");
    sck(cudaMemcpyAsync(lastv, I.outLast, sizeof lastv, cudaMemcpyDeviceToHost, st), "status");
    sck(cudaMemcpyAsync(tns, I.outTime, sizeof tns, cudaMemcpyDeviceToHost, st), "status");
    sck(cudaMemcpyAsync(&errv, I.err, sizeof errv, cudaMemcpyDeviceToHost, st), "status");
    sck(cudaStreamSynchronize(st), "status sync");
    if (btm_history *h = s.req.hist) {
        h->status = outv[0];
        h->converged = outv[1];
        h->diverged = outv[2];
        h->final_iter = outv[3];
        h->iterations_run = outv[4];
        h->inner_iterations = innerv[0];
        for (int q = 0; q < 4; ++q) h->inner_split[q] = innerv[q + 1];
        h->polish_start = outv[7];
        for (int q = 0; q < 6; ++q) h->last_residual[q] = lastv[q];
        for (int q = 0; q < btm::kPhaseSlots; ++q) h->phase_ms[q] = 1e-6 * (double)tns[q];
        h->solve_ms = tns[btm::kPhaseSlots + 1] > tns[btm::kPhaseSlots]
                           ? 1e-6 * (double)(tns[btm::kPhaseSlots + 1] - tns[btm::kPhaseSlots]) : 0.0;
        h->finish_ms = h->solve_ms;
        btm_host::download_obs(s.C, I, h, st);
    }
    if (s.req.out) {
        btm_host::download_state(s.C, I, s.req.out, st, S->stage);
        s.req.out->turb_established = outv[5];
    }
    if (s.req.warm_tag >= 0 && !errv && outv[2] == 0) {
        TagState &T = S->tags[s.req.warm_tag];
        if (!T.d) {
            const size_t nb = (size_t)std::max(s.C->nB, 1);
            T.bytes = 8 * ((size_t)kTagCellArrays * s.C->nC + (size_t)kTagBndArrays * nb);
            if (S->used + (int64_t)T.bytes > S->budget) throw SrvError(BTM_ERR_NOMEM, "tag state exceeds the HBM budget");
            sck(cudaMalloc((void **)&T.d, T.bytes), "cudaMalloc(tag)");
            sck(cudaEventCreateWithFlags(&T.ready, cudaEventDisableTiming), "event");
            S->used += (int64_t)T.bytes;
            T.C = s.C;
        }
        tag_copy(s.C, I, T, true, st);
        sck(cudaEventRecord(T.ready, st), "event");
        T.turbEst = outv[5];
        T.solveZ = I.solveZ;
        T.valid = true;
        if (!T.hasNorm) {
            for (int q = 0; q < 3; ++q) T.norm[q] = lastv[6 + q];
            T.hasNorm = true;
        }
    }
    S->hFlags[s.flag] = 0;
    s.state = Slot::FREE;
    if (errv) throw SrvError(BTM_ERR_TIMEOUT, "a bounded device wait timed out; the solve was abandoned");
}

}  // namespace

extern "C" {

int btm_server_create(int32_t max_slots, int64_t hbm_budget_bytes, btm_server **out) {
    if (!out || max_slots <= 0 || hbm_budget_bytes <= 0) return sfail(BTM_ERR_ARG, "bad server arguments");
    *out = nullptr;
    if (int e = btm_host::ensure_device()) return e;
    btm_server *S = new btm_server();
    try {
        S->maxSlots = max_slots;
        S->budget = hbm_budget_bytes;
        sck(cudaHostAlloc((void **)&S->hFlags, sizeof(int32_t) * max_slots, cudaHostAllocMapped), "cudaHostAlloc");
        std::memset(S->hFlags, 0, sizeof(int32_t) * max_slots);
        sck(cudaHostGetDevicePointer((void **)&S->dFlags, S->hFlags, 0), "cudaHostGetDevicePointer");
        S->streams.resize(8);
        for (auto &st : S->streams) sck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
        sck(cudaStreamCreateWithFlags(&S->copyStream, cudaStreamNonBlocking), "stream");
    } catch (const std::exception &e) {
        btm_server_destroy(S);
        return sfail(BTM_ERR_CUDA, e.what());
    }
    *out = S;
    return BTM_OK;
}

void btm_server_destroy(btm_server *S) {
    if (!S) return;
    for (auto &st : S->streams) if (st) cudaStreamSynchronize(st);
    if (S->copyStream) cudaStreamSynchronize(S->copyStream);
    for (auto &p : S->slots) btm_host::free_slab(p->slab);
    for (auto &kv : S->tags) {
        if (kv.second.d) cudaFree(kv.second.d);
        if (kv.second.ready) cudaEventDestroy(kv.second.ready);
    }
    for (auto &st : S->streams) if (st) cudaStreamDestroy(st);
    if (S->copyStream) cudaStreamDestroy(S->copyStream);
    if (S->hFlags) cudaFreeHost(S->hFlags);
    delete S;
}

int btm_server_submit(btm_server *S, const btm_request *r) {
    if (!S || !r || !r->c || !r->coeffs) return sfail(BTM_ERR_ARG, "null argument");
    if (r->init && r->init->mode != BTM_INIT_COLD && r->init->mode != BTM_INIT_WARM)
        return sfail(BTM_ERR_ARG, "requests start cold, warm from a state, or from their tag");
    std::lock_guard<std::mutex> lock(S->mtx);
    try {
        btm_case *C = r->c;
        const bool mixed = C->settings.precision == BTM_PREC_MIXED;
        if (C->nC > btm_host::block_max_cells())
            throw SrvError(BTM_ERR_ARG, "the server runs one-CTA instances: meshes up to " +
                                            std::to_string(btm_host::block_max_cells()) + " cells");
        Slot *slot = nullptr;
        for (auto &p : S->slots)
            if (p->state == Slot::FREE && p->C == C && p->mixed == mixed) { slot = p.get(); break; }
        if (!slot) {
            if ((int)S->slots.size() >= S->maxSlots) {
                // recycle a free slot of another case when the slot count is exhausted
                for (auto &p : S->slots)
                    if (p->state == Slot::FREE) {
                        S->used -= slab_bytes(*p);
                        btm_host::free_slab(p->slab);
                        const int flag = p->flag;
                        p.reset(new Slot());
                        p->flag = flag;
                        slot = p.get();
                        break;
                    }
                if (!slot) return BTM_EAGAIN;
            } else {
                S->slots.emplace_back(new Slot());
                slot = S->slots.back().get();
                slot->flag = (int)S->slots.size() - 1;
            }
            slot->C = C;
            slot->mixed = mixed;
            try {
                btm_host::make_slab(C, slot->slab);
                if (mixed) btm_host::ensure_mixed(C, slot->slab);
            } catch (const std::exception &) {
                btm_host::free_slab(slot->slab);
                slot->C = nullptr;
                return BTM_EAGAIN;
            }
            if (S->used + slab_bytes(*slot) > S->budget) {
                btm_host::free_slab(slot->slab);
                slot->C = nullptr;
                return BTM_EAGAIN;
            }
            S->used += slab_bytes(*slot);
        }
        // instance descriptor and initial state
        btm::DevInst &I = slot->slab.inst;
        auto tagIt = r->warm_tag >= 0 ? S->tags.find(r->warm_tag) : S->tags.end();
        const bool fromTag = tagIt != S->tags.end() && tagIt->second.valid && tagIt->second.C == C;
        if (fromTag) {
            btm_init cold{};
            cold.mode = 0;
            btm_host::fill_inst(C, I, r->coeffs, r->variant, &cold);
            I.initMode = 1;
            I.turbEstIn = tagIt->second.turbEst;
            I.solveZ = tagIt->second.solveZ;
            if (r->flags & BTM_REQ_TAG_NORMS && tagIt->second.hasNorm) {
                I.normFixed = 1;
                for (int q = 0; q < 3; ++q) I.normIn[q] = tagIt->second.norm[q];
            }
            sck(cudaStreamWaitEvent(S->copyStream, tagIt->second.ready, 0), "stream wait");
            tag_copy(C, I, tagIt->second, false, S->copyStream);
        } else {
            btm_host::fill_inst(C, I, r->coeffs, r->variant, r->init);
            if (r->init && r->init->mode == 1) {
                if (!r->init->warm) throw SrvError(BTM_ERR_ARG, "warm init without a state");
                btm_host::upload_state(C, I, r->init->warm, S->copyStream, S->stage);
            }
        }
        I.hist = nullptr;
        I.histCap = 0;
        const int64_t held = slab_bytes(*slot);
        btm_host::ensure_obs(C, slot->slab, r->hist && r->hist->predictions);
        btm_host::ensure_inj(C, slot->slab);
        btm_host::ensure_ramg(C, slot->slab);
        S->used += slab_bytes(*slot) - held;   // buffers allocated on first use
        S->hFlags[slot->flag] = 0;
        I.doneFlag = S->dFlags + slot->flag;
        sck(cudaMemsetAsync(I.barrier, 0, 512, S->copyStream), "memset control");
        slot->req = *r;
        slot->state = Slot::PENDING;
    } catch (const SrvError &e) {
        return sfail(e.code, e.what());
    } catch (const std::exception &e) {
        return sfail(BTM_ERR_INTERNAL, e.what());
    }
    return BTM_OK;
}

int btm_server_flush(btm_server *S) {
    if (!S) return sfail(BTM_ERR_ARG, "null server");
    std::lock_guard<std::mutex> lock(S->mtx);
    try {
        dispatch(S);
    } catch (const SrvError &e) {
        return sfail(e.code, e.what());
    } catch (const std::exception &e) {
        return sfail(BTM_ERR_INTERNAL, e.what());
    }
    return BTM_OK;
}

int btm_server_poll(btm_server *S, int32_t timeout_ms, int64_t *ids, int32_t cap, int32_t *n_done) {
    if (!S || (cap > 0 && !ids) || !n_done) return sfail(BTM_ERR_ARG, "null argument");
    *n_done = 0;
    const auto deadline = Clock::now() + std::chrono::milliseconds(std::max(timeout_ms, 0));
    try {
        {
            std::lock_guard<std::mutex> lock(S->mtx);
            dispatch(S);
        }
        for (;;) {
            {
                std::lock_guard<std::mutex> lock(S->mtx);
                for (auto &p : S->slots) {
                    if (*n_done >= cap) break;
                    if (p->state != Slot::RUNNING) continue;
                    if (((volatile int32_t *)S->hFlags)[p->flag] == 0) continue;
                    const int64_t id = p->req.id;
                    complete(S, *p);
                    ids[(*n_done)++] = id;
                }
            }
            if (*n_done > 0) return BTM_OK;
            if (Clock::now() >= deadline) return BTM_EAGAIN;
            std::this_thread::sleep_for(std::chrono::microseconds(100));
        }
    } catch (const SrvError &e) {
        return sfail(e.code, e.what());
    } catch (const std::exception &e) {
        return sfail(BTM_ERR_INTERNAL, e.what());
    }
}

int btm_server_stats(const btm_server *S, int32_t *busy_slots, int32_t *slots, int64_t *bytes, int32_t *inflight) {
    if (!S) return sfail(BTM_ERR_ARG, "null server");
    int busy = 0, run = 0;
    for (auto &p : S->slots) {
        if (p->state != Slot::FREE) ++busy;
        if (p->state == Slot::RUNNING) ++run;
    }
    if (busy_slots) *busy_slots = busy;
    if (slots) *slots = (int32_t)S->slots.size();
    if (bytes) *bytes = S->used;
    if (inflight) *inflight = run;
    return BTM_OK;
}

}  // extern "C"
