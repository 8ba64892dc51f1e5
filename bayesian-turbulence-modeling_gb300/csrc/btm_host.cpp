// btm_host.cpp - host driver of the GB300 SIMPLE / SST engine and the C ABI
// declared in include/btm_gb300.h.
//
// A case (mesh + BCs + viscosity + settings) is preprocessed once into
// device-resident structure-of-arrays: internal/boundary face data, per-cell
// face gather lists in ascending face order (the order in which the
// reference's face loops reach each cell), per-face boundary-condition codes,
// and the pressure AMG hierarchy (aggregation, Galerkin gather lists,
// colouring).  Solves reuse per-case instance slabs; each solve is one
// persistent launch (btm_engine.cu).
#include "btm_common.h"
#include "btm_host_internal.h"

#include "../../include/btm_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;
thread_local double g_launch_ms = 0.0;

struct BtmError : std::runtime_error {
    int code;
    BtmError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        throw BtmError(BTM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

// ---------------------------------------------------------------------------
// device arena: one allocation, 256-byte aligned sub-arrays
// ---------------------------------------------------------------------------
struct Arena {
    std::vector<char> host;
    size_t off = 0;
    template <class T>
    size_t put(const T *src, size_t n) {
        off = (off + 255) & ~size_t(255);
        size_t at = off;
        size_t bytes = n * sizeof(T);
        if (host.size() < off + bytes + 256) host.resize(std::max(host.size() * 2, off + bytes + 256));
        if (bytes) std::memcpy(host.data() + off, src, bytes);
        off += bytes;
        return at;
    }
    template <class T>
    size_t put(const std::vector<T> &v) { return put(v.data(), v.size()); }
};

// ---------------------------------------------------------------------------
// AMG setup (host, once per case)
// ---------------------------------------------------------------------------
struct HLevel {
    int n = 0;
    // CSR with rows sorted by column; entry ids index the level's value array
    // (level 0: the LDU array diag|upper|lower; coarser: CSR positions)
    std::vector<int> rowPtr, colIdx, entry, diagPos;
    std::vector<double> val;   // geometric values (aggregation only)
    std::vector<int> map;      // -> next level
    int nCoarse = 0;
    std::vector<int> aggOff, aggMem;
    std::vector<int> gOff, gIdx;  // Galerkin gather of this level's entries (levels >= 1)
    std::vector<int> colorOff, colorRows;
    int nColors = 0;
};

// buildAggregates (core/include/LinearSolver.hpp:407-443), applied to the
// geometric pressure Laplacian: greedy seeds with strength > 0.25, then
// orphans join their strongest aggregated neighbour.
int aggregate(const HLevel &L, std::vector<int> &map) {
    const int n = L.n;
    map.assign(n, -1);
    std::vector<double> diag(n, 0.0);
    for (int i = 0; i < n; ++i)
        if (L.diagPos[i] >= 0) diag[i] = L.val[L.diagPos[i]];
    int nCoarse = 0;
    for (int i = 0; i < n; ++i) {
        if (map[i] >= 0) continue;
        int agg = nCoarse++;
        map[i] = agg;
        double aii = std::abs(diag[i]);
        for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1]; ++j) {
            int c = L.colIdx[j];
            if (c == i || map[c] >= 0) continue;
            double ajj = std::abs(diag[c]);
            double strength = std::abs(L.val[j]) / std::sqrt(aii * ajj + 1e-30);
            if (strength > 0.25) map[c] = agg;
        }
    }
    for (int i = 0; i < n; ++i) {
        if (map[i] >= 0) continue;
        double bestStr = -1.0;
        int bestAgg = 0;
        for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1]; ++j) {
            int c = L.colIdx[j];
            if (c == i && map[c] < 0) continue;
            if (map[c] >= 0 && std::abs(L.val[j]) > bestStr) {
                bestStr = std::abs(L.val[j]);
                bestAgg = map[c];
            }
        }
        map[i] = bestAgg;
    }
    return nCoarse;
}

// Plain aggregation with a row-relative strength measure, for levels where
// the reference rule stalls (see build_case).  a_ij is strong when
// |a_ij| > 0.25 max_k!=i |a_ik|, so every row has a strong neighbour.  Pass 1
// seeds an aggregate at i with its strong neighbours only when none of them
// is aggregated yet (the reference rule seeds every unaggregated row, which
// on Galerkin levels of a stretched 3-D mesh leaves ~97 % singletons); pass 2
// joins each remaining row to its strongest aggregated neighbour (decided on
// the pass-1 aggregates only); pass 3 groups what is left with its
// unaggregated strong neighbours.
int aggregate_plain(const HLevel &L, std::vector<int> &map) {
    const int n = L.n;
    map.assign(n, -1);
    std::vector<double> rmax(n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1]; ++j)
            if (L.colIdx[j] != i) rmax[i] = std::max(rmax[i], std::abs(L.val[j]));
    auto strong = [&](int i, int j) { return L.colIdx[j] != i && std::abs(L.val[j]) > 0.25 * rmax[i]; };
    int nCoarse = 0;
    for (int i = 0; i < n; ++i) {
        if (map[i] >= 0) continue;
        bool seed = true;
        for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1] && seed; ++j)
            if (strong(i, j) && map[L.colIdx[j]] >= 0) seed = false;
        if (!seed) continue;
        const int agg = nCoarse++;
        map[i] = agg;
        for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1]; ++j)
            if (strong(i, j)) map[L.colIdx[j]] = agg;
    }
    std::vector<int> join(n, -1);
    for (int i = 0; i < n; ++i) {
        if (map[i] >= 0) continue;
        double best = -1.0;
        for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1]; ++j) {
            const int c = L.colIdx[j];
            if (c != i && map[c] >= 0 && std::abs(L.val[j]) > best) {
                best = std::abs(L.val[j]);
                join[i] = map[c];
            }
        }
    }
    for (int i = 0; i < n; ++i)
        if (join[i] >= 0) map[i] = join[i];
    for (int i = 0; i < n; ++i) {
        if (map[i] >= 0) continue;
        const int agg = nCoarse++;
        map[i] = agg;
        for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1]; ++j)
            if (strong(i, j) && map[L.colIdx[j]] < 0) map[L.colIdx[j]] = agg;
    }
    return nCoarse;
}

// Galerkin product A_c = P^T A P for piecewise-constant P: builds the coarse
// CSR, its geometric values and, per coarse entry, the list of fine entry ids
// that sum into it (members ascending, then fine columns ascending).
void galerkin(HLevel &F, HLevel &C) {
    const int nc = F.nCoarse;
    C.n = nc;
    F.aggOff.assign(nc + 1, 0);
    for (int i = 0; i < F.n; ++i) F.aggOff[F.map[i] + 1]++;
    for (int I = 0; I < nc; ++I) F.aggOff[I + 1] += F.aggOff[I];
    F.aggMem.assign(F.n, 0);
    std::vector<int> cur(F.aggOff.begin(), F.aggOff.end() - 1);
    for (int i = 0; i < F.n; ++i) F.aggMem[cur[F.map[i]]++] = i;

    C.rowPtr.assign(nc + 1, 0);
    C.colIdx.clear(); C.val.clear(); C.gOff.assign(1, 0); C.gIdx.clear();
    std::vector<int> marker(nc, -1), slot(nc, 0);
    std::vector<std::vector<int>> lists;
    std::vector<int> cols;
    std::vector<double> vals;
    for (int I = 0; I < nc; ++I) {
        cols.clear(); vals.clear(); lists.clear();
        for (int q = F.aggOff[I]; q < F.aggOff[I + 1]; ++q) {
            int i = F.aggMem[q];
            for (int j = F.rowPtr[i]; j < F.rowPtr[i + 1]; ++j) {
                int J = F.map[F.colIdx[j]];
                if (marker[J] != I) {
                    marker[J] = I;
                    slot[J] = (int)cols.size();
                    cols.push_back(J);
                    vals.push_back(0.0);
                    lists.emplace_back();
                }
                vals[slot[J]] += F.val[j];
                lists[slot[J]].push_back(F.entry[j]);
            }
        }
        std::vector<int> order(cols.size());
        for (size_t e = 0; e < order.size(); ++e) order[e] = (int)e;
        std::sort(order.begin(), order.end(), [&](int a, int b) { return cols[a] < cols[b]; });
        for (int e : order) {
            C.colIdx.push_back(cols[e]);
            C.val.push_back(vals[e]);
            for (int id : lists[e]) C.gIdx.push_back(id);
            C.gOff.push_back((int)C.gIdx.size());
        }
        C.rowPtr[I + 1] = (int)C.colIdx.size();
    }
    C.entry.resize(C.colIdx.size());
    for (size_t e = 0; e < C.entry.size(); ++e) C.entry[e] = (int)e;
    C.diagPos.assign(nc, -1);
    for (int I = 0; I < nc; ++I)
        for (int j = C.rowPtr[I]; j < C.rowPtr[I + 1]; ++j)
            if (C.colIdx[j] == I) C.diagPos[I] = j;
}

// Colouring for the multicolour Gauss-Seidel smoother: a two-colouring when
// the graph is bipartite (quad meshes), else greedy in row order.
void colour(HLevel &L) {
    const int n = L.n;
    std::vector<int> col(n, -1);
    bool bip = true;
    std::deque<int> q;
    for (int s = 0; s < n && bip; ++s) {
        if (col[s] >= 0) continue;
        col[s] = 0;
        q.push_back(s);
        while (!q.empty() && bip) {
            int i = q.front();
            q.pop_front();
            for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1]; ++j) {
                int c = L.colIdx[j];
                if (c == i) continue;
                if (col[c] < 0) { col[c] = 1 - col[i]; q.push_back(c); }
                else if (col[c] == col[i]) { bip = false; break; }
            }
        }
    }
    if (!bip) {
        col.assign(n, -1);
        std::vector<int> mark;
        for (int i = 0; i < n; ++i) {
            mark.assign(mark.size(), 0);
            for (int j = L.rowPtr[i]; j < L.rowPtr[i + 1]; ++j) {
                int c = L.colIdx[j];
                if (c != i && col[c] >= 0) {
                    if ((int)mark.size() <= col[c]) mark.resize(col[c] + 1, 0);
                    mark[col[c]] = 1;
                }
            }
            int k = 0;
            while (k < (int)mark.size() && mark[k]) ++k;
            col[i] = k;
            if ((int)mark.size() <= k) mark.resize(k + 1, 0);
        }
    }
    int nColors = 0;
    for (int c : col) nColors = std::max(nColors, c + 1);
    L.nColors = nColors;
    L.colorOff.assign(nColors + 1, 0);
    for (int c : col) L.colorOff[c + 1]++;
    for (int c = 0; c < nColors; ++c) L.colorOff[c + 1] += L.colorOff[c];
    L.colorRows.assign(n, 0);
    std::vector<int> cur(L.colorOff.begin(), L.colorOff.end() - 1);
    for (int i = 0; i < n; ++i) L.colorRows[cur[col[i]]++] = i;
}

}  // namespace

namespace {
int block_max_cells();

std::once_flag g_dev_once;
int g_dev_status = 0;
std::string g_dev_msg;

int ensure_device() {
    std::call_once(g_dev_once, [] {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0) {
            g_dev_status = BTM_ERR_NODEVICE;
            g_dev_msg = std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "count 0");
        }
    });
    if (g_dev_status) g_err = g_dev_msg;
    return g_dev_status;
}

btm::DevSettings dev_settings(const btm_settings &s) {
    btm::DevSettings d{};
    d.maxIter = s.max_iterations;
    d.innerIter = s.inner_iterations;
    d.turbStart = s.turb_start_iter;
    d.turbInterval = s.turb_update_interval;
    d.nutFloorIters = s.nut_floor_iters;
    d.useWallFn = s.use_wall_functions;
    d.momSolver = s.momentum_solver;
    d.turbSolver = s.turbulence_solver;
    d.pSolver = s.pressure_solver;
    d.convTol = s.convergence_tol;
    d.divLimit = s.divergence_limit;
    d.alphaU = s.alpha_u;
    d.alphaP = s.alpha_p;
    d.alphaK = s.alpha_k;
    d.alphaW = s.alpha_omega;
    d.innerTol = s.inner_tolerance;
    for (int i = 0; i < 3; ++i) d.bodyForce[i] = s.body_force[i];
    d.kMin = s.k_min;
    d.kMax = s.k_max;
    d.omegaMin = s.omega_min;
    d.vonKarman = s.von_karman;
    d.alphaInj = s.alpha_injection;
    d.aaDepth = s.anderson_depth;
    return d;
}

void check_settings(const btm_settings &s) {
    if (s.turb_update_interval <= 0) throw BtmError(BTM_ERR_ARG, "turb_update_interval must be positive");
    for (int code : {s.pressure_solver, s.momentum_solver, s.turbulence_solver}) {
        if (code == BTM_LS_GAUSSSEIDEL && s.precision == BTM_PREC_MIXED)
            throw BtmError(BTM_ERR_ARG, "the GaussSeidel linear solver runs in the FP64 engine only");
        if (code < 0 || code > 3) throw BtmError(BTM_ERR_ARG, "unknown linear solver code");
    }
    if (!(s.alpha_u > 0) || !(s.alpha_k > 0) || !(s.alpha_omega > 0))
        throw BtmError(BTM_ERR_ARG, "relaxation factors must be positive");
    if (s.precision != BTM_PREC_FP64 && s.precision != BTM_PREC_MIXED)
        throw BtmError(BTM_ERR_ARG, "unknown precision code");
    if (s.amg_order < BTM_AMG_AUTO || s.amg_order > BTM_AMG_MULTICOLOUR)
        throw BtmError(BTM_ERR_ARG, "unknown amg_order code");
    if (s.anderson_depth < 0 || s.anderson_depth > BTM_ANDERSON_MAX)
        throw BtmError(BTM_ERR_ARG, "anderson_depth must be in [0, BTM_ANDERSON_MAX]");
}

// hostOnly: stop after the (validated) host AMG hierarchy and return it
// without touching the device; forceGrid >= 0 overrides whether the mesh is
// treated as a cooperative-grid mesh (test hook)
void build_case(btm_case *C, const btm_mesh *m, const btm_patch_bc *bcs, std::vector<HLevel> *hostOnly = nullptr,
                int forceGrid = -1) {
    const int nC = m->n_cells, nF = m->n_faces, nIF = m->n_internal_faces, nP = m->n_patches;
    if (nC <= 0 || nF < nIF || nIF < 0 || nP < 0) throw BtmError(BTM_ERR_ARG, "bad mesh sizes");
    const int nB = nF - nIF;
    C->nC = nC; C->nIF = nIF; C->nB = nB; C->nF = nF; C->nP = nP;
    for (int f = 0; f < nF; ++f) {
        int o = m->owner[f], n = m->neighbour[f];
        if (o < 0 || o >= nC) throw BtmError(BTM_ERR_ARG, "face owner out of range");
        if (f < nIF ? (n < 0 || n >= nC) : (n >= 0))
            throw BtmError(BTM_ERR_ARG, "internal faces must come first and have a neighbour");
    }
    // patch membership: every boundary face in at most one patch
    std::vector<int> facePatch(nB, -1), faceSlot(nB, -1);
    for (int p = 0; p < nP; ++p)
        for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) {
            int f = m->patch_faces[q];
            if (f < nIF || f >= nF) throw BtmError(BTM_ERR_ARG, "patch face is not a boundary face");
            if (facePatch[f - nIF] >= 0) throw BtmError(BTM_ERR_ARG, "boundary face listed in two patches");
            facePatch[f - nIF] = p;
            faceSlot[f - nIF] = q - m->patch_offset[p];
        }

    Arena A;
    btm::DevMesh &D = C->dmesh;
    std::memset(&D, 0, sizeof D);
    D.nC = nC; D.nIF = nIF; D.nB = nB; D.nF = nF;
    bool hasOutlet = false;
    for (int p = 0; p < nP; ++p)
        if (m->patch_type[p] == BTM_PATCH_OUTLET && m->patch_offset[p + 1] > m->patch_offset[p]) hasOutlet = true;
    D.hasOutlet = hasOutlet;
    D.rhieChow = (!hasOutlet || C->settings.rhie_chow_all_meshes) ? 1 : 0;
    bool is2d = true;
    for (int f = 0; f < nF; ++f)
        if (m->face_normal[3 * f + 2] != 0.0) is2d = false;
    C->is2d = is2d;
    D.is2d = is2d;

    // internal faces
    std::vector<double> w(nIF), area(nIF), dC(nIF), nx(nIF), ny(nIF), nz(nIF), sx(nIF), sy(nIF), sz(nIF),
        ex(nIF), ey(nIF), ez(nIF);
    std::vector<int> own(nIF), nbr(nIF);
    for (int f = 0; f < nIF; ++f) {
        own[f] = m->owner[f]; nbr[f] = m->neighbour[f];
        w[f] = m->face_weight[f];
        area[f] = m->face_area[f];
        double del = m->face_delta[f];
        dC[f] = std::max(del, 1e-20);
        nx[f] = m->face_normal[3 * f]; ny[f] = m->face_normal[3 * f + 1]; nz[f] = m->face_normal[3 * f + 2];
        sx[f] = nx[f] * area[f]; sy[f] = ny[f] * area[f]; sz[f] = nz[f] * area[f];
        double dd = std::max(del, 1e-30);
        ex[f] = m->face_d[3 * f] / dd; ey[f] = m->face_d[3 * f + 1] / dd; ez[f] = m->face_d[3 * f + 2] / dd;
    }
    // boundary faces
    std::vector<int> bown(nB), bwall(nB, 0), bout(nB, 0), bcU(nB, btm::BC_NONE), bcP(nB, btm::BC_NONE),
        bcK(nB, btm::BC_NONE), bcW(nB, btm::BC_NONE), bcPp(nB, 1);
    std::vector<double> barea(nB), bdC(nB), bdW(nB), bnx(nB), bny(nB), bnz(nB), bsx(nB), bsy(nB), bsz(nB),
        bvUx(nB, 0.0), bvUy(nB, 0.0), bvUz(nB, 0.0), bvP(nB, 0.0), bvK(nB, 0.0), bvW(nB, 0.0);
    bool bcZeroZ = true;
    for (int b = 0; b < nB; ++b) {
        int f = nIF + b;
        bown[b] = m->owner[f];
        barea[b] = m->face_area[f];
        bdC[b] = std::max(m->face_delta[f], 1e-20);
        bdW[b] = std::max(m->face_delta[f], 1e-20);
        bnx[b] = m->face_normal[3 * f]; bny[b] = m->face_normal[3 * f + 1]; bnz[b] = m->face_normal[3 * f + 2];
        bsx[b] = bnx[b] * barea[b]; bsy[b] = bny[b] * barea[b]; bsz[b] = bnz[b] * barea[b];
        int p = facePatch[b];
        if (p < 0) continue;
        int kk = faceSlot[b];
        int ptype = m->patch_type[p];
        bwall[b] = ptype == BTM_PATCH_WALL;
        bout[b] = ptype == BTM_PATCH_OUTLET;
        bcPp[b] = ptype == BTM_PATCH_OUTLET ? 1 : 0;
        const btm_patch_bc &bc = bcs[p];
        switch (bc.u_type) {
            case BTM_BC_WALL_NO_SLIP: bcU[b] = btm::BC_FIXED; break;
            case BTM_BC_WALL_MOVING:
                bcU[b] = btm::BC_FIXED;
                bvUx[b] = bc.u_value[0]; bvUy[b] = bc.u_value[1]; bvUz[b] = bc.u_value[2];
                break;
            case BTM_BC_INLET_VELOCITY:
            case BTM_BC_DIRICHLET:
                bcU[b] = btm::BC_FIXED;
                if (bc.u_profile) {
                    bvUx[b] = bc.u_profile[3 * kk]; bvUy[b] = bc.u_profile[3 * kk + 1]; bvUz[b] = bc.u_profile[3 * kk + 2];
                } else {
                    bvUx[b] = bc.u_value[0]; bvUy[b] = bc.u_value[1]; bvUz[b] = bc.u_value[2];
                }
                break;
            case BTM_BC_SYMMETRY: bcU[b] = btm::BC_SYMMETRY; break;
            default: bcU[b] = btm::BC_ZEROGRAD; break;
        }
        if (bcU[b] == btm::BC_FIXED && bvUz[b] != 0.0) bcZeroZ = false;
        if (bc.p_type == BTM_BC_OUTLET_PRESSURE || bc.p_type == BTM_BC_DIRICHLET) {
            bcP[b] = btm::BC_FIXED; bvP[b] = bc.p_value;
        } else {
            bcP[b] = btm::BC_ZEROGRAD;
        }
        if (bc.k_type == BTM_BC_WALL_KOMEGA) { bcK[b] = btm::BC_FIXED; bvK[b] = 0.0; }
        else if (bc.k_type == BTM_BC_DIRICHLET) { bcK[b] = btm::BC_FIXED; bvK[b] = bc.k_profile ? bc.k_profile[kk] : bc.k_value; }
        else bcK[b] = btm::BC_ZEROGRAD;
        if (bc.omega_type == BTM_BC_WALL_KOMEGA) bcW[b] = btm::BC_WALL_OMEGA;
        else if (bc.omega_type == BTM_BC_DIRICHLET) { bcW[b] = btm::BC_FIXED; bvW[b] = bc.omega_profile ? bc.omega_profile[kk] : bc.omega_value; }
        else bcW[b] = btm::BC_ZEROGRAD;
    }
    C->bcZeroZ = bcZeroZ;

    // cell gather lists
    std::vector<int> cfOff(nC + 1, 0), cbOff(nC + 1, 0), cbpOff(nC + 1, 0), pin(nC, -1);
    for (int f = 0; f < nIF; ++f) { cfOff[own[f] + 1]++; cfOff[nbr[f] + 1]++; }
    for (int c = 0; c < nC; ++c) cfOff[c + 1] += cfOff[c];
    std::vector<int> cfFace(cfOff[nC]), cfOther(cfOff[nC]);
    {
        std::vector<int> cur(cfOff.begin(), cfOff.end() - 1);
        for (int f = 0; f < nIF; ++f) {
            int o = own[f], n = nbr[f];
            cfFace[cur[o]] = f; cfOther[cur[o]++] = n;
            cfFace[cur[n]] = f; cfOther[cur[n]++] = -(o + 1);
        }
    }
    int maxCF = 0;
    for (int c = 0; c < nC; ++c) maxCF = std::max(maxCF, cfOff[c + 1] - cfOff[c]);
    for (int b = 0; b < nB; ++b) cbOff[bown[b] + 1]++;
    for (int c = 0; c < nC; ++c) cbOff[c + 1] += cbOff[c];
    std::vector<int> cbFace(std::max(1, cbOff[nC]));
    {
        std::vector<int> cur(cbOff.begin(), cbOff.end() - 1);
        for (int b = 0; b < nB; ++b) cbFace[cur[bown[b]]++] = b;
    }
    for (int p = 0; p < nP; ++p)
        for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) cbpOff[m->owner[m->patch_faces[q]] + 1]++;
    for (int c = 0; c < nC; ++c) cbpOff[c + 1] += cbpOff[c];
    std::vector<int> cbpFace(std::max(1, cbpOff[nC]));
    {
        std::vector<int> cur(cbpOff.begin(), cbpOff.end() - 1);
        for (int p = 0; p < nP; ++p)
            for (int q = m->patch_offset[p]; q < m->patch_offset[p + 1]; ++q) {
                int f = m->patch_faces[q];
                cbpFace[cur[m->owner[f]]++] = f - nIF;
                if (m->patch_type[p] == BTM_PATCH_WALL) pin[m->owner[f]] = f - nIF;
            }
    }
    D.maxCellFaces = maxCF;

    // ---- pressure AMG hierarchy on the geometric Laplacian ----------------
    std::vector<HLevel> lv(1);
    {
        HLevel &L0 = lv[0];
        L0.n = nC;
        // LDU values with aP = 1: coefficient (w Vo + (1-w) Vn) A / delta
        std::vector<double> diag(nC, 0.0), coef(nIF);
        for (int f = 0; f < nIF; ++f) {
            double dpf = w[f] * m->cell_volume[own[f]] + (1.0 - w[f]) * m->cell_volume[nbr[f]];
            coef[f] = dpf * area[f] / dC[f];
            diag[own[f]] += coef[f];
            diag[nbr[f]] += coef[f];
        }
        for (int b = 0; b < nB; ++b)
            if (bout[b]) diag[bown[b]] += m->cell_volume[bown[b]] * barea[b] / bdC[b];
        if (!hasOutlet) diag[0] += std::abs(diag[0]) > 1e-30 ? diag[0] : 1.0;
        // CSR rows sorted by column; entry ids into diag|upper|lower
        L0.rowPtr.assign(nC + 1, 0);
        for (int c = 0; c < nC; ++c) L0.rowPtr[c + 1] = L0.rowPtr[c] + 1 + (cfOff[c + 1] - cfOff[c]);
        L0.colIdx.resize(L0.rowPtr[nC]);
        L0.entry.resize(L0.rowPtr[nC]);
        L0.val.resize(L0.rowPtr[nC]);
        L0.diagPos.assign(nC, -1);
        std::vector<std::pair<int, int>> row;
        for (int c = 0; c < nC; ++c) {
            row.clear();
            row.push_back({c, c});
            for (int e = cfOff[c]; e < cfOff[c + 1]; ++e) {
                int f = cfFace[e], oth = cfOther[e];
                if (oth >= 0) row.push_back({oth, nC + f});              // upper: row own, col nbr
                else row.push_back({-(oth + 1), nC + nIF + f});           // lower: row nbr, col own
            }
            std::stable_sort(row.begin(), row.end(), [](auto &a, auto &b) { return a.first < b.first; });
            int pos = L0.rowPtr[c];
            for (auto &pr : row) {
                L0.colIdx[pos] = pr.first;
                L0.entry[pos] = pr.second;
                int id = pr.second;
                L0.val[pos] = id < nC ? diag[id] : -coef[(id - nC) % nIF];
                if (pr.first == c) L0.diagPos[c] = pos;
                ++pos;
            }
        }
    }
    // cooperative-grid meshes keep a dense coarsest level of up to
    // kCoarseDirectGrid rows (level 0 is always coarsened once)
    const bool gridMesh = forceGrid >= 0 ? forceGrid != 0 : nC > block_max_cells();
    const int directMax = gridMesh ? btm::kCoarseDirectGrid : btm::kCoarseDirect;
    while ((int)lv.size() < btm::kMaxLevels && lv.back().n > btm::kCoarseDirect &&
           (lv.size() == 1 || lv.back().n > directMax)) {
        HLevel &F = lv.back();
        int nc = aggregate(F, F.map);
        // On cooperative-grid meshes a level that the reference rule shrinks
        // by less than 20 % is aggregated by aggregate_plain instead: on a
        // stretched 3-D duct the reference rule stalls at ~18 % of the fine
        // size and fills the 20-level cap with near-identical levels, each
        // costing a full set of grid-wide sweeps.
        if (directMax > btm::kCoarseDirect && nc > 0.8 * F.n) nc = aggregate_plain(F, F.map);
        if (nc == 0 || nc >= F.n) { F.map.clear(); break; }
        F.nCoarse = nc;
        HLevel Cl;
        galerkin(F, Cl);
        lv.push_back(std::move(Cl));
    }
    for (auto &L : lv) colour(L);
    const int nL = (int)lv.size();
    // forward Gauss-Seidel wavefronts of the level-0 CSR for the
    // reference-order AMG: depth(i) = 1 + max depth of i's lower-index
    // neighbours; rows grouped by depth, ascending within a group
    std::vector<int> wf0Off, wf0Rows;
    {
        const HLevel &L0 = lv[0];
        std::vector<int> depth(nC, 0);
        int maxD = 0;
        for (int i = 0; i < nC; ++i) {
            int d = 0;
            for (int j = L0.rowPtr[i]; j < L0.rowPtr[i + 1]; ++j)
                if (L0.colIdx[j] < i) d = std::max(d, depth[L0.colIdx[j]] + 1);
            depth[i] = d;
            maxD = std::max(maxD, d);
        }
        const int nWf = nC > 0 ? maxD + 1 : 0;
        wf0Off.assign(nWf + 1, 0);
        for (int i = 0; i < nC; ++i) wf0Off[depth[i] + 1]++;
        for (int w = 0; w < nWf; ++w) wf0Off[w + 1] += wf0Off[w];
        wf0Rows.assign(nC, 0);
        std::vector<int> cur(wf0Off.begin(), wf0Off.end() - (nWf > 0 ? 1 : 0));
        for (int i = 0; i < nC; ++i) wf0Rows[cur[depth[i]]++] = i;
        D.nWf0 = nWf;
        D.nnz0 = (int32_t)L0.colIdx.size();
    }
    // bandwidth of the cell numbering (banded pressure-correction solve of the
    // mixed engine on one-CTA meshes)
    {
        int bw = 0;
        for (int f = 0; f < nIF; ++f) bw = std::max(bw, std::abs(own[f] - nbr[f]));
        D.band = (!gridMesh && bw > 0 && bw <= btm::kBandMax) ? bw : 0;
    }
    D.nLevels = nL;
    D.coarseDirect = lv.back().n <= directMax ? 1 : 0;
    C->amgCoarseN = lv.back().n;

    // ---- index validation: every gather index the kernels use is checked
    // against the buffer it indexes before anything reaches the device ------
    auto inRange = [](const std::vector<int> &v, int lo, int hi, const char *what) {
        for (int x : v)
            if (x < lo || x >= hi) throw BtmError(BTM_ERR_INTERNAL, std::string("index out of range: ") + what);
    };
    inRange(cfFace, 0, std::max(nIF, 1), "cfFace");
    for (int x : cfOther)
        if (!((x >= 0 && x < nC) || (x < 0 && -(x + 1) < nC))) throw BtmError(BTM_ERR_INTERNAL, "cfOther");
    if (cbOff[nC] > 0) inRange(std::vector<int>(cbFace.begin(), cbFace.begin() + cbOff[nC]), 0, nB, "cbFace");
    if (cbpOff[nC] > 0) inRange(std::vector<int>(cbpFace.begin(), cbpFace.begin() + cbpOff[nC]), 0, nB, "cbpFace");
    inRange(pin, -1, std::max(nB, 1), "pinFace");
    for (int l = 0; l < (int)lv.size(); ++l) {
        const HLevel &L = lv[l];
        inRange(L.colIdx, 0, L.n, "colIdx");
        inRange(L.colorRows, 0, L.n, "colorRows");
        if ((int)L.colorRows.size() != L.n) throw BtmError(BTM_ERR_INTERNAL, "colour partition");
        if (l >= 1) {
            const int fineSize = l == 1 ? nC + 2 * nIF : (int)lv[l - 1].colIdx.size();
            inRange(L.gIdx, 0, fineSize, "gIdx");
            if ((int)L.gOff.size() != (int)L.colIdx.size() + 1) throw BtmError(BTM_ERR_INTERNAL, "gOff");
            for (int I = 0; I < L.n; ++I)
                if (L.diagPos[I] >= (int)L.colIdx.size()) throw BtmError(BTM_ERR_INTERNAL, "diagPos");
        }
        if (l + 1 < (int)lv.size()) {
            inRange(L.map, 0, lv[l + 1].n, "map");
            inRange(L.aggMem, 0, L.n, "aggMem");
            if ((int)L.aggOff.size() != lv[l + 1].n + 1 || L.aggOff.back() != L.n)
                throw BtmError(BTM_ERR_INTERNAL, "aggOff");
        }
    }

    if (hostOnly) {
        *hostOnly = std::move(lv);
        return;
    }

    // ---- upload ------------------------------------------------------------
    struct Rec { size_t at; };
    auto P = [&](const auto &v) { return A.put(v); };
    size_t o_own = P(own), o_nbr = P(nbr), o_w = P(w), o_area = P(area), o_dC = P(dC), o_nx = P(nx), o_ny = P(ny),
           o_nz = P(nz), o_sx = P(sx), o_sy = P(sy), o_sz = P(sz), o_ex = P(ex), o_ey = P(ey), o_ez = P(ez);
    size_t o_bown = P(bown), o_barea = P(barea), o_bdC = P(bdC), o_bdW = P(bdW), o_bnx = P(bnx), o_bny = P(bny),
           o_bnz = P(bnz), o_bsx = P(bsx), o_bsy = P(bsy), o_bsz = P(bsz), o_bwall = P(bwall), o_bout = P(bout),
           o_bcU = P(bcU), o_bcP = P(bcP), o_bcK = P(bcK), o_bcW = P(bcW), o_bcPp = P(bcPp), o_bvUx = P(bvUx),
           o_bvUy = P(bvUy), o_bvUz = P(bvUz), o_bvP = P(bvP), o_bvK = P(bvK), o_bvW = P(bvW);
    std::vector<double> vol(m->cell_volume, m->cell_volume + nC), wd(m->wall_distance, m->wall_distance + nC);
    size_t o_vol = P(vol), o_wd = P(wd), o_cfOff = P(cfOff), o_cfFace = P(cfFace), o_cfOther = P(cfOther),
           o_cbOff = P(cbOff), o_cbFace = P(cbFace), o_cbpOff = P(cbpOff), o_cbpFace = P(cbpFace), o_pin = P(pin);
    // FP32 geometry for the mixed-precision engine; reciprocals are formed in
    // FP64 and rounded once
    auto f32 = [](const std::vector<double> &v) { return std::vector<float>(v.begin(), v.end()); };
    auto recip32 = [](const std::vector<double> &v, double guard, double dflt) {
        std::vector<float> r(v.size());
        for (size_t i = 0; i < v.size(); ++i) r[i] = (float)(v[i] > guard ? 1.0 / v[i] : dflt);
        return r;
    };
    const size_t g_w = P(f32(w)), g_area = P(f32(area)), g_rdel = P(recip32(dC, 0.0, 0.0)), g_nx = P(f32(nx)),
                 g_ny = P(f32(ny)), g_nz = P(f32(nz)), g_ex = P(f32(ex)), g_ey = P(f32(ey)), g_ez = P(f32(ez)),
                 g_barea = P(f32(barea)), g_brdel = P(recip32(bdC, 0.0, 0.0)), g_bnx = P(f32(bnx)),
                 g_bny = P(f32(bny)), g_bnz = P(f32(bnz)), g_vol = P(f32(vol)), g_rvol = P(recip32(vol, 1e-30, 1.0)),
                 g_wd = P(f32(wd));
    std::vector<double> aOverD(nIF), baOverD(nB);
    for (int f = 0; f < nIF; ++f) aOverD[f] = area[f] / dC[f];
    for (int b = 0; b < nB; ++b) baOverD[b] = barea[b] / bdC[b];
    const size_t o_aod = P(aOverD), o_baod = P(baOverD);
    struct LevOff { size_t rowPtr, colIdx, diagPos, gOff, gIdx, map, aggOff, aggMem, colorOff, colorRows; };
    const size_t o_r0Ent = P(lv[0].entry), o_wf0Off = P(wf0Off), o_wf0Rows = P(wf0Rows);
    std::vector<LevOff> lo(nL);
    int64_t valTot = 0, vecTot = 0;
    for (int l = 0; l < nL; ++l) {
        HLevel &L = lv[l];
        LevOff &q = lo[l];
        q.rowPtr = P(L.rowPtr); q.colIdx = P(L.colIdx); q.diagPos = P(L.diagPos);
        q.gOff = P(L.gOff); q.gIdx = P(L.gIdx); q.map = P(L.map); q.aggOff = P(L.aggOff); q.aggMem = P(L.aggMem);
        q.colorOff = P(L.colorOff); q.colorRows = P(L.colorRows);
        btm::AmgLevelDev &dl = D.lev[l];
        dl.n = L.n;
        dl.nnz = l == 0 ? 0 : (int)L.colIdx.size();
        dl.nColors = L.nColors;
        if (l >= 1) {
            dl.valOff = valTot; valTot += (L.colIdx.size() + 31) & ~size_t(31);
            dl.vecOff = vecTot; vecTot += (L.n + 31) & ~31;
        }
    }
    D.amgValTotal = valTot;
    D.amgVecTotal = vecTot;
    C->amgValTotal = valTot;
    C->amgVecTotal = vecTot;
    char *base = nullptr;
    ck(cudaMalloc((void **)&base, A.off + 256), "cudaMalloc(mesh)");
    C->meshArena = base;
    ck(cudaMemcpy(base, A.host.data(), A.off, cudaMemcpyHostToDevice), "cudaMemcpy(mesh)");
    auto I32 = [&](size_t at) { return (const int32_t *)(base + at); };
    auto F64 = [&](size_t at) { return (const double *)(base + at); };
    D.own = I32(o_own); D.nbr = I32(o_nbr); D.w = F64(o_w); D.area = F64(o_area); D.deltaC = F64(o_dC);
    D.nx = F64(o_nx); D.ny = F64(o_ny); D.nz = F64(o_nz); D.sfx = F64(o_sx); D.sfy = F64(o_sy); D.sfz = F64(o_sz);
    D.ex = F64(o_ex); D.ey = F64(o_ey); D.ez = F64(o_ez);
    D.bown = I32(o_bown); D.barea = F64(o_barea); D.bdeltaC = F64(o_bdC); D.bdeltaW = F64(o_bdW);
    D.bnx = F64(o_bnx); D.bny = F64(o_bny); D.bnz = F64(o_bnz); D.bsfx = F64(o_bsx); D.bsfy = F64(o_bsy);
    D.bsfz = F64(o_bsz); D.bwall = I32(o_bwall); D.bout = I32(o_bout); D.bcU = I32(o_bcU); D.bcP = I32(o_bcP);
    D.bcK = I32(o_bcK); D.bcW = I32(o_bcW); D.bcPp = I32(o_bcPp); D.bvUx = F64(o_bvUx); D.bvUy = F64(o_bvUy);
    D.bvUz = F64(o_bvUz); D.bvP = F64(o_bvP); D.bvK = F64(o_bvK); D.bvW = F64(o_bvW);
    D.vol = F64(o_vol); D.wd = F64(o_wd); D.cfOff = I32(o_cfOff); D.cfFace = I32(o_cfFace); D.cfOther = I32(o_cfOther);
    D.cbOff = I32(o_cbOff); D.cbFace = I32(o_cbFace); D.cbpOff = I32(o_cbpOff); D.cbpFace = I32(o_cbpFace);
    D.pinFace = I32(o_pin);
    D.aOverD = F64(o_aod);
    D.r0Ent = I32(o_r0Ent);
    D.wf0Off = I32(o_wf0Off);
    D.wf0Rows = I32(o_wf0Rows);
    D.baOverD = F64(o_baod);
    auto F32 = [&](size_t at) { return (const float *)(base + at); };
    btm::DevGeom32 &G = D.g32;
    G.w = F32(g_w); G.area = F32(g_area); G.rdelta = F32(g_rdel); G.nx = F32(g_nx); G.ny = F32(g_ny);
    G.nz = F32(g_nz); G.ex = F32(g_ex); G.ey = F32(g_ey); G.ez = F32(g_ez); G.barea = F32(g_barea);
    G.brdelta = F32(g_brdel); G.bnx = F32(g_bnx); G.bny = F32(g_bny); G.bnz = F32(g_bnz); G.vol = F32(g_vol);
    G.rvol = F32(g_rvol); G.wd = F32(g_wd);
    for (int l = 0; l < nL; ++l) {
        btm::AmgLevelDev &dl = D.lev[l];
        dl.rowPtr = I32(lo[l].rowPtr); dl.colIdx = I32(lo[l].colIdx); dl.diagPos = I32(lo[l].diagPos);
        dl.gOff = I32(lo[l].gOff); dl.gIdx = I32(lo[l].gIdx); dl.map = I32(lo[l].map);
        dl.aggOff = I32(lo[l].aggOff); dl.aggMem = I32(lo[l].aggMem);
        dl.colorOff = I32(lo[l].colorOff); dl.colorRows = I32(lo[l].colorRows);
    }
    ck(cudaMalloc((void **)&C->dMeshPtr, sizeof(btm::DevMesh)), "cudaMalloc(DevMesh)");
    ck(cudaMemcpy(C->dMeshPtr, &D, sizeof D, cudaMemcpyHostToDevice), "cudaMemcpy(DevMesh)");
}

// Carve one instance slab (fields + work + AMG + control words).
void make_slab(btm_case *C, Slab &S) {
    const int nC = C->nC, nIF = C->nIF, nB = C->nB;
    const int nc = C->dmesh.coarseDirect ? C->amgCoarseN : 1;  // dense inverse only when small
    const size_t al = 32;  // doubles: 256-byte alignment
    auto up = [&](size_t n) { return (n + al - 1) & ~(al - 1); };
    size_t cell = up(nC), face = up(std::max(nIF, 1)), bnd = up(std::max(nB, 1));
    size_t doubles = 0;
    doubles += 38 * cell;                     // cell arrays
    doubles += cell + 2 * face;               // diag|upper|lower (contiguous, unpadded inside)
    doubles += face;                          // fflux
    doubles += 7 * bnd;                       // boundary arrays
    doubles += up(C->amgValTotal) + 3 * up(C->amgVecTotal) + up(nC + C->amgVecTotal);
    doubles += up((size_t)nc * nc) + up((size_t)4 * nc * nc);
    int gridBlocks = C->maxGridBlocks > 0 ? C->maxGridBlocks : 1024;
    doubles += up((size_t)2 * gridBlocks * btm::kRedSlots);
    doubles += 32;                            // outLast
    size_t bytes = doubles * 8 + 1024;        // + control words
    char *base = nullptr;
    ck(cudaMalloc((void **)&base, bytes), "cudaMalloc(instance)");
    S.dptr = base;
    S.bytes = bytes;
    btm::DevInst &I = S.inst;
    std::memset(&I, 0, sizeof I);
    double *d = (double *)base;
    auto take = [&](size_t n) { double *p = d; d += up(n); return p; };
    double **cells[] = {&I.ux, &I.uy, &I.uz, &I.p, &I.k, &I.om, &I.nut, &I.f1, &I.f2, &I.pk, &I.cdkw, &I.smag,
                        &I.gpx, &I.gpy, &I.gpz, &I.src, &I.aPx, &I.pp, &I.kold, &I.omold, &I.r, &I.rh,
                        &I.pv, &I.v, &I.s, &I.t, &I.ph, &I.sh, &I.rd};
    for (double **pp : cells) *pp = take(nC);
    for (int q = 0; q < 9; ++q) I.g[q] = take(nC);
    I.diag = d;
    I.upper = d + nC;
    I.lower = d + nC + nIF;
    d += up((size_t)nC + 2 * (size_t)nIF);
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
    I.gpart = take((size_t)2 * gridBlocks * btm::kRedSlots);
    I.outLast = take(32);
    char *ctl = (char *)d;
    I.barrier = (unsigned int *)ctl;
    I.err = (int32_t *)(ctl + 64);
    I.out = (int32_t *)(ctl + 128);
    I.outInner = (int64_t *)(ctl + 192);
    I.outTime = (uint64_t *)(ctl + 256);
    I.M = C->dMeshPtr;
    if ((size_t)(ctl + 512 - base) > bytes) throw BtmError(BTM_ERR_INTERNAL, "slab overflow");
}

// FP32 bulk of a slab for the mixed-precision engine, allocated on the first
// mixed solve that uses the slab.
void ensure_mixed(btm_case *C, Slab &S) {
    if (S.dptr32) return;
    const int nC = C->nC, nIF = C->nIF, nB = C->nB;
    const int nc = C->dmesh.coarseDirect ? C->amgCoarseN : 1;
    const size_t al = 64;  // floats: 256-byte alignment
    auto up = [&](size_t n) { return (n + al - 1) & ~(al - 1); };
    const size_t cell = up(nC), face = up(std::max(nIF, 1)), bnd = up(std::max(nB, 1));
    size_t floats = 0;
    floats += 32 * cell;                      // cell arrays
    floats += up((size_t)nC + 2 * (size_t)nIF) + 2 * face + bnd;
    floats += up(std::max<int64_t>(C->amgValTotal, 1)) + 3 * up(std::max<int64_t>(C->amgVecTotal, 1)) +
              up((size_t)nC + C->amgVecTotal) + up((size_t)2 * nc * nc) + up((size_t)8 * nc * nc);
    floats += 2 * face + 2 * cell;            // FP64 mass flux [nIF] and right-hand side [nC]
    floats += up((size_t)nC * (2 * btm::kBandMax + 1)) + cell;   // banded Cholesky factor (two layouts), 1 / diagonal
    const size_t aaLen = (size_t)btm::kAaFields * nC;             // Anderson vectors
    floats += 2 * up(2 * aaLen) + up(aaLen) + 2 * up(btm::kAndersonMax * aaLen);
    const size_t bytes = floats * 4 + 512;
    char *base = nullptr;
    ck(cudaMalloc((void **)&base, bytes), "cudaMalloc(instance fp32)");
    S.dptr32 = base;
    S.bytes32 = bytes;
    btm::DevWork32 &F = S.inst.f;
    float *d = (float *)base;
    auto take = [&](size_t n) { float *p = d; d += up(n); return p; };
    float **cells[] = {&F.nut, &F.f1, &F.f2, &F.pk, &F.cdkw, &F.smag, &F.src, &F.aPx, &F.pp, &F.r, &F.rh,
                       &F.pv, &F.v, &F.s, &F.t, &F.ph, &F.sh, &F.rd, &F.x};
    for (float **pp : cells) *pp = take(nC);
    for (int q = 0; q < 9; ++q) F.g[q] = take(nC);
    for (int q = 0; q < 3; ++q) F.gp[q] = take(nC);
    F.diag = d;
    F.upper = d + nC;
    F.lower = d + nC + nIF;
    d += up((size_t)nC + 2 * (size_t)nIF);
    F.tflux = take(std::max(nIF, 1));
    F.dcoef = take(std::max(nIF, 1));
    F.ppb = take(std::max(nB, 1));
    F.amgVal = take(std::max<int64_t>(C->amgValTotal, 1));
    F.amgX = take(std::max<int64_t>(C->amgVecTotal, 1));
    F.amgB = take(std::max<int64_t>(C->amgVecTotal, 1));
    F.amgR = take(std::max<int64_t>(C->amgVecTotal, 1));
    F.amgRd = take((size_t)nC + C->amgVecTotal);
    F.ainv = (double *)take((size_t)2 * nc * nc);
    F.gj = (double *)take((size_t)8 * nc * nc);
    F.mflux = (double *)take(2 * (size_t)std::max(nIF, 1));
    F.src64 = (double *)take(2 * (size_t)nC);
    F.band = take((size_t)nC * (2 * btm::kBandMax + 1));
    F.bandRd = take(nC);
    F.aaX = (double *)take(2 * aaLen);
    F.aaGprev = (double *)take(2 * aaLen);
    F.aaFprev = take(aaLen);
    F.aaDF = take(btm::kAndersonMax * aaLen);
    F.aaDG = take(btm::kAndersonMax * aaLen);
    if ((size_t)((char *)d - base) > bytes) throw BtmError(BTM_ERR_INTERNAL, "fp32 slab overflow");
}

// Observation outputs [n_obs + 1] of a slab, allocated on the first solve
// that asks for predictions.
void ensure_obs(btm_case *C, Slab &S, bool want) {
    const int n = C->dmesh.obs.n;
    if (!want || n == 0) {
        S.inst.obsOut = nullptr;
        return;
    }
    if (S.obsCap < n + 1) {
        if (S.dObs) cudaFree(S.dObs);
        S.dObs = nullptr;
        S.obsCap = 0;
        ck(cudaMalloc((void **)&S.dObs, sizeof(double) * (n + 1)), "cudaMalloc(observations)");
        S.obsCap = n + 1;
    }
    S.inst.obsOut = S.dObs;
}

void download_obs(btm_case *C, const btm::DevInst &I, btm_history *h, cudaStream_t st) {
    if (!I.obsOut || !h || !h->predictions) return;
    const int n = C->dmesh.obs.n;
    std::vector<double> v(n + 1);
    ck(cudaMemcpyAsync(v.data(), I.obsOut, sizeof(double) * (n + 1), cudaMemcpyDeviceToHost, st), "observations");
    ck(cudaStreamSynchronize(st), "observations");
    for (int k = 0; k < n; ++k) h->predictions[k] = v[k];
    h->log_lik = v[n];
}

void free_slab(Slab &S) {
    if (S.dptr) cudaFree(S.dptr);
    if (S.dptr32) cudaFree(S.dptr32);
    if (S.dObs) cudaFree(S.dObs);
    if (S.dInj) cudaFree(S.dInj);
    if (S.dRamg) cudaFree(S.dRamg);
    S = Slab();
}

void ensure_inj(btm_case *C, Slab &S) {
    if (!C->dmesh.bTarget) {
        S.inst.inj = nullptr;
        return;
    }
    if (!S.dInj) ck(cudaMalloc((void **)&S.dInj, sizeof(double) * 9 * (size_t)C->nC), "cudaMalloc(injection)");
    S.inst.inj = S.dInj;
}

// Reference-order AMG (btm_ramg.cuh): used by FP64 solves on one-CTA meshes
// when asked for, or automatically when the level-0 forward Gauss-Seidel
// needs at most kAutoRefAmgWavefronts wavefronts (unstructured or renumbered
// meshes; grid-ordered meshes would serialise into ~nx + ny wavefronts).
constexpr int kAutoRefAmgWavefronts = 32;
int use_ref_amg(const btm_case *C) {
    const btm_settings &s = C->settings;
    if (C->nC > block_max_cells() || s.precision != BTM_PREC_FP64) return 0;
    if (s.pressure_solver != BTM_LS_AMG && s.momentum_solver != BTM_LS_AMG && s.turbulence_solver != BTM_LS_AMG)
        return 0;
    if (s.amg_order == BTM_AMG_REFERENCE) return 1;
    if (s.amg_order == BTM_AMG_MULTICOLOUR) return 0;
    return C->dmesh.nWf0 <= kAutoRefAmgWavefronts ? 1 : 0;
}

// Pools of the reference-order AMG carved from `base` (nullptr: size only);
// returns the bytes used.
size_t ramg_layout(const btm_case *C, char *base, btm::RamgWork &W) {
    const int nC = C->nC, nnz0 = C->dmesh.nnz0;
    const int R = 2 * nC + 64, E = 3 * nnz0 + 256;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base ? base + off : nullptr;
        off += (bytes + 255) & ~size_t(255);
        return p;
    };
    auto D = [&](size_t n) { return (double *)take(8 * std::max<size_t>(n, 1)); };
    auto I = [&](size_t n) { return (int32_t *)take(4 * std::max<size_t>(n, 1)); };
    W.rowPool = R;
    W.entPool = E;
    W.val = D(E); W.dg = D(R); W.rd = D(nC + R); W.x = D(R); W.b = D(R); W.r = D(R); W.cv = D(nnz0);
    W.ptr = I(R + 64); W.col = I(E); W.cj = I(nnz0); W.coff = I(nC + 1);
    W.map = I(nC + R); W.memOff = I(R + 64); W.mem = I(nC + R);
    W.seed = I(nC); W.aux = I(nC); W.aux2 = I(nC);
    W.wfOff = I(R + 64); W.wfRows = I(R);
    W.lev = I((btm::kMaxLevels + 2) * 16);
    return off;
}

void ensure_ramg(btm_case *C, Slab &S) {
    if (!S.inst.S.refAmg) return;
    if (!S.dRamg) {
        btm::RamgWork W{};
        const size_t bytes = ramg_layout(C, nullptr, W);
        ck(cudaMalloc(&S.dRamg, bytes), "cudaMalloc(reference AMG)");
        S.bytesRamg = bytes;
        ramg_layout(C, (char *)S.dRamg, S.inst.rg);
    }
}

// aniso::sym3Eigenvalues + barycentricMargin (core/include/AnisotropyTools.hpp:23-67):
// descending eigenvalues of the symmetric target by the trigonometric closed
// form, then the most negative barycentric coordinate
double barycentric_margin(const double *b) {
    const double xx = b[0], yy = b[1], zz = b[2], xy = b[3], xz = b[4], yz = b[5];
    const double q = (xx + yy + zz) / 3.0;
    const double dxx = xx - q, dyy = yy - q, dzz = zz - q;
    const double p2 = (dxx * dxx + dyy * dyy + dzz * dzz + 2.0 * (xy * xy + xz * xz + yz * yz)) / 6.0;
    const double p = std::sqrt(std::max(p2, 0.0));
    double l0, l1, l2;
    if (p < 1e-30) {
        l0 = l1 = l2 = q;
    } else {
        const double inv = 1.0 / p;
        const double m00 = dxx * inv, m11 = dyy * inv, m22 = dzz * inv;
        const double m01 = xy * inv, m02 = xz * inv, m12 = yz * inv;
        double r = 0.5 * (m00 * (m11 * m22 - m12 * m12) - m01 * (m01 * m22 - m12 * m02) +
                          m02 * (m01 * m12 - m11 * m02));
        r = std::max(-1.0, std::min(1.0, r));
        const double phi = std::acos(r) / 3.0;
        l0 = q + 2.0 * p * std::cos(phi);
        l2 = q + 2.0 * p * std::cos(phi + 2.0943951023931953);
        l1 = 3.0 * q - l0 - l2;
    }
    const double c1 = l0 - l1, c2 = 2.0 * (l1 - l2), c3 = 3.0 * l2 + 1.0;
    return std::min(c1, std::min(c2, c3));
}

void fill_inst(btm_case *C, btm::DevInst &I, const double *coeffs, int variant, const btm_init *init) {
    I.S = dev_settings(C->settings);
    I.S.refAmg = use_ref_amg(C);
    I.obsOut = nullptr;
    I.inj = nullptr;
    I.nu = C->nu;
    for (int q = 0; q < 11; ++q) I.coeff[q] = coeffs[q];
    I.variant = variant;
    I.initMode = init ? init->mode : 0;
    bool zeroZ = C->is2d && C->bcZeroZ && C->settings.body_force[2] == 0.0;
    if (I.initMode == 0) {
        double u[3] = {1.0, 0.0, 0.0}, p = 0.0, k = 1e-4, w = 1.0;
        if (init) { u[0] = init->u[0]; u[1] = init->u[1]; u[2] = init->u[2]; p = init->p; k = init->k; w = init->omega; }
        I.init[0] = u[0]; I.init[1] = u[1]; I.init[2] = u[2]; I.init[3] = p; I.init[4] = k; I.init[5] = w;
        if (u[2] != 0.0) zeroZ = false;
        I.turbEstIn = 0;
    } else {
        const btm_state *ws = init->warm;
        for (int c = 0; c < C->nC && zeroZ; ++c) if (ws->U[3 * c + 2] != 0.0) zeroZ = false;
        for (int b = 0; b < C->nB && zeroZ; ++b) if (ws->Ub[3 * b + 2] != 0.0) zeroZ = false;
        I.turbEstIn = ws->turb_established;
    }
    I.solveZ = zeroZ ? 0 : 1;
    I.normFixed = 0;
}

// host staging for SoA <-> AoS conversion
void upload_state(btm_case *C, const btm::DevInst &I, const btm_state *ws, cudaStream_t st,
                  std::vector<double> &stage) {
    const int nC = C->nC, nB = C->nB;
    stage.resize((size_t)17 * std::max(nC, nB) + 16);
    auto send = [&](double *dst, const double *src, int n) {
        if (n > 0) ck(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, st), "upload");
    };
    double *h = stage.data();
    for (int c = 0; c < nC; ++c) { h[c] = ws->U[3 * c]; h[nC + c] = ws->U[3 * c + 1]; h[2 * nC + c] = ws->U[3 * c + 2]; }
    send(I.ux, h, nC); send(I.uy, h + nC, nC); send(I.uz, h + 2 * nC, nC);
    double *hb = h + 3 * nC;
    for (int b = 0; b < nB; ++b) { hb[b] = ws->Ub[3 * b]; hb[nB + b] = ws->Ub[3 * b + 1]; hb[2 * nB + b] = ws->Ub[3 * b + 2]; }
    send(I.ubx, hb, nB); send(I.uby, hb + nB, nB); send(I.ubz, hb + 2 * nB, nB);
    send(I.p, ws->p, nC); send(I.pb, ws->pb, nB);
    send(I.k, ws->k, nC); send(I.kb, ws->kb, nB);
    send(I.om, ws->omega, nC); send(I.omb, ws->omegab, nB);
    if (ws->nuT) send(I.nut, ws->nuT, nC);
    if (ws->F1) send(I.f1, ws->F1, nC);
    if (ws->F2) send(I.f2, ws->F2, nC);
    if (ws->Pk) send(I.pk, ws->Pk, nC);
    if (ws->CDkw) send(I.cdkw, ws->CDkw, nC);
    ck(cudaStreamSynchronize(st), "upload sync");
}

void download_state(btm_case *C, const btm::DevInst &I, btm_state *o, cudaStream_t st, std::vector<double> &stage) {
    const int nC = C->nC, nB = C->nB;
    stage.resize((size_t)17 * std::max(nC, nB) + 16);
    auto get = [&](double *dst, const double *src, int n) {
        if (dst && n > 0) ck(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, st), "download");
    };
    double *h = stage.data();
    if (o->U) { get(h, I.ux, nC); get(h + nC, I.uy, nC); get(h + 2 * nC, I.uz, nC); }
    double *hb = h + 3 * nC;
    if (o->Ub) { get(hb, I.ubx, nB); get(hb + nB, I.uby, nB); get(hb + 2 * nB, I.ubz, nB); }
    get(o->p, I.p, nC); get(o->pb, I.pb, nB); get(o->k, I.k, nC); get(o->kb, I.kb, nB);
    get(o->omega, I.om, nC); get(o->omegab, I.omb, nB); get(o->nuT, I.nut, nC); get(o->F1, I.f1, nC);
    get(o->F2, I.f2, nC); get(o->Pk, I.pk, nC); get(o->CDkw, I.cdkw, nC);
    ck(cudaStreamSynchronize(st), "download sync");
    if (o->U)
        for (int c = 0; c < nC; ++c) { o->U[3 * c] = h[c]; o->U[3 * c + 1] = h[nC + c]; o->U[3 * c + 2] = h[2 * nC + c]; }
    if (o->Ub)
        for (int b = 0; b < nB; ++b) { o->Ub[3 * b] = hb[b]; o->Ub[3 * b + 1] = hb[nB + b]; o->Ub[3 * b + 2] = hb[2 * nB + b]; }
}

// Launch-shape policy (overridable for tuning): instances up to
// BTM_BLOCK_MAX_CELLS cells run one CTA each; CTAs have 256 threads (two
// instances per SM) when every instance in the launch has at most
// BTM_SMALL_CELLS cells, else 512.
int env_int(const char *name, int dflt) {
    const char *e = std::getenv(name);
    return e ? std::atoi(e) : dflt;
}
int block_max_cells() {
    static int v = env_int("BTM_BLOCK_MAX_CELLS", 16384);
    return v;
}
int block_threads_for(int maxCells) {
    static int forced = env_int("BTM_BLOCK_THREADS", 0);
    static int small = env_int("BTM_SMALL_CELLS", 1024);
    if (forced == 256 || forced == 512) return forced;
    return maxCells <= small ? 256 : 512;
}

// ---- launch-shape autotuner ---------------------------------------------------
// A case that runs one CTA per instance (block mode) can launch 256-thread
// CTAs (two per SM with the engines' 128 registers per thread) or 512-thread
// CTAs (one per SM).  On its first solve the tuner times both on a probe
// batch of up to two instances per SM (cold starts of the case with the
// request's coefficients, kTuneIters outer iterations, convergence test off,
// on slabs allocated for the probe and freed after it) and keeps the faster
// for the case and engine.  The choice belongs to the case, not to a batch,
// so an instance's reductions (and its result bits) are the same alone and
// in any batch.  BTM_BLOCK_THREADS=256|512 forces a shape, BTM_AUTOTUNE=0
// keeps the size rule (256 threads up to BTM_SMALL_CELLS cells).
constexpr int kTuneIters = 40;
constexpr int kTuneRepeats = 2;                     // timed launches per shape
constexpr size_t kTuneBytes = size_t(512) << 20;   // device memory the probe slabs may take

int case_threads(const btm_case *C, int engine) {
    static int forced = env_int("BTM_BLOCK_THREADS", 0);
    if (forced == 256 || forced == 512) return forced;
    if (C->tunedThreads[engine] > 0) return C->tunedThreads[engine];
    return block_threads_for(C->nC);
}

void autotune_case(btm_case *C, const double *coeffs, int variant) {
    static int enabled = env_int("BTM_AUTOTUNE", 1);
    const int engine = C->settings.precision == BTM_PREC_MIXED ? 1 : 0;
    if (!enabled || C->tunedThreads[engine] != 0 || C->nC > block_max_cells() || C->dmesh.bTarget) return;
    int dev = 0, sms = 1;
    ck(cudaGetDevice(&dev), "device");
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    std::vector<Slab> probe(1);
    make_slab(C, probe[0]);
    if (engine == 1) ensure_mixed(C, probe[0]);
    const size_t per = probe[0].bytes + probe[0].bytes32;
    const int nProbe = (int)std::max<size_t>(1, std::min<size_t>(2 * (size_t)sms, kTuneBytes / std::max<size_t>(per, 1)));
    cudaStream_t st = C->stream;
    btm::DevInst *d = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    auto release = [&]() {
        cudaStreamSynchronize(st);
        for (Slab &S : probe) free_slab(S);
        if (d) cudaFree(d);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    };
    try {
        probe.resize(nProbe);
        std::vector<btm::DevInst> arr;
        bool refAmg = false;
        for (int q = 0; q < nProbe; ++q) {
            Slab &S = probe[q];
            if (!S.dptr) make_slab(C, S);
            if (engine == 1) ensure_mixed(C, S);
            fill_inst(C, S.inst, coeffs, variant, nullptr);
            S.inst.S.maxIter = kTuneIters;
            S.inst.S.convTol = 0.0;
            ensure_ramg(C, S);
            refAmg = refAmg || S.inst.S.refAmg;
            ck(cudaMemsetAsync(S.inst.barrier, 0, 512, st), "memset control");
            arr.push_back(S.inst);
        }
        ck(cudaMalloc((void **)&d, sizeof(btm::DevInst) * nProbe), "cudaMalloc(tune insts)");
        ck(cudaMemcpyAsync(d, arr.data(), sizeof(btm::DevInst) * nProbe, cudaMemcpyHostToDevice, st), "tune insts");
        ck(cudaEventCreate(&ev[0]), "event");
        ck(cudaEventCreate(&ev[1]), "event");
        const size_t smem = engine == 1 ? btm::mixed_smem_bytes(C->nC, C->nIF, C->amgVecTotal, C->amgValTotal,
                                                                C->dmesh.coarseDirect ? C->amgCoarseN : 1, C->dmesh.band)
                                        : 0;
        const int shapes[2] = {256, 512};
        auto launch = [&](int k, int n) {
            const int e = engine == 0 ? btm::engine_launch_block(d, n, shapes[k], st, refAmg, C->nC)
                                      : btm::mixed_launch_block(d, n, shapes[k], smem, st);
            if (e) throw BtmError(BTM_ERR_CUDA, std::string("tune launch: ") + cudaGetErrorString((cudaError_t)e));
        };
        // one untimed single-instance launch per shape first (module load,
        // shared-memory attributes), then each shape timed twice in
        // alternating order; the faster time of each counts
        for (int k = 0; k < 2; ++k) launch(k, 1);
        ck(cudaStreamSynchronize(st), "tune");
        float ms[2] = {0.0f, 0.0f};
        for (int rep = 0; rep < 2 * kTuneRepeats; ++rep) {
            const int k = (rep & 1) ^ ((rep >> 1) & 1);   // 256, 512, 512, 256, ...
            ck(cudaEventRecord(ev[0], st), "event");
            launch(k, nProbe);
            ck(cudaEventRecord(ev[1], st), "event");
            ck(cudaStreamSynchronize(st), "tune");
            float t = 0.0f;
            ck(cudaEventElapsedTime(&t, ev[0], ev[1]), "event time");
            if (ms[k] == 0.0f || t < ms[k]) ms[k] = t;
        }
        C->tuneMs[engine][0] = ms[0];
        C->tuneMs[engine][1] = ms[1];
        C->tuneProbe[engine] = nProbe;
        C->tunedThreads[engine] = ms[1] < ms[0] ? 512 : 256;
    } catch (...) {
        release();
        throw;
    }
    release();
}

struct Job {
    btm_case *C;
    Slab *S;
    int idx;
};

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *btm_last_error(void) { return g_err.c_str(); }

int btm_case_launch_shape(const btm_case *c, int32_t precision, int32_t *threads, int32_t *tuned, int32_t *probe,
                          double *probe_ms) {
    if (!c || !threads || (precision != BTM_PREC_FP64 && precision != BTM_PREC_MIXED))
        return fail(BTM_ERR_ARG, "bad argument");
    const int engine = precision == BTM_PREC_MIXED ? 1 : 0;
    *threads = c->nC > block_max_cells() ? 0 : case_threads(c, engine);
    if (tuned) *tuned = c->tunedThreads[engine] > 0 ? 1 : 0;
    if (probe) *probe = c->tuneProbe[engine];
    if (probe_ms) { probe_ms[0] = c->tuneMs[engine][0]; probe_ms[1] = c->tuneMs[engine][1]; }
    return BTM_OK;
}
double btm_last_launch_ms(void) { return g_launch_ms; }
int btm_abi_version(void) { return BTM_ABI_VERSION; }

// Test hook: the host AMG hierarchy btm_case_create builds for `mesh` (no
// device involved).  grid: 1 / 0 treat the mesh as a cooperative-grid mesh or
// not, -1 decide by size.  Outputs: the level count, each level's size, the
// aggregation maps of the levels that have one (concatenated, level 0 first)
// and level 0's CSR (rows sorted by column; values of the geometric pressure
// Laplacian the aggregation runs on).  Pass NULL arrays to query the sizes:
// *maps_len and *nnz0 are always set.
int btm_debug_amg_hierarchy(const btm_mesh *mesh, const btm_patch_bc *bcs, int32_t grid, int32_t *n_levels,
                            int32_t *sizes, int32_t *maps, int32_t *maps_len, int32_t *row_ptr0, int32_t *col0,
                            double *val0, int32_t *nnz0) {
    if (!mesh || !n_levels || !maps_len || !nnz0 || (mesh->n_patches > 0 && !bcs))
        return fail(BTM_ERR_ARG, "null argument");
    btm_case *C = new btm_case();
    try {
        std::vector<HLevel> lv;
        build_case(C, mesh, bcs, &lv, grid);
        *n_levels = (int32_t)lv.size();
        int32_t len = 0;
        for (const HLevel &L : lv) len += (int32_t)L.map.size();
        *maps_len = len;
        *nnz0 = (int32_t)lv[0].colIdx.size();
        if (sizes)
            for (size_t l = 0; l < lv.size(); ++l) sizes[l] = lv[l].n;
        if (maps) {
            int32_t at = 0;
            for (const HLevel &L : lv)
                for (int v : L.map) maps[at++] = v;
        }
        if (row_ptr0) std::copy(lv[0].rowPtr.begin(), lv[0].rowPtr.end(), row_ptr0);
        if (col0) std::copy(lv[0].colIdx.begin(), lv[0].colIdx.end(), col0);
        if (val0) std::copy(lv[0].val.begin(), lv[0].val.end(), val0);
    } catch (const BtmError &e) {
        delete C;
        return fail(e.code, e.what());
    } catch (const std::exception &e) {
        delete C;
        return fail(BTM_ERR_INTERNAL, e.what());
    }
    delete C;
    return BTM_OK;
}

int btm_case_create(const btm_mesh *mesh, const btm_patch_bc *bcs, double nu, const btm_settings *settings,
                    btm_case **out) {
    if (!mesh || !settings || !out || (mesh->n_patches > 0 && !bcs)) return fail(BTM_ERR_ARG, "null argument");
    *out = nullptr;
    // argument errors first, with or without a device
    try {
        check_settings(*settings);
    } catch (const BtmError &e) {
        return fail(e.code, e.what());
    }
    if (int e = ensure_device()) return e;
    btm_case *C = new btm_case();
    try {
        C->nu = nu;
        C->settings = *settings;
        int blocks = 0;
        if (btm::engine_grid_blocks(&blocks) != 0) throw BtmError(BTM_ERR_CUDA, "occupancy query failed");
        C->maxGridBlocks = blocks;
        build_case(C, mesh, bcs);
        ck(cudaStreamCreateWithFlags(&C->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    } catch (const BtmError &e) {
        btm_case_destroy(C);
        return fail(e.code, e.what());
    } catch (const std::exception &e) {
        btm_case_destroy(C);
        return fail(BTM_ERR_INTERNAL, e.what());
    }
    *out = C;
    return BTM_OK;
}

void btm_case_destroy(btm_case *C) {
    if (!C) return;
    for (Slab &s : C->slabs) free_slab(s);
    if (C->meshArena) cudaFree(C->meshArena);
    if (C->obsArena) cudaFree(C->obsArena);
    if (C->injTarget) cudaFree(C->injTarget);
    if (C->dMeshPtr) cudaFree(C->dMeshPtr);
    if (C->stream) cudaStreamDestroy(C->stream);
    delete C;
}

int btm_case_info(const btm_case *C, int32_t *n_cells, int32_t *n_boundary_faces, int32_t *n_amg_levels,
                  int32_t *is_2d) {
    if (!C) return fail(BTM_ERR_ARG, "null case");
    if (n_cells) *n_cells = C->nC;
    if (n_boundary_faces) *n_boundary_faces = C->nB;
    if (n_amg_levels) *n_amg_levels = C->dmesh.nLevels;
    if (is_2d) *is_2d = C->is2d ? 1 : 0;
    return BTM_OK;
}

int btm_case_set_settings(btm_case *C, const btm_settings *s) {
    if (!C || !s) return fail(BTM_ERR_ARG, "null argument");
    try {
        check_settings(*s);
    } catch (const BtmError &e) {
        return fail(e.code, e.what());
    }
    bool rc = (!C->dmesh.hasOutlet || s->rhie_chow_all_meshes) ? 1 : 0;
    if (rc != (C->dmesh.rhieChow != 0)) {
        C->dmesh.rhieChow = rc;
        cudaError_t e = cudaMemcpy(C->dMeshPtr, &C->dmesh, sizeof C->dmesh, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(BTM_ERR_CUDA, cudaGetErrorString(e));
    }
    C->settings = *s;
    return BTM_OK;
}

// ForwardModel::setTargetAnisotropy (incompressible/src/ForwardModel.cpp:22-26)
// for the case: the target on the device and its realizability, checked once
// (SIMPLESolver.cpp:295-307 re-checks the same constant target every outer
// iteration).
int btm_case_set_target_anisotropy(btm_case *C, const double *b6) {
    if (!C) return fail(BTM_ERR_ARG, "null case");
    try {
        double *dT = nullptr;
        bool allReal = true;
        double maxViol = 0.0;
        if (b6) {
            for (size_t i = 0; i < 6 * (size_t)C->nC; ++i)
                if (!std::isfinite(b6[i])) throw BtmError(BTM_ERR_ARG, "target anisotropy has a non-finite entry");
            for (int c = 0; c < C->nC; ++c) {
                const double margin = barycentric_margin(b6 + 6 * (size_t)c);
                if (margin < -1e-6) {
                    allReal = false;
                    maxViol = std::max(maxViol, -margin);
                }
            }
            ck(cudaMalloc((void **)&dT, sizeof(double) * 6 * (size_t)C->nC), "cudaMalloc(target anisotropy)");
            cudaError_t e = cudaMemcpy(dT, b6, sizeof(double) * 6 * (size_t)C->nC, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) {
                cudaFree(dT);
                throw BtmError(BTM_ERR_CUDA, cudaGetErrorString(e));
            }
        }
        btm::DevMesh D = C->dmesh;
        D.bTarget = dT;
        cudaError_t e = cudaMemcpy(C->dMeshPtr, &D, sizeof D, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (dT) cudaFree(dT);
            throw BtmError(BTM_ERR_CUDA, cudaGetErrorString(e));
        }
        if (C->injTarget) cudaFree(C->injTarget);
        C->injTarget = dT;
        C->dmesh = D;
        C->injAllRealizable = allReal;
        C->injMaxViolation = maxViol;
    } catch (const BtmError &e) {
        return fail(e.code, e.what());
    } catch (const std::exception &e) {
        return fail(BTM_ERR_INTERNAL, e.what());
    }
    return BTM_OK;
}

int btm_case_injection_realizability(const btm_case *C, int32_t *active, int32_t *all_realizable,
                                     double *max_violation) {
    if (!C) return fail(BTM_ERR_ARG, "null case");
    if (active) *active = C->dmesh.bTarget ? 1 : 0;
    if (all_realizable) *all_realizable = C->injAllRealizable ? 1 : 0;
    if (max_violation) *max_violation = C->injMaxViolation;
    return BTM_OK;
}

// ObservationOperator::evaluate's searches and constants
// (core/include/ObservationOperator.hpp:159-364), resolved once per case:
// nearest cell / nearest patch face by squared distance, first minimum wins;
// q_ref = 0.5 U_ref^2 (times rho for a tap); wall distances floored at 1e-20.
int btm_case_set_observations(btm_case *C, const btm_mesh *m, int32_t n, const btm_observable *obs) {
    if (!C || n < 0 || (n > 0 && (!m || !obs))) return fail(BTM_ERR_ARG, "null argument");
    try {
        btm::ObsDev O{};
        void *arena = nullptr;
        if (n > 0) {
            if (m->n_cells != C->nC || m->n_faces != C->nF || m->n_internal_faces != C->nIF)
                throw BtmError(BTM_ERR_ARG, "btm_case_set_observations: mesh does not match the case");
            const int nIF = m->n_internal_faces;
            std::vector<int32_t> kind(n), at(n), cnt(n), comp(n);
            std::vector<double> observed(n), var(n), c0(n, 1.0), c1(n, 0.0);
            std::vector<int32_t> fOwn, fBnd;
            std::vector<double> fNx, fNy, fNz, fArea, fDelta, fX;
            auto list_face = [&](int f) {
                fOwn.push_back(m->owner[f]);
                fBnd.push_back(f - nIF);
                fNx.push_back(m->face_normal[3 * f]);
                fNy.push_back(m->face_normal[3 * f + 1]);
                fNz.push_back(m->face_normal[3 * f + 2]);
                fArea.push_back(m->face_area[f]);
                fDelta.push_back(std::max(m->face_delta[f], 1e-20));
                fX.push_back(m->face_center[3 * f]);
            };
            auto dist2 = [](const double *c, const double *loc) {
                const double d0 = c[0] - loc[0], d1 = c[1] - loc[1], d2 = c[2] - loc[2];
                const double a = d0 * d0, b = d1 * d1, e = d2 * d2;
                return (a + b) + e;
            };
            for (int k = 0; k < n; ++k) {
                const btm_observable &o = obs[k];
                if (o.type < BTM_OBS_DRAG || o.type > BTM_OBS_REATTACHMENT)
                    throw BtmError(BTM_ERR_ARG, "btm_case_set_observations: unknown observable type");
                kind[k] = o.type;
                observed[k] = o.observed;
                const double so = o.sigma_obs * o.sigma_obs, sm = o.sigma_model * o.sigma_model;
                var[k] = so + sm;
                if (var[k] < 1e-30) var[k] = 1e-30;
                comp[k] = o.component == 0 ? 0 : (o.component == 1 ? 1 : 2);
                const double qref = (0.5 * o.ref_velocity) * o.ref_velocity;
                if (o.type == BTM_OBS_PRESSURE_TAP || o.type == BTM_OBS_VELOCITY) {
                    int best = 0;
                    double bd = 0.0;
                    for (int c = 0; c < m->n_cells; ++c) {
                        const double d = dist2(m->cell_center + 3 * c, o.location);
                        if (c == 0 || d < bd) { bd = d; best = c; }
                    }
                    at[k] = best;
                    cnt[k] = 0;
                    if (o.type == BTM_OBS_PRESSURE_TAP) {
                        const double q = ((0.5 * o.ref_density) * o.ref_velocity) * o.ref_velocity;
                        c0[k] = std::max(q, 1e-20);
                        c1[k] = o.ref_pressure;
                    }
                    continue;
                }
                if (o.patch < 0 || o.patch >= m->n_patches)
                    throw BtmError(BTM_ERR_ARG, "btm_case_set_observations: patch index out of range");
                const int p0 = m->patch_offset[o.patch], p1 = m->patch_offset[o.patch + 1];
                for (int q = p0; q < p1; ++q)
                    if (m->patch_faces[q] < nIF || m->patch_faces[q] >= m->n_faces)
                        throw BtmError(BTM_ERR_ARG, "btm_case_set_observations: patch face is not a boundary face");
                at[k] = (int)fOwn.size();
                if (o.type == BTM_OBS_SKIN_FRICTION) {
                    cnt[k] = p1 > p0 ? 1 : 0;
                    c0[k] = std::max(qref, 1e-20);
                    if (p1 > p0) {
                        int best = p0;
                        double bd = 0.0;
                        for (int q = p0; q < p1; ++q) {
                            const double d = dist2(m->face_center + 3 * m->patch_faces[q], o.location);
                            if (q == p0 || d < bd) { bd = d; best = q; }
                        }
                        list_face(m->patch_faces[best]);
                    }
                    continue;
                }
                cnt[k] = p1 - p0;
                for (int q = p0; q < p1; ++q) list_face(m->patch_faces[q]);
                if (o.type == BTM_OBS_DRAG) c0[k] = qref * o.ref_area;
                if (o.type == BTM_OBS_REATTACHMENT) c1[k] = p1 > p0 ? m->face_center[3 * m->patch_faces[p1 - 1]] : 0.0;
            }
            const size_t nf = std::max<size_t>(fOwn.size(), 1);
            const size_t al = 32;  // doubles: 256-byte alignment
            auto up = [&](size_t x) { return (x + al - 1) & ~(al - 1); };
            const size_t words = 4 * up(n) + 4 * up(n) + 2 * up(nf) + 6 * up(nf);
            ck(cudaMalloc(&arena, words * 8), "cudaMalloc(observation plan)");
            char *d = (char *)arena;
            auto put = [&](const void *src, size_t bytes, size_t cap) {
                char *p = d;
                if (bytes) ck(cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice), "cudaMemcpy(observation plan)");
                d += cap * 8;
                return (void *)p;
            };
            O.n = n;
            O.kind = (const int32_t *)put(kind.data(), 4 * n, up(n));
            O.at = (const int32_t *)put(at.data(), 4 * n, up(n));
            O.cnt = (const int32_t *)put(cnt.data(), 4 * n, up(n));
            O.comp = (const int32_t *)put(comp.data(), 4 * n, up(n));
            O.observed = (const double *)put(observed.data(), 8 * n, up(n));
            O.var = (const double *)put(var.data(), 8 * n, up(n));
            O.c0 = (const double *)put(c0.data(), 8 * n, up(n));
            O.c1 = (const double *)put(c1.data(), 8 * n, up(n));
            O.fOwn = (const int32_t *)put(fOwn.data(), 4 * fOwn.size(), up(nf));
            O.fBnd = (const int32_t *)put(fBnd.data(), 4 * fBnd.size(), up(nf));
            O.fNx = (const double *)put(fNx.data(), 8 * fNx.size(), up(nf));
            O.fNy = (const double *)put(fNy.data(), 8 * fNy.size(), up(nf));
            O.fNz = (const double *)put(fNz.data(), 8 * fNz.size(), up(nf));
            O.fArea = (const double *)put(fArea.data(), 8 * fArea.size(), up(nf));
            O.fDelta = (const double *)put(fDelta.data(), 8 * fDelta.size(), up(nf));
            O.fX = (const double *)put(fX.data(), 8 * fX.size(), up(nf));
            if ((size_t)(d - (char *)arena) > words * 8) throw BtmError(BTM_ERR_INTERNAL, "observation plan overflow");
        }
        btm::DevMesh D = C->dmesh;
        D.obs = O;
        cudaError_t e = cudaMemcpy(C->dMeshPtr, &D, sizeof D, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (arena) cudaFree(arena);
            throw BtmError(BTM_ERR_CUDA, cudaGetErrorString(e));
        }
        if (C->obsArena) cudaFree(C->obsArena);
    if (C->injTarget) cudaFree(C->injTarget);
        C->obsArena = arena;
        C->dmesh = D;
    } catch (const BtmError &e) {
        return fail(e.code, e.what());
    } catch (const std::exception &e) {
        return fail(BTM_ERR_INTERNAL, e.what());
    }
    return BTM_OK;
}

// Per-call device buffers and events of btm_solve_batch, released when the
// call returns or throws (cudaFree waits for work still using them).
struct CallResources {
    std::vector<void *> dev;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> joins;   // fork / join events of concurrent group launches
    CallResources() = default;
    CallResources(const CallResources &) = delete;
    CallResources &operator=(const CallResources &) = delete;
    ~CallResources() {
        for (void *p : dev)
            if (p) cudaFree(p);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : joins)
            if (e) cudaEventDestroy(e);
    }
};

// Streams on which the launch groups of one batch (instances of different
// engines or CTA sizes) run side by side: a few per device, created on first
// use and kept for the life of the process.  Calls from several host threads
// may share them; their work then queues behind each other, which changes
// timing only.
constexpr int kGroupStreams = 4;
cudaStream_t group_stream(int k) {
    static std::mutex mtx;
    static std::vector<std::array<cudaStream_t, kGroupStreams>> pool;
    int dev = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mtx);
    if ((int)pool.size() <= dev) pool.resize(dev + 1, std::array<cudaStream_t, kGroupStreams>{});
    cudaStream_t &s = pool[dev][k % kGroupStreams];
    if (!s) ck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate(group)");
    return s;
}

int btm_solve_batch(int32_t n, btm_case *const *cases, const double *coeffs, const int32_t *variants,
                    const btm_init *inits, btm_state *outs, btm_history *hists) {
    if (n < 0 || (n > 0 && (!cases || !coeffs))) return fail(BTM_ERR_ARG, "null argument");
    if (n == 0) return BTM_OK;
    if (int e = ensure_device()) return e;
    try {
        // first one-CTA solve of a case: choose its launch shape
        for (int i = 0; i < n; ++i)
            if (cases[i]) autotune_case(cases[i], coeffs + 11 * (size_t)i, variants ? variants[i] : 0);
        // take per-case slabs (reused across calls)
        std::vector<Job> jobs(n);
        std::vector<int> used;
        std::vector<btm_case *> distinct;
        for (int i = 0; i < n; ++i) {
            btm_case *C = cases[i];
            if (!C) throw BtmError(BTM_ERR_ARG, "null case in batch");
            int slot = 0;
            for (int j = 0; j < i; ++j) if (cases[j] == C) ++slot;
            while ((int)C->slabs.size() <= slot) {
                C->slabs.emplace_back();
                make_slab(C, C->slabs.back());
            }
            jobs[i] = {C, nullptr, i};
            if (std::find(distinct.begin(), distinct.end(), C) == distinct.end()) distinct.push_back(C);
        }
        std::vector<int> slotOf(n, 0);
        for (int i = 0; i < n; ++i) {
            int slot = 0;
            for (int j = 0; j < i; ++j) if (cases[j] == cases[i]) ++slot;
            jobs[i].S = &cases[i]->slabs[slot];
        }
        cudaStream_t st = cases[0]->stream;
        std::vector<double> stage;
        std::vector<btm::DevInst> hostInsts;
        std::vector<int> blockIdx, gridIdx, mixIdx;
        std::vector<std::vector<double>> histBufs(n);
        std::vector<double *> histDev(n, nullptr);
        CallResources res;
        for (int i = 0; i < n; ++i) {
            Job &J = jobs[i];
            btm::DevInst &I = J.S->inst;
            const btm_init *ini = inits ? &inits[i] : nullptr;
            if (ini && ini->mode == BTM_INIT_DEVICE) {
                // continue from the state this slab holds: the kernel skips
                // initialisation, turbEstablished and the z switch carry over
                if (!J.S->hasState) throw BtmError(BTM_ERR_ARG, "device warm start before any solve of this slot");
                const int solveZ = I.solveZ;
                fill_inst(J.C, I, coeffs + 11 * (size_t)i, variants ? variants[i] : 0, nullptr);
                I.initMode = 1;
                I.turbEstIn = J.S->lastTurbEst;
                I.solveZ = solveZ;
            } else {
                if (ini && ini->mode != BTM_INIT_COLD && ini->mode != BTM_INIT_WARM)
                    throw BtmError(BTM_ERR_ARG, "unknown init mode");
                fill_inst(J.C, I, coeffs + 11 * (size_t)i, variants ? variants[i] : 0, ini);
                if (ini && ini->mode == BTM_INIT_WARM) {
                    if (!ini->warm) throw BtmError(BTM_ERR_ARG, "warm init without a state");
                    upload_state(J.C, I, ini->warm, st, stage);
                }
            }
            I.hist = nullptr;
            I.histCap = 0;
            if (hists && hists[i].residuals && hists[i].residual_capacity > 0) {
                ck(cudaMalloc((void **)&histDev[i], sizeof(double) * 6 * hists[i].residual_capacity), "cudaMalloc(hist)");
                res.dev.push_back(histDev[i]);
                I.hist = histDev[i];
                I.histCap = hists[i].residual_capacity;
            }
            ck(cudaMemsetAsync(I.barrier, 0, 512, st), "memset control");
            const bool mixed = J.C->settings.precision == BTM_PREC_MIXED;
            if (mixed) ensure_mixed(J.C, *J.S);
            ensure_obs(J.C, *J.S, hists && hists[i].predictions);
            ensure_inj(J.C, *J.S);
            ensure_ramg(J.C, *J.S);
            if (mixed && J.C->nC <= block_max_cells()) {
                mixIdx.push_back(i);
            } else if (!mixed && J.C->nC <= block_max_cells()) {
                blockIdx.push_back(i);
            } else {
                gridIdx.push_back(i);
            }
        }
        // one persistent launch per engine and launch shape for all
        // block-mode instances: an instance runs with its case's shape
        // (autotuned or by rule), whatever else is in the batch, so its
        // result is the same bits alone and in any batch
        ck(cudaEventCreate(&res.ev[0]), "event");
        ck(cudaEventCreate(&res.ev[1]), "event");
        cudaEvent_t ev0 = res.ev[0], ev1 = res.ev[1];
        btm::DevInst *dInsts = nullptr;
        const size_t nBlock = blockIdx.size() + mixIdx.size();
        if (nBlock > 0) {
            struct Group { int engine, threads; std::vector<int> idx; };
            std::vector<Group> groups;
            for (int engine = 0; engine < 2; ++engine)
                for (int threads : {256, 512}) {
                    Group g{engine, threads, {}};
                    for (int i : engine == 0 ? blockIdx : mixIdx)
                        if (case_threads(jobs[i].C, engine) == threads) g.idx.push_back(i);
                    if (!g.idx.empty()) groups.push_back(std::move(g));
                }
            std::vector<btm::DevInst> arr;
            for (const Group &g : groups)
                for (int i : g.idx) arr.push_back(jobs[i].S->inst);
            ck(cudaMalloc((void **)&dInsts, sizeof(btm::DevInst) * arr.size()), "cudaMalloc(insts)");
            res.dev.push_back(dInsts);
            ck(cudaMemcpyAsync(dInsts, arr.data(), sizeof(btm::DevInst) * arr.size(), cudaMemcpyHostToDevice, st), "insts");
            ck(cudaEventRecord(ev0, st), "event");
            // more than one group: each on its own stream, forked from and
            // joined back into the call's stream, so the groups run at the
            // same time instead of one after the other
            const bool fork = groups.size() > 1;
            size_t at = 0;
            for (size_t gi = 0; gi < groups.size(); ++gi) {
                const Group &g = groups[gi];
                cudaStream_t gs = st;
                if (fork) {
                    gs = group_stream((int)gi);
                    ck(cudaStreamWaitEvent(gs, ev0, 0), "fork");
                }
                int maxCells = 0;
                bool refAmg = false;
                size_t smem = 0;
                for (int i : g.idx) {
                    const btm_case *Cm = jobs[i].C;
                    maxCells = std::max(maxCells, Cm->nC);
                    refAmg = refAmg || jobs[i].S->inst.S.refAmg;
                    if (g.engine == 1)
                        smem = std::max(smem, btm::mixed_smem_bytes(Cm->nC, Cm->nIF, Cm->amgVecTotal, Cm->amgValTotal,
                                                                    Cm->dmesh.coarseDirect ? Cm->amgCoarseN : 1,
                                                                    Cm->dmesh.band));
                }
                const int e = g.engine == 0
                                  ? btm::engine_launch_block(dInsts + at, (int)g.idx.size(), g.threads, gs, refAmg, maxCells)
                                  : btm::mixed_launch_block(dInsts + at, (int)g.idx.size(), g.threads, smem, gs);
                if (e) throw BtmError(BTM_ERR_CUDA, std::string("block launch: ") + cudaGetErrorString((cudaError_t)e));
                if (fork) {
                    cudaEvent_t j = nullptr;
                    ck(cudaEventCreateWithFlags(&j, cudaEventDisableTiming), "event");
                    res.joins.push_back(j);
                    ck(cudaEventRecord(j, gs), "join");
                    ck(cudaStreamWaitEvent(st, j, 0), "join");
                }
                at += g.idx.size();
            }
        } else {
            ck(cudaEventRecord(ev0, st), "event");
        }
        for (int i : gridIdx) {
            btm::DevInst *dI = nullptr;
            ck(cudaMalloc((void **)&dI, sizeof(btm::DevInst)), "cudaMalloc(inst)");
            res.dev.push_back(dI);
            ck(cudaMemcpyAsync(dI, &jobs[i].S->inst, sizeof(btm::DevInst), cudaMemcpyHostToDevice, st), "inst");
            int e;
            if (jobs[i].C->settings.precision == BTM_PREC_MIXED) {
                int mb = 0;
                e = btm::mixed_grid_blocks(&mb);
                // the grid reduction buffers of the slab hold maxGridBlocks CTAs
                if (!e) e = btm::mixed_launch_grid(dI, std::min(mb, jobs[i].C->maxGridBlocks), st);
            } else {
                e = btm::engine_launch_grid(dI, jobs[i].C->maxGridBlocks, st);
            }
            if (e) throw BtmError(BTM_ERR_CUDA, std::string("grid launch: ") + cudaGetErrorString((cudaError_t)e));
        }
        ck(cudaEventRecord(ev1, st), "event");
        cudaError_t se = cudaStreamSynchronize(st);
        float ms = 0.0f;
        if (se == cudaSuccess && cudaEventElapsedTime(&ms, ev0, ev1) == cudaSuccess) g_launch_ms = ms;
        if (se != cudaSuccess) throw BtmError(BTM_ERR_CUDA, std::string("solve: ") + cudaGetErrorString(se));
        // per-instance device timestamps: [8] start, [9] end of each solve
        std::vector<std::array<uint64_t, btm::kPhaseSlots + 2>> times(n);
        uint64_t t0 = 0;
        for (int i = 0; i < n; ++i) {
            ck(cudaMemcpy(times[i].data(), jobs[i].S->inst.outTime, sizeof(uint64_t) * (btm::kPhaseSlots + 2),
                          cudaMemcpyDeviceToHost),
               "status");
            const uint64_t ts = times[i][btm::kPhaseSlots];
            if (ts && (!t0 || ts < t0)) t0 = ts;
        }
        for (int i = 0; i < n; ++i) {
            Job &J = jobs[i];
            const btm::DevInst &I = J.S->inst;
            int32_t outv[8];
            int64_t innerv[5] = {0, 0, 0, 0, 0};
            int32_t errv = 0;
            double lastv[6];
            ck(cudaMemcpy(outv, I.out, sizeof outv, cudaMemcpyDeviceToHost), "status");
            ck(cudaMemcpy(innerv, I.outInner, sizeof innerv, cudaMemcpyDeviceToHost), "status");
            ck(cudaMemcpy(lastv, I.outLast, sizeof lastv, cudaMemcpyDeviceToHost), "status");
            ck(cudaMemcpy(&errv, I.err, sizeof errv, cudaMemcpyDeviceToHost), "status");
            J.S->hasState = errv == 0;
            J.S->lastTurbEst = outv[5];
            const uint64_t *tns = times[i].data();
            if (hists) {
                btm_history &h = hists[i];
                h.status = outv[0];
                h.converged = outv[1];
                h.diverged = outv[2];
                h.final_iter = outv[3];
                h.iterations_run = outv[4];
                h.inner_iterations = innerv[0];
                for (int q = 0; q < 4; ++q) h.inner_split[q] = innerv[q + 1];
                h.polish_start = outv[7];
                for (int q = 0; q < 6; ++q) h.last_residual[q] = lastv[q];
                for (int q = 0; q < btm::kPhaseSlots; ++q) h.phase_ms[q] = 1e-6 * (double)tns[q];
                const uint64_t t1 = tns[btm::kPhaseSlots], t2 = tns[btm::kPhaseSlots + 1];
                h.solve_ms = t2 > t1 ? 1e-6 * (double)(t2 - t1) : 0.0;
                h.finish_ms = (t0 && t2 > t0) ? 1e-6 * (double)(t2 - t0) : 0.0;
                if (histDev[i]) {
                    int rows = std::min(h.residual_capacity, outv[4]);
                    ck(cudaMemcpy(h.residuals, histDev[i], sizeof(double) * 6 * rows, cudaMemcpyDeviceToHost), "hist");
                }
                download_obs(J.C, I, &h, st);
            }
            if (outs) {
                download_state(J.C, I, &outs[i], st, stage);
                outs[i].turb_established = outv[5];
            }
            if (errv) throw BtmError(BTM_ERR_TIMEOUT, "a bounded device wait timed out; the solve was abandoned");
        }
    } catch (const BtmError &e) {
        return fail(e.code, e.what());
    } catch (const std::exception &e) {
        return fail(BTM_ERR_INTERNAL, e.what());
    }
    return BTM_OK;
}

int btm_wall_distance(int32_t n_cells, const double *cell_centre, int32_t n_wall, const double *wall_centre,
                      double *out) {
    if (n_cells < 0 || n_wall < 0 || (n_cells > 0 && (!cell_centre || !out)) || (n_wall > 0 && !wall_centre))
        return fail(BTM_ERR_ARG, "bad wall-distance arguments");
    if (n_cells == 0) return BTM_OK;
    if (n_wall == 0) {
        for (int c = 0; c < n_cells; ++c) out[c] = 1e10;
        return BTM_OK;
    }
    if (int e = ensure_device()) return e;
    double *d = nullptr;
    const size_t nc = (size_t)n_cells, nw = (size_t)n_wall;
    try {
        ck(cudaMalloc((void **)&d, 8 * (3 * nc + 3 * nw + nc)), "cudaMalloc(wall distance)");
        ck(cudaMemcpy(d, cell_centre, 8 * 3 * nc, cudaMemcpyHostToDevice), "upload");
        ck(cudaMemcpy(d + 3 * nc, wall_centre, 8 * 3 * nw, cudaMemcpyHostToDevice), "upload");
        int e = btm::engine_wall_distance(d, n_cells, d + 3 * nc, n_wall, d + 3 * nc + 3 * nw, nullptr);
        if (e) throw BtmError(BTM_ERR_CUDA, std::string("wall distance: ") + cudaGetErrorString((cudaError_t)e));
        ck(cudaMemcpy(out, d + 3 * nc + 3 * nw, 8 * nc, cudaMemcpyDeviceToHost), "download");
    } catch (const BtmError &e) {
        if (d) cudaFree(d);
        return fail(e.code, e.what());
    }
    cudaFree(d);
    return BTM_OK;
}

int btm_solve(btm_case *c, const double *coeffs, int32_t variant, const btm_init *init, btm_state *out,
              btm_history *hist) {
    if (!c || !coeffs) return fail(BTM_ERR_ARG, "null argument");
    btm_case *cs[1] = {c};
    return btm_solve_batch(1, cs, coeffs, &variant, init, out, hist);
}

// Test hook: see the phase list in btm_gb300.h.  `in` packs the state
// [U(3nC) p k omega nuT F1 F2 Pk CDkw Smag aP (nC each) Ub(3nB) pb kb omegab (nB each)]
// followed by the linear system [diag(nC) upper(nIF) lower(nIF) source(nC) x(nC)].
int btm_debug_phase(btm_case *C, int32_t phase, const double *coeffs, int32_t variant, int32_t arg,
                    const double *in, int64_t n_in, double *out, int64_t n_out) {
    if (!C || !coeffs || !in || !out) return fail(BTM_ERR_ARG, "null argument");
    const int nC = C->nC, nIF = C->nIF, nB = C->nB;
    const int64_t need = 13LL * nC + 6LL * nB + 3LL * nC + 2LL * nIF;
    if (n_in < need) return fail(BTM_ERR_ARG, "debug input too small");
    if (nC > 65536) return fail(BTM_ERR_ARG, "debug phases run on one CTA: mesh too large");
    try {
        if (C->slabs.empty()) { C->slabs.emplace_back(); make_slab(C, C->slabs.back()); }
        Slab &S = C->slabs[0];
        btm::DevInst &I = S.inst;
        btm_init ini{};
        ini.mode = 1;
        fill_inst(C, I, coeffs, variant, nullptr);
        ensure_ramg(C, S);
        I.initMode = 1;
        I.dbgPhase = phase;
        I.dbgArg = arg;
        cudaStream_t st = C->stream;
        const double *q = in;
        std::vector<double> U(q, q + 3 * (size_t)nC);
        q += 3 * (size_t)nC;
        double *cellDst[] = {I.p, I.k, I.om, I.nut, I.f1, I.f2, I.pk, I.cdkw, I.smag, I.aPx};
        std::vector<double> ux(nC), uy(nC), uz(nC);
        for (int c = 0; c < nC; ++c) { ux[c] = U[3 * c]; uy[c] = U[3 * c + 1]; uz[c] = U[3 * c + 2]; }
        ck(cudaMemcpyAsync(I.ux, ux.data(), 8 * nC, cudaMemcpyHostToDevice, st), "dbg");
        ck(cudaMemcpyAsync(I.uy, uy.data(), 8 * nC, cudaMemcpyHostToDevice, st), "dbg");
        ck(cudaMemcpyAsync(I.uz, uz.data(), 8 * nC, cudaMemcpyHostToDevice, st), "dbg");
        for (double *dst : cellDst) {
            ck(cudaMemcpyAsync(dst, q, 8 * (size_t)nC, cudaMemcpyHostToDevice, st), "dbg");
            q += nC;
        }
        std::vector<double> bx(nB), by(nB), bz(nB);
        for (int b = 0; b < nB; ++b) { bx[b] = q[3 * b]; by[b] = q[3 * b + 1]; bz[b] = q[3 * b + 2]; }
        q += 3 * (size_t)nB;
        if (nB > 0) {
            ck(cudaMemcpyAsync(I.ubx, bx.data(), 8 * nB, cudaMemcpyHostToDevice, st), "dbg");
            ck(cudaMemcpyAsync(I.uby, by.data(), 8 * nB, cudaMemcpyHostToDevice, st), "dbg");
            ck(cudaMemcpyAsync(I.ubz, bz.data(), 8 * nB, cudaMemcpyHostToDevice, st), "dbg");
        }
        for (double *dst : {I.pb, I.kb, I.omb}) {
            if (nB > 0) ck(cudaMemcpyAsync(dst, q, 8 * (size_t)nB, cudaMemcpyHostToDevice, st), "dbg");
            q += nB;
        }
        ck(cudaMemcpyAsync(I.diag, q, 8 * ((size_t)nC + 2 * nIF), cudaMemcpyHostToDevice, st), "dbg");
        q += nC + 2 * (size_t)nIF;
        ck(cudaMemcpyAsync(I.src, q, 8 * (size_t)nC, cudaMemcpyHostToDevice, st), "dbg");
        q += nC;
        ck(cudaMemcpyAsync(I.pp, q, 8 * (size_t)nC, cudaMemcpyHostToDevice, st), "dbg");
        ck(cudaMemcpyAsync(I.r, q, 8 * (size_t)nC, cudaMemcpyHostToDevice, st), "dbg");
        btm::DevInst *dI = nullptr;
        ck(cudaMalloc((void **)&dI, sizeof I), "cudaMalloc(dbg)");
        ck(cudaMemcpyAsync(dI, &I, sizeof I, cudaMemcpyHostToDevice, st), "dbg");
        int e = btm::engine_launch_debug(dI, st);
        cudaError_t se = cudaStreamSynchronize(st);
        cudaFree(dI);
        if (e) throw BtmError(BTM_ERR_CUDA, cudaGetErrorString((cudaError_t)e));
        if (se != cudaSuccess) throw BtmError(BTM_ERR_CUDA, cudaGetErrorString(se));
        if (phase == BTM_PHASE_AMG_LEVELS) {
            if (!I.S.refAmg) throw BtmError(BTM_ERR_ARG, "the hierarchy phase needs amg_order = reference (FP64)");
            const btm::RamgWork &W = I.rg;
            double last[4];
            ck(cudaMemcpy(last, I.outLast, sizeof last, cudaMemcpyDeviceToHost), "dbg out");
            const int nLev = (int)last[0];
            std::vector<int32_t> lev((btm::kMaxLevels + 2) * 16);
            ck(cudaMemcpy(lev.data(), W.lev, 4 * lev.size(), cudaMemcpyDeviceToHost), "dbg out");
            auto field = [&](int l, int f) { return lev[l * btm::kRamgLevInts + f]; };
            std::vector<double> o;
            o.push_back(nLev);
            for (int l = 0; l < 21; ++l) o.push_back(l < nLev ? field(l, btm::RL_N) : 0);
            auto ints = [&](const int32_t *d, int n) {
                std::vector<int32_t> h(std::max(n, 1));
                if (n > 0) ck(cudaMemcpy(h.data(), d, 4 * (size_t)n, cudaMemcpyDeviceToHost), "dbg out");
                for (int q = 0; q < n; ++q) o.push_back(h[q]);
            };
            for (int l = 0; l + 1 < nLev; ++l) ints(W.map + field(l, btm::RL_MAP), field(l, btm::RL_N));
            for (int l = 1; l < nLev; ++l) {
                const int n = field(l, btm::RL_N), nnz = field(l, btm::RL_NNZ);
                ints(W.ptr + field(l, btm::RL_PTR), n + 1);
                ints(W.col + field(l, btm::RL_ENT), nnz);
                std::vector<double> h(std::max(nnz, 1));
                if (nnz > 0)
                    ck(cudaMemcpy(h.data(), W.val + field(l, btm::RL_ENT), 8 * (size_t)nnz, cudaMemcpyDeviceToHost),
                       "dbg out");
                for (int q = 0; q < nnz; ++q) o.push_back(h[q]);
            }
            if ((int64_t)o.size() > n_out) throw BtmError(BTM_ERR_ARG, "debug output too small");
            std::copy(o.begin(), o.end(), out);
            return BTM_OK;
        }
        std::vector<const double *> srcs;
        std::vector<int64_t> lens;
        switch (phase) {
            case BTM_PHASE_GRAD: srcs = {I.gpx, I.gpy, I.gpz}; lens = {nC, nC, nC}; break;
            case BTM_PHASE_SST: srcs = {I.nut, I.f1, I.f2, I.pk, I.cdkw, I.smag}; lens.assign(6, nC); break;
            case BTM_PHASE_MOMENTUM: srcs = {I.diag, I.src, I.aPx}; lens = {nC + 2LL * nIF, nC, nC}; break;
            case BTM_PHASE_PRESSURE:
            case BTM_PHASE_KEQ:
            case BTM_PHASE_OMEGAEQ: srcs = {I.diag, I.src}; lens = {nC + 2LL * nIF, nC}; break;
            case BTM_PHASE_SPMV: srcs = {I.v}; lens = {nC}; break;
            case BTM_PHASE_BICGSTAB:
            case BTM_PHASE_AMGPCG:
            case BTM_PHASE_PCG:
            case BTM_PHASE_GS: srcs = {I.pp, I.outLast}; lens = {nC, 4}; break;
            default: throw BtmError(BTM_ERR_ARG, "unknown debug phase");
        }
        int64_t total = 0;
        for (auto l : lens) total += l;
        if (n_out < total) throw BtmError(BTM_ERR_ARG, "debug output too small");
        double *o = out;
        for (size_t j = 0; j < srcs.size(); ++j) {
            ck(cudaMemcpy(o, srcs[j], 8 * (size_t)lens[j], cudaMemcpyDeviceToHost), "dbg out");
            o += lens[j];
        }
    } catch (const BtmError &e) {
        return fail(e.code, e.what());
    } catch (const std::exception &e) {
        return fail(BTM_ERR_INTERNAL, e.what());
    }
    return BTM_OK;
}

}  // extern "C"

// ---- helpers shared with btm_noalloc.cu ----------------------------------
namespace btm_host {
int ensure_device() { return ::ensure_device(); }
void set_error(const std::string &msg) { g_err = msg; }
void set_launch_ms(double ms) { g_launch_ms = ms; }
void fill_inst(btm_case *C, btm::DevInst &I, const double *coeffs, int variant, const btm_init *init) {
    ::fill_inst(C, I, coeffs, variant, init);
}
int block_max_cells() { return ::block_max_cells(); }
int block_threads_for(int maxCells) { return ::block_threads_for(maxCells); }
int case_threads(const btm_case *C, int engine) { return ::case_threads(C, engine); }
void make_slab(btm_case *C, Slab &S) { ::make_slab(C, S); }
void ensure_mixed(btm_case *C, Slab &S) { ::ensure_mixed(C, S); }
void ensure_obs(btm_case *C, Slab &S, bool want) { ::ensure_obs(C, S, want); }
void download_obs(btm_case *C, const btm::DevInst &I, btm_history *h, cudaStream_t st) {
    ::download_obs(C, I, h, st);
}
void free_slab(Slab &S) { ::free_slab(S); }
void ensure_inj(btm_case *C, Slab &S) { ::ensure_inj(C, S); }
void ensure_ramg(btm_case *C, Slab &S) { ::ensure_ramg(C, S); }
size_t ramg_layout(const btm_case *C, char *base, btm::RamgWork &W) { return ::ramg_layout(C, base, W); }
void upload_state(btm_case *C, const btm::DevInst &I, const btm_state *ws, cudaStream_t st,
                  std::vector<double> &stage) {
    ::upload_state(C, I, ws, st, stage);
}
void download_state(btm_case *C, const btm::DevInst &I, btm_state *o, cudaStream_t st,
                    std::vector<double> &stage) {
    ::download_state(C, I, o, st, stage);
}
}  // namespace btm_host
