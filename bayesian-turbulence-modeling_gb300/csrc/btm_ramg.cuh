// btm_ramg.cuh - the reference's AMG-preconditioned CG (AMGSolver,
// core/include/LinearSolver.hpp:497-656) on one CTA, with the hierarchy
// rebuilt from the actual matrix at every solve and every Gauss-Seidel sweep
// in the reference's row order.
//
// The reference's setup and smoother are sequential loops over rows.  Both
// are evaluated here in parallel with the sequential results:
//
//   * Forward Gauss-Seidel (CSRMatrix::gaussSeidelSweep, :328-337): row i
//     reads the new x of its lower-index neighbours and the old x of the
//     higher-index ones.  Rows are grouped into wavefronts by the depth of
//     the "lower-index neighbour" DAG (depth(i) = 1 + max depth of its
//     lower-index neighbours); a wavefront's rows are independent, and every
//     row sums its terms in the reference's order.
//   * Greedy aggregation (buildAggregates, :407-443): a row becomes a seed
//     exactly when no lower-index seed claims it, and it is claimed by the
//     lowest-index seed whose row entry for it is strong.  That recursion runs
//     over the same wavefronts; aggregate ids are the seeds' prefix count in
//     row order.  (The reference's second pass never finds an unassigned row:
//     every row is a seed or claimed in the first.)  The aggregation maps are
//     therefore bit-identical to the reference's.
//   * Galerkin product (galerkinProduct, :446-485): an aggregate's members
//     are its seed and the rows its seed claimed, all in the seed's row; each
//     coarse entry sums its fine entries in (fine row ascending, fine column
//     ascending) order, as the reference's single pass over the fine rows.
//
// Levels of at most kRamgWarpRows rows run on warp 0 alone (warp barriers
// instead of CTA barriers).  Dot products of the CG loop are parallel trees,
// and the smoother multiplies by reciprocal diagonals where the reference
// divides: both differ from the reference in the last bits only.
//
// Coarse levels live in per-instance pools sized at twice the fine rows and
// three times the fine entries; a level that would not fit ends the
// hierarchy (it becomes the coarsest level, smoothed by the reference's 50
// sweeps), which typical 2-D and 3-D meshes never reach.
#pragma once
#include "btm_common.h"
#include "btm_team.cuh"

namespace btm {

constexpr int kRamgMinCoarse = 50;     // minCoarseSize_ (LinearSolver.hpp:509)
constexpr int kRamgCoarseSweeps = 50;  // coarseSweeps_
constexpr int kRamgMaxCoarsen = 20;    // maxLevels_
constexpr int kRamgWarpRows = 192;     // levels up to this size run on warp 0

// One level as the device functions see it.  Level 0 reads its values from
// the LDU system through entry ids (the lduToCSR layout built per case).
struct RLevel {
    int n, nWf;
    const int32_t *ptr, *col, *ent;
    const double *val, *dg, *ldu;
    const int32_t *wfOff, *wfRows;
    const double *rd;               // 1/diag where |diag| > 1e-30, else 0
    double *x, *b, *r;
    const int32_t *map;             // this level -> next level (null at the coarsest)
    const int32_t *memOff, *mem;    // next level's members in this level, ascending
    __device__ __forceinline__ double v(int j) const { return ent ? ldu[ent[j]] : val[j]; }
    __device__ __forceinline__ double d(int i) const { return ent ? ldu[i] : dg[i]; }
};

__device__ __forceinline__ RLevel ramg_level(const DevMesh &M, const DevInst &I, int l) {
    const RamgWork &W = I.rg;
    const int32_t *t = W.lev + l * kRamgLevInts;
    RLevel L;
    L.n = t[RL_N];
    L.ldu = I.diag;
    if (l == 0) {
        L.ptr = M.lev[0].rowPtr; L.col = M.lev[0].colIdx; L.ent = M.r0Ent;
        L.val = nullptr; L.dg = nullptr;
        L.wfOff = M.wf0Off; L.wfRows = M.wf0Rows; L.nWf = M.nWf0;
        L.x = W.xs ? W.xs : I.s;
        L.b = I.r; L.r = I.t; L.rd = W.rd;
    } else {
        L.ptr = W.ptr + t[RL_PTR]; L.col = W.col + t[RL_ENT]; L.ent = nullptr;
        L.val = W.val + t[RL_ENT]; L.dg = W.dg + t[RL_VEC];
        L.wfOff = W.wfOff + t[RL_WFO]; L.wfRows = W.wfRows + t[RL_VEC]; L.nWf = t[RL_NWF];
        L.x = W.xs ? W.xs + M.nC + t[RL_VEC] : W.x + t[RL_VEC];
        L.b = W.b + t[RL_VEC]; L.r = W.r + t[RL_VEC]; L.rd = W.rd + M.nC + t[RL_VEC];
    }
    L.map = t[RL_MAP] >= 0 ? W.map + t[RL_MAP] : nullptr;
    L.memOff = t[RL_MAP] >= 0 ? W.memOff + t[RL_MOFF] : nullptr;
    L.mem = t[RL_MAP] >= 0 ? W.mem + t[RL_MEM] : nullptr;
    return L;
}

// ---- CTA helpers ------------------------------------------------------------
__device__ __forceinline__ int ramg_warp_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Exclusive prefix sum of a[0..n) in place over the CTA; returns the total.
__device__ int ramg_scan(int32_t *a, int n) {
    __shared__ int sh[33];
    const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, w = t >> 5, nw = nt >> 5;
    const int chunk = (n + nt - 1) / nt;
    const int lo = min(n, t * chunk), hi = min(n, lo + chunk);
    int s = 0;
    for (int i = lo; i < hi; ++i) s += a[i];
    const int inc = ramg_warp_scan(s);
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int v = lane < nw ? sh[lane] : 0;
        const int vi = ramg_warp_scan(v);
        if (lane < nw) sh[lane] = vi - v;
        if (lane == 31) sh[32] = vi;
    }
    __syncthreads();
    int run = sh[w] + inc - s;
    for (int i = lo; i < hi; ++i) {
        const int v = a[i];
        a[i] = run;
        run += v;
    }
    const int total = sh[32];
    __syncthreads();
    return total;
}

// ---- smoother, residual, transfer (the CTA, or warp 0 when `wm`) ------------
struct RGroup {
    int rank, size;
    bool wm;
    __device__ __forceinline__ void sync() const {
        if (wm) __syncwarp();
        else __syncthreads();
    }
};

// CSRMatrix::gaussSeidelSweep (LinearSolver.hpp:328-337), wavefront by
// wavefront.  The reference divides by the diagonal; the sweep multiplies by
// the reciprocal formed once per setup (at most one unit in the last place
// per update), which keeps the FP64 division sequence off the chain of
// dependent operations every wavefront waits for.
__device__ __noinline__ void ramg_gs(const RGroup &g, const RLevel &L) {
    for (int w = 0; w < L.nWf; ++w) {
        for (int q = L.wfOff[w] + g.rank; q < L.wfOff[w + 1]; q += g.size) {
            const int i = L.wfRows[q];
            double s = L.b[i];
            for (int j = L.ptr[i]; j < L.ptr[i + 1]; ++j) {
                const int c = L.col[j];
                if (c != i) s -= L.v(j) * L.x[c];
            }
            const double ri = L.rd[i];
            if (ri != 0.0) L.x[i] = s * ri;
        }
        g.sync();
    }
}

// CSRMatrix::residual (:318-326), then the restriction of the V-cycle
// (:571-575): coarse b = sum of the members' residuals in ascending row
// order, coarse x = 0
__device__ __noinline__ void ramg_restrict(const RGroup &g, const RLevel &L, const RLevel &Cl) {
    for (int i = g.rank; i < L.n; i += g.size) {
        double s = 0.0;
        for (int j = L.ptr[i]; j < L.ptr[i + 1]; ++j) s += L.v(j) * L.x[L.col[j]];
        L.r[i] = L.b[i] - s;
    }
    g.sync();
    for (int J = g.rank; J < Cl.n; J += g.size) {
        double s = 0.0;
        for (int q = L.memOff[J]; q < L.memOff[J + 1]; ++q) s += L.r[L.mem[q]];
        Cl.b[J] = s;
        Cl.x[J] = 0.0;
    }
    g.sync();
}

__device__ __noinline__ void ramg_prolong(const RGroup &g, const RLevel &L, const RLevel &Cl) {
    for (int i = g.rank; i < L.n; i += g.size) L.x[i] = L.x[i] + Cl.x[L.map[i]];
    g.sync();
}

// AMGSolver::vcycle (:553-589) over levels [l0, l1] (l1 the coarsest)
__device__ void ramg_vcycle_range(const RGroup &g, const DevMesh &M, const DevInst &I, int l0, int l1, bool down,
                                  bool up) {
    if (down) {
        for (int l = l0; l < l1; ++l) {
            const RLevel L = ramg_level(M, I, l), Cl = ramg_level(M, I, l + 1);
            ramg_gs(g, L);
            ramg_gs(g, L);
            ramg_restrict(g, L, Cl);
        }
    }
    if (down && up) {
        const RLevel Lc = ramg_level(M, I, l1);
        for (int s = 0; s < kRamgCoarseSweeps; ++s) ramg_gs(g, Lc);
    }
    if (up) {
        for (int l = l1 - 1; l >= l0; --l) {
            const RLevel L = ramg_level(M, I, l), Cl = ramg_level(M, I, l + 1);
            ramg_prolong(g, L, Cl);
            ramg_gs(g, L);
            ramg_gs(g, L);
        }
    }
}

// ---- hierarchy setup (AMGSolver::setup, :516-551) ---------------------------
// Wavefronts of a coarse level: depth by relaxation (ping-pong), then rows
// bucketed by depth.  Returns the wavefront count.
template <class T>
__device__ int ramg_wavefronts(T &tm, const RamgWork &W, const int32_t *ptr, const int32_t *col, int n,
                               int32_t *wfOff, int32_t *wfRows) {
    int32_t *a = W.aux, *b = W.aux2;
    for (int i = tm.rank(); i < n; i += tm.size()) a[i] = 0;
    tm.sync();
    for (int it = 0; it <= n; ++it) {
        double ch[1] = {0.0};
        for (int i = tm.rank(); i < n; i += tm.size()) {
            int dd = 0;
            for (int j = ptr[i]; j < ptr[i + 1]; ++j) {
                const int c = col[j];
                if (c < i) dd = max(dd, a[c] + 1);
            }
            b[i] = dd;
            if (dd != a[i]) ch[0] = 1.0;
        }
        tm.template maxr<1>(ch);
        int32_t *tmp = a; a = b; b = tmp;
        if (ch[0] == 0.0) break;
    }
    // a holds the depths; count, scan and place
    double mx[1] = {0.0};
    for (int i = tm.rank(); i < n; i += tm.size()) mx[0] = smax(mx[0], (double)a[i]);
    tm.template maxr<1>(mx);
    const int nWf = (int)mx[0] + 1;
    for (int q = tm.rank(); q <= nWf; q += tm.size()) wfOff[q] = 0;
    tm.sync();
    for (int i = tm.rank(); i < n; i += tm.size()) atomicAdd(&wfOff[a[i]], 1);
    tm.sync();
    ramg_scan(wfOff, nWf + 1);
    for (int q = tm.rank(); q < nWf; q += tm.size()) b[q] = wfOff[q];
    tm.sync();
    for (int i = tm.rank(); i < n; i += tm.size()) wfRows[atomicAdd(&b[a[i]], 1)] = i;
    tm.sync();
    return nWf;
}

// Builds levels 1.. from level 0 (whose values are the current system) and
// every level's reciprocal diagonals.  Returns the level count.
template <class T>
__device__ __noinline__ int ramg_setup(T &tm, const DevMesh &M, DevInst &I) {
    const RamgWork &W = I.rg;
    const int n0 = M.nC;
    if (tm.leader()) {
        int32_t *t = W.lev;
        t[RL_N] = n0; t[RL_PTR] = 0; t[RL_ENT] = 0; t[RL_VEC] = 0; t[RL_MAP] = -1; t[RL_NWF] = M.nWf0;
    }
    for (int i = tm.rank(); i < n0; i += tm.size()) {
        const double d = I.diag[i];
        W.rd[i] = fabs(d) > 1e-30 ? 1.0 / d : 0.0;
    }
    tm.sync();
    int nLev = 1;
    int rowsUsed = 0, entsUsed = 0, ptrUsed = 0, wfoUsed = 0, mapUsed = 0, moffUsed = 0, memUsed = 0;
    for (int l = 0; l < kRamgMaxCoarsen; ++l) {
        const RLevel L = ramg_level(M, I, l);
        const int n = L.n;
        if (n <= kRamgMinCoarse) break;
        int32_t *claim = W.seed;
        // 1. seeds and claims, wavefront by wavefront
        for (int w = 0; w < L.nWf; ++w) {
            for (int q = L.wfOff[w] + tm.rank(); q < L.wfOff[w + 1]; q += tm.size()) {
                const int i = L.wfRows[q];
                const double ajj = fabs(L.d(i));
                int cl = -1;
                for (int j = L.ptr[i]; j < L.ptr[i + 1] && cl < 0; ++j) {
                    const int c = L.col[j];
                    if (c >= i) break;
                    if (claim[c] != -1) continue;   // c is not a seed
                    // the seed's own row entry for i decides (every occurrence)
                    const double aii = fabs(L.d(c));
                    for (int jj = L.ptr[c]; jj < L.ptr[c + 1]; ++jj) {
                        if (L.col[jj] != i) continue;
                        const double strength = fabs(L.v(jj)) / sqrt(aii * ajj + 1e-30);
                        if (strength > 0.25) { cl = c; break; }
                    }
                }
                claim[i] = cl;
            }
            tm.sync();
        }
        // 2. aggregate ids: the seeds' prefix count in row order
        int32_t *aid = W.aux;
        for (int i = tm.rank(); i < n; i += tm.size()) aid[i] = claim[i] == -1 ? 1 : 0;
        tm.sync();
        const int nc = ramg_scan(aid, n);
        if (nc == 0 || nc >= n) break;
        // a level that does not fit the pools ends the hierarchy here
        if (rowsUsed + nc > W.rowPool || memUsed + n > W.rowPool + n0 || mapUsed + n > W.rowPool + n0 ||
            moffUsed + nc + 1 > W.rowPool + 64 || ptrUsed + nc + 1 > W.rowPool + 64 ||
            wfoUsed + nc + 1 > W.rowPool + 64)
            break;
        // 3. map, member counts (seed + the rows it claimed, adjacent duplicates once)
        int32_t *map = W.map + mapUsed;
        int32_t *moff = W.memOff + moffUsed;
        for (int i = tm.rank(); i < n; i += tm.size()) map[i] = claim[i] == -1 ? aid[i] : aid[claim[i]];
        for (int i = tm.rank(); i < n; i += tm.size()) {
            if (claim[i] != -1) continue;
            int cnt = 1;
            for (int j = L.ptr[i]; j < L.ptr[i + 1]; ++j) {
                const int c = L.col[j];
                if (c > i && claim[c] == i && !(j > L.ptr[i] && L.col[j - 1] == c)) ++cnt;
            }
            moff[aid[i]] = cnt;
        }
        if (tm.leader()) moff[nc] = 0;
        tm.sync();
        ramg_scan(moff, nc + 1);
        int32_t *mem = W.mem + memUsed;
        for (int i = tm.rank(); i < n; i += tm.size()) {
            if (claim[i] != -1) continue;
            int at = moff[aid[i]];
            mem[at++] = i;
            for (int j = L.ptr[i]; j < L.ptr[i + 1]; ++j) {
                const int c = L.col[j];
                if (c > i && claim[c] == i && !(j > L.ptr[i] && L.col[j - 1] == c)) mem[at++] = c;
            }
        }
        tm.sync();
        // 4. Galerkin contributions in (member ascending, column ascending) order
        int32_t *coff = W.coff;
        for (int J = tm.rank(); J < nc; J += tm.size()) {
            int cnt = 0;
            for (int q = moff[J]; q < moff[J + 1]; ++q) cnt += L.ptr[mem[q] + 1] - L.ptr[mem[q]];
            coff[J] = cnt;
        }
        if (tm.leader()) coff[nc] = 0;
        tm.sync();
        ramg_scan(coff, nc + 1);
        for (int J = tm.rank(); J < nc; J += tm.size()) {
            int k = coff[J];
            for (int q = moff[J]; q < moff[J + 1]; ++q) {
                const int m = mem[q];
                for (int j = L.ptr[m]; j < L.ptr[m + 1]; ++j) {
                    W.cj[k] = map[L.col[j]];
                    W.cv[k] = L.v(j);
                    ++k;
                }
            }
            // sum equal coarse columns in arrival order (0.0 + first, as the
            // reference's default-constructed map entry), then sort by column
            const int o = coff[J], e = coff[J + 1];
            int dcount = 0;
            for (int kk = o; kk < e; ++kk) {
                const int Jc = W.cj[kk];
                const double vv = W.cv[kk];
                int p = o;
                while (p < o + dcount && W.cj[p] != Jc) ++p;
                if (p < o + dcount) {
                    W.cv[p] += vv;
                } else {
                    W.cj[o + dcount] = Jc;
                    W.cv[o + dcount] = 0.0 + vv;
                    ++dcount;
                }
            }
            for (int a = o + 1; a < o + dcount; ++a) {
                const int kc = W.cj[a];
                const double kv = W.cv[a];
                int b = a - 1;
                while (b >= o && W.cj[b] > kc) {
                    W.cj[b + 1] = W.cj[b];
                    W.cv[b + 1] = W.cv[b];
                    --b;
                }
                W.cj[b + 1] = kc;
                W.cv[b + 1] = kv;
            }
            W.aux2[J] = dcount;
        }
        tm.sync();
        // 5. the coarse CSR into the pools
        int32_t *cptr = W.ptr + ptrUsed;
        for (int J = tm.rank(); J < nc; J += tm.size()) cptr[J] = W.aux2[J];
        if (tm.leader()) cptr[nc] = 0;
        tm.sync();
        const int nnzc = ramg_scan(cptr, nc + 1);
        if (entsUsed + nnzc > W.entPool) break;
        int32_t *ccol = W.col + entsUsed;
        double *cval = W.val + entsUsed, *cdg = W.dg + rowsUsed;
        for (int J = tm.rank(); J < nc; J += tm.size()) {
            const int o = coff[J];
            double dJ = 0.0;
            for (int q = cptr[J]; q < cptr[J + 1]; ++q) {
                const int Jc = W.cj[o + q - cptr[J]];
                const double vv = W.cv[o + q - cptr[J]];
                ccol[q] = Jc;
                cval[q] = vv;
                if (Jc == J) dJ = vv;
            }
            cdg[J] = dJ;
            W.rd[n0 + rowsUsed + J] = fabs(dJ) > 1e-30 ? 1.0 / dJ : 0.0;
        }
        tm.sync();
        // 6. the new level's wavefronts
        int32_t *cwfo = W.wfOff + wfoUsed;
        const int nWf = ramg_wavefronts(tm, W, cptr, ccol, nc, cwfo, W.wfRows + rowsUsed);
        if (tm.leader()) {
            int32_t *t = W.lev + l * kRamgLevInts;
            t[RL_MAP] = mapUsed; t[RL_MOFF] = moffUsed; t[RL_MEM] = memUsed;
            int32_t *u = W.lev + (l + 1) * kRamgLevInts;
            u[RL_N] = nc; u[RL_PTR] = ptrUsed; u[RL_ENT] = entsUsed; u[RL_VEC] = rowsUsed; u[RL_MAP] = -1;
            u[RL_WFO] = wfoUsed; u[RL_NWF] = nWf; u[RL_NNZ] = nnzc;
        }
        mapUsed += n; moffUsed += nc + 1; memUsed += n;
        ptrUsed += nc + 1; entsUsed += nnzc; rowsUsed += nc; wfoUsed += nWf + 1;
        ++nLev;
        tm.sync();
    }
    tm.sync();
    return nLev;
}

template <class T>
__device__ void ramg_vcycle(T &tm, const DevMesh &M, const DevInst &I, int nLev) {
    const int32_t *lev = I.rg.lev;
    int lw = nLev - 1;
    while (lw > 0 && lev[(lw - 1) * kRamgLevInts + RL_N] <= kRamgWarpRows) --lw;
    if (lev[lw * kRamgLevInts + RL_N] > kRamgWarpRows) lw = nLev;   // no level small enough
    const RGroup all{(int)threadIdx.x, (int)blockDim.x, false};
    if (lw == 0) {
        // every level is small: all of it on warp 0
        if (threadIdx.x < 32) {
            const RGroup w0{(int)threadIdx.x, 32, true};
            ramg_vcycle_range(w0, M, I, 0, nLev - 1, true, true);
        }
        __syncthreads();
        return;
    }
    if (lw < nLev) {
        ramg_vcycle_range(all, M, I, 0, lw, true, false);
        if (threadIdx.x < 32) {
            const RGroup w0{(int)threadIdx.x, 32, true};
            ramg_vcycle_range(w0, M, I, lw, nLev - 1, true, true);
        }
        __syncthreads();
        ramg_vcycle_range(all, M, I, 0, lw, false, true);
    } else {
        ramg_vcycle_range(all, M, I, 0, nLev - 1, true, true);
    }
}

// The V-cycle preconditioner z = M r on levels [0, nLev): level 0's b is I.r
// and the result z is left in I.s.  Levels from the first one of at most
// kRamgWarpRows rows down to the coarsest run on warp 0.  With the
// shared-memory copy of the level vectors (W.xs), level 0's x starts at zero
// there and is copied to I.s at the end; otherwise the caller zeroes I.s.
template <class T>
__device__ void ramg_precondition(T &tm, const DevMesh &M, const DevInst &I, int nLev) {
    if (I.rg.xs) {
        for (int c = threadIdx.x; c < M.nC; c += blockDim.x) I.rg.xs[c] = 0.0;
        __syncthreads();
    }
    ramg_vcycle(tm, M, I, nLev);
    if (I.rg.xs) {
        for (int c = threadIdx.x; c < M.nC; c += blockDim.x) I.s[c] = I.rg.xs[c];
        __syncthreads();
    }
}

}  // namespace btm
