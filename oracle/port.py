"""ctypes access to the plain-C restatement (oracle/_build/libbtm_oracle.so).

TEST INFRASTRUCTURE ONLY: the checker used by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg.  Inputs are described duck-typed (any object
with the mesh / boundary-condition / settings attributes), so this module
imports nothing from the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from .cabi import (History, Init, MeshDesc, PatchBC, Settings, mesh_desc, state_arrays,
                   state_from_arrays)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbtm_oracle.so")
_lib = None

SOLVER_CODES = {"PCG": 0, "BiCGSTAB": 1, "GaussSeidel": 2, "AMG": 3}


def build(force: bool = False) -> str:
    """Compile the restatement with oracle/Makefile (gcc, no contraction)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.oracle_solve.argtypes = [C.POINTER(MeshDesc), C.POINTER(PatchBC), C.c_double,
                                   C.POINTER(Settings), dp, C.c_int, C.POINTER(Init),
                                   C.c_void_p, C.POINTER(History)]
        L.oracle_green_gauss.argtypes = [C.POINTER(MeshDesc), dp, dp, dp]
        L.oracle_set_target_anisotropy.argtypes = [dp]
        L.oracle_set_target_anisotropy.restype = None
        L.oracle_amg_levels.argtypes = [C.c_int, ip, ip, dp, C.c_int, ip, ip]
        L.oracle_amg_levels.restype = C.c_int
        L.oracle_sst_point.argtypes = [dp, C.c_int, C.c_int, dp]
        L.oracle_sst_point.restype = C.c_double
        L.oracle_apply_bcs.argtypes = [C.POINTER(MeshDesc), C.POINTER(PatchBC), C.c_double, C.c_void_p]
        L.oracle_apply_bcs.restype = None
        L.oracle_transpose_stress.argtypes = [C.POINTER(MeshDesc), dp, dp, dp, C.c_int, dp]
        L.oracle_transpose_stress.restype = None
        L.oracle_sst_fields.argtypes = [C.POINTER(MeshDesc), dp, C.c_int, C.c_double] + [dp] * 12
        L.oracle_assemble.argtypes = [C.POINTER(MeshDesc), C.POINTER(PatchBC), C.c_double,
                                      C.POINTER(Settings), dp, C.c_int, C.c_void_p, dp, dp,
                                      dp, dp, dp, dp, dp]
        L.oracle_matvec.argtypes = [C.c_int, C.c_int, ip, ip, dp, dp, dp, dp, dp]
        L.oracle_linear_solve.argtypes = [C.c_int, C.c_int, C.c_int, ip, ip, dp, dp, dp, dp, dp,
                                          C.c_int, C.c_double, dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


# ---- duck-typed input conversion ------------------------------------------
def mesh_arrays(mesh) -> dict:
    """Mesh arrays in the btm_mesh layout from any object exposing the mesh
    attributes (owner, neighbour, face_*, cell_*, wall_dist, patches, n_internal)."""
    if isinstance(mesh, dict):
        return mesh
    off = np.zeros(len(mesh.patches) + 1, np.int32)
    for i, p in enumerate(mesh.patches):
        off[i + 1] = off[i] + len(p[2])
    faces = (np.concatenate([np.asarray(p[2], np.int32) for p in mesh.patches])
             if mesh.patches else np.zeros(0, np.int32))
    codes = {"wall": 1, "inlet": 2, "outlet": 3, "symmetry": 4}
    wd = mesh.wall_dist if mesh.wall_dist is not None else np.full(mesh.cell_volume.size, 1e10)
    return dict(owner=mesh.owner, neighbour=mesh.neighbour, face_center=mesh.face_center,
                face_normal=mesh.face_normal, face_area=mesh.face_area, face_delta=mesh.face_delta,
                face_d=mesh.face_d, face_weight=mesh.face_weight, cell_center=mesh.cell_center,
                cell_volume=mesh.cell_volume, wall_dist=wd, n_internal=mesh.n_internal,
                patch_type=np.array([codes.get(p[1], 0) for p in mesh.patches], np.int32),
                patch_offset=off, patch_faces=faces)


def bc_array(bcs):
    """btm_patch_bc[] from an object with velocityBC/pressureBC/kBC/omegaBC lists
    (entries with .type, .value, .vecValue, .vecProfile, .scalarProfile)."""
    n = len(bcs.velocityBC)
    arr = (PatchBC * max(n, 1))()
    keep = []
    for p in range(n):
        u, pp, k, w = bcs.velocityBC[p], bcs.pressureBC[p], bcs.kBC[p], bcs.omegaBC[p]
        b = arr[p]
        b.u_type, b.p_type, b.k_type, b.omega_type = int(u.type), int(pp.type), int(k.type), int(w.type)
        v = u.vecValue
        b.u_value[0], b.u_value[1], b.u_value[2] = (v.x, v.y, v.z) if hasattr(v, "x") else tuple(v)
        b.p_value, b.k_value, b.omega_value = float(pp.value), float(k.value), float(w.value)
        for attr, src in (("u_profile", getattr(u, "vecProfile", None)),
                          ("k_profile", getattr(k, "scalarProfile", None)),
                          ("omega_profile", getattr(w, "scalarProfile", None))):
            if src is not None and len(src):
                a = np.ascontiguousarray(src, np.float64)
                keep.append(a)
                setattr(b, attr, _d(a))
    return arr, keep


def settings_struct(s) -> Settings:
    st = Settings()
    st.max_iterations = int(s.max_iterations)
    st.convergence_tol = float(s.convergence_tol)
    st.divergence_limit = float(s.divergence_limit)
    st.alpha_u, st.alpha_p = float(s.alpha_u), float(s.alpha_p)
    st.alpha_k, st.alpha_omega = float(s.alpha_k), float(s.alpha_omega)
    st.inner_iterations = int(s.inner_iterations)
    st.inner_tolerance = float(s.inner_tolerance)
    st.turb_start_iter = int(s.turb_start_iter)
    st.turb_update_interval = int(s.turb_update_interval)
    st.nut_floor_iters = int(s.nut_floor_iters)
    st.rhie_chow_all_meshes = int(bool(s.rhie_chow_all_meshes))
    bf = s.body_force
    st.body_force[0], st.body_force[1], st.body_force[2] = (bf.x, bf.y, bf.z) if hasattr(bf, "x") else tuple(bf)
    st.k_min, st.k_max, st.omega_min = float(s.k_min), float(s.k_max), float(s.omega_min)
    st.use_wall_functions = int(bool(s.use_wall_functions))
    st.von_karman, st.wall_fn_E = float(s.von_karman), float(s.wall_fn_E)
    st.pressure_solver = SOLVER_CODES.get(getattr(s, "pressure_solver", "AMG"), 1)
    st.momentum_solver = SOLVER_CODES.get(getattr(s, "momentum_solver", "BiCGSTAB"), 1)
    st.turbulence_solver = SOLVER_CODES.get(getattr(s, "turbulence_solver", "BiCGSTAB"), 1)
    st.alpha_injection = float(getattr(s, "alpha_injection", 0.3))
    return st


def make_init(u=(1.0, 0.0, 0.0), p=0.0, k=1e-4, omega=1.0, warm=None):
    ini = Init()
    keep = None
    if warm is None:
        ini.mode = 0
        ini.u[0], ini.u[1], ini.u[2] = u
        ini.p, ini.k, ini.omega = p, k, omega
    else:
        ini.mode = 1
        st, keep = state_from_arrays(warm)
        keep = (st, keep)
        ini.warm = C.pointer(st)
    return ini, keep


# ---- calls -----------------------------------------------------------------
def solve(mesh, bcs, nu, settings, coeffs, variant=0, u=(1.0, 0.0, 0.0), p=0.0, k=1e-4,
          omega=1.0, warm=None, residual_capacity=0, b_target=None):
    """Run the restated SIMPLE solve; returns (state dict, history dict).
    b_target: Reynolds-stress injection target, (n_cells*6,) xx yy zz xy xz yz."""
    m = mesh_arrays(mesh)
    md, keep_m = mesh_desc(m)
    bca, keep_b = bc_array(bcs)
    st = settings_struct(settings)
    ini, keep_i = make_init(u, p, k, omega, warm)
    nC, nB = int(m["cell_volume"].size), int(m["owner"].size) - int(m["n_internal"])
    arrays, state = state_arrays(nC, nB)
    hist = History()
    res = None
    if residual_capacity:
        res = np.zeros((residual_capacity, 6))
        hist.residual_capacity = residual_capacity
        hist.residuals = _d(res)
    cf = np.ascontiguousarray(coeffs, np.float64)
    bt = None if b_target is None else np.ascontiguousarray(np.asarray(b_target, np.float64).reshape(-1))
    lib().oracle_set_target_anisotropy(_d(bt) if bt is not None else None)
    try:
        lib().oracle_solve(C.byref(md), bca, float(nu), C.byref(st), _d(cf), int(variant), C.byref(ini),
                           C.cast(C.pointer(state), C.c_void_p), C.byref(hist))
    finally:
        lib().oracle_set_target_anisotropy(None)
    arrays["turb_established"] = state.turb_established
    h = dict(status=hist.status, converged=hist.converged, diverged=hist.diverged,
             final_iter=hist.final_iter, iterations_run=hist.iterations_run,
             inner_iterations=hist.inner_iterations, last_residual=list(hist.last_residual))
    if res is not None:
        h["residuals"] = res[:hist.iterations_run]
    return arrays, h


def green_gauss(mesh, phi, phib):
    m = mesh_arrays(mesh)
    md, keep = mesh_desc(m)
    g = np.zeros((int(m["cell_volume"].size), 3))
    lib().oracle_green_gauss(C.byref(md), _d(np.ascontiguousarray(phi, np.float64)),
                             _d(np.ascontiguousarray(phib, np.float64)), _d(g))
    return g


def sst_fields(mesh, coeffs, variant, nu, U, Ub, k, kb, om, omb):
    m = mesh_arrays(mesh)
    md, keep = mesh_desc(m)
    nC = int(m["cell_volume"].size)
    outs = [np.zeros(nC) for _ in range(6)]
    ins = [np.ascontiguousarray(a, np.float64) for a in (U, Ub, k, kb, om, omb)]
    cf = np.ascontiguousarray(coeffs, np.float64)
    lib().oracle_sst_fields(C.byref(md), _d(cf), int(variant), float(nu), *[_d(a) for a in ins],
                            *[_d(o) for o in outs])
    return dict(zip(("nuT", "F1", "F2", "Pk", "CDkw", "Smag"), outs))


def assemble(mesh, bcs, nu, settings, coeffs, kind, state, aP=None, Smag=None):
    """kind 0/1/2 momentum x/y/z, 3 pressure correction, 4 k, 5 omega."""
    m = mesh_arrays(mesh)
    md, keep_m = mesh_desc(m)
    bca, keep_b = bc_array(bcs)
    st = settings_struct(settings)
    nC, nIF = int(m["cell_volume"].size), int(m["n_internal"])
    sv, keep_s = state_from_arrays(state)
    diag, src, aPo = np.zeros(nC), np.zeros(nC), np.zeros(nC)
    upper, lower = np.zeros(max(nIF, 1)), np.zeros(max(nIF, 1))
    aPi = np.ascontiguousarray(aP if aP is not None else np.zeros(nC), np.float64)
    Sm = np.ascontiguousarray(Smag if Smag is not None else np.zeros(nC), np.float64)
    cf = np.ascontiguousarray(coeffs, np.float64)
    lib().oracle_assemble(C.byref(md), bca, float(nu), C.byref(st), _d(cf), int(kind),
                          C.cast(C.pointer(sv), C.c_void_p), _d(aPi), _d(Sm), _d(diag), _d(upper),
                          _d(lower), _d(src), _d(aPo))
    return dict(diag=diag, upper=upper[:nIF], lower=lower[:nIF], source=src, aP=aPo)


def matvec(own, nbr, diag, upper, lower, x):
    own = np.ascontiguousarray(own, np.int32)
    nbr = np.ascontiguousarray(nbr, np.int32)
    y = np.zeros(len(diag))
    a = [np.ascontiguousarray(v, np.float64) for v in (diag, upper, lower, x)]
    lib().oracle_matvec(len(diag), own.size, _i(own), _i(nbr), *[_d(v) for v in a], _d(y))
    return y


def linear_solve(kind, own, nbr, diag, upper, lower, source, x0, max_iter, tol):
    own = np.ascontiguousarray(own, np.int32)
    nbr = np.ascontiguousarray(nbr, np.int32)
    x = np.array(x0, dtype=np.float64)
    res = np.zeros(4)
    a = [np.ascontiguousarray(v, np.float64) for v in (diag, upper, lower, source)]
    lib().oracle_linear_solve(int(kind), x.size, own.size, _i(own), _i(nbr), *[_d(v) for v in a],
                              _d(x), int(max_iter), float(tol), _d(res))
    return x, res


def amg_levels(row_ptr, col_idx, values, max_levels=21):
    """AMGSolver::setup's coarsening on a CSR matrix: (sizes, [maps per level])."""
    n = len(row_ptr) - 1
    rp = np.ascontiguousarray(row_ptr, np.int32)
    ci = np.ascontiguousarray(col_idx, np.int32)
    va = np.ascontiguousarray(values, np.float64)
    sizes = np.zeros(max_levels, np.int32)
    maps = np.zeros(max(1, n * max_levels), np.int32)
    nl = lib().oracle_amg_levels(n, rp.ctypes.data_as(C.POINTER(C.c_int)), ci.ctypes.data_as(C.POINTER(C.c_int)),
                                 _d(va), max_levels, sizes.ctypes.data_as(C.POINTER(C.c_int)),
                                 maps.ctypes.data_as(C.POINTER(C.c_int)))
    out, at = [], 0
    for l in range(nl - 1):
        out.append(maps[at:at + sizes[l]].copy())
        at += sizes[l]
    return sizes[:nl].tolist(), out


SST_POINT = {"production": 0, "production_omega": 1, "F1": 2, "F2": 3, "nut": 4}


def sst_point(name, *args, coeffs=None, variant=0):
    """One SSTModel point function of the restatement (see SST_POINT)."""
    from rans_sst_py._types import COEFF_DEFAULTS
    cf = np.ascontiguousarray(COEFF_DEFAULTS if coeffs is None else coeffs, np.float64)
    a = np.ascontiguousarray(args + (0.0,) * (5 - len(args)), np.float64)
    return float(lib().oracle_sst_point(_d(cf), int(variant), SST_POINT[name], _d(a)))


def apply_bcs(mesh, bcs, nu, U, p=None, k=None, omega=None):
    """The reference's four apply*BC functions on cell values: returns the
    state dict with its boundary values (Ub, pb, kb, omegab) filled."""
    m = mesh_arrays(mesh)
    md, keep_m = mesh_desc(m)
    bca, keep_b = bc_array(bcs)
    nC, nB = int(m["cell_volume"].size), int(m["owner"].size) - int(m["n_internal"])
    arrays, state = state_arrays(nC, nB)
    arrays["U"][:] = U
    for name, v in (("p", p), ("k", k), ("omega", omega)):
        if v is not None:
            arrays[name][:] = v
    lib().oracle_apply_bcs(C.byref(md), bca, float(nu), C.cast(C.pointer(state), C.c_void_p))
    return arrays


def transpose_stress(mesh, coeff, U, Ub, comp):
    """transposeStressSource (zero wall coefficient) of the restatement."""
    m = mesh_arrays(mesh)
    md, keep = mesh_desc(m)
    a = [np.ascontiguousarray(v, np.float64) for v in (coeff, U, Ub)]
    out = np.zeros(int(m["cell_volume"].size))
    lib().oracle_transpose_stress(C.byref(md), *[_d(v) for v in a], int(comp), _d(out))
    return out
