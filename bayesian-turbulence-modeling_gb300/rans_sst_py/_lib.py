"""ctypes binding of libbtm_gb300.so (the C ABI in include/btm_gb300.h).

Loading never falls back to anything: if the library cannot be built or
loaded, or no CUDA device is visible, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)

BTM_OK = 0


class BtmMesh(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_internal_faces", C.c_int32),
                ("n_patches", C.c_int32), ("owner", _ip), ("neighbour", _ip),
                ("face_center", _dp), ("face_normal", _dp), ("face_area", _dp),
                ("face_delta", _dp), ("face_d", _dp), ("face_weight", _dp),
                ("cell_center", _dp), ("cell_volume", _dp), ("wall_distance", _dp),
                ("patch_type", _ip), ("patch_offset", _ip), ("patch_faces", _ip)]


class BtmPatchBC(C.Structure):
    _fields_ = [("u_type", C.c_int32), ("p_type", C.c_int32), ("k_type", C.c_int32),
                ("omega_type", C.c_int32), ("u_value", C.c_double * 3), ("p_value", C.c_double),
                ("k_value", C.c_double), ("omega_value", C.c_double), ("u_profile", _dp),
                ("k_profile", _dp), ("omega_profile", _dp)]


class BtmSettings(C.Structure):
    _fields_ = [("max_iterations", C.c_int32), ("convergence_tol", C.c_double),
                ("divergence_limit", C.c_double), ("alpha_u", C.c_double), ("alpha_p", C.c_double),
                ("alpha_k", C.c_double), ("alpha_omega", C.c_double),
                ("inner_iterations", C.c_int32), ("inner_tolerance", C.c_double),
                ("turb_start_iter", C.c_int32), ("turb_update_interval", C.c_int32),
                ("nut_floor_iters", C.c_int32), ("rhie_chow_all_meshes", C.c_int32),
                ("body_force", C.c_double * 3), ("k_min", C.c_double), ("k_max", C.c_double),
                ("omega_min", C.c_double), ("use_wall_functions", C.c_int32),
                ("von_karman", C.c_double), ("wall_fn_E", C.c_double),
                ("pressure_solver", C.c_int32), ("momentum_solver", C.c_int32),
                ("turbulence_solver", C.c_int32), ("precision", C.c_int32), ("alpha_injection", C.c_double),
                ("amg_order", C.c_int32), ("anderson_depth", C.c_int32)]


class BtmState(C.Structure):
    _fields_ = [(n, _dp) for n in ("U", "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw",
                                   "Ub", "pb", "kb", "omegab")] + [("turb_established", C.c_int32)]


class BtmInit(C.Structure):
    _fields_ = [("mode", C.c_int32), ("u", C.c_double * 3), ("p", C.c_double), ("k", C.c_double),
                ("omega", C.c_double), ("warm", C.POINTER(BtmState))]


class BtmHistory(C.Structure):
    _fields_ = [("status", C.c_int32), ("converged", C.c_int32), ("diverged", C.c_int32),
                ("final_iter", C.c_int32), ("iterations_run", C.c_int32),
                ("inner_iterations", C.c_int64), ("last_residual", C.c_double * 6),
                ("residual_capacity", C.c_int32), ("residuals", _dp), ("phase_ms", C.c_double * 10),
                ("solve_ms", C.c_double), ("finish_ms", C.c_double), ("inner_split", C.c_int64 * 4),
                ("polish_start", C.c_int32), ("predictions", _dp), ("log_lik", C.c_double)]


class BtmObservable(C.Structure):
    _fields_ = [("type", C.c_int32), ("patch", C.c_int32), ("component", C.c_int32),
                ("location", C.c_double * 3), ("observed", C.c_double), ("sigma_obs", C.c_double),
                ("sigma_model", C.c_double), ("ref_area", C.c_double), ("ref_velocity", C.c_double),
                ("ref_pressure", C.c_double), ("ref_density", C.c_double)]


SOLVER_CODES = {"PCG": 0, "BiCGSTAB": 1, "GaussSeidel": 2, "AMG": 3}
PRECISION_CODES = {"fp64": 0, "mixed": 1}
AMG_ORDER_CODES = {"auto": 0, "reference": 1, "multicolour": 2}
ANDERSON_DEPTH_DEFAULT = 8   # SolverSettings.anderson_depth
PHASES = {"grad": 1, "sst": 2, "momentum": 3, "pressure": 4, "k": 5, "omega": 6, "spmv": 7,
          "bicgstab": 8, "amgpcg": 9, "pcg": 11, "amg_levels": 12, "gs": 13}

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.lib_path()


def lib():
    """Build if needed and load libbtm_gb300.so (raises on any failure)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = C.CDLL(path)
            L.btm_last_error.restype = C.c_char_p
            L.btm_abi_version.restype = C.c_int
            L.btm_case_create.argtypes = [C.POINTER(BtmMesh), C.POINTER(BtmPatchBC), C.c_double,
                                          C.POINTER(BtmSettings), C.POINTER(C.c_void_p)]
            L.btm_case_destroy.argtypes = [C.c_void_p]
            L.btm_case_destroy.restype = None
            L.btm_case_info.argtypes = [C.c_void_p] + [C.POINTER(C.c_int32)] * 4
            L.btm_case_launch_shape.argtypes = [C.c_void_p, C.c_int32] + [C.POINTER(C.c_int32)] * 3 + \
                [C.POINTER(C.c_double)]
            L.btm_case_set_settings.argtypes = [C.c_void_p, C.POINTER(BtmSettings)]
            L.btm_case_set_observations.argtypes = [C.c_void_p, C.POINTER(BtmMesh), C.c_int32,
                                                    C.POINTER(BtmObservable)]
            L.btm_case_set_target_anisotropy.argtypes = [C.c_void_p, _dp]
            L.btm_case_injection_realizability.argtypes = [C.c_void_p, C.POINTER(C.c_int32),
                                                           C.POINTER(C.c_int32), C.POINTER(C.c_double)]
            L.btm_solve.argtypes = [C.c_void_p, _dp, C.c_int32, C.POINTER(BtmInit), C.POINTER(BtmState),
                                    C.POINTER(BtmHistory)]
            L.btm_solve_noalloc.argtypes = [C.c_void_p, _dp, C.c_int32, C.POINTER(BtmInit), C.POINTER(BtmState),
                                            C.POINTER(BtmHistory)]
            L.btm_solve_batch.argtypes = [C.c_int32, C.POINTER(C.c_void_p), _dp, _ip, C.POINTER(BtmInit),
                                          C.POINTER(BtmState), C.POINTER(BtmHistory)]
            L.btm_last_launch_ms.restype = C.c_double
            L.btm_debug_phase.argtypes = [C.c_void_p, C.c_int32, _dp, C.c_int32, C.c_int32, _dp, C.c_int64,
                                          _dp, C.c_int64]
            _lib = L
    return _lib


class BtmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"btm error {code}: {msg}")
        self.code = code


def check(rc: int) -> None:
    if rc != BTM_OK:
        raise BtmError(rc, lib().btm_last_error().decode())


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)


PATCH_CODES = {"wall": 1, "inlet": 2, "outlet": 3, "symmetry": 4}


def mesh_struct(mesh):
    """BtmMesh over a Mesh object's arrays; returns (struct, keep-alive list)."""
    keep = []

    def d(a, dtype=np.float64):
        a = np.ascontiguousarray(a, dtype)
        keep.append(a)
        return a

    if mesh.wall_dist is None:
        mesh.compute_wall_distance()
    off, faces = mesh.patch_offsets()
    s = BtmMesh()
    s.n_cells, s.n_faces = mesh.n_cells(), mesh.n_faces()
    s.n_internal_faces, s.n_patches = mesh.n_internal_faces(), mesh.n_patches()
    s.owner = iptr(d(mesh.owner, np.int32))
    s.neighbour = iptr(d(mesh.neighbour, np.int32))
    s.face_center = dptr(d(mesh.face_center))
    s.face_normal = dptr(d(mesh.face_normal))
    s.face_area = dptr(d(mesh.face_area))
    s.face_delta = dptr(d(mesh.face_delta))
    s.face_d = dptr(d(mesh.face_d))
    s.face_weight = dptr(d(mesh.face_weight))
    s.cell_center = dptr(d(mesh.cell_center))
    s.cell_volume = dptr(d(mesh.cell_volume))
    s.wall_distance = dptr(d(mesh.wall_dist))
    s.patch_type = iptr(d(np.array([PATCH_CODES.get(t, 0) for t in mesh.patch_types()], np.int32), np.int32))
    s.patch_offset = iptr(d(off, np.int32))
    s.patch_faces = iptr(d(faces if faces.size else np.zeros(1, np.int32), np.int32))
    return s, keep


def bc_structs(bcs):
    n = len(bcs.velocityBC)
    arr = (BtmPatchBC * max(n, 1))()
    keep = []
    for p in range(n):
        u, pp, k, w = bcs.velocityBC[p], bcs.pressureBC[p], bcs.kBC[p], bcs.omegaBC[p]
        b = arr[p]
        b.u_type, b.p_type, b.k_type, b.omega_type = int(u.type), int(pp.type), int(k.type), int(w.type)
        b.u_value[0], b.u_value[1], b.u_value[2] = u.vecValue.x, u.vecValue.y, u.vecValue.z
        b.p_value, b.k_value, b.omega_value = pp.value, k.value, w.value
        for attr, src in (("u_profile", u.vecProfile), ("k_profile", k.scalarProfile),
                          ("omega_profile", w.scalarProfile)):
            if src is not None and len(src):
                a = np.ascontiguousarray(src, np.float64)
                keep.append(a)
                setattr(b, attr, dptr(a))
    return arr, keep


def settings_struct(s) -> BtmSettings:
    st = BtmSettings()
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
    st.body_force[0], st.body_force[1], st.body_force[2] = bf.x, bf.y, bf.z
    st.k_min, st.k_max, st.omega_min = float(s.k_min), float(s.k_max), float(s.omega_min)
    st.use_wall_functions = int(bool(s.use_wall_functions))
    st.von_karman, st.wall_fn_E = float(s.von_karman), float(s.wall_fn_E)
    st.pressure_solver = SOLVER_CODES.get(s.pressure_solver, 1)
    st.momentum_solver = SOLVER_CODES.get(s.momentum_solver, 1)
    st.turbulence_solver = SOLVER_CODES.get(s.turbulence_solver, 1)
    prec = getattr(s, "precision", "fp64")
    if prec not in PRECISION_CODES:
        raise ValueError(f"precision must be one of {sorted(PRECISION_CODES)}, not {prec!r}")
    st.precision = PRECISION_CODES[prec]
    st.alpha_injection = float(getattr(s, "alpha_injection", 0.3))
    order = getattr(s, "amg_order", "auto")
    if order not in AMG_ORDER_CODES:
        raise ValueError(f"amg_order must be one of {sorted(AMG_ORDER_CODES)}, not {order!r}")
    st.amg_order = AMG_ORDER_CODES[order]
    st.anderson_depth = int(getattr(s, "anderson_depth", ANDERSON_DEPTH_DEFAULT))
    return st


CELL_FIELDS = ("p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw")
BND_FIELDS = ("pb", "kb", "omegab")


def new_state(n_cells: int, n_bnd: int) -> dict:
    st = {"U": np.zeros((n_cells, 3)), "Ub": np.zeros((max(n_bnd, 1), 3))}
    for f in CELL_FIELDS:
        st[f] = np.zeros(n_cells)
    for f in BND_FIELDS:
        st[f] = np.zeros(max(n_bnd, 1))
    st["turb_established"] = 0
    return st


def state_struct(st: dict) -> BtmState:
    s = BtmState()
    for k in ("U", "Ub") + CELL_FIELDS + BND_FIELDS:
        a = st[k]
        assert a.flags["C_CONTIGUOUS"] and a.dtype == np.float64
        setattr(s, k, dptr(a))
    s.turb_established = int(st.get("turb_established", 0))
    return s


def observable_structs(mesh, obs_op):
    """The btm_observable records of an ObservationOperator (None: none), in
    its order, patches resolved to indices of `mesh`; returns (array, n)."""
    items = obs_op.observables() if obs_op is not None else []
    arr = (BtmObservable * max(len(items), 1))()
    for i, o in enumerate(items):
        a = arr[i]
        a.type = int(o.type)
        a.patch = mesh.patch_by_name(o.patchName) if o.patchName else -1
        a.component = int(o.component)
        a.location[0], a.location[1], a.location[2] = o.location.x, o.location.y, o.location.z
        a.observed, a.sigma_obs, a.sigma_model = o.observed, o.sigma_obs, o.sigma_model
        a.ref_area, a.ref_velocity = o.referenceArea, o.refVelocity
        a.ref_pressure, a.ref_density = o.refPressure, o.refDensity
    return arr, len(items)


class Case:
    """Owning handle of a device-resident case (btm_case_create/destroy)."""

    def __init__(self, mesh, bcs, nu, settings):
        L = lib()
        self._L = L
        ms, keep_m = mesh_struct(mesh)
        bc, keep_b = bc_structs(bcs)
        st = settings_struct(settings)
        h = C.c_void_p()
        check(L.btm_case_create(C.byref(ms), bc, float(nu), C.byref(st), C.byref(h)))
        self.h = h
        self._mesh = mesh
        self.n_cells = mesh.n_cells()
        self.n_bnd = mesh.n_boundary_faces()
        self.n_internal = mesh.n_internal_faces()
        self.n_obs = 0

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self._L.btm_case_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        v = [C.c_int32() for _ in range(4)]
        check(self._L.btm_case_info(self.h, *[C.byref(x) for x in v]))
        return dict(n_cells=v[0].value, n_boundary_faces=v[1].value, n_amg_levels=v[2].value,
                    is_2d=bool(v[3].value))

    def launch_shape(self, precision="fp64"):
        """The case's one-CTA launch shape in an engine (btm_case_launch_shape):
        CTA threads, whether the autotuner chose them, its probe size and the
        probe times of 256- and 512-thread CTAs (ms)."""
        th, tu, pr = C.c_int32(), C.c_int32(), C.c_int32()
        ms = (C.c_double * 2)()
        check(self._L.btm_case_launch_shape(self.h, PRECISION_CODES[precision], C.byref(th), C.byref(tu), C.byref(pr),
                                            ms))
        return dict(threads=th.value, tuned=bool(tu.value), probe=pr.value, probe_ms=[ms[0], ms[1]])

    def set_settings(self, settings):
        st = settings_struct(settings)
        check(self._L.btm_case_set_settings(self.h, C.byref(st)))

    def set_observations(self, obs_op):
        """Attach an ObservationOperator (None: detach): every later solve of
        this case evaluates its observables and the log-likelihood on the
        device (btm_case_set_observations)."""
        mesh = self._mesh
        arr, n = observable_structs(mesh, obs_op)
        ms, keep = mesh_struct(mesh)
        check(self._L.btm_case_set_observations(self.h, C.byref(ms), n, arr))
        self.n_obs = n

    def set_target_anisotropy(self, b6):
        """Reynolds-stress injection target, (n_cells*6,) xx yy zz xy xz yz
        per cell, applied to every later solve of the case; None clears it
        (btm_case_set_target_anisotropy)."""
        if b6 is None:
            check(self._L.btm_case_set_target_anisotropy(self.h, None))
            return
        b6 = np.ascontiguousarray(np.asarray(b6, np.float64).reshape(-1))
        if b6.size != 6 * self.n_cells:
            raise RuntimeError("setTargetAnisotropy: expected nCells*6 values")
        check(self._L.btm_case_set_target_anisotropy(self.h, dptr(b6)))

    def injection_realizability(self):
        """(active, all_realizable, max_violation) of the case's target."""
        a, r, v = C.c_int32(), C.c_int32(), C.c_double()
        check(self._L.btm_case_injection_realizability(self.h, C.byref(a), C.byref(r), C.byref(v)))
        return bool(a.value), bool(r.value), float(v.value)
