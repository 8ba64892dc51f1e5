"""ctypes access to oracle/_ref/libref_driver.so: the unmodified reference
solver compiled from its own sources (see oracle/Makefile).

TEST INFRASTRUCTURE ONLY.  Available only where the reference sources exist
(the golden-vector generator under tests/golden/ runs it).  Nothing in the
product imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .cabi import PatchBC, Settings, Init, State, History, state_arrays  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libref_driver.so")

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference driver not built (make -C oracle ref)")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.ref_last_error.restype = C.c_char_p
        for name, args in (("ref_mesh_load", [C.c_char_p]),
                           ("ref_mesh_channel", [C.c_int, C.c_int, C.c_double, C.c_double]),
                           ("ref_mesh_channel_re", [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]),
                           ("ref_mesh_plate", [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]),
                           ("ref_mesh_bfs", [C.c_int] * 4 + [C.c_double] * 6),
                           ("ref_mesh_curved_periodic", [dp, dp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double])):
            f = getattr(L, name)
            f.restype = vp
            f.argtypes = args
        L.ref_mesh_free.argtypes = [vp]
        L.ref_mesh_wall_distance.argtypes = [vp]
        L.ref_mesh_set_patch_type.argtypes = [vp, C.c_char_p, C.c_char_p]
        L.ref_mesh_save.argtypes = [vp, C.c_char_p]
        L.ref_mesh_sizes.argtypes = [vp, ip]
        L.ref_mesh_dump.argtypes = [vp] + [ip] * 3 + [dp] * 9 + [ip] * 5 + [dp]
        L.ref_mesh_patch_names.argtypes = [vp, C.c_char_p, C.c_int]
        L.ref_bc_preset.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double, ip, dp]
        L.ref_solve.argtypes = [vp, C.POINTER(PatchBC), C.c_double, C.POINTER(Settings), dp, C.c_int,
                                C.POINTER(Init), C.POINTER(State), C.POINTER(History), C.c_int]
        L.ref_green_gauss.argtypes = [vp, dp, dp, dp]
        L.ref_set_target_anisotropy.argtypes = [dp, C.c_int]
        L.ref_set_target_anisotropy.restype = None
        L.ref_sst_fields.argtypes = [vp, dp, C.c_int, C.c_double] + [dp] * 12
        L.ref_observe.argtypes = [vp, C.c_int, C.c_void_p, C.c_double, C.POINTER(State), dp, dp]
        L.ref_linear_solve.argtypes = [C.c_int, C.c_int, C.c_int, ip, ip, dp, dp, dp, dp, dp, C.c_int,
                                       C.c_double, dp]
        L.ref_matvec.argtypes = [C.c_int, C.c_int, ip, ip, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class RefMesh:
    """Owning handle of a reference Mesh object."""

    def __init__(self, handle):
        if not handle:
            raise RuntimeError(lib().ref_last_error().decode())
        self.h = C.c_void_p(handle)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ref_mesh_free(self.h)
            self.h = None

    @staticmethod
    def load(path):
        return RefMesh(lib().ref_mesh_load(path.encode()))

    @staticmethod
    def channel(nx, ny, Lx, Ly, Re=None, yp=1.0):
        if Re is None:
            return RefMesh(lib().ref_mesh_channel(nx, ny, Lx, Ly))
        return RefMesh(lib().ref_mesh_channel_re(nx, ny, Lx, Ly, Re, yp))

    @staticmethod
    def plate(nx, ny, Lx, Ly, Re, yp=1.0):
        return RefMesh(lib().ref_mesh_plate(nx, ny, Lx, Ly, Re, yp))

    @staticmethod
    def bfs(nxu, nxd, nyu, nyd, Lu, Ld, hs, H, Re=0.0, yp=1.0):
        return RefMesh(lib().ref_mesh_bfs(nxu, nxd, nyu, nyd, Lu, Ld, hs, H, Re, yp))

    @staticmethod
    def curved_periodic(xn, yb, ytop, ny, Re, yp=1.0):
        xn = np.ascontiguousarray(xn, np.float64)
        yb = np.ascontiguousarray(yb, np.float64)
        return RefMesh(lib().ref_mesh_curved_periodic(_d(xn), _d(yb), xn.size, ytop, ny, Re, yp))

    def wall_distance(self):
        lib().ref_mesh_wall_distance(self.h)

    def set_patch_type(self, name, t):
        lib().ref_mesh_set_patch_type(self.h, name.encode(), t.encode())

    def save(self, path):
        if lib().ref_mesh_save(self.h, path.encode()) != 0:
            raise RuntimeError(lib().ref_last_error().decode())

    def dump(self) -> dict:
        s = np.zeros(6, np.int32)
        lib().ref_mesh_sizes(self.h, _i(s))
        nC, nF, nIF, nP, nN, ncf = (int(v) for v in s)
        out = dict(owner=np.zeros(nF, np.int32), neighbour=np.zeros(nF, np.int32),
                   face_patch=np.zeros(nF, np.int32), face_center=np.zeros((nF, 3)),
                   face_normal=np.zeros((nF, 3)), face_area=np.zeros(nF), face_delta=np.zeros(nF),
                   face_d=np.zeros((nF, 3)), face_weight=np.zeros(nF), cell_center=np.zeros((nC, 3)),
                   cell_volume=np.zeros(nC), wall_dist=np.full(nC, np.nan),
                   cell_face_offset=np.zeros(nC + 1, np.int32), cell_faces=np.zeros(ncf, np.int32),
                   patch_type=np.zeros(nP, np.int32), patch_offset=np.zeros(nP + 1, np.int32),
                   nodes=np.zeros((nN, 3)))
        # patch faces count is the number of boundary faces on normal meshes
        out["patch_faces"] = np.zeros(max(nF, 1), np.int32)
        o = out
        lib().ref_mesh_dump(self.h, _i(o["owner"]), _i(o["neighbour"]), _i(o["face_patch"]),
                            _d(o["face_center"]), _d(o["face_normal"]), _d(o["face_area"]),
                            _d(o["face_delta"]), _d(o["face_d"]), _d(o["face_weight"]),
                            _d(o["cell_center"]), _d(o["cell_volume"]), _d(o["wall_dist"]),
                            _i(o["cell_face_offset"]), _i(o["cell_faces"]), _i(o["patch_type"]),
                            _i(o["patch_offset"]), _i(o["patch_faces"]), _d(o["nodes"]))
        o["patch_faces"] = o["patch_faces"][:o["patch_offset"][-1]]
        buf = C.create_string_buffer(1 << 16)
        lib().ref_mesh_patch_names(self.h, buf, 1 << 16)
        o["patch_names"] = buf.value.decode().split("\n")[:-1]
        o["n_internal"] = nIF
        return o

    def bc_preset(self, kind: int, Uin: float, kIn: float, omIn: float):
        np_ = self.dump()["patch_type"].size
        types = np.zeros(4 * np_, np.int32)
        vals = np.zeros(6 * np_)
        if lib().ref_bc_preset(self.h, kind, Uin, kIn, omIn, _i(types), _d(vals)) != 0:
            raise RuntimeError("bad preset")
        return types.reshape(np_, 4), vals.reshape(np_, 6)

    def solve(self, bcs, nu: float, settings: Settings, coeffs, variant: int, init: Init,
              n_cells: int, n_bnd: int, residual_capacity: int = 0, verbose: int = 0, b_target=None):
        arrays, st = state_arrays(n_cells, n_bnd)
        bt = None if b_target is None else np.ascontiguousarray(np.asarray(b_target, np.float64).reshape(-1))
        lib().ref_set_target_anisotropy(_d(bt) if bt is not None else None, n_cells)
        hist = History()
        res = None
        if residual_capacity:
            res = np.zeros((residual_capacity, 6))
            hist.residual_capacity = residual_capacity
            hist.residuals = _d(res)
        cf = np.ascontiguousarray(coeffs, np.float64)
        try:
            rc = lib().ref_solve(self.h, bcs, nu, C.byref(settings), _d(cf), variant, C.byref(init),
                                 C.byref(st), C.byref(hist), verbose)
        finally:
            lib().ref_set_target_anisotropy(None, 0)
        if rc != 0:
            raise RuntimeError(lib().ref_last_error().decode())
        arrays["turb_established"] = st.turb_established
        return arrays, hist, res

    def observe(self, observables, nu: float, state: dict):
        """The reference ObservationOperator on `state` (arrays U, p, k, omega,
        nuT and the boundary values): predictions and the log-likelihood.
        `observables` is a ctypes array of btm_observable records."""
        n = len(observables)
        keep = []

        def arr(a):
            a = np.ascontiguousarray(a, np.float64).reshape(-1)
            keep.append(a)
            return _d(a)

        st = State()
        st.U, st.Ub = arr(state["U"]), arr(state["Ub"])
        st.p, st.pb = arr(state["p"]), arr(state["pb"])
        st.k, st.kb = arr(state["k"]), arr(state["kb"])
        st.omega, st.omegab = arr(state["omega"]), arr(state["omegab"])
        st.nuT = arr(state["nuT"])
        pred = np.zeros(max(n, 1))
        ll = np.zeros(1)
        if lib().ref_observe(self.h, n, C.cast(observables, C.c_void_p), float(nu), C.byref(st), _d(pred),
                             _d(ll)) != 0:
            raise RuntimeError(lib().ref_last_error().decode())
        return pred[:n].tolist(), float(ll[0])

    def green_gauss(self, phi, phib):
        nC = phi.size
        g = np.zeros((nC, 3))
        lib().ref_green_gauss(self.h, _d(np.ascontiguousarray(phi)), _d(np.ascontiguousarray(phib)), _d(g))
        return g

    def sst_fields(self, coeffs, variant, nu, U, Ub, k, kb, om, omb):
        nC = k.size
        outs = [np.zeros(nC) for _ in range(6)]
        cf = np.ascontiguousarray(coeffs, np.float64)
        args = [np.ascontiguousarray(a, np.float64) for a in (U, Ub, k, kb, om, omb)]
        lib().ref_sst_fields(self.h, _d(cf), variant, nu, *[_d(a) for a in args], *[_d(o) for o in outs])
        return dict(zip(("nuT", "F1", "F2", "Pk", "CDkw", "Smag"), outs))


def linear_solve(kind, own, nbr, diag, upper, lower, source, x0, max_iter, tol):
    own = np.ascontiguousarray(own, np.int32)
    nbr = np.ascontiguousarray(nbr, np.int32)
    x = np.array(x0, dtype=np.float64)
    res = np.zeros(4)
    arrs = [np.ascontiguousarray(a, np.float64) for a in (diag, upper, lower, source)]
    lib().ref_linear_solve(kind, x.size, own.size, _i(own), _i(nbr), *[_d(a) for a in arrs], _d(x),
                           max_iter, tol, _d(res))
    return x, res


def matvec(own, nbr, diag, upper, lower, x):
    own = np.ascontiguousarray(own, np.int32)
    nbr = np.ascontiguousarray(nbr, np.int32)
    y = np.zeros(len(diag))
    arrs = [np.ascontiguousarray(a, np.float64) for a in (diag, upper, lower, x)]
    lib().ref_matvec(len(diag), own.size, _i(own), _i(nbr), *[_d(a) for a in arrs], _d(y))
    return y
