"""ctypes mirrors of the plain-C structs declared in include/btm_gb300.h, for
the CPU checkers (the restatement in simple_oracle.c and the reference driver).

TEST INFRASTRUCTURE ONLY; kept separate from the product's own bindings so the
checker shares no code with the thing it checks.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class MeshDesc(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("n_faces", C.c_int32), ("n_internal_faces", C.c_int32),
                ("n_patches", C.c_int32), ("owner", _ip), ("neighbour", _ip),
                ("face_center", _dp), ("face_normal", _dp), ("face_area", _dp),
                ("face_delta", _dp), ("face_d", _dp), ("face_weight", _dp),
                ("cell_center", _dp), ("cell_volume", _dp), ("wall_distance", _dp),
                ("patch_type", _ip), ("patch_offset", _ip), ("patch_faces", _ip)]


class PatchBC(C.Structure):
    _fields_ = [("u_type", C.c_int32), ("p_type", C.c_int32), ("k_type", C.c_int32),
                ("omega_type", C.c_int32), ("u_value", C.c_double * 3), ("p_value", C.c_double),
                ("k_value", C.c_double), ("omega_value", C.c_double), ("u_profile", _dp),
                ("k_profile", _dp), ("omega_profile", _dp)]


class Settings(C.Structure):
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


class State(C.Structure):
    _fields_ = [(n, _dp) for n in ("U", "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw",
                                   "Ub", "pb", "kb", "omegab")] + [("turb_established", C.c_int32)]


class Init(C.Structure):
    _fields_ = [("mode", C.c_int32), ("u", C.c_double * 3), ("p", C.c_double), ("k", C.c_double),
                ("omega", C.c_double), ("warm", C.POINTER(State))]


class History(C.Structure):
    _fields_ = [("status", C.c_int32), ("converged", C.c_int32), ("diverged", C.c_int32),
                ("final_iter", C.c_int32), ("iterations_run", C.c_int32),
                ("inner_iterations", C.c_int64), ("last_residual", C.c_double * 6),
                ("residual_capacity", C.c_int32), ("residuals", _dp), ("phase_ms", C.c_double * 10),
                ("solve_ms", C.c_double), ("finish_ms", C.c_double), ("inner_split", C.c_int64 * 4),
                ("polish_start", C.c_int32), ("predictions", C.POINTER(C.c_double)), ("log_lik", C.c_double)]


CELL_FIELDS = ("p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw")
BND_FIELDS = ("pb", "kb", "omegab")


def state_arrays(n_cells: int, n_bnd: int):
    """Allocate numpy arrays for a full state and a State struct pointing at them."""
    arrays = {"U": np.zeros((n_cells, 3)), "Ub": np.zeros((max(n_bnd, 0), 3))}
    for f in CELL_FIELDS:
        arrays[f] = np.zeros(n_cells)
    for f in BND_FIELDS:
        arrays[f] = np.zeros(max(n_bnd, 0))
    st = State()
    for k, a in arrays.items():
        setattr(st, k, a.ctypes.data_as(_dp))
    return arrays, st


def state_from_arrays(arrays: dict):
    """State struct viewing caller arrays (kept alive by the caller)."""
    st = State()
    keep = {}
    for k in ("U", "Ub") + CELL_FIELDS + BND_FIELDS:
        a = np.ascontiguousarray(arrays[k], np.float64)
        keep[k] = a
        setattr(st, k, a.ctypes.data_as(_dp))
    st.turb_established = int(arrays.get("turb_established", 0))
    return st, keep


def mesh_desc(m: dict):
    """MeshDesc over a dict of numpy mesh arrays (keys as in refdriver.RefMesh.dump)."""
    keep = {}

    def d(name, dtype):
        a = np.ascontiguousarray(m[name], dtype)
        keep[name] = a
        return a.ctypes.data_as(_dp if dtype == np.float64 else _ip)

    md = MeshDesc()
    md.n_cells = int(np.asarray(m["cell_volume"]).size)
    md.n_faces = int(np.asarray(m["owner"]).size)
    md.n_internal_faces = int(m["n_internal"])
    md.n_patches = int(np.asarray(m["patch_type"]).size)
    md.owner, md.neighbour = d("owner", np.int32), d("neighbour", np.int32)
    md.face_center, md.face_normal = d("face_center", np.float64), d("face_normal", np.float64)
    md.face_area, md.face_delta = d("face_area", np.float64), d("face_delta", np.float64)
    md.face_d, md.face_weight = d("face_d", np.float64), d("face_weight", np.float64)
    md.cell_center, md.cell_volume = d("cell_center", np.float64), d("cell_volume", np.float64)
    md.wall_distance = d("wall_dist", np.float64)
    md.patch_type, md.patch_offset = d("patch_type", np.int32), d("patch_offset", np.int32)
    md.patch_faces = d("patch_faces", np.int32)
    return md, keep
