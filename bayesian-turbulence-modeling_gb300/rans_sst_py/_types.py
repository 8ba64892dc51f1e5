"""Host-side value types of the drop-in module, mirroring the reference's
pybind11 surface (python/Bindings.cpp:276-465) with the same names, fields,
defaults and error behaviour."""
from __future__ import annotations

import enum
import math
from typing import List, Optional, Sequence

import numpy as np


class Vec3:
    """3-vector (core/include/Mesh.hpp:11-33, Bindings.cpp:461-465)."""

    __slots__ = ("x", "y", "z")

    def __init__(self, x: float = 0.0, y: float = 0.0, z: float = 0.0):
        self.x, self.y, self.z = float(x), float(y), float(z)

    def as_tuple(self):
        return (self.x, self.y, self.z)

    def __repr__(self):
        return f"Vec3({self.x}, {self.y}, {self.z})"


def _vec(v) -> Vec3:
    if isinstance(v, Vec3):
        return v
    x, y, z = v
    return Vec3(x, y, z)


class EvaluationStatus(enum.IntEnum):
    """EvaluationStatus (core/include/EvaluationTypes.hpp:6-12); the Python
    name of Diverged is DivergenceDetected as in Bindings.cpp:276-281."""

    Converged = 0
    Unconverged = 1
    DivergenceDetected = 2
    InvalidParameters = 3
    Unknown = 4

    def __str__(self):
        return "EvaluationStatus." + self.name


class EvaluationResult:
    """EvaluationResult (EvaluationTypes.hpp:24-29): read-only attributes."""

    __slots__ = ("_status", "_loglik", "_pred", "_iters")

    def __init__(self, status=EvaluationStatus.Unknown, log_lik=-1e30, predictions=None,
                 simple_iters=0):
        self._status = EvaluationStatus(status)
        self._loglik = float(log_lik)
        self._pred = list(predictions or [])
        self._iters = int(simple_iters)

    status = property(lambda s: s._status)
    log_lik = property(lambda s: s._loglik)
    predictions = property(lambda s: list(s._pred))
    simple_iters = property(lambda s: s._iters)

    def __repr__(self):
        return (f"EvaluationResult(status={self._status.name}, log_lik={self._loglik}, "
                f"simple_iters={self._iters}, n_pred={len(self._pred)})")


COEFF_NAMES = ("sigma_k1", "sigma_w1", "beta1", "alpha1", "sigma_k2", "sigma_w2", "beta2",
               "alpha2", "betaStar", "a1", "kappa")
COEFF_DEFAULTS = (0.85, 0.5, 0.075, 5.0 / 9.0, 1.0, 0.856, 0.0828, 0.44, 0.09, 0.31, 0.41)
COEFF_LOWER = (0.1, 0.1, 0.01, 0.1, 0.1, 0.1, 0.01, 0.1, 0.01, 0.1, 0.35)
COEFF_UPPER = (2.0, 2.0, 0.2, 1.5, 2.0, 2.0, 0.2, 1.5, 0.2, 0.8, 0.50)


class SSTCoefficients:
    """SST constants (core/include/SSTModel.hpp:9-40)."""

    def __init__(self):
        for n, v in zip(COEFF_NAMES, COEFF_DEFAULTS):
            setattr(self, n, v)

    def to_vector(self) -> List[float]:
        return [float(getattr(self, n)) for n in COEFF_NAMES]

    @staticmethod
    def from_vector(v: Sequence[float]) -> "SSTCoefficients":
        if len(v) != 11:
            raise RuntimeError("Expected 11 SST coefficients")
        c = SSTCoefficients()
        for n, x in zip(COEFF_NAMES, v):
            setattr(c, n, float(x))
        return c


class InferenceParameterSet:
    """theta <-> 11 SST coefficients (core/include/InferenceParameters.hpp:18-162)."""

    def __init__(self, name: str = "", active_indices: Sequence[int] = (), base=None):
        self.name = name
        self.activeIndices = list(active_indices)
        self.base = base if base is not None else SSTCoefficients()

    def n_active(self) -> int:
        return len(self.activeIndices)

    def active_names(self) -> List[str]:
        return [COEFF_NAMES[i] for i in self.activeIndices]

    def pack(self, c: SSTCoefficients) -> List[float]:
        full = c.to_vector()
        return [full[i] for i in self.activeIndices]

    def unpack(self, theta: Sequence[float]) -> SSTCoefficients:
        theta = list(theta)
        if len(theta) != self.n_active():
            raise RuntimeError(f"theta size mismatch: expected {self.n_active()}, got {len(theta)}")
        full = self.base.to_vector()
        for i, idx in enumerate(self.activeIndices):
            full[idx] = float(theta[i])
        return SSTCoefficients.from_vector(full)

    def unpack_vector(self, theta: Sequence[float]) -> List[float]:
        return self.unpack(theta).to_vector()

    def lower_bounds(self) -> List[float]:
        return [COEFF_LOWER[i] for i in self.activeIndices]

    def upper_bounds(self) -> List[float]:
        return [COEFF_UPPER[i] for i in self.activeIndices]

    def in_bounds(self, theta: Sequence[float]) -> bool:
        """InferenceParameterSet::inBounds (InferenceParameters.hpp:102-111):
        a size mismatch is out of bounds; NaN/Inf are out of bounds."""
        theta = list(theta)
        if len(theta) != self.n_active():
            return False
        lo, hi = self.lower_bounds(), self.upper_bounds()
        for i in range(self.n_active()):
            t = float(theta[i])
            if t < lo[i] or t > hi[i]:
                return False
            if math.isnan(t) or math.isinf(t):
                return False
        return True

    @staticmethod
    def a1_betaStar():
        return InferenceParameterSet("a1_betaStar", [9, 8])

    @staticmethod
    def inlet_turb():
        return InferenceParameterSet("inletTurb", [2, 1])

    @staticmethod
    def near_wall4():
        return InferenceParameterSet("nearWall4", [9, 8, 2, 0])

    @staticmethod
    def all11():
        return InferenceParameterSet("all11", list(range(11)))

    @staticmethod
    def live10():
        return InferenceParameterSet("live10", list(range(10)))

    @staticmethod
    def from_indices(name: str, indices: Sequence[int]):
        idx = list(indices)
        if not idx:
            raise RuntimeError("fromIndices: need at least one active index")
        for i, a in enumerate(idx):
            if a < 0 or a > 10:
                raise RuntimeError("fromIndices: index out of range [0,10]")
            if a in idx[i + 1:]:
                raise RuntimeError("fromIndices: duplicate index")
        return InferenceParameterSet(name, idx)


class SolverSettings:
    """SolverSettings (core/include/FlowFields.hpp:53-132) with the snake_case
    attribute names of Bindings.cpp:414-441.  pressure_solver /
    momentum_solver / turbulence_solver are also settable here,
    `precision` ("fp64", the reference's arithmetic, or "mixed": FP32 bulk
    with FP64 state, defects and refinement) selects the device engine, and
    `amg_order` ("auto", "reference" or "multicolour") the form of the FP64
    engine's AMG-preconditioned CG (BTM_AMG_* in the C header), and
    `anderson_depth` (0 .. 8) the depth of the Anderson acceleration of the
    mixed engine's outer iteration (0: plain SIMPLE iterations; the FP64
    engine, the reference's drop-in, ignores it)."""

    def __init__(self):
        self.max_iterations = 500
        self.convergence_tol = 1e-5
        self.divergence_limit = 1e6
        self.alpha_u = 0.7
        self.alpha_p = 0.3
        self.alpha_k = 0.5
        self.alpha_omega = 0.5
        self.alpha_t = 0.7
        self.inner_iterations = 200
        self.inner_tolerance = 1e-3
        self.turb_start_iter = 5
        self.turb_update_interval = 1
        self.nut_floor_iters = 500
        self.rhie_chow_all_meshes = False
        self.alpha_injection = 0.3
        self.body_force = Vec3(0.0, 0.0, 0.0)
        self.k_min = 1e-10
        self.k_max = 1e10
        self.omega_min = 1e-6
        self.report_interval = 10
        self.verbose = True
        self.pressure_solver = "AMG"
        self.momentum_solver = "BiCGSTAB"
        self.turbulence_solver = "BiCGSTAB"
        self.use_wall_functions = False
        self.von_karman = 0.41
        self.wall_fn_E = 9.0
        self.sst_variant = 0
        self.precision = "fp64"
        self.amg_order = "auto"
        self.anderson_depth = 8

    def copy(self) -> "SolverSettings":
        s = SolverSettings()
        s.__dict__.update(self.__dict__)
        s.body_force = Vec3(*_vec(self.body_force).as_tuple())
        return s


class BCType(enum.IntEnum):
    """BCType (core/include/BoundaryCondition.hpp:12-18)."""

    Dirichlet = 0
    Neumann = 1
    InletVelocity = 2
    OutletPressure = 3
    WallNoSlip = 4
    WallKOmega = 5
    WallMoving = 6
    Symmetry = 7
    Cyclic = 8


class PatchBC:
    """PatchBC (BoundaryCondition.hpp:20-32)."""

    def __init__(self, type=BCType.Neumann, value=0.0, vec_value=(0.0, 0.0, 0.0), patch_name=""):  # noqa: A002
        self.type = BCType(type)
        self.value = float(value)
        self.vecValue = _vec(vec_value)
        self.patchName = patch_name
        self.vecProfile: Optional[np.ndarray] = None
        self.scalarProfile: Optional[np.ndarray] = None


class FlowBoundaryConditions:
    """Per-patch BCs of U, p, k, omega with the reference presets
    (core/include/BoundaryCondition.hpp:36-190)."""

    def __init__(self):
        self.velocityBC: List[PatchBC] = []
        self.pressureBC: List[PatchBC] = []
        self.kBC: List[PatchBC] = []
        self.omegaBC: List[PatchBC] = []

    @staticmethod
    def channel_defaults(mesh, Uin: float, kIn: float, omIn: float) -> "FlowBoundaryConditions":
        bc = FlowBoundaryConditions()
        for name, ptype in zip(mesh.patch_names(), mesh.patch_types()):
            if ptype == "wall":
                u = PatchBC(BCType.WallNoSlip, patch_name=name)
                p = PatchBC(BCType.Neumann, patch_name=name)
                k = PatchBC(BCType.WallKOmega, patch_name=name)
                w = PatchBC(BCType.WallKOmega, patch_name=name)
            elif ptype == "inlet":
                u = PatchBC(BCType.InletVelocity, 0.0, (Uin, 0.0, 0.0), name)
                p = PatchBC(BCType.Neumann, 0.0, patch_name=name)
                k = PatchBC(BCType.Dirichlet, kIn, patch_name=name)
                w = PatchBC(BCType.Dirichlet, omIn, patch_name=name)
            elif ptype == "outlet":
                u = PatchBC(BCType.Neumann, patch_name=name)
                p = PatchBC(BCType.OutletPressure, 0.0, patch_name=name)
                k = PatchBC(BCType.Neumann, patch_name=name)
                w = PatchBC(BCType.Neumann, patch_name=name)
            elif ptype == "symmetry":
                u = PatchBC(BCType.Symmetry, patch_name=name)
                p = PatchBC(BCType.Neumann, patch_name=name)
                k = PatchBC(BCType.Neumann, patch_name=name)
                w = PatchBC(BCType.Neumann, patch_name=name)
            else:
                u, p, k, w = (PatchBC(patch_name=name) for _ in range(4))
            bc.velocityBC.append(u)
            bc.pressureBC.append(p)
            bc.kBC.append(k)
            bc.omegaBC.append(w)
        return bc

    @staticmethod
    def bfs_defaults(mesh, Uin, kIn, omIn):
        return FlowBoundaryConditions.channel_defaults(mesh, Uin, kIn, omIn)

    @staticmethod
    def flat_plate_defaults(mesh, Uinf, kIn, omIn):
        bc = FlowBoundaryConditions.channel_defaults(mesh, Uinf, kIn, omIn)
        for p, name in enumerate(mesh.patch_names()):
            if name == "top":
                bc.velocityBC[p] = PatchBC(BCType.Dirichlet, 0.0, (Uinf, 0.0, 0.0), name)
                bc.pressureBC[p] = PatchBC(BCType.Neumann, 0.0, patch_name=name)
                bc.kBC[p] = PatchBC(BCType.Dirichlet, kIn, patch_name=name)
                bc.omegaBC[p] = PatchBC(BCType.Dirichlet, omIn, patch_name=name)
        return bc

    @staticmethod
    def couette_defaults(mesh, Uwall, kIn, omIn):
        bc = FlowBoundaryConditions.channel_defaults(mesh, 0.5 * Uwall, kIn, omIn)
        for p, name in enumerate(mesh.patch_names()):
            if name == "top":
                bc.velocityBC[p] = PatchBC(BCType.WallMoving, 0.0, (Uwall, 0.0, 0.0), name)
            elif name == "inlet":
                bc.velocityBC[p] = PatchBC(BCType.Neumann, patch_name=name)
                bc.pressureBC[p] = PatchBC(BCType.Neumann, patch_name=name)
                bc.kBC[p] = PatchBC(BCType.Neumann, patch_name=name)
                bc.omegaBC[p] = PatchBC(BCType.Neumann, patch_name=name)
        return bc

    @staticmethod
    def periodic_couette(mesh, Uwall: float, top: str = "top_wall") -> "FlowBoundaryConditions":
        """Streamwise-periodic plane Couette (no reference counterpart): the
        wall patches keep the channel wall BCs, the `top` patch translates at
        Uwall (WallMoving); no inlet/outlet."""
        bc = FlowBoundaryConditions.channel_defaults(mesh, 0.0, 0.0, 0.0)
        for p, name in enumerate(mesh.patch_names()):
            if name == top:
                bc.velocityBC[p] = PatchBC(BCType.WallMoving, 0.0, (Uwall, 0.0, 0.0), name)
        return bc

    @staticmethod
    def _patch_index(mesh, name):
        for p, n in enumerate(mesh.patch_names()):
            if n == name:
                return p
        raise RuntimeError("FlowBoundaryConditions: unknown patch '" + name + "'")

    def set_velocity_profile(self, mesh, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        if v.ndim != 2 or v.shape[1] != 3:
            raise RuntimeError("velocity profile must be (n_faces, 3)")
        p = self._patch_index(mesh, name)
        if v.shape[0] != mesh.patches[p][2].size:
            raise RuntimeError("velocity profile size != patch face count")
        self.velocityBC[p].vecProfile = v

    def set_k_profile(self, mesh, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        p = self._patch_index(mesh, name)
        if v.size != mesh.patches[p][2].size:
            raise RuntimeError("k profile size != patch face count")
        self.kBC[p].scalarProfile = v

    def set_omega_profile(self, mesh, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        p = self._patch_index(mesh, name)
        if v.size != mesh.patches[p][2].size:
            raise RuntimeError("omega profile size != patch face count")
        self.omegaBC[p].scalarProfile = v
