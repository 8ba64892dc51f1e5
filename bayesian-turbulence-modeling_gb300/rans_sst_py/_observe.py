"""Observation operator H(fields) and the Gaussian log-likelihood, host side.

Mirror of the reference ObservationOperator
(core/include/ObservationOperator.hpp:46-378): the same observable kinds, the
same nearest-cell / nearest-wall-face searches (first minimum wins), the same
molecular wall-shear definitions and sub-face interpolated zero crossings.
"""
from __future__ import annotations

import enum
import math
from typing import List

import numpy as np

from ._types import Vec3, _vec


class ObsType(enum.IntEnum):
    Drag = 0
    PressureTap = 1
    VelocityProfile = 2
    SkinFriction = 3
    SeparationPoint = 4
    ReattachmentLength = 5


class _Obs:
    __slots__ = ("type", "observed", "sigma_obs", "sigma_model", "patchName", "location",
                 "component", "referenceArea", "refVelocity", "refPressure", "refDensity")

    def __init__(self, t, observed, sigma, sigma_model):
        self.type = t
        self.observed = float(observed)
        self.sigma_obs = float(sigma)
        self.sigma_model = float(sigma_model)
        self.patchName = ""
        self.location = Vec3()
        self.component = 0
        self.referenceArea = 1.0
        self.refVelocity = 1.0
        self.refPressure = 0.0
        self.refDensity = 1.0

    def total_variance(self):
        return self.sigma_obs * self.sigma_obs + self.sigma_model * self.sigma_model


def _norm2(a, loc):
    d0 = a[..., 0] - loc.x
    d1 = a[..., 1] - loc.y
    d2 = a[..., 2] - loc.z
    return d0 * d0 + d1 * d1 + d2 * d2


class ObservationOperator:
    """Bindings.cpp:444-458 surface plus the pressure-tap / separation adders."""

    def __init__(self):
        self._obs: List[_Obs] = []

    def add_drag(self, wall_patch, cd_obs, sigma, ref_area, ref_vel, sigma_model=0.0):
        o = _Obs(ObsType.Drag, cd_obs, sigma, sigma_model)
        o.patchName, o.referenceArea, o.refVelocity = wall_patch, float(ref_area), float(ref_vel)
        self._obs.append(o)

    def add_pressure_tap(self, location, cp_obs, sigma, ref_vel, sigma_model=0.0, ref_pressure=0.0,
                         ref_density=1.0):
        o = _Obs(ObsType.PressureTap, cp_obs, sigma, sigma_model)
        o.location, o.refVelocity = _vec(location), float(ref_vel)
        o.refPressure, o.refDensity = float(ref_pressure), float(ref_density)
        self._obs.append(o)

    def add_velocity_profile(self, location, component, u_obs, sigma, sigma_model=0.0):
        o = _Obs(ObsType.VelocityProfile, u_obs, sigma, sigma_model)
        o.location, o.component = _vec(location), int(component)
        self._obs.append(o)

    def add_skin_friction(self, wall_patch, location, cf_obs, sigma, ref_vel, sigma_model=0.0):
        o = _Obs(ObsType.SkinFriction, cf_obs, sigma, sigma_model)
        o.patchName, o.location, o.refVelocity = wall_patch, _vec(location), float(ref_vel)
        self._obs.append(o)

    def add_separation_point(self, wall_patch, xsep_obs, sigma, sigma_model=0.0):
        o = _Obs(ObsType.SeparationPoint, xsep_obs, sigma, sigma_model)
        o.patchName = wall_patch
        self._obs.append(o)

    def add_reattachment_length(self, wall_patch, xr_obs, sigma, sigma_model=0.0):
        o = _Obs(ObsType.ReattachmentLength, xr_obs, sigma, sigma_model)
        o.patchName = wall_patch
        self._obs.append(o)

    def n_obs(self) -> int:
        return len(self._obs)

    def observables(self):
        return list(self._obs)

    # ---- evaluation (ObservationOperator.hpp:159-364) ----------------------
    @staticmethod
    def _nearest_cell(mesh, loc):
        return int(np.argmin(_norm2(mesh.cell_center, loc)))

    @staticmethod
    def _patch_faces(mesh, name):
        return mesh.patches[mesh.patch_by_name(name)][2]

    def _drag(self, mesh, f, nu, o):
        faces = self._patch_faces(mesh, o.patchName)
        force = 0.0
        nIF = mesh.n_internal
        for fi in faces:
            ow = mesh.owner[fi]
            Sf = mesh.face_area[fi]
            force += f["p"][ow] * mesh.face_normal[fi, 0] * Sf
            delta = max(mesh.face_delta[fi], 1e-20)
            Uw_x = f["Ub"][fi - nIF, 0]
            tau_x = nu * (f["U"][ow, 0] - Uw_x) / delta
            force += tau_x * Sf
        dyn = 0.5 * o.refVelocity * o.refVelocity
        return force / (dyn * o.referenceArea)

    def _cf(self, mesh, f, nu, o):
        faces = self._patch_faces(mesh, o.patchName)
        if faces.size == 0:
            return 0.0
        fi = int(faces[int(np.argmin(_norm2(mesh.face_center[faces], o.location)))])
        ow = mesh.owner[fi]
        delta = max(mesh.face_delta[fi], 1e-20)
        Uc = f["U"][ow]
        n = mesh.face_normal[fi]
        dot = Uc[0] * n[0] + Uc[1] * n[1] + Uc[2] * n[2]
        ut = (Uc[0] - n[0] * dot, Uc[1] - n[1] * dot, Uc[2] - n[2] * dot)
        tau = nu * math.sqrt(ut[0] * ut[0] + ut[1] * ut[1] + ut[2] * ut[2]) / delta
        dyn = 0.5 * o.refVelocity * o.refVelocity
        return tau / max(dyn, 1e-20)

    def _velocity(self, mesh, f, o):
        comp = 0 if o.component == 0 else (1 if o.component == 1 else 2)
        return float(f["U"][self._nearest_cell(mesh, o.location), comp])

    def _pressure(self, mesh, f, o):
        ci = self._nearest_cell(mesh, o.location)
        dyn = 0.5 * o.refDensity * o.refVelocity * o.refVelocity
        return (f["p"][ci] - o.refPressure) / max(dyn, 1e-20)

    @staticmethod
    def _wall_tau_x(mesh, f, nu, faces):
        ow = mesh.owner[faces]
        delta = np.maximum(mesh.face_delta[faces], 1e-20)
        Uc = f["U"][ow]
        n = mesh.face_normal[faces]
        dot = Uc[:, 0] * n[:, 0] + Uc[:, 1] * n[:, 1] + Uc[:, 2] * n[:, 2]
        utx = Uc[:, 0] - n[:, 0] * dot
        return nu * utx / delta, mesh.face_center[faces, 0]

    def _separation(self, mesh, f, nu, o):
        faces = self._patch_faces(mesh, o.patchName)
        taus, xs = self._wall_tau_x(mesh, f, nu, faces)
        have, prev_tau, prev_x = False, 1.0, 0.0
        for tau, x in zip(taus, xs):
            if have and prev_tau > 0 and tau <= 0:
                denom = prev_tau - tau
                frac = prev_tau / denom if abs(denom) > 1e-30 else 0.0
                return prev_x + frac * (x - prev_x)
            prev_tau, prev_x, have = tau, x, True
        return 0.0

    def _reattachment(self, mesh, f, nu, o):
        faces = self._patch_faces(mesh, o.patchName)
        xr_default = float(mesh.face_center[faces[-1], 0]) if faces.size else 0.0
        taus, xs = self._wall_tau_x(mesh, f, nu, faces)
        have, prev_tau, prev_x = False, -1.0, 0.0
        for tau, x in zip(taus, xs):
            if have and prev_tau < 0 and tau >= 0:
                denom = tau - prev_tau
                frac = (-prev_tau) / denom if abs(denom) > 1e-30 else 0.0
                return prev_x + frac * (x - prev_x)
            prev_tau, prev_x, have = tau, x, True
        return xr_default

    def evaluate(self, mesh, fields: dict, nu: float) -> List[float]:
        out = []
        for o in self._obs:
            if o.type == ObsType.Drag:
                out.append(float(self._drag(mesh, fields, nu, o)))
            elif o.type == ObsType.PressureTap:
                out.append(float(self._pressure(mesh, fields, o)))
            elif o.type == ObsType.VelocityProfile:
                out.append(float(self._velocity(mesh, fields, o)))
            elif o.type == ObsType.SkinFriction:
                out.append(float(self._cf(mesh, fields, nu, o)))
            elif o.type == ObsType.SeparationPoint:
                out.append(float(self._separation(mesh, fields, nu, o)))
            else:
                out.append(float(self._reattachment(mesh, fields, nu, o)))
        return out

    def log_likelihood(self, mesh, fields: dict, nu: float, pred=None) -> float:
        if pred is None:
            pred = self.evaluate(mesh, fields, nu)
        ll = 0.0
        for o, p in zip(self._obs, pred):
            var = o.total_variance()
            if var < 1e-30:
                var = 1e-30
            diff = p - o.observed
            ll += -0.5 * diff * diff / var
        return ll
