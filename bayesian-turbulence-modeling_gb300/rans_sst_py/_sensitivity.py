"""ParameterSensitivity with the warm-started finite-difference Jacobian as one
batched device launch (incompressible/include/ParameterSensitivity.hpp:48-81,
incompressible/src/ParameterSensitivity.cpp:26-37, 691-745).

The reference runs the 22 warm re-solves of eta_jacobian_warm_fd one after
another; here they are independent instances of one solve_batch launch, each
warm-started from the same converged state, and the observation operator and
the Gaussian log-likelihood of each are evaluated on the device at the end of
its solve (only those numbers leave the device).  For observe/log_lik at the
kept state, closure fields are recomputed on the device (the SST phase,
reference-rounded) and the nu_t floor 0.1 nu is applied as the reference does.  The tangent / adjoint
ground-work methods of the reference class are outside the rebuilt path.
"""
from __future__ import annotations

import copy
from typing import List

import numpy as np

from ._forward import solve, solve_batch
from ._lib import PHASES, Case, check, dptr, lib
from ._types import EvaluationStatus, SolverSettings, Vec3, _vec


class TangentGradientResult:
    """TangentGradientResult (ParameterSensitivity.hpp): d_obs_d_theta is
    n_obs x 11, log_lik_gradient has 11 entries; krylov_converged[j] is 1 when
    both warm solves of coefficient j ran without divergence."""

    def __init__(self, n_obs: int):
        self.d_obs_d_theta = [[0.0] * 11 for _ in range(n_obs)]
        self.log_lik_gradient = [0.0] * 11
        self.krylov_iters = [0] * 11
        self.krylov_rel_res = [0.0] * 11
        self.krylov_converged = [0] * 11
        self.n_residual_evals = 0


def _closure_fields(case: Case, coeffs, variant: int, state: dict) -> dict:
    """SSTModel::computeFields at `state` on the device: nu_t, F1, F2, Pk, CDkw."""
    nC, nB, nIF = case.n_cells, case.n_bnd, case.n_internal
    zeros = np.zeros(nC)
    parts = [np.asarray(state["U"], float).ravel()] + [np.asarray(state.get(k, zeros), float) for k in (
        "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw")] + [zeros, zeros]
    parts += [np.asarray(state["Ub"], float).ravel(), np.asarray(state["pb"], float),
              np.asarray(state["kb"], float), np.asarray(state["omegab"], float)]
    parts += [np.zeros(nC + 2 * nIF), zeros, zeros]
    inp = np.ascontiguousarray(np.concatenate(parts))
    out = np.zeros(6 * nC)
    cf = np.ascontiguousarray(np.asarray(coeffs, float))
    check(lib().btm_debug_phase(case.h, PHASES["sst"], dptr(cf), int(variant), 0, dptr(inp), inp.size, dptr(out),
                                out.size))
    o = out.reshape(6, nC)
    return {"nuT": o[0].copy(), "F1": o[1].copy(), "F2": o[2].copy(), "Pk": o[3].copy(), "CDkw": o[4].copy()}


class ParameterSensitivity:
    """The incompressible ParameterSensitivity surface on the device solver
    (python/Bindings.cpp:537-581): state, observation and the warm-FD
    Jacobian."""

    def __init__(self, mesh, obs_op, bcs, nu: float, settings: SolverSettings = None,
                 u_init=Vec3(1.0, 0.0, 0.0), p_init: float = 0.0, k_init: float = 1e-4, omega_init: float = 1.0):
        self._mesh = mesh
        self._obs = copy.deepcopy(obs_op)
        self._bcs = copy.deepcopy(bcs)
        self._nu = float(nu)
        self._settings = (settings or SolverSettings()).copy()
        u = _vec(u_init)
        self._init = dict(u=(u.x, u.y, u.z), p=float(p_init), k=float(k_init), omega=float(omega_init))
        self._case = Case(mesh, self._bcs, self._nu, self._settings)
        self._state = None

    def solve_state(self, theta11) -> EvaluationStatus:
        """Cold solve at theta (11 SST constants); the state is kept."""
        out = solve(self._case, np.asarray(theta11, float), self._settings.sst_variant, self._init)
        self._state = out.state
        return out.status

    def has_state(self) -> bool:
        return self._state is not None

    def n_cells(self) -> int:
        return self._mesh.n_cells()

    def n_obs(self) -> int:
        return self._obs.n_obs()

    def _observed(self, theta11, state):
        f = dict(state)
        f.update(_closure_fields(self._case, theta11, self._settings.sst_variant, state))
        f["nuT"] = np.maximum(f["nuT"], 0.1 * self._nu)
        pred = self._obs.evaluate(self._mesh, f, self._nu)
        return pred, self._obs.log_likelihood(self._mesh, f, self._nu, pred)

    def observe(self, theta11) -> List[float]:
        if self._state is None:
            raise RuntimeError("no state: call solve_state first")
        return self._observed(theta11, self._state)[0]

    def log_lik(self, theta11) -> float:
        if self._state is None:
            raise RuntimeError("no state: call solve_state first")
        return self._observed(theta11, self._state)[1]

    def eta_jacobian_warm_fd(self, theta, h_rel: float = 5e-4, h_floor: float = 1e-7, warm_max_iter: int = 0,
                             warm_tol: float = 0.0) -> TangentGradientResult:
        """Central differences of the observables and of the log-likelihood in
        all 11 constants, from 22 warm re-solves run as one batched launch."""
        out = TangentGradientResult(self.n_obs())
        if self._state is None:
            return out
        theta = np.asarray(theta, float)
        warm = self._settings.copy()
        if warm_max_iter > 0:
            warm.max_iterations = int(warm_max_iter)
        if warm_tol > 0.0:
            warm.convergence_tol = float(warm_tol)
        wcase = Case(self._mesh, self._bcs, self._nu, warm)
        wcase.set_observations(self._obs)
        steps, thetas = [], []
        for j in range(11):
            hr = min(h_rel, 1e-5) if j in (8, 9) else h_rel
            h = max(hr * abs(theta[j]), h_floor)
            steps.append(h)
            for sgn in (1.0, -1.0):
                tp = theta.copy()
                tp[j] += sgn * h
                thetas.append(tp)
        # observables and log-likelihoods are evaluated on the device: only
        # they leave it, not the 22 states
        outs = solve_batch([wcase] * 22, np.array(thetas), [self._settings.sst_variant] * 22,
                           [self._state] * 22, want_state=False)
        for o in outs:
            out.n_residual_evals += o.final_iter
        for j in range(11):
            op, om = outs[2 * j], outs[2 * j + 1]
            ok = not op.diverged and not om.diverged
            out.krylov_converged[j] = 1 if ok else 0
            if not ok:
                continue
            ep, lp = op.predictions, op.log_lik
            em, lm = om.predictions, om.log_lik
            for i in range(self.n_obs()):
                out.d_obs_d_theta[i][j] = (ep[i] - em[i]) / (2.0 * steps[j])
            out.log_lik_gradient[j] = (lp - lm) / (2.0 * steps[j])
        wcase.close()
        return out

    def _outside(self, *args, **kwargs):
        raise NotImplementedError("the tangent / adjoint ground-work of ParameterSensitivity is outside the "
                                  "rebuilt forward-model path")

    residual = d_residual_d_theta = d_obs_d_theta = eta_jacobian_tangent = eta_jacobian_tangent_coupled = _outside
