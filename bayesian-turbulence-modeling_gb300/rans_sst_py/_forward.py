"""Forward model G(x, theta) on the GB300 engine.

``ForwardModel`` mirrors the reference class of the same name
(incompressible/include/ForwardModel.hpp:75-139,
incompressible/src/ForwardModel.cpp:29-122, bound at python/Bindings.cpp:468-519):
bounds check -> InvalidParameters, theta -> 11 SST coefficients, warm-start
cache (50 entries, Euclidean radius 0.5), one device solve, status
classification, observables and log-likelihood, the same sentinels
(-1e30 invalid, -1e6 diverged/unknown) and no exception out of evaluate().

``solve`` / ``solve_batch`` expose the device solve directly (cold or warm
start, full state out), the batched form running many theta/case instances
in one persistent launch.
"""
from __future__ import annotations

import ctypes as C
import math
import threading
from collections import deque
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import BtmHistory, BtmInit, Case, check, dptr, lib, new_state, state_struct
from ._types import (EvaluationResult, EvaluationStatus, InferenceParameterSet, SolverSettings,
                     Vec3, _vec)

STATUS_FROM_CODE = {0: EvaluationStatus.Converged, 1: EvaluationStatus.Unconverged,
                    2: EvaluationStatus.DivergenceDetected, 3: EvaluationStatus.InvalidParameters,
                    4: EvaluationStatus.Unknown}


class SolveOutput:
    """State and convergence record of one device solve."""

    def __init__(self, state: Optional[dict], hist: BtmHistory, residuals=None, predictions=None):
        self.state = state
        # observables of the case's observation operator, evaluated on the
        # device (None when the case has none attached)
        self.predictions = [float(v) for v in predictions] if predictions is not None else None
        self.log_lik = float(hist.log_lik) if predictions is not None else None
        self.status = STATUS_FROM_CODE.get(hist.status, EvaluationStatus.Unknown)
        self.converged = bool(hist.converged)
        self.diverged = bool(hist.diverged)
        self.final_iter = int(hist.final_iter)
        self.iterations_run = int(hist.iterations_run)
        self.inner_iterations = int(hist.inner_iterations)
        self.last_residual = list(hist.last_residual)
        self.phase_ms = list(hist.phase_ms)
        self.solve_ms = float(hist.solve_ms)
        self.finish_ms = float(hist.finish_ms)
        self.inner_split = list(hist.inner_split)
        self.polish_start = int(hist.polish_start)
        self.residuals = residuals


def _init_struct(init, keep):
    ini = BtmInit()
    if isinstance(init, str):
        if init != "device":
            raise ValueError("init must be a dict, a state or 'device'")
        ini.mode = 2    # BTM_INIT_DEVICE: continue from the state left on the device
        return ini
    if init is None:
        init = {}
    if isinstance(init, dict) and "U" in init:
        ini.mode = 1
        st = state_struct(init)
        keep.append(st)
        ini.warm = C.pointer(st)
    else:
        u = _vec(init.get("u", (1.0, 0.0, 0.0)))
        ini.mode = 0
        ini.u[0], ini.u[1], ini.u[2] = u.x, u.y, u.z
        ini.p = float(init.get("p", 0.0))
        ini.k = float(init.get("k", 1e-4))
        ini.omega = float(init.get("omega", 1.0))
    return ini


def solve_batch(cases: Sequence[Case], coeffs, variants=None, inits=None, want_state=True,
                history_capacity: int = 0, observe: bool = True) -> List[SolveOutput]:
    """Run len(cases) independent solves in one device launch.

    coeffs: (n, 11) SST constants; inits: per instance a dict with either
    {"u", "p", "k", "omega"} (cold uniform start) or a full state dict (warm),
    or "device": continue from the final state the previous solve left on the
    device (the k-th instance of a case resumes the k-th instance's state).
    observe: evaluate the observation operator attached to a case
    (Case.set_observations) on the device; with want_state=False only the
    predictions and the log-likelihood leave the device.
    """
    n = len(cases)
    coeffs = np.ascontiguousarray(np.asarray(coeffs, np.float64).reshape(n, 11))
    var = np.ascontiguousarray(np.zeros(n, np.int32) if variants is None else np.asarray(variants, np.int32))
    keep = []
    ini_arr = (BtmInit * n)()
    for i in range(n):
        ini_arr[i] = _init_struct(None if inits is None else inits[i], keep)
    states = [new_state(c.n_cells, c.n_bnd) if want_state else None for c in cases]
    st_arr = (_lib.BtmState * n)()
    if want_state:
        for i in range(n):
            st_arr[i] = state_struct(states[i])
    hist = (BtmHistory * n)()
    res_bufs = [None] * n
    if history_capacity:
        for i in range(n):
            res_bufs[i] = np.zeros((history_capacity, 6))
            hist[i].residual_capacity = history_capacity
            hist[i].residuals = dptr(res_bufs[i])
    preds = [None] * n
    if observe:
        for i in range(n):
            if cases[i].n_obs > 0:
                preds[i] = np.zeros(cases[i].n_obs)
                hist[i].predictions = dptr(preds[i])
    handles = (C.c_void_p * n)(*[c.h.value for c in cases])
    check(lib().btm_solve_batch(n, handles, dptr(coeffs), var.ctypes.data_as(C.POINTER(C.c_int32)),
                                ini_arr, st_arr if want_state else None, hist))
    outs = []
    for i in range(n):
        if want_state:
            states[i]["turb_established"] = int(st_arr[i].turb_established)
        r = None
        if res_bufs[i] is not None:
            r = res_bufs[i][:min(history_capacity, hist[i].iterations_run)]
        outs.append(SolveOutput(states[i], hist[i], r, preds[i]))
    return outs


def solve(case: Case, coeffs, variant: int = 0, init=None, want_state=True, history_capacity=0,
          observe: bool = True) -> SolveOutput:
    return solve_batch([case], [coeffs], [variant], [init], want_state, history_capacity, observe)[0]


class _WarmStartCache:
    """WarmStartCache (ForwardModel.hpp:18-72): nearest theta within a
    Euclidean radius, copied under the lock; FIFO eviction at maxSize."""

    def __init__(self, max_size=50, threshold=0.5):
        self.max_size, self.threshold = max_size, threshold
        self._q = deque()
        self._lock = threading.Lock()

    @staticmethod
    def _dist(a, b):
        s = 0.0
        for i in range(min(len(a), len(b))):
            d = a[i] - b[i]
            s += d * d
        return math.sqrt(s)

    def find_nearest(self, theta):
        with self._lock:
            best, best_d = None, self.threshold
            for th, st in self._q:
                d = self._dist(theta, th)
                if d < best_d:
                    best_d, best = d, st
            if best is None:
                return None
            return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in best.items()}

    def store(self, theta, state):
        with self._lock:
            self._q.append((list(theta), {k: (v.copy() if isinstance(v, np.ndarray) else v)
                                          for k, v in state.items()}))
            while len(self._q) > self.max_size:
                self._q.popleft()

    def size(self):
        with self._lock:
            return len(self._q)

    def clear(self):
        with self._lock:
            self._q.clear()


_NO_INJECTION = {"active": False, "checked_iters": 0, "all_realizable": True, "max_violation": 0.0}


class ForwardModel:
    """Drop-in for rans_sst_py.ForwardModel (python/Bindings.cpp:468-519)."""

    def __init__(self, mesh, param_set: InferenceParameterSet, obs_op, bcs, nu: float,
                 settings: Optional[SolverSettings] = None, u_init=Vec3(1, 0, 0), p_init: float = 0.0,
                 k_init: float = 1e-4, omega_init: float = 1.0):
        import copy
        self._mesh = mesh                    # kept by reference, as the reference does
        self._param_set = param_set
        self._obs = copy.deepcopy(obs_op)    # copied by value (ForwardModel.hpp:125-129)
        self._bcs = copy.deepcopy(bcs)
        self._nu = float(nu)
        self._settings = (settings or SolverSettings()).copy()
        u = _vec(u_init)
        self._init = {"u": (u.x, u.y, u.z), "p": float(p_init), "k": float(k_init),
                      "omega": float(omega_init)}
        self._case: Optional[Case] = None
        self._cache = _WarmStartCache(50, 0.5)
        self._last: Optional[dict] = None
        self._last_solve: Optional[SolveOutput] = None
        self._b6: Optional[np.ndarray] = None
        self._last_inj = _NO_INJECTION.copy()

    def _get_case(self) -> Case:
        if self._case is None:
            self._case = Case(self._mesh, self._bcs, self._nu, self._settings)
            if self._obs.n_obs() > 0:
                self._case.set_observations(self._obs)
            if self._b6 is not None:
                self._case.set_target_anisotropy(self._b6)
        return self._case

    def evaluate(self, theta) -> EvaluationResult:
        theta = [float(t) for t in theta]
        if not self._param_set.in_bounds(theta):
            return EvaluationResult(EvaluationStatus.InvalidParameters, -1e30, [], 0)
        try:
            coeffs = self._param_set.unpack(theta).to_vector()
            case = self._get_case()
            # injected solves neither read nor fill the warm-start cache
            # (ForwardModel.cpp:50-57, 83-85)
            injected = self._b6 is not None
            warm = None if injected else self._cache.find_nearest(theta)
            out = solve(case, coeffs, int(self._settings.sst_variant), warm if warm is not None else self._init)
            self._last_solve = out
            if injected:
                _, real, viol = case.injection_realizability()
                self._last_inj = {"active": True, "checked_iters": out.iterations_run, "all_realizable": real,
                                  "max_violation": viol}
            else:
                self._last_inj = _NO_INJECTION.copy()
            if out.status == EvaluationStatus.Unknown:
                raise RuntimeError("device solve abandoned")
            if out.diverged:
                self._last = None
                return EvaluationResult(EvaluationStatus.DivergenceDetected, -1e6, [], out.final_iter)
            status = EvaluationStatus.Converged if out.converged else EvaluationStatus.Unconverged
            if out.converged and not injected:
                self._cache.store(theta, out.state)
            self._last = out.state
            # observables and log-likelihood come from the device evaluation
            # at the end of the solve (ObservationOperator.hpp:186-378)
            if out.predictions is not None:
                pred, ll = out.predictions, out.log_lik
            else:
                pred, ll = [], 0.0
            return EvaluationResult(status, ll, pred, out.final_iter)
        except Exception as e:  # nothing escapes evaluate (ForwardModel.cpp:99-104)
            if self._settings.verbose:
                print("ForwardModel exception:", e)
            return EvaluationResult(EvaluationStatus.Unknown, -1e6, [], 0)

    def penalized_log_likelihood(self, theta) -> float:
        res = self.evaluate(theta)
        if res.status in (EvaluationStatus.Converged, EvaluationStatus.Unconverged):
            return res.log_lik
        if res.status in (EvaluationStatus.DivergenceDetected, EvaluationStatus.Unknown):
            return -1e6
        return -1e30

    def param_set(self) -> InferenceParameterSet:
        return self._param_set

    def has_last_fields(self) -> bool:
        return self._last is not None

    def last_fields(self) -> Dict[str, np.ndarray]:
        if self._last is None:
            raise RuntimeError("No fields available — call evaluate() first")
        s = self._last
        return {"U": s["U"].copy(), "p": s["p"].copy(), "k": s["k"].copy(), "omega": s["omega"].copy(),
                "nuT": s["nuT"].copy(), "F1": s["F1"].copy(), "F2": s["F2"].copy(), "Pk": s["Pk"].copy()}

    def last_state(self) -> Optional[dict]:
        """Full state of the last retained solve (cell and boundary arrays)."""
        return self._last

    def cache_size(self) -> int:
        return self._cache.size()

    def clear_cache(self) -> None:
        self._cache.clear()

    # ---- a-posteriori Reynolds-stress injection (python/Bindings.cpp:485-518,
    # ForwardModel.hpp:110-118): the per-cell target is applied on the device
    # by every later evaluate() until cleared
    def set_target_anisotropy(self, b_target):
        b = np.asarray(b_target, np.float64)
        if b.ndim != 3 or b.shape[1] != 3 or b.shape[2] != 3:
            raise RuntimeError("set_target_anisotropy: expected (n_cells, 3, 3)")
        b6 = np.empty((b.shape[0], 6))
        b6[:, 0], b6[:, 1], b6[:, 2] = b[:, 0, 0], b[:, 1, 1], b[:, 2, 2]
        b6[:, 3] = 0.5 * (b[:, 0, 1] + b[:, 1, 0])
        b6[:, 4] = 0.5 * (b[:, 0, 2] + b[:, 2, 0])
        b6[:, 5] = 0.5 * (b[:, 1, 2] + b[:, 2, 1])
        if b6.size != 6 * self._mesh.n_cells():
            raise RuntimeError("setTargetAnisotropy: expected nCells*6 values")
        self._b6 = b6.reshape(-1)
        if self._case is not None:
            self._case.set_target_anisotropy(self._b6)

    def clear_target_anisotropy(self):
        self._b6 = None
        if self._case is not None:
            self._case.set_target_anisotropy(None)

    def has_target_anisotropy(self) -> bool:
        return self._b6 is not None

    def injection_diagnostics(self):
        """InjectionDiagnostics of the last evaluate (SIMPLESolver.hpp:83-88)."""
        return dict(self._last_inj)
