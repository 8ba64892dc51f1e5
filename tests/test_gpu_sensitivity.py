"""Warm-FD Jacobian (ParameterSensitivity.eta_jacobian_warm_fd) as one batched
launch, against the same central differences computed with the oracle
(warm re-solves, closure recomputation and the nu_t floor as
incompressible/src/ParameterSensitivity.cpp:691-745 does)."""
import numpy as np
import pytest

import cases
from rans_sst_py import ObservationOperator, ParameterSensitivity, Vec3

pytestmark = pytest.mark.gpu


def test_warm_fd_matches_oracle(oracle):
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    s = cases.channel_settings(3000, 1e-8)
    obs = ObservationOperator()
    obs.add_velocity_profile(Vec3(0.5, 0.5, 0.0), 0, 15.0, 0.5)
    obs.add_velocity_profile(Vec3(0.5, 0.05, 0.0), 0, 10.0, 0.5)
    obs.add_skin_friction("bottom_wall", Vec3(0.5, 0.0, 0.0), 0.005, 5e-4, 15.0)
    ps = ParameterSensitivity(m, obs, bcs, nu, s, Vec3(*init["u"]), init["p"], init["k"], init["omega"])
    theta = np.array(cases.COEFF_DEFAULTS)
    ps.solve_state(theta)
    assert ps.has_state()
    res = ps.eta_jacobian_warm_fd(theta, warm_max_iter=40, warm_tol=0.0)
    assert all(res.krylov_converged)

    # the same on the CPU restatement
    base, _ = oracle.solve(m, bcs, nu, s, theta, 0, **init)
    sw = s.copy()
    sw.max_iterations, sw.convergence_tol = 40, 0.0
    J = np.zeros((obs.n_obs(), 11))
    g = np.zeros(11)
    for j in range(11):
        hr = min(5e-4, 1e-5) if j in (8, 9) else 5e-4
        h = max(hr * abs(theta[j]), 1e-7)
        vals = []
        for sgn in (1.0, -1.0):
            tp = theta.copy()
            tp[j] += sgn * h
            st, _ = oracle.solve(m, bcs, nu, sw, tp, 0, warm=base)
            cl = oracle.sst_fields(m, tp, 0, nu, st["U"], st["Ub"], st["k"], st["kb"], st["omega"], st["omegab"])
            f = dict(st)
            f.update({k: cl[k] for k in ("nuT", "F1", "F2", "Pk", "CDkw")})
            f["nuT"] = np.maximum(f["nuT"], 0.1 * nu)
            pred = obs.evaluate(m, f, nu)
            vals.append((np.array(pred), obs.log_likelihood(m, f, nu, pred)))
        J[:, j] = (vals[0][0] - vals[1][0]) / (2 * h)
        g[j] = (vals[0][1] - vals[1][1]) / (2 * h)
    Jd = np.array(res.d_obs_d_theta)
    scale = np.maximum(np.abs(J).max(axis=1, keepdims=True), 1e-12)
    assert np.max(np.abs(Jd - J) / scale) <= 1e-5
    assert np.max(np.abs(np.array(res.log_lik_gradient) - g)) <= 1e-5 * max(np.max(np.abs(g)), 1e-12)
