"""tests/python/test_periodic_mesh_binding.py:15-53 of the reference, the
solve half: a body-force-driven coupled solve on the periodic curved-channel
mesh through ForwardModel (the drop-in surface), on the device."""
import numpy as np
import pytest

import rans_sst_py as rs

pytestmark = pytest.mark.gpu


def test_periodic_curved_mesh_solves_with_body_force():
    nx, ny, Lx, y_top = 30, 20, 4.5, 3.0
    xn = np.linspace(0.0, Lx, nx + 1)
    yb = 0.5 * (1.0 + np.cos(2.0 * np.pi * xn / Lx))
    mesh = rs.Mesh.make_curved_channel_periodic_2d(xn, yb, y_top, ny, Re=2800.0, yPlusTarget=1.0)
    mesh.compute_wall_distance()
    k_in, om_in, nu = 1e-4, 10.0, 3.0e-4
    bcs = rs.FlowBoundaryConditions.channel_defaults(mesh, 1.0, k_in, om_in)
    s = rs.SolverSettings()
    s.max_iterations = 15000
    s.convergence_tol = 1.0e-4
    s.alpha_u, s.alpha_p = 0.4, 0.25
    s.verbose = False
    s.body_force = rs.Vec3(4.0e-3, 0.0, 0.0)
    obs = rs.ObservationOperator()
    obs.add_reattachment_length("bottom_wall", xr_obs=2.0, sigma=1.0)
    ps = rs.InferenceParameterSet.a1_betaStar()
    fm = rs.ForwardModel(mesh, ps, obs, bcs, nu, s, rs.Vec3(0.3, 0.0, 0.0), 0.0, k_in, om_in)
    r = fm.evaluate(list(ps.pack(rs.SSTCoefficients())))
    assert str(r.status).split(".")[-1] in ("Converged", "Unconverged")
    assert fm.has_last_fields()
    U = np.asarray(fm.last_fields()["U"]).reshape(-1, 3)
    vols = np.asarray(mesh.cell_volumes())
    assert np.all(np.isfinite(U))
    assert float(np.sum(U[:, 0] * vols) / np.sum(vols)) > 0.05
