"""Host-side checks of the ForwardModel surface that need no GPU: the
injection target's shape check and symmetrisation (python/Bindings.cpp:488-505),
the invalid-parameter sentinel, and the default injection diagnostics."""
import numpy as np
import pytest

import cases
import rans_sst_py as rs


def _model():
    m, bcs, nu, init = cases.periodic_channel(8, 180.0)
    ps = rs.InferenceParameterSet.from_indices("c3", [8, 0, 1, 9, 2, 10])
    return m, ps, rs.ForwardModel(m, ps, rs.ObservationOperator(), bcs, nu, cases.channel_settings(10, 0.0))


def test_target_anisotropy_shape_and_symmetrisation():
    m, ps, fm = _model()
    n = m.n_cells()
    with pytest.raises(RuntimeError, match=r"\(n_cells, 3, 3\)"):
        fm.set_target_anisotropy(np.zeros((n, 3)))
    with pytest.raises(RuntimeError, match="nCells\\*6"):
        fm.set_target_anisotropy(np.zeros((n + 2, 3, 3)))
    assert not fm.has_target_anisotropy()
    b = np.zeros((n, 3, 3))
    b[:, 0, 1], b[:, 1, 0] = 0.1, 0.3          # asymmetric input: averaged
    b[:, 1, 2], b[:, 2, 1] = -0.2, 0.0
    b[:, 0, 0] = 0.05
    fm.set_target_anisotropy(b)
    assert fm.has_target_anisotropy()
    b6 = fm._b6.reshape(n, 6)
    assert np.allclose(b6[:, 0], 0.05) and np.allclose(b6[:, 3], 0.2) and np.allclose(b6[:, 5], -0.1)
    assert np.all(b6[:, 4] == 0.0)
    fm.clear_target_anisotropy()
    assert not fm.has_target_anisotropy()
    assert fm.injection_diagnostics() == {"active": False, "checked_iters": 0, "all_realizable": True,
                                          "max_violation": 0.0}


def test_out_of_bounds_theta_needs_no_solve():
    m, ps, fm = _model()
    theta = list(ps.pack(rs.SSTCoefficients()))
    theta[5] = 0.30                               # kappa below its 0.35 bound
    r = fm.evaluate(theta)
    assert r.status == rs.EvaluationStatus.InvalidParameters and r.log_lik == -1e30
    assert fm.penalized_log_likelihood(theta) == -1e30
