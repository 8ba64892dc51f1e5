"""BTM_INIT_DEVICE: a warm start from the final state the previous solve left
on the device gives the same bits as a warm start from the downloaded state
(the host round trip of the reference's warm-start cache, without the copies)."""
import numpy as np
import pytest

import cases
from rans_sst_py import BtmError, Case, solve

pytestmark = pytest.mark.gpu


def test_device_warm_start_matches_host_warm_start():
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    case = Case(m, bcs, nu, cases.channel_settings(300, 0.0))
    th = np.array(cases.COEFF_DEFAULTS)
    th2 = th * 1.02
    first = solve(case, th, 0, init)
    host = solve(case, th2, 0, first.state)
    again = solve(case, th, 0, init)                 # the slot holds th's final state again
    for f in ("U", "p", "k", "omega", "nuT"):
        assert np.array_equal(again.state[f], first.state[f])
    dev = solve(case, th2, 0, "device")
    assert dev.iterations_run == host.iterations_run
    for f in ("U", "p", "k", "omega", "nuT", "F1", "F2", "Ub", "pb", "kb", "omegab"):
        assert np.array_equal(dev.state[f], host.state[f]), f
    fresh = Case(m, bcs, nu, cases.channel_settings(10, 0.0))
    with pytest.raises(BtmError):
        solve(fresh, th, 0, "device")
