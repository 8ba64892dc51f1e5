"""The observation operator against the reference's own ObservationOperator
(core/include/ObservationOperator.hpp:186-378).  tests/golden/observe.npz
holds the predictions and log-likelihood the reference computed
(tests/golden/make_golden.py `observe`) on two reference states: the
converged permuted backward-facing step with all six observable kinds, and
the stagnated 4x128 Re_tau 550 channel.  The host operator must reproduce
them bit for bit; the device evaluation is checked in test_gpu_observe.py."""
import numpy as np
import pytest

import cases

FIELDS = ("U", "Ub", "p", "pb", "k", "kb", "omega", "omegab", "nuT")


def _state(name, prefix):
    g = cases.load_golden(name)
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    return m, {f: np.array(g[f"{prefix}_{f}"]) for f in FIELDS}, float(g["nu"])


@pytest.mark.parametrize("tag,name,prefix,make", [("bfs", "bfs_perm_1920", "conv", cases.bfs_operator),
                                                  ("chan", "c1_chan550_4x128", "stag", cases.channel_operator)])
def test_host_operator_matches_reference(tag, name, prefix, make):
    gold = cases.load_golden("observe")
    m, st, nu = _state(name, prefix)
    op = make()
    pred = op.evaluate(m, st, nu)
    ll = op.log_likelihood(m, st, nu, pred)
    assert np.array_equal(np.array(pred), gold[f"{tag}_pred"]), (pred, gold[f"{tag}_pred"])
    assert ll == float(gold[f"{tag}_loglik"])


def test_reference_outputs_are_physical():
    """The golden's outputs themselves: channel skin friction 2 u_tau^2 /
    U_ref^2 (body force 1, u_tau = 1), the step's reattachment downstream of
    the step and upstream of the outlet."""
    g = cases.load_golden("observe")
    assert abs(g["chan_pred"][0] - 2.0) < 1e-3 and abs(g["chan_pred"][1] - 2.0) < 1e-3
    assert 2.0 < g["bfs_pred"][8] < 30.0
