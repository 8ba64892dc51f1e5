"""Observation operator on the device (btm_case_set_observations): the
predictions and the log-likelihood evaluated from the final state of a solve
are bit-identical to the host ObservationOperator (the mirror of
ObservationOperator.hpp:159-378) on the downloaded fields, in both engines,
in the served loop and on the cooperative grid."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import cases
from rans_sst_py import (Case, FlowBoundaryConditions, ObservationOperator, Server, SolverSettings, Vec3,
                         solve, solve_batch)

pytestmark = pytest.mark.gpu


def _bfs_operator():
    o = ObservationOperator()
    o.add_drag("bottom_wall_down", 0.01, 0.002, 1.0, 1.0)
    o.add_pressure_tap(Vec3(6.0, 0.5, 0.0), -0.05, 0.01, 1.0)
    o.add_velocity_profile(Vec3(3.0, 0.3, 0.0), 0, -0.1, 0.05)
    o.add_velocity_profile(Vec3(3.0, 0.3, 0.0), 1, 0.0, 0.05, 0.01)
    o.add_skin_friction("bottom_wall_down", Vec3(10.0, 0.0, 0.0), 0.002, 5e-4, 1.0)
    o.add_skin_friction("top_wall", Vec3(12.0, 3.0, 0.0), 0.003, 5e-4, 1.0)
    o.add_separation_point("bottom_wall_down", 0.5, 0.1)
    o.add_reattachment_length("bottom_wall_down", 6.0, 0.5)
    o.add_reattachment_length("step_face", 0.0, 0.5)
    return o


def _bfs_warm(precision, iters=30):
    g = cases.load_golden("bfs_perm_1920")
    if "conv_U" not in g or not int(g["conv_converged"]):
        pytest.skip("BFS golden has no converged state")
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    m.compute_wall_distance()
    d = json.loads(bytes(g["settings"]).decode())
    s = SolverSettings()
    for k, v in d.items():
        setattr(s, k, Vec3(*v) if k == "body_force" else v)
    s.max_iterations, s.convergence_tol, s.precision = iters, 0.0, precision
    a = g["init"]
    bcs = FlowBoundaryConditions.bfs_defaults(m, 1.0, float(a[4]), float(a[5]))
    warm = {f: np.array(g[f"conv_{f}"]) for f in ("U", "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw",
                                                   "Ub", "pb", "kb", "omegab")}
    warm["turb_established"] = int(g["conv_turb_established"])
    return m, bcs, float(g["nu"]), s, warm


def _host(op, m, state, nu):
    pred = op.evaluate(m, state, nu)
    return pred, op.log_likelihood(m, state, nu, pred)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bfs_observables_bit_identical_to_host(precision):
    """All six observable kinds on the permuted BFS (recirculating, so the
    reattachment crossing exists), 30 iterations continued from the
    reference's converged state."""
    m, bcs, nu, s, warm = _bfs_warm(precision)
    op = _bfs_operator()
    case = Case(m, bcs, nu, s)
    case.set_observations(op)
    out = solve(case, cases.COEFF_DEFAULTS, 0, warm)
    pred, ll = _host(op, m, out.state, nu)
    assert out.predictions == pred
    assert out.log_lik == ll
    faces = m.patches[m.patch_by_name("bottom_wall_down")][2]
    assert pred[7] < m.face_center[faces[-1], 0], pred      # the reattachment crossing was found


def test_state_free_batch_and_detach():
    """want_state=False returns the same predictions (nothing but them leaves
    the device); a detached operator evaluates nothing.  60 iterations: the
    BFS settings start the turbulence model (and with it theta's effect) at
    iteration 30."""
    m, bcs, nu, s, warm = _bfs_warm("fp64", 60)
    op = _bfs_operator()
    case = Case(m, bcs, nu, s)
    case.set_observations(op)
    th = np.array(cases.COEFF_DEFAULTS)
    th2 = th * 1.05
    full = solve_batch([case, case], [th, th2], None, [warm, warm])
    lean = solve_batch([case, case], [th, th2], None, [warm, warm], want_state=False)
    for a, b in zip(full, lean):
        assert b.state is None
        assert a.predictions == b.predictions and a.log_lik == b.log_lik
        assert a.predictions == _host(op, m, a.state, nu)[0]
    assert full[0].predictions != full[1].predictions
    case.set_observations(None)
    assert solve(case, th, 0, warm).predictions is None


def test_served_predictions_match_solo():
    """Served requests without state download carry the device predictions of
    the same solve run alone."""
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    s = cases.channel_settings(400, 0.0)
    op = ObservationOperator()
    op.add_skin_friction("bottom_wall", Vec3(0.5, 0.0, 0.5), 0.006, 0.001, 16.0)
    op.add_velocity_profile(Vec3(0.5, 1.0, 0.5), 0, 18.0, 1.0)
    op.add_velocity_profile(Vec3(0.5, 0.1, 0.5), 0, 9.0, 1.0)
    case = Case(m, bcs, nu, s)
    case.set_observations(op)
    rng = np.random.default_rng(5)
    thetas = [np.array(cases.COEFF_DEFAULTS) * (1.0 + 0.02 * rng.standard_normal(11)) for _ in range(6)]
    srv = Server(max_slots=8, hbm_budget_bytes=1 << 30)
    ids = {srv.submit(case, th, init=init, want_state=False): i for i, th in enumerate(thetas)}
    got = {}
    while len(got) < len(ids):
        for rid, out in srv.poll(timeout_ms=2000):
            got[ids[rid]] = out
    srv.close()
    for i, th in enumerate(thetas):
        solo = solve(case, th, 0, init)
        assert got[i].state is None
        assert got[i].predictions == solo.predictions and got[i].log_lik == solo.log_lik
        assert solo.predictions == _host(op, m, solo.state, nu)[0]


GRID_OBS_SCRIPT = """
import sys, json
sys.path[:0] = {paths!r}
import numpy as np
import cases
from rans_sst_py import Case, ObservationOperator, Vec3, solve
m, bcs, nu, init = cases.periodic_channel(32, 180.0)
op = ObservationOperator()
op.add_skin_friction("top_wall", Vec3(0.5, 2.0, 0.5), 0.006, 0.001, 16.0)
op.add_velocity_profile(Vec3(0.5, 0.7, 0.5), 0, 18.0, 1.0)
op.add_pressure_tap(Vec3(0.5, 1.0, 0.5), 0.0, 1.0, 16.0)
res = {{}}
for prec in ("fp64", "mixed"):
    s = cases.channel_settings(300, 0.0); s.precision = prec
    case = Case(m, bcs, nu, s)
    case.set_observations(op)
    out = solve(case, cases.COEFF_DEFAULTS, 0, init)
    pred = op.evaluate(m, out.state, nu)
    res[prec] = bool(out.predictions == pred and out.log_lik == op.log_likelihood(m, out.state, nu, pred))
print(json.dumps(res))
"""


def test_grid_mode_observables():
    """On the cooperative grid the leader reads the state other CTAs wrote
    (L1-bypassing loads): still bit-identical, both engines."""
    paths = [os.path.dirname(os.path.abspath(__file__)), cases.ROOT, cases.PKG]
    env = dict(os.environ, BTM_BLOCK_MAX_CELLS="64")
    r = subprocess.run([sys.executable, "-c", GRID_OBS_SCRIPT.format(paths=paths)], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert json.loads(r.stdout.strip().splitlines()[-1]) == {"fp64": True, "mixed": True}


STATE_FIELDS = ("U", "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw", "Ub", "pb", "kb", "omegab")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("tag,name,prefix,make", [("bfs", "bfs_perm_1920", "conv", cases.bfs_operator),
                                                  ("chan", "c1_chan550_4x128", "stag", cases.channel_operator)])
def test_device_operator_matches_reference(precision, tag, name, prefix, make):
    """The device evaluation (a zero-iteration warm solve, so the final state
    is the reference's state) against the predictions and log-likelihood the
    reference's own ObservationOperator computed (tests/golden/observe.npz):
    bit-identical."""
    gold = cases.load_golden("observe")
    g = cases.load_golden(name)
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    m.compute_wall_distance()
    a = g["init"]
    if tag == "bfs":
        bcs = FlowBoundaryConditions.bfs_defaults(m, 1.0, float(a[4]), float(a[5]))
        s = cases.bfs_settings(0, 0.0)
    else:
        bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
        s = cases.channel_settings(0, 0.0)
    s.precision = precision
    case = Case(m, bcs, float(g["nu"]), s)
    case.set_observations(make())
    warm = {f: np.array(g[f"{prefix}_{f}"]) for f in STATE_FIELDS}
    warm["turb_established"] = int(g[f"{prefix}_turb_established"])
    out = solve(case, cases.COEFF_DEFAULTS, 0, warm, want_state=False)
    assert out.iterations_run == 0
    assert np.array_equal(np.array(out.predictions), gold[f"{tag}_pred"]), (out.predictions, gold[f"{tag}_pred"])
    assert out.log_lik == float(gold[f"{tag}_loglik"])
