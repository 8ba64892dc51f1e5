"""Pin the CPU restatement (oracle/simple_oracle.c) to the reference itself.

The golden vectors were written by the unmodified reference solver
(tests/golden/make_golden.py).  The restatement follows the reference
operation order with contraction disabled, so on x86-64 (where the goldens
were made) every result must be bit-identical.  On another architecture only
the C library's tanh may round differently; the comparisons then allow a few
ulp and the multi-iteration pins 1e-12.
"""
import json
import platform

import numpy as np
import pytest

import cases
from rans_sst_py import FlowBoundaryConditions, SolverSettings, Vec3

SAME_PLATFORM = platform.machine() in ("x86_64", "AMD64")
FIELDS = ("U", "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw", "Ub", "pb", "kb", "omegab")


def settings_from(g):
    d = json.loads(bytes(g["settings"]).decode())
    s = SolverSettings()
    for k, v in d.items():
        setattr(s, k, Vec3(*v) if k == "body_force" else v)
    return s


def init_from(g):
    a = g["init"]
    return dict(u=tuple(a[:3]), p=float(a[3]), k=float(a[4]), omega=float(a[5]))


def mesh_from(g):
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    m.compute_wall_distance()
    assert np.array_equal(m.wall_dist, g["wall_dist"])
    return m


def assert_same(a, b, rtol):
    a, b = np.asarray(a), np.asarray(b)
    if SAME_PLATFORM and rtol is not None and rtol <= 1e-15:
        assert np.array_equal(a, b)
    else:
        scale = max(np.max(np.abs(b)), 1e-300)
        assert np.max(np.abs(a - b)) <= max(rtol, 1e-15) * scale


@pytest.fixture(scope="module")
def units():
    return cases.load_golden("units")


def test_green_gauss_pin(oracle, units):
    m = mesh_from(units)
    g = oracle.green_gauss(m, units["gg_phi"], units["gg_phib"])
    assert np.array_equal(g, units["gg_grad"])


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_sst_fields_pin(oracle, units, variant):
    m = mesh_from(units)
    r = oracle.sst_fields(m, units["sst_coeffs"], variant, float(units["nu"]), units["sst_in_U"],
                          units["sst_in_Ub"], units["sst_in_k"], units["sst_in_kb"], units["sst_in_om"],
                          units["sst_in_omb"])
    for key in ("nuT", "F1", "F2", "Pk", "CDkw", "Smag"):
        assert_same(r[key], units[f"sst{variant}_{key}"], 0.0 if SAME_PLATFORM else 4e-16)


def test_matvec_pin(oracle, units):
    m = mesh_from(units)
    nIF = m.n_internal_faces()
    y = oracle.matvec(m.owner[:nIF], m.neighbour[:nIF], units["ls_diag"], units["ls_upper"],
                      units["ls_lower"], units["ls_x0"])
    assert np.array_equal(y, units["ls_y"])


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_linear_solver_pin(oracle, units, kind):
    """PCG (0), BiCGSTAB (1), Gauss-Seidel (2), AMG-PCG (3): same iterates,
    same iteration count, same residuals as the reference solvers."""
    m = mesh_from(units)
    nIF, nC = m.n_internal_faces(), m.n_cells()
    if kind in (0, 3):
        x, res = oracle.linear_solve(kind, m.owner[:nIF], m.neighbour[:nIF], units["ls_sdiag"], units["ls_sym"],
                                     units["ls_sym"], units["ls_src"], np.zeros(nC), 200, 1e-6)
    else:
        x, res = oracle.linear_solve(kind, m.owner[:nIF], m.neighbour[:nIF], units["ls_diag"], units["ls_upper"],
                                     units["ls_lower"], units["ls_src"], units["ls_x0"], 200, 1e-6)
    assert np.array_equal(x, units[f"ls{kind}_x"])
    assert np.array_equal(res, units[f"ls{kind}_res"])


@pytest.fixture(scope="module")
def chan180():
    return cases.load_golden("chan180_4x32")


@pytest.mark.parametrize("n", [1, 5, 50])
def test_short_solve_pin(oracle, chan180, n):
    """N outer iterations of the full SIMPLE loop from a cold start."""
    g = chan180
    m = mesh_from(g)
    s = settings_from(g)
    s.max_iterations, s.convergence_tol = n, 0.0
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    st, h = oracle.solve(m, bcs, float(g["nu"]), s, cases.COEFF_DEFAULTS, 0, **init_from(g))
    for f in FIELDS:
        assert_same(st[f], g[f"pin{n}_{f}"], 0.0 if SAME_PLATFORM else 1e-12)
    assert h["iterations_run"] == int(g[f"pin{n}_iterations_run"])


def test_converged_solve_pin(oracle, chan180):
    """Cold solve to the 1e-8 scaled residual: same stopping iteration, same state."""
    g = chan180
    m = mesh_from(g)
    s = settings_from(g)
    s.max_iterations, s.convergence_tol = 20000, 1e-8
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    st, h = oracle.solve(m, bcs, float(g["nu"]), s, cases.COEFF_DEFAULTS, 0, **init_from(g))
    assert h["converged"] == 1
    if SAME_PLATFORM:
        assert h["final_iter"] == int(g["conv_final_iter"])
    for f in ("U", "p", "k", "omega", "nuT"):
        assert_same(st[f], g[f"conv_{f}"], 0.0 if SAME_PLATFORM else 1e-9)


def test_bfs_short_pin(oracle):
    g = cases.load_golden("bfs_perm_1920")
    m = mesh_from(g)
    s = settings_from(g)
    nu = float(g["nu"])
    ini = init_from(g)
    bcs = FlowBoundaryConditions.bfs_defaults(m, 1.0, ini["k"], ini["omega"])
    for n in (1, 5, 40):
        s.max_iterations, s.convergence_tol = n, 0.0
        st, h = oracle.solve(m, bcs, nu, s, cases.COEFF_DEFAULTS, 0, **ini)
        for f in FIELDS:
            assert_same(st[f], g[f"pin{n}_{f}"], 0.0 if SAME_PLATFORM else 1e-12)


def test_bfs_continuation_pin(oracle):
    """200 iterations warm-started from the reference's converged BFS state."""
    g = cases.load_golden("bfs_perm_1920")
    m = mesh_from(g)
    s = settings_from(g)
    s.max_iterations, s.convergence_tol = 200, 0.0
    ini = init_from(g)
    bcs = FlowBoundaryConditions.bfs_defaults(m, 1.0, ini["k"], ini["omega"])
    warm = {f: g[f"conv_{f}"] for f in FIELDS}
    warm["turb_established"] = int(g["conv_turb_established"])
    st, h = oracle.solve(m, bcs, float(g["nu"]), s, cases.COEFF_DEFAULTS, 0, warm=warm)
    for f in FIELDS:
        assert_same(st[f], g[f"cont200_{f}"], 0.0 if SAME_PLATFORM else 1e-12)


def test_duct_short_pin(oracle):
    g = cases.load_golden("duct_4x16x16")
    m = mesh_from(g)
    s = settings_from(g)
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    for n in (1, 5):
        s.max_iterations, s.convergence_tol = n, 0.0
        st, h = oracle.solve(m, bcs, float(g["nu"]), s, cases.COEFF_DEFAULTS, 0, **init_from(g))
        for f in FIELDS:
            assert_same(st[f], g[f"pin{n}_{f}"], 0.0 if SAME_PLATFORM else 1e-12)


@pytest.mark.parametrize("stage", ["pin50", "conv"])
def test_injection_pin(oracle, stage):
    """Reynolds-stress injection (SIMPLESolver.cpp:205-315) on the Re_tau 180
    channel: 50 iterations from the cold start, and the cold solve to the 1e-8
    scaled residual (same stopping iteration, same state)."""
    g = cases.load_golden("chan180_inject_4x32")
    m = mesh_from(g)
    s = settings_from(g)
    if stage == "pin50":
        s.max_iterations, s.convergence_tol = 50, 0.0
    else:
        s.max_iterations, s.convergence_tol = 20000, 1e-8
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    assert np.array_equal(cases.injection_target(m), g["b_target"])
    st, h = oracle.solve(m, bcs, float(g["nu"]), s, cases.COEFF_DEFAULTS, 0, **init_from(g),
                         b_target=g["b_target"])
    if stage == "conv":
        assert h["converged"] == 1
        if SAME_PLATFORM:
            assert h["final_iter"] == int(g["conv_final_iter"])
    for f in FIELDS:
        assert_same(st[f], g[f"{stage}_{f}"], 0.0 if SAME_PLATFORM else 1e-9)


@pytest.mark.parametrize("stage,n", [("pin50", 50), ("pin2000", 2000)])
def test_wall_function_pin(oracle, stage, n):
    """useWallFunctions on (eddy viscosity at wall faces in the momentum flux,
    the blended omega wall value; SIMPLESolver.cpp:115, 894-903)."""
    g = cases.load_golden("chan180_wallfn_4x32")
    m = mesh_from(g)
    s = settings_from(g)
    assert s.use_wall_functions
    s.max_iterations, s.convergence_tol = n, 0.0
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    st, h = oracle.solve(m, bcs, float(g["nu"]), s, cases.COEFF_DEFAULTS, 0, **init_from(g))
    assert h["iterations_run"] == int(g[f"{stage}_iterations_run"])
    for f in FIELDS:
        assert_same(st[f], g[f"{stage}_{f}"], 0.0 if SAME_PLATFORM else 1e-9)
