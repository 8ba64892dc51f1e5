"""Mixed-precision engine (precision = "mixed"): FP32 assembly, closure,
gradients, Krylov and AMG work around an FP64 flow state, FP64 equation
defects and an FP64-refined pressure correction.

The error bar is 1e-6 relative L2 against the FP64 reference solution (the
reference's converged and stagnated fields stored in tests/golden), for U, k,
omega and nu_t; pressure is compared against the dynamic pressure scale
(periodic domains fix p only up to a near-constant level).
"""
import json

import numpy as np
import pytest

import cases
from rans_sst_py import FlowBoundaryConditions, SolverSettings, Vec3, Case, solve, solve_batch
from rans_sst_py._lib import BtmError

pytestmark = pytest.mark.gpu

COEFF = cases.COEFF_DEFAULTS
TOL_FIELDS = 1e-6


def settings_from(g, tol, cap):
    d = json.loads(bytes(g["settings"]).decode())
    s = SolverSettings()
    for k, v in d.items():
        setattr(s, k, Vec3(*v) if k == "body_force" else v)
    s.max_iterations, s.convergence_tol = cap, tol
    s.precision = "mixed"
    return s


def init_from(g):
    a = g["init"]
    return dict(u=tuple(a[:3]), p=float(a[3]), k=float(a[4]), omega=float(a[5]))


def mesh_from(g):
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    m.compute_wall_distance()
    return m


def errors(state, g, pre):
    out = {f: cases.rel_l2(state[f], g[f"{pre}_{f}"]) for f in ("U", "k", "omega", "nuT")}
    U = g[f"{pre}_U"]
    q = 0.5 * np.max(np.sum(U * U, axis=1))
    out["p"] = float(np.linalg.norm(state["p"] - g[f"{pre}_p"]) / (q * np.sqrt(len(U))))
    return out


def _check(errs, tol=TOL_FIELDS):
    for f, e in errs.items():
        assert e <= tol, (f, e, errs)


@pytest.mark.parametrize("name", ["chan180_4x32", "couette_4x32"])
def test_mixed_converged_matches_fp64_reference(name):
    """Cold start to the 1e-8 scaled residual in mixed precision; the converged
    fields agree with the reference's stagnated FP64 solution within 1e-6."""
    g = cases.load_golden(name)
    m = mesh_from(g)
    bcs = (FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0) if name.startswith("chan")
           else cases.couette_case(4, 32)[1])
    case = Case(m, bcs, float(g["nu"]), settings_from(g, 1e-8, 4 * int(g["conv_iterations_run"])))
    out = solve(case, COEFF, 0, init_from(g))
    assert out.converged
    _check(errors(out.state, g, "stag"))


def test_mixed_c1_stagnation():
    """The benchmarked mesh (4x128, ratio 1.08, Re_tau 550) in mixed precision,
    run to the reference's stagnation iteration count: the fixed point agrees
    with the reference's stagnated FP64 fields within 1e-6."""
    g = cases.load_golden("c1_chan550_4x128")
    m = mesh_from(g)
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    case = Case(m, bcs, float(g["nu"]), settings_from(g, 0.0, int(g["stag_iterations_run"])))
    out = solve(case, COEFF, 0, init_from(g))
    assert out.iterations_run == int(g["stag_iterations_run"])
    _check(errors(out.state, g, "stag"))


def test_mixed_duct3d_stagnation():
    """3-D duct (z-momentum active), fixed iteration count as the golden."""
    g = cases.load_golden("duct_4x16x16")
    m = mesh_from(g)
    case = Case(m, FlowBoundaryConditions.channel_defaults(m, 0, 0, 0), float(g["nu"]),
                settings_from(g, 0.0, int(g["stag_iterations_run"])))
    out = solve(case, COEFF, 0, init_from(g))
    _check(errors(out.state, g, "stag"))


def test_mixed_batch_matches_solo_bitwise():
    """A mixed instance gives bit-identical results alone and inside a batch
    with FP64 and mixed instances of other meshes."""
    m1, b1, nu1, i1 = cases.periodic_channel(32, 180.0)
    m2, b2, nu2, i2 = cases.couette_case(4, 16)
    s1 = cases.channel_settings(300, 0.0)
    s1.precision = "mixed"
    s2 = cases.couette_settings(300, 0.0)
    c1 = Case(m1, b1, nu1, s1)
    c2 = Case(m2, b2, nu2, s2)
    th = np.array(COEFF)
    th2 = th.copy()
    th2[9] *= 1.1
    solo = solve(c1, th2, 0, i1)
    batch = solve_batch([c2, c1, c1, c2], [th, th2, th, th2], None, [i2, i1, i1, i2])
    for f in ("U", "p", "k", "omega", "nuT"):
        assert np.array_equal(solo.state[f], batch[1].state[f]), f


def test_mixed_warm_start_matches_fp64_warm_start():
    """Warm start from the converged state of a nearby theta (the warm-start
    cache use): the mixed engine reaches the same outcome and fields as the
    FP64 engine started from the same state."""
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    th = np.array(COEFF)
    th2 = th.copy()
    th2[9] *= 1.02
    outs = {}
    for prec in ("fp64", "mixed"):
        s = cases.channel_settings(20000, 1e-8)
        s.precision = prec
        case = Case(m, bcs, nu, s)
        first = solve(case, th, 0, init)
        assert first.converged
        outs[prec] = solve(case, th2, 0, first.state)
    assert outs["mixed"].status == outs["fp64"].status
    for f in ("U", "k", "omega", "nuT"):
        assert cases.rel_l2(outs["mixed"].state[f], outs["fp64"].state[f]) <= TOL_FIELDS, f


GRID_SCRIPT = """
import sys, json
sys.path[:0] = {paths!r}
import cases
from rans_sst_py import FlowBoundaryConditions, Case, solve
from rans_sst_py._lib import lib
g = cases.load_golden("chan180_4x32")
m = cases.mesh_from_bytes(bytes(g["mesh"])); m.compute_wall_distance()
a = g["init"]
ini = dict(u=tuple(a[:3]), p=float(a[3]), k=float(a[4]), omega=float(a[5]))
res = {{}}
for name, it, tol in (("conv", 20000, 1e-8), ("stag", int(g["stag_iterations_run"]), 0.0)):
    if name == "stag" and {precision!r} != "fp64":
        continue
    s = cases.channel_settings(it, tol); s.precision = {precision!r}
    case = Case(m, FlowBoundaryConditions.channel_defaults(m, 0, 0, 0), float(g["nu"]), s)
    out = solve(case, cases.COEFF_DEFAULTS, 0, ini)
    res[name] = dict(converged=out.converged, iterations=out.iterations_run,
                     err={{f: cases.rel_l2(out.state[f], g["stag_" + f]) for f in ("U", "k", "omega", "nuT")}})
print(json.dumps(res))
"""


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_grid_mode_converges_to_reference(precision):
    """Meshes above the one-CTA size run over a cooperative grid, with a dense
    coarsest AMG level of up to 1024 rows solved by the whole grid.  Forced
    onto the grid path (BTM_BLOCK_MAX_CELLS below the mesh size, in a child
    process: the limit is read once per process), the Re_tau = 180 channel
    converges to the reference's stagnated fields within 1e-6, and the FP64
    engine run to the reference's stagnation count matches them within 1e-8."""
    import json
    import os
    import subprocess
    import sys
    paths = [os.path.dirname(os.path.abspath(__file__)), cases.ROOT, cases.PKG]
    env = dict(os.environ, BTM_BLOCK_MAX_CELLS="64")
    r = subprocess.run([sys.executable, "-c", GRID_SCRIPT.format(paths=paths, precision=precision)], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["conv"]["converged"]
    _check(res["conv"]["err"])
    if precision == "fp64":
        for f, e in res["stag"]["err"].items():
            assert e <= 1e-8, (f, e)


def test_anderson_converges_to_reference_fixed_point_sooner():
    """Anderson acceleration of the mixed engine's outer iteration (the
    default anderson_depth 8) changes the path, not the fixed point: on the
    benchmarked 4x128 Re_tau 550 channel it converges to within 1e-7 of the
    reference's stagnated FP64 fields (60000 iterations) in less than half the
    outer iterations of the plain mixed iteration (anderson_depth 0), which
    stops about 1e-6 from them."""
    g = cases.load_golden("c1_chan550_4x128")
    m = mesh_from(g)
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    outs = {}
    for depth in (0, 8):
        s = settings_from(g, 1e-8, 60000)
        s.anderson_depth = depth
        outs[depth] = solve(Case(m, bcs, float(g["nu"]), s), COEFF, 0, init_from(g))
        assert outs[depth].converged, depth
    assert outs[8].iterations_run < 0.5 * outs[0].iterations_run, (outs[8].iterations_run, outs[0].iterations_run)
    U = g["stag_U"]
    q = 0.5 * np.max(np.sum(U * U, axis=1))
    for depth, tol in ((8, 1e-7), (0, 1e-5)):
        st = outs[depth].state
        for f in ("U", "k", "omega", "nuT"):
            assert cases.rel_l2(st[f], g[f"stag_{f}"]) <= tol, (depth, f)
        dp = (st["p"] - st["p"].mean()) - (g["stag_p"] - g["stag_p"].mean())
        assert np.linalg.norm(dp) / (q * np.sqrt(len(U))) <= tol, depth
