"""Generate the golden vectors under tests/golden/ by running the UNMODIFIED
reference solver (compiled from its own sources by `make -C oracle ref`,
driven through oracle/ref_driver.cpp).  Run in a checkout where the
reference sources exist:

    make -C oracle ref
    python tests/golden/make_golden.py [case ...]
    python tests/golden/make_golden.py bfs_perm_1920+cont   # add the continuation run
    python tests/golden/make_golden.py bfs_perm_1920+stag   # add the stagnation run
    python tests/golden/make_golden.py bfs_perm_1920+startup   # add the 3000-iteration start-up

Each .npz holds the exact mesh (MSH1 bytes), the case inputs (nu, settings as
JSON, initial state) and the reference outputs.  Stagnation states are the
reference run for a fixed, large iteration count with the convergence test
disabled (tol 0): two FP64 implementations stopped at a 1e-8 scaled residual
can differ by ~1e-6, run to stagnation they agree to round-off.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import cases  # noqa: E402
from oracle import port  # noqa: E402
from oracle import refdriver as rd  # noqa: E402
from oracle.cabi import History  # noqa: E402

COEFF = np.array(cases.COEFF_DEFAULTS)
FIELDS = ("U", "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw", "Ub", "pb", "kb", "omegab")


def settings_json(s) -> np.ndarray:
    d = {k: (v if not hasattr(v, "x") else [v.x, v.y, v.z]) for k, v in s.__dict__.items()}
    return np.frombuffer(json.dumps(d, sort_keys=True).encode(), np.uint8)


def ref_solve(mesh_bytes, mesh, bcs, nu, s, init, coeffs=COEFF, variant=0, residual_capacity=0, b_target=None):
    path = "/tmp/_golden_mesh.msh"
    with open(path, "wb") as fh:
        fh.write(mesh_bytes)
    rm = rd.RefMesh.load(path)
    rm.wall_distance()
    bca, keep = port.bc_array(bcs)
    st = port.settings_struct(s)
    ini, _ = port.make_init(**init)
    t0 = time.time()
    arrays, hist, res = rm.solve(bca, nu, st, coeffs, variant, ini, mesh.n_cells(), mesh.n_boundary_faces(),
                                 residual_capacity, b_target=b_target)
    dt = time.time() - t0
    info = dict(final_iter=hist.final_iter, iterations_run=hist.iterations_run, converged=hist.converged,
                diverged=hist.diverged, seconds=dt)
    return arrays, info, res


def pack(prefix, arrays, info, out):
    for f in FIELDS:
        out[f"{prefix}_{f}"] = arrays[f]
    out[f"{prefix}_turb_established"] = np.array(arrays["turb_established"])
    for k, v in info.items():
        out[f"{prefix}_{k}"] = np.array(v)


def base_record(mesh, nu, s, init):
    mb = cases.mesh_to_bytes(mesh)
    return mb, {"mesh": np.frombuffer(mb, np.uint8), "wall_dist": mesh.wall_dist, "nu": np.array(nu),
                "settings": settings_json(s),
                "init": np.array([*init["u"], init["p"], init["k"], init["omega"]])}


def make_chan180():
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    s = cases.channel_settings(20000, 0.0)
    mb, out = base_record(m, nu, s, init)
    for n in (1, 5, 50):
        s.max_iterations, s.convergence_tol = n, 0.0
        a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
        pack(f"pin{n}", a, info, out)
    s.max_iterations, s.convergence_tol = 20000, 1e-8
    a, info, res = ref_solve(mb, m, bcs, nu, s, init, residual_capacity=20000)
    pack("conv", a, info, out)
    out["conv_residuals"] = res[:info["iterations_run"]]
    s.max_iterations, s.convergence_tol = 20000, 0.0
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
    pack("stag", a, info, out)
    return out


def make_c1():
    """The plane-channel workload: 4x128, geometric ratio 1.08 from each wall,
    Re_tau = 550 (nu = 1/550, body force 1), U0 = 20, k0 = 1e-2, omega0 = 10."""
    m, bcs, nu, init = cases.periodic_channel(128, 550.0, ratio=1.08)
    s = cases.channel_settings(60000, 1e-8)
    mb, out = base_record(m, nu, s, init)
    a, info, res = ref_solve(mb, m, bcs, nu, s, init, residual_capacity=60000)
    pack("conv", a, info, out)
    out["conv_residuals"] = res[:info["iterations_run"]:100]
    s.max_iterations, s.convergence_tol = 60000, 0.0
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
    pack("stag", a, info, out)
    return out


def make_bfs():
    m, bcs, nu, init = cases.bfs_case()
    s = cases.bfs_settings(1, 0.0)
    mb, out = base_record(m, nu, s, init)
    for n in (1, 5, 40):
        s.max_iterations = n
        a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
        pack(f"pin{n}", a, info, out)
    # converged state: the reference settings to the 1e-8 scaled residual
    s.max_iterations, s.convergence_tol = int(os.environ.get("BFS_CONV_ITERS", "150000")), 1e-8
    a, info, res = ref_solve(mb, m, bcs, nu, s, init, residual_capacity=s.max_iterations)
    pack("conv", a, info, out)
    out["conv_residuals"] = res[:info["iterations_run"]:100]
    return out


def add_bfs_continuation():
    """Extend bfs_perm_1920.npz (keeping its expensive converged run) with the
    reference continued for 200 outer iterations from its converged state
    (warm start, convergence test off): the comparator for the device
    engines started from the same state."""
    path = os.path.join(HERE, "bfs_perm_1920.npz")
    g = dict(np.load(path))
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    m.compute_wall_distance()
    nu = float(g["nu"])
    init = dict(u=tuple(g["init"][:3]), p=float(g["init"][3]), k=float(g["init"][4]), omega=float(g["init"][5]))
    from rans_sst_py import FlowBoundaryConditions
    bcs = FlowBoundaryConditions.bfs_defaults(m, 1.0, init["k"], init["omega"])
    s = cases.bfs_settings(200, 0.0)
    warm = {f: g[f"conv_{f}"] for f in FIELDS}
    warm["turb_established"] = int(g["conv_turb_established"])
    a, info, res = ref_solve(bytes(g["mesh"]), m, bcs, nu, s, dict(warm=warm), residual_capacity=200)
    pack("cont200", a, info, g)
    g["cont200_residuals"] = res[:info["iterations_run"]]
    return g


def _bfs_golden_inputs():
    path = os.path.join(HERE, "bfs_perm_1920.npz")
    g = dict(np.load(path))
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    m.compute_wall_distance()
    init = dict(u=tuple(g["init"][:3]), p=float(g["init"][3]), k=float(g["init"][4]), omega=float(g["init"][5]))
    from rans_sst_py import FlowBoundaryConditions
    bcs = FlowBoundaryConditions.bfs_defaults(m, 1.0, init["k"], init["omega"])
    return g, m, bcs, float(g["nu"]), init


def add_bfs_startup(iters=3000):
    """Extend bfs_perm_1920.npz with the reference's cold start run for
    `iters` outer iterations (convergence test off): its trajectory through
    the laminar start-up and the switch-on of the turbulence model, the part
    of the solve that is sensitive to the pressure solver's smoother."""
    g, m, bcs, nu, init = _bfs_golden_inputs()
    s = cases.bfs_settings(iters, 0.0)
    a, info, res = ref_solve(bytes(g["mesh"]), m, bcs, nu, s, init, residual_capacity=iters)
    pack(f"pin{iters}", a, info, g)
    g[f"pin{iters}_residuals"] = res[:info["iterations_run"]]
    return g


def add_bfs_stagnation(iters=40000):
    """Extend bfs_perm_1920.npz with the reference continued from its converged
    state for `iters` outer iterations with the convergence test off: its
    stagnation state, the comparator for a device solve continued the same
    way from its own converged state."""
    g, m, bcs, nu, init = _bfs_golden_inputs()
    s = cases.bfs_settings(iters, 0.0)
    warm = {f: g[f"conv_{f}"] for f in FIELDS}
    warm["turb_established"] = int(g["conv_turb_established"])
    a, info, _ = ref_solve(bytes(g["mesh"]), m, bcs, nu, s, dict(warm=warm))
    pack("stag", a, info, g)
    return g


def make_couette():
    m, bcs, nu, init = cases.couette_case()
    s = cases.couette_settings(30000, 1e-8)
    mb, out = base_record(m, nu, s, init)
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
    pack("conv", a, info, out)
    s.max_iterations, s.convergence_tol = 30000, 0.0
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
    pack("stag", a, info, out)
    return out


def make_duct():
    m, bcs, nu, init = cases.duct_case()
    s = cases.channel_settings(1, 0.0)
    mb, out = base_record(m, nu, s, init)
    for n in (1, 5):
        s.max_iterations = n
        a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
        pack(f"pin{n}", a, info, out)
    s.max_iterations, s.convergence_tol = int(os.environ.get("DUCT_STAG_ITERS", "15000")), 0.0
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
    pack("stag", a, info, out)
    return out


def make_units():
    """Known-answer vectors for the pieces: Green-Gauss gradient, SST fields and
    the four linear solvers on seeded random inputs (BFS mesh)."""
    rng = np.random.default_rng(1234)
    m, bcs, nu, init = cases.bfs_case(4, 12, 8, 4)
    mb, out = base_record(m, nu, cases.bfs_settings(1, 0.0), init)
    path = "/tmp/_golden_mesh.msh"
    with open(path, "wb") as fh:
        fh.write(mb)
    rm = rd.RefMesh.load(path)
    rm.wall_distance()
    nC, nB, nIF = m.n_cells(), m.n_boundary_faces(), m.n_internal_faces()
    phi, phib = rng.normal(size=nC), rng.normal(size=nB)
    out["gg_phi"], out["gg_phib"], out["gg_grad"] = phi, phib, rm.green_gauss(phi, phib)
    U, Ub = rng.normal(size=(nC, 3)) * [1, 0.3, 0], rng.normal(size=(nB, 3)) * [1, 0.3, 0]
    k, kb = rng.uniform(1e-5, 1e-2, nC), rng.uniform(0, 1e-2, nB)
    om, omb = rng.uniform(1, 1e4, nC), rng.uniform(1, 1e4, nB)
    for name, v in (("U", U), ("Ub", Ub), ("k", k), ("kb", kb), ("om", om), ("omb", omb)):
        out["sst_in_" + name] = v
    coeffs = COEFF * rng.uniform(0.8, 1.2, 11)
    out["sst_coeffs"] = coeffs
    for variant in (0, 1, 2):
        r = rm.sst_fields(coeffs, variant, nu, U, Ub, k, kb, om, omb)
        for key, v in r.items():
            out[f"sst{variant}_{key}"] = v
    own, nbr = m.owner[:nIF], m.neighbour[:nIF]
    # a diagonally dominant nonsymmetric and a symmetric (Laplacian-like) system
    up, lo = -rng.uniform(0.1, 1.0, nIF), -rng.uniform(0.1, 1.0, nIF)
    diag = np.zeros(nC)
    np.add.at(diag, own, -lo)
    np.add.at(diag, nbr, -up)
    diag += rng.uniform(0.05, 0.5, nC)
    src, x0 = rng.normal(size=nC), rng.normal(size=nC)
    sym = -rng.uniform(0.1, 1.0, nIF)
    sdiag = np.zeros(nC)
    np.add.at(sdiag, own, -sym)
    np.add.at(sdiag, nbr, -sym)
    sdiag[0] *= 2.0
    for name, v in (("diag", diag), ("upper", up), ("lower", lo), ("src", src), ("x0", x0),
                    ("sdiag", sdiag), ("sym", sym)):
        out["ls_" + name] = v
    out["ls_y"] = rd.matvec(own, nbr, diag, up, lo, x0)
    for kind in (0, 1, 2, 3):
        if kind in (0, 3):
            x, res = rd.linear_solve(kind, own, nbr, sdiag, sym, sym, src, np.zeros(nC), 200, 1e-6)
        else:
            x, res = rd.linear_solve(kind, own, nbr, diag, up, lo, src, x0, 200, 1e-6)
        out[f"ls{kind}_x"], out[f"ls{kind}_res"] = x, res
    return out


def make_chan180_inject():
    """Reynolds-stress injection (SIMPLESolver.cpp:205-315) on the Re_tau 180
    4x32 channel: cases.injection_target (a realizable, wall-normal varying
    shear anisotropy with the sign of the mean shear) at the default alphaInjection 0.3; 50 iterations from
    the cold start, the converged stop and the stagnation state."""
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    b6 = cases.injection_target(m)
    s = cases.channel_settings(50, 0.0)
    mb, out = base_record(m, nu, s, init)
    out["b_target"] = b6
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init, b_target=b6)
    pack("pin50", a, info, out)
    s.max_iterations, s.convergence_tol = 20000, 1e-8
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init, b_target=b6)
    pack("conv", a, info, out)
    s.max_iterations, s.convergence_tol = 20000, 0.0
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init, b_target=b6)
    pack("stag", a, info, out)
    return out


def make_chan180_wallfn():
    """Wall functions on (useWallFunctions: eddy viscosity at wall faces in the
    momentum flux, the blended omega wall value, SIMPLESolver.cpp:115, 894-903)
    on the Re_tau 180 4x32 channel: 50, 2000 and 20000 iterations (its
    stagnation) from the cold start."""
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    s = cases.channel_settings(50, 0.0)
    s.use_wall_functions = True
    mb, out = base_record(m, nu, s, init)
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
    pack("pin50", a, info, out)
    s.max_iterations = 2000
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
    pack("pin2000", a, info, out)
    s.max_iterations = 20000
    a, info, _ = ref_solve(mb, m, bcs, nu, s, init)
    pack("stag", a, info, out)
    return out


FOAM_BLOCKS = {"b432": (4, 3, 2, 0.15, 3), "b653": (6, 5, 3, 0.2, 11)}


def make_foam_blocks():
    """The reference's OpenFOAM polyMesh loader (Mesh::loadOpenFOAM,
    core/src/Mesh.cpp:50-265) on cases.write_polymesh_block fixtures: the
    loaded topology and geometry."""
    import tempfile
    out = {}
    keys = ("owner", "neighbour", "face_patch", "face_center", "face_normal", "face_area", "face_delta",
            "face_d", "face_weight", "cell_center", "cell_volume", "cell_face_offset", "cell_faces", "nodes")
    for tag, args in FOAM_BLOCKS.items():
        with tempfile.TemporaryDirectory() as d:
            path = cases.write_polymesh_block(os.path.join(d, "polyMesh"), *args)
            r = rd.RefMesh.load(path).dump()
        out[f"{tag}_args"] = np.array(args, dtype=np.float64)
        out[f"{tag}_n_internal"] = np.array(r["n_internal"])
        for k in keys:
            out[f"{tag}_{k}"] = r[k]
        out[f"{tag}_patch_names"] = np.frombuffer("\n".join(r["patch_names"]).encode(), np.uint8)
    return out


def make_observe():
    """The reference ObservationOperator (core/include/ObservationOperator.hpp:
    186-378) evaluated by the reference itself on reference states: the
    converged permuted backward-facing step (cases.bfs_operator: all six
    kinds) and the stagnated 4x128 Re_tau 550 channel (cases.channel_operator).
    Requires bfs_perm_1920.npz and c1_chan550_4x128.npz."""
    from rans_sst_py._lib import observable_structs
    out = {}
    for tag, name, prefix, op in (("bfs", "bfs_perm_1920", "conv", cases.bfs_operator()),
                                  ("chan", "c1_chan550_4x128", "stag", cases.channel_operator())):
        g = np.load(os.path.join(HERE, name + ".npz"))
        m = cases.mesh_from_bytes(bytes(g["mesh"]))
        path = "/tmp/_golden_mesh.msh"
        with open(path, "wb") as fh:
            fh.write(bytes(g["mesh"]))
        rm = rd.RefMesh.load(path)
        rm.wall_distance()
        arr, n = observable_structs(m, op)
        state = {f: g[f"{prefix}_{f}"] for f in ("U", "Ub", "p", "pb", "k", "kb", "omega", "omegab", "nuT")}
        pred, ll = rm.observe(arr, float(g["nu"]), state)
        out[f"{tag}_pred"] = np.array(pred)
        out[f"{tag}_loglik"] = np.array(ll)
        out[f"{tag}_source"] = np.frombuffer(f"{name}:{prefix}".encode(), np.uint8)
    return out


def make_outputs():
    """The reference's own wall diagnostics (python/wall_diagnostics.py:77-100,
    cf_along_wall, imported from the reference sources) on the stagnated 4x128
    Re_tau 550 channel, both walls, reference velocities 1 and 20."""
    ref_root = os.environ.get("BTM_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference")
    ref_py = os.path.join(ref_root, "python")
    sys.path.insert(0, ref_py)
    import wall_diagnostics as wd
    g = np.load(os.path.join(HERE, "c1_chan550_4x128.npz"))
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    st = {f: g[f"stag_{f}"] for f in ("U", "p", "k", "omega", "nuT")}
    out = {}
    for wall in ("bottom_wall", "top_wall"):
        for uref in (1.0, 20.0):
            r = wd.cf_along_wall(m, st, float(g["nu"]), wall, uref)
            for key in ("x", "y", "cf"):
                out[f"{wall}_{uref:g}_{key}"] = np.asarray(r[key])
            out[f"{wall}_{uref:g}_mean"] = np.array(r["mean"])
    return out


MAKERS = {"units": make_units, "foam_blocks": make_foam_blocks, "chan180_4x32": make_chan180, "bfs_perm_1920": make_bfs,
          "couette_4x32": make_couette, "duct_4x16x16": make_duct, "c1_chan550_4x128": make_c1,
          "chan180_inject_4x32": make_chan180_inject, "chan180_wallfn_4x32": make_chan180_wallfn,
          "observe": make_observe, "outputs": make_outputs}
# makers that extend an existing file instead of producing a new case
EXTENDERS = {"bfs_perm_1920+cont": add_bfs_continuation, "bfs_perm_1920+stag": add_bfs_stagnation,
             "bfs_perm_1920+startup": add_bfs_startup}


def main(names):
    if not rd.available():
        raise SystemExit("reference driver not built: make -C oracle ref")
    for name in names or list(MAKERS):
        t0 = time.time()
        if name in EXTENDERS:
            out = EXTENDERS[name]()
            name = name.split("+")[0]
        else:
            out = MAKERS[name]()
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB in {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
