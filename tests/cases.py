"""Named test workloads shared by the golden generator and the tests.

Each case is (mesh, boundary conditions, nu, settings, initial state).  Meshes
are built by the product's factories; the golden generator stores the exact
mesh (MSH1 bytes) next to the reference results, and the tests rebuild the
mesh from those bytes so both sides see identical geometry on any machine.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "bayesian-turbulence-modeling_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

from rans_sst_py import FlowBoundaryConditions, Mesh, SolverSettings, Vec3  # noqa: E402
from rans_sst_py._types import COEFF_DEFAULTS  # noqa: E402

GOLDEN = os.path.join(HERE, "golden")


def ratio_for_first_cell(y1: float, n_half: int, h: float = 1.0) -> float:
    """Geometric growth ratio whose first cell of n_half cells over height h is y1."""
    lo, hi = 1.0 + 1e-12, 3.0
    for _ in range(200):
        r = 0.5 * (lo + hi)
        tot = y1 * (r ** n_half - 1.0) / (r - 1.0)
        if tot < h:
            lo = r
        else:
            hi = r
    return 0.5 * (lo + hi)


def injection_target(m) -> np.ndarray:
    """A realizable Reynolds-stress injection target for channel meshes,
    (n_cells*6,) xx yy zz xy xz yz: fixed normal anisotropies and a shear
    anisotropy 0.15 tanh(3 (y - 1)) that changes sign across the centreline
    with the mean shear (the sign of the Boussinesq b_xy = -nu_t S_xy / k)."""
    eta = m.cell_center[:, 1] - 1.0
    b = np.zeros((m.n_cells(), 6))
    b[:, 0], b[:, 1], b[:, 2] = 0.12, -0.08, -0.04
    b[:, 3] = 0.15 * np.tanh(3.0 * eta)
    return b.reshape(-1)


def channel_settings(max_iter: int, tol: float) -> SolverSettings:
    s = SolverSettings()
    s.verbose = False
    s.body_force = Vec3(1.0, 0.0, 0.0)
    s.max_iterations = max_iter
    s.convergence_tol = tol
    return s


def periodic_channel(ny: int, re_tau: float, nx: int = 4, ratio: float = None, y_plus: float = 0.4):
    """Streamwise-periodic channel at Re_tau (body force 1, nu = 1/Re_tau)."""
    if ratio is None:
        ratio = ratio_for_first_cell(y_plus / re_tau, ny // 2)
    m = Mesh.make_channel_periodic_geometric(nx, ny, 1.0, 1.0, ratio)
    m.compute_wall_distance()
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    init = dict(u=(20.0, 0.0, 0.0), p=0.0, k=1e-2, omega=10.0)
    return m, bcs, 1.0 / re_tau, init


def bfs_case(nxu=8, nxd=48, nyu=24, nyd=12, seed=7, nut_ratio=100.0):
    """Backward-facing step (h=1, H=3, Lu=4, Ld=30, Re_h=36000), cells permuted
    with numpy.random.default_rng(seed).permutation.  Inlet Tu = 1%; the inlet
    and initial omega use nu_t/nu = 100, the reference BFS driver's start-up
    ratio (python/case_library.py:127-129): with nu_t/nu = 10 the reference
    solver diverges during its laminar start-up iterations."""
    m = Mesh.make_backward_facing_step_2d(nxu, nxd, nyu, nyd, 4.0, 30.0, 1.0, 3.0, 36000.0, 1.0)
    if seed is not None:
        m = m.permuted(np.random.default_rng(seed).permutation(m.n_cells()))
    m.compute_wall_distance()
    nu = 1.0 / 36000.0
    k_in = 1.5 * 0.01 ** 2
    om_in = k_in / (nut_ratio * nu)
    bcs = FlowBoundaryConditions.bfs_defaults(m, 1.0, k_in, om_in)
    init = dict(u=(1.0, 0.0, 0.0), p=0.0, k=k_in, omega=om_in)
    return m, bcs, nu, init


def bfs_settings(max_iter: int, tol: float) -> SolverSettings:
    """python/bfs_reference.py:11-31 settings with the given cap/tolerance."""
    s = SolverSettings()
    s.verbose = False
    s.max_iterations = max_iter
    s.convergence_tol = tol
    s.divergence_limit = 1e8
    s.alpha_u, s.alpha_p, s.alpha_k, s.alpha_omega = 0.3, 0.2, 0.4, 0.4
    s.inner_iterations = 300
    s.inner_tolerance = 1e-4
    s.turb_start_iter = 30
    s.turb_update_interval = 2
    return s


def couette_case(nx=4, ny=32, re_tau=500.0, u_wall=None):
    """Streamwise-periodic plane Couette: bottom wall at rest, top wall moving."""
    ratio = ratio_for_first_cell(0.4 / re_tau, ny // 2)
    m = Mesh.make_channel_periodic_geometric(nx, ny, 1.0, 1.0, ratio)
    m.compute_wall_distance()
    if u_wall is None:
        u_wall = 2.0 * 20.0
    bcs = FlowBoundaryConditions.periodic_couette(m, u_wall)
    init = dict(u=(0.5 * u_wall, 0.0, 0.0), p=0.0, k=1e-2, omega=10.0)
    return m, bcs, 1.0 / re_tau, init


def couette_settings(max_iter, tol):
    s = SolverSettings()
    s.verbose = False
    s.max_iterations = max_iter
    s.convergence_tol = tol
    return s


def duct_case(nx=4, ny=16, nz=16, re_tau=150.0, ratio=1.25):
    m = Mesh.make_square_duct_periodic_3d(nx, ny, nz, 10.0, 2.0, ratio)
    m.compute_wall_distance()
    bcs = FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    init = dict(u=(15.0, 0.0, 0.0), p=0.0, k=1e-2, omega=10.0)
    return m, bcs, 1.0 / re_tau, init


def mesh_from_bytes(b: bytes) -> Mesh:
    import tempfile
    with tempfile.NamedTemporaryFile(suffix=".msh", delete=False) as fh:
        fh.write(b)
        path = fh.name
    try:
        m = Mesh.load_from_file(path)
    finally:
        os.unlink(path)
    return m


def mesh_to_bytes(m: Mesh) -> bytes:
    import tempfile
    with tempfile.NamedTemporaryFile(suffix=".msh", delete=False) as fh:
        path = fh.name
    try:
        m.save_binary(path)
        with open(path, "rb") as fh:
            return fh.read()
    finally:
        os.unlink(path)


def load_golden(name: str) -> dict:
    path = os.path.join(GOLDEN, name + ".npz")
    z = np.load(path, allow_pickle=False)
    return {k: z[k] for k in z.files}


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


_FOAM_BANNER = """/*--------------------------------*- C++ -*----------------------------------*\\
  =========                 |
  \\\\      /  F ield         | test fixture
   \\\\    /   O peration     |
    \\\\  /    A nd           |
     \\\\/     M anipulation  |
\\*---------------------------------------------------------------------------*/
FoamFile
{{
    version     2.0;
    format      ascii;
    class       {cls};
    location    "constant/polyMesh";
    {note}object      {obj};
}}
// * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * //

"""


def write_polymesh_block(path, nx, ny, nz, perturb=0.15, seed=3):
    """An OpenFOAM ASCII polyMesh of an nx x ny x nz hex block on [0,2]x[0,1]x
    [0,0.5] with interior nodes jittered by +-perturb of a cell size (seeded),
    so interior faces are warped: internal faces in OpenFOAM upper-triangular
    order, then patches inlet/outlet (patch), bottom/top (wall), front/back
    (empty)."""
    os.makedirs(path, exist_ok=True)
    rng = np.random.default_rng(seed)
    hx, hy, hz = 2.0 / nx, 1.0 / ny, 0.5 / nz
    nid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)  # noqa: E731
    cid = lambda i, j, k: i + nx * (j + ny * k)               # noqa: E731
    pts = np.zeros(((nx + 1) * (ny + 1) * (nz + 1), 3))
    for k in range(nz + 1):
        for j in range(ny + 1):
            for i in range(nx + 1):
                p = np.array([i * hx, j * hy, k * hz])
                if 0 < i < nx and 0 < j < ny and 0 < k < nz:
                    p += perturb * np.array([hx, hy, hz]) * rng.uniform(-1.0, 1.0, 3)
                pts[nid(i, j, k)] = p
    xf = lambda i, j, k: [nid(i, j, k), nid(i, j + 1, k), nid(i, j + 1, k + 1), nid(i, j, k + 1)]  # noqa: E731
    yf = lambda i, j, k: [nid(i, j, k), nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j, k)]  # noqa: E731
    zf = lambda i, j, k: [nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k)]  # noqa: E731
    faces, owner, neigh = [], [], []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                c = cid(i, j, k)
                if i + 1 < nx:
                    faces.append(xf(i + 1, j, k)); owner.append(c); neigh.append(cid(i + 1, j, k))
                if j + 1 < ny:
                    faces.append(yf(i, j + 1, k)); owner.append(c); neigh.append(cid(i, j + 1, k))
                if k + 1 < nz:
                    faces.append(zf(i, j, k + 1)); owner.append(c); neigh.append(cid(i, j, k + 1))
    patches = []

    def patch(name, ptype, cells_faces):
        start = len(faces)
        for c, f in cells_faces:
            faces.append(f); owner.append(c)
        patches.append((name, ptype, len(faces) - start, start))

    patch("inlet", "patch", [(cid(0, j, k), xf(0, j, k)[::-1]) for k in range(nz) for j in range(ny)])
    patch("outlet", "patch", [(cid(nx - 1, j, k), xf(nx, j, k)) for k in range(nz) for j in range(ny)])
    patch("bottom", "wall", [(cid(i, 0, k), yf(i, 0, k)[::-1]) for k in range(nz) for i in range(nx)])
    patch("top", "wall", [(cid(i, ny - 1, k), yf(i, ny, k)) for k in range(nz) for i in range(nx)])
    patch("front", "empty", [(cid(i, j, 0), zf(i, j, 0)[::-1]) for j in range(ny) for i in range(nx)])
    patch("back", "empty", [(cid(i, j, nz - 1), zf(i, j, nz)) for j in range(ny) for i in range(nx)])
    note = 'note        "nPoints:{} nCells:{} nFaces:{} nInternalFaces:{}";\n    '.format(
        len(pts), nx * ny * nz, len(faces), len(neigh))

    def write(name, cls, body, with_note=False):
        with open(os.path.join(path, name), "w") as fh:
            fh.write(_FOAM_BANNER.format(cls=cls, obj=name, note=note if with_note else ""))
            fh.write(body)
            fh.write("\n// ************************************************************************* //\n")

    write("points", "vectorField", "\n{}\n(\n{}\n)\n".format(
        len(pts), "\n".join("({!r} {!r} {!r})".format(*map(float, p)) for p in pts)))
    write("faces", "faceList", "\n{}\n(\n{}\n)\n".format(
        len(faces), "\n".join("4({} {} {} {})".format(*f) for f in faces)))
    write("owner", "labelList", "\n{}\n(\n{}\n)\n".format(len(owner), "\n".join(map(str, owner))), True)
    write("neighbour", "labelList", "\n{}\n(\n{}\n)\n".format(len(neigh), "\n".join(map(str, neigh))), True)
    body = "\n{}\n(\n".format(len(patches))
    for name, ptype, nf, start in patches:
        body += "    {}\n    {{\n        type            {};\n".format(name, ptype)
        if ptype == "wall":
            body += "        inGroups        List<word> 1(wall);\n"
        body += "        nFaces          {};\n        startFace       {};\n    }}\n".format(nf, start)
    body += ")\n"
    write("boundary", "polyBoundaryMesh", body)
    return path


def bfs_operator():
    """All six observable kinds on the backward-facing step (recirculating,
    so separation and reattachment crossings exist; the step face has none)."""
    from rans_sst_py import ObservationOperator, Vec3
    o = ObservationOperator()
    o.add_drag("bottom_wall_down", 0.01, 0.002, 1.0, 1.0)
    o.add_pressure_tap(Vec3(6.0, 0.5, 0.0), -0.05, 0.01, 1.0)
    o.add_pressure_tap(Vec3(2.0, 1.5, 0.0), 0.02, 0.01, 1.0, 0.001, 0.1, 1.2)
    o.add_velocity_profile(Vec3(3.0, 0.3, 0.0), 0, -0.1, 0.05)
    o.add_velocity_profile(Vec3(3.0, 0.3, 0.0), 1, 0.0, 0.05, 0.01)
    o.add_skin_friction("bottom_wall_down", Vec3(10.0, 0.0, 0.0), 0.002, 5e-4, 1.0)
    o.add_skin_friction("top_wall", Vec3(12.0, 3.0, 0.0), 0.003, 5e-4, 1.0)
    o.add_separation_point("bottom_wall_down", 0.5, 0.1)
    o.add_reattachment_length("bottom_wall_down", 6.0, 0.5)
    o.add_reattachment_length("step_face", 0.0, 0.5)
    return o


def channel_operator():
    """Channel outputs: skin friction on both walls, streamwise velocity at
    five wall distances, a pressure tap, the wall drag, and a separation
    point that does not exist (attached flow: the reference's default)."""
    from rans_sst_py import ObservationOperator, Vec3
    o = ObservationOperator()
    o.add_skin_friction("bottom_wall", Vec3(0.5, 0.0, 0.5), 0.0066, 0.001, 1.0)
    o.add_skin_friction("top_wall", Vec3(0.5, 2.0, 0.5), 0.0066, 0.001, 1.0)
    for y, u in ((0.001, 0.5), (0.01, 5.0), (0.1, 14.0), (0.5, 19.0), (1.0, 21.0)):
        o.add_velocity_profile(Vec3(0.5, y, 0.5), 0, u, 0.5)
    o.add_pressure_tap(Vec3(0.5, 1.0, 0.5), 0.0, 0.01, 20.0)
    o.add_drag("bottom_wall", 0.0, 0.001, 1.0, 20.0)
    o.add_separation_point("bottom_wall", 0.5, 0.1)
    return o
