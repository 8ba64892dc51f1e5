"""Known-answer checks of the reference's own test suite, restated against the
oracle (the CPU restatement of the solver) and the host-side package:

  * tests/cpp/test_infra_fixes.cpp:45-93, 112-167 - one in-place Gauss-Seidel
    sweep, the parameter-set size guard, warm-start cache copies, and the
    Rhie-Chow switch on a bounded channel leaving the bulk flow unchanged;
  * tests/cpp/test_periodic_channel.cpp:48-178 - cosine-bump periodic mesh
    geometry, a body-force-driven flat periodic channel (streamwise
    invariance, global momentum balance) and a bump channel staying finite;
  * tests/cpp/test_sst_production_2003.cpp:51-123 - the omega-production
    limiter algebra;
  * tests/cpp/test_couette_bc.cpp, tests/cpp/test_bfs_lemoin_bc.cpp - moving
    wall, symmetry top and per-face inlet profiles;
  * tests/cpp/test_mesh_bfs.cpp:31-131 - step-mesh counts and patch order;
  * tests/cpp/test_nut_floor_release.cpp:52-112 - the start-up nu_t floor and
    the molecular skin friction;
  * tests/cpp/test_convergence_accounting.cpp:41-95 - carried turbulence norms;
  * tests/cpp/test_transpose_stress.cpp:40-137 - manufactured transpose-stress
    sources;
  * tests/python/test_periodic_mesh_binding.py:15-27 - the periodic factory
    surface (the solve half runs on the GPU in test_gpu_reference_binding.py).
"""
import math

import numpy as np
import pytest

import cases
from rans_sst_py import FlowBoundaryConditions, InferenceParameterSet, Mesh, SolverSettings, Vec3
from rans_sst_py._forward import _WarmStartCache


def test_gauss_seidel_one_sweep(oracle):
    """A true in-place ascending sweep: 0.5, 0.25, 0.625 (Jacobi would give
    0.5, 0, 0.5)."""
    x, _ = oracle.linear_solve(2, [0, 1], [1, 2], [2.0, 2.0, 2.0], [-1.0, -1.0], [-1.0, -1.0], [1.0, 0.0, 1.0],
                               [0.0, 0.0, 0.0], 1, 1e-30)
    assert abs(x[0] - 0.5) < 1e-15 and abs(x[1] - 0.25) < 1e-15 and abs(x[2] - 0.625) < 1e-15


def test_parameter_set_size_guard():
    ps = InferenceParameterSet.a1_betaStar()
    assert ps.in_bounds([0.31, 0.09])
    assert not ps.in_bounds([0.31])
    assert not ps.in_bounds([0.31, 0.09, 0.5])
    assert not ps.in_bounds([])
    assert InferenceParameterSet.live10().n_active() == 10


def test_warm_start_cache_copy_survives_eviction():
    cache = _WarmStartCache(max_size=1, threshold=10.0)
    cache.store([0.3, 0.09], {"p": np.full(12, 3.5)})
    hit = cache.find_nearest([0.31, 0.09])
    assert hit is not None
    cache.store([0.9, 0.19], {"p": np.full(12, -7.0)})   # evicts the source entry
    assert abs(hit["p"][0] - 3.5) < 1e-15


def _cosine_mesh(nx, ny, Lx, y_top, bump, Re=0.0):
    xn = np.array([Lx * i / nx for i in range(nx + 1)])
    yb = 0.5 * bump * (1.0 + np.cos(2.0 * math.pi * xn / Lx))
    return Mesh.make_curved_channel_periodic_2d(list(xn), list(yb), y_top, ny, Re, 1.0)


def test_cosine_bump_geometry():
    nx, ny, Lx, y_top, bump = 24, 10, 4.0, 3.0, 1.0
    m = _cosine_mesh(nx, ny, Lx, y_top, bump)
    assert m.n_cells() == nx * ny
    vol = m.cell_volumes()
    assert np.all(vol > 0.0)
    exact = 0.0
    for i in range(nx):
        x0, x1 = Lx * i / nx, Lx * (i + 1) / nx
        g0 = y_top - 0.5 * bump * (1.0 + math.cos(2.0 * math.pi * x0 / Lx))
        g1 = y_top - 0.5 * bump * (1.0 + math.cos(2.0 * math.pi * x1 / Lx))
        exact += 0.5 * (g0 + g1) * (x1 - x0)
    assert abs(vol.sum() - exact) < 1e-10 * exact
    assert np.all(np.abs(np.linalg.norm(m.face_normal, axis=1) - 1.0) < 1e-12)
    own, nbr = m.owner[:m.n_internal], m.neighbour[:m.n_internal]
    wrap = (own % nx == nx - 1) & (nbr % nx == 0) & (own // nx == nbr // nx)
    assert wrap.sum() == ny
    assert np.all(m.face_delta[:m.n_internal][wrap] < 2.0 * Lx / nx)


def _channel_settings(max_iter, tol, alpha_u, alpha_p, fb):
    s = SolverSettings()
    s.verbose = False
    s.max_iterations, s.convergence_tol = max_iter, tol
    s.alpha_u, s.alpha_p = alpha_u, alpha_p
    s.body_force = Vec3(fb, 0.0, 0.0)
    return s


FLAT = dict(nx=24, ny=28, Lx=3.0, H=1.0, nu=2.0e-4, fb=5.0e-3)


def _flat_inputs():
    nx, Lx = FLAT["nx"], FLAT["Lx"]
    xn = [Lx * i / nx for i in range(nx + 1)]
    m = Mesh.make_curved_channel_periodic_2d(xn, [0.0] * (nx + 1), FLAT["H"], FLAT["ny"], 2500.0, 1.0)
    m.compute_wall_distance()
    return m, FlowBoundaryConditions.channel_defaults(m, 1.0, 1e-4, 10.0)


def _flat_solve(oracle, max_iter):
    m, bcs = _flat_inputs()
    s = _channel_settings(max_iter, 1e-4, 0.5, 0.3, FLAT["fb"])
    st, h = oracle.solve(m, bcs, FLAT["nu"], s, cases.COEFF_DEFAULTS, 0, u=(0.3, 0.0, 0.0), p=0.0, k=1e-4,
                         omega=10.0)
    return m, st, h


@pytest.fixture(scope="module")
def flat_channel(oracle):
    return _flat_solve(oracle, 12000)


def test_flat_periodic_channel_balance(flat_channel):
    """Body-force-driven SST channel: converged, streamwise invariant to 1e-6
    of the bulk velocity, and the discrete wall shear balances the drive
    within 5 %."""
    m, st, h = flat_channel
    nx, ny, nu, fb = FLAT["nx"], FLAT["ny"], FLAT["nu"], FLAT["fb"]
    assert not h["diverged"] and h["converged"]
    U = st["U"]
    vol = m.cell_volumes()
    u_bulk = float((U[:, 0] * vol).sum() / vol.sum())
    assert u_bulk > 0.1
    cols = np.arange(ny) * nx
    assert np.max(np.abs(U[cols, 0] - U[cols + nx // 2, 0])) < 1e-6 * u_bulk
    drive = fb * vol.sum()
    shear = 0.0
    for p in range(m.n_patches()):
        for f in m.patches[p][2]:
            shear += nu * U[m.owner[f], 0] / m.face_delta[f] * m.face_area[f]
    assert abs(shear - drive) / drive < 0.05


def test_cosine_bump_channel_stays_finite(oracle):
    m = _cosine_mesh(36, 24, 4.5, 3.0, 1.0)
    m.compute_wall_distance()
    bcs = FlowBoundaryConditions.channel_defaults(m, 1.0, 1e-4, 10.0)
    s = _channel_settings(15000, 1e-4, 0.4, 0.25, 4.0e-3)
    st, h = oracle.solve(m, bcs, 3.0e-4, s, cases.COEFF_DEFAULTS, 0, u=(0.3, 0.0, 0.0), p=0.0, k=1e-4,
                         omega=10.0)
    assert not h["diverged"]
    assert np.all(np.isfinite(st["U"][:, 0])) and np.all(np.isfinite(st["p"]))
    u_max = np.max(np.abs(st["U"][:, 0]))
    assert 0.05 < u_max < 100.0


def test_bounded_channel_rhie_chow_switch(oracle):
    """An outlet channel converges with and without the Rhie-Chow dissipation
    forced on, and the switch leaves the bulk velocity within 1 %."""
    m = Mesh.make_channel_2d(16, 12, 4.0, 1.0, 5000.0, 1.0)
    m.compute_wall_distance()
    bcs = FlowBoundaryConditions.channel_defaults(m, 1.0, 1e-4, 10.0)
    vol = m.cell_volumes()
    ub = {}
    for flag in (False, True):
        s = _channel_settings(20000, 1e-3, 0.5, 0.3, 0.0)
        s.rhie_chow_all_meshes = flag
        st, h = oracle.solve(m, bcs, 2.0e-4, s, cases.COEFF_DEFAULTS, 0, u=(1.0, 0.0, 0.0), p=0.0, k=1e-4,
                             omega=10.0)
        assert not h["diverged"] and h["converged"], flag
        ub[flag] = float((st["U"][:, 0] * vol).sum() / vol.sum())
    assert abs(ub[True] - ub[False]) < 0.01 * abs(ub[False])


# ---- tests/cpp/test_sst_production_2003.cpp:51-123 (SST point algebra) ------
def test_omega_production_limiter(oracle):
    P = lambda *a: oracle.sst_point("production_omega", *a)    # noqa: E731
    Pk = lambda *a: oracle.sst_point("production", *a)         # noqa: E731
    b_star = 0.09

    def close(a, b, rtol):
        return abs(a - b) <= rtol * max(max(abs(a), abs(b)), 1e-300)

    assert close(P(0.01, 1.0, 1.0, 100.0), 1.0, 1e-14)                  # limiter inactive: S^2
    lim = 10.0 * b_star * 1.0 * 1.0 / 1.0
    assert close(P(1.0, 100.0, 1.0, 1.0), lim, 1e-14)                   # active: 10 b* k w / nuT
    assert P(1.0, 100.0, 1.0, 1.0) < 1e-3 * 100.0 ** 2
    for nut in (1e-12, 1e-6, 1e-2, 0.5, 3.0):                           # never above S^2
        for S in (0.0, 0.3, 3.0, 300.0):
            for k in (1e-8, 1e-2, 1.0, 50.0):
                for w in (1e-3, 1.0, 1e4):
                    assert P(nut, S, k, w) <= S * S + 1e-14
    assert close(P(0.0, 2.0, 0.5, 200.0), 4.0, 1e-14)                   # nuT -> 0 selects S^2
    for nut, S, k, w in ((0.01, 1.0, 1.0, 100.0), (1.0, 100.0, 1.0, 1.0), (0.2, 5.0, 2.0, 30.0)):
        assert close(P(nut, S, k, w), Pk(nut, S, k, w) / nut, 1e-12)    # = production / nuT
    rho, mu_t, S, k, w = 1.7, 0.4, 40.0, 3.0, 8.0
    assert close(min(S * S, 10.0 * b_star * rho * k * w / mu_t), P(mu_t / rho, S, k, w), 1e-12)


# ---- tests/cpp/test_couette_bc.cpp:42-90 (moving-wall velocity BC) ----------
def test_couette_moving_wall_bc(oracle):
    from rans_sst_py import BCType
    m = Mesh.make_channel_2d(8, 16, 2.0, 2.0)
    m.compute_wall_distance()
    bc = FlowBoundaryConditions.couette_defaults(m, 2.0, 1e-3, 100.0)
    names = m.patch_names()
    top, bottom, inlet = names.index("top"), names.index("bottom"), names.index("inlet")
    assert bc.velocityBC[top].type == BCType.WallMoving
    assert abs(bc.velocityBC[top].vecValue.x - 2.0) < 1e-12
    assert abs(bc.velocityBC[top].vecValue.y) < 1e-12 and abs(bc.velocityBC[top].vecValue.z) < 1e-12
    assert bc.velocityBC[bottom].type == BCType.WallNoSlip
    assert bc.velocityBC[inlet].type == BCType.Neumann
    assert bc.kBC[top].type == BCType.WallKOmega and bc.omegaBC[top].type == BCType.WallKOmega
    st = oracle.apply_bcs(m, bc, 1e-3, np.zeros((m.n_cells(), 3)))
    nIF = m.n_internal
    for p, want in ((top, 2.0), (bottom, 0.0)):
        faces = m.patches[p][2]
        assert faces.size > 0
        assert np.all(np.abs(st["Ub"][faces - nIF, 0] - want) < 1e-12)


# ---- tests/cpp/test_bfs_lemoin_bc.cpp:45-112 (symmetry top, inlet profiles) --
def test_bfs_symmetry_top_and_inlet_profiles(oracle):
    from rans_sst_py import BCType
    m = Mesh.make_backward_facing_step_2d(8, 12, 10, 8, 4.0, 10.0, 1.0, 6.0)
    m.set_patch_type("top_wall", "symmetry")
    m.compute_wall_distance()
    p_top = m.patch_by_name("top_wall")
    assert m.patch_types()[p_top] == "symmetry"
    top_faces = m.patches[p_top][2]
    assert m.wall_dist[m.owner[top_faces[top_faces.size // 2]]] > 1.0     # the top is no wall
    bc = FlowBoundaryConditions.bfs_defaults(m, 1.0, 1e-3, 10.0)
    assert bc.velocityBC[p_top].type == BCType.Symmetry
    assert bc.kBC[p_top].type == BCType.Neumann and bc.omegaBC[p_top].type == BCType.Neumann
    assert bc.velocityBC[m.patch_by_name("bottom_wall_down")].type == BCType.WallNoSlip
    nIF = m.n_internal
    U = np.tile([0.7, 0.3, 0.0], (m.n_cells(), 1))
    st = oracle.apply_bcs(m, bc, 1e-4, U)
    b0 = top_faces[0] - nIF
    assert abs(st["Ub"][b0, 1]) < 1e-14 and abs(st["Ub"][b0, 0] - 0.7) < 1e-14
    inlet = m.patches[m.patch_by_name("inlet")][2]
    nf = inlet.size
    j = np.arange(nf)
    bc.set_velocity_profile(m, "inlet", np.stack([0.1 * j, 0 * j, 0 * j], axis=1).astype(float))
    bc.set_k_profile(m, "inlet", 1e-4 * (j + 1))
    bc.set_omega_profile(m, "inlet", 2.0 * (j + 1))
    st = oracle.apply_bcs(m, bc, 1e-4, U, k=np.full(m.n_cells(), 9.0), omega=np.full(m.n_cells(), 9.0))
    bi = inlet - nIF
    assert np.all(np.abs(st["Ub"][bi, 0] - 0.1 * j) < 1e-14)
    assert np.all(np.abs(st["kb"][bi] - 1e-4 * (j + 1)) < 1e-18)
    assert np.all(np.abs(st["omegab"][bi] - 2.0 * (j + 1)) < 1e-12)


# ---- tests/cpp/test_mesh_bfs.cpp:31-131 (counts and patch order) ------------
@pytest.mark.parametrize("args", [(6, 12, 8, 6, 6.0, 20.0, 1.0, 3.0, 37600.0, 1.0),
                                  (20, 40, 20, 15, 6.0, 20.0, 1.0, 3.0, 37600.0, 1.0)])
def test_bfs_mesh_counts_and_patches(args):
    nxu, nxd, nyu, nyd = args[:4]
    m = Mesh.make_backward_facing_step_2d(*args)
    nxt = nxu + nxd
    cells = nxt * nyu + nxd * nyd
    internal = nxt * (nyu - 1) + nxd * (nyd - 1) + nxd + (nxt - 1) * nyu + (nxd - 1) * nyd
    boundary = nxt + nxu + nyd + nxd + nyu + (nyu + nyd)
    assert m.n_cells() == cells and m.n_internal_faces() == internal
    assert m.n_faces() == internal + boundary
    assert m.patch_names() == ["top_wall", "bottom_wall_up", "step_face", "bottom_wall_down", "inlet", "outlet"]
    assert all(m.patches[p][2].size > 0 for p in range(m.n_patches()))
    m.compute_wall_distance()
    assert m.wall_dist.size == cells and np.all(np.isfinite(m.wall_dist)) and np.all(m.wall_dist >= 0.0)
    assert np.all(m.cell_volumes() > 0.0) and np.all(m.face_area > 0.0)
    assert np.all((m.owner >= 0) & (m.owner < cells))
    assert np.all((m.neighbour[:internal] >= 0) & (m.neighbour[:internal] < cells))
    assert np.all(m.neighbour[internal:] < 0)
    assert np.all(m.face_patch[internal:] >= 0)


def test_bfs_mesh_default_stretching():
    m = Mesh.make_backward_facing_step_2d(8, 16, 8, 6, 6.0, 20.0, 1.0, 3.0)
    assert m.n_cells() == (8 + 16) * 8 + 16 * 6


# ---- tests/cpp/test_nut_floor_release.cpp:52-112 (startup nu_t floor) -------
def _min_wall_nut(st):
    nx, ny = FLAT["nx"], FLAT["ny"]
    nut = st["nuT"]
    return min(nut[:nx].min(), nut[(ny - 1) * nx:ny * nx].min())


def test_nut_floor_binds_in_the_startup_window(oracle):
    m, st, h = _flat_solve(oracle, 200)      # before turbStart + nuTFloorIters
    assert _min_wall_nut(st) >= 0.1 * FLAT["nu"] * (1.0 - 1e-12)


def test_nut_floor_released_and_cf_molecular(flat_channel):
    from rans_sst_py import ObservationOperator
    m, st, h = flat_channel
    nu = FLAT["nu"]
    assert h["converged"] and not h["diverged"]
    assert _min_wall_nut(st) < 0.02 * nu
    obs = ObservationOperator()
    obs.add_skin_friction("bottom_wall", Vec3(1.5, 0.0, 0.0), 0.0, 1.0, 1.0)
    cf0 = obs.evaluate(m, st, nu)[0]
    assert cf0 > 0.0
    scaled = dict(st)
    scaled["nuT"] = np.full_like(st["nuT"], 5.0 * nu)
    assert obs.evaluate(m, scaled, nu)[0] == cf0


# ---- tests/cpp/test_convergence_accounting.cpp:41-95 (carried norms) --------
def test_turbulence_norms_carried_between_updates(oracle):
    m, bcs = _flat_inputs()
    s = _channel_settings(12000, 1e-4, 0.5, 0.3, FLAT["fb"])
    s.turb_start_iter, s.turb_update_interval = 30, 3
    st, h = oracle.solve(m, bcs, FLAT["nu"], s, cases.COEFF_DEFAULTS, 0, u=(0.3, 0.0, 0.0), p=0.0, k=1e-4,
                         omega=10.0, residual_capacity=12000)
    assert h["converged"]
    r = h["residuals"]
    carried = 0
    for i in range(30, r.shape[0]):
        assert r[i, 4] > 0.0 and r[i, 5] > 0.0
        if (i - 30) % 3 != 0:
            assert r[i, 4] == r[i - 1, 4] and r[i, 5] == r[i - 1, 5]
            carried += 1
    assert carried > 10
    assert r[-1, 4] < 1e-4 and r[-1, 5] < 1e-4


# ---- tests/cpp/test_transpose_stress.cpp:40-137 (manufactured fields) --------
def _manufactured(m, u_fn, c_fn):
    cc, fc = m.cell_center, m.face_center[m.n_internal:]
    U = np.array([u_fn(x, y) for x, y in cc[:, :2]])
    Ub = np.array([u_fn(x, y) for x, y in fc[:, :2]])
    coeff = np.array([c_fn(x, y) for x, y in cc[:, :2]])
    return coeff, U, Ub


def test_transpose_stress_manufactured(oracle):
    nx, ny = 12, 14
    m = Mesh.make_channel_2d(nx, ny, 2.0, 1.0)
    vol = m.cell_volumes()
    idx = np.arange(m.n_cells())
    interior = (idx % nx >= 2) & (idx % nx < nx - 2) & (idx // nx >= 2) & (idx // nx < ny - 2)
    # exactness: coeff = c0, U = (a x^2, 0, 0) -> src_x / V = 2 a c0
    a, c0 = 0.8, 0.35
    coeff, U, Ub = _manufactured(m, lambda x, y: (a * x * x, 0.0, 0.0), lambda x, y: c0)
    sx = oracle.transpose_stress(m, coeff, U, Ub, 0) / vol
    assert np.all(np.abs(sx[interior] - 2.0 * a * c0) < 1e-11)
    # discrimination: coeff = b y, U = (g y, d x, 0): src_x / V = b d (not b g),
    # exact in the wall rows too because the coefficient is zero at the wall
    b, g, d = 0.6, 1.3, 0.4
    coeff, U, Ub = _manufactured(m, lambda x, y: (g * y, d * x, 0.0), lambda x, y: b * y)
    sx = oracle.transpose_stress(m, coeff, U, Ub, 0) / vol
    sy = oracle.transpose_stress(m, coeff, U, Ub, 1) / vol
    wall_row = np.arange(2, nx - 2)
    assert np.all(np.abs(sx[wall_row] - b * d) < 1e-11)
    assert np.all(np.abs(sx[interior] - b * d) < 1e-11)
    assert np.all(np.abs(sx[interior] - b * g) > 0.1 * abs(b * (g - d)))
    assert np.all(np.abs(sy[interior]) < 1e-11)
    # parallel shear: the source vanishes identically
    coeff, U, Ub = _manufactured(m, lambda x, y: (math.tanh(4.0 * (y - 0.5)), 0.0, 0.0),
                                 lambda x, y: 0.02 + 0.05 * y * (1.0 - y))
    for comp in (0, 1):
        assert np.all(np.abs(oracle.transpose_stress(m, coeff, U, Ub, comp)) < 1e-14)


# ---- tests/python/test_periodic_mesh_binding.py:15-27 (factory surface) ------
def test_periodic_curved_mesh_binding_surface():
    nx, ny, Lx, y_top = 30, 20, 4.5, 3.0
    xn = np.linspace(0.0, Lx, nx + 1)
    yb = 0.5 * (1.0 + np.cos(2.0 * np.pi * xn / Lx))
    m = Mesh.make_curved_channel_periodic_2d(xn, yb, y_top, ny, Re=2800.0, yPlusTarget=1.0)
    m.compute_wall_distance()
    assert set(m.patch_names()) == {"bottom_wall", "top_wall"}
    assert set(m.patch_types()) == {"wall"}
    assert m.n_cells() == nx * ny
