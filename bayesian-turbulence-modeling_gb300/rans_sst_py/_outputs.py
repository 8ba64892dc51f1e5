"""Host-side outputs of a channel solve: the wall skin friction and the mean
profile in wall units, as the reference's calibration layer extracts them
(python/wall_diagnostics.py:77-100, python/UQ/datasets/channel_baseline.py:
130-175).  Pure numpy on a downloaded state; no device work."""
from __future__ import annotations

import numpy as np


def cf_along_wall(mesh, fields, nu: float, wall_patch: str, ref_vel: float) -> dict:
    """Skin-friction coefficient on every face of `wall_patch`: the molecular
    shear nu |U_t| / delta of the owner cell's tangential velocity over
    0.5 ref_vel^2 (wall_diagnostics.cf_along_wall)."""
    info = mesh.wall_patch_data(wall_patch)
    own = np.asarray(info["owner"], int)
    delta = np.maximum(np.asarray(info["delta"], float), 1e-30)
    normal = np.asarray(info["normal"], float)
    center = np.asarray(info["center"], float)
    U = np.asarray(fields["U"], float)
    q = 0.5 * ref_vel ** 2
    Up = U[own]
    un = np.sum(Up * normal, axis=1)
    ut = Up - un[:, None] * normal
    cf = nu * np.linalg.norm(ut, axis=1) / delta / q
    return {"x": center[:, 0], "y": center[:, 1], "cf": cf,
            "mean": float(np.mean(cf)) if cf.size else float("nan"),
            "max": float(np.max(cf)) if cf.size else float("nan")}


def channel_profile(mesh, fields, nu: float, half_height: float = 1.0, wall_patch: str = "bottom_wall",
                    ref_vel: float = 1.0, x_frac: float = 0.97, developed_frac: float = 0.85) -> dict:
    """The channel outputs in wall units (channel_baseline.py:130-175): u_tau
    from the skin friction averaged over the developed part of the wall
    (x > developed_frac * L_x; all of it on a streamwise-periodic channel),
    Re_tau, and the column of cells nearest x_frac * L_x from the wall to the
    centreline: y+, U+, k+, nu_t / nu, omega+."""
    cc = mesh.cell_centers()
    x, y = cc[:, 0], cc[:, 1]
    U = np.asarray(fields["U"])[:, 0]
    cf = cf_along_wall(mesh, fields, nu, wall_patch, ref_vel)
    lx = float(np.max(mesh.face_centers()[:, 0]) - np.min(mesh.face_centers()[:, 0]))
    x0 = float(np.min(mesh.face_centers()[:, 0]))
    dev = cf["x"] > x0 + developed_frac * lx
    if not np.any(dev):
        dev = np.ones_like(cf["cf"], bool)
    cf_dev = float(np.mean(cf["cf"][dev]))
    u_tau = ref_vel * np.sqrt(cf_dev / 2.0)
    xs = np.unique(x)
    x_col = xs[np.argmin(np.abs(xs - (x0 + x_frac * lx)))]
    col = np.abs(x - x_col) < 1e-9
    yb = y[col]
    keep = yb <= half_height + 1e-12
    order = np.argsort(yb[keep])
    sel = lambda a: np.asarray(a)[col][keep][order]  # noqa: E731
    return {"u_tau": u_tau, "re_tau": u_tau * half_height / nu, "cf": cf_dev,
            "yplus": yb[keep][order] * u_tau / nu, "U": sel(U) / u_tau,
            "k": sel(fields["k"]) / u_tau ** 2, "nu_t": sel(fields["nuT"]) / nu,
            "omega": sel(fields["omega"]) * nu / u_tau ** 2}
