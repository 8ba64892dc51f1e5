"""Channel outputs (rans_sst_py.cf_along_wall, channel_profile): the skin
friction matches the reference's own wall diagnostics bit for bit
(tests/golden/outputs.npz, made by python/wall_diagnostics.py:77-100 of the
reference on its stagnated 4x128 Re_tau 550 state), and the wall-unit
profile (channel_baseline.py:130-175) is consistent with it."""
import numpy as np
import pytest

import cases
from rans_sst_py import cf_along_wall, channel_profile


def _c1():
    g = cases.load_golden("c1_chan550_4x128")
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    return m, {f: np.array(g[f"stag_{f}"]) for f in ("U", "p", "k", "omega", "nuT")}, float(g["nu"])


@pytest.mark.parametrize("wall", ["bottom_wall", "top_wall"])
@pytest.mark.parametrize("uref", [1.0, 20.0])
def test_cf_along_wall_matches_reference(wall, uref):
    gold = cases.load_golden("outputs")
    m, st, nu = _c1()
    r = cf_along_wall(m, st, nu, wall, uref)
    for key in ("x", "y", "cf"):
        assert np.array_equal(r[key], gold[f"{wall}_{uref:g}_{key}"]), key
    assert r["mean"] == float(gold[f"{wall}_{uref:g}_mean"])


def test_channel_profile_in_wall_units():
    m, st, nu = _c1()
    p = channel_profile(m, st, nu)
    # body force 1 on a half-height-1 channel: u_tau = 1, Re_tau = 550
    assert abs(p["u_tau"] - 1.0) < 1e-3 and abs(p["re_tau"] - 550.0) < 1.0
    assert len(p["yplus"]) == 64 and np.all(np.diff(p["yplus"]) > 0)
    assert p["yplus"][0] < 1.0                                  # first cell y+ < 1 (ratio 1.08)
    assert abs(p["U"][0] - p["yplus"][0]) < 0.05 * p["yplus"][0]  # viscous sublayer U+ = y+
    assert 18.0 < p["U"][-1] < 26.0                              # centreline U+ at Re_tau 550
