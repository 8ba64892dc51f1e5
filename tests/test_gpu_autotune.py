"""Launch-shape autotuner (btm_case_launch_shape): the first one-CTA solve of
a case times 256- and 512-thread CTAs on a probe batch and keeps the faster;
the shape belongs to the case, so a solve gives the same bits alone and
inside a batch that mixes meshes of other sizes."""
import numpy as np
import pytest

import cases
from rans_sst_py import Case, solve, solve_batch

pytestmark = pytest.mark.gpu


def test_first_solve_tunes_the_case():
    m, bcs, nu, init = cases.periodic_channel(64, 180.0)
    case = Case(m, bcs, nu, cases.channel_settings(20, 0.0))
    before = case.launch_shape("fp64")
    assert not before["tuned"] and before["threads"] in (256, 512)
    solve(case, cases.COEFF_DEFAULTS, 0, init, want_state=False)
    sh = case.launch_shape("fp64")
    assert sh["tuned"] and sh["probe"] >= 1
    t256, t512 = sh["probe_ms"]
    assert t256 > 0.0 and t512 > 0.0
    assert sh["threads"] == (512 if t512 < t256 else 256)
    assert not case.launch_shape("mixed")["tuned"]      # tuned per engine


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_same_bits_alone_and_in_a_mixed_size_batch(precision):
    small = cases.periodic_channel(32, 180.0)
    large = cases.periodic_channel(512, 180.0, nx=4)      # 2048 cells
    cs = []
    for m, bcs, nu, init in (small, large):
        s = cases.channel_settings(150, 0.0)
        s.precision = precision
        cs.append((Case(m, bcs, nu, s), init))
    coeffs = np.array(cases.COEFF_DEFAULTS)
    alone = [solve(c, coeffs, 0, init) for c, init in cs]
    mixed = solve_batch([cs[0][0], cs[1][0], cs[0][0]], [coeffs] * 3, None, [cs[0][1], cs[1][1], cs[0][1]])
    for a, b in ((alone[0], mixed[0]), (alone[1], mixed[1]), (alone[0], mixed[2])):
        for f in ("U", "p", "k", "omega", "nuT"):
            assert np.array_equal(a.state[f], b.state[f]), f
