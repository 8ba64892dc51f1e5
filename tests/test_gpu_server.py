"""Served request loop (rans_sst_py.Server over btm_server_*): continuous
batching.  Requests submitted while others run are admitted as slots free up
and overlap on the device; every result is the same bits alone (solve) and in
the mix, and warm-start tags continue from the device-resident last field."""
import time

import numpy as np
import pytest

import cases
from rans_sst_py import Case, Server, solve

pytestmark = pytest.mark.gpu

COEFF = np.array(cases.COEFF_DEFAULTS)
FIELDS = ("U", "p", "k", "omega", "nuT")


def _cases():
    m1, b1, nu1, i1 = cases.periodic_channel(32, 180.0)
    m2, b2, nu2, i2 = cases.couette_case(4, 16)
    s1 = cases.channel_settings(1500, 0.0)
    s1.precision = "mixed"
    s2 = cases.couette_settings(400, 0.0)
    return (Case(m1, b1, nu1, s1), i1), (Case(m2, b2, nu2, s2), i2)


def _drain(srv, n, timeout_s=120.0):
    got = {}
    t0 = time.time()
    while len(got) < n and time.time() - t0 < timeout_s:
        for rid, out in srv.poll(timeout_ms=20):
            got[rid] = out
    assert len(got) == n
    return got


def test_server_mix_matches_solo_bitwise():
    (c1, i1), (c2, i2) = _cases()
    thetas = [COEFF * (1.0 + 0.01 * j) for j in range(6)]
    srv = Server(max_slots=64, hbm_budget_bytes=1 << 30)
    reqs = {}
    # a first group, launched ...
    for j in range(3):
        reqs[srv.submit(c1, thetas[j], init=i1)] = (c1, thetas[j], i1)
    reqs[srv.submit(c2, thetas[0], init=i2)] = (c2, thetas[0], i2)
    srv.flush()
    # ... and a second one admitted while the first is on the device
    for j in range(3, 6):
        reqs[srv.submit(c1, thetas[j], init=i1)] = (c1, thetas[j], i1)
    reqs[srv.submit(c2, thetas[1], init=i2)] = (c2, thetas[1], i2)
    assert None not in reqs
    got = _drain(srv, len(reqs))
    for rid, (c, th, ini) in reqs.items():
        solo = solve(c, th, 0, ini)
        for f in FIELDS:
            assert np.array_equal(got[rid].state[f], solo.state[f]), (rid, f)
        assert got[rid].iterations_run == solo.iterations_run
    srv.close()


def test_server_warm_tag_continues_from_device_state():
    (c1, i1), _ = _cases()
    srv = Server(max_slots=8, hbm_budget_bytes=1 << 30)
    a = srv.submit(c1, COEFF, init=i1, tag=7)
    first = _drain(srv, 1)[a]
    th2 = COEFF.copy()
    th2[9] *= 1.02
    b = srv.submit(c1, th2, init=i1, tag=7)   # the tag's state wins over `init`
    second = _drain(srv, 1)[b]
    ref = solve(c1, th2, 0, first.state)
    for f in FIELDS:
        assert np.array_equal(second.state[f], ref.state[f]), f
    srv.close()


def test_server_admission_by_budget():
    (c1, i1), _ = _cases()
    srv = Server(max_slots=8, hbm_budget_bytes=1 << 30)
    assert srv.submit(c1, COEFF, init=i1) is not None
    one_slot = srv.stats()["bytes"]
    srv.close()
    srv = Server(max_slots=8, hbm_budget_bytes=2 * one_slot + one_slot // 2)
    ids = [srv.submit(c1, COEFF, init=i1) for _ in range(3)]
    assert ids[0] is not None and ids[1] is not None and ids[2] is None
    done = _drain(srv, 2)
    assert set(done) == {ids[0], ids[1]}
    assert srv.submit(c1, COEFF, init=i1) is not None   # a recycled slot
    _drain(srv, 1)
    srv.close()


def test_server_poll_is_bounded():
    srv = Server(max_slots=4, hbm_budget_bytes=1 << 28)
    t0 = time.time()
    assert srv.poll(timeout_ms=50) == []
    assert time.time() - t0 < 5.0
    srv.close()
