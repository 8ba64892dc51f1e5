"""btm_solve_noalloc: the allocation-free solve entry point.

It exists for callers that cannot allocate device memory while serving
requests (programs whose device memory belongs to their own pool or budget,
and latency-critical loops that cannot pay for cudaMalloc/cudaFree per
request).  It runs the same kernel as btm_solve with its scratch in a static
16 MiB device array, so its results must equal btm_solve's bit for bit.  The
array keeps the previous call's contents, so every check here runs at least
two calls in a row, some with a different mesh and other coefficients in
between.  This file sorts last so a failure here never hides the other GPU
tests.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from rans_sst_py import ObservationOperator, Vec3
from rans_sst_py._lib import BtmError, BtmHistory, BtmInit, Case, check, dptr, lib, new_state, state_struct

pytestmark = pytest.mark.gpu

FIELDS = ("U", "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw", "Ub", "pb", "kb", "omegab")


def _call(fn, case, coeffs, init, hist_rows=0, n_obs=0, res=None):
    st = new_state(case.n_cells, case.n_bnd)
    s = state_struct(st)
    h = BtmHistory()
    if hist_rows:
        if res is None:
            res = np.zeros((hist_rows, 6))
        h.residual_capacity = hist_rows
        h.residuals = dptr(res)
    preds = None
    if n_obs:
        preds = np.zeros(n_obs)
        h.predictions = dptr(preds)
    cf = np.ascontiguousarray(coeffs, np.float64)
    check(fn(case.h, dptr(cf), 0, C.byref(init), C.byref(s), C.byref(h)))
    st["turb_established"] = s.turb_established
    return st, h, res, preds


def _cold(init):
    ini = BtmInit()
    ini.mode = 0
    ini.u[0], ini.u[1], ini.u[2] = init["u"]
    ini.p, ini.k, ini.omega = init["p"], init["k"], init["omega"]
    return ini


def _identical(a, b):
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), f


def _channel(iters, tol=0.0):
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    return Case(m, bcs, nu, cases.channel_settings(iters, tol)), init


def test_noalloc_matches_btm_solve_twice():
    case, init = _channel(400)
    coeffs = np.array(cases.COEFF_DEFAULTS)
    ref, href, rref, _ = _call(lib().btm_solve, case, coeffs, _cold(init), hist_rows=400)
    for _ in range(2):  # the static scratch keeps the last call's contents
        got, h, r, _ = _call(lib().btm_solve_noalloc, case, coeffs, _cold(init), hist_rows=400)
        _identical(got, ref)
        assert h.iterations_run == href.iterations_run == 400
        assert h.status == href.status
        assert np.array_equal(r, rref)


def test_noalloc_result_independent_of_leftover_scratch():
    """A solve of another mesh with other coefficients between two channel
    solves leaves different contents in the shared array; the channel result
    must not change."""
    case, init = _channel(300)
    coeffs = np.array(cases.COEFF_DEFAULTS)
    ref, _, _, _ = _call(lib().btm_solve, case, coeffs, _cold(init))
    first, _, _, _ = _call(lib().btm_solve_noalloc, case, coeffs, _cold(init))
    _identical(first, ref)
    mc, bc, nuc, ic = cases.couette_case(4, 32)
    couette = Case(mc, bc, nuc, cases.couette_settings(250, 0.0))
    other = np.array(cases.COEFF_DEFAULTS) * 1.07
    _call(lib().btm_solve_noalloc, couette, other, _cold(ic))
    again, _, _, _ = _call(lib().btm_solve_noalloc, case, coeffs, _cold(init))
    _identical(again, ref)


def test_noalloc_history_only_rows_written():
    """A solve that converges well before the history capacity returns the
    rows it wrote (equal to btm_solve's) and leaves the caller's rows beyond
    them untouched, although the array still holds a longer earlier run's
    residuals there."""
    rows = 4000
    long_case, init = _channel(rows, 0.0)
    coeffs = np.array(cases.COEFF_DEFAULTS)
    _call(lib().btm_solve_noalloc, long_case, coeffs, _cold(init), hist_rows=rows)   # fills every row
    case, _ = _channel(rows, 1e-4)
    _, href, rref, _ = _call(lib().btm_solve, case, coeffs, _cold(init), hist_rows=rows,
                             res=np.full((rows, 6), -7.0))
    n = href.iterations_run
    assert href.converged and n < rows - 1000
    for _ in range(2):
        _, h, r, _ = _call(lib().btm_solve_noalloc, case, coeffs, _cold(init), hist_rows=rows,
                           res=np.full((rows, 6), -7.0))
        assert h.iterations_run == n and h.converged
        assert np.array_equal(r[:n], rref[:n])
        assert np.all(r[n:] == -7.0)


def test_noalloc_observations_match():
    """Observables attached to the case are evaluated by the allocation-free
    call too: predictions and log-likelihood equal btm_solve's."""
    case, init = _channel(200)
    m, _, _, _ = cases.periodic_channel(32, 180.0)
    op = ObservationOperator()
    op.add_skin_friction("bottom_wall", Vec3(0.5, 0.0, 0.5), 0.006, 0.001, 16.0)
    op.add_velocity_profile(Vec3(0.5, 1.0, 0.5), 0, 18.0, 1.0)
    op.add_velocity_profile(Vec3(0.5, 0.1, 0.5), 0, 9.0, 1.0)
    case.set_observations(op)
    coeffs = np.array(cases.COEFF_DEFAULTS)
    _, href, _, pref = _call(lib().btm_solve, case, coeffs, _cold(init), n_obs=3)
    assert np.all(np.isfinite(pref))
    for _ in range(2):
        _, h, _, p = _call(lib().btm_solve_noalloc, case, coeffs, _cold(init), n_obs=3)
        assert np.array_equal(p, pref)
        assert h.log_lik == href.log_lik


def test_noalloc_reports_its_launch_time():
    tiny, init = _channel(1)
    coeffs = np.array(cases.COEFF_DEFAULTS)
    _call(lib().btm_solve, tiny, coeffs, _cold(init))
    case, _ = _channel(400)
    _, h, _, _ = _call(lib().btm_solve_noalloc, case, coeffs, _cold(init))
    ms = lib().btm_last_launch_ms()
    assert ms >= 0.9 * h.solve_ms > 0.0


def test_noalloc_warm_start_matches():
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    case = Case(m, bcs, nu, cases.channel_settings(150, 0.0))
    coeffs = np.array(cases.COEFF_DEFAULTS)
    first, _, _, _ = _call(lib().btm_solve, case, coeffs, _cold(init))
    keep = state_struct(first)
    warm = BtmInit()
    warm.mode = 1
    warm.warm = C.pointer(keep)
    ref, _, _, _ = _call(lib().btm_solve, case, coeffs * 1.01, warm)
    for _ in range(2):
        got, _, _, _ = _call(lib().btm_solve_noalloc, case, coeffs * 1.01, warm)
        _identical(got, ref)


def test_noalloc_rejects_oversized_mesh():
    m, bcs, nu, init = cases.periodic_channel(512, 180.0, nx=34, ratio=1.01)  # 17408 cells > 16384
    case = Case(m, bcs, nu, cases.channel_settings(1, 0.0))
    with pytest.raises(BtmError, match="btm_solve_noalloc"):
        _call(lib().btm_solve_noalloc, case, np.array(cases.COEFF_DEFAULTS), _cold(init))


def test_noalloc_rejects_oversized_history():
    """A small mesh whose requested residual history would not fit beside its
    scratch in the 16 MiB array is rejected, not truncated."""
    case, init = _channel(1)
    with pytest.raises(BtmError, match="bytes of scratch"):
        _call(lib().btm_solve_noalloc, case, np.array(cases.COEFF_DEFAULTS), _cold(init), hist_rows=400000)
