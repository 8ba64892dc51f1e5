"""btm_solve_noalloc: the allocation-free solve entry point.

It exists for callers that cannot allocate device memory while serving
requests (programs whose device memory belongs to their own pool or budget,
and latency-critical loops that cannot pay for cudaMalloc/cudaFree per
request).  It runs the same kernel as btm_solve with its scratch in a static
16 MiB device array, so its results must equal btm_solve's; the array is
reused, so two calls in a row must both match.  This file sorts last so a
failure here never hides the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from rans_sst_py._lib import (BtmError, BtmHistory, BtmInit, Case, check, dptr, lib, new_state,
                              state_struct)

pytestmark = pytest.mark.gpu

FIELDS = ("U", "p", "k", "omega", "nuT", "F1", "F2", "Pk", "CDkw", "Ub", "pb", "kb", "omegab")


def _call(fn, case, coeffs, init, hist_rows=0):
    st = new_state(case.n_cells, case.n_bnd)
    s = state_struct(st)
    h = BtmHistory()
    res = None
    if hist_rows:
        res = np.zeros((hist_rows, 6))
        h.residual_capacity = hist_rows
        h.residuals = dptr(res)
    cf = np.ascontiguousarray(coeffs, np.float64)
    check(fn(case.h, dptr(cf), 0, C.byref(init), C.byref(s), C.byref(h)))
    st["turb_established"] = s.turb_established
    return st, h, res


def _cold(init):
    ini = BtmInit()
    ini.mode = 0
    ini.u[0], ini.u[1], ini.u[2] = init["u"]
    ini.p, ini.k, ini.omega = init["p"], init["k"], init["omega"]
    return ini


def _same(a, b, tol=1e-12):
    for f in FIELDS:
        assert cases.rel_l2(a[f], b[f]) <= tol, f


def test_noalloc_matches_btm_solve_twice():
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    case = Case(m, bcs, nu, cases.channel_settings(400, 0.0))
    coeffs = np.array(cases.COEFF_DEFAULTS)
    ref, href, rref = _call(lib().btm_solve, case, coeffs, _cold(init), hist_rows=400)
    for _ in range(2):  # the static scratch keeps the last call's contents
        got, h, r = _call(lib().btm_solve_noalloc, case, coeffs, _cold(init), hist_rows=400)
        _same(got, ref)
        assert h.iterations_run == href.iterations_run == 400
        assert h.status == href.status
        assert np.allclose(r, rref, rtol=1e-12, atol=0.0)


def test_noalloc_warm_start_matches():
    m, bcs, nu, init = cases.periodic_channel(32, 180.0)
    case = Case(m, bcs, nu, cases.channel_settings(150, 0.0))
    coeffs = np.array(cases.COEFF_DEFAULTS)
    first, _, _ = _call(lib().btm_solve, case, coeffs, _cold(init))
    keep = state_struct(first)
    warm = BtmInit()
    warm.mode = 1
    warm.warm = C.pointer(keep)
    ref, _, _ = _call(lib().btm_solve, case, coeffs * 1.01, warm)
    for _ in range(2):
        got, _, _ = _call(lib().btm_solve_noalloc, case, coeffs * 1.01, warm)
        _same(got, ref)


def test_noalloc_rejects_oversized_mesh():
    m, bcs, nu, init = cases.periodic_channel(512, 180.0, nx=34, ratio=1.01)  # 17408 cells > 16384
    case = Case(m, bcs, nu, cases.channel_settings(1, 0.0))
    with pytest.raises(BtmError, match="btm_solve_noalloc"):
        _call(lib().btm_solve_noalloc, case, np.array(cases.COEFF_DEFAULTS), _cold(init))
