"""Served request loop (btm_server_* in include/btm_gb300.h): continuous
batching of forward-solve requests on one GPU.

    srv = Server(max_slots=304, hbm_budget_bytes=8 << 30)
    rid = srv.submit(case, coeffs, init=..., tag=chain_id)   # None: not admitted now
    for rid, out in srv.poll(timeout_ms=5):                  # completed requests
        ...

A request is admitted when its case has a free solve slot, or a new slot fits
the slot count and the HBM budget; admitted requests start at the next poll
or flush while earlier ones keep running, and each finishes on its own.
`tag` keeps the final state on the device and starts the next request with
the same tag (and case) from it, as an MCMC chain's last field.  When the case
has an observation operator attached (Case.set_observations), each result
carries the device-evaluated predictions and log-likelihood; with
want_state=False nothing else leaves the device.
"""
from __future__ import annotations

import ctypes as C
import itertools
from typing import List, Optional, Tuple

import numpy as np

from . import _lib
from ._forward import SolveOutput, _init_struct
from ._lib import BtmHistory, BtmInit, BtmState, check, dptr, lib, new_state, state_struct

BTM_EAGAIN = 1
BTM_REQ_TAG_NORMS = 1


class BtmRequest(C.Structure):
    _fields_ = [("id", C.c_int64), ("c", C.c_void_p), ("coeffs", _lib._dp), ("variant", C.c_int32),
                ("init", C.POINTER(BtmInit)), ("warm_tag", C.c_int64), ("out", C.POINTER(BtmState)),
                ("hist", C.POINTER(BtmHistory)), ("flags", C.c_int32)]


def _bind(L):
    if getattr(L, "_server_bound", False):
        return L
    L.btm_server_create.argtypes = [C.c_int32, C.c_int64, C.POINTER(C.c_void_p)]
    L.btm_server_destroy.argtypes = [C.c_void_p]
    L.btm_server_destroy.restype = None
    L.btm_server_submit.argtypes = [C.c_void_p, C.POINTER(BtmRequest)]
    L.btm_server_flush.argtypes = [C.c_void_p]
    L.btm_server_poll.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.c_int32, C.POINTER(C.c_int32)]
    L.btm_server_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int32)]
    L._server_bound = True
    return L


class Server:
    """Owning handle of a resident request loop."""

    def __init__(self, max_slots: int = 304, hbm_budget_bytes: int = 8 << 30):
        self._L = _bind(lib())
        h = C.c_void_p()
        check(self._L.btm_server_create(int(max_slots), int(hbm_budget_bytes), C.byref(h)))
        self.h = h
        self._ids = itertools.count()
        self._live = {}   # id -> buffers that must outlive the request

    def submit(self, case, coeffs, variant: int = 0, init=None, tag: int = -1,
               want_state: bool = True, tag_norms: bool = False) -> Optional[int]:
        """Admit one request; returns its id, or None when no slot / memory is free now.

        tag_norms: a tag-started solve scales its residuals by those of the
        tag's first (cold) solve (BTM_REQ_TAG_NORMS) instead of by its own
        first defects as the reference does."""
        rid = next(self._ids)
        keep = []
        cf = np.ascontiguousarray(np.asarray(coeffs, np.float64).reshape(11))
        ini = _init_struct(init, keep)
        state = new_state(case.n_cells, case.n_bnd) if want_state else None
        st = state_struct(state) if want_state else None
        hist = BtmHistory()
        pred = None
        if case.n_obs > 0:
            # observables evaluated on the device at the end of the solve
            pred = np.zeros(case.n_obs)
            hist.predictions = dptr(pred)
        req = BtmRequest(rid, case.h.value, dptr(cf), int(variant), C.pointer(ini), int(tag),
                         C.pointer(st) if st is not None else None, C.pointer(hist),
                         BTM_REQ_TAG_NORMS if tag_norms else 0)
        rc = self._L.btm_server_submit(self.h, C.byref(req))
        if rc == BTM_EAGAIN:
            return None
        check(rc)
        self._live[rid] = (case, cf, ini, keep, state, st, hist, req, pred)
        return rid

    def flush(self):
        check(self._L.btm_server_flush(self.h))

    def poll(self, timeout_ms: int = 0, cap: int = 1024) -> List[Tuple[int, SolveOutput]]:
        ids = (C.c_int64 * cap)()
        n = C.c_int32(0)
        rc = self._L.btm_server_poll(self.h, int(timeout_ms), ids, cap, C.byref(n))
        if rc == BTM_EAGAIN:
            return []
        check(rc)
        done = []
        for i in range(n.value):
            rid = int(ids[i])
            case, cf, ini, keep, state, st, hist, req, pred = self._live.pop(rid)
            if state is not None:
                state["turb_established"] = int(st.turb_established)
            done.append((rid, SolveOutput(state, hist, None, pred)))
        return done

    def stats(self) -> dict:
        b, s, inf = C.c_int32(), C.c_int32(), C.c_int32()
        by = C.c_int64()
        check(self._L.btm_server_stats(self.h, C.byref(b), C.byref(s), C.byref(by), C.byref(inf)))
        return dict(busy_slots=b.value, slots=s.value, bytes=by.value, inflight=inf.value)

    @property
    def pending(self) -> int:
        return len(self._live)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self._L.btm_server_destroy(self.h)
            self.h = C.c_void_p()
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
