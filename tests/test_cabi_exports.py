"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/btm_gb300.h declares (no compute call: runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

from cases import ROOT

HEADER = os.path.join(ROOT, "include", "btm_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(btm_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("btm_case_create", "btm_case_destroy", "btm_solve", "btm_solve_batch", "btm_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from rans_sst_py import _build
    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"not exported: {missing}"
    lib.btm_abi_version.restype = ctypes.c_int
    assert lib.btm_abi_version() == 6


def test_build_targets_sm103a_only():
    from rans_sst_py import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_device_fails_loudly():
    """Without a GPU the product path raises instead of falling back."""
    import rans_sst_py
    from rans_sst_py._lib import BtmError, Case
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except Exception:
        pass
    m = rans_sst_py.Mesh.make_channel_2d(4, 8, 1.0, 1.0)
    bcs = rans_sst_py.FlowBoundaryConditions.channel_defaults(m, 1.0, 1e-4, 1.0)
    with pytest.raises(BtmError):
        Case(m, bcs, 1e-3, rans_sst_py.SolverSettings())


@pytest.mark.parametrize("field,value,code", [
    ("anderson_depth", 9, "anderson_depth"),
    ("anderson_depth", -1, "anderson_depth"),
    ("amg_order", 3, "amg_order"),
    ("turb_update_interval", 0, "turb_update_interval"),
])
def test_settings_rejected_before_any_device_work(field, value, code):
    """btm_case_create validates the settings (BTM_ERR_ARG, message naming
    the field) before it looks for a device, so an invalid setting is
    reported the same way on a machine without a GPU."""
    import ctypes as C
    import rans_sst_py
    from rans_sst_py import _lib
    m = rans_sst_py.Mesh.make_channel_2d(4, 8, 1.0, 1.0)
    bcs = rans_sst_py.FlowBoundaryConditions.channel_defaults(m, 1.0, 1e-4, 1.0)
    st = _lib.settings_struct(rans_sst_py.SolverSettings())
    setattr(st, field, value)
    md, keep_m = _lib.mesh_struct(m)
    bca, keep_b = _lib.bc_structs(bcs)
    L = _lib.lib()
    h = C.c_void_p()
    rc = L.btm_case_create(C.byref(md), bca, C.c_double(1e-3), C.byref(st), C.byref(h))
    assert rc == -1, rc                      # BTM_ERR_ARG
    assert code in L.btm_last_error().decode()
