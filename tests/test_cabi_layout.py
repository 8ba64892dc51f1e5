"""The ctypes mirrors of the C-ABI structs (rans_sst_py/_lib.py, _server.py and
the oracle's copy in oracle/cabi.py) match include/btm_gb300.h field for
field: same names, offsets and sizes, checked against a C program compiled
from the header with the host C compiler (no GPU needed)."""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import pytest

import cases  # noqa: F401  (puts the package on sys.path)
from rans_sst_py import _lib, _server

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")

STRUCTS = {
    "btm_mesh": _lib.BtmMesh,
    "btm_patch_bc": _lib.BtmPatchBC,
    "btm_settings": _lib.BtmSettings,
    "btm_state": _lib.BtmState,
    "btm_init": _lib.BtmInit,
    "btm_history": _lib.BtmHistory,
    "btm_observable": _lib.BtmObservable,
    "btm_request": _server.BtmRequest,
}


def _c_layout():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "btm_gb300.h"', "int main(void) {"]
    for name, cls in STRUCTS.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'printf("{name}.{field} %zu\\n", offsetof({name}, {field}));')
    lines += ["return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as fh:
            fh.write("\n".join(lines))
        subprocess.run([cc, "-I", INCLUDE, src, "-o", exe], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return dict((k, int(v)) for k, v in (ln.split() for ln in out.splitlines()))


def test_ctypes_structs_match_header():
    lay = _c_layout()
    for name, cls in STRUCTS.items():
        assert C.sizeof(cls) == lay[name], name
        for field, _ in cls._fields_:
            assert getattr(cls, field).offset == lay[f"{name}.{field}"], f"{name}.{field}"


def test_oracle_mirror_matches_header():
    import sys
    sys.path.insert(0, ROOT)
    from oracle import cabi
    lay = _c_layout()
    pairs = {"btm_patch_bc": "PatchBC", "btm_settings": "Settings", "btm_state": "State", "btm_init": "Init",
             "btm_history": "History"}
    for cname, pyname in pairs.items():
        cls = getattr(cabi, pyname, None)
        if cls is None:
            continue
        assert C.sizeof(cls) == lay[cname], cname
        for field, _ in cls._fields_:
            assert getattr(cls, field).offset == lay[f"{cname}.{field}"], f"{cname}.{field}"
