"""In-tree build of libbtm_gb300.so (CUDA engine + C++ host driver, C ABI).

Compiles the translation units in csrc/ with nvcc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, and links them into
<package>/_build/libbtm_gb300.so.  A stamp of the source contents skips the
rebuild when nothing changed.

The FP64 engine (btm_engine.cu) is compiled with -fmad=false: every
multiply-add stays two IEEE operations so that assembly, gradients and
mat-vecs round exactly like the reference's face loops.  The mixed-precision
engine (btm_mixed.cu) keeps contraction on.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
INCLUDE = os.path.join(os.path.dirname(PKG_ROOT), "include")
LIB_NAME = "libbtm_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["btm_engine.cu", "btm_mixed.cu", "btm_host.cpp", "btm_server.cpp", "btm_noalloc.cu"]
HEADERS = ["btm_common.h", "btm_host_internal.h", "btm_team.cuh", "btm_bc.cuh", "btm_phases64.cuh",
           "btm_observe.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbtm_gb300.so")


def lib_path() -> str:
    return os.path.join(BUILD, LIB_NAME)


def _stamp() -> str:
    h = hashlib.sha256()
    for name in SOURCES + HEADERS:
        with open(os.path.join(CSRC, name), "rb") as fh:
            h.update(fh.read())
    with open(os.path.join(INCLUDE, "btm_gb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(ARCH).encode())
    h.update(b"host-fp-contract-off")
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if needed) and return the path of libbtm_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    stamp_file = os.path.join(BUILD, "stamp.txt")
    stamp = _stamp()
    out = lib_path()
    if not force and os.path.exists(out) and os.path.exists(stamp_file):
        with open(stamp_file) as fh:
            if fh.read().strip() == stamp:
                return out
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]
    # host code: no floating-point contraction (gcc on Arm fuses a*b+c into an
    # FMA by default), so host-side geometry and observation constants round
    # like the reference and numpy
    host = ["-Xcompiler", "-ffp-contract=off"]
    jobs = [
        [cc] + common + ["-fmad=false", "-c", os.path.join(CSRC, "btm_engine.cu"), "-o",
                         os.path.join(BUILD, "btm_engine.o")],
        [cc] + common + host + ["-x", "cu", "-c", os.path.join(CSRC, "btm_host.cpp"), "-o",
                                os.path.join(BUILD, "btm_host.o")],
        [cc] + common + host + ["-x", "cu", "-c", os.path.join(CSRC, "btm_server.cpp"), "-o",
                                os.path.join(BUILD, "btm_server.o")],
        [cc] + common + ["-c", os.path.join(CSRC, "btm_noalloc.cu"), "-o", os.path.join(BUILD, "btm_noalloc.o")],
        [cc] + common + ["-c", os.path.join(CSRC, "btm_mixed.cu"), "-o", os.path.join(BUILD, "btm_mixed.o")],
    ]

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    tmp = out + ".tmp"
    run([cc] + ARCH + ["-shared", "-o", tmp, os.path.join(BUILD, "btm_engine.o"),
                       os.path.join(BUILD, "btm_host.o"), os.path.join(BUILD, "btm_noalloc.o"),
                       os.path.join(BUILD, "btm_mixed.o"), os.path.join(BUILD, "btm_server.o"),
                       "-cudart", "static"])
    os.replace(tmp, out)
    with open(stamp_file, "w") as fh:
        fh.write(stamp)
    return out
