"""OpenFOAM ASCII polyMesh reader: Mesh::loadOpenFOAM (core/src/Mesh.cpp:50-265).

The five polyMesh files (points, faces, owner, neighbour, boundary) are read
the way the reference reads them: the element count is the first line that
parses as an integer outside the FoamFile header, the data follows the first
line that is exactly "(", and entries are whitespace-separated tokens.  Face
centres are node averages, face area vectors the fan sum of half cross
products about that centre, in node order; cell centres, volumes, face deltas
and interpolation weights then follow the reference's geometry passes
(Mesh.compute_geometry).  The arithmetic follows the reference's operation
order, so the geometry is bit-identical to the reference loader's.
"""
from __future__ import annotations

import os
import re
from typing import List, Tuple

import numpy as np

_INT = re.compile(r"[+-]?\d+")
_TOKEN = re.compile(r"\(|\)|[^\s()]+")


def _strip_comment(line: str) -> str:
    pos = line.find("//")
    return line if pos < 0 else line[:pos]


def _read_count(lines: List[str], i: int) -> Tuple[int, int]:
    """readFoamCount: the first line (comments removed, trimmed) that starts
    with an integer and not with one of the header letters."""
    while i < len(lines):
        line = _strip_comment(lines[i]).strip(" \t\r")
        i += 1
        if not line or line[0] in "/FOovCa{}":
            continue
        m = _INT.match(line)
        if m:
            return int(m.group(0)), i
    raise RuntimeError("Could not read count")


def _skip_header(lines: List[str], i: int) -> int:
    """skipFoamHeader: past the first line that is exactly "(" once leading
    blanks and comments are removed."""
    while i < len(lines):
        line = _strip_comment(lines[i]).lstrip(" \t\r")
        i += 1
        if line == "(":
            return i
    raise RuntimeError("Could not find data block")


def _open(poly_dir: str, name: str, what: str) -> Tuple[List[str], int, int]:
    path = os.path.join(poly_dir, name)
    try:
        with open(path) as fh:
            lines = fh.read().split("\n")
    except OSError:
        raise RuntimeError(what) from None
    n, i = _read_count(lines, 0)
    i = _skip_header(lines, i)
    return lines, n, i


def _tokens(lines: List[str], i: int):
    return _TOKEN.findall("\n".join(lines[i:]))


def load_openfoam(poly_dir: str):
    from ._mesh import Mesh, _Builder

    # points
    lines, n_pts, i = _open(poly_dir, "points", "Cannot open points file")
    tok = _tokens(lines, i)
    nodes = np.empty((n_pts, 3))
    t = 0
    for p in range(n_pts):
        t += 1                                        # '('
        nodes[p] = (float(tok[t]), float(tok[t + 1]), float(tok[t + 2]))
        t += 4                                        # x y z ')'
    # faces
    lines, n_faces, i = _open(poly_dir, "faces", "Cannot open faces file")
    tok = _tokens(lines, i)
    face_nodes: List[List[int]] = []
    t = 0
    for f in range(n_faces):
        nv = int(tok[t])
        face_nodes.append([int(v) for v in tok[t + 2:t + 2 + nv]])
        t += nv + 3                                   # nv '(' ... ')'
    # owner / neighbour
    lines, n_own, i = _open(poly_dir, "owner", "Cannot open owner file in " + poly_dir)
    tok = _tokens(lines, i)
    owner = np.full(n_faces, -1, np.int32)
    owner[:n_own] = [int(v) for v in tok[:n_own]]
    lines, n_nbr, i = _open(poly_dir, "neighbour", "Cannot open neighbour file in " + poly_dir)
    tok = _tokens(lines, i)
    neigh = np.full(n_faces, -1, np.int32)
    neigh[:n_nbr] = [int(v) for v in tok[:n_nbr]]
    n_cells = int(max(owner.max(initial=-1), neigh.max(initial=-1))) + 1

    # boundary patches
    patches = []
    face_patch = np.full(n_faces, -1, np.int32)
    bpath = os.path.join(poly_dir, "boundary")
    if os.path.exists(bpath):
        lines, n_p, i = _open(poly_dir, "boundary", "Cannot open boundary file")
        for p in range(n_p):
            name = ""
            while i < len(lines):
                line = _strip_comment(lines[i]).strip(" \t\r")
                i += 1
                if line and line not in ("{", "}"):
                    name = line
                    break
            ptype, nf, start = "", 0, 0
            while i < len(lines):
                line = _strip_comment(lines[i]).lstrip(" \t\r")
                i += 1
                if "}" in line:
                    break
                parts = line.split()
                if not parts:
                    continue
                if parts[0] == "type" and len(parts) > 1:
                    ptype = parts[1][:-1] if parts[1].endswith(";") else parts[1]
                elif parts[0] in ("nFaces", "startFace") and len(parts) > 1:
                    m = _INT.match(parts[1])
                    if m:
                        if parts[0] == "nFaces":
                            nf = int(m.group(0))
                        else:
                            start = int(m.group(0))
            ids = np.arange(start, start + nf, dtype=np.int32)
            face_patch[ids] = p
            patches.append((name, ptype, ids))

    # face geometry: node-average centre, fan of half cross products
    center = np.zeros((n_faces, 3))
    area_vec = np.zeros((n_faces, 3))
    counts = np.array([len(fn) for fn in face_nodes], dtype=np.int64)
    for nv in np.unique(counts):
        sel = np.nonzero(counts == nv)[0]
        idx = np.array([face_nodes[f] for f in sel], dtype=np.int64)
        ctr = np.zeros((sel.size, 3))
        for j in range(nv):
            ctr = ctr + nodes[idx[:, j]]
        ctr = ctr / float(nv)
        an = np.zeros((sel.size, 3))
        for j in range(nv):
            a = nodes[idx[:, j]] - ctr
            b = nodes[idx[:, (j + 1) % nv]] - ctr
            cx = a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1]
            cy = a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2]
            cz = a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]
            an = an + np.stack([cx, cy, cz], 1) * 0.5
        center[sel] = ctr
        area_vec[sel] = an
    area = np.sqrt(area_vec[:, 0] * area_vec[:, 0] + area_vec[:, 1] * area_vec[:, 1] +
                   area_vec[:, 2] * area_vec[:, 2])
    with np.errstate(divide="ignore", invalid="ignore"):
        normal = np.where(area[:, None] > 1e-300, area_vec / area[:, None], 0.0)

    b = _Builder(n_cells)
    b.add(owner, neigh, center, normal, area)
    m = b.finish()
    m.face_patch = face_patch
    m.patches = patches
    m.n_internal = n_nbr
    m.nodes = nodes
    m.compute_geometry()
    return m
