"""Unstructured finite-volume mesh: factories, geometry, MSH1 I/O, renumbering.

Host-side mirror of the reference ``Mesh`` (core/include/Mesh.hpp:84-198,
core/src/Mesh.cpp).  Geometry is computed with the same floating-point
operations in the same order as the reference factories, so a mesh built here
is bit-identical to the one the reference builds (pinned by
tests/test_mesh_parity.py against fixtures written by the reference itself).
One-dimensional coordinate stretching uses ``math`` (the C library's tanh/pow),
never numpy's vectorised transcendental kernels, for the same reason.

Arrays (all numpy, C order):
  owner, neighbour        int32 [nF]   (neighbour = -1 on boundary faces)
  face_patch              int32 [nF]   (patchID, -1 on internal faces)
  face_center/normal/d    f64 [nF,3]
  face_area/delta/weight  f64 [nF]
  cell_center             f64 [nC,3]
  cell_volume             f64 [nC]
  cell_face_offset/faces  int32 CSR of each cell's face list (creation order)
  nodes                   f64 [nN,3]
  patches                 list of (name, type, int32 face ids)
"""
from __future__ import annotations

import math
import os
import struct
from typing import List, Optional, Sequence, Tuple

import numpy as np

PATCH_TYPE_CODES = {"wall": 1, "inlet": 2, "outlet": 3, "symmetry": 4}
MSH1_MAGIC = 0x4D534831  # "MSH1" (core/src/Mesh.cpp:602)


def _tanh_stretch_first_cell(extent: float, n: int, s: float) -> float:
    # first cell height of the symmetric tanh map (Mesh.cpp:1088-1091)
    return 0.5 * extent * (1.0 + math.tanh(s * (2.0 / n - 1.0)) / math.tanh(s))


def _bisect_tanh_stretch(extent: float, n: int, y1t: float, default: float) -> float:
    """Stretch parameter whose first cell height equals y1t (Mesh.cpp:1081-1113,
    1310-1326, 425-437): 100 bisection steps on [0.1, 20]."""
    if not (y1t < extent / n):
        return default
    s_lo, s_hi = 0.1, 20.0
    if y1t < _tanh_stretch_first_cell(extent, n, s_hi):
        return s_hi
    for _ in range(100):
        sm = 0.5 * (s_lo + s_hi)
        if _tanh_stretch_first_cell(extent, n, sm) > y1t:
            s_lo = sm
        else:
            s_hi = sm
        if s_hi - s_lo < 1e-10:
            break
    return 0.5 * (s_lo + s_hi)


def _tanh_nodes(extent: float, n: int, stretch: float, offset: float = 0.0) -> np.ndarray:
    out = np.empty(n + 1)
    for j in range(n + 1):
        eta = j / n
        v = 0.5 * extent * (1.0 + math.tanh(stretch * (2.0 * eta - 1.0)) / math.tanh(stretch))
        out[j] = v if offset == 0.0 else offset + v
    return out


def _norm3(v: np.ndarray) -> np.ndarray:
    # Vec3::norm: sqrt(x*x + y*y + z*z), evaluated left to right
    return np.sqrt(v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1] + v[..., 2] * v[..., 2])


class _Builder:
    """Accumulates faces in creation order and each cell's face list."""

    def __init__(self, n_cells: int):
        self.n_cells = n_cells
        self.owner: List[np.ndarray] = []
        self.neigh: List[np.ndarray] = []
        self.center: List[np.ndarray] = []
        self.normal: List[np.ndarray] = []
        self.area: List[np.ndarray] = []
        self.patch: List[np.ndarray] = []
        self.patches: List[Tuple[str, str, np.ndarray]] = []
        self.n_faces = 0

    def add(self, owner, neigh, center, normal, area, patch_id=-1):
        owner = np.asarray(owner, dtype=np.int32).ravel()
        n = owner.size
        self.owner.append(owner)
        self.neigh.append(np.asarray(neigh, dtype=np.int32).ravel() if neigh is not None
                          else np.full(n, -1, np.int32))
        self.center.append(np.asarray(center, dtype=np.float64).reshape(n, 3))
        self.normal.append(np.broadcast_to(np.asarray(normal, dtype=np.float64), (n, 3)).copy())
        self.area.append(np.asarray(area, dtype=np.float64).ravel())
        self.patch.append(np.full(n, patch_id, np.int32))
        ids = np.arange(self.n_faces, self.n_faces + n, dtype=np.int32)
        self.n_faces += n
        return ids

    def add_patch(self, name, ptype, owner, center, normal, area):
        pid = len(self.patches)
        ids = self.add(owner, None, center, normal, area, pid)
        self.patches.append((name, ptype, ids))
        return ids

    def finish(self) -> "Mesh":
        m = Mesh()
        m.owner = np.concatenate(self.owner)
        m.neighbour = np.concatenate(self.neigh)
        m.face_center = np.concatenate(self.center)
        m.face_normal = np.concatenate(self.normal)
        m.face_area = np.concatenate(self.area)
        m.face_patch = np.concatenate(self.patch)
        nF = m.owner.size
        m.n_internal = int(np.count_nonzero(m.neighbour >= 0))
        m.face_delta = np.zeros(nF)
        m.face_d = np.zeros((nF, 3))
        m.face_weight = np.full(nF, 0.5)
        m.patches = [(n, t, f.astype(np.int32)) for (n, t, f) in self.patches]
        # each cell's faces in creation order (Cell::faces push_back order)
        cells = np.concatenate([m.owner, m.neighbour[m.neighbour >= 0]])
        faces = np.concatenate([np.arange(nF, dtype=np.int32),
                                np.nonzero(m.neighbour >= 0)[0].astype(np.int32)])
        order = np.lexsort((faces, cells))
        m.cell_faces = faces[order].astype(np.int32)
        counts = np.bincount(cells, minlength=self.n_cells)
        m.cell_face_offset = np.zeros(self.n_cells + 1, np.int32)
        np.cumsum(counts, out=m.cell_face_offset[1:])
        m.cell_center = np.zeros((self.n_cells, 3))
        m.cell_volume = np.zeros(self.n_cells)
        m.nodes = np.zeros((0, 3))
        return m


class Mesh:
    """Finite-volume mesh with the reference's accessors (python/Bindings.cpp:325-374)."""

    def __init__(self):
        self.owner = np.zeros(0, np.int32)
        self.neighbour = np.zeros(0, np.int32)
        self.face_patch = np.zeros(0, np.int32)
        self.face_center = np.zeros((0, 3))
        self.face_normal = np.zeros((0, 3))
        self.face_area = np.zeros(0)
        self.face_delta = np.zeros(0)
        self.face_d = np.zeros((0, 3))
        self.face_weight = np.zeros(0)
        self.cell_center = np.zeros((0, 3))
        self.cell_volume = np.zeros(0)
        self.cell_face_offset = np.zeros(1, np.int32)
        self.cell_faces = np.zeros(0, np.int32)
        self.nodes = np.zeros((0, 3))
        self.patches: List[Tuple[str, str, np.ndarray]] = []
        self.n_internal = 0
        self.wall_dist: Optional[np.ndarray] = None

    # ---- counts / introspection (Bindings.cpp:362-374) -------------------
    def n_cells(self) -> int:
        return int(self.cell_volume.size)

    def n_faces(self) -> int:
        return int(self.owner.size)

    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])

    def n_patches(self) -> int:
        return len(self.patches)

    def n_internal_faces(self) -> int:
        return int(self.n_internal)

    def n_boundary_faces(self) -> int:
        return self.n_faces() - self.n_internal

    def patch_names(self) -> List[str]:
        return [p[0] for p in self.patches]

    def patch_types(self) -> List[str]:
        return [p[1] for p in self.patches]

    def patch_by_name(self, name: str) -> int:
        for i, p in enumerate(self.patches):
            if p[0] == name:
                return i
        raise RuntimeError("Patch not found: " + name)

    def set_patch_type(self, name: str, type: str) -> None:  # noqa: A002 (reference keyword)
        i = self.patch_by_name(name)
        n, _, f = self.patches[i]
        self.patches[i] = (n, type, f)

    def wall_patch_data(self, name: str) -> dict:
        idx = [i for i, p in enumerate(self.patches) if p[0] == name]
        if not idx:
            raise RuntimeError("Mesh::wall_patch_data: unknown patch '" + name + "'")
        pname, ptype, f = self.patches[idx[0]]
        return {"name": pname, "type": ptype, "n_faces": int(f.size),
                "owner": self.owner[f].astype(np.int32), "delta": self.face_delta[f].copy(),
                "center": self.face_center[f].copy(), "normal": self.face_normal[f].copy(),
                "area": self.face_area[f].copy()}

    def cell_centers(self) -> np.ndarray:
        return self.cell_center.copy()

    def cell_volumes(self) -> np.ndarray:
        return self.cell_volume.copy()

    def node_coords(self) -> np.ndarray:
        return self.nodes.copy()

    def face_centers(self) -> np.ndarray:
        return self.face_center.copy()

    def wall_distance(self) -> np.ndarray:
        if self.wall_dist is None:
            return np.zeros(0)
        return self.wall_dist.copy()

    def patch_type_codes(self) -> np.ndarray:
        return np.array([PATCH_TYPE_CODES.get(p[1], 0) for p in self.patches], np.int32)

    def patch_offsets(self) -> Tuple[np.ndarray, np.ndarray]:
        off = np.zeros(len(self.patches) + 1, np.int32)
        for i, p in enumerate(self.patches):
            off[i + 1] = off[i] + p[2].size
        faces = (np.concatenate([p[2] for p in self.patches]).astype(np.int32)
                 if self.patches else np.zeros(0, np.int32))
        return off, faces

    # ---- geometry --------------------------------------------------------
    def _compute_face_geometry(self) -> None:
        """Mesh::computeFaceGeometry (core/src/Mesh.cpp:301-315)."""
        nIF = self.n_internal
        o = self.owner
        d = np.empty_like(self.face_center)
        d[:nIF] = self.cell_center[self.neighbour[:nIF]] - self.cell_center[o[:nIF]]
        d[nIF:] = self.face_center[nIF:] - self.cell_center[o[nIF:]]
        delta = _norm3(d)
        delta[delta < 1e-30] = 1e-20
        self.face_d = d
        self.face_delta = delta

    def _compute_interpolation_weights(self) -> None:
        """Mesh::ComputeInterpolationWeights (core/src/Mesh.cpp:318-328)."""
        nIF = self.n_internal
        fc = self.face_center[:nIF]
        dP = _norm3(fc - self.cell_center[self.owner[:nIF]])
        dN = _norm3(fc - self.cell_center[self.neighbour[:nIF]])
        s = dP + dN
        with np.errstate(divide="ignore", invalid="ignore"):
            w = np.where(s > 1e-30, dN / s, 0.5)
        self.face_weight = np.full(self.n_faces(), 0.5)
        self.face_weight[:nIF] = w

    def _compute_cell_centers_and_volumes(self) -> None:
        """Mesh::computeCellCentersAndVolumes (core/src/Mesh.cpp:269-298): the
        centre is the running sum of face centres in the cell's face order
        divided by the face count; the volume is |sum sign*Sf.(cf-cC)|/3."""
        nC = self.n_cells() if self.cell_volume.size else self.cell_face_offset.size - 1
        off = self.cell_face_offset
        counts = np.diff(off)
        maxf = int(counts.max()) if nC else 0
        ctr = np.zeros((nC, 3))
        for j in range(maxf):
            has = counts > j
            fidx = self.cell_faces[off[:-1][has] + j]
            ctr[has] = ctr[has] + self.face_center[fidx]
        ctr = ctr / counts[:, None].astype(np.float64)
        vol = np.zeros(nC)
        cells = np.arange(nC)
        for j in range(maxf):
            has = counts > j
            fidx = self.cell_faces[off[:-1][has] + j]
            sf = self.face_normal[fidx] * self.face_area[fidx][:, None]
            rel = self.face_center[fidx] - ctr[has]
            dot = sf[:, 0] * rel[:, 0] + sf[:, 1] * rel[:, 1] + sf[:, 2] * rel[:, 2]
            sign = np.where(self.owner[fidx] == cells[has], 1.0, -1.0)
            vol[has] = vol[has] + sign * dot
        vol = np.abs(vol) / 3.0
        vol[vol < 1e-30] = 1e-20
        self.cell_center = ctr
        self.cell_volume = vol

    def compute_geometry(self) -> None:
        """Mesh::computeGeometry (core/src/Mesh.cpp:331-342)."""
        self._compute_cell_centers_and_volumes()
        self._compute_face_geometry()
        self._compute_interpolation_weights()

    def compute_wall_distance(self, chunk: int = 1 << 22, device: bool = False) -> None:
        """Mesh::computeWallDistance (core/src/Mesh.cpp:345-373): brute-force
        minimum over the wall-patch face centres of |c - wp|, 1e10 without walls.
        device=True runs the same O(n_cells * n_wall) search on the GPU
        (btm_wall_distance, bit-identical)."""
        wall = [p[2] for p in self.patches if p[1] == "wall"]
        nC = self.n_cells()
        if not wall or sum(w.size for w in wall) == 0:
            self.wall_dist = np.full(nC, 1e10)
            return
        wp = self.face_center[np.concatenate(wall)]
        if device:
            import ctypes as C
            from ._lib import check, dptr, lib
            cc = np.ascontiguousarray(self.cell_center, np.float64)
            wpc = np.ascontiguousarray(wp, np.float64)
            out = np.empty(nC)
            L = lib()
            L.btm_wall_distance.argtypes = [C.c_int32, C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]
            check(L.btm_wall_distance(nC, dptr(cc), wpc.shape[0], dptr(wpc), dptr(out)))
            self.wall_dist = out
            return
        out = np.empty(nC)
        step = max(1, chunk // max(1, wp.shape[0]))
        for s in range(0, nC, step):
            cc = self.cell_center[s:s + step]
            dx = cc[:, None, 0] - wp[None, :, 0]
            dy = cc[:, None, 1] - wp[None, :, 1]
            dz = cc[:, None, 2] - wp[None, :, 2]
            out[s:s + step] = np.sqrt(dx * dx + dy * dy + dz * dz).min(axis=1)
        self.wall_dist = out

    # ---- renumbering -----------------------------------------------------
    def permuted(self, perm: Sequence[int]) -> "Mesh":
        """Relabel cells: old cell c becomes cell perm[c].  Faces keep their
        order (internal first), owner/neighbour roles and patch face order;
        only the cell ids in owner/neighbour and the cell arrays move."""
        perm = np.asarray(perm, dtype=np.int64)
        nC = self.n_cells()
        if perm.shape != (nC,) or not np.array_equal(np.sort(perm), np.arange(nC)):
            raise ValueError("perm must be a permutation of range(n_cells)")
        m = Mesh()
        m.owner = perm[self.owner].astype(np.int32)
        nb = self.neighbour.copy()
        nb[nb >= 0] = perm[nb[nb >= 0]]
        m.neighbour = nb.astype(np.int32)
        for name in ("face_patch", "face_center", "face_normal", "face_area", "face_delta",
                     "face_d", "face_weight", "nodes"):
            setattr(m, name, getattr(self, name).copy())
        m.patches = [(n, t, f.copy()) for (n, t, f) in self.patches]
        m.n_internal = self.n_internal
        inv = np.empty(nC, np.int64)
        inv[perm] = np.arange(nC)
        m.cell_center = self.cell_center[inv]
        m.cell_volume = self.cell_volume[inv]
        counts = np.diff(self.cell_face_offset)[inv]
        m.cell_face_offset = np.zeros(nC + 1, np.int32)
        np.cumsum(counts, out=m.cell_face_offset[1:])
        m.cell_faces = np.concatenate(
            [self.cell_faces[self.cell_face_offset[c]:self.cell_face_offset[c + 1]] for c in inv]
        ).astype(np.int32) if nC else np.zeros(0, np.int32)
        if self.wall_dist is not None:
            m.wall_dist = self.wall_dist[inv]
        return m

    # ---- MSH1 binary format (core/src/Mesh.cpp:602-713) -----------------
    def save_binary(self, path: str) -> None:
        nC, nF, nN, nP = self.n_cells(), self.n_faces(), self.n_nodes(), self.n_patches()
        face_dt = np.dtype([("o", "<i4"), ("n", "<i4"), ("p", "<i4"), ("c", "<f8", 3),
                            ("nrm", "<f8", 3), ("a", "<f8"), ("dl", "<f8"), ("d", "<f8", 3),
                            ("w", "<f8")])
        fr = np.empty(nF, face_dt)
        fr["o"], fr["n"], fr["p"] = self.owner, self.neighbour, self.face_patch
        fr["c"], fr["nrm"], fr["a"] = self.face_center, self.face_normal, self.face_area
        fr["dl"], fr["d"], fr["w"] = self.face_delta, self.face_d, self.face_weight
        with open(path, "wb") as fh:
            fh.write(struct.pack("<I5i", MSH1_MAGIC, nC, nF, nN, nP, self.n_internal))
            fh.write(np.ascontiguousarray(self.nodes, "<f8").tobytes())
            fh.write(fr.tobytes())
            counts = np.diff(self.cell_face_offset)
            uniform = nC > 0 and np.all(counts == counts[0])
            if uniform:
                k = int(counts[0])
                cdt = np.dtype([("c", "<f8", 3), ("v", "<f8"), ("nf", "<i4"), ("f", "<i4", k)])
                cr = np.empty(nC, cdt)
                cr["c"], cr["v"], cr["nf"] = self.cell_center, self.cell_volume, k
                cr["f"] = self.cell_faces.reshape(nC, k)
                fh.write(cr.tobytes())
            else:
                for c in range(nC):
                    a, b = self.cell_face_offset[c], self.cell_face_offset[c + 1]
                    fh.write(np.asarray(self.cell_center[c], "<f8").tobytes())
                    fh.write(struct.pack("<di", self.cell_volume[c], b - a))
                    fh.write(np.asarray(self.cell_faces[a:b], "<i4").tobytes())
            for name, ptype, faces in self.patches:
                nb, tb = name.encode(), ptype.encode()
                fh.write(struct.pack("<i", len(nb)) + nb + struct.pack("<i", len(tb)) + tb)
                fh.write(struct.pack("<i", faces.size))
                fh.write(np.asarray(faces, "<i4").tobytes())

    @staticmethod
    def _load_binary(path: str) -> "Mesh":
        with open(path, "rb") as fh:
            buf = fh.read()
        magic, nC, nF, nN, nP, nIF = struct.unpack_from("<I5i", buf, 0)
        if magic != MSH1_MAGIC:
            raise RuntimeError("Invalid binary mesh magic number")
        pos = 24
        m = Mesh()
        m.nodes = np.frombuffer(buf, "<f8", nN * 3, pos).reshape(nN, 3).copy()
        pos += nN * 24
        face_dt = np.dtype([("o", "<i4"), ("n", "<i4"), ("p", "<i4"), ("c", "<f8", 3),
                            ("nrm", "<f8", 3), ("a", "<f8"), ("dl", "<f8"), ("d", "<f8", 3),
                            ("w", "<f8")])
        fr = np.frombuffer(buf, face_dt, nF, pos)
        pos += nF * face_dt.itemsize
        m.owner, m.neighbour, m.face_patch = (fr["o"].astype(np.int32), fr["n"].astype(np.int32),
                                              fr["p"].astype(np.int32))
        m.face_center, m.face_normal = fr["c"].copy(), fr["nrm"].copy()
        m.face_area, m.face_delta = fr["a"].copy(), fr["dl"].copy()
        m.face_d, m.face_weight = fr["d"].copy(), fr["w"].copy()
        m.n_internal = nIF
        cc = np.empty((nC, 3))
        cv = np.empty(nC)
        off = np.zeros(nC + 1, np.int32)
        flist = []
        for c in range(nC):
            cc[c] = np.frombuffer(buf, "<f8", 3, pos)
            cv[c], k = struct.unpack_from("<di", buf, pos + 24)
            pos += 36
            flist.append(np.frombuffer(buf, "<i4", k, pos))
            pos += 4 * k
            off[c + 1] = off[c] + k
        m.cell_center, m.cell_volume, m.cell_face_offset = cc, cv, off
        m.cell_faces = (np.concatenate(flist).astype(np.int32) if flist else np.zeros(0, np.int32))
        for _ in range(nP):
            (ln,) = struct.unpack_from("<i", buf, pos)
            name = buf[pos + 4:pos + 4 + ln].decode()
            pos += 4 + ln
            (lt,) = struct.unpack_from("<i", buf, pos)
            ptype = buf[pos + 4:pos + 4 + lt].decode()
            pos += 4 + lt
            (k,) = struct.unpack_from("<i", buf, pos)
            faces = np.frombuffer(buf, "<i4", k, pos + 4).astype(np.int32)
            pos += 4 + 4 * k
            m.patches.append((name, ptype, faces))
        return m

    @staticmethod
    def load_from_file(path: str) -> "Mesh":
        """Mesh::loadFromFile (core/src/Mesh.cpp:21-47): '.msh' is MSH1; an
        OpenFOAM polyMesh directory is read by the ASCII polyMesh reader."""
        if os.path.isdir(path):
            from ._foam import load_openfoam
            if os.path.exists(os.path.join(path, "points")) and os.path.exists(os.path.join(path, "faces")):
                return load_openfoam(path)
            pm = os.path.join(path, "constant", "polyMesh")
            if os.path.exists(os.path.join(pm, "points")):
                return load_openfoam(pm)
            raise RuntimeError("Cannot find polyMesh in: " + path)
        ext = os.path.splitext(path)[1]
        if ext in (".foam", ""):
            from ._foam import load_openfoam
            return load_openfoam(path)
        if ext == ".msh":
            return Mesh._load_binary(path)
        raise RuntimeError("Unknown mesh format: " + ext)

    # ---- reference factories ---------------------------------------------
    @staticmethod
    def _rect_channel(nx: int, ny: int, Lx: float, Ly: float, xc, yc, top_type: str = "wall") -> "Mesh":
        """Face/cell construction shared by makeChannel2D (both overloads) and
        makePlate2D (core/src/Mesh.cpp:719-870, 880-1059, 1063-1277)."""
        dz = 1.0
        xc = np.asarray(xc, dtype=np.float64)
        yc = np.asarray(yc, dtype=np.float64)
        b = _Builder(nx * ny)
        I, J = np.meshgrid(np.arange(nx), np.arange(ny - 1))
        I, J = I.ravel(), J.ravel()
        b.add(J * nx + I, (J + 1) * nx + I,
              np.stack([0.5 * (xc[I] + xc[I + 1]), yc[J + 1], np.full(I.size, 0.5 * dz)], 1),
              (0.0, 1.0, 0.0), (xc[I + 1] - xc[I]) * dz)
        I, J = np.meshgrid(np.arange(nx - 1), np.arange(ny))
        I, J = I.ravel(), J.ravel()
        b.add(J * nx + I, J * nx + I + 1,
              np.stack([xc[I + 1], 0.5 * (yc[J] + yc[J + 1]), np.full(I.size, 0.5 * dz)], 1),
              (1.0, 0.0, 0.0), (yc[J + 1] - yc[J]) * dz)
        i = np.arange(nx)
        b.add_patch("bottom", "wall", i,
                    np.stack([0.5 * (xc[i] + xc[i + 1]), np.zeros(nx), np.full(nx, 0.5 * dz)], 1),
                    (0.0, -1.0, 0.0), (xc[i + 1] - xc[i]) * dz)
        b.add_patch("top", top_type, (ny - 1) * nx + i,
                    np.stack([0.5 * (xc[i] + xc[i + 1]), np.full(nx, Ly), np.full(nx, 0.5 * dz)], 1),
                    (0.0, 1.0, 0.0), (xc[i + 1] - xc[i]) * dz)
        j = np.arange(ny)
        b.add_patch("inlet", "inlet", j * nx,
                    np.stack([np.zeros(ny), 0.5 * (yc[j] + yc[j + 1]), np.full(ny, 0.5 * dz)], 1),
                    (-1.0, 0.0, 0.0), (yc[j + 1] - yc[j]) * dz)
        b.add_patch("outlet", "outlet", j * nx + nx - 1,
                    np.stack([np.full(ny, Lx), 0.5 * (yc[j] + yc[j + 1]), np.full(ny, 0.5 * dz)], 1),
                    (1.0, 0.0, 0.0), (yc[j + 1] - yc[j]) * dz)
        m = b.finish()
        I, J = np.meshgrid(np.arange(nx), np.arange(ny))
        I, J = I.ravel(), J.ravel()
        m.cell_center = np.stack([0.5 * (xc[I] + xc[I + 1]), 0.5 * (yc[J] + yc[J + 1]),
                                  np.full(I.size, 0.5 * dz)], 1)
        m.cell_volume = (xc[I + 1] - xc[I]) * (yc[J + 1] - yc[J]) * dz
        m.nodes = _plane_nodes(xc, yc, dz)
        m._compute_face_geometry()
        m._compute_interpolation_weights()
        return m

    @staticmethod
    def make_channel_2d(nx: int, ny: int, Lx: float, Ly: float, Re: Optional[float] = None,
                        yPlusTarget: float = 1.0) -> "Mesh":
        """Mesh::makeChannel2D, both overloads (core/src/Mesh.cpp:719, 1063)."""
        xc = [Lx * i / nx for i in range(nx + 1)]
        if Re is None:
            yc = _tanh_nodes(Ly, ny, 2.0)
        else:
            Cf = 0.058 * math.pow(Re, -0.2)
            u_tau = math.sqrt(Cf / 2.0)
            nu = (Ly / 2.0) / Re
            y1_target = yPlusTarget * nu / u_tau
            stretch = _bisect_tanh_stretch(Ly, ny, y1_target, 0.0)
            if stretch > 1e-12:
                yc = _tanh_nodes(Ly, ny, stretch)
            else:
                yc = np.array([Ly * j / ny for j in range(ny + 1)])
        return Mesh._rect_channel(nx, ny, Lx, Ly, xc, yc)

    @staticmethod
    def make_plate_2d(nx: int, ny: int, Lx: float, Ly: float, Re: float,
                      y_plus_target: float = 1.0) -> "Mesh":
        """Mesh::makePlate2D (core/src/Mesh.cpp:880-1059): geometric growth from
        the wall, far-field 'top' patch of type 'patch'."""
        Cf = 0.058 * math.pow(Re, -0.2)
        u_tau = math.sqrt(Cf / 2.0)
        nu = (Ly / 2.0) / Re
        y1_target = y_plus_target * nu / u_tau
        y1_uniform = Ly / ny
        ratio = 1.0
        if y1_target < y1_uniform:
            def total(r):
                return y1_target * (math.pow(r, ny) - 1.0) / (r - 1.0)
            r_lo, r_hi = 1.0 + 1e-9, 1.5
            if total(r_hi) < Ly:
                ratio = r_hi
            else:
                for _ in range(200):
                    r_mid = 0.5 * (r_lo + r_hi)
                    if total(r_mid) < Ly:
                        r_lo = r_mid
                    else:
                        r_hi = r_mid
                    if r_hi - r_lo < 1e-12:
                        break
                ratio = 0.5 * (r_lo + r_hi)
        yc = np.zeros(ny + 1)
        if ratio > 1.0 + 1e-9:
            h = y1_target
            for j in range(1, ny + 1):
                yc[j] = yc[j - 1] + h
                h *= ratio
            scale = Ly / yc[ny]
            for j in range(1, ny + 1):
                yc[j] *= scale
        else:
            for j in range(ny + 1):
                yc[j] = Ly * j / ny
        xc = [Lx * i / nx for i in range(nx + 1)]
        return Mesh._rect_channel(nx, ny, Lx, Ly, xc, yc, top_type="patch")

    @staticmethod
    def make_backward_facing_step_2d(nx_up: int, nx_down: int, ny_up: int, ny_down: int,
                                     Lu: float, Ld: float, h_s: float, H: float,
                                     Re: float = 0.0, yPlusTarget: float = 1.0) -> "Mesh":
        """Mesh::makeBackwardFacingStep2D (core/src/Mesh.cpp:1280-1547).  The
        8-argument form is Re = 0 (fixed tanh stretch 2)."""
        nx_tot = nx_up + nx_down
        dz = 1.0
        H_up = H - h_s
        xc = np.zeros(nx_tot + 1)
        for i in range(nx_up + 1):
            xc[i] = -Lu + Lu * i / nx_up
        for i in range(1, nx_down + 1):
            xc[nx_up + i] = Ld * i / nx_down

        def stretch_for(extent, n):
            if Re > 0:
                Cf = 0.058 * math.pow(Re, -0.2)
                u_tau = math.sqrt(Cf / 2.0)
                nu = extent / Re
                y1t = yPlusTarget * nu / u_tau
                return _bisect_tanh_stretch(extent, n, y1t, 2.0)
            return 2.0

        s_up = stretch_for(H_up, ny_up)
        yu = np.empty(ny_up + 1)
        for j in range(ny_up + 1):
            eta = j / ny_up
            yu[j] = h_s + 0.5 * H_up * (1.0 + math.tanh(s_up * (2.0 * eta - 1.0)) / math.tanh(s_up))
        s_lo = stretch_for(h_s, ny_down)
        yl = np.empty(ny_down + 1)
        for j in range(ny_down + 1):
            eta = j / ny_down
            yl[j] = 0.5 * h_s * (1.0 + math.tanh(s_lo * (2.0 * eta - 1.0)) / math.tanh(s_lo))

        def cid_up(i, j):
            return j * nx_tot + i

        def cid_low(i, j):
            return nx_tot * ny_up + j * nx_down + i

        nC = nx_tot * ny_up + nx_down * ny_down
        b = _Builder(nC)
        half = 0.5 * dz
        I, J = (a.ravel() for a in np.meshgrid(np.arange(nx_tot), np.arange(ny_up - 1)))
        b.add(cid_up(I, J), cid_up(I, J + 1),
              np.stack([0.5 * (xc[I] + xc[I + 1]), yu[J + 1], np.full(I.size, half)], 1),
              (0.0, 1.0, 0.0), (xc[I + 1] - xc[I]) * dz)
        I, J = (a.ravel() for a in np.meshgrid(np.arange(nx_down), np.arange(ny_down - 1)))
        xa, xb = xc[nx_up + I], xc[nx_up + I + 1]
        b.add(cid_low(I, J), cid_low(I, J + 1),
              np.stack([0.5 * (xa + xb), yl[J + 1], np.full(I.size, half)], 1),
              (0.0, 1.0, 0.0), (xb - xa) * dz)
        i = np.arange(nx_down)
        xa, xb = xc[nx_up + i], xc[nx_up + i + 1]
        b.add(cid_up(nx_up + i, 0), cid_low(i, ny_down - 1),
              np.stack([0.5 * (xa + xb), np.full(nx_down, h_s), np.full(nx_down, half)], 1),
              (0.0, -1.0, 0.0), (xb - xa) * dz)
        I, J = (a.ravel() for a in np.meshgrid(np.arange(nx_tot - 1), np.arange(ny_up)))
        b.add(cid_up(I, J), cid_up(I + 1, J),
              np.stack([xc[I + 1], 0.5 * (yu[J] + yu[J + 1]), np.full(I.size, half)], 1),
              (1.0, 0.0, 0.0), (yu[J + 1] - yu[J]) * dz)
        I, J = (a.ravel() for a in np.meshgrid(np.arange(nx_down - 1), np.arange(ny_down)))
        b.add(cid_low(I, J), cid_low(I + 1, J),
              np.stack([xc[nx_up + I + 1], 0.5 * (yl[J] + yl[J + 1]), np.full(I.size, half)], 1),
              (1.0, 0.0, 0.0), (yl[J + 1] - yl[J]) * dz)
        i = np.arange(nx_tot)
        b.add_patch("top_wall", "wall", cid_up(i, ny_up - 1),
                    np.stack([0.5 * (xc[i] + xc[i + 1]), np.full(nx_tot, H), np.full(nx_tot, half)], 1),
                    (0.0, 1.0, 0.0), (xc[i + 1] - xc[i]) * dz)
        i = np.arange(nx_up)
        b.add_patch("bottom_wall_up", "wall", cid_up(i, 0),
                    np.stack([0.5 * (xc[i] + xc[i + 1]), np.full(nx_up, h_s), np.full(nx_up, half)], 1),
                    (0.0, -1.0, 0.0), (xc[i + 1] - xc[i]) * dz)
        j = np.arange(ny_down)
        b.add_patch("step_face", "wall", cid_low(0, j),
                    np.stack([np.zeros(ny_down), 0.5 * (yl[j] + yl[j + 1]), np.full(ny_down, half)], 1),
                    (-1.0, 0.0, 0.0), (yl[j + 1] - yl[j]) * dz)
        i = np.arange(nx_down)
        xa, xb = xc[nx_up + i], xc[nx_up + i + 1]
        b.add_patch("bottom_wall_down", "wall", cid_low(i, 0),
                    np.stack([0.5 * (xa + xb), np.zeros(nx_down), np.full(nx_down, half)], 1),
                    (0.0, -1.0, 0.0), (xb - xa) * dz)
        j = np.arange(ny_up)
        b.add_patch("inlet", "inlet", cid_up(0, j),
                    np.stack([np.full(ny_up, -Lu), 0.5 * (yu[j] + yu[j + 1]), np.full(ny_up, half)], 1),
                    (-1.0, 0.0, 0.0), (yu[j + 1] - yu[j]) * dz)
        ju, jl = np.arange(ny_up), np.arange(ny_down)
        b.add_patch("outlet", "outlet",
                    np.concatenate([cid_up(nx_tot - 1, ju), cid_low(nx_down - 1, jl)]),
                    np.concatenate([
                        np.stack([np.full(ny_up, Ld), 0.5 * (yu[ju] + yu[ju + 1]), np.full(ny_up, half)], 1),
                        np.stack([np.full(ny_down, Ld), 0.5 * (yl[jl] + yl[jl + 1]), np.full(ny_down, half)], 1)]),
                    (1.0, 0.0, 0.0),
                    np.concatenate([(yu[ju + 1] - yu[ju]) * dz, (yl[jl + 1] - yl[jl]) * dz]))
        m = b.finish()
        cc = np.zeros((nC, 3))
        cv = np.zeros(nC)
        I, J = (a.ravel() for a in np.meshgrid(np.arange(nx_tot), np.arange(ny_up)))
        c = cid_up(I, J)
        cc[c] = np.stack([0.5 * (xc[I] + xc[I + 1]), 0.5 * (yu[J] + yu[J + 1]), np.full(I.size, half)], 1)
        cv[c] = (xc[I + 1] - xc[I]) * (yu[J + 1] - yu[J]) * dz
        I, J = (a.ravel() for a in np.meshgrid(np.arange(nx_down), np.arange(ny_down)))
        c = cid_low(I, J)
        xa, xb = xc[nx_up + I], xc[nx_up + I + 1]
        cc[c] = np.stack([0.5 * (xa + xb), 0.5 * (yl[J] + yl[J + 1]), np.full(I.size, half)], 1)
        cv[c] = (xb - xa) * (yl[J + 1] - yl[J]) * dz
        m.cell_center, m.cell_volume = cc, cv
        m._compute_face_geometry()
        m._compute_interpolation_weights()
        return m

    @staticmethod
    def make_curved_channel_periodic_2d(x_nodes, y_bottom, y_top: float, ny: int, Re: float,
                                        yPlusTarget: float = 1.0) -> "Mesh":
        """Mesh::makeCurvedChannelPeriodic2D (core/src/Mesh.cpp:395-598)."""
        xN = np.asarray(x_nodes, dtype=np.float64).ravel()
        yB = np.asarray(y_bottom, dtype=np.float64).ravel()
        nx = xN.size - 1
        if nx < 3 or yB.size != nx + 1:
            raise RuntimeError("makeCurvedChannelPeriodic2D: need nx+1 x nodes and matching yBottom samples")
        if abs(yB[0] - yB[-1]) > 1e-12:
            raise RuntimeError("makeCurvedChannelPeriodic2D: yBottom must be periodic (first == last sample)")
        meanH = 0.0
        for i in range(nx + 1):
            meanH += (y_top - yB[i])
        meanH /= (nx + 1)
        stretch = 2.0
        if Re > 0:
            Cf = 0.058 * math.pow(Re, -0.2)
            u_tau = math.sqrt(Cf / 2.0)
            nu = meanH / Re
            y1t = yPlusTarget * nu / u_tau
            stretch = _bisect_tanh_stretch(meanH, ny, y1t, 2.0)
        eta = np.empty(ny + 1)
        for j in range(ny + 1):
            e = j / ny
            eta[j] = 0.5 * (1.0 + math.tanh(stretch * (2.0 * e - 1.0)) / math.tanh(stretch))
        Y = yB[:, None] + (y_top - yB[:, None]) * eta[None, :]
        return periodic_quad_mesh(xN, Y, ("bottom_wall", "wall"), ("top_wall", "wall"))

    # ---- factories with no reference counterpart (workload meshes) -------
    @staticmethod
    def make_channel_periodic_geometric(nx: int, ny: int, Lx: float = 1.0, h: float = 1.0,
                                        ratio: float = 1.08) -> "Mesh":
        """Flat streamwise-periodic plane channel, y in [0, 2h], ny cells with
        geometric growth `ratio` from each wall (ny even, ny/2 per half).  Wrap
        faces are internal faces with periodic-image geometry, built by the same
        construction as makeCurvedChannelPeriodic2D (flat bottom).  Patches:
        bottom_wall, top_wall (type wall)."""
        if ny % 2:
            raise ValueError("ny must be even")
        half = ny // 2
        yh = _geometric_half(half, h, ratio)
        y = np.concatenate([yh, 2.0 * h - yh[::-1][1:]])
        xN = np.array([Lx * i / nx for i in range(nx + 1)])
        Y = np.broadcast_to(y[None, :], (nx + 1, ny + 1)).copy()
        return periodic_quad_mesh(xN, Y, ("bottom_wall", "wall"), ("top_wall", "wall"))

    @staticmethod
    def make_square_duct_periodic_3d(nx: int, ny: int, nz: int, Lx: float = 10.0,
                                     side: float = 2.0, ratio: float = 1.05) -> "Mesh":
        """Streamwise(x)-periodic square duct, cross-section [0,side]^2, hex
        cells with geometric growth `ratio` from all four walls.  Internal faces:
        x-normal (incl. one wrap column with periodic-image geometry), then
        y-normal, then z-normal; patches: bottom_wall, top_wall, side_wall_lo,
        side_wall_hi (all walls)."""
        return duct_mesh(nx, ny, nz, Lx, side, ratio)


def _plane_nodes(xc, yc, dz):
    xc = np.asarray(xc, dtype=np.float64)
    yc = np.asarray(yc, dtype=np.float64)
    X, Y = np.meshgrid(xc, yc)
    pts = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1)
    back = pts.copy()
    back[:, 2] = dz
    return np.concatenate([pts, back])


def _geometric_half(n_half: int, h: float, ratio: float) -> np.ndarray:
    y1 = h * (ratio - 1.0) / (math.pow(ratio, n_half) - 1.0) if ratio != 1.0 else h / n_half
    yh = np.zeros(n_half + 1)
    step = y1
    for j in range(1, n_half + 1):
        yh[j] = yh[j - 1] + step
        step *= ratio
    yh = yh * (h / yh[n_half])
    yh[n_half] = h
    return yh


def periodic_quad_mesh(xN: np.ndarray, Y: np.ndarray, bottom=("bottom_wall", "wall"),
                       top=("top_wall", "wall")) -> Mesh:
    """Streamwise-periodic terrain-following quad mesh with node heights
    Y[i, j] (i over the nx+1 x nodes, j over ny+1 rows).  Geometry and face
    order follow makeCurvedChannelPeriodic2D (core/src/Mesh.cpp:446-598):
    exact shoelace centroids/areas, vertical internal faces, one wrap column
    whose d/delta/weight use the neighbour's periodic image, horizontal internal
    faces, then the bottom and top wall patches."""
    nx = xN.size - 1
    ny = Y.shape[1] - 1
    dz = 1.0
    Lx = xN[-1] - xN[0]
    nC = nx * ny
    I, J = (a.ravel() for a in np.meshgrid(np.arange(nx), np.arange(ny)))
    px = [xN[I], xN[I + 1], xN[I + 1], xN[I]]
    py = [Y[I, J], Y[I + 1, J], Y[I + 1, J + 1], Y[I, J + 1]]
    A2 = np.zeros(nC)
    cxA = np.zeros(nC)
    cyA = np.zeros(nC)
    for kv in range(4):
        kn = (kv + 1) % 4
        cross = px[kv] * py[kn] - px[kn] * py[kv]
        A2 = A2 + cross
        cxA = cxA + (px[kv] + px[kn]) * cross
        cyA = cyA + (py[kv] + py[kn]) * cross
    A = 0.5 * A2
    cc = np.zeros((nC, 3))
    cid = J * nx + I
    cc[cid, 0] = cxA / (6.0 * A)
    cc[cid, 1] = cyA / (6.0 * A)
    cc[cid, 2] = 0.5 * dz
    cv = np.zeros(nC)
    cv[cid] = np.abs(A) * dz

    def edge(x0, y0, x1, y1, plus_x):
        ex, ey = x1 - x0, y1 - y0
        ln = np.sqrt(ex * ex + ey * ey)
        center = np.stack([0.5 * (x0 + x1), 0.5 * (y0 + y1), np.full(np.size(x0), 0.5 * dz)], 1)
        area = ln * dz
        if plus_x:
            normal = np.stack([ey / ln, -ex / ln, np.zeros(np.size(x0))], 1)
        else:
            normal = np.stack([-ey / ln, ex / ln, np.zeros(np.size(x0))], 1)
        return center, normal, area

    b = _Builder(nC)
    # vertical internal faces: j outer, i inner (i < nx-1)
    I, J = (a.ravel() for a in np.meshgrid(np.arange(nx - 1), np.arange(ny)))
    c, n, a = edge(xN[I + 1], Y[I + 1, J], xN[I + 1], Y[I + 1, J + 1], True)
    fv = b.add(J * nx + I, J * nx + I + 1, c, n, a)
    # wrap faces
    j = np.arange(ny)
    c, n, a = edge(np.full(ny, xN[nx]), Y[nx, j], np.full(ny, xN[nx]), Y[nx, j + 1], True)
    fw = b.add(j * nx + nx - 1, j * nx, c, n, a)
    # horizontal internal faces
    I, J = (a_.ravel() for a_ in np.meshgrid(np.arange(nx), np.arange(ny - 1)))
    c, n, a = edge(xN[I], Y[I, J + 1], xN[I + 1], Y[I + 1, J + 1], False)
    fh = b.add(J * nx + I, (J + 1) * nx + I, c, n, a)
    i = np.arange(nx)
    c, n, a = edge(xN[i], Y[i, 0], xN[i + 1], Y[i + 1, 0], True)
    fb = b.add_patch(bottom[0], bottom[1], i, c, n, a)
    c, n, a = edge(xN[i], Y[i, ny], xN[i + 1], Y[i + 1, ny], False)
    ft = b.add_patch(top[0], top[1], (ny - 1) * nx + i, c, n, a)
    m = b.finish()
    m.cell_center, m.cell_volume = cc, cv
    nF = m.n_faces()
    d = np.zeros((nF, 3))
    delta = np.zeros(nF)
    w = np.full(nF, 0.5)
    fc = m.face_center

    def set_dw(fidx, cO, cN):
        dd = cN - cO
        d[fidx] = dd
        delta[fidx] = np.maximum(_norm3(dd), 1e-20)
        dP = _norm3(fc[fidx] - cO)
        dN = _norm3(fc[fidx] - cN)
        s = dP + dN
        w[fidx] = np.where(s > 1e-30, dN / np.where(s > 1e-30, s, 1.0), 0.5)

    for fidx in (fv, fh):
        set_dw(fidx, cc[m.owner[fidx]], cc[m.neighbour[fidx]])
    img = cc[m.neighbour[fw]].copy()
    img[:, 0] = img[:, 0] + Lx
    set_dw(fw, cc[m.owner[fw]], img)
    for fidx in (fb, ft):
        dd = fc[fidx] - cc[m.owner[fidx]]
        d[fidx] = dd
        delta[fidx] = np.maximum(_norm3(dd), 1e-20)
    m.face_d, m.face_delta, m.face_weight = d, delta, w
    X = np.broadcast_to(xN[:, None], Y.shape)
    pts = np.stack([X.T.ravel(), Y.T.ravel(), np.zeros(X.size)], 1)
    back = pts.copy()
    back[:, 2] = dz
    m.nodes = np.concatenate([pts, back])
    return m


def duct_mesh(nx: int, ny: int, nz: int, Lx: float, side: float, ratio: float) -> Mesh:
    """Hexahedral x-periodic square duct (see Mesh.make_square_duct_periodic_3d).
    Cells are axis-aligned boxes: centre = box midpoint, volume = dx*dy*dz."""
    if ny % 2 or nz % 2:
        raise ValueError("ny and nz must be even")
    xN = np.array([Lx * i / nx for i in range(nx + 1)])
    hy = _geometric_half(ny // 2, 0.5 * side, ratio)
    yN = np.concatenate([hy, side - hy[::-1][1:]])
    hz = _geometric_half(nz // 2, 0.5 * side, ratio)
    zN = np.concatenate([hz, side - hz[::-1][1:]])
    nC = nx * ny * nz

    def cid(i, j, k):
        return (k * ny + j) * nx + i

    xm = 0.5 * (xN[:-1] + xN[1:])
    ym = 0.5 * (yN[:-1] + yN[1:])
    zm = 0.5 * (zN[:-1] + zN[1:])
    dx = xN[1:] - xN[:-1]
    dy = yN[1:] - yN[:-1]
    dzz = zN[1:] - zN[:-1]
    b = _Builder(nC)
    # x-normal internal faces (i < nx-1), then the wrap column
    K, J, I = (a.ravel() for a in np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx - 1), indexing="ij"))
    fx = b.add(cid(I, J, K), cid(I + 1, J, K),
               np.stack([xN[I + 1], ym[J], zm[K]], 1), (1.0, 0.0, 0.0), dy[J] * dzz[K])
    K, J = (a.ravel() for a in np.meshgrid(np.arange(nz), np.arange(ny), indexing="ij"))
    fw = b.add(cid(nx - 1, J, K), cid(0, J, K),
               np.stack([np.full(J.size, xN[nx]), ym[J], zm[K]], 1), (1.0, 0.0, 0.0), dy[J] * dzz[K])
    K, J, I = (a.ravel() for a in np.meshgrid(np.arange(nz), np.arange(ny - 1), np.arange(nx), indexing="ij"))
    fy = b.add(cid(I, J, K), cid(I, J + 1, K),
               np.stack([xm[I], yN[J + 1], zm[K]], 1), (0.0, 1.0, 0.0), dx[I] * dzz[K])
    K, J, I = (a.ravel() for a in np.meshgrid(np.arange(nz - 1), np.arange(ny), np.arange(nx), indexing="ij"))
    fz = b.add(cid(I, J, K), cid(I, J, K + 1),
               np.stack([xm[I], ym[J], zN[K + 1]], 1), (0.0, 0.0, 1.0), dx[I] * dy[J])
    K, I = (a.ravel() for a in np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij"))
    fb = b.add_patch("bottom_wall", "wall", cid(I, 0, K),
                     np.stack([xm[I], np.zeros(I.size), zm[K]], 1), (0.0, -1.0, 0.0), dx[I] * dzz[K])
    ft = b.add_patch("top_wall", "wall", cid(I, ny - 1, K),
                     np.stack([xm[I], np.full(I.size, side), zm[K]], 1), (0.0, 1.0, 0.0), dx[I] * dzz[K])
    J, I = (a.ravel() for a in np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij"))
    fs0 = b.add_patch("side_wall_lo", "wall", cid(I, J, 0),
                      np.stack([xm[I], ym[J], np.zeros(I.size)], 1), (0.0, 0.0, -1.0), dx[I] * dy[J])
    fs1 = b.add_patch("side_wall_hi", "wall", cid(I, J, nz - 1),
                      np.stack([xm[I], ym[J], np.full(I.size, side)], 1), (0.0, 0.0, 1.0), dx[I] * dy[J])
    m = b.finish()
    K, J, I = (a.ravel() for a in np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij"))
    c = cid(I, J, K)
    cc = np.zeros((nC, 3))
    cc[c] = np.stack([xm[I], ym[J], zm[K]], 1)
    cv = np.zeros(nC)
    cv[c] = dx[I] * dy[J] * dzz[K]
    m.cell_center, m.cell_volume = cc, cv
    nF = m.n_faces()
    d = np.zeros((nF, 3))
    delta = np.zeros(nF)
    w = np.full(nF, 0.5)
    fcen = m.face_center

    def set_dw(fidx, cO, cN):
        dd = cN - cO
        d[fidx] = dd
        delta[fidx] = np.maximum(_norm3(dd), 1e-20)
        dP = _norm3(fcen[fidx] - cO)
        dN = _norm3(fcen[fidx] - cN)
        s = dP + dN
        w[fidx] = dN / s

    for fidx in (fx, fy, fz):
        set_dw(fidx, cc[m.owner[fidx]], cc[m.neighbour[fidx]])
    img = cc[m.neighbour[fw]].copy()
    img[:, 0] = img[:, 0] + Lx
    set_dw(fw, cc[m.owner[fw]], img)
    for fidx in (fb, ft, fs0, fs1):
        dd = fcen[fidx] - cc[m.owner[fidx]]
        d[fidx] = dd
        delta[fidx] = np.maximum(_norm3(dd), 1e-20)
    m.face_d, m.face_delta, m.face_weight = d, delta, w
    return m
