"""OpenFOAM polyMesh ingest (Mesh.load_from_file on a polyMesh or case
directory) against the reference loader (Mesh::loadOpenFOAM,
core/src/Mesh.cpp:50-265): topology, face and cell geometry, interpolation
weights bit-identical to the reference's output on warped hex blocks
(tests/golden/foam_blocks.npz, written by the reference itself)."""
import os

import numpy as np
import pytest

import cases
from rans_sst_py import Mesh

KEYS = ("owner", "neighbour", "face_patch", "face_center", "face_normal", "face_area", "face_delta", "face_d",
        "face_weight", "cell_center", "cell_volume", "cell_face_offset", "cell_faces", "nodes")


@pytest.mark.parametrize("tag", ["b432", "b653"])
def test_polymesh_matches_reference_loader(tmp_path, tag):
    g = cases.load_golden("foam_blocks")
    nx, ny, nz, perturb, seed = g[f"{tag}_args"]
    poly = cases.write_polymesh_block(str(tmp_path / "constant" / "polyMesh"), int(nx), int(ny), int(nz),
                                      float(perturb), int(seed))
    for path in (poly, str(tmp_path)):                # a polyMesh directory, or its case directory
        m = Mesh.load_from_file(path)
        assert m.n_internal == int(g[f"{tag}_n_internal"])
        assert m.patch_names() == bytes(g[f"{tag}_patch_names"]).decode().split("\n")
        assert m.patch_types() == ["patch", "patch", "wall", "wall", "empty", "empty"]
        for k in KEYS:
            assert np.array_equal(getattr(m, k), g[f"{tag}_{k}"]), k


def test_polymesh_errors(tmp_path):
    with pytest.raises(RuntimeError, match="Cannot find polyMesh"):
        Mesh.load_from_file(str(tmp_path))
    poly = cases.write_polymesh_block(str(tmp_path / "pm"), 2, 2, 1)
    os.remove(os.path.join(poly, "neighbour"))
    with pytest.raises(RuntimeError, match="neighbour"):
        Mesh.load_from_file(poly)
