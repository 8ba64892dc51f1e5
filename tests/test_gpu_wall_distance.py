"""Device wall distance (btm_wall_distance, Mesh.compute_wall_distance(device=True)):
bit-identical to the host brute force of Mesh::computeWallDistance
(core/src/Mesh.cpp:345-373) on 2-D, permuted and 3-D meshes."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["bfs_perm_1920", "chan180_4x32", "duct_4x16x16"])
def test_device_wall_distance_matches_host(name):
    g = cases.load_golden(name)
    m = cases.mesh_from_bytes(bytes(g["mesh"]))
    m.compute_wall_distance()
    host = m.wall_dist.copy()
    assert np.array_equal(host, g["wall_dist"])
    m.compute_wall_distance(device=True)
    assert np.array_equal(m.wall_dist, host)


def test_device_wall_distance_large_bfs():
    """The 122,880-cell backward-facing step with permuted cell ids."""
    from rans_sst_py import Mesh
    m = Mesh.make_backward_facing_step_2d(64, 384, 192, 96, 4.0, 30.0, 1.0, 3.0, 36000.0, 1.0)
    m = m.permuted(np.random.default_rng(7).permutation(m.n_cells()))
    m.compute_wall_distance()
    host = m.wall_dist.copy()
    m.compute_wall_distance(device=True)
    assert np.array_equal(m.wall_dist, host)
