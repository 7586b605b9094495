"""The reference's own known-answer tests, applied to the oracle and to the product's host code.

Sources: src/vdb/data_structure.rs:423-485 (coordinate maths) and
src/vdb/vdb345.rs:702-723 (set_voxel / get_voxel round trip).
"""
import numpy as np
import pytest

import oracle as orc
import woxel_gb300 as wx

# N3 = (LOG2_D 3, TOTAL 3), N4 = (4, 7), N5 = (5, 12)


def test_global_to_node_kat():  # data_structure.rs:423-437
    assert orc.global_to_node((-1, 0, 0), 3) == (-8, 0, 0)
    assert orc.global_to_node((-142, 2431, 102), 7) == (-256, 2304, 0)
    assert orc.global_to_node((-1, 0, -42141), 12) == (-4096, 0, -45056)


def test_mask_sizes_and_dims_kat():  # data_structure.rs:439-466
    assert (512 // 64, 4096 // 64, 32768 // 64) == (8, 64, 512)
    assert (1 << 3, 1 << 7, 1 << 12) == (8, 128, 4096)


def test_bit_index_kat():  # data_structure.rs:468-474
    assert orc.global_to_offset((0, 0, 0), 3, 3) == 0
    assert orc.global_to_offset((1, 2, 3), 3, 3) == 83
    assert orc.global_to_offset((121321, 212123, 3121), 4, 7) == 3382
    assert orc.global_to_offset((1, 2, 3), 5, 12) == 0


def test_child_offset_round_trip_kat():  # data_structure.rs:476-485
    for c in [(1, 2, 3), (15, 15, 0), (8, 9, 10)]:
        assert orc.offset_to_child(orc.child_to_offset(c, 4), 4) == c


def test_set_get_voxel_round_trip_kat():  # vdb345.rs:702-723
    pts = [(0, 0, 0), (123, 78, 3), (34, 123, 46), (102, 79, 28)]
    t = orc.Tree()
    for i, p in enumerate(pts):
        t.set_voxel(p, i)
    for i, p in enumerate(pts):
        kind, val, _ = t.get_voxel(p)
        assert kind == "Leaf" and val == i
    assert t.get_voxel((5000, 0, 0))[0] == "Bkgr"


def test_product_topology_matches_set_voxel():
    """The product's topology builder yields the same masks()/origins() as set_voxel."""
    rng = np.random.default_rng(7)
    ijk = rng.integers(-5000, 5000, size=(400, 3)).astype(np.int32)
    t = orc.Tree.from_voxels(ijk)
    om = t.masks()
    pm = wx.Topology.from_voxels(ijk).masks()
    for k in om:
        np.testing.assert_array_equal(om[k], pm[k], err_msg=k)


def test_compute_sdf_single_voxel():
    """vdb345.rs:725-741 runs compute_sdf on voxel (5,6,7) and prints leaf 0; pin the values it prints."""
    t = orc.Tree.from_voxels([(5, 6, 7)])
    v = t.view()
    a3, s3 = v["atlas"][2], v["dims"][2][0]
    leaf = np.array([a3[(z * s3 + y) * s3 + x] for x in range(8) for y in range(8) for z in range(8)]).reshape(8, 8, 8)
    # Chebyshev distance to (5,6,7) inside the leaf, except cells on a face shared with a missing
    # neighbour leaf see "1" through get_voxel (vdb345.rs:470-476).
    assert leaf[5, 6, 7] == 1  # active voxel texel = its value (set to 1 by the oracle)
    assert leaf[4, 6, 7] == 1 and leaf[5, 5, 6] == 1
    assert leaf[0, 0, 0] == 1  # corner cell borders missing leaves -> 1
    assert leaf[1, 1, 1] == 2  # interior: min over 26-neighbourhood chains
