"""compute_sdf at the benchmark's sizes: the oracle's literal restatement of
vdb345.rs:290-670, run on grids the oracle generated itself, against the product's
parallel per-level sweep (topology.cpp) on the grids the product generated.

* the 2000-sphere grid (476,014 leaves, 3,037 N4, 8 N5): every word of the three
  atlases (N5, N4 and N3 skip distances and child indices, reference layout) equal;
* the [-2048,0)^3 octant of the 4096^3 noise grid (one N5, 367,660 leaves; the whole
  2.68M-leaf grid takes the single-threaded oracle several minutes): the same.

A product SDF bug that shows only on large grids would make these differ, while the
GPU-vs-oracle render tests (which can be handed either view) would not see it.
"""
import numpy as np

import oracle as orc
import woxel_gb300 as wx
from test_oracle_workloads import assert_masks_equal, first_n5_slice
from woxel_gb300 import workloads as W


def assert_views_equal(ov: dict, pv: dict):
    assert_masks_equal(ov, pv)
    for i in range(3):
        assert tuple(ov["dims"][i]) == tuple(pv["dims"][i])
        a, b = np.asarray(ov["atlas"][i]).ravel(), np.asarray(pv["atlas"][i]).ravel()
        assert a.size == b.size
        bad = np.flatnonzero(a != b)
        assert bad.size == 0, f"atlas {i}: {bad.size} words differ, first at {bad[:5]}"


def test_spheres_grid_sdf_oracle_equals_product(oracle_spheres_view):
    ov = oracle_spheres_view
    pv = W.spheres_topology().view()
    assert ov["dims"][2][0] == 632
    assert_views_equal(ov, pv)
    # the skip distances are not trivial: leaf-level tiles reach several voxels
    a3 = np.asarray(ov["atlas"][2])
    assert a3.max() >= 4


def test_noise_grid_octant_sdf_oracle_equals_product():
    ov = orc.workload_view("noise", box=(-2048, 0))
    pv = wx.Topology.from_masks(first_n5_slice(W.noise_topology().masks())).view()
    assert ov["vals3"].size // 16 == 367660
    assert_views_equal(ov, pv)
