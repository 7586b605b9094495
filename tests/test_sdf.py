"""Product SDF + flattening (topology.cpp) against the oracle's literal compute_sdf/atlas restatement.

The oracle walks the tree like vdb345.rs:290-670 (get_voxel for cross-node neighbours);
the product sweeps each level with per-node halos. Masks, origins and all three
atlases must be identical word for word.
"""
import numpy as np
import pytest

import oracle as orc
import woxel_gb300 as wx


def compare_views(topo):
    pv = topo.view()
    ov = orc.Tree.from_masks(topo.masks()).view()
    for k in ("kids5", "vals5", "kids4", "vals4", "vals3", "origins"):
        np.testing.assert_array_equal(ov[k], pv[k], err_msg=k)
    for i in range(3):
        assert tuple(ov["dims"][i]) == tuple(pv["dims"][i])
        np.testing.assert_array_equal(ov["atlas"][i], pv["atlas"][i], err_msg=f"atlas {i}")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_sparse(seed):
    rng = np.random.default_rng(seed)
    compare_views(wx.Topology.from_voxels(rng.integers(-300, 300, size=(300, 3)).astype(np.int32)))


def test_dense_cluster():
    rng = np.random.default_rng(4)
    compare_views(wx.Topology.from_voxels(rng.integers(-20, 20, size=(2000, 3)).astype(np.int32)))


def test_node_boundaries():
    ijk = np.array([[-1, -1, -1], [0, 0, 0], [4095, 0, 0], [4096, 5, 5], [-4097, 3, 3], [127, 127, 127],
                    [128, 128, 128], [-8, 7, -9]], np.int32)
    compare_views(wx.Topology.from_voxels(ijk))


def test_sphere_config1():
    topo = wx.Topology.sphere((0, 0, 0), 64.0, 3.0)
    assert topo.counts == (8, 8, 1706) and topo.active_voxels == 308214
    compare_views(topo)


def test_parallel_wavefront_equals_sequential_sweep():
    """The multi-threaded dependency-ordered sweep gives the single-threaded Gauss-Seidel result."""
    views = []
    for nthreads in (1, 8):
        topo = wx.Topology.spheres(count=150, rmin=4.0, rmax=30.0, lo=-300.0, hi=300.0, band=3.0, seed=7)
        assert topo.counts[2] > 5000  # takes the parallel path
        topo.sdf(nthreads)
        views.append(topo.atlas())
    for i in range(3):
        np.testing.assert_array_equal(views[0][0][i], views[1][0][i], err_msg=f"atlas {i}")


def test_active_tiles_count_as_empty():
    """Value-mask bits on N4/N5 slots (active tiles) are tiles for the SDF but hits for the march."""
    topo = wx.Topology.from_voxels(np.array([[3, 3, 3], [300, 40, 40]], np.int32))
    m = topo.masks()
    m["vals4"][0] |= 1 << 9   # an active N3-sized tile in the first N4
    m["vals5"][0] |= 1 << 20  # an active N4-sized tile in the first N5
    compare_views(wx.Topology.from_masks(m))


def test_from_masks_round_trip_and_validation():
    topo = wx.Topology.sphere((10, -20, 30), 20.0, 2.0)
    m = topo.masks()
    again = wx.Topology.from_masks(m).masks()
    for k in m:
        np.testing.assert_array_equal(m[k], again[k])
    bad = dict(m)
    bad["vals3"] = m["vals3"][:-16]  # one leaf missing
    with pytest.raises(wx.WxError):
        wx.Topology.from_masks(bad)
