"""GPU SDF build (wx_grid_build_gpu) against the host build (wx_grid_build): every device pool
word for word — N5/N4 slot words, leaf bytes and the leaf overflow table — so the GPU sweeps
reproduce the sequential Gauss-Seidel order of compute_sdf (vdb345.rs:290-670) exactly."""
import numpy as np
import pytest

import woxel_gb300 as wx
from parity import compare, gpu_render, oracle_render, oracle_view
from woxel_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def assert_same_pools(ctx, topo, label):
    g_cpu = ctx.build_grid(topo)
    g_gpu = ctx.build_grid(topo, gpu=True)
    a, b = g_cpu.pools(), g_gpu.pools()
    for k in ("slot5", "slot4", "leaf", "ovf"):
        assert a[k].shape == b[k].shape, f"{label}: {k} shape {a[k].shape} vs {b[k].shape}"
        bad = np.nonzero(a[k].reshape(-1) != b[k].reshape(-1))[0]
        assert bad.size == 0, f"{label}: {k} differs at {bad.size} words, first {bad[:5]}"
    assert g_cpu.info == g_gpu.info
    return g_cpu, g_gpu, a


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_sparse(cuda_ctx, seed):
    rng = np.random.default_rng(seed)
    topo = wx.Topology.from_voxels(rng.integers(-300, 300, size=(3000, 3)).astype(np.int32))
    assert_same_pools(cuda_ctx, topo, f"sparse{seed}")


def test_dense_cluster_and_node_boundaries(cuda_ctx):
    rng = np.random.default_rng(4)
    assert_same_pools(cuda_ctx, wx.Topology.from_voxels(rng.integers(-20, 20, size=(20000, 3)).astype(np.int32)),
                      "dense")
    ijk = np.array([[-1, -1, -1], [0, 0, 0], [4095, 0, 0], [4096, 5, 5], [-4097, 3, 3], [127, 127, 127],
                    [128, 128, 128], [-8, 7, -9], [-4096 * 3, 4096 * 2, 0]], np.int32)
    assert_same_pools(cuda_ctx, wx.Topology.from_voxels(ijk), "boundaries")


def test_active_tiles_and_far_root_keys(cuda_ctx):
    """Active tiles (value bits on N5/N4 slots) and N5 keys spread over a box too large for the
    root table (the neighbour lookup then scans the origins)."""
    topo = wx.Topology.from_voxels(np.array([[3, 3, 3], [300, 40, 40], [4096 * 1500, 4096 * 1500, 0]], np.int32))
    m = topo.masks()
    m["vals4"][0] |= 1 << 9
    m["vals5"][0] |= 1 << 20
    assert_same_pools(cuda_ctx, wx.Topology.from_masks(m), "tiles")


def test_sphere_renders_identically(cuda_ctx):
    topo = wx.Topology.sphere((0, 0, 0), 64.0, 3.0)
    _, g_gpu, _ = assert_same_pools(cuda_ctx, topo, "sphere64")
    st = wx.state_build(eye=(0, 0, 200), target=(0, 0, 0), aspect=4 / 3, fovy=60.0, width=160.0, mode=3)
    rg, hg = gpu_render(cuda_ctx, g_gpu, st, 160, 120)
    ro, ho = oracle_render(oracle_view(topo), st, 160, 120)
    compare(rg, hg, ro, ho, label="gpu-sdf sphere")


def test_leaf_distances_beyond_a_byte(cuda_ctx):
    """A solid 66^3 block of leaves with one active voxel: interior distances reach ~264, so the
    overflow table is filled on both paths and must agree entry for entry."""
    n = 66
    g = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3) * 8
    masks = np.zeros((g.shape[0], 8), np.uint64)
    masks[0, 0] = 1
    topo = wx.Topology.from_leaves(g.astype(np.int32), masks)
    _, _, pools = assert_same_pools(cuda_ctx, topo, "block66")
    assert pools["ovf"].shape[0] > 1000
    assert (pools["ovf"][:, 1] >= 255).all() and (np.diff(pools["ovf"][:, 0].astype(np.int64)) > 0).all()


def test_benchmark_grid(cuda_ctx):
    """The 2000-sphere benchmark grid (476k leaves)."""
    assert_same_pools(cuda_ctx, W.spheres_topology(), "spheres")
