"""Failure detection without a GPU fault (the reference panics instead: wgpu_context.rs:44-101).

* The GPU SDF build's bounded waits: with a wait limit of one poll, CTAs whose container is not
  ready give up, set the error flag and return; the build reports WX_ERR_TIMEOUT, creates no
  grid, and the context goes on working (the same build with the default limit succeeds and
  equals the host build).
"""
import numpy as np
import pytest

import woxel_gb300 as wx
from parity import compare, gpu_render, oracle_render, oracle_view

pytestmark = pytest.mark.gpu


def dense_block(n_leaves_side: int) -> wx.Topology:
    """A solid cube of fully active leaves: in the forward sweep only its first corner leaf is
    ready at the start, every other leaf waits for a neighbour."""
    k = np.arange(n_leaves_side) * 8 - 4 * n_leaves_side
    o = np.stack(np.meshgrid(k, k, k, indexing="ij"), -1).reshape(-1, 3).astype(np.int32)
    m = np.full((o.shape[0], 8), np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64)
    m[::3, 2] = 0  # some empty voxels, so the leaves carry distances
    return wx.Topology.from_leaves(o, m)


def test_sdf_wait_bound_expires_and_context_recovers(cuda_ctx):
    topo = dense_block(12)
    try:
        cuda_ctx.set_sdf_wait_limit(1)
        with pytest.raises(wx.WxError) as ei:
            cuda_ctx.build_grid(topo, gpu=True)
        assert ei.value.args[0] == 6 and "bound" in ei.value.args[1]  # WX_ERR_TIMEOUT
    finally:
        cuda_ctx.set_sdf_wait_limit(0)
    g_gpu = cuda_ctx.build_grid(topo, gpu=True)
    g_cpu = cuda_ctx.build_grid(topo)
    a, b = g_cpu.pools(), g_gpu.pools()
    for k in ("slot5", "slot4", "leaf", "ovf"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    st = wx.state_build(eye=(150.0, 90.0, 200.0), target=(0, 0, 0), aspect=4 / 3, fovy=60.0, width=128.0, mode=3)
    rg, hg = gpu_render(cuda_ctx, g_gpu, st, 128, 96)
    ro, ho = oracle_render(oracle_view(topo), st, 128, 96)
    compare(rg, hg, ro, ho, label="after the expired wait")
    g_gpu.release()
    g_cpu.release()
