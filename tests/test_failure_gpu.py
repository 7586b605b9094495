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
        assert ei.value.status == 6 and "bound" in str(ei.value)  # WX_ERR_TIMEOUT
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


# ---------------------------------------------------------------------------
# Injected allocation failures: every call reports WX_ERR_OOM and leaves the
# context (or server) usable.
# ---------------------------------------------------------------------------
OOM = 3


def expect_oom(fn, *a, **kw):
    wx.inject_alloc_failures(1)
    try:
        with pytest.raises(wx.WxError) as ei:
            fn(*a, **kw)
        assert ei.value.status == OOM, str(ei.value)
    finally:
        wx.inject_alloc_failures(0)


def test_injected_allocation_failures(cuda_ctx):
    import torch

    topo = wx.Topology.sphere((0, 0, 0), 40.0, 3.0)
    expect_oom(cuda_ctx.build_grid, topo)
    expect_oom(cuda_ctx.build_grid, topo, gpu=True)
    grid = cuda_ctx.build_grid(topo)
    st = wx.state_build(eye=(0.0, 30.0, 150.0), target=(0, 0, 0), aspect=4 / 3, fovy=60.0, width=96.0, mode=3)
    # A fresh context has no staging buffer yet: pageable host outputs need one.
    other = wx.Context(0)
    rgba = np.zeros((72, 96, 4), np.uint8)
    hits = np.zeros((72, 96), wx.HIT_DTYPE)
    expect_oom(other.render, grid, st, 96, 72, rgba, hits)
    other.render(grid, st, 96, 72, rgba, hits)
    torch.cuda.synchronize()
    ra, ha = gpu_render(cuda_ctx, grid, st, 96, 72)
    np.testing.assert_array_equal(rgba, ra)
    np.testing.assert_array_equal(hits.view(np.uint8), ha.view(np.uint8))
    other.close()
    # Server: its slots at creation, its output arena at the first submission.
    expect_oom(wx.Server, cuda_ctx, budget_bytes=1 << 30)
    srv = wx.Server(cuda_ctx, budget_bytes=1 << 30)
    gid = srv.add_grid(grid)
    req = wx.Server.request(gid, st, 96, 72, user=5)
    expect_oom(srv.submit, req)
    srv.submit(req)
    res = []
    for _ in range(500):
        res += srv.poll(8, wait_ms=20)
        if res:
            break
    assert len(res) == 1 and res[0].status == 0
    got, _ = srv.fetch(res[0])
    np.testing.assert_array_equal(got, ra)
    srv.release(res[0].ticket)
    srv.close()
    grid.release()


# ---------------------------------------------------------------------------
# Cancelling admitted server requests, including one whose tiles are in a launch
# already running on the GPU (the batched kernel reads the cancel table before
# every tile).
# ---------------------------------------------------------------------------
def test_server_cancels_admitted_requests_mid_render(cuda_ctx):
    import time

    from woxel_gb300 import workloads as W

    grid = cuda_ctx.build_grid(W.spheres_topology())
    srv = wx.Server(cuda_ctx, budget_bytes=8 << 30, max_inflight=1, slice_tiles=1 << 20)
    gid = srv.add_grid(grid)
    eyes = wx.orbit_eyes(8, 3000.0, 77)
    reqs = []
    # 4K frames. The first submission starts a launch of its own; the next requests arrive
    # while it runs and share the second launch (about 1M tiles: requests 1-4 and the start
    # of 5), which runs for several milliseconds.
    for i in range(8):
        w, h = (3840, 2160) if i < 7 else (640, 480)
        st = wx.state_build(eye=tuple(float(x) for x in eyes[i]), target=(0, 0, 0), aspect=w / h, fovy=60.0,
                            width=float(w), mode=3)
        reqs.append(wx.Server.request(gid, st, w, h, user=i))
    tickets = [srv.submit(r) for r in reqs]
    t0 = time.time()
    while srv.stats["launches"] < 2 and time.time() - t0 < 10:
        pass
    srv.cancel(tickets[4])  # last request of the running launch: its tiles come last in its queue
    srv.cancel(tickets[6])  # in the next launch: dropped before it is launched
    got, t0 = [], time.time()
    while len(got) < 8 and time.time() - t0 < 60:
        got += srv.poll(16, wait_ms=20)
    assert len(got) == 8
    stats = srv.stats
    assert stats["cancelled"] == 2 and stats["completed"] == 6
    assert stats["tiles_cancelled_launched"] > 0, stats
    assert stats["tiles_cancelled_queued"] > 0, stats
    with pytest.raises(wx.WxError):
        srv.cancel(tickets[0])  # finished
    for res in got:
        if res.user in (4, 6):
            assert res.status == 7 and not res.rgba8  # WX_ERR_CANCELLED, no buffers
        else:
            assert res.status == 0
            q = reqs[res.user]
            rgba, _ = srv.fetch(res)
            ra, _ = gpu_render(cuda_ctx, grid, q.state, q.width, q.height, hits=False)
            np.testing.assert_array_equal(rgba, ra, err_msg=f"request {res.user}")
        srv.release(res.ticket)
    srv.close()
    grid.release()
