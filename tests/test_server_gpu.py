"""Serving (wx_server_*): continuous batching of render requests over resident grids.

Every result must be the same whether the request is rendered alone (wx_render) or
in the mix, split across time slices and sharing launches with other requests.
"""
import time

import numpy as np
import pytest

import woxel_gb300 as wx
from parity import dispatch_mask, gpu_render

pytestmark = pytest.mark.gpu

MB = 1 << 20


@pytest.fixture(scope="module")
def grids(cuda_ctx):
    rng = np.random.default_rng(9)
    return [cuda_ctx.build_grid(wx.Topology.sphere((0, 0, 0), 64.0, 3.0)),
            cuda_ctx.build_grid(wx.Topology.from_voxels(rng.integers(-300, 300, size=(4000, 3)).astype(np.int32)))]


def make_requests(n, seed, hits=True):
    rng = np.random.default_rng(seed)
    sizes = [(64, 48), (120, 64), (33, 17), (160, 120), (8, 4), (96, 96), (7, 3), (200, 52)]
    out = []
    for i in range(n):
        w, h = sizes[int(rng.integers(0, len(sizes)))]
        eye = tuple(float(x) for x in rng.uniform(-400, 400, 3))
        st = wx.state_build(eye=eye, target=(0, 0, 0), aspect=w / h, fovy=65.0, width=float(w),
                            mode=[3, 0, 1, 2, 4][i % 5])
        out.append(wx.Server.request(i % 2, st, w, h, hits=hits, user=i))
    return out


def check_against_alone(ctx, srv, grids, reqs, results):
    for res in results:
        assert res.status == 0
        q = reqs[res.user]
        rgba, hits = srv.fetch(res, hits=bool(q.want_hits))
        ra, ha = gpu_render(ctx, grids[q.grid_id], q.state, q.width, q.height)
        m = dispatch_mask(q.width, q.height)
        np.testing.assert_array_equal(rgba[m], ra[m], err_msg=f"request {res.user} rgba")
        if q.want_hits:
            np.testing.assert_array_equal(hits[m].view(np.uint8), ha[m].view(np.uint8),
                                          err_msg=f"request {res.user} hits")
        srv.release(res.ticket)


def drain(srv, n, timeout=60.0):
    got, t0 = [], time.time()
    while len(got) < n and time.time() - t0 < timeout:
        got.extend(srv.poll(64, wait_ms=20))
    assert len(got) == n, f"only {len(got)} of {n} results"
    return got


@pytest.mark.parametrize("slice_tiles,inflight", [(37, 3), (1000, 2), (0, 1)])
def test_results_same_alone_and_in_the_mix(cuda_ctx, grids, slice_tiles, inflight):
    srv = wx.Server(cuda_ctx, budget_bytes=256 * MB, max_inflight=inflight, slice_tiles=slice_tiles)
    for g in grids:
        srv.add_grid(g)
    reqs = make_requests(40, seed=slice_tiles)
    for q in reqs:
        srv.submit(q)
    results = drain(srv, len(reqs))
    check_against_alone(cuda_ctx, srv, grids, reqs, results)
    st = srv.stats
    assert st["completed"] == len(reqs) and st["arena_in_use"] == 0
    if slice_tiles == 37:
        assert st["launches"] > 5  # requests were split across slices and shared launches
    srv.close()


def test_fifo_mode_matches(cuda_ctx, grids):
    srv = wx.Server(cuda_ctx, budget_bytes=128 * MB, fifo=True)
    for g in grids:
        srv.add_grid(g)
    reqs = make_requests(12, seed=3)
    for q in reqs:
        srv.submit(q)
    results = drain(srv, len(reqs))
    check_against_alone(cuda_ctx, srv, grids, reqs, results)
    assert srv.stats["launches"] == sum(1 for q in reqs if (q.width // 8) * (q.height // 4) > 0)
    srv.close()


def test_budget_admission_waits_for_releases(cuda_ctx, grids):
    """An arena that holds about two requests still serves many, as results are released."""
    budget = grids[0].info["device_bytes"] + grids[1].info["device_bytes"] + 2 * (160 * 120 * 36 + 512)
    srv = wx.Server(cuda_ctx, budget_bytes=budget, slice_tiles=64)
    for g in grids:
        srv.add_grid(g)
    reqs = [wx.Server.request(i % 2, wx.state_build(eye=(200.0, 50.0 + i, 90.0), target=(0, 0, 0), aspect=4 / 3,
                                                    width=160.0), 160, 120, hits=True, user=i) for i in range(10)]
    with pytest.raises(wx.WxError):
        srv.submit(wx.Server.request(0, reqs[0].state, 4000, 3000))  # larger than the whole arena
    for q in reqs:
        srv.submit(q)
    done = []
    t0 = time.time()
    while len(done) < len(reqs) and time.time() - t0 < 60:
        for r in srv.poll(8, wait_ms=20):
            done.append(r)
            assert srv.stats["arena_in_use"] <= srv.stats["arena_bytes"]
            check_against_alone(cuda_ctx, srv, grids, reqs, [r])
    assert len(done) == len(reqs)
    srv.close()


def test_cancel_pending(cuda_ctx, grids):
    budget = grids[0].info["device_bytes"] + grids[1].info["device_bytes"] + 160 * 120 * 4 + 256
    srv = wx.Server(cuda_ctx, budget_bytes=budget)
    for g in grids:
        srv.add_grid(g)
    st = wx.state_build(eye=(150.0, 20.0, 80.0), target=(0, 0, 0), aspect=4 / 3, width=160.0)
    t1 = srv.submit(wx.Server.request(0, st, 160, 120, user=1))
    t2 = srv.submit(wx.Server.request(1, st, 160, 120, user=2))  # waits: the arena holds one result
    first = drain(srv, 1)
    assert first[0].ticket == t1 and first[0].status == 0
    assert srv.stats["pending"] == 1  # t1 is not released, so t2 cannot be admitted
    srv.cancel(t2)
    rest = drain(srv, 1)
    assert rest[0].ticket == t2 and rest[0].status == 7  # WX_ERR_CANCELLED
    with pytest.raises(wx.WxError):
        srv.cancel(t1)  # already rendered
    srv.release(t1)
    srv.release(t2)
    assert srv.stats["arena_in_use"] == 0
    srv.close()


def test_replay_open_loop(cuda_ctx, grids):
    srv = wx.Server(cuda_ctx, budget_bytes=512 * MB, slice_tiles=256)
    for g in grids:
        srv.add_grid(g)
    reqs = make_requests(60, seed=11, hits=False)
    rng = np.random.default_rng(1)
    arrivals = np.cumsum(rng.exponential(1 / 2000.0, size=len(reqs)))
    res = srv.replay(reqs, list(arrivals), release=True, timeout_s=60)
    lat = np.array([r.t_done - r.t_submit for r in res])
    assert all(r.status == 0 for r in res) and (lat > 0).all()
    assert srv.stats["arena_in_use"] == 0
    srv.close()
