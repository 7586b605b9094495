"""Error paths of the C ABI on a GPU context: every misuse returns a status (raised here as
WxError) and leaves the context usable; degenerate inputs are handled without faults."""
import numpy as np
import pytest
import torch

import woxel_gb300 as wx
from parity import compare, gpu_render, oracle_render, oracle_view

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sphere(cuda_ctx):
    topo = wx.Topology.sphere((0, 0, 0), 40.0, 3.0)
    return topo, oracle_view(topo), cuda_ctx.build_grid(topo)


def state(w=64, h=48, mode=3):
    return wx.state_build(eye=(0, 0, 150), target=(0, 0, 0), aspect=w / h, fovy=60.0, width=float(w), mode=mode)


def still_renders(ctx, view, grid):
    st = state()
    rg, hg = gpu_render(ctx, grid, st, 64, 48)
    ro, ho = oracle_render(view, st, 64, 48)
    compare(rg, hg, ro, ho, label="after an error")


def test_render_rejects_bad_arguments(cuda_ctx, sphere):
    _, view, grid = sphere
    out = torch.zeros(64 * 48 * 4 + 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(wx.WxError, match="too large"):
        cuda_ctx.render(grid, state(), 65536, 65536, out, None)      # 2^32 pixels
    with pytest.raises(wx.WxError, match="aligned"):
        cuda_ctx.render(grid, state(), 64, 48, out.data_ptr() + 1, None)
    hits = torch.zeros(64 * 48 * 32 + 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(wx.WxError, match="aligned"):
        cuda_ctx.render(grid, state(), 64, 48, out, hits.data_ptr() + 8)
    with pytest.raises(wx.WxError):
        cuda_ctx.render(grid, state(), 64, 48, None, None)
    still_renders(cuda_ctx, view, grid)


def test_frames_below_one_tile_write_nothing(cuda_ctx, sphere):
    _, _, grid = sphere
    for w, h in [(7, 48), (64, 3), (0, 0)]:
        out = torch.full((max(1, w * h) * 4,), 9, dtype=torch.uint8, device="cuda")
        cuda_ctx.render(grid, state(max(w, 1), max(h, 1)), w, h, out, None)
        torch.cuda.synchronize()
        assert (out.cpu().numpy() == 9).all()


def test_tuning_rejects_out_of_range_values(cuda_ctx, sphere):
    _, view, grid = sphere
    before = cuda_ctx.tuning
    for bad in [dict(kernel=3), dict(kernel=-1), dict(tile_width=12), dict(warps_per_block=0),
                dict(warps_per_block=9), dict(blocks_per_sm=-1), dict(blocks_per_sm=65), dict(tile_order=2),
                dict(tile_order=-1)]:
        with pytest.raises(wx.WxError, match="range"):
            cuda_ctx.set_tuning(**dict(before, **bad))
        assert cuda_ctx.tuning == before
    still_renders(cuda_ctx, view, grid)


def test_level_set_values_are_checked(cuda_ctx, sphere):
    topo, _, grid = sphere
    vals = topo.sphere_values((0, 0, 0), 40.0, 3.0)
    for band in (0.0, -1.0, float("nan"), float("inf")):
        with pytest.raises(wx.WxError, match="band"):
            grid.set_values(vals, band)
    with pytest.raises(ValueError):
        grid.set_values(vals[:-1], 3.0)


def test_malformed_view_is_rejected(cuda_ctx):
    topo = wx.Topology.from_voxels(np.array([[1, 2, 3], [200, 5, 9]], np.int32))
    view = topo.view()
    bad = dict(view)
    a4 = view["atlas"][1].copy()
    kids = np.unpackbits(view["kids4"].view(np.uint8), bitorder="little")
    slot = int(np.nonzero(kids)[0][0])  # a child slot of the first N4: its texel is the leaf index
    d = view["dims"][1][0]
    x, y, z = slot >> 8, (slot >> 4) & 15, slot & 15
    a4[(z * d + y) * d + x] = 10 ** 6  # child index far beyond the leaf count
    bad["atlas"] = [view["atlas"][0], a4, view["atlas"][2]]
    with pytest.raises(wx.WxError, match="out of range"):
        cuda_ctx.upload_view(bad)
    short = dict(view)
    short["dims"] = [view["dims"][0], view["dims"][1], (1, 1, 1)]
    with pytest.raises(wx.WxError):
        cuda_ctx.upload_view(short)


def test_empty_grid_on_both_build_paths(cuda_ctx):
    topo = wx.Topology.from_voxels(np.zeros((0, 3), np.int32))
    for gpu in (False, True):
        grid = cuda_ctx.build_grid(topo, gpu=gpu)
        assert grid.info["n3"] == 0
        rg, hg = gpu_render(cuda_ctx, grid, state(), 64, 48)
        assert (wx.hit_fields(hg)["state"] == 1).all()
