"""Shared helpers for parity tests: render on the GPU through the C ABI and compare with the oracle.

Tolerances (stated by the path's contract): hit voxel ijk, node index, state,
level, step count and last-step mask bit-exact; hit t within 1e-5 relative;
RGBA8 within 1 LSB. The march position p is also compared bit-exactly.
"""
from __future__ import annotations

import numpy as np

import oracle as orc
import woxel_gb300 as wx

T_RTOL = 1e-5
RGBA_LSB = 1


def gpu_render(ctx, grid, state, width, height, hits=True, host=False):
    """Render one frame; device (torch) buffers by default, host numpy buffers with host=True."""
    if host:
        rgba = np.zeros((height, width, 4), np.uint8)
        h = np.zeros((height, width), wx.HIT_DTYPE) if hits else None
        ctx.render(grid, state, width, height, rgba, h)
        import torch

        torch.cuda.synchronize()
        return rgba, h
    import torch

    rgba_d = torch.zeros(height * width * 4, dtype=torch.uint8, device="cuda")
    hits_d = torch.zeros(height * width * 32, dtype=torch.uint8, device="cuda") if hits else None
    ctx.render(grid, state, width, height, rgba_d, hits_d, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    rgba = rgba_d.cpu().numpy().reshape(height, width, 4)
    h = hits_d.cpu().numpy().view(wx.HIT_DTYPE).reshape(height, width) if hits else None
    return rgba, h


def oracle_view(topo) -> dict:
    """The view the oracle renders for a product topology: its masks (the grid's input,
    which the oracle's own generators reproduce bit for bit) flattened by the oracle's
    compute_sdf and atlas(), so that no parity test hands the oracle the product's SDF."""
    return orc.Tree.from_masks(topo.masks()).view()


def oracle_render(view, state, width, height, nthreads=8, tiles=None):
    return orc.render(view, wx.state_bytes(state), width, height, nthreads=nthreads, hits=True, tiles=tiles)[:2]


def dispatch_mask(width, height):
    m = np.zeros((height, width), bool)
    m[: 4 * (height // 4), : 8 * (width // 8)] = True
    return m


def compare(rgba_g, hits_g, rgba_o, hits_o, where=None, label=""):
    """Assert parity; returns a summary dict. `where` selects the pixels to compare."""
    if where is None:
        where = dispatch_mask(rgba_g.shape[1], rgba_g.shape[0])
    hg, ho = hits_g[where], hits_o[where]
    fg, fo = wx.hit_fields(hg), wx.hit_fields(ho)
    for k in ("state", "level", "mask", "steps", "node", "shadow"):
        bad = np.nonzero(fg[k] != fo[k])[0]
        assert bad.size == 0, f"{label}: {k} differs at {bad.size} pixels, first {bad[:5]}: {fg[k][bad[:5]]} vs {fo[k][bad[:5]]}"
    np.testing.assert_array_equal(fg["ijk"], fo["ijk"], err_msg=f"{label}: ijk")
    pbits_g, pbits_o = hg["p"].view(np.uint32), ho["p"].view(np.uint32)
    p_exact = bool(np.array_equal(pbits_g, pbits_o))
    assert p_exact, f"{label}: march position p differs at {(pbits_g != pbits_o).any(-1).sum()} pixels"
    tg, to = hg["t"].astype(np.float64), ho["t"].astype(np.float64)
    np.testing.assert_allclose(tg, to, rtol=T_RTOL, atol=0, err_msg=f"{label}: t")
    dg = np.abs(rgba_g[where].astype(np.int16) - rgba_o[where].astype(np.int16))
    assert dg.max(initial=0) <= RGBA_LSB, f"{label}: rgba differs by {dg.max()} LSB"
    return {"pixels": int(where.sum()), "rgba_exact": bool(dg.max(initial=0) == 0),
            "t_exact": bool(np.array_equal(hg["t"].view(np.uint32), ho["t"].view(np.uint32)))}
